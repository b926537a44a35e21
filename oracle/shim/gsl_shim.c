/*
 * oracle/shim/gsl_shim.c -- the GSL subset declared in gsl/pa_gsl_shim.h.
 * TEST INFRASTRUCTURE ONLY.
 *
 * LU: Gaussian elimination with partial pivoting on the largest |a_ij| of the
 * column (GSL's documented choice), in place, P A = L U with unit-diagonal L.
 * Eigen: cyclic Jacobi rotations for a small symmetric matrix; only the
 * coincidences tool calls it (init.c:1185-1202), never the search.
 */
#include "gsl/pa_gsl_shim.h"

#include <stdlib.h>
#include <string.h>

gsl_vector *gsl_vector_alloc(size_t n) {
  gsl_vector *v = (gsl_vector *)calloc(1, sizeof(*v));
  v->size = n;
  v->stride = 1;
  v->data = (double *)calloc(n ? n : 1, sizeof(double));
  v->owner = 1;
  return v;
}

void gsl_vector_free(gsl_vector *v) {
  if (!v) return;
  if (v->owner) free(v->data);
  free(v);
}

double gsl_vector_get(const gsl_vector *v, size_t i) { return v->data[i * v->stride]; }
void gsl_vector_set(gsl_vector *v, size_t i, double x) { v->data[i * v->stride] = x; }

gsl_vector_view gsl_vector_view_array(double *base, size_t n) {
  gsl_vector_view w;
  memset(&w, 0, sizeof(w));
  w.vector.size = n;
  w.vector.stride = 1;
  w.vector.data = base;
  return w;
}

gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2) {
  gsl_matrix *m = (gsl_matrix *)calloc(1, sizeof(*m));
  m->size1 = n1;
  m->size2 = n2;
  m->tda = n2;
  m->data = (double *)calloc(n1 * n2 ? n1 * n2 : 1, sizeof(double));
  m->owner = 1;
  return m;
}

void gsl_matrix_free(gsl_matrix *m) {
  if (!m) return;
  if (m->owner) free(m->data);
  free(m);
}

gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2) {
  gsl_matrix_view v;
  memset(&v, 0, sizeof(v));
  v.matrix.size1 = n1;
  v.matrix.size2 = n2;
  v.matrix.tda = n2;
  v.matrix.data = base;
  return v;
}

double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j) {
  return m->data[i * m->tda + j];
}

int gsl_matrix_transpose(gsl_matrix *m) {
  if (m->size1 != m->size2) return 1;
  for (size_t i = 0; i < m->size1; i++)
    for (size_t j = i + 1; j < m->size2; j++) {
      double t = m->data[i * m->tda + j];
      m->data[i * m->tda + j] = m->data[j * m->tda + i];
      m->data[j * m->tda + i] = t;
    }
  return 0;
}

gsl_vector_view gsl_matrix_column(gsl_matrix *m, size_t j) {
  gsl_vector_view w;
  memset(&w, 0, sizeof(w));
  w.vector.size = m->size1;
  w.vector.stride = m->tda;
  w.vector.data = m->data + j;
  return w;
}

gsl_permutation *gsl_permutation_alloc(size_t n) {
  gsl_permutation *p = (gsl_permutation *)calloc(1, sizeof(*p));
  p->size = n;
  p->data = (size_t *)calloc(n ? n : 1, sizeof(size_t));
  for (size_t i = 0; i < n; i++) p->data[i] = i;
  return p;
}

void gsl_permutation_free(gsl_permutation *p) {
  if (!p) return;
  free(p->data);
  free(p);
}

int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum) {
  const size_t n = A->size1;
  double *a = A->data;
  const size_t t = A->tda;
  for (size_t i = 0; i < n; i++) p->data[i] = i;
  *signum = 1;
  for (size_t j = 0; j + 1 < n; j++) {
    size_t piv = j;
    double best = fabs(a[j * t + j]);
    for (size_t i = j + 1; i < n; i++) {
      double v = fabs(a[i * t + j]);
      if (v > best) { best = v; piv = i; }
    }
    if (piv != j) {
      for (size_t k = 0; k < n; k++) {
        double tmp = a[j * t + k];
        a[j * t + k] = a[piv * t + k];
        a[piv * t + k] = tmp;
      }
      size_t tp = p->data[j];
      p->data[j] = p->data[piv];
      p->data[piv] = tp;
      *signum = -*signum;
    }
    double ajj = a[j * t + j];
    if (ajj != 0.0) {
      for (size_t i = j + 1; i < n; i++) {
        double lij = a[i * t + j] / ajj;
        a[i * t + j] = lij;
        for (size_t k = j + 1; k < n; k++) a[i * t + k] -= lij * a[j * t + k];
      }
    }
  }
  return 0;
}

int gsl_linalg_LU_solve(const gsl_matrix *LU, const gsl_permutation *p,
                        const gsl_vector *b, gsl_vector *x) {
  const size_t n = LU->size1;
  const double *a = LU->data;
  const size_t t = LU->tda;
  /* x = P b */
  for (size_t i = 0; i < n; i++) gsl_vector_set(x, i, gsl_vector_get(b, p->data[i]));
  /* forward: L y = P b (unit diagonal) */
  for (size_t i = 0; i < n; i++) {
    double s = gsl_vector_get(x, i);
    for (size_t k = 0; k < i; k++) s -= a[i * t + k] * gsl_vector_get(x, k);
    gsl_vector_set(x, i, s);
  }
  /* backward: U x = y */
  for (size_t ii = n; ii-- > 0;) {
    double s = gsl_vector_get(x, ii);
    for (size_t k = ii + 1; k < n; k++) s -= a[ii * t + k] * gsl_vector_get(x, k);
    gsl_vector_set(x, ii, s / a[ii * t + ii]);
  }
  return 0;
}

/* inverse from the LU factors, one column per unit vector */
int gsl_linalg_LU_invert(const gsl_matrix *LU, const gsl_permutation *p, gsl_matrix *inv) {
  const size_t n = LU->size1;
  gsl_vector *e = gsl_vector_alloc(n), *x = gsl_vector_alloc(n);
  for (size_t j = 0; j < n; j++) {
    for (size_t i = 0; i < n; i++) gsl_vector_set(e, i, i == j ? 1.0 : 0.0);
    gsl_linalg_LU_solve(LU, p, e, x);
    for (size_t i = 0; i < n; i++) inv->data[i * inv->tda + j] = gsl_vector_get(x, i);
  }
  gsl_vector_free(e);
  gsl_vector_free(x);
  return 0;
}

gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(size_t n) {
  gsl_eigen_symmv_workspace *w = (gsl_eigen_symmv_workspace *)calloc(1, sizeof(*w));
  w->size = n;
  return w;
}

void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace *w) { free(w); }

int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec,
                    gsl_eigen_symmv_workspace *w) {
  (void)w;
  const size_t n = A->size1;
  double *a = A->data;
  const size_t t = A->tda;
  for (size_t i = 0; i < n; i++)
    for (size_t j = 0; j < n; j++) evec->data[i * evec->tda + j] = (i == j);
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = 0;
    for (size_t i = 0; i < n; i++)
      for (size_t j = i + 1; j < n; j++) off += a[i * t + j] * a[i * t + j];
    if (off < 1e-300) break;
    for (size_t pp = 0; pp < n; pp++)
      for (size_t q = pp + 1; q < n; q++) {
        double apq = a[pp * t + q];
        if (apq == 0.0) continue;
        double theta = (a[q * t + q] - a[pp * t + pp]) / (2.0 * apq);
        double tt = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(tt * tt + 1.0), s = tt * c;
        for (size_t k = 0; k < n; k++) {
          double akp = a[k * t + pp], akq = a[k * t + q];
          a[k * t + pp] = c * akp - s * akq;
          a[k * t + q] = s * akp + c * akq;
        }
        for (size_t k = 0; k < n; k++) {
          double apk = a[pp * t + k], aqk = a[q * t + k];
          a[pp * t + k] = c * apk - s * aqk;
          a[q * t + k] = s * apk + c * aqk;
        }
        for (size_t k = 0; k < n; k++) {
          double vkp = evec->data[k * evec->tda + pp], vkq = evec->data[k * evec->tda + q];
          evec->data[k * evec->tda + pp] = c * vkp - s * vkq;
          evec->data[k * evec->tda + q] = s * vkp + c * vkq;
        }
      }
  }
  for (size_t i = 0; i < n; i++) gsl_vector_set(eval, i, a[i * t + i]);
  return 0;
}
