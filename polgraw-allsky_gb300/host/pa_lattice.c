/*
 * pa_lattice.c -- input generation: the grid generator's lattice, the
 * grid.bin of a data segment (its grid-generating matrix M, the reduced
 * Fisher matrix and the unnormalised matrix), from the segment's
 * ephemeris.
 *
 * The reference grid generator (gridgen/main.cpp:955-1166) covers the
 * four-dimensional (frequency, spindown, two sky coordinates) parameter
 * space with a lattice whose cells fit in hyper-spheres of radius
 * sqrt(1 - c0) (c0 = minimal match squared) after the reduced Fisher matrix
 * has been turned into the identity, under the constraint that the
 * frequency step is the Fourier resolution 2 pi N / nfft:
 *   S1 (gridgen/src/DensityS1.cpp:22-150): the A4* lattice vector of
 *       smallest length not below that step, rotated onto the frequency
 *       axis by Givens rotations (num.cpp:386-490), scaled to the step;
 *   S2 (gridgen/src/GridS2.cpp:24-348): the A4* cell tilted about the
 *       frequency axis by the angle alpha at which the cell's covering
 *       radius is 1, found by bisection (35 steps) over a deep-hole search
 *       (21 rounds of a 5^4 grid of trial points shrinking by 3), or taken
 *       from the generator's table of precomputed cells (dataS2.txt) when it
 *       holds this step computed with at least as many steps;
 *   the method chosen from the step (main.cpp:1578-1606), the basis mapped
 *   back through the inverse Cholesky factor of the Fisher matrix and
 *   scaled by sqrt(1 - c0) (GridS2.cpp:427-438, GridS1.cpp:44-55), and the
 *   grid.bin layout of main.cpp:1042-1160.
 * Restated here with the same arithmetic in the same order (the grid
 * generator is built without fused multiply-adds, and so is this file), so
 * that grid.bin equals the reference's bit for bit.  Host code, run once
 * per segment; it takes under a second.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/polgraw_gb300_host.h"

#define EPS 1e-12 /* num.cpp:352-355: 1 / 10^12 */
#define PI_ 3.14159265358979323846

/* ---- 4x4 linear algebra on row-major arrays (num.cpp:158-350) ---- */

static double vlen(const double *v, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s += v[i] * v[i];
  return sqrt(s);
}

/* the (dim-1)x(dim-1) matrix without row p and column q */
static void minor_of(const double *m, int p, int q, int dim, double *out) {
  int k = 0;
  for (int i = 0; i < dim; i++)
    for (int j = 0; j < dim; j++)
      if (i != p && j != q) out[k++] = m[dim * i + j];
}

/* determinant by expansion along the first row */
static double det_n(const double *m, int dim) {
  if (dim == 2) return m[0] * m[3] - m[1] * m[2];
  double sum = 0.0, mi[9];
  for (int j = 0; j < dim; j++) {
    minor_of(m, 0, j, dim, mi);
    const double s = (j % 2 == 0) ? 1.0 : -1.0;
    sum += s * m[j] * det_n(mi, dim - 1);
  }
  return sum;
}

/* inverse by the transposed cofactor matrix over the first-row expansion */
static void inv4(const double *m, double *out) {
  double cof[16], mi[9];
  for (int p = 0; p < 4; p++)
    for (int q = 0; q < 4; q++) {
      minor_of(m, p, q, 4, mi);
      const double s = ((p + q) % 2 == 0) ? 1.0 : -1.0;
      cof[4 * p + q] = s * det_n(mi, 3);
    }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) out[4 * i + j] = cof[4 * j + i];
  double d = 0.0;
  for (int i = 0; i < 4; i++) d += m[i] * out[4 * i];
  for (int k = 0; k < 16; k++) out[k] /= d;
}

/* lower Cholesky factor */
static void chol4(const double *v, double *l) {
  for (int k = 0; k < 16; k++) l[k] = 0.0;
  for (int j = 0; j < 4; j++)
    for (int i = j; i < 4; i++) {
      double s = 0.0;
      for (int k = 0; k < j; k++) s += l[4 * i + k] * l[4 * j + k];
      if (i == j)
        l[4 * i + j] = sqrt(v[4 * i + j] - s);
      else
        l[4 * i + j] = (v[4 * i + j] - s) / l[4 * j + j];
    }
}

static void mul4(const double *a, const double *b, double *out) {
  double t[16];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      double s = 0.0;
      for (int p = 0; p < 4; p++) s += a[4 * i + p] * b[4 * p + j];
      t[4 * i + j] = s;
    }
  memcpy(out, t, sizeof t);
}

/* the Fourier step in the space of hyper-spheres, num.cpp:492-503 */
static double dw_prim(double c0, unsigned nfft, unsigned n) {
  const double w0 = 2. * PI_ * (double)n / (double)nfft;
  return w0 / (2. * sqrt(3.0 * (1.0 - c0)));
}

/* ---- S2: the tilted A4* cell (GridS2.cpp) ---- */

typedef struct {
  double a[4][4]; /* the four edge directions perpendicular to the frequency axis, unit length */
  unsigned nfft, n;
  double c0;
  int nradius;
} S2;

static void s2_init(S2 *g) {
  const double sq5 = sqrt(5), sq5_3 = sqrt(5.0 / 3.0), sq5_6 = sqrt(5.0 / 6.0);
  const double a[4][4] = {{0., -sq5_6 / 2.0, -sq5_3 / 2.0, -sq5 / 2.0},
                          {0., sqrt(7.5) / 2.0, 0., 0.},
                          {0., -sq5_6 / 2.0, sq5_3, 0.},
                          {0., -sq5_6 / 2.0, -sq5_3 / 2.0, sq5 / 2.0}};
  for (int k = 0; k < 4; k++) {
    const double l = vlen(a[k], 4);
    for (int i = 0; i < 4; i++) g->a[k][i] = a[k][i] / l;
  }
}

/* the cell's vertices at tilt alpha: the four edges, and with `all` the
 * eleven sums of them and the origin, in the generator's order */
static int s2_vertices(const S2 *g, double alpha, int all, double v[16][4]) {
  const double dwp4 = dw_prim(g->c0, g->nfft, g->n) / 4.0;
  const double dt = dwp4 * tan(alpha);
  for (int k = 0; k < 4; k++) {
    v[k][0] = dwp4;
    for (int i = 1; i < 4; i++) v[k][i] = g->a[k][i] * dt;
  }
  if (!all) return 4;
  static const int pairs[11][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3},
                                   {0, 7}, {3, 7}, {2, 6}, {1, 6}, {6, 7}};
  for (int m = 0; m < 11; m++)
    for (int i = 0; i < 4; i++) v[4 + m][i] = v[pairs[m][0]][i] + v[pairs[m][1]][i];
  for (int i = 0; i < 4; i++) v[15][i] = 0.0;
  return 16;
}

/* the point hole + sum_k shrink_k edge_k and its distance to the nearest
 * vertex (GridS2.cpp:160-191) */
static double s2_trial(const double v[16][4], const double shrink[4], const double hole[4], double pt[4]) {
  double v1[4], v3[4];
  for (int i = 0; i < 4; i++) {
    const double x1 = shrink[0] * v[0][i], x2 = shrink[1] * v[1][i];
    const double x3 = shrink[2] * v[2][i], x4 = shrink[3] * v[3][i];
    v1[i] = x1 + x2;
    v3[i] = x3 + x4;
  }
  for (int i = 0; i < 4; i++) v1[i] = v1[i] + v3[i];
  for (int i = 0; i < 4; i++) pt[i] = v1[i] + hole[i];
  double best = 0.0;
  for (int k = 0; k < 16; k++) {
    double d[4];
    for (int i = 0; i < 4; i++) d[i] = pt[i] - v[k][i];
    const double r = vlen(d, 4);
    if (k == 0 || r < best) best = r;
  }
  return best;
}

/* covering radius of the cell at tilt alpha: the deepest hole found by
 * NRadius + 1 rounds of 5^4 trial points around the current hole, each
 * round a third the size of the last (GridS2.cpp:193-234) */
static double s2_radius(const S2 *g, double alpha) {
  double v[16][4];
  s2_vertices(g, alpha, 1, v);
  double hole[4] = {0., 0., 0., 0.};
  for (int k = 0; k < 4; k++)
    for (int i = 0; i < 4; i++) hole[i] = hole[i] + v[k][i];
  for (int i = 0; i < 4; i++) hole[i] = 0.5 * hole[i];
  double sa = -1. / 3., sb = 1. / 3., dd = 1. / 6.;
  double best_r = 0.0, best_pt[4] = {0., 0., 0., 0.};
  for (int n = 0; n <= g->nradius; n++) {
    for (double i = sa; i <= sb; i += dd)
      for (double j = sa; j <= sb; j += dd)
        for (double k = sa; k <= sb; k += dd)
          for (double o = sa; o <= sb; o += dd) {
            const double shrink[4] = {i, j, k, o};
            double pt[4];
            const double r = s2_trial(v, shrink, hole, pt);
            if (r > best_r) {
              best_r = r;
              memcpy(best_pt, pt, sizeof pt);
            }
          }
    memcpy(hole, best_pt, sizeof hole);
    sa *= 1. / 3.;
    sb *= 1. / 3.;
    dd *= 1. / 3.;
  }
  return best_r;
}

/* the tilt at which the covering radius crosses 1: bisection on
 * [0.001, pi/2]; the result is the last middle point if its radius is
 * (within 1e-12) at most 1, else the left end of the last step
 * (GridS2.cpp:236-270) */
static double s2_alpha(const S2 *g, int nalpha) {
  double left = 0.001, right = PI_ / 2.;
  double r_mid = 0.0, a_mid = 0.0, a_left = 0.0;
  for (int it = 0; it < nalpha; it++) {
    const double diff = fabs(right - left);
    const double mid = left + 0.5 * diff;
    const double r_left = s2_radius(g, left);
    a_left = left;
    r_mid = s2_radius(g, mid);
    a_mid = mid;
    const int sl = (r_left - 1.) > 0 ? 1 : -1, sm = (r_mid - 1.) > 0 ? 1 : -1;
    if (sl != sm)
      right = mid;
    else
      left = mid;
  }
  return (r_mid - 1. <= EPS) ? a_mid : a_left;
}

/* The generator's table of S2 cells (dataS2.txt: a header line, then per
 * line the frequency step, density, alpha, radius and the bisection and
 * deep-hole depths they were computed with): the alpha of the last entry
 * whose step is within 1e-12 of dwp and whose depths are at least
 * (nalpha, nradius) (GridS2.cpp:305-336, 440-463).  Returns 1 and sets
 * *alpha when there is one. */
static int s2_table(const char *path, double dwp, int nalpha, int nradius, double *alpha) {
  FILE *f = path ? fopen(path, "r") : NULL;
  if (!f) return 0;
  int c;
  while ((c = fgetc(f)) != EOF && c != '\n') {
  }
  double w, dens, al, rad;
  int na, nr;
  int found = 0, use = 0;
  double a_found = 0.0;
  while (fscanf(f, "%lf %lf %lf %lf %d %d", &w, &dens, &al, &rad, &na, &nr) == 6) {
    if (w <= dwp + EPS && w >= dwp - EPS) {
      found = 1;
      a_found = al;
      use = !(na < nalpha || nr < nradius);
    }
  }
  fclose(f);
  if (found && use) *alpha = a_found;
  return found && use;
}

/* S2 basis in the space of hyper-spheres: the frequency step along the
 * first axis and three edges of the cell at the tilt (GridS2.cpp:288-348) */
static void s2_basis(const S2 *g, double alpha, double b[16]) {
  double v[16][4];
  s2_vertices(g, alpha, 0, v);
  for (int k = 0; k < 16; k++) b[k] = 0.0;
  for (int i = 1; i < 4; i++)
    for (int j = 0; j < 4; j++) b[4 * i + j] = v[i][j];
  b[0] = dw_prim(g->c0, g->nfft, g->n);
}

/* ---- S1: the A4* lattice rotated onto the frequency axis (DensityS1.cpp) ---- */

/* sine and cosine of the Givens rotation that zeroes d against c
 * (num.cpp:386-410) */
static void givens(double c, double d, double *sn, double *cs) {
  *sn = 0.;
  *cs = 1.;
  if (fabs(d) < EPS) return;
  const double cd = sqrt(c * c + d * d);
  if (cd < EPS) return;
  *sn = fabs(d / cd);
  *cs = fabs(c / cd);
}

/* the rotation of num.cpp:412-473 in the plane of axis pair `axis`
 * (0: coordinates 2,3; 1: 1,2; 2: 0,1), `left` for the opposite sense */
static void rot_matrix(double sn, double cs, int axis, int left, double tr[16]) {
  for (int k = 0; k < 16; k++) tr[k] = 0.0;
  const double s = left ? -sn : sn;
  if (axis == 0) {
    tr[0] = tr[5] = 1.0;
    tr[10] = cs;
    tr[11] = s;
    tr[14] = -s;
    tr[15] = cs;
  } else if (axis == 1) {
    tr[0] = tr[15] = 1.0;
    tr[5] = cs;
    tr[6] = s;
    tr[9] = -s;
    tr[10] = cs;
  } else {
    tr[10] = tr[15] = 1.0;
    tr[0] = cs;
    tr[1] = s;
    tr[4] = -s;
    tr[5] = cs;
  }
}

/* zero element (u, q) of the basis v against (u, q - 1) by a rotation of
 * the coordinates (num.cpp:475-490) */
static void rot_step(double v[16], int u, int axis, int q) {
  double sn, cs, tr[16], trt[16], r[16];
  givens(v[4 * u + q - 1], v[4 * u + q], &sn, &cs);
  rot_matrix(sn, cs, axis, 0, tr);
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) trt[4 * i + j] = tr[4 * j + i];
  mul4(v, trt, r);
  if (fabs(r[4 * u + q]) > EPS) {
    rot_matrix(sn, cs, axis, 1, tr);
    for (int i = 0; i < 4; i++)
      for (int j = 0; j < 4; j++) trt[4 * i + j] = tr[4 * j + i];
    mul4(v, trt, r);
  }
  memcpy(v, r, sizeof r);
}

/* The candidate lattice vectors of S1 and their order.  The generator sorts
 * them by distance with its C++ library's std::sort and takes the first;
 * lattice symmetry makes exact ties common, and std::sort leaves the order
 * of equal keys to its algorithm, so the choice among tied vectors is the
 * one that algorithm makes.  The GNU C++ library's std::sort is the
 * introsort of Musser (1997): quicksort rounds with the median of the
 * second, middle and last elements moved to the front as the pivot and an
 * unguarded two-sided partition, while a range holds more than 16
 * elements and the depth budget 2 floor(log2 n) lasts (a range that
 * exhausts it is heap-sorted), then one insertion sort over the whole
 * array, the first 16 elements guarded and the rest unguarded.  It is
 * restated below step for step on (distance, coefficients) records. */
typedef struct {
  double d;
  int w[4];
} Cand;

static void cswap(Cand *a, Cand *b) {
  const Cand t = *a;
  *a = *b;
  *b = t;
}

/* sift `v` down from `hole` in the heap base[0, len) rooted at `top`, then
 * up again */
static void heap_adjust(Cand *base, long hole, long len, Cand v) {
  const long top = hole;
  long child = hole;
  while (child < (len - 1) / 2) {
    child = 2 * (child + 1);
    if (base[child].d < base[child - 1].d) child--;
    base[hole] = base[child];
    hole = child;
  }
  if ((len & 1) == 0 && child == (len - 2) / 2) {
    child = 2 * (child + 1);
    base[hole] = base[child - 1];
    hole = child - 1;
  }
  long parent = (hole - 1) / 2;
  while (hole > top && base[parent].d < v.d) {
    base[hole] = base[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  base[hole] = v;
}

static void heap_sort(Cand *first, Cand *last) {
  const long len = last - first;
  if (len < 2) return;
  for (long parent = (len - 2) / 2;; parent--) {
    heap_adjust(first, parent, len, first[parent]);
    if (parent == 0) break;
  }
  while (last - first > 1) {
    --last;
    const Cand v = *last;
    *last = *first;
    heap_adjust(first, 0, last - first, v);
  }
}

static void intro_loop(Cand *first, Cand *last, int depth) {
  while (last - first > 16) {
    if (depth == 0) {
      heap_sort(first, last);
      return;
    }
    --depth;
    /* median of first[1], the middle and last[-1] to the front */
    Cand *a = first + 1, *b = first + (last - first) / 2, *c = last - 1;
    if (a->d < b->d) {
      if (b->d < c->d)
        cswap(first, b);
      else if (a->d < c->d)
        cswap(first, c);
      else
        cswap(first, a);
    } else if (a->d < c->d) {
      cswap(first, a);
    } else if (b->d < c->d) {
      cswap(first, c);
    } else {
      cswap(first, b);
    }
    /* partition [first + 1, last) about *first */
    Cand *lo = first + 1, *hi = last;
    for (;;) {
      while (lo->d < first->d) ++lo;
      --hi;
      while (first->d < hi->d) --hi;
      if (!(lo < hi)) break;
      cswap(lo, hi);
      ++lo;
    }
    intro_loop(lo, last, depth);
    last = lo;
  }
}

static void linear_insert(Cand *pos) {
  const Cand v = *pos;
  Cand *next = pos - 1;
  while (v.d < next->d) {
    *pos = *next;
    pos = next;
    --next;
  }
  *pos = v;
}

static void guarded_insertion(Cand *first, Cand *last) {
  if (first == last) return;
  for (Cand *i = first + 1; i != last; ++i) {
    if (i->d < first->d) {
      const Cand v = *i;
      memmove(first + 1, first, sizeof(Cand) * (size_t)(i - first));
      *first = v;
    } else {
      linear_insert(i);
    }
  }
}

static void gnu_sort(Cand *first, Cand *last) {
  const long n = last - first;
  if (n <= 1) return;
  int lg = 0;
  while ((2L << lg) <= n) lg++;
  intro_loop(first, last, 2 * lg);
  if (n > 16) {
    guarded_insertion(first, first + 16);
    for (Cand *i = first + 16; i != last; ++i) linear_insert(i);
  } else {
    guarded_insertion(first, last);
  }
}

static int s1_basis(double c0, unsigned nfft, unsigned n, double q0[16]) {
  const double dwp = dw_prim(c0, nfft, n);
  const int hd = (int)ceil(dwp / sqrt(2.0)) + 3;
  double a4[16] = {0.};
  a4[0] = sqrt(2.0);
  a4[4] = a4[8] = a4[12] = 1.0 / (2.0 * sqrt(2));
  a4[5] = sqrt(7.5) / 2.0;
  a4[9] = a4[13] = -sqrt(5.0 / 6.0) / 2.0;
  a4[10] = sqrt(5.0 / 3.0);
  a4[14] = -a4[10] / 2.0;
  a4[15] = sqrt(5) / 2.0;
  /* the lattice vectors sum_r w_r a4_r (w in [0, hd]^4, some w_r = 1) not
   * shorter than dwp, in the generator's enumeration order, sorted by their
   * excess length; the first is the one used (DensityS1.cpp:50-106) */
  const long cap = (long)(hd + 1) * (hd + 1) * (hd + 1) * (hd + 1);
  Cand *cand = (Cand *)malloc(sizeof(Cand) * (size_t)cap);
  if (!cand) return PA_ERR_NOMEM;
  long nc = 0;
  for (int i = 0; i <= hd; i++)
    for (int j = 0; j <= hd; j++)
      for (int k = 0; k <= hd; k++)
        for (int l = 0; l <= hd; l++) {
          if (!(i == 1 || j == 1 || k == 1 || l == 1)) continue;
          const int w[4] = {i, j, k, l};
          double vt[4] = {0., 0., 0., 0.};
          for (int p = 0; p < 4; p++)
            for (int q = 0; q < 4; q++) vt[p] += (0.0 + w[q] * a4[4 * q + p]);
          const double d = vlen(vt, 4);
          if (d >= dwp) {
            cand[nc].d = d - dwp;
            memcpy(cand[nc].w, w, sizeof w);
            nc++;
          }
        }
  if (nc == 0) {
    free(cand);
    return PA_ERR_ARG;
  }
  gnu_sort(cand, cand + nc);
  int best[4];
  memcpy(best, cand[0].w, sizeof best);
  free(cand);
  double qq[4] = {0., 0., 0., 0.};
  for (int p = 0; p < 4; p++)
    for (int q = 0; q < 4; q++) qq[p] += (0.0 + best[q] * a4[4 * q + p]);
  const double dlqq = vlen(qq, 4);
  int wi = 0;
  for (int i = 3; i >= 0; i--)
    if (best[i] == 1) wi = i;
  int r = 0;
  for (int j = 0; j < 4; j++) q0[r++] = qq[j];
  for (int i = 0; i < 4; i++)
    if (i != wi)
      for (int j = 0; j < 4; j++) q0[r++] = a4[4 * i + j];
  int j = 0;
  for (int i = 3; i > 0; i--) rot_step(q0, 0, j++, i);
  j = 0;
  for (int i = 3; i > 1; i--) rot_step(q0, 1, j++, i);
  rot_step(q0, 2, 0, 3);
  double dg[16] = {0.};
  dg[0] = dwp / dlqq;
  dg[5] = dg[10] = dg[15] = 1.0;
  mul4(q0, dg, q0);
  return PA_OK;
}

/* the method of main.cpp:1578-1606 from the frequency step */
static int choose_method(double c0, unsigned nfft, unsigned n) {
  const double sq2 = sqrt(2);
  const double x = dw_prim(c0, nfft, n);
  if (x <= sqrt(3)) {
    if (x < 1.64) return (x > sq2 - EPS && x < sq2 + EPS) ? 1 : 2;
    return 1;
  }
  return x < 1.81 ? 2 : 1;
}

int pa_gridgen(const double *rSSB, const double *rDet, long long n, double epsm, const pa_gridgen_opts *o,
               pa_gridgen_out *out) {
  if (!rSSB || !rDet || !o || !out || n < 5 || o->nfft_exp < 1 || o->nfft_exp > 30 || !(o->c0 > 0. && o->c0 < 1.))
    return PA_ERR_ARG;
  const unsigned nfft = 1u << o->nfft_exp;
  if ((unsigned long long)n > nfft) return PA_ERR_ARG; /* GridS2.cpp:96-100, DensityS1.cpp:34 */
  const unsigned nn = (unsigned)n;
  double fisher[16];
  int rc = pa_fisher_reduced(rSSB, rDet, n, epsm, o->xi, fisher);
  if (rc) return rc;
  const int method = o->method ? o->method : choose_method(o->c0, nfft, nn);
  double base[16];
  double alpha = 0.0;
  int from_table = 0;
  if (method == 2) {
    S2 g;
    s2_init(&g);
    g.nfft = nfft;
    g.n = nn;
    g.c0 = o->c0;
    g.nradius = o->nradius;
    from_table = s2_table(o->table, dw_prim(o->c0, nfft, nn), o->nalpha, o->nradius, &alpha);
    if (!from_table) alpha = s2_alpha(&g, o->nalpha);
    s2_basis(&g, alpha, base);
  } else if (method == 1) {
    if ((rc = s1_basis(o->c0, nfft, nn, base))) return rc;
  } else {
    return PA_ERR_ARG;
  }
  /* back to the parameter space: basis times the inverse Cholesky factor of
   * the Fisher matrix, scaled by sqrt(1 - c0) */
  double l[16], li[16], t[16];
  chol4(fisher, l);
  inv4(l, li);
  mul4(base, li, t);
  const double rs = sqrt(1.0 - o->c0);
  for (int k = 0; k < 16; k++) out->Mn[k] = rs * t[k];
  /* grid.bin (main.cpp:1042-1160): fftpad, M = Mn / N with the spindown
   * column divided by N once more, the Fisher matrix, Mn */
  out->fftpad = (int)(log2((double)nfft) - ceil(log2((double)nn)) + 1);
  for (int k = 0; k < 16; k++) out->M[k] = out->Mn[k] / nn;
  out->M[1] = out->M[1] / nn;
  out->M[5] = out->M[5] / nn;
  out->M[9] = out->M[9] / nn;
  out->M[13] = out->M[13] / nn;
  memcpy(out->fisher, fisher, sizeof fisher);
  out->method = method;
  out->alpha = method == 2 ? alpha : 0.0;
  out->alpha_from_table = from_table;
  out->density = fabs(pow(PI_, 2.0) / (2.0 * det_n(base, 4)));
  return PA_OK;
}

int pa_gridgen_write(const char *path, const pa_gridgen_out *out) {
  FILE *f = path && out ? fopen(path, "wb") : NULL;
  if (!f) return PA_ERR_ARG;
  int ok = fwrite(&out->fftpad, sizeof(int), 1, f) == 1 && fwrite(out->M, sizeof(double), 16, f) == 16 &&
           fwrite(out->fisher, sizeof(double), 16, f) == 16 && fwrite(out->Mn, sizeof(double), 16, f) == 16;
  ok = (fclose(f) == 0) && ok;
  return ok ? PA_OK : PA_ERR_ARG;
}
