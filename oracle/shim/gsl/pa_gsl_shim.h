/*
 * oracle/shim/gsl/pa_gsl_shim.h -- the small GSL subset the reference search
 * calls, re-implemented for the oracle build.  TEST INFRASTRUCTURE ONLY.
 *
 * GSL is not installed in this container; the reference uses it (unpinned
 * version) for one 4x4 LU solve that maps an injected signal onto the grid
 * (search/network/src-cpu/init.c:541-557) and for a symmetric eigensystem
 * used only by the coincidences tool (init.c:1185-1202, not on the search
 * path).  Semantics follow GSL's documented API: row-major matrices, LU with
 * partial pivoting (P A = L U), vectors with stride.
 */
#ifndef PA_SHIM_GSL_H
#define PA_SHIM_GSL_H

#include <stddef.h>
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { size_t size; size_t stride; double *data; void *block; int owner; } gsl_vector;
typedef struct { gsl_vector vector; } gsl_vector_view;
typedef struct { size_t size1, size2, tda; double *data; void *block; int owner; } gsl_matrix;
typedef struct { gsl_matrix matrix; } gsl_matrix_view;
typedef struct { size_t size; size_t *data; } gsl_permutation;
typedef struct { size_t size; } gsl_eigen_symmv_workspace;

gsl_vector *gsl_vector_alloc(size_t n);
void gsl_vector_free(gsl_vector *v);
double gsl_vector_get(const gsl_vector *v, size_t i);
void gsl_vector_set(gsl_vector *v, size_t i, double x);
gsl_vector_view gsl_vector_view_array(double *base, size_t n);

gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix *m);
gsl_matrix_view gsl_matrix_view_array(double *base, size_t n1, size_t n2);
int gsl_matrix_transpose(gsl_matrix *m);
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j);
gsl_vector_view gsl_matrix_column(gsl_matrix *m, size_t j);

gsl_permutation *gsl_permutation_alloc(size_t n);
void gsl_permutation_free(gsl_permutation *p);

int gsl_linalg_LU_decomp(gsl_matrix *A, gsl_permutation *p, int *signum);
int gsl_linalg_LU_invert(const gsl_matrix *LU, const gsl_permutation *p, gsl_matrix *inv);
int gsl_linalg_LU_solve(const gsl_matrix *LU, const gsl_permutation *p,
                        const gsl_vector *b, gsl_vector *x);

gsl_eigen_symmv_workspace *gsl_eigen_symmv_alloc(size_t n);
void gsl_eigen_symmv_free(gsl_eigen_symmv_workspace *w);
int gsl_eigen_symmv(gsl_matrix *A, gsl_vector *eval, gsl_matrix *evec,
                    gsl_eigen_symmv_workspace *w);

#ifdef __cplusplus
}
#endif
#endif
