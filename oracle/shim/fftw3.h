/*
 * oracle/shim/fftw3.h -- minimal FFTW3-API shim (the subset the reference
 * coherent search calls), backed by the oracle's own FP64 Stockham FFT.
 *
 * TEST INFRASTRUCTURE ONLY.  It exists so that the reference's unmodified
 * search/network/src-cpu sources can be compiled in this container, where
 * FFTW 3.3.x (the reference's pinned dependency, src-cpu/Makefile:7) is not
 * installed.  Call sites it serves: init.c:831,841,848-852,857,950-962 and
 * jobcore.c:331-332,355-356,629-630 (plus threaded planning in the OpenMP
 * variant, src-openmp/init.c:807,833).
 *
 * fftw_complex is always `double _Complex` here: the reference relies on
 * that (it includes <complex.h> before <fftw3.h> and assigns/multiplies
 * fftw_complex values as C99 complex numbers, jobcore.c:320,360,636).
 */
#ifndef PA_SHIM_FFTW3_H
#define PA_SHIM_FFTW3_H

#include <complex.h>
#include <stdio.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef double _Complex fftw_complex;
typedef struct pa_shim_fftw_plan_s *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_DESTROY_INPUT (1U << 0)
#define FFTW_UNALIGNED (1U << 1)
#define FFTW_PRESERVE_INPUT (1U << 4)
#define FFTW_PATIENT (1U << 5)
#define FFTW_ESTIMATE (1U << 6)
#define FFTW_EXHAUSTIVE (1U << 3)

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out);
void fftw_destroy_plan(fftw_plan p);

void *fftw_malloc(size_t n);
void fftw_free(void *p);

int fftw_import_wisdom_from_file(FILE *input_file);
void fftw_export_wisdom_to_file(FILE *output_file);
void fftw_forget_wisdom(void);
void fftw_cleanup(void);

int fftw_init_threads(void);
void fftw_plan_with_nthreads(int nthreads);
void fftw_cleanup_threads(void);

#ifdef __cplusplus
}
#endif

#endif
