/*
 * oracle/oracle.h -- CPU oracle for the coherent network search hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C, all-FP64 restatement of the
 * reference's job_core() and the helpers it calls.  It is the parity
 * reference for the CUDA library: only the tests, the smoke check and the CPU-baseline leg
 * of bench.py load it.  The product never links or calls it.
 *
 * Parity is pinned by comparing this oracle's candidates against the
 * unmodified reference search (search/network/src-cpu) compiled in this
 * container against the FFTW/GSL shims in oracle/shim (outputs committed as
 * golden fixtures under tests/golden/).
 *
 * It uses the same plain structs as the product's C-ABI (include/
 * polgraw_gb300.h) so that both see byte-identical inputs.
 */
#ifndef PA_ORACLE_H
#define PA_ORACLE_H

#include "../include/polgraw_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ora_ctx ora_ctx;

/* search_settings() (settings.c:16-81) plus the Ninterp/nfftf assignments of
 * plan_fftw() (init.c:835,844).  Inputs: sett->dt, sett->fpo, sett->nod,
 * sett->fftpad.  Everything else is derived. */
void ora_search_settings(pa_settings *sett);

/* rogcvir() (settings.c:253-275): amplitude-modulation coefficients c1..c9
 * from latitude ephi and orientation egam (radians). */
void ora_rogcvir(double ephi, double egam, double amod[9]);

/* var() (auxi.c:124-139) and crf0 (init.c:359-370): sig2 = crf0 * var. */
double ora_sig2(const double *xDat, int N);

/* Creates a context holding copies of the inputs, the FFT plans and the
 * cos/sin(omr i) tables (init.c:444-455).  nthreads <= 0: OpenMP default. */
ora_ctx *ora_create(const pa_settings *sett, const pa_detector *det, int nifo,
                    int nthreads);
void ora_destroy(ora_ctx *c);

/* job_core() (jobcore.c:189-695).  Appends records/indices like
 * pa_job_core().  Optional diagnostics:
 *   pre_a/pre_b : nifo*N interleaved complex, the prelude output
 *   aa_out/bb_out
 *   F_ss, F_out : when F_out != NULL, the normalised F (nmax-nmin values) of
 *                 spindown F_ss is copied out.
 * Returns 0, or -1 when the capacity would be exceeded (*needed set). */
int ora_job_core(ora_ctx *c, int pm, int mm, int nn, const pa_opts *opts,
                 const pa_range *s_range, int *sgnlc, double *sgnlv, int cap,
                 pa_cand_idx *idx, int *FNum, int *needed, double *pre_a,
                 double *pre_b, double *aa_out, double *bb_out, int F_ss,
                 double *F_out);

/* Oracle FFT exposed for the FFT tests (sign -1 forward, +1 backward),
 * interleaved complex in/out of length n. */
int ora_fft(int n, int sign, const double *in, double *out);

/* Number of spindowns job_core() would run for (mm, nn) (jobcore.c:424-444). */
int ora_spindown_range(const pa_settings *sett, int mm, int nn,
                       const pa_opts *opts, const pa_range *s_range,
                       int *smin, int *smax);

/* Followup (followup/src/followup.c).
 * ora_fstatnet: Fstatnet() at sgnlo = (f, s, delta, alpha) with the sky
 *   set-up of evaluate_simplex() (followup.c:413-535, 986-1009); out[11] as
 *   the reference's fstat_out (out[5] = -F).
 * ora_fstatnet_grad: F and dF/d(f, s, delta, alpha), FP64 forward
 *   differentiation (the reference gradient of the adjoint tests).
 * ora_amoeba: the reference simplex (followup.c:1126-1174); max_evals > 0
 *   bounds the evaluations; returns the number of evaluations. */
void ora_fstatnet(ora_ctx *c, const double sgnlo[4], double out[11]);
double ora_fstatnet_grad(ora_ctx *c, const double sgnlo[4], double grad[4]);
int ora_amoeba(ora_ctx *c, double point[4], const double pc2[4], double tol, int max_evals,
               double out[11]);

/* Coincidences (coincidences/src/coincidences.c:117-600), oracle_coinc.c.
 * ora_coinc_vedva: manage_grid_matrix()'s transformation matrix
 *   (init.c:1185-1210) through the GSL shim's eigensystem.
 * ora_coinc_run: all frames in the given order (the reference's directory
 *   order); results read back like pa_coinc_get / pa_coinc_cells. */
typedef struct ora_coinc ora_coinc;
int ora_coinc_vedva(const double *fisher, double *vedva);
ora_coinc *ora_coinc_run(const pa_coinc_cfg *cfg, int nframes, const int *frames,
                         const double *const *recs, const long long *nrec,
                         pa_coinc_summary *sum);
int ora_coinc_get(const ora_coinc *o, int *frameinfo, pa_coinc_rec *recs, int *fra, int *ops);
int ora_coinc_cells(const ora_coinc *o, int *cells, unsigned char *keep);
void ora_coinc_free(ora_coinc *o);

#ifdef __cplusplus
}
#endif
#endif
