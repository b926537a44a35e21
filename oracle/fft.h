/*
 * oracle/fft.h -- FP64 complex FFT of power-of-two length for the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY.  This file belongs to the CPU oracle: it is
 * linked into the oracle restatement of the coherent search (oracle.c) and
 * into the FFTW-API shim that lets the unmodified reference search be
 * compiled here.  Nothing in the product (the CUDA library) uses it.
 *
 * Semantics follow FFTW's fftw_plan_dft_1d / fftw_execute_dft as used by the
 * reference at search/network/src-cpu/init.c:848-852 and jobcore.c:331,355,629:
 * unnormalised transform, sign -1 = forward (exp(-2 pi i jk/n)), sign +1 =
 * backward, in-place allowed.  Only power-of-two lengths are needed (nfft,
 * Ninterp = 2 nfft, nfftf = fftpad nfft, settings.c:34, init.c:835,844).
 */
#ifndef PA_ORACLE_FFT_H
#define PA_ORACLE_FFT_H

#include <complex.h>

typedef struct oracle_fft_plan {
  int n;                 /* transform length (power of two) */
  int log2n;
  int sign;              /* -1 forward, +1 backward */
  double complex *tw;    /* tw[m] = exp(sign 2 pi i m / n), m < n */
} oracle_fft_plan;

/* Returns NULL if n is not a power of two >= 1. */
oracle_fft_plan *oracle_fft_plan_create(int n, int sign);
void oracle_fft_plan_destroy(oracle_fft_plan *p);

/* out may equal in.  Thread-safe: the plan is read-only during execution and
 * the scratch buffer is allocated per call. */
void oracle_fft_exec(const oracle_fft_plan *p, const double complex *in,
                     double complex *out);

#endif
