/*
 * oracle/fft.c -- iterative Stockham autosort FFT, radix 4 with one trailing
 * radix-2 stage for odd log2(n).  FP64 throughout.
 *
 * TEST INFRASTRUCTURE ONLY (CPU oracle and the FFTW-API shim); see fft.h.
 *
 * Algorithm (decimation in frequency, Stockham autosort): a length-L block
 * with stride s is split into four quarter-length sub-sequences
 *   y[q + s(4p+k)] = W_L^{kp} * sum_r x[q + s(p + r L/4)] * W_4^{kr}
 * for p < L/4, q < s, k < 4, after which the sub-problem has length L/4 and
 * stride 4s.  The data ping-pong between the caller's output and one scratch
 * buffer; no bit reversal is needed.  Twiddles come from one table of
 * exp(sign 2 pi i m / n) evaluated in FP64 with the angle reduced to the first
 * octant, so each entry is correctly rounded to within one ulp.
 */
#include "fft.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static int ilog2_exact(int n) {
  int l = 0;
  if (n < 1) return -1;
  while ((1 << l) < n) l++;
  return ((1 << l) == n) ? l : -1;
}

/* exp(sign 2 pi i m / n) with the angle folded into [0, pi/4]. */
static double complex twiddle(long m, long n, int sign) {
  /* 8 m / n = octant index + fraction; work with integers to stay exact */
  long m8 = 8 * m;
  long oct = m8 / n;                /* 0..7 */
  long rem = m8 - oct * n;          /* 0..n-1, angle within octant = rem/n * pi/4 */
  double c, s;
  double a;
  /* fold: odd octants measure from the next octant boundary */
  if (oct & 1) a = (double)(n - rem) / (double)n * (M_PI / 4.0);
  else a = (double)rem / (double)n * (M_PI / 4.0);
  double ca = cos(a), sa = sin(a);
  switch (oct) {
    case 0: c = ca;  s = sa;  break;            /* [0, pi/4)      */
    case 1: c = sa;  s = ca;  break;            /* [pi/4, pi/2)   */
    case 2: c = -sa; s = ca;  break;            /* [pi/2, 3pi/4)  */
    case 3: c = -ca; s = sa;  break;            /* [3pi/4, pi)    */
    case 4: c = -ca; s = -sa; break;            /* [pi, 5pi/4)    */
    case 5: c = -sa; s = -ca; break;            /* [5pi/4, 3pi/2) */
    case 6: c = sa;  s = -ca; break;            /* [3pi/2, 7pi/4) */
    default: c = ca; s = -sa; break;            /* [7pi/4, 2pi)   */
  }
  return c + (double)sign * s * I;
}

oracle_fft_plan *oracle_fft_plan_create(int n, int sign) {
  int l = ilog2_exact(n);
  if (l < 0 || (sign != -1 && sign != 1)) return NULL;
  oracle_fft_plan *p = (oracle_fft_plan *)calloc(1, sizeof(*p));
  if (!p) return NULL;
  p->n = n;
  p->log2n = l;
  p->sign = sign;
  p->tw = (double complex *)malloc((size_t)n * sizeof(double complex));
  if (!p->tw) { free(p); return NULL; }
  for (long m = 0; m < n; m++) p->tw[m] = twiddle(m, n, sign);
  return p;
}

void oracle_fft_plan_destroy(oracle_fft_plan *p) {
  if (!p) return;
  free(p->tw);
  free(p);
}

void oracle_fft_exec(const oracle_fft_plan *p, const double complex *in,
                     double complex *out) {
  const int n = p->n;
  if (n == 1) { out[0] = in[0]; return; }
  double complex *scratch = (double complex *)malloc((size_t)n * sizeof(double complex));
  /* Number of stages decides which buffer receives the final result; choose
   * the start buffer so that the last stage writes into `out`. */
  int nstages = p->log2n / 2 + (p->log2n & 1);
  double complex *x, *y;
  if (nstages & 1) {          /* odd number of stages: start in scratch */
    memcpy(scratch, in, (size_t)n * sizeof(double complex));
    x = scratch; y = out;
  } else {
    if (out != in) memcpy(out, in, (size_t)n * sizeof(double complex));
    x = out; y = scratch;
  }
  /* +-i factor of the radix-4 butterfly: sign -1 -> -i, +1 -> +i */
  const double complex jj = (double)p->sign * I;
  long L = n, s = 1;
  while (L >= 4) {
    const long L4 = L / 4;
    const long tstride = n / L;          /* W_L^e = tw[e * n / L] */
    for (long pp = 0; pp < L4; pp++) {
      const double complex w1 = p->tw[pp * tstride];
      const double complex w2 = p->tw[2 * pp * tstride];
      const double complex w3 = p->tw[3 * pp * tstride];
      const double complex *x0 = x + s * pp;
      const double complex *x1 = x + s * (pp + L4);
      const double complex *x2 = x + s * (pp + 2 * L4);
      const double complex *x3 = x + s * (pp + 3 * L4);
      double complex *y0 = y + s * (4 * pp);
      for (long q = 0; q < s; q++) {
        const double complex a = x0[q], b = x1[q], c = x2[q], d = x3[q];
        const double complex apc = a + c, amc = a - c;
        const double complex bpd = b + d, jbmd = jj * (b - d);
        y0[q]         = apc + bpd;
        y0[q + s]     = w1 * (amc + jbmd);
        y0[q + 2 * s] = w2 * (apc - bpd);
        y0[q + 3 * s] = w3 * (amc - jbmd);
      }
    }
    double complex *t = x; x = y; y = t;
    L = L4;
    s *= 4;
  }
  if (L == 2) {
    for (long q = 0; q < s; q++) {
      const double complex a = x[q], b = x[q + s];
      y[q] = a + b;
      y[q + s] = a - b;
    }
    double complex *t = x; x = y; y = t;
  }
  /* x now holds the result and, by the stage-count choice above, x == out */
  if (x != out) memcpy(out, x, (size_t)n * sizeof(double complex));
  free(scratch);
}
