/*
 * oracle/oracle.c -- all-FP64 CPU restatement of the reference coherent
 * search hot path.  TEST INFRASTRUCTURE ONLY (see oracle.h): the parity
 * reference for the CUDA library and the timed CPU baseline ("port") of
 * bench.py.
 *
 * Each function follows the reference file:line named in its comment, with
 * the same floating-point expression order (the build uses
 * -ffp-contract=off so no FMA contraction changes roundings), so that on the
 * same inputs it reproduces the reference's candidates and F values to
 * rounding level.  The spindown loop runs under OpenMP like
 * search/network/src-openmp/jobcore.c:455-478; candidates are gathered per
 * spindown and appended in the serial order of src-cpu/jobcore.c:449-695.
 */
#define _GNU_SOURCE
#include "oracle.h"

#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "fft.h"

#define SQR(x) ((x) * (x))
#define C_OMEGA_R 7.2921151467064e-5             /* settings.h:31 */
#define C_SIDDAY (2. * M_PI / C_OMEGA_R)          /* settings.h:32 */

struct ora_ctx {
  pa_settings sett;
  int nifo;
  int nthreads;
  double *lines;            /* 2*numlines_band */
  double *xDat[PA_MAX_DETECTORS], *DetSSB[PA_MAX_DETECTORS];
  pa_detector det[PA_MAX_DETECTORS];
  double *cosmodf, *sinmodf, *t2;
  oracle_fft_plan *plan, *pl_int, *pl_inv;
  int arr_len;
};

/* settings.c:16-81, init.c:835,844 */
void ora_search_settings(pa_settings *s) {
  double dt = s->dt;
  double B = 0.5 / dt;
  double oms = 2. * M_PI * (s->fpo) * dt;
  double omr = C_OMEGA_R * dt;
  int N = (int)floor(s->nod * C_SIDDAY / dt + 0.5);   /* round macro, auxi.h:14 */
  int nfft = 1 << (int)ceil(log(N) / log(2.));
  double fdotmin = 0.5e-8, fdotmax = 0.5e-9;          /* settings.c:46-48 */
  s->B = B;
  s->oms = oms;
  s->omr = omr;
  s->N = N;
  s->nfft = nfft;
  s->s = 1;
  s->Smax = 2. * M_PI * fdotmin * dt * dt;
  s->Smin = 2. * M_PI * fdotmax * dt * dt;
  s->nd = 2;
  s->interpftpad = 2;
  s->nmin = s->fftpad * PA_NAV * s->B;
  s->nmax = (s->nfft / 2 - PA_NAV * s->B) * s->fftpad;
  s->Ninterp = s->interpftpad * s->nfft;
  s->nfftf = s->fftpad * s->nfft;
}

/* settings.c:253-275 */
void ora_rogcvir(double ephi, double egam, double c[9]) {
  c[0] = .25 * sin(2. * egam) * (1 + SQR(sin(ephi)));
  c[1] = -.5 * cos(2. * egam) * sin(ephi);
  c[2] = .5 * sin(2. * egam) * sin(2. * ephi);
  c[3] = -cos(2. * egam) * cos(ephi);
  c[4] = .75 * sin(2. * egam) * SQR(cos(ephi));
  c[5] = cos(2. * egam) * sin(ephi);
  c[6] = .5 * sin(2. * egam) * (1. + SQR(sin(ephi)));
  c[7] = cos(2. * egam) * cos(ephi);
  c[8] = .5 * sin(2. * egam) * sin(2. * ephi);
}

/* auxi.c:124-139 and init.c:359-370 */
double ora_sig2(const double *x, int n) {
  int nz = 0;
  for (int j = 0; j < n; j++)
    if (!x[j]) nz++;
  double crf0 = (double)n / (n - nz);
  double mean = 0., v = 0.;
  for (int i = 0; i < n; i++) mean += x[i];
  mean /= n;
  for (int i = 0; i < n; i++) v += SQR(x[i] - mean);
  v /= (n - 1);
  return crf0 * v;
}

/* auxi.c:16-24 */
static void lin2ast(double be1, double be2, int pm, double sepsm, double cepsm,
                    double *sinal, double *cosal, double *sindel, double *cosdel) {
  *sindel = be1 * sepsm - (2 * pm - 3) * sqrt(1. - SQR(be1) - SQR(be2)) * cepsm;
  *cosdel = sqrt(1. - SQR(*sindel));
  *sinal = (be1 - sepsm * (*sindel)) / (cepsm * (*cosdel));
  *cosal = be2 / (*cosdel);
}

/* settings.c:281-325 */
static void modvir(double sinal, double cosal, double sindel, double cosdel,
                   int Np, const pa_detector *d, const double *cosmodf,
                   const double *sinmodf, double *aa, double *bb) {
  const double *k = d->amod;
  double cosalfr = cosal * (d->cphir) + sinal * (d->sphir);
  double sinalfr = sinal * (d->cphir) - cosal * (d->sphir);
  double c2d = SQR(cosdel);
  double c2sd = sindel * cosdel;
  for (int t = 0; t < Np; t++) {
    double c = cosalfr * cosmodf[t] + sinalfr * sinmodf[t];
    double s = sinalfr * cosmodf[t] - cosalfr * sinmodf[t];
    double c2s = 2. * SQR(c);
    double cs = c * s;
    aa[t] = k[0] * (2. - c2d) * c2s + k[1] * (2. - c2d) * 2. * cs + k[2] * c2sd * c +
            k[3] * c2sd * s - k[0] * (2. - c2d) + k[4] * c2d;
    bb[t] = k[5] * sindel * c2s + k[6] * sindel * 2. * cs + k[7] * cosdel * c +
            k[8] * cosdel * s - k[5] * sindel;
  }
}

/* auxi.c:56-81: natural cubic spline through y[0..n-1], unit spacing.  The
 * pivot sequence 2/(y2[i-1]+4) is real; the reference forms it as a complex
 * number with zero imaginary part, which rounds identically. */
static void spline(const double complex *y, int n, double complex *y2,
                   double complex *u) {
  double *p = (double *)malloc((size_t)n * sizeof(double));
  p[0] = 0.;
  u[0] = 0.;
  for (int i = 1; i < n - 1; ++i) {
    double invp = 2. / (p[i - 1] + 4.);
    p[i] = -.5 * invp;
    double complex d = y[i - 1] - 2. * y[i] + y[i + 1];
    u[i] = (-.5 * u[i - 1] + 3. * d) * invp;
  }
  y2[n - 1] = 0.;
  for (int k = n - 2; k >= 0; --k) y2[k] = p[k] * y2[k + 1] + u[k];
  free(p);
}

/* auxi.c:83-96 */
static double complex splint(const double complex *ya, const double complex *y2a,
                             int n, double x) {
  if (x < 0 || x > n - 1) return 0.;
  int klo = (int)floor(x);
  int khi = klo + 1;
  double a = khi - x;
  double b = x - klo;
  /* khi == n only when x == n-1 exactly; then b == 0 and the reference's
   * out-of-range read is multiplied by zero.  Clamp the index instead. */
  int kh = khi < n ? khi : n - 1;
  return a * ya[klo] + b * ya[kh] +
         ((a * a * a - a) * y2a[klo] + (b * b * b - b) * y2a[kh]) / 6.0;
}

/* auxi.c:98-122 */
static void splintpad(const double complex *ya, const double *shftf, int N,
                      int interpftpad, double complex *out) {
  int n = interpftpad * N;
  double complex *y2 = (double complex *)malloc((size_t)n * sizeof(double complex));
  double complex *u = (double complex *)malloc((size_t)n * sizeof(double complex));
  spline(ya, n, y2, u);
  for (int i = 0; i < N; ++i) {
    double x = interpftpad * (i - shftf[i]);
    out[i] = splint(ya, y2, n, x);
  }
  free(u);
  free(y2);
}

/* auxi.c:214-240 (pxout unused by the search) */
static void fstat_norm(double *F, int nfft, int nav) {
  double *fr = F;
  for (int j = 0; j < nfft / nav; j++) {
    double mu = 0.;
    for (int i = 0; i < nav; i++) mu += *fr++;
    mu /= 2. * nav;
    fr -= nav;
    for (int i = 0; i < nav; i++) *fr++ /= mu;
  }
}

ora_ctx *ora_create(const pa_settings *sett, const pa_detector *det, int nifo,
                    int nthreads) {
  if (nifo < 1 || nifo > PA_MAX_DETECTORS) return NULL;
  ora_ctx *c = (ora_ctx *)calloc(1, sizeof(*c));
  c->sett = *sett;
  c->nifo = nifo;
  c->nthreads = nthreads;
  const int N = sett->N;
  if (sett->numlines_band > 0) {
    c->lines = (double *)malloc(2 * sizeof(double) * sett->numlines_band);
    memcpy(c->lines, sett->lines, 2 * sizeof(double) * sett->numlines_band);
  }
  c->sett.lines = c->lines;
  for (int n = 0; n < nifo; n++) {
    c->det[n] = det[n];
    c->xDat[n] = (double *)malloc(sizeof(double) * N);
    c->DetSSB[n] = (double *)malloc(sizeof(double) * 3 * N);
    memcpy(c->xDat[n], det[n].xDat, sizeof(double) * N);
    memcpy(c->DetSSB[n], det[n].DetSSB, sizeof(double) * 3 * N);
    c->det[n].xDat = c->xDat[n];
    c->det[n].DetSSB = c->DetSSB[n];
  }
  /* init.c:444-455 */
  c->t2 = (double *)malloc(sizeof(double) * N);
  c->cosmodf = (double *)malloc(sizeof(double) * N);
  c->sinmodf = (double *)malloc(sizeof(double) * N);
  for (int i = 0; i < N; i++) {
    double omrt = (sett->omr) * i;
    c->t2[i] = SQR((double)i);
    c->cosmodf[i] = cos(omrt);
    c->sinmodf[i] = sin(omrt);
  }
  /* init.c:838-852 */
  c->arr_len = sett->fftpad * sett->nfft > sett->Ninterp ? sett->fftpad * sett->nfft
                                                          : sett->Ninterp;
  c->plan = oracle_fft_plan_create(sett->nfftf, -1);
  c->pl_int = oracle_fft_plan_create(sett->nfft, -1);
  c->pl_inv = oracle_fft_plan_create(sett->Ninterp, +1);
  if (!c->plan || !c->pl_int || !c->pl_inv) {
    ora_destroy(c);
    return NULL;
  }
  return c;
}

void ora_destroy(ora_ctx *c) {
  if (!c) return;
  for (int n = 0; n < c->nifo; n++) {
    free(c->xDat[n]);
    free(c->DetSSB[n]);
  }
  free(c->lines);
  free(c->t2);
  free(c->cosmodf);
  free(c->sinmodf);
  oracle_fft_plan_destroy(c->plan);
  oracle_fft_plan_destroy(c->pl_int);
  oracle_fft_plan_destroy(c->pl_inv);
  free(c);
}

int ora_fft(int n, int sign, const double *in, double *out) {
  oracle_fft_plan *p = oracle_fft_plan_create(n, sign);
  if (!p) return -1;
  oracle_fft_exec(p, (const double complex *)in, (double complex *)out);
  oracle_fft_plan_destroy(p);
  return 0;
}

/* jobcore.c:424-444 */
int ora_spindown_range(const pa_settings *sett, int mm, int nn,
                       const pa_opts *opts, const pa_range *s_range, int *smin_o,
                       int *smax_o) {
  int smin = s_range->sst, smax = s_range->spndr[1];
  const double *M = sett->M;
  if (!opts->use_range) {
    smin = trunc((sett->Smin - nn * M[9] - mm * M[13]) / M[5]);
    smax = trunc(-(nn * M[9] + mm * M[13] + sett->Smax) / M[5]);
    if (smin > smax) {
      int t = smin;
      smin = smax;
      smax = t;
    }
  }
  if (opts->s0_flag) smin = smax;
  *smin_o = smin;
  *smax_o = smax;
  return smax >= smin ? smax - smin + 1 : 0;
}

typedef struct { int ss, ii; double rec[PA_NPAR]; double F; } ora_cand;

int ora_job_core(ora_ctx *c, int pm, int mm, int nn, const pa_opts *opts,
                 const pa_range *s_range, int *sgnlc, double *sgnlv, int cap,
                 pa_cand_idx *idx, int *FNum, int *needed, double *pre_a,
                 double *pre_b, double *aa_out, double *bb_out, int F_ss,
                 double *F_out) {
  const pa_settings *sett = &c->sett;
  const double *M = sett->M;
  const int N = sett->N, nifo = c->nifo;
  double sgnlt[PA_NPAR];
  if (needed) *needed = 0;

  /* jobcore.c:243-248 */
  double al1 = nn * M[10] + mm * M[14];
  double al2 = nn * M[11] + mm * M[15];
  if ((SQR(al1) + SQR(al2)) / SQR(sett->oms) > 1.) return 0;

  double sinalt, cosalt, sindelt, cosdelt;
  lin2ast(al1 / sett->oms, al2 / sett->oms, pm, sett->sepsm, sett->cepsm, &sinalt,
          &cosalt, &sindelt, &cosdelt);
  sgnlt[2] = asin(sindelt);
  sgnlt[3] = fmod(atan2(sinalt, cosalt) + 2. * M_PI, 2. * M_PI);
  double het0 = fmod(nn * M[8] + mm * M[12], M[0]);
  const int nyqst = (sett->nfft) / 2 + 1;

  double complex *xDatma = (double complex *)malloc(sizeof(double complex) * N * nifo);
  double complex *xDatmb = (double complex *)malloc(sizeof(double complex) * N * nifo);
  double *tmp1 = (double *)malloc(sizeof(double) * N * nifo);
  double *aa_t = (double *)malloc(sizeof(double) * N * nifo);
  double *bb_t = (double *)malloc(sizeof(double) * N * nifo);
  double *shft = (double *)malloc(sizeof(double) * N);
  double *shftf = (double *)malloc(sizeof(double) * N);
  double complex *xa = (double complex *)malloc(sizeof(double complex) * c->arr_len);
  double complex *xb = (double complex *)malloc(sizeof(double complex) * c->arr_len);

  /* jobcore.c:270-372: per-detector prelude */
  for (int n = 0; n < nifo; ++n) {
    const pa_detector *d = &c->det[n];
    double *aa = aa_t + (size_t)n * N, *bb = bb_t + (size_t)n * N;
    double complex *ma = xDatma + (size_t)n * N, *mb = xDatmb + (size_t)n * N;
    double *t1 = tmp1 + (size_t)n * N;
    modvir(sinalt, cosalt, sindelt, cosdelt, N, d, c->cosmodf, c->sinmodf, aa, bb);
    double nS0 = cosalt * cosdelt, nS1 = sinalt * cosdelt, nS2 = sindelt;
    const double *D = d->DetSSB;
    double shft1 = nS0 * D[0] + nS1 * D[1] + nS2 * D[2];
    for (int i = 0; i < N; ++i) {
      shft[i] = nS0 * D[i * 3] + nS1 * D[i * 3 + 1] + nS2 * D[i * 3 + 2];
      shftf[i] = shft[i] - shft1;
      t1[i] = c->t2[i] + (double)(2 * i) * shft[i];
    }
    for (int i = 0; i < N; ++i) {
      double phase = het0 * i + sett->oms * shft[i];
      double sp, cp;
      sincos(phase, &sp, &cp);
      double complex exph = cp - I * sp;
      ma[i] = d->xDat[i] * aa[i] * exph;
      mb[i] = d->xDat[i] * bb[i] * exph;
    }
    for (int i = 0; i < N; ++i) {
      xa[i] = ma[i];
      xb[i] = mb[i];
    }
    for (int i = N; i < sett->nfft; ++i) xa[i] = xb[i] = 0.;
    oracle_fft_exec(c->pl_int, xa, xa);
    oracle_fft_exec(c->pl_int, xb, xb);
    /* jobcore.c:338-352: keep [0, nyqst), move [nyqst, nfft) to the top of
     * the Ninterp array, zero the gap */
    const int shift = sett->Ninterp - sett->nfft;
    for (int i = nyqst + shift, j = nyqst; i < sett->Ninterp; ++i, ++j) {
      xa[i] = xa[j];
      xb[i] = xb[j];
    }
    for (int i = nyqst; i < nyqst + shift; ++i) xa[i] = xb[i] = 0.;
    oracle_fft_exec(c->pl_inv, xa, xa);
    oracle_fft_exec(c->pl_inv, xb, xb);
    double ft = (double)sett->interpftpad / sett->Ninterp;
    for (int i = 0; i < sett->Ninterp; ++i) {
      xa[i] *= ft;
      xb[i] *= ft;
    }
    splintpad(xa, shftf, N, sett->interpftpad, ma);
    splintpad(xb, shftf, N, sett->interpftpad, mb);
  }

  /* jobcore.c:375-393 */
  double aa = 0., bb = 0.;
  for (int n = 0; n < nifo; ++n) {
    double at = 0., bt = 0.;
    const double *an = aa_t + (size_t)n * N, *bn = bb_t + (size_t)n * N;
    for (int i = 0; i < N; ++i) {
      at += SQR(an[i]);
      bt += SQR(bn[i]);
    }
    double complex *ma = xDatma + (size_t)n * N, *mb = xDatmb + (size_t)n * N;
    for (int i = 0; i < N; ++i) {
      ma[i] /= c->det[n].sig2;
      mb[i] /= c->det[n].sig2;
    }
    aa += at / c->det[n].sig2;
    bb += bt / c->det[n].sig2;
  }
  if (pre_a) memcpy(pre_a, xDatma, sizeof(double complex) * N * nifo);
  if (pre_b) memcpy(pre_b, xDatmb, sizeof(double complex) * N * nifo);
  if (aa_out) *aa_out = aa;
  if (bb_out) *bb_out = bb;
  free(xa);
  free(xb);
  free(shft);
  free(shftf);
  free(aa_t);
  free(bb_t);

  int smin, smax;
  int nss = ora_spindown_range(sett, mm, nn, opts, s_range, &smin, &smax);

  /* per-spindown candidate lists, merged in ss order afterwards */
  ora_cand **cl = (ora_cand **)calloc(nss > 0 ? nss : 1, sizeof(ora_cand *));
  int *cn = (int *)calloc(nss > 0 ? nss : 1, sizeof(int));
  const int nbins = sett->nmax - sett->nmin;

#ifdef _OPENMP
  int nth = c->nthreads > 0 ? c->nthreads : omp_get_max_threads();
#pragma omp parallel num_threads(nth)
#endif
  {
    double complex *fxa = (double complex *)malloc(sizeof(double complex) * c->arr_len);
    double complex *fxb = (double complex *)malloc(sizeof(double complex) * c->arr_len);
    double *F = (double *)malloc(sizeof(double) * 2 * sett->nfft);
#ifdef _OPENMP
#pragma omp for schedule(static, 4)
#endif
    for (int k = 0; k < nss; ++k) {
      const int ss = smin + k;
      double s1 = opts->s0_flag ? 0. : ss * M[5] + nn * M[9] + mm * M[13];
      double het1 = fmod(ss * M[4], M[0]);
      if (het1 < 0) het1 += M[0];
      double sgnl0 = het0 + het1;
      /* jobcore.c:528-535 and 604-611 (GNUSINCOS form) */
      for (int n = 0; n < nifo; ++n) {
        const double complex *ma = xDatma + (size_t)n * N, *mb = xDatmb + (size_t)n * N;
        const double *t1 = tmp1 + (size_t)n * N;
        for (int i = N - 1; i != -1; --i) {
          double phase = het1 * i + s1 * t1[i];
          double sp, cp;
          sincos(phase, &sp, &cp);
          double complex exph = cp - I * sp;
          if (n == 0) {
            fxa[i] = ma[i] * exph;
            fxb[i] = mb[i] * exph;
          } else {
            fxa[i] += ma[i] * exph;
            fxb[i] += mb[i] * exph;
          }
        }
      }
      for (int i = sett->fftpad * sett->nfft - 1; i != N - 1; --i) fxa[i] = fxb[i] = 0.;
      oracle_fft_exec(c->plan, fxa, fxa);
      oracle_fft_exec(c->plan, fxb, fxb);
      for (int i = sett->nmin; i < sett->nmax; i++)
        F[i] = (SQR(creal(fxa[i])) + SQR(cimag(fxa[i]))) / aa +
               (SQR(creal(fxb[i])) + SQR(cimag(fxb[i]))) / bb;
      if (!(opts->white_flag)) fstat_norm(F + sett->nmin, nbins, PA_NAVFSTAT);
      if (F_out && ss == F_ss) memcpy(F_out, F + sett->nmin, sizeof(double) * nbins);
      /* jobcore.c:659-695 */
      int ncap = 0;
      ora_cand *list = NULL;
      for (int i = sett->nmin; i < sett->nmax; i++) {
        double Fc;
        if ((Fc = F[i]) > opts->trl) {
          int ii = i;
          while (++i < sett->nmax && F[i] > opts->trl) {
            if (F[i] >= Fc) {
              ii = i;
              Fc = F[i];
            }
          }
          double rec[PA_NPAR];
          rec[0] = 2. * M_PI * ii / ((double)sett->fftpad * sett->nfft) + sgnl0;
          rec[1] = s1;
          rec[2] = sgnlt[2];
          rec[3] = sgnlt[3];
          rec[4] = sqrt(2. * (Fc - sett->nd));
          int veto = 0;
          for (int q = 0; q < sett->numlines_band; q++)
            if (rec[0] >= sett->lines[2 * q] && rec[0] <= sett->lines[2 * q + 1]) {
              veto = 1;
              break;
            }
          if (!veto) {
            if (cn[k] == ncap) {
              ncap = ncap ? 2 * ncap : 16;
              list = (ora_cand *)realloc(list, sizeof(ora_cand) * ncap);
            }
            ora_cand *o = &list[cn[k]++];
            o->ss = ss;
            o->ii = ii;
            memcpy(o->rec, rec, sizeof(rec));
            o->F = Fc;
          }
        }
      }
      cl[k] = list;
    }
    free(fxa);
    free(fxb);
    free(F);
  }

  int total = 0;
  for (int k = 0; k < nss; k++) total += cn[k];
  int rc = 0;
  if (*sgnlc + total > cap) {
    if (needed) *needed = *sgnlc + total;
    rc = -1;
  } else {
    for (int k = 0; k < nss; k++)
      for (int q = 0; q < cn[k]; q++) {
        ora_cand *o = &cl[k][q];
        memcpy(sgnlv + (size_t)PA_NPAR * (*sgnlc), o->rec, sizeof(o->rec));
        if (idx) {
          pa_cand_idx *x = &idx[*sgnlc];
          x->pm = pm;
          x->mm = mm;
          x->nn = nn;
          x->ss = o->ss;
          x->ii = o->ii;
          x->F = (float)o->F;
        }
        (*sgnlc)++;
      }
    *FNum += nss;
  }
  for (int k = 0; k < nss; k++) free(cl[k]);
  free(cl);
  free(cn);
  free(xDatma);
  free(xDatmb);
  free(tmp1);
  return rc;
}

/* ------------------------------------------------------------------------
 * Followup: demodulated network F-statistic (followup/src/followup.c)
 * ------------------------------------------------------------------------ */

/* Sky set-up of one evaluation point (followup.c:986-1009): sin/cos of
 * alpha = sgnlo[3] and delta = sgnlo[2], the source unit vector, and
 * modvir() per detector into aa[n], bb[n]. */
static void fu_setup(const ora_ctx *c, const double *sgnlo, double nS[3],
                     double **aa, double **bb) {
  double sinalt = sin(sgnlo[3]), cosalt = cos(sgnlo[3]);
  double sindelt = sin(sgnlo[2]), cosdelt = cos(sgnlo[2]);
  nS[0] = cosalt * cosdelt;
  nS[1] = sinalt * cosdelt;
  nS[2] = sindelt;
  for (int n = 0; n < c->nifo; n++)
    modvir(sinalt, cosalt, sindelt, cosdelt, c->sett.N, &c->det[n], c->cosmodf,
           c->sinmodf, aa[n], bb[n]);
}

/* Fstatnet() (followup.c:413-535): matched filter of every detector at
 * (f, s, delta, alpha), phase f (i + shft) + s i^2 + (oms + 2 s i) shft
 * (:460-462), weights 1/sig2 (:496-506), out[0..3] amplitude estimates,
 * out[4] SNR sqrt(2(F-2)), out[5] = -F, out[6..9] the point, out[10] SNR
 * from the amplitudes.  cos/sin per sample as the reference's vector calls
 * (:467-470) with the C library's cos and sin. */
void ora_fstatnet(ora_ctx *c, const double sgnlo[4], double out[11]) {
  const int N = c->sett.N, nifo = c->nifo;
  double nS[3];
  double *aa[PA_MAX_DETECTORS], *bb[PA_MAX_DETECTORS];
  double complex *xa[PA_MAX_DETECTORS], *xb[PA_MAX_DETECTORS];
  for (int n = 0; n < nifo; n++) {
    aa[n] = (double *)malloc(sizeof(double) * N);
    bb[n] = (double *)malloc(sizeof(double) * N);
    xa[n] = (double complex *)malloc(sizeof(double complex) * N);
    xb[n] = (double complex *)malloc(sizeof(double complex) * N);
  }
  fu_setup(c, sgnlo, nS, aa, bb);
  double *phase = (double *)malloc(sizeof(double) * N);
  double *cph = (double *)malloc(sizeof(double) * N);
  double *sph = (double *)malloc(sizeof(double) * N);
  double complex xasum = 0, xbsum = 0;
  double sa = 0., sb = 0.;
  const double oms = c->sett.oms;
  for (int n = 0; n < nifo; n++) {
    const double *R = c->DetSSB[n];
    for (int i = 0; i < N; i++) {
      double shft = nS[0] * R[i * 3] + nS[1] * R[i * 3 + 1] + nS[2] * R[i * 3 + 2];
      phase[i] = sgnlo[0] * (double)(i + shft) + (sgnlo[1] * i * i) +
                 ((oms + 2. * sgnlo[1] * i) * shft);
    }
    for (int i = 0; i < N; i++) {
      cph[i] = cos(phase[i]);
      sph[i] = sin(phase[i]);
    }
    for (int i = 0; i < N; i++) {
      double complex exph = cph[i] - I * sph[i];
      xa[n][i] = c->xDat[n][i] * aa[n][i] * exph;
      xb[n][i] = c->xDat[n][i] * bb[n][i] * exph;
    }
  }
  for (int n = 0; n < nifo; n++) {
    double at = 0., bt = 0.;
    const double sig2 = c->det[n].sig2;
    for (int i = 0; i < N; i++) {
      at += SQR(aa[n][i]);
      bt += SQR(bb[n][i]);
    }
    for (int i = 0; i < N; i++) {
      xa[n][i] /= sig2;
      xb[n][i] /= sig2;
      xasum += xa[n][i];
      xbsum += xb[n][i];
    }
    sa += at / sig2;
    sb += bt / sig2;
  }
  out[5] = -(((SQR(creal(xasum)) + SQR(cimag(xasum))) / sa) +
             ((SQR(creal(xbsum)) + SQR(cimag(xbsum))) / sb));
  out[0] = 2 * creal(xasum) / sa;
  out[1] = 2 * creal(xbsum) / sb;
  out[2] = -2 * cimag(xasum) / sa;
  out[3] = -2 * cimag(xbsum) / sb;
  out[4] = sqrt(2 * (-out[5] - 2));
  for (int j = 0; j < 4; j++) out[6 + j] = sgnlo[j];
  out[10] = sqrt(SQR(2 * creal(xasum)) + SQR(2 * creal(xbsum)) +
                 SQR(2 * cimag(xasum)) + SQR(2 * cimag(xbsum)));
  for (int n = 0; n < nifo; n++) {
    free(aa[n]);
    free(bb[n]);
    free(xa[n]);
    free(xb[n]);
  }
  free(phase);
  free(cph);
  free(sph);
}

/* F = -out[5] of ora_fstatnet() and its gradient with respect to
 * (f, s, delta, alpha) in FP64, by forward differentiation of every factor:
 *   X_a = sum w a e^{-i phi},  A = sum a^2/sig2  (w = xDat/sig2),
 *   dF = 2 Re(conj(X_a) dX_a)/A - |X_a|^2 dA/A^2 + (same for b),
 *   dX_a = sum w (da - i a dphi) e^{-i phi},
 *   dphi/df = i + shft, dphi/ds = i^2 + 2 i shft,
 *   dphi/d(delta, alpha) = (f + oms + 2 s i) dshft/d(delta, alpha),
 * with a, b and their sky derivatives from the modvir() formula
 * (settings.c:281-325).  The reference gradient of the adjoint tests. */
double ora_fstatnet_grad(ora_ctx *c, const double sgnlo[4], double grad[4]) {
  const int N = c->sett.N;
  const double f = sgnlo[0], s = sgnlo[1], oms = c->sett.oms;
  const double sd = sin(sgnlo[2]), cd = cos(sgnlo[2]);
  const double sa_ = sin(sgnlo[3]), ca_ = cos(sgnlo[3]);
  const double nS[3] = {ca_ * cd, sa_ * cd, sd};
  const double nD[3] = {-ca_ * sd, -sa_ * sd, cd};      /* d nS / d delta */
  const double nA[3] = {-sa_ * cd, ca_ * cd, 0.};       /* d nS / d alpha */
  double complex Xa = 0, Xb = 0, dXa[4] = {0}, dXb[4] = {0};
  double A = 0, B = 0, dA[4] = {0}, dB[4] = {0};
  for (int n = 0; n < c->nifo; n++) {
    const pa_detector *d = &c->det[n];
    const double *k = d->amod;
    const double *R = c->DetSSB[n];
    const double is2 = 1. / d->sig2;
    const double cosalfr = ca_ * d->cphir + sa_ * d->sphir;
    const double sinalfr = sa_ * d->cphir - ca_ * d->sphir;
    const double c2d = cd * cd, c2sd = sd * cd;
    const double dc2d = -2. * sd * cd, dc2sd = cd * cd - sd * sd;
    for (int i = 0; i < N; i++) {
      const double cm = c->cosmodf[i], sm = c->sinmodf[i];
      const double cc = cosalfr * cm + sinalfr * sm;
      const double ss = sinalfr * cm - cosalfr * sm;
      /* d cc/d alpha = -ss, d ss/d alpha = cc */
      const double c2s = 2. * cc * cc, cs = cc * ss;
      const double a = k[0] * (2. - c2d) * c2s + k[1] * (2. - c2d) * 2. * cs + k[2] * c2sd * cc +
                       k[3] * c2sd * ss - k[0] * (2. - c2d) + k[4] * c2d;
      const double b = k[5] * sd * c2s + k[6] * sd * 2. * cs + k[7] * cd * cc + k[8] * cd * ss -
                       k[5] * sd;
      const double a_al = k[0] * (2. - c2d) * (-4. * cs) + k[1] * (2. - c2d) * 2. * (cc * cc - ss * ss) +
                          k[2] * c2sd * (-ss) + k[3] * c2sd * cc;
      const double a_de = (-k[0] * c2s - 2. * k[1] * cs + k[0] + k[4]) * dc2d +
                          (k[2] * cc + k[3] * ss) * dc2sd;
      const double b_al = k[5] * sd * (-4. * cs) + k[6] * sd * 2. * (cc * cc - ss * ss) +
                          k[7] * cd * (-ss) + k[8] * cd * cc;
      const double b_de = cd * (k[5] * c2s + 2. * k[6] * cs - k[5]) - sd * (k[7] * cc + k[8] * ss);
      const double r0 = R[3 * i], r1 = R[3 * i + 1], r2 = R[3 * i + 2];
      const double shft = nS[0] * r0 + nS[1] * r1 + nS[2] * r2;
      const double sh_de = nD[0] * r0 + nD[1] * r1 + nD[2] * r2;
      const double sh_al = nA[0] * r0 + nA[1] * r1;
      const double di = (double)i;
      const double phi = f * (di + shft) + s * di * di + (oms + 2. * s * di) * shft;
      const double om = f + oms + 2. * s * di;
      const double dphi[4] = {di + shft, di * di + 2. * di * shft, om * sh_de, om * sh_al};
      const double da[4] = {0., 0., a_de, a_al}, db[4] = {0., 0., b_de, b_al};
      const double complex E = cos(phi) - I * sin(phi);
      const double w = c->xDat[n][i] * is2;
      Xa += w * a * E;
      Xb += w * b * E;
      A += a * a * is2;
      B += b * b * is2;
      for (int j = 0; j < 4; j++) {
        dXa[j] += w * (da[j] - I * a * dphi[j]) * E;
        dXb[j] += w * (db[j] - I * b * dphi[j]) * E;
        dA[j] += 2. * a * da[j] * is2;
        dB[j] += 2. * b * db[j] * is2;
      }
    }
  }
  const double Pa = SQR(creal(Xa)) + SQR(cimag(Xa)), Pb = SQR(creal(Xb)) + SQR(cimag(Xb));
  for (int j = 0; j < 4; j++)
    grad[j] = 2. * creal(conj(Xa) * dXa[j]) / A - Pa * dA[j] / (A * A) +
              2. * creal(conj(Xb) * dXb[j]) / B - Pb * dB[j] / (B * B);
  return Pa / A + Pb / B;
}

/* simplex_extremes() (followup.c:1011-1040) on fx[.][5] = -F. */
static void fu_extremes(double fx[5][11], int dim, int *ihi, int *ilo, int *inhi) {
  int hi, lo, nhi;
  if (fx[0][5] > fx[1][5]) {
    hi = 0;
    lo = nhi = 1;
  } else {
    hi = 1;
    lo = nhi = 0;
  }
  for (int i = 2; i < dim + 1; i++) {
    if (fx[i][5] <= fx[lo][5]) lo = i;
    else if (fx[i][5] > fx[hi][5]) {
      nhi = hi;
      hi = i;
    } else if (fx[i][5] > fx[nhi][5]) nhi = i;
  }
  *ihi = hi;
  *ilo = lo;
  *inhi = nhi;
}

/* update_simplex() (followup.c:1055-1087): the point midpoint + scale*line
 * replaces the worst vertex when it is better than fmax. */
static int fu_update(ora_ctx *c, double sx[5][4], double fx[5][11], int dim, double fmax,
                     int ihi, const double *mid, const double *line, double scale, int *nev) {
  double next[4], f2[11];
  for (int i = 0; i < dim; i++) next[i] = mid[i] + scale * line[i];
  ora_fstatnet(c, next, f2);
  (*nev)++;
  if (f2[5] < fmax) {
    for (int i = 0; i < dim; i++) sx[ihi][i] = next[i];
    for (int j = 0; j < 11; j++) fx[ihi][j] = f2[j];
    return 1;
  }
  return 0;
}

/* amoeba() (followup.c:1126-1174) with make_simplex (:971-984),
 * evaluate_simplex (:986-1009), simplex_bearings (:1042-1053),
 * contract_simplex (:1089-1118) and check_tol (:1120-1124, ZEPS 1e-14,
 * followup.c:71).  The reference loops until check_tol holds; max_evals
 * (when > 0) bounds the evaluations.  Returns the number of evaluations;
 * point[] and out[] receive the best vertex. */
int ora_amoeba(ora_ctx *c, double point[4], const double pc2[4], double tol, int max_evals,
               double out[11]) {
  const int dim = 4;
  double sx[5][4], fx[5][11], mid[4], line[4];
  int nev = 0, ihi, ilo, inhi;
  for (int i = 0; i < dim + 1; i++)
    for (int j = 0; j < dim; j++) sx[i][j] = point[j];
  for (int i = 0; i < dim; i++) sx[i][i] = sx[i][i] + pc2[i];
  for (int i = 0; i < dim + 1; i++, nev++) ora_fstatnet(c, sx[i], fx[i]);
  for (;;) {
    fu_extremes(fx, dim, &ihi, &ilo, &inhi);
    for (int j = 0; j < dim; j++) mid[j] = 0.0;
    for (int i = 0; i < dim + 1; i++)
      if (i != ihi)
        for (int j = 0; j < dim; j++) mid[j] += sx[i][j];
    for (int j = 0; j < dim; j++) {
      mid[j] /= dim;
      line[j] = sx[ihi][j] - mid[j];
    }
    {
      double fmax = fx[ihi][5], fmin = fx[ilo][5];
      if (fabs(fmax - fmin) < (fabs(fmax) + fabs(fmin)) * tol + 1e-14) break;
    }
    if (max_evals > 0 && nev >= max_evals) break;
    fu_update(c, sx, fx, dim, fx[ihi][5], ihi, mid, line, -1.0, &nev);
    if (fx[ihi][5] < fx[ilo][5]) {
      fu_update(c, sx, fx, dim, fx[ihi][5], ihi, mid, line, -2.0, &nev);
    } else if (fx[ihi][5] > fx[inhi][5]) {
      if (!fu_update(c, sx, fx, dim, fx[ihi][5], ihi, mid, line, 0.5, &nev)) {
        for (int i = 0; i < dim + 1; i++) {
          if (i != ilo) {
            for (int j = 0; j < dim; j++) sx[i][j] = (sx[ilo][j] + sx[i][j]) * 0.5;
            ora_fstatnet(c, sx[i], fx[i]);
            nev++;
          }
        }
      }
    }
  }
  for (int j = 0; j < dim; j++) point[j] = sx[ilo][j];
  for (int j = 0; j < 11; j++) out[j] = fx[ilo][j];
  return nev;
}
