/*
 * oracle/ref_followup_driver.c -- TEST INFRASTRUCTURE ONLY.
 *
 * Drives the UNMODIFIED reference followup program (followup/src/followup.c,
 * its settings.c and search/network/src-cpu/auxi.c, compiled from where they
 * lie by oracle/build_oracle.py into oracle/_ref/libfollowup_ref.so) through
 * its own functions:
 *   evaluate_simplex(dim = 0)  -- one point: sky set-up + modvir + Fstatnet
 *                                 (followup.c:986-1009, 413-535)
 *   amoeba()                   -- the simplex maximiser (followup.c:1126-1174)
 * with the globals (ifo[], Search_settings, Aux_arrays) filled from the same
 * plain pa_settings/pa_detector structs the product and the oracle take.
 * Used only to generate the followup golden fixtures in tests/golden.
 *
 * main() of followup.c is renamed at compile time; the set-up functions it
 * calls (option parsing, file reading, injection, clean-up) are not used
 * here and are defined below as stubs that stop the program.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "auxi.h"
#include "settings.h"
#include "struct.h"

#include "polgraw_gb300.h"

void evaluate_simplex(double **simplex, int dim, double **fx, Search_settings *sett,
                      Aux_arrays *aux, double *nS, double **sigaa_max, double **sigbb_max);
double *amoeba(Search_settings *sett, Aux_arrays *aux, double *point, double *nS,
               double *res_max, int dim, double tol, double *pc2, double **sigaa_max,
               double **sigbb_max);
extern long pa_yep_cos_calls;

static Search_settings S;
static Aux_arrays AUX;
static double *SA[MAX_DETECTORS], *SB[MAX_DETECTORS];

#define NOT_USED(name) \
  void name(void) { fprintf(stderr, #name " is not used by the driver\n"); abort(); }
NOT_USED(handle_opts)
NOT_USED(init_arrays)
NOT_USED(read_grid)
NOT_USED(add_signal)
NOT_USED(cleanup_followup)

/* Fills the reference's globals: settings (followup settings.c:17-60 fields
 * used by Fstatnet/modvir), per-detector data, and the cos/sin(omr i)
 * tables of init_arrays (followup init.c:464-475). */
int ref_fu_init(const pa_settings *s, const pa_detector *det, int nifo) {
  if (nifo < 1 || nifo > MAX_DETECTORS) return -1;
  memset(&S, 0, sizeof(S));
  S.fpo = s->fpo;
  S.dt = s->dt;
  S.B = s->B;
  S.oms = s->oms;
  S.omr = s->omr;
  S.N = s->N;
  S.nd = s->nd;
  S.nod = s->nod;
  S.nifo = nifo;
  S.sepsm = s->sepsm;
  S.cepsm = s->cepsm;
  const int N = s->N;
  for (int n = 0; n < nifo; n++) {
    ifo[n].sig.xDat = (double *)malloc(sizeof(double) * N);
    ifo[n].sig.DetSSB = (double *)malloc(sizeof(double) * 3 * N);
    memcpy(ifo[n].sig.xDat, det[n].xDat, sizeof(double) * N);
    memcpy(ifo[n].sig.DetSSB, det[n].DetSSB, sizeof(double) * 3 * N);
    ifo[n].sig.sig2 = det[n].sig2;
    ifo[n].sig.sphir = det[n].sphir;
    ifo[n].sig.cphir = det[n].cphir;
    Ampl_mod_coeff *a = &ifo[n].amod;
    a->c1 = det[n].amod[0];
    a->c2 = det[n].amod[1];
    a->c3 = det[n].amod[2];
    a->c4 = det[n].amod[3];
    a->c5 = det[n].amod[4];
    a->c6 = det[n].amod[5];
    a->c7 = det[n].amod[6];
    a->c8 = det[n].amod[7];
    a->c9 = det[n].amod[8];
    SA[n] = (double *)calloc(N, sizeof(double));
    SB[n] = (double *)calloc(N, sizeof(double));
  }
  AUX.t2 = (double *)calloc(N, sizeof(double));
  AUX.cosmodf = (double *)calloc(N, sizeof(double));
  AUX.sinmodf = (double *)calloc(N, sizeof(double));
  for (int i = 0; i < N; i++) {
    double omrt = (S.omr) * i;
    AUX.t2[i] = sqr((double)i);
    AUX.cosmodf[i] = cos(omrt);
    AUX.sinmodf[i] = sin(omrt);
  }
  return 0;
}

/* The reference's own evaluation of one point; out[11] = fstat_out. */
void ref_fu_fstatnet(const double sgnlo[4], double out[11]) {
  double p[4], row[11], nS[3];
  memcpy(p, sgnlo, sizeof(p));
  double *pt[1] = {p};
  double *fx[1] = {row};
  evaluate_simplex(pt, 0, fx, &S, &AUX, nS, SA, SB);
  memcpy(out, row, sizeof(row));
}

/* The reference simplex from point with initial steps pc2; returns the
 * number of F-statistic evaluations it made. */
long ref_fu_amoeba(double point[4], const double pc2[4], double tol, double out[11]) {
  double nS[3], res[11], steps[4];
  memcpy(steps, pc2, sizeof(steps));
  long c0 = pa_yep_cos_calls;
  double *r = amoeba(&S, &AUX, point, nS, res, 4, tol, steps, SA, SB);
  memcpy(out, r, 11 * sizeof(double));
  return (pa_yep_cos_calls - c0) / (S.nifo > 0 ? S.nifo : 1);
}
