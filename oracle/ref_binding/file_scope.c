/* GB300 job_core: declarations added to jobcore.c after its includes */
#include <stddef.h>
#include <stdlib.h>
#include "polgraw_gb300.h"

/* the library's structs follow the reference's field for field */
_Static_assert(sizeof(pa_range) == sizeof(Search_range), "pa_range size");
_Static_assert(offsetof(pa_range, pmr) == offsetof(Search_range, pmr) &&
               offsetof(pa_range, mr) == offsetof(Search_range, mr) &&
               offsetof(pa_range, nr) == offsetof(Search_range, nr) &&
               offsetof(pa_range, spndr) == offsetof(Search_range, spndr) &&
               offsetof(pa_range, pst) == offsetof(Search_range, pst) &&
               offsetof(pa_range, mst) == offsetof(Search_range, mst) &&
               offsetof(pa_range, nst) == offsetof(Search_range, nst) &&
               offsetof(pa_range, sst) == offsetof(Search_range, sst), "pa_range offsets");
_Static_assert(sizeof(FLOAT_TYPE) == sizeof(double), "trigger records are doubles");
_Static_assert(NPAR == PA_NPAR, "values per trigger record");
_Static_assert(sizeof(((Detector_settings *)0)->amod) == sizeof(((pa_detector *)0)->amod), "amod c1..c9");
_Static_assert(sizeof(((Search_settings *)0)->lines[0]) == 2 * sizeof(double), "line veto pairs");

static pa_ctx *pa_context;    /* created at the first sky point */
static int pa_sgnlv_cap;      /* candidates sgnlv holds */

static pa_ctx *make_ctx(Search_settings *sett) {
  pa_settings s;
  memset(&s, 0, sizeof(s));
  s.fpo = sett->fpo; s.dt = sett->dt; s.B = sett->B; s.oms = sett->oms; s.omr = sett->omr;
  s.Smin = sett->Smin; s.Smax = sett->Smax; s.sepsm = sett->sepsm; s.cepsm = sett->cepsm;
  s.nfft = sett->nfft; s.nod = sett->nod; s.N = sett->N; s.nfftf = sett->nfftf;
  s.nmax = sett->nmax; s.nmin = sett->nmin; s.s = sett->s; s.nd = sett->nd;
  s.interpftpad = sett->interpftpad; s.fftpad = sett->fftpad; s.Ninterp = sett->Ninterp;
  s.nifo = sett->nifo;
  memcpy(s.M, sett->M, sizeof(s.M));          /* 16 doubles, column-major */
  s.numlines_band = sett->numlines_band;
  s.lines = &sett->lines[0][0];
  pa_detector det[MAX_DETECTORS];
  for (int n = 0; n < sett->nifo; n++) {
    det[n].xDat = ifo[n].sig.xDat;              /* after add_signal() */
    det[n].DetSSB = ifo[n].sig.DetSSB;
    det[n].sig2 = ifo[n].sig.sig2;
    det[n].sphir = ifo[n].sig.sphir;
    det[n].cphir = ifo[n].sig.cphir;
    memcpy(det[n].amod, &ifo[n].amod, sizeof(det[n].amod));
  }
  pa_config cfg = { PA_PREC_MIXED, PA_PHASE_FIXED, 0, 0 };
  int st = 0;
  pa_ctx *ctx = pa_create(&s, det, sett->nifo, &cfg, &st);
  if (!ctx) {
    fprintf(stderr, "pa_create: %s\n", pa_last_error(NULL));
    exit(EXIT_FAILURE);
  }
  pa_sgnlv_cap = 2 * sett->nfft;                /* sgnlv holds NPAR*2*nfft values (jobcore.c:82) */
  return ctx;
}
