/*
 * oracle/oracle_coinc.c -- CPU restatement of the coincidence step that
 * consumes the search's trigger files: read_trigger_files() of
 * coincidences/src/coincidences.c:117-600 and the transformation matrix of
 * manage_grid_matrix() (search/network/src-cpu/init.c:1142-1210).
 *
 * TEST INFRASTRUCTURE ONLY: the parity reference of pa_coinc_* (only tests/ and
 * bench.py's CPU leg load it).  Plain sequential C, FP64 without FMA
 * contraction (built with -ffp-contract=off), so that every cell index and
 * every mean is the value the reference computes on x86-64.
 *
 * The reference's observable quirks are kept, because its output files
 * depend on them:
 *  - the duplicate scan of a frame compares its last sorted row with the row
 *    that the candidate table holds one position further, which is left over
 *    from an earlier frame (or zero: the table starts calloc'ed,
 *    coincidences.c:130-132); when they are equal the frame's last run is
 *    not written (coincidences.c:343-352);
 *  - the index of the highest-SNR duplicate doubles as the "run in progress"
 *    flag, so a run whose best member is the frame's first in-band record
 *    (index 0) is resolved as if no maximum had been recorded
 *    (coincidences.c:355-412);
 *  - the coincidence table is filled from row 1 (coindx is incremented when
 *    a run reaches mincoin, before the run's end is stored) and the last run
 *    of the sorted table is counted but never stored, so it is written as a
 *    record of multiplicity 0 (coincidences.c:455-541);
 *  - sorts are glibc qsort() on row pointers, a stable merge sort at these
 *    sizes; ties keep their input order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"
#include "shim/gsl/pa_gsl_shim.h"

struct ora_coinc {
  int nframes;
  int frameinfo[256][3];
  long long raw, inband, unique;
  int *cells;            /* [inband][4], read order */
  unsigned char *keep;   /* [inband] */
  pa_coinc_rec *recs;
  int nrecs;
  int *fra, *ops;
  long long nmembers;
  int maxcoin, maxcoin_index;
};

/* manage_grid_matrix(), init.c:1185-1210: eigen decomposition by GSL's
 * gsl_eigen_symmv (here the shim's), vedva[i][j] = eigvec[i][j] sqrt(eigval[j]). */
int ora_coinc_vedva(const double *fisher, double *vedva) {
  double m[16];
  memcpy(m, fisher, sizeof(m));
  gsl_matrix_view mv = gsl_matrix_view_array(m, 4, 4);
  gsl_vector *eval = gsl_vector_alloc(4);
  gsl_matrix *evec = gsl_matrix_alloc(4, 4);
  gsl_eigen_symmv_workspace *w = gsl_eigen_symmv_alloc(4);
  gsl_eigen_symmv(&mv.matrix, eval, evec, w);
  gsl_eigen_symmv_free(w);
  double eigval[4], eigvec[4][4];
  for (int i = 0; i < 4; i++) {
    eigval[i] = gsl_vector_get(eval, i);
    gsl_vector_view col = gsl_matrix_column(evec, i);
    for (int j = 0; j < 4; j++) eigvec[j][i] = gsl_vector_get(&col.vector, j);
  }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) vedva[4 * i + j] = eigvec[i][j] * sqrt(eigval[j]);
  gsl_vector_free(eval);
  gsl_matrix_free(evec);
  return 0;
}

/* ---- stable merge sort of row indices ---------------------------------- */

typedef int (*ora_cmp)(const void *ctx, int a, int b); /* <0: a before b */

static void msort_rec(int *v, int *tmp, int n, ora_cmp cmp, const void *ctx) {
  if (n < 2) return;
  int h = n / 2;
  msort_rec(v, tmp, h, cmp, ctx);
  msort_rec(v + h, tmp, n - h, cmp, ctx);
  int i = 0, j = h, k = 0;
  while (i < h && j < n) tmp[k++] = (cmp(ctx, v[j], v[i]) < 0) ? v[j++] : v[i++];
  while (i < h) tmp[k++] = v[i++];
  while (j < n) tmp[k++] = v[j++];
  memcpy(v, tmp, sizeof(int) * n);
}

static void stable_sort(int *v, int n, ora_cmp cmp, const void *ctx) {
  int *tmp = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  msort_rec(v, tmp, n, cmp, ctx);
  free(tmp);
}

/* way2compare_4c (coincidences.c:72-85): descending on the four cells */
static int cmp_cells_desc(const void *ctx, int a, int b) {
  const int *c = (const int *)ctx;
  for (int j = 0; j < 4; j++) {
    int d = c[4 * b + j] - c[4 * a + j];
    if (d) return d;
  }
  return 0;
}

/* way2compare_c1 (coincidences.c:87-94): descending multiplicity */
static int cmp_weight_desc(const void *ctx, int a, int b) {
  const int *w = (const int *)ctx;
  return w[b] - w[a];
}

static int same4(const int *x, const int *y) {
  return x[0] == y[0] && x[1] == y[1] && x[2] == y[2] && x[3] == y[3];
}

ora_coinc *ora_coinc_run(const pa_coinc_cfg *cfg, int nframes, const int *frames,
                         const double *const *recs, const long long *nrec,
                         pa_coinc_summary *sum) {
  if (!cfg || nframes < 0 || nframes > 255 || cfg->mincoin < 1) return NULL;
  ora_coinc *o = (ora_coinc *)calloc(1, sizeof(*o));
  o->nframes = nframes;
  const double N = (double)cfg->N;
  const double sqrN = pow(cfg->N, 2);           /* coincidences.c:187 */
  const double omsN = cfg->oms * cfg->N;        /* coincidences.c:188 */
  const double lo = M_PI_2 - cfg->narrowdown, hi = M_PI_2 + cfg->narrowdown;
  double v[4][4];                               /* coincidences.c:182-184 */
  for (int j = 0; j < 4; j++)
    for (int i = 0; i < 4; i++) v[i][j] = cfg->vedva[i][j] / cfg->scale[j];
  const double se = sin(PA_C_EPSMA), ce = cos(PA_C_EPSMA);

  long long total = 0;
  for (int f = 0; f < nframes; f++) total += nrec[f];
  o->raw = total;
  int *cells = (int *)malloc(sizeof(int) * 4 * (total > 0 ? total : 1));
  double *cf = (double *)malloc(sizeof(double) * 5 * (total > 0 ? total : 1));
  int *orgpos = (int *)malloc(sizeof(int) * (total > 0 ? total : 1));
  unsigned char *keep = (unsigned char *)calloc(total > 0 ? total : 1, 1);
  /* survivors (allcandi / allcandf): index into the in-band arrays */
  int *surv = (int *)malloc(sizeof(int) * (total > 0 ? total : 1));
  int *sframe = (int *)malloc(sizeof(int) * (total > 0 ? total : 1));
  long long nin = 0, nsurv = 0;
  /* the candidate table's rows left over from earlier frames */
  int *persist = NULL;
  long long plen = 0;

  for (int f = 0; f < nframes; f++) {
    const long long base = nin;
    const double *r = recs[f];
    /* coincidences.c:229-270: band, frame shift, SNR cut, cells */
    for (long long p = 0; p < nrec[f]; p++) {
      double c[5];
      memcpy(c, r + 5 * p, sizeof(c));
      if (!((c[0] > lo) && (c[0] < hi))) continue;
      c[0] = c[0] + 2. * c[1] * (cfg->N) * (cfg->refr - frames[f]);
      if (!(((c[0] > 0) && (c[0] < M_PI)) && (c[4] > cfg->snrcutoff))) continue;
      double tmp[4];
      tmp[0] = c[0] * N;
      tmp[1] = c[1] * sqrN;
      /* ast2lin (auxi.c:26-35) with epsm = C_EPSMA */
      const double be0 = ce * sin(c[3]) * cos(c[2]) + se * sin(c[2]);
      const double be1 = cos(c[3]) * cos(c[2]);
      tmp[2] = omsN * be0;
      tmp[3] = omsN * be1;
      for (int j = 0; j < 4; j++)
        cells[4 * nin + j] = (int)round(tmp[0] * v[0][j] + tmp[1] * v[1][j] + tmp[2] * v[2][j] +
                                        tmp[3] * v[3][j] + 0.5 * cfg->shift[j]);
      memcpy(cf + 5 * nin, c, sizeof(c));
      orgpos[nin] = (int)p;
      nin++;
    }
    const int n = (int)(nin - base);
    o->frameinfo[f][0] = frames[f];
    o->frameinfo[f][1] = n;
    /* coincidences.c:315: sort the frame's rows */
    int *ord = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
    for (int i = 0; i < n; i++) ord[i] = i;
    stable_sort(ord, n, cmp_cells_desc, cells + 4 * base);
    /* the row one past the frame's last: left over or zero */
    int stale[4] = {0, 0, 0, 0};
    if (n < plen) memcpy(stale, persist + 4 * (long long)n, sizeof(stale));
    /* coincidences.c:317-413: runs of equal cells, best SNR kept */
    const double *snr = cf + 5 * base + 4;
    int maxsnridx = 0, maxi = 0, good = 0;
    double candsnr = 0;
    for (int i = 0; i < n; i++) {
      const int *ci = cells + 4 * (base + ord[i]);
      const int *cn = (i + 1 < n) ? cells + 4 * (base + ord[i + 1]) : stale;
      const int idx = ord[i];
      if (!same4(ci, cn)) {
        int k = i, kidx = idx;
        if (maxsnridx) { k = maxi; kidx = maxsnridx; }
        (void)k; /* candi[k] and candf[kidx] are the same record */
        keep[base + kidx] = 1;
        surv[nsurv] = (int)(base + kidx);
        sframe[nsurv] = frames[f];
        nsurv++;
        good++;
        maxsnridx = 0;
      } else {
        const int idx1 = (i + 1 < n) ? ord[i + 1] : -1;
        /* a stale neighbour continues the run to the frame's end: nothing
         * more is written, whichever SNR it would compare */
        if (idx1 < 0) break;
        if (!maxsnridx) {
          maxsnridx = (snr[5 * idx] > snr[5 * idx1]) ? idx : idx1;
          maxi = (snr[5 * idx] > snr[5 * idx1]) ? i : i + 1;
          candsnr = snr[5 * maxsnridx];
        } else {
          if (snr[5 * idx] > candsnr) {
            maxsnridx = idx; maxi = i; candsnr = snr[5 * idx];
          } else if (snr[5 * idx1] > candsnr) {
            maxsnridx = idx1; maxi = i + 1; candsnr = snr[5 * idx1];
          }
        }
      }
    }
    o->frameinfo[f][2] = good;
    /* the frame's sorted rows now occupy positions 0 .. n-1 of the table */
    if (n > plen) {
      persist = (int *)realloc(persist, sizeof(int) * 4 * (size_t)n);
      plen = n;
    }
    for (int i = 0; i < n; i++) memcpy(persist + 4 * (long long)i, cells + 4 * (base + ord[i]), sizeof(int) * 4);
    free(ord);
  }
  o->inband = nin;
  o->unique = nsurv;

  /* coincidences.c:445-447: global sort of the survivors */
  const int G = (int)nsurv;
  int *gord = (int *)malloc(sizeof(int) * (G > 0 ? G : 1));
  int *gcells = (int *)malloc(sizeof(int) * 4 * (G > 0 ? G : 1));
  for (int i = 0; i < G; i++) {
    gord[i] = i;
    memcpy(gcells + 4 * i, cells + 4 * (long long)surv[i], sizeof(int) * 4);
  }
  stable_sort(gord, G, cmp_cells_desc, gcells);

  /* coincidences.c:449-486: runs of equal cells; imtr rows from index 1 */
  int numc = cfg->mincoin > 0 ? G / cfg->mincoin : 0;
  int tab = numc > G + 1 ? numc : G + 1; /* room for every store */
  int *im_end = (int *)calloc(tab, sizeof(int)), *im_w = (int *)calloc(tab, sizeof(int));
  int coindx = 0, weight = 1, hi_used = 0;
  for (int i = 0; i < G - 1; i++) {
    if (same4(gcells + 4 * gord[i], gcells + 4 * gord[i + 1])) {
      weight++;
      if (weight == cfg->mincoin) coindx++;
    } else {
      if (weight >= cfg->mincoin) {
        im_end[coindx] = i;
        im_w[coindx] = weight;
        if (coindx + 1 > hi_used) hi_used = coindx + 1;
      }
      weight = 1;
    }
  }
  int rows = numc > hi_used ? numc : hi_used;
  int *qord = (int *)malloc(sizeof(int) * (rows > 0 ? rows : 1));
  for (int q = 0; q < rows; q++) qord[q] = q;
  stable_sort(qord, rows, cmp_weight_desc, im_w);

  /* coincidences.c:488-541: the records */
  o->nrecs = coindx;
  o->recs = (pa_coinc_rec *)calloc(coindx > 0 ? coindx : 1, sizeof(pa_coinc_rec));
  long long nm = 0;
  for (int q = 0; q < coindx; q++) nm += im_w[qord[q]];
  o->nmembers = nm;
  o->fra = (int *)malloc(sizeof(int) * (nm > 0 ? nm : 1));
  o->ops = (int *)malloc(sizeof(int) * (nm > 0 ? nm : 1));
  o->maxcoin = rows > 0 ? im_w[qord[0]] : 0;
  o->maxcoin_index = 0;
  double maxsnr = 0;
  long long m = 0;
  for (int q = 0; q < coindx; q++) {
    const int j = im_end[qord[q]], w = im_w[qord[q]];
    double mean[5] = {0, 0, 0, 0, 0};
    o->recs[q].w = w;
    o->recs[q].first = (int)m;
    for (int i = 0; i < w; i++) {
      const int s = gord[j - i];
      const double *c = cf + 5 * (long long)surv[s];
      for (int l = 0; l < 4; l++) mean[l] += c[l];
      mean[4] += c[4] * c[4];
      o->ops[m] = orgpos[surv[s]];
      o->fra[m] = sframe[s];
      m++;
    }
    for (int l = 0; l < 4; l++) mean[l] /= w;
    mean[4] = sqrt(mean[4]);
    memcpy(o->recs[q].mean, mean, sizeof(mean));
    if (!q) maxsnr = mean[4];
    if (w == o->maxcoin && mean[4] > maxsnr) {
      maxsnr = mean[4];
      o->maxcoin_index = q;
    }
  }
  o->cells = cells;
  o->keep = keep;
  free(cf);
  free(orgpos);
  free(surv);
  free(sframe);
  free(persist);
  free(gord);
  free(gcells);
  free(im_end);
  free(im_w);
  free(qord);
  if (sum) {
    memset(sum, 0, sizeof(*sum));
    sum->nframes = nframes;
    sum->raw = o->raw;
    sum->inband = o->inband;
    sum->unique = o->unique;
    sum->ncoin = o->nrecs;
    sum->nmembers = o->nmembers;
    sum->maxcoin = o->maxcoin;
    sum->maxcoin_index = o->maxcoin_index;
  }
  return o;
}

int ora_coinc_get(const ora_coinc *o, int *frameinfo, pa_coinc_rec *recs, int *fra, int *ops) {
  if (frameinfo) memcpy(frameinfo, o->frameinfo, sizeof(int) * 3 * o->nframes);
  if (recs) memcpy(recs, o->recs, sizeof(pa_coinc_rec) * o->nrecs);
  if (fra) memcpy(fra, o->fra, sizeof(int) * o->nmembers);
  if (ops) memcpy(ops, o->ops, sizeof(int) * o->nmembers);
  return 0;
}

int ora_coinc_cells(const ora_coinc *o, int *cells, unsigned char *keep) {
  if (cells) memcpy(cells, o->cells, sizeof(int) * 4 * o->inband);
  if (keep) memcpy(keep, o->keep, o->inband);
  return 0;
}

void ora_coinc_free(ora_coinc *o) {
  if (!o) return;
  free(o->cells);
  free(o->keep);
  free(o->recs);
  free(o->fra);
  free(o->ops);
  free(o);
}
