/*
 * pa_host.c -- host side of the GB300 drop-in network search (set-up and
 * sky loop around job_core).  See include/polgraw_gb300_host.h for the list
 * of reference functions each part stands in for.
 *
 * Deliberate differences from the reference host:
 *  - detectors are taken in sorted name order instead of readdir() order
 *    (settings.c:108-156), so runs are reproducible across filesystems; the
 *    order only changes the rounding of the detector sum;
 *  - errors return codes instead of calling exit() inside library code;
 *  - the candidate buffer grows instead of overflowing when one sky point
 *    yields more than its remaining capacity (jobcore.c:82 allocates
 *    2*nfft records and never checks);
 *  - an empty state file means "nothing to do" (the reference then runs
 *    with uninitialised loop starts, init.c:888-895).
 */
#define _GNU_SOURCE
#include "../../include/polgraw_gb300_host.h"

#include <dirent.h>
#include <errno.h>
#include <fcntl.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>
#include <time.h>
#include <unistd.h>

#define SQR(x) ((x) * (x))
#define C_OMEGA_R 7.2921151467064e-5
#define C_SIDDAY (2. * M_PI / C_OMEGA_R)
#define RAD_TO_DEG (180 / M_PI)
#define C_EPSMA (84381.448 / 3600. / RAD_TO_DEG)
#define ROUND(x) floor((x) + 0.5)

typedef struct pa_cmdline {
  int white_flag, s0_flag, checkp_flag, veto_flag, help_flag;
  int ident, band, hemi, nod;
  double trl, narrowdown;
  char prefix[512], dtaprefix[512], label[512], range[512], getrange[512],
      qname[512], usedet[32], addsig[512], wd[512];
  int precision, phase_mode, sbatch, skybatch, device, graphs;
} pa_cmdline;

typedef struct host_det {
  char name[3];
  char xdatname[1024];
  double ephi, elam, egam;
  double *xDat, *DetSSB, *aa, *bb;
  double phir, epsm, sphir, cphir, sepsm, cepsm, crf0, sig2;
  int Nzeros;
  double amod[9];
  double (*lines)[2];
  int numlines;
} host_det;

struct pa_host {
  pa_cmdline opts;
  pa_settings sett;
  double M[16];
  int nifo;
  host_det ifo[PA_MAX_DETECTORS];
  pa_detector det[PA_MAX_DETECTORS];
  double (*lines)[2]; /* band lines, PA_MAXL */
  double *cosmodf, *sinmodf, *t2;
  pa_range s_range;
  int FNum;
  int nothing_to_do;
};

/* ------------------------------------------------------------------ */
/* option parsing: init.c:28-281 */

static void print_help(void) {
  printf("polgraw-allsky periodic GWs: search for candidate signals with the F-statistic\n");
  printf("(GB300 implementation of the network search hot path)\n");
  printf("Usage: ./gwsearch-gb300 -[switch1] <value1> -[switch2] <value2> ...\n");
  printf("Switches are:\n\n");
  printf("-data         Data directory (default is .)\n");
  printf("-output       Output directory (default is ./candidates)\n");
  printf("-ident        Frame number\n");
  printf("-band         Band number\n");
  printf("-label        Custom label for the input and output files\n");
  printf("-range        Use file with grid range or pulsar position\n");
  printf("-getrange     Write grid ranges & exit (ignore -r)\n");
  printf("-cwd          Change to directory <dir>\n");
  printf("-threshold    Threshold for the F-statistic (default is 20)\n");
  printf("-hemisphere   Hemisphere (default is 0 - does both)\n");
  printf("-fpo          Reference band frequency fpo value\n");
  printf("-dt           Data sampling time dt (default value: 0.5)\n");
  printf("-usedet       Use only detectors from string (default is use all available)\n");
  printf("-addsig       Add signal with parameters from <file>\n");
  printf("-nod          Number of days\n");
  printf("-narrowdown   Narrow-down the frequency band (range [0, 0.5] +- around center)\n");
  printf("-precision    mixed (default) or fp64\n");
  printf("-phase        spindown phase form in the mixed precision: f64, fixed (default), ff\n");
  printf("-sbatch       spindowns per fused launch (default: automatic)\n");
  printf("-skybatch     sky points per batched call (default 1)\n");
  printf("-device       CUDA device ordinal (default 0)\n");
  printf("-graphs       1: capture each batch of sky points into a CUDA graph (default 0)\n\n");
  printf("Also:\n\n");
  printf("--whitenoise      White Gaussian noise assumed\n");
  printf("--nospindown      Spindowns neglected\n");
  printf("--nocheckpoint    State file won't be created (no checkpointing)\n");
  printf("--vetolines       Veto known lines from files in data directory\n");
  printf("--help            This help\n");
}

static int handle_opts(pa_host *h, int argc, char **argv) {
  pa_cmdline *o = &h->opts;
  pa_settings *s = &h->sett;
  memset(o, 0, sizeof(*o));
  o->trl = 20;
  strcpy(o->prefix, "./candidates");
  strcpy(o->dtaprefix, ".");
  s->fpo = -1;
  s->dt = 0.5;
  o->narrowdown = 0.5;
  s->nod = 0;
  o->precision = PA_PREC_MIXED;
  o->phase_mode = PA_PHASE_FIXED;
  o->skybatch = 1;
  int help_flag = 0, white_flag = 0, s0_flag = 0, checkp_flag = 1, veto_flag = 0;
  struct option long_options[] = {
      {"help", no_argument, &help_flag, 1},
      {"whitenoise", no_argument, &white_flag, 1},
      {"nospindown", no_argument, &s0_flag, 1},
      {"nocheckpoint", no_argument, &checkp_flag, 0},
      {"vetolines", no_argument, &veto_flag, 1},
      {"ident", required_argument, 0, 'i'},
      {"band", required_argument, 0, 'b'},
      {"output", required_argument, 0, 'o'},
      {"data", required_argument, 0, 'd'},
      {"label", required_argument, 0, 'l'},
      {"range", required_argument, 0, 'r'},
      {"getrange", required_argument, 0, 'g'},
      {"cwd", required_argument, 0, 'c'},
      {"threshold", required_argument, 0, 't'},
      {"hemisphere", required_argument, 0, 'h'},
      {"fpo", required_argument, 0, 'p'},
      {"addsig", required_argument, 0, 'x'},
      {"nod", required_argument, 0, 'y'},
      {"usedet", required_argument, 0, 'u'},
      {"dt", required_argument, 0, 's'},
      {"narrowdown", required_argument, 0, 'n'},
      {"precision", required_argument, 0, 1001},
      {"phase", required_argument, 0, 1002},
      {"sbatch", required_argument, 0, 1003},
      {"skybatch", required_argument, 0, 1004},
      {"device", required_argument, 0, 1005},
      {"graphs", required_argument, 0, 1006},
      {0, 0, 0, 0}};
  optind = 1;
  while (1) {
    int option_index = 0;
    int c = getopt_long_only(argc, argv, "i:b:o:d:l:r:g:c:t:h:p:x:y:s:u:n:",
                             long_options, &option_index);
    if (c == -1) break;
    switch (c) {
      case 'i': o->ident = atoi(optarg); break;
      case 't': o->trl = atof(optarg); break;
      case 'h': o->hemi = (int)atof(optarg); break;
      case 'b': o->band = atoi(optarg); break;
      case 'o': snprintf(o->prefix, sizeof o->prefix, "%s", optarg); break;
      case 'd': snprintf(o->dtaprefix, sizeof o->dtaprefix, "%s", optarg); break;
      case 'l':
        o->label[0] = '_';
        snprintf(o->label + 1, sizeof o->label - 1, "%s", optarg);
        break;
      case 'r': snprintf(o->range, sizeof o->range, "%s", optarg); break;
      case 'g': snprintf(o->getrange, sizeof o->getrange, "%s", optarg); break;
      case 'c': snprintf(o->wd, sizeof o->wd, "%s", optarg); break;
      case 'p': s->fpo = atof(optarg); break;
      case 'x': snprintf(o->addsig, sizeof o->addsig, "%s", optarg); break;
      case 'y': s->nod = atoi(optarg); break;
      case 's': s->dt = atof(optarg); break;
      case 'u': snprintf(o->usedet, sizeof o->usedet, "%s", optarg); break;
      case 'n': o->narrowdown = atof(optarg); break;
      case 1001:
        if (!strcmp(optarg, "fp64")) o->precision = PA_PREC_FP64;
        else if (!strcmp(optarg, "mixed")) o->precision = PA_PREC_MIXED;
        else { fprintf(stderr, "-precision must be mixed or fp64\n"); return PA_HOST_EXIT_FAILURE; }
        break;
      case 1002:
        if (!strcmp(optarg, "f64")) o->phase_mode = PA_PHASE_F64;
        else if (!strcmp(optarg, "fixed")) o->phase_mode = PA_PHASE_FIXED;
        else if (!strcmp(optarg, "ff")) o->phase_mode = PA_PHASE_FF;
        else { fprintf(stderr, "-phase must be f64, fixed or ff\n"); return PA_HOST_EXIT_FAILURE; }
        break;
      case 1003: o->sbatch = atoi(optarg); break;
      case 1004: o->skybatch = atoi(optarg) > 0 ? atoi(optarg) : 1; break;
      case 1005: o->device = atoi(optarg); break;
      case 1006: o->graphs = atoi(optarg) != 0; break;
      default: break;
    }
  }
  if (help_flag) {
    print_help();
    return PA_HOST_EXIT_SUCCESS;
  }
  if (!(s->nod)) {
    printf("Number of days not set... Exiting\n");
    return PA_HOST_EXIT_FAILURE;
  }
  printf("Number of days is %d\n", s->nod);
  o->narrowdown *= M_PI;
  o->white_flag = white_flag;
  o->s0_flag = s0_flag;
  o->checkp_flag = checkp_flag;
  o->veto_flag = veto_flag;
  printf("Input data directory is %s\n", o->dtaprefix);
  printf("Output directory is %s\n", o->prefix);
  printf("Frame and band numbers are %d and %d\n", o->ident, o->band);
  if (!(s->fpo >= 0)) s->fpo = 10. + 0.96875 * o->band * (0.5 / s->dt);
  printf("The reference frequency fpo is %f\n", s->fpo);
  printf("The data sampling time dt is %f\n", s->dt);
  if (o->white_flag) printf("Assuming white Gaussian noise\n");
  if (o->trl != 20) printf("Threshold for the F-statistic is %lf\n", o->trl);
  if (o->hemi) printf("Search for hemisphere %d\n", o->hemi);
  if (o->s0_flag) printf("Assuming s_1 = 0.\n");
  if (strlen(o->label)) printf("Using '%s' as data label\n", o->label);
  if (strlen(o->getrange)) {
    printf("Writing full grid ranges to '%s'\n", o->getrange);
    if (strlen(o->range)) {
      o->range[0] = '\0';
      printf("     WARNING! -r option will be ignored...\n");
    }
  }
  if (strlen(o->range)) printf("Obtaining grid range from '%s'\n", o->range);
  if (strlen(o->addsig)) printf("Adding signal from '%s'\n", o->addsig);
  if (o->wd[0]) {
    printf("Changing working directory to %s\n", o->wd);
    if (chdir(o->wd)) {
      perror(o->wd);
      return PA_HOST_EXIT_FAILURE;
    }
  }
  if (o->veto_flag) printf("Known lines will be vetoed (reading from files in the data directory)\n");
  return PA_HOST_OK;
}

/* ------------------------------------------------------------------ */
/* grid and settings: init.c:287-321, settings.c:16-81 */

static int read_grid(pa_host *h) {
  char filename[1200];
  pa_cmdline *o = &h->opts;
  if (strlen(o->usedet) == 2)
    snprintf(filename, sizeof filename, "%s/%03d/%s/grid.bin", o->dtaprefix, o->ident, o->usedet);
  else
    snprintf(filename, sizeof filename, "%s/%03d/grid.bin", o->dtaprefix, o->ident);
  FILE *data = fopen(filename, "r");
  if (!data) {
    perror(filename);
    return PA_HOST_EXIT_FAILURE;
  }
  printf("Using grid file from %s\n", filename);
  int fftpad = 0;
  if (fread(&fftpad, sizeof(int), 1, data) != 1 || fread(h->M, sizeof(double), 16, data) != 16) {
    fclose(data);
    fprintf(stderr, "%s: short grid file\n", filename);
    return PA_HOST_EXIT_FAILURE;
  }
  fclose(data);
  h->sett.fftpad = fftpad;
  printf("Using fftpad from the grid file: %d\n", fftpad);
  memcpy(h->sett.M, h->M, sizeof(h->M));
  return PA_HOST_OK;
}

static void search_settings(pa_settings *s) {
  double dt = s->dt;
  double B = 0.5 / dt;
  s->B = B;
  s->oms = 2. * M_PI * (s->fpo) * dt;
  s->omr = C_OMEGA_R * dt;
  s->N = (int)ROUND(s->nod * C_SIDDAY / dt);
  s->nfft = 1 << (int)ceil(log(s->N) / log(2.));
  s->s = 1;
  double fdotmin = 0.5e-8, fdotmax = 0.5e-9;
  s->Smax = 2. * M_PI * fdotmin * dt * dt;
  s->Smin = 2. * M_PI * fdotmax * dt * dt;
  s->nd = 2;
  s->interpftpad = 2;
  s->nmin = s->fftpad * PA_NAV * s->B;
  s->nmax = (s->nfft / 2 - PA_NAV * s->B) * s->fftpad;
  s->numlines_band = 0;
  s->Ninterp = s->interpftpad * s->nfft; /* plan_fftw, init.c:835 */
  s->nfftf = s->fftpad * s->nfft;        /* init.c:844 */
}

/* settings.c:92-246 */
static int cmp_names(const void *a, const void *b) { return strcmp((const char *)a, (const char *)b); }

static int detectors_settings(pa_host *h) {
  pa_cmdline *o = &h->opts;
  char dirname[1200];
  snprintf(dirname, sizeof dirname, "%s/%03d", o->dtaprefix, o->ident);
  char names[64][3];
  int nn = 0;
  DIR *dp = opendir(dirname);
  if (!dp) {
    perror("Couldn't open the input directory...");
    printf("No subdirectories with detector data found. Exiting...\n");
    return PA_HOST_EXIT_FAILURE;
  }
  struct dirent *ep;
  while ((ep = readdir(dp)) && nn < 64) {
    if (strlen(ep->d_name) != 2 || ep->d_name[0] == '.') continue;
    char p[1300];
    snprintf(p, sizeof p, "%s/%s", dirname, ep->d_name);
    struct stat st;
    if (stat(p, &st) || !S_ISDIR(st.st_mode)) continue;
    if (strlen(o->usedet) && !strstr(o->usedet, ep->d_name)) continue;
    memcpy(names[nn], ep->d_name, 3);
    nn++;
  }
  closedir(dp);
  qsort(names, nn, sizeof(names[0]), cmp_names);
  int nifo = 0;
  for (int k = 0; k < nn && nifo < PA_MAX_DETECTORS; k++) {
    char x[1400];
    snprintf(x, sizeof x, "%s/%03d/%s/xdatc_%03d_%04d%s.bin", o->dtaprefix, o->ident, names[k],
             o->ident, o->band, o->label);
    FILE *f = fopen(x, "r");
    if (!f) {
      printf("Directory %s exists, but no input file found:\n%s missing...\n", names[k], x);
      continue;
    }
    fclose(f);
    host_det *d = &h->ifo[nifo];
    memcpy(d->name, names[k], 3);
    snprintf(d->xdatname, sizeof d->xdatname, "%s", x);
    if (!strcmp("V1", d->name)) {
      d->ephi = (43. + 37. / 60. + 53.0880 / 3600.) / RAD_TO_DEG;
      d->elam = (10. + 30. / 60. + 16.1885 / 3600.) / RAD_TO_DEG;
      d->egam = (135. - (19.0 + 25. / 60.0 + 57.96 / 3600.)) / RAD_TO_DEG;
    } else if (!strcmp("H1", d->name)) {
      d->ephi = (46 + (27 + 18.528 / 60.) / 60.) / RAD_TO_DEG;
      d->elam = -(119 + (24 + 27.5657 / 60.) / 60.) / RAD_TO_DEG;
      d->egam = 170.9994 / RAD_TO_DEG;
    } else if (!strcmp("L1", d->name)) {
      d->ephi = (30 + (33 + 46.4196 / 60.) / 60.) / RAD_TO_DEG;
      d->elam = -(90 + (46 + 27.2654 / 60.) / 60.) / RAD_TO_DEG;
      d->egam = 242.7165 / RAD_TO_DEG;
    } else {
      printf("Meh, unknown detector %s (see settings.c) Exiting...\n", d->name);
      return PA_HOST_EXIT_FAILURE;
    }
    printf("Using %s IFO as detector #%d... %s as input time series data\n", d->name, nifo,
           d->xdatname);
    nifo++;
  }
  h->nifo = nifo;
  h->sett.nifo = nifo;
  if (!nifo) {
    printf("No subdirectories with detector data found. Exiting...\n");
    return PA_HOST_EXIT_FAILURE;
  }
  printf("Settings - number of detectors: %d\n", nifo);
  return PA_HOST_OK;
}

/* init.c:326-457 (the per-detector part; aux tables below) */
static int init_arrays(pa_host *h) {
  pa_settings *s = &h->sett;
  const int N = s->N;
  for (int i = 0; i < h->nifo; i++) {
    host_det *d = &h->ifo[i];
    d->xDat = (double *)calloc(N, sizeof(double));
    FILE *f = fopen(d->xdatname, "r");
    if (!f) {
      perror(d->xdatname);
      return PA_HOST_EXIT_FAILURE;
    }
    size_t got = fread(d->xDat, sizeof(double), N, f);
    (void)got; /* like the reference: a short file leaves zeros (gaps) */
    fclose(f);
    int nz = 0;
    for (int j = 0; j < N; j++)
      if (!d->xDat[j]) nz++;
    d->Nzeros = nz;
    d->crf0 = (double)N / (N - d->Nzeros);
    /* var(), auxi.c:124-139 */
    double mean = 0., var = 0.;
    for (int j = 0; j < N; j++) mean += d->xDat[j];
    mean /= N;
    for (int j = 0; j < N; j++) var += SQR(d->xDat[j] - mean);
    var /= (N - 1);
    d->sig2 = d->crf0 * var;
    d->DetSSB = (double *)calloc(3 * (size_t)N, sizeof(double));
    char filename[1300];
    snprintf(filename, sizeof filename, "%s/%03d/%s/DetSSB.bin", h->opts.dtaprefix, h->opts.ident,
             d->name);
    f = fopen(filename, "r");
    if (!f) {
      perror(filename);
      return PA_HOST_EXIT_FAILURE;
    }
    got = fread(d->DetSSB, sizeof(double), 3 * (size_t)N, f);
    got = fread(&d->phir, sizeof(double), 1, f);
    got = fread(&d->epsm, sizeof(double), 1, f);
    fclose(f);
    printf("Using %s as detector %s ephemerids...\n", filename, d->name);
    d->sphir = sin(d->phir);
    d->cphir = cos(d->phir);
    d->sepsm = sin(d->epsm);
    d->cepsm = cos(d->epsm);
    d->aa = (double *)calloc(N, sizeof(double));
    d->bb = (double *)calloc(N, sizeof(double));
  }
  for (int i = 1; i < h->nifo; i++)
    if (!(h->ifo[i - 1].sepsm == h->ifo[i].sepsm)) {
      printf("The parameter epsm (DetSSB.bin) differs for detectors %s and %s. Aborting...\n",
             h->ifo[i - 1].name, h->ifo[i].name);
      return PA_HOST_EXIT_FAILURE;
    }
  s->sepsm = h->ifo[0].sepsm;
  s->cepsm = h->ifo[0].cepsm;
  h->t2 = (double *)calloc(N, sizeof(double));
  h->cosmodf = (double *)calloc(N, sizeof(double));
  h->sinmodf = (double *)calloc(N, sizeof(double));
  for (int i = 0; i < N; i++) {
    double omrt = (s->omr) * i;
    h->t2[i] = SQR((double)i);
    h->cosmodf[i] = cos(omrt);
    h->sinmodf[i] = sin(omrt);
  }
  return PA_HOST_OK;
}

/* ------------------------------------------------------------------ */
/* line veto: settings.c:327-656 */

static int read_lines(pa_host *h, host_det *ifo) {
  pa_settings *s = &h->sett;
  char linefile[1200], line[128] = {0};
  snprintf(linefile, sizeof linefile, "%s/O1LinesToBeCleaned_%s_v1.txt", h->opts.dtaprefix,
           ifo->name);
  FILE *data = fopen(linefile, "r");
  if (!data) {
    printf("No known lines file %s for %s IFO found. Continuing without.\n", linefile, ifo->name);
    return 0;
  }
  double(*l)[7] = (double(*)[7])calloc(PA_MAXL, sizeof(double[7]));
  int lnum = 0;
  while (fgets(line, 128, data) != NULL && lnum < PA_MAXL) {
    if (*line == '%') continue;
    int j = 0;
    char *save = NULL;
    for (char *t = strtok_r(line, "\t ", &save); t != NULL && j < 7; t = strtok_r(NULL, "\t ", &save))
      l[lnum][j++] = atof(t);
    lnum++;
  }
  fclose(data);
  const int N = s->N;
  const double *D = ifo->DetSSB;
  double dEmax[3] = {0}, dtEmax[3] = {0};
  for (int i = 0; i < N - 1; i++)
    for (int j = 0; j < 3; j++) {
      double dE = fabs(D[(i + 1) * 3 + j] - D[i * 3 + j]);
      if (dE > dEmax[j]) dEmax[j] = dE;
      double dtE = fabs(D[(i + 1) * 3 + j] * (i + 1) - D[i * 3 + j] * i) * s->dt;
      if (dtE > dtEmax[j]) dtEmax[j] = dtE;
    }
  double fdotMax = 0.5e-8, normdtEmax = 0., normdEmax = 0.;
  for (int j = 0; j < 3; j++) {
    normdtEmax += pow(dtEmax[j], 2.);
    normdEmax += pow(dEmax[j], 2.);
  }
  ifo->lines = (double(*)[2])calloc(PA_MAXL, sizeof(double[2]));
  int j = 0;
  for (int i = 0; i < lnum; i++) {
    int line_type = (int)(l[i][1]);
    int indf = (int)(l[i][3]);
    int indl = (int)(l[i][4]);
    double Dfmaxmax;
    switch (line_type) {
      case 0:
        if (j >= PA_MAXL) break;
        Dfmaxmax = 2. * fdotMax * (s->N * s->dt + sqrt(normdtEmax)) + l[i][0] * sqrt(normdEmax);
        ifo->lines[j][0] = l[i][0] - Dfmaxmax;
        ifo->lines[j][1] = l[i][0] + Dfmaxmax;
        j++;
        break;
      case 1:
      case 2:
        for (int k = indf; k <= indl && j < PA_MAXL; k++) {
          double linefreq = l[i][2] + k * l[i][0];
          Dfmaxmax = 2. * fdotMax * (s->N * s->dt + sqrt(normdtEmax)) + linefreq * sqrt(normdEmax);
          double w = line_type == 1 ? Dfmaxmax : k * Dfmaxmax;
          ifo->lines[j][0] = linefreq - w;
          ifo->lines[j][1] = linefreq + w;
          j++;
        }
        break;
    }
  }
  ifo->numlines = j;
  free(l);
  printf("Number of known lines in %s: %d\n", ifo->name, ifo->numlines);
  return 0;
}

static void narrow_down_band(pa_host *h) {
  h->lines[0][0] = 0;
  h->lines[0][1] = M_PI_2 - h->opts.narrowdown;
  h->lines[1][0] = M_PI_2 + h->opts.narrowdown;
  h->lines[1][1] = M_PI;
  h->sett.numlines_band = 2;
  printf("Band is narrowed-down to [%f, %f]\n", h->lines[0][1], h->lines[1][0]);
}

static void lines_in_band(pa_host *h) {
  pa_settings *s = &h->sett;
  int k = 0;
  if (h->opts.narrowdown < 0.5 * M_PI) k = s->numlines_band;
  double bs = s->fpo, be = s->fpo + s->B;
  for (int i = 0; i < h->nifo; i++) {
    printf("Looking for known lines for %s between %f and %f...\n", h->ifo[i].name, bs, be);
    for (int j = 0; j < h->ifo[i].numlines && k < PA_MAXL; j++) {
      double l = h->ifo[i].lines[j][0], r = h->ifo[i].lines[j][1];
      if (!(r < bs || l > be)) {
        double ll = l > bs ? l : bs;
        double lr = r < be ? r : be;
        h->lines[k][0] = (ll - bs) / (s->B) * M_PI;
        h->lines[k][1] = (lr - bs) / (s->B) * M_PI;
        printf("%s: %f %f %f %f\n", h->ifo[i].name, ll, lr, h->lines[k][0], h->lines[k][1]);
        k++;
      }
    }
  }
  s->numlines_band = k;
}

static int compare_lines(const void *a, const void *b) {
  const double *da = (const double *)a, *db = (const double *)b;
  int d1 = (da[0] > db[0]) - (da[0] < db[0]);
  if (d1 != 0) return d1;
  return (da[1] > db[1]) - (da[1] < db[1]);
}

static int fraction_of_band_vetoed(pa_host *h) {
  pa_settings *s = &h->sett;
  qsort(h->lines, s->numlines_band, 2 * sizeof(double), compare_lines);
  double ll = 0.;
  for (int i = 0; i < s->numlines_band; i++) {
    if (i > 0 && (h->lines[i][0] < h->lines[i - 1][1]))
      ll += h->lines[i][1] - h->lines[i - 1][1];
    else
      ll += h->lines[i][1] - h->lines[i][0];
  }
  ll /= M_PI;
  printf("Veto fraction for band %04d: %f\n", h->opts.band, ll);
  if (!(ll < 1)) {
    printf("This band is fully vetoed. My work here is done, exiting...\n");
    return PA_HOST_EXIT_SUCCESS;
  }
  return PA_HOST_OK;
}

/* settings.c:253-275 */
static void rogcvir(host_det *d) {
  d->amod[0] = .25 * sin(2. * d->egam) * (1 + SQR(sin(d->ephi)));
  d->amod[1] = -.5 * cos(2. * d->egam) * sin(d->ephi);
  d->amod[2] = .5 * sin(2. * d->egam) * sin(2. * d->ephi);
  d->amod[3] = -cos(2. * d->egam) * cos(d->ephi);
  d->amod[4] = .75 * sin(2. * d->egam) * SQR(cos(d->ephi));
  d->amod[5] = cos(2. * d->egam) * sin(d->ephi);
  d->amod[6] = .5 * sin(2. * d->egam) * (1. + SQR(sin(d->ephi)));
  d->amod[7] = cos(2. * d->egam) * cos(d->ephi);
  d->amod[8] = .5 * sin(2. * d->egam) * sin(2. * d->ephi);
}

/* settings.c:281-325, host copy used by the injection */
static void modvir_host(pa_host *h, double sinal, double cosal, double sindel, double cosdel,
                        host_det *d) {
  const double *k = d->amod;
  double cosalfr = cosal * (d->cphir) + sinal * (d->sphir);
  double sinalfr = sinal * (d->cphir) - cosal * (d->sphir);
  double c2d = SQR(cosdel), c2sd = sindel * cosdel;
  for (int t = 0; t < h->sett.N; t++) {
    double c = cosalfr * h->cosmodf[t] + sinalfr * h->sinmodf[t];
    double s = sinalfr * h->cosmodf[t] - cosalfr * h->sinmodf[t];
    double c2s = 2. * SQR(c), cs = c * s;
    d->aa[t] = k[0] * (2. - c2d) * c2s + k[1] * (2. - c2d) * 2. * cs + k[2] * c2sd * c +
               k[3] * c2sd * s - k[0] * (2. - c2d) + k[4] * c2d;
    d->bb[t] = k[5] * sindel * c2s + k[6] * sindel * 2. * cs + k[7] * cosdel * c +
               k[8] * cosdel * s - k[5] * sindel;
  }
}

/* ------------------------------------------------------------------ */
/* small dense linear algebra */

/* LU with partial pivoting on |a_ij| (the documented GSL method used at
 * init.c:541-551) and solve of A x = b for a 4x4 row-major matrix. */
static void lu4_solve(double A[16], const double b[4], double x[4]) {
  int perm[4] = {0, 1, 2, 3};
  for (int j = 0; j < 3; j++) {
    int piv = j;
    double best = fabs(A[j * 4 + j]);
    for (int i = j + 1; i < 4; i++)
      if (fabs(A[i * 4 + j]) > best) {
        best = fabs(A[i * 4 + j]);
        piv = i;
      }
    if (piv != j) {
      for (int k = 0; k < 4; k++) {
        double t = A[j * 4 + k];
        A[j * 4 + k] = A[piv * 4 + k];
        A[piv * 4 + k] = t;
      }
      int t = perm[j];
      perm[j] = perm[piv];
      perm[piv] = t;
    }
    if (A[j * 4 + j] != 0.0)
      for (int i = j + 1; i < 4; i++) {
        double lij = A[i * 4 + j] / A[j * 4 + j];
        A[i * 4 + j] = lij;
        for (int k = j + 1; k < 4; k++) A[i * 4 + k] -= lij * A[j * 4 + k];
      }
  }
  for (int i = 0; i < 4; i++) x[i] = b[perm[i]];
  for (int i = 0; i < 4; i++)
    for (int k = 0; k < i; k++) x[i] -= A[i * 4 + k] * x[k];
  for (int i = 3; i >= 0; i--) {
    for (int k = i + 1; k < 4; k++) x[i] -= A[i * 4 + k] * x[k];
    x[i] /= A[i * 4 + i];
  }
}

/* Crout LU with implicit row scaling and its back-substitution, the
 * algorithm of auxi.c:242-343, used by gridr(). */
static int ludcmp4(double *a, int n, int *indx, double *d) {
  int imax = -1;
  double vv[8];
  *d = 1.0;
  for (int i = 0; i < n; i++) {
    double big = 0.0;
    for (int j = 0; j < n; j++)
      if (fabs(a[n * i + j]) > big) big = fabs(a[n * i + j]);
    if (big == 0.0) return 1;
    vv[i] = 1.0 / big;
  }
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < j; i++) {
      double sum = a[n * i + j];
      for (int k = 0; k < i; k++) sum -= a[n * i + k] * a[n * k + j];
      a[n * i + j] = sum;
    }
    double big = 0.0;
    for (int i = j; i < n; i++) {
      double sum = a[n * i + j];
      for (int k = 0; k < j; k++) sum -= a[n * i + k] * a[n * k + j];
      a[n * i + j] = sum;
      double dum = vv[i] * fabs(sum);
      if (dum >= big) {
        big = dum;
        imax = i;
      }
    }
    if (j != imax) {
      for (int k = 0; k < n; k++) {
        double dum = a[n * imax + k];
        a[n * imax + k] = a[n * j + k];
        a[n * j + k] = dum;
      }
      *d = -(*d);
      vv[imax] = vv[j];
    }
    indx[j] = imax;
    if (a[n * j + j] == 0.0) a[n * j + j] = 1.0e-20;
    double dum = 1.0 / (a[n * j + j]);
    for (int i = j + 1; i < n; i++) a[n * i + j] *= dum;
  }
  return 0;
}

static void lubksb4(const double *a, int n, const int *indx, double *b) {
  int ii = -1;
  for (int i = 0; i < n; i++) {
    int ip = indx[i];
    double sum = b[ip];
    b[ip] = b[i];
    if (ii >= 0)
      for (int j = ii; j <= i - 1; j++) sum -= a[n * i + j] * b[j];
    else if (sum)
      ii = i;
    b[i] = sum;
  }
  for (int i = n - 1; i >= 0; i--) {
    double sum = b[i];
    for (int j = i + 1; j < n; j++) sum -= a[n * i + j] * b[j];
    b[i] = sum / a[n * i + i];
  }
}

/* auxi.c:143-212 */
static void gridr(const double *M, int *spndr, int *nr, int *mr, double oms, double Smax) {
  double Mp[16], smx[64], d;
  int indx[4];
  double Ob = M_PI, cof = oms + Ob;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) Mp[4 * i + j] = M[4 * j + i];
  ludcmp4(Mp, 4, indx, &d);
  for (int i = 0; i < 8; i++) {
    smx[8 * i + 2] = cof;
    smx[8 * i + 6] = -cof;
  }
  for (int i = 0; i < 4; i++) {
    smx[16 * i + 3] = smx[16 * i + 7] = cof;
    smx[16 * i + 11] = smx[16 * i + 15] = -cof;
  }
  for (int i = 0; i < 8; i++) {
    smx[4 * i] = Ob;
    smx[4 * i + 32] = -Ob;
  }
  for (int i = 0; i < 2; i++)
    for (int j = 0; j < 4; j++) {
      smx[32 * i + 4 * j + 1] = -Smax;
      smx[32 * i + 4 * j + 17] = 0.;
    }
  for (int i = 0; i < 16; i++) lubksb4(Mp, 4, indx, smx + 4 * i);
  spndr[0] = nr[0] = mr[0] = 16384;
  spndr[1] = nr[1] = mr[1] = -16384;
  for (int i = 0; i < 16; i++) {
    if (floor(smx[4 * i + 1]) < spndr[0]) spndr[0] = floor(smx[4 * i + 1]);
    if (ceil(smx[4 * i + 1]) > spndr[1]) spndr[1] = ceil(smx[4 * i + 1]);
    if (floor(smx[4 * i + 2]) < nr[0]) nr[0] = floor(smx[4 * i + 2]);
    if (ceil(smx[4 * i + 2]) > nr[1]) nr[1] = ceil(smx[4 * i + 2]);
    if (floor(smx[4 * i + 3]) < mr[0]) mr[0] = floor(smx[4 * i + 3]);
    if (ceil(smx[4 * i + 3]) > mr[1]) mr[1] = ceil(smx[4 * i + 3]);
  }
}

/* ------------------------------------------------------------------ */
/* injection: init.c:462-651 */

static int add_signal(pa_host *h) {
  pa_settings *s = &h->sett;
  pa_range *r = &h->s_range;
  const int N = s->N;
  int gsize = 0, reffr = 0;
  double snr = 0, h0 = 0, sum = 0., sigma_noise = 1.0;
  double sgnlo[8] = {0}, sgnlol[4];
  char amporsnr[8] = {0};
  FILE *data = fopen(h->opts.addsig, "r");
  if (!data) {
    perror(h->opts.addsig);
    return PA_HOST_EXIT_FAILURE;
  }
  if (fscanf(data, "%7s", amporsnr) != 1) amporsnr[0] = 0;
  if (!strcmp(amporsnr, "amp")) {
    if (fscanf(data, "%le %d %d", &h0, &gsize, &reffr) != 3) goto bad;
    printf("add_signal(): GW amplitude h0 is %le\n", h0);
  } else if (!strcmp(amporsnr, "snr")) {
    if (fscanf(data, "%le %d %d", &snr, &gsize, &reffr) != 3) goto bad;
    printf("add_signal(): GW (network) signal-to-noise ratio is %le\n", snr);
  } else {
    goto bad;
  }
  for (int i = 0; i < 8; i++)
    if (fscanf(data, "%le", sgnlo + i) != 1) goto bad;
  fclose(data);

  sgnlo[0] += -2. * sgnlo[1] * (N) * (reffr - h->opts.ident);
  if (sgnlo[0] < 0 || sgnlo[0] > M_PI) {
    printf("add_signal(): injected frequency outside the band. Exiting...\n");
    return PA_HOST_EXIT_FAILURE;
  }
  double cof = s->oms + sgnlo[0];
  sgnlol[0] = sgnlo[0];
  sgnlol[1] = sgnlo[1];
  /* ast2lin (auxi.c:26-53) with C_EPSMA */
  double be[2];
  be[0] = cos(C_EPSMA) * sin(sgnlo[3]) * cos(sgnlo[2]) + sin(C_EPSMA) * sin(sgnlo[2]);
  be[1] = cos(sgnlo[3]) * cos(sgnlo[2]);
  double d1 = asin(be[0] * sin(C_EPSMA) + sqrt(1. - be[0] * be[0] - be[1] * be[1]) * cos(C_EPSMA)) -
              sgnlo[2];
  r->pmr[0] = (fabs(d1) < 10. * 2.220446049250313e-16) ? 1 : 2;
  sgnlol[2] = be[0] * cof;
  sgnlol[3] = be[1] * cof;
  /* solve M x = sgnlol (the row-major view of the column-major M, then
   * transposed, init.c:544-550) */
  double A[16], x[4];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) A[4 * i + j] = s->M[4 * j + i];
  lu4_solve(A, sgnlol, x);
  r->spndr[0] = ROUND(x[1]);
  r->nr[0] = ROUND(x[2]);
  r->mr[0] = ROUND(x[3]);
  r->spndr[1] = r->spndr[0] + gsize;
  r->spndr[0] -= gsize;
  r->nr[1] = r->nr[0] + gsize;
  r->nr[0] -= gsize;
  r->mr[1] = r->mr[0] + gsize;
  r->mr[0] -= gsize;
  r->pmr[1] = r->pmr[0];
  printf("add_signal(): following grid range is used (spndr, nr, mr, pmr pairs)\n");
  printf("%d %d %d %d %d %d %d %d\n", r->spndr[0], r->spndr[1], r->nr[0], r->nr[1], r->mr[0],
         r->mr[1], r->pmr[0], r->pmr[1]);

  double sindadd = sin(sgnlo[2]), cosdadd = cos(sgnlo[2]);
  double sinaadd = sin(sgnlo[3]), cosaadd = cos(sgnlo[3]);
  double phaseshift = sgnlo[0] * N * (reffr - h->opts.ident) +
                      sgnlo[1] * pow(N * (reffr - h->opts.ident), 2);
  double **signadd = (double **)malloc(h->nifo * sizeof(double *));
  for (int n = 0; n < h->nifo; n++) {
    host_det *d = &h->ifo[n];
    signadd[n] = (double *)malloc(N * sizeof(double));
    modvir_host(h, sinaadd, cosaadd, sindadd, cosdadd, d);
    double nS[3] = {cosaadd * cosdadd, sinaadd * cosdadd, sindadd};
    for (int i = 0; i < N; i++) {
      double shiftadd = 0.;
      for (int j = 0; j < 3; j++) shiftadd += nS[j] * d->DetSSB[i * 3 + j];
      double phaseadd = sgnlo[0] * i + sgnlo[1] * h->t2[i] + (cof + 2. * sgnlo[1] * i) * shiftadd -
                        phaseshift;
      signadd[n][i] = sgnlo[4] * (d->aa[i]) * cos(phaseadd) + sgnlo[6] * (d->aa[i]) * sin(phaseadd) +
                      sgnlo[5] * (d->bb[i]) * cos(phaseadd) + sgnlo[7] * (d->bb[i]) * sin(phaseadd);
      sum += pow(signadd[n][i], 2.);
    }
  }
  if (snr) h0 = (snr * sigma_noise) / (sqrt(sum));
  for (int n = 0; n < h->nifo; n++) {
    for (int i = 0; i < N; i++)
      if (h->ifo[n].xDat[i]) h->ifo[n].xDat[i] += h0 * signadd[n][i];
    free(signadd[n]);
  }
  free(signadd);
  return PA_HOST_OK;
bad:
  fclose(data);
  printf("Problem with the signal file. Exiting...\n");
  return PA_HOST_EXIT_FAILURE;
}

/* init.c:656-804 */
static int set_search_range(pa_host *h) {
  pa_range *r = &h->s_range;
  if (h->opts.hemi) {
    r->pmr[0] = r->pmr[1] = h->opts.hemi;
  } else {
    r->pmr[0] = 1;
    r->pmr[1] = 2;
  }
  if (strlen(h->opts.range)) {
    FILE *data = fopen(h->opts.range, "r");
    if (!data) {
      perror(h->opts.range);
      return PA_HOST_EXIT_FAILURE;
    }
    int got = fscanf(data, "%d %d %d %d %d %d %d %d", r->spndr, 1 + r->spndr, r->nr, 1 + r->nr,
                     r->mr, 1 + r->mr, r->pmr, 1 + r->pmr);
    (void)got;
    fclose(data);
  } else {
    gridr(h->sett.M, r->spndr, r->nr, r->mr, h->sett.oms, h->sett.Smax);
    if (strlen(h->opts.getrange)) {
      FILE *data = fopen(h->opts.getrange, "w");
      if (!data) {
        printf("Can't open %s file for writing\n", h->opts.getrange);
        return PA_HOST_EXIT_FAILURE;
      }
      fprintf(data, "%d %d\n%d %d\n%d %d\n%d %d\n", r->spndr[0], r->spndr[1], r->nr[0], r->nr[1],
              r->mr[0], r->mr[1], r->pmr[0], r->pmr[1]);
      printf("Wrote input data grid ranges to %s\n", h->opts.getrange);
      fclose(data);
    }
  }
  printf("set_search_range() - the grid ranges are maximally this:\n");
  printf("(spndr, nr, mr, pmr pairs): %d %d %d %d %d %d %d %d\n", r->spndr[0], r->spndr[1],
         r->nr[0], r->nr[1], r->mr[0], r->mr[1], r->pmr[0], r->pmr[1]);
  printf("Smin: %le, -Smax: %le\n", h->sett.Smin, h->sett.Smax);
  return PA_HOST_OK;
}

/* init.c:868-917 */
static int read_checkpoints(pa_host *h) {
  pa_range *r = &h->s_range;
  pa_cmdline *o = &h->opts;
  r->pst = r->pmr[0];
  r->mst = r->mr[0];
  r->nst = r->nr[0];
  r->sst = r->spndr[0];
  h->FNum = 0;
  if (!o->checkp_flag) return PA_HOST_OK;
  if (o->hemi)
    snprintf(o->qname, sizeof o->qname, "state_%03d_%04d%s_%d.dat", o->ident, o->band, o->label,
             o->hemi);
  else
    snprintf(o->qname, sizeof o->qname, "state_%03d_%04d%s.dat", o->ident, o->band, o->label);
  FILE *state = fopen(o->qname, "r");
  if (state) {
    if (fscanf(state, "%d %d %d %d %d", &r->pst, &r->mst, &r->nst, &r->sst, &h->FNum) == EOF) {
      fprintf(stderr, "State file empty: nothing to do...\n");
      h->nothing_to_do = 1;
    }
    fclose(state);
  }
  return PA_HOST_OK;
}

/* ------------------------------------------------------------------ */

pa_host *pa_host_create(int argc, char **argv, int *rc) {
  pa_host *h = (pa_host *)calloc(1, sizeof(*h));
  h->lines = (double(*)[2])calloc(PA_MAXL, sizeof(double[2]));
  int r = handle_opts(h, argc, argv);
  if (rc) *rc = r;
  if (r != PA_HOST_OK) {
    pa_host_destroy(h);
    return NULL;
  }
  return h;
}

int pa_host_setup(pa_host *h) {
  int rc;
  struct stat buffer;
  if (stat(h->opts.prefix, &buffer) == -1) {
    if (errno == ENOENT) {
      if (mkdir(h->opts.prefix, S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH) == -1) {
        perror(h->opts.prefix);
        return PA_HOST_EXIT_FAILURE;
      }
    } else {
      perror(h->opts.prefix);
      return PA_HOST_EXIT_FAILURE;
    }
  }
  if ((rc = read_grid(h))) return rc;
  search_settings(&h->sett);
  if ((rc = detectors_settings(h))) return rc;
  if ((rc = init_arrays(h))) return rc;
  if (h->opts.narrowdown < 0.5 * M_PI) narrow_down_band(h);
  if (h->opts.veto_flag) {
    for (int i = 0; i < h->nifo; i++) {
      printf("Reading known lines data for %s from %s\n", h->ifo[i].name, h->opts.dtaprefix);
      read_lines(h, &h->ifo[i]);
    }
    lines_in_band(h);
  }
  if (h->sett.numlines_band) {
    printf("list of excluded frequencies in band (in radians):\n");
    for (int k = 0; k < h->sett.numlines_band; k++) printf("%f %f\n", h->lines[k][0], h->lines[k][1]);
    if ((rc = fraction_of_band_vetoed(h))) return rc;
  } else {
    printf("Veto fraction for band %04d: %f\n", h->opts.band, 0.);
  }
  h->sett.lines = &h->lines[0][0];
  for (int i = 0; i < h->nifo; i++) rogcvir(&h->ifo[i]);
  if (strlen(h->opts.addsig)) {
    if ((rc = add_signal(h))) return rc;
  } else {
    if ((rc = set_search_range(h))) return rc;
  }
  if (strlen(h->opts.getrange)) return PA_HOST_EXIT_SUCCESS;
  if ((rc = read_checkpoints(h))) return rc;
  for (int i = 0; i < h->nifo; i++) {
    pa_detector *d = &h->det[i];
    host_det *s = &h->ifo[i];
    d->xDat = s->xDat;
    d->DetSSB = s->DetSSB;
    d->sig2 = s->sig2;
    d->sphir = s->sphir;
    d->cphir = s->cphir;
    memcpy(d->amod, s->amod, sizeof(d->amod));
  }
  return h->nothing_to_do ? PA_HOST_EXIT_SUCCESS : PA_HOST_OK;
}

static int append_triggers(const char *outname, const double *sgnlv, int sgnlc) {
  int fd = open(outname, O_WRONLY | O_CREAT | O_APPEND, S_IRUSR | S_IWUSR | S_IRGRP | S_IROTH);
  if (fd < 0) {
    perror(outname);
    return -1;
  }
  struct flock lck;
  memset(&lck, 0, sizeof(lck));
  lck.l_type = F_WRLCK;
  lck.l_whence = 0;
  lck.l_start = 0L;
  lck.l_len = 0L;
  if (fcntl(fd, F_SETLKW, &lck) < 0) perror("fcntl()");
  size_t bytes = (size_t)sgnlc * PA_NPAR * sizeof(double);
  const char *p = (const char *)sgnlv;
  while (bytes) {
    ssize_t w = write(fd, p, bytes);
    if (w <= 0) {
      perror("write()");
      close(fd);
      return -1;
    }
    bytes -= (size_t)w;
    p += w;
  }
  if (close(fd) < 0) perror("close()");
  return 0;
}

int pa_host_search(pa_host *h, pa_ctx *ctx) {
  pa_settings *sett = &h->sett;
  pa_range *r = &h->s_range;
  pa_opts opts;
  pa_host_core_opts(h, &opts);
  struct timespec t0, t1;
  clock_gettime(CLOCK_REALTIME, &t0);
  int cap = 2 * sett->nfft;
  double *sgnlv = (double *)calloc((size_t)PA_NPAR * cap, sizeof(double));
  int sgnlc = 0;
  FILE *state = NULL;
  if (h->opts.checkp_flag) state = fopen(h->opts.qname, "w");
  char outname[1400];
  const int skyb = h->opts.skybatch > 0 ? h->opts.skybatch : 1;
  pa_sky *tasks = (pa_sky *)malloc(sizeof(pa_sky) * skyb);
  int rc_out = PA_HOST_OK;
  /* Host-side fault injection (tests of checkpoint/resume): with
   * PA_HOST_STOP_AT_SKY=k the search stops like a crash right after writing
   * the state file for its k-th sky-point batch (0-based), before that
   * batch's GPU work: buffered candidates are dropped, the state file stays. */
  const char *stop_env = getenv("PA_HOST_STOP_AT_SKY");
  const long stop_at = stop_env ? strtol(stop_env, NULL, 10) : -1;
  long batch_no = 0;

  for (int pm = r->pst; pm <= r->pmr[1]; ++pm) {
    snprintf(outname, sizeof outname, "%s/triggers_%03d_%04d%s_%d.bin", h->opts.prefix,
             h->opts.ident, h->opts.band, h->opts.label, pm);
    int mm = r->mst, nn = r->nst;
    while (mm <= r->mr[1]) {
      /* collect up to skyb sky points in loop order (jobcore.c:97-98) */
      int nt = 0;
      while (nt < skyb && mm <= r->mr[1]) {
        tasks[nt].pm = pm;
        tasks[nt].mm = mm;
        tasks[nt].nn = nn;
        nt++;
        if (++nn > r->nr[1]) {
          nn = r->nr[0];
          ++mm;
        }
      }
      if (state) {
        if (ftruncate(fileno(state), 0)) perror("ftruncate");
        fprintf(state, "%d %d %d %d %d\n", pm, tasks[0].mm, tasks[0].nn, r->sst, h->FNum);
        fseek(state, 0, SEEK_SET);
      }
      if (batch_no++ == stop_at) {
        rc_out = PA_HOST_INTERRUPTED;
        goto done;
      }
      for (;;) {
        int needed = 0, st;
        if (nt == 1)
          st = pa_job_core(ctx, pm, tasks[0].mm, tasks[0].nn, &opts, r, &sgnlc, sgnlv, cap, NULL,
                           &h->FNum, &needed);
        else
          st = pa_search_batch(ctx, tasks, nt, &opts, r, &sgnlc, sgnlv, cap, NULL, &h->FNum,
                               &needed);
        if (st == PA_ERR_CAPACITY) {
          int ncap = needed + 2 * sett->nfft;
          double *nb = (double *)realloc(sgnlv, sizeof(double) * PA_NPAR * (size_t)ncap);
          if (!nb) {
            rc_out = PA_HOST_EXIT_FAILURE;
            goto done;
          }
          sgnlv = nb;
          cap = ncap;
          continue;
        }
        if (st != PA_OK) {
          fprintf(stderr, "job_core failed: %s\n", pa_last_error(ctx));
          rc_out = PA_HOST_EXIT_FAILURE;
          goto done;
        }
        break;
      }
      r->sst = r->spndr[0];
      if (sgnlc > sett->nfft) {
        if (append_triggers(outname, sgnlv, sgnlc)) {
          rc_out = PA_HOST_EXIT_FAILURE;
          goto done;
        }
        sgnlc = 0;
      }
    }
    r->nst = r->nr[0];
    r->mst = r->mr[0];
    if (append_triggers(outname, sgnlv, sgnlc)) {
      rc_out = PA_HOST_EXIT_FAILURE;
      goto done;
    }
    sgnlc = 0;
  }
done:
  if (state) fclose(state);
  free(sgnlv);
  free(tasks);
  clock_gettime(CLOCK_REALTIME, &t1);
  printf("Time elapsed: %e s\n", (t1.tv_sec - t0.tv_sec) + (t1.tv_nsec - t0.tv_nsec) * 1e-9);
  return rc_out;
}

int pa_host_main(int argc, char **argv) {
  printf("Code version : gb300\n");
  int rc = 0;
  pa_host *h = pa_host_create(argc, argv, &rc);
  if (!h) return rc == PA_HOST_EXIT_SUCCESS ? 0 : 1;
  rc = pa_host_setup(h);
  if (rc != PA_HOST_OK) {
    pa_host_destroy(h);
    return rc == PA_HOST_EXIT_SUCCESS ? 0 : 1;
  }
  pa_config cfg;
  pa_host_config(h, &cfg);
  int st = 0;
  pa_ctx *ctx = pa_create(&h->sett, h->det, h->nifo, &cfg, &st);
  if (!ctx) {
    fprintf(stderr, "pa_create failed (%d): %s\n", st, pa_last_error(NULL));
    pa_host_destroy(h);
    return 1;
  }
  if (h->opts.graphs) pa_set_graphs(ctx, 1);
  rc = pa_host_search(h, ctx);
  pa_destroy(ctx);
  if (rc == PA_HOST_OK && h->opts.checkp_flag) {
    FILE *state = fopen(h->opts.qname, "w");
    if (state) fclose(state);
  }
  pa_host_destroy(h);
  if (rc == PA_HOST_INTERRUPTED) return 3;
  return rc == PA_HOST_OK ? 0 : 1;
}

void pa_host_destroy(pa_host *h) {
  if (!h) return;
  for (int i = 0; i < PA_MAX_DETECTORS; i++) {
    free(h->ifo[i].xDat);
    free(h->ifo[i].DetSSB);
    free(h->ifo[i].aa);
    free(h->ifo[i].bb);
    free(h->ifo[i].lines);
  }
  free(h->lines);
  free(h->cosmodf);
  free(h->sinmodf);
  free(h->t2);
  free(h);
}

const pa_settings *pa_host_settings(const pa_host *h) { return &h->sett; }

const pa_detector *pa_host_detectors(const pa_host *h, int *nifo) {
  if (nifo) *nifo = h->nifo;
  return h->det;
}

const pa_range *pa_host_range(const pa_host *h) { return &h->s_range; }

void pa_host_core_opts(const pa_host *h, pa_opts *o) {
  o->trl = h->opts.trl;
  o->white_flag = h->opts.white_flag;
  o->s0_flag = h->opts.s0_flag;
  o->use_range = (strcmp(h->opts.addsig, "") || strcmp(h->opts.range, "")) ? 1 : 0;
}

void pa_host_config(const pa_host *h, pa_config *c) {
  memset(c, 0, sizeof(*c));
  c->precision = h->opts.precision;
  c->phase_mode = h->opts.phase_mode;
  c->spindown_batch = h->opts.sbatch;
  c->device = h->opts.device;
}

const char *pa_host_detector_name(const pa_host *h, int i) {
  if (i < 0 || i >= h->nifo) return "";
  return h->ifo[i].name;
}
