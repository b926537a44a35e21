/*
 * pa_coinc_host.c -- the coincidence program (coincidences-gb300) around
 * the device coincidence step pa_coinc_* (csrc/pa_coinc.cu).
 *
 * Same command line, inputs and outputs as the reference program
 * coincidences/src/coincidences.c with handle_opts_coinc() and
 * manage_grid_matrix() (search/network/src-cpu/init.c:972-1210):
 *   -data -output -shift -scale -refr -fpo -dt -trigname -refloc -mincoin
 *   -narrowdown -snrcutoff -nod, --help; plus -device <ordinal>.
 * It reads the trigger files of the data directory in directory order
 * (readdir), takes the frame number from the first '_'-separated part of the
 * name that starts with a digit, writes <output>/<shift>_<scale>_<trigname>.coi
 * with the reference's record layout and prints the same summary line to
 * stderr.  Differences: mincoin must be >= 2 (with 1 the reference counts no
 * coincidence and reports an arbitrary run); at most 255 frames (the
 * reference's frame table has 256 rows, the first unused); an unreadable
 * trigger file is reported and skipped (the reference closes a NULL file).
 */
#include <dirent.h>
#include <errno.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/types.h>

#include "../../include/polgraw_gb300_host.h"

#define C_OMEGA_R 7.2921151467064e-5
#define C_SIDDAY (2. * M_PI / C_OMEGA_R)
#define ROUND(x) floor((x) + 0.5)

typedef struct coinc_opts {
  int shift, scale, refr, mincoin, nod, device;
  double fpo, dt, narrowdown, snrcutoff;
  char prefix[512], dtaprefix[512], trigname[512], refloc[512];
} coinc_opts;

static void coinc_help(void) {
  printf("polgraw-allsky periodic GWs: search for concidences among candidates\n");
  printf("Usage: ./coincidences -[switch1] <value1> -[switch2] <value2> ...\n");
  printf("Switches are:\n\n");
  printf("-data         Data directory (default is ./candidates)\n");
  printf("-output       Output directory (default is ./coinc-results)\n");
  printf("-shift        Cell shifts in fsda directions (4 digit number, e.g. 0101, default 0000)\n");
  printf("-scale        Cell scaling in fsda directions (4 digit number, e.g. 4824, default 1111)\n");
  printf("-refr         Reference frame number\n");
  printf("-fpo          Reference band frequency fpo value\n");
  printf("-dt           Data sampling time dt (default value: 0.5)\n");
  printf("-trigname     Part of triggers' name (for identifying files)\n");
  printf("-refloc       Location of the reference grid.bin and starting_date files\n");
  printf("-mincoin      Minimal number of coincidences recorded\n");
  printf("-narrowdown   Narrow-down the frequency band (range [0, 0.5] +- around center)\n");
  printf("-nod          Number of days\n");
  printf("-snrcutoff    Signal-to-noise threshold cutoff (default value: 6)\n");
  printf("-device       CUDA device ordinal (default 0)\n\n");
  printf("Also:\n\n");
  printf("--help\t\tThis help\n");
}

/* handle_opts_coinc (init.c:972-1122); returns 0, or the exit code */
static int coinc_handle_opts(coinc_opts *o, int argc, char **argv) {
  memset(o, 0, sizeof(*o));
  strcpy(o->prefix, "./coinc-results");
  strcpy(o->dtaprefix, "./candidates");
  o->dt = 0.5;
  o->mincoin = 3;
  o->narrowdown = 0.5;
  o->scale = 1111;
  o->snrcutoff = 6;
  static int help_flag = 0;
  static struct option long_options[] = {
      {"help", no_argument, &help_flag, 1},   {"shift", required_argument, 0, 's'},
      {"scale", required_argument, 0, 'z'},   {"refr", required_argument, 0, 'r'},
      {"output", required_argument, 0, 'o'},  {"data", required_argument, 0, 'd'},
      {"fpo", required_argument, 0, 'p'},     {"dt", required_argument, 0, 't'},
      {"trigname", required_argument, 0, 'e'}, {"refloc", required_argument, 0, 'g'},
      {"mincoin", required_argument, 0, 'm'}, {"narrowdown", required_argument, 0, 'n'},
      {"snrcutoff", required_argument, 0, 'c'}, {"nod", required_argument, 0, 'y'},
      {"device", required_argument, 0, 'D'},  {0, 0, 0, 0}};
  help_flag = 0;
  optind = 1;
  while (1) {
    if (help_flag) {
      coinc_help();
      return PA_HOST_EXIT_SUCCESS;
    }
    int option_index = 0;
    int c = getopt_long_only(argc, argv, "p:o:d:s:z:r:t:e:g:m:n:c:y:D:", long_options, &option_index);
    if (c == -1) break;
    switch (c) {
      case 'p': o->fpo = atof(optarg); break;
      case 's': o->shift = (int)atof(optarg); break;
      case 'z': o->scale = atoi(optarg); break;
      case 'r': o->refr = atoi(optarg); break;
      case 'o': snprintf(o->prefix, sizeof(o->prefix), "%s", optarg); break;
      case 'd': snprintf(o->dtaprefix, sizeof(o->dtaprefix), "%s", optarg); break;
      case 't': o->dt = atof(optarg); break;
      case 'e': snprintf(o->trigname, sizeof(o->trigname), "%s", optarg); break;
      case 'g': snprintf(o->refloc, sizeof(o->refloc), "%s", optarg); break;
      case 'm': o->mincoin = atoi(optarg); break;
      case 'n': o->narrowdown = atof(optarg); break;
      case 'c': o->snrcutoff = atof(optarg); break;
      case 'y': o->nod = atoi(optarg); break;
      case 'D': o->device = atoi(optarg); break;
      default: break;
    }
  }
  if (help_flag) {
    coinc_help();
    return PA_HOST_EXIT_SUCCESS;
  }
  o->narrowdown *= M_PI;
  if (!o->nod) {
    printf("Number of days not set... Exiting\n");
    return PA_HOST_EXIT_FAILURE;
  }
  printf("Number of days is %d\n", o->nod);
  printf("The SNR threshold cutoff is %.12f, ", o->snrcutoff);
  printf("corresponding to F-statistic value of %.12f\n", pow(o->snrcutoff, 2) / 2. + 2);
  return 0;
}

/* the first '_'-separated part of the name that starts with a digit
 * (coincidences.c:206-215); *first gets the name's first part, which is what
 * the reference prints after cutting the name in place */
static int frame_from_name(const char *name, char *first, size_t nfirst) {
  char buf[512];
  snprintf(buf, sizeof(buf), "%s", name);
  char *p = buf, *tok;
  int frame = -1, k = 0;
  while ((tok = strsep(&p, "_")) != NULL) {
    if (k++ == 0) snprintf(first, nfirst, "%s", tok);
    if (tok[0] >= '0' && tok[0] <= '9') {
      frame = atoi(tok);
      break;
    }
  }
  return frame;
}

int pa_coinc_main(int argc, char **argv) {
  coinc_opts o;
  int rc = coinc_handle_opts(&o, argc, argv);
  if (rc == PA_HOST_EXIT_SUCCESS) return 0;
  if (rc) return 1;
  struct stat st;
  if (stat(o.prefix, &st) == -1) {
    if (errno == ENOENT) {
      if (mkdir(o.prefix, S_IRWXU | S_IRGRP | S_IXGRP | S_IROTH | S_IXOTH) == -1) {
        perror(o.prefix);
        return 1;
      }
    } else {
      perror(o.prefix);
      return 1;
    }
  }
  /* manage_grid_matrix (init.c:1142-1210) */
  char filename[1100];
  double fisher[16], vedva[16];
  snprintf(filename, sizeof(filename), "%s/grid.bin", o.refloc);
  FILE *g = fopen(filename, "r");
  if (!g) {
    perror(filename);
    return 1;
  }
  printf("Reading the reference grid.bin at %s\n", o.refloc);
  int fftpad = 0;
  double M[16];
  if (fread(&fftpad, sizeof(int), 1, g) != 1 || fread(M, sizeof(double), 16, g) != 16 ||
      fread(fisher, sizeof(double), 16, g) != 16) {
    fclose(g);
    fprintf(stderr, "%s: short file\n", filename);
    return 1;
  }
  fclose(g);
  printf("fftpad from the grid file: %d\n", fftpad);
  pa_coinc_vedva(fisher, vedva);
  /* search_settings (settings.c:16-81): N and oms */
  const int N = (int)ROUND(o.nod * C_SIDDAY / o.dt);
  const double oms = 2. * M_PI * o.fpo * o.dt;
  printf("Settings dt: %f, oms: %f\n", o.dt, oms);
  printf("Reference frame number: %d\n", o.refr);

  pa_coinc_cfg cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.N = N;
  cfg.oms = oms;
  memcpy(cfg.vedva, vedva, sizeof(vedva));
  int val = o.shift, i;
  for (i = 0; i < 4; i++) cfg.shift[i] = 0;
  for (i = 3; val > 0 && i >= 0; i--, val /= 10)
    if (val % 10) cfg.shift[i] = val % 10;
  printf("Cell shifts  in f, s, d, a directions: ");
  for (i = 0; i < 4; i++) printf("%d ", cfg.shift[i]);
  printf("\n");
  val = o.scale;
  for (i = 0; i < 4; i++) cfg.scale[i] = 1;
  for (i = 3; val > 0 && i >= 0; i--, val /= 10)
    if (val % 10) cfg.scale[i] = val % 10;
  printf("Cell scaling in f, s, d, a directions: ");
  for (i = 0; i < 4; i++) printf("%d ", cfg.scale[i]);
  printf("\n");
  cfg.refr = o.refr;
  cfg.narrowdown = o.narrowdown;
  cfg.snrcutoff = o.snrcutoff;
  cfg.mincoin = o.mincoin;
  cfg.device = o.device;
  int status = 0;
  pa_coinc *cc = pa_coinc_create(&cfg, &status);
  if (!cc) {
    fprintf(stderr, "coincidences-gb300: %s\n", pa_coinc_last_error(NULL));
    return 1;
  }

  char first[256][64];
  int nframes = 0, current_frame = 0;
  DIR *dp = opendir(o.dtaprefix);
  if (dp) {
    struct dirent *ep;
    while ((ep = readdir(dp))) {
      if (!((ep->d_type == DT_REG) || (ep->d_type == DT_LNK)) || strstr(ep->d_name, o.trigname) == NULL) continue;
      if (nframes == 255) {
        fprintf(stderr, "coincidences-gb300: more than 255 trigger files\n");
        pa_coinc_destroy(cc);
        closedir(dp);
        return 1;
      }
      snprintf(filename, sizeof(filename), "%s/%s", o.dtaprefix, ep->d_name);
      /* a name without a number keeps the previous frame number */
      const int fr = frame_from_name(ep->d_name, first[nframes], sizeof(first[0]));
      if (fr >= 0) current_frame = fr;
      const int frame = current_frame;
      FILE *data = fopen(filename, "r");
      if (!data) {
        perror(filename);
        continue;
      }
      fseek(data, 0, SEEK_END);
      const long bytes = ftell(data);
      fseek(data, 0, SEEK_SET);
      const long long n = bytes / (long)(5 * sizeof(double));
      double *rec = (double *)malloc(sizeof(double) * 5 * (n > 0 ? n : 1));
      const long long got = (long long)fread(rec, sizeof(double) * 5, (size_t)n, data);
      fclose(data);
      rc = pa_coinc_add_frame(cc, frame, rec, got);
      free(rec);
      if (rc) {
        fprintf(stderr, "coincidences-gb300: %s\n", pa_coinc_last_error(cc));
        pa_coinc_destroy(cc);
        closedir(dp);
        return 1;
      }
      nframes++;
    }
    closedir(dp);
  }
  pa_coinc_summary sum;
  rc = pa_coinc_run(cc, &sum);
  if (rc) {
    fprintf(stderr, "coincidences-gb300: %s\n", pa_coinc_last_error(cc));
    pa_coinc_destroy(cc);
    return 1;
  }
  int *frameinfo = (int *)malloc(sizeof(int) * 3 * (nframes > 0 ? nframes : 1));
  pa_coinc_rec *recs = (pa_coinc_rec *)malloc(sizeof(pa_coinc_rec) * (sum.ncoin > 0 ? sum.ncoin : 1));
  int *fra = (int *)malloc(sizeof(int) * (sum.nmembers > 0 ? sum.nmembers : 1));
  int *ops = (int *)malloc(sizeof(int) * (sum.nmembers > 0 ? sum.nmembers : 1));
  pa_coinc_get(cc, frameinfo, recs, fra, ops);
  for (i = 0; i < nframes; i++)
    printf("Reading %s... Frame %d: %d/%d\n", first[i], frameinfo[3 * i], frameinfo[3 * i + 2], frameinfo[3 * i + 1]);
  printf("Total number of candidates from all frames: %lld\n", sum.unique);

  /* coincidences.c:476-533 */
  char outname[1200];
  snprintf(outname, sizeof(outname), "%s/%04d_%04d_%s.coi", o.prefix, o.shift, o.scale, o.trigname);
  FILE *out = fopen(outname, "w");
  if (!out) {
    perror(outname);
    pa_coinc_destroy(cc);
    return 1;
  }
  for (int q = 0; q < sum.ncoin; q++) {
    unsigned short w = (unsigned short)recs[q].w;
    float meanf[5];
    unsigned short fr16[256];
    for (int l = 0; l < 5; l++) meanf[l] = (float)recs[q].mean[l];
    for (int k = 0; k < recs[q].w && k < 256; k++) fr16[k] = (unsigned short)fra[recs[q].first + k];
    fwrite(&w, sizeof(unsigned short), 1, out);
    fwrite(meanf, sizeof(float), 5, out);
    fwrite(fr16, sizeof(unsigned short), w, out);
    fwrite(ops + recs[q].first, sizeof(int), w, out);
  }
  fclose(out);
  /* coincidences.c:563-593 */
  if (sum.ncoin > 0 && sum.maxcoin >= o.mincoin) {
    const pa_coinc_rec *m = &recs[sum.maxcoin_index];
    fprintf(stderr, "%s %04d %5f %5hu %5d %15.8le %5.8le %5.8le %5.8le %5le ", o.trigname, o.shift, o.fpo,
            (unsigned short)nframes, sum.maxcoin, m->mean[0], m->mean[1], m->mean[2], m->mean[3], m->mean[4]);
    for (i = 0; i < nframes; i++)
      fprintf(stderr, "%d %d %d ", frameinfo[3 * i], frameinfo[3 * i + 1], frameinfo[3 * i + 2]);
    for (i = 0; i < sum.maxcoin; i++) fprintf(stderr, "%d ", fra[m->first + i]);
    fprintf(stderr, "\n");
  }
  free(frameinfo);
  free(recs);
  free(fra);
  free(ops);
  pa_coinc_destroy(cc);
  return 0;
}
