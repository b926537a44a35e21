/*
 * gridgen-gb300 -- the grid generator's command line over pa_gridgen():
 * reads <dir>rSSB.bin, <dir>rDet.bin and <dir>DetSSB.bin (the directory is
 * concatenated with the file names, as gridgen/main.cpp:617-635 does, so it
 * needs its trailing '/'), writes <dir>grid.bin, and prints the fftpad and
 * the three matrices.  Options (gridgen/main.cpp:62-79): -m minimal match
 * (c0 = m^2 with six decimals) or -c covariance, -n log2 of the FFT length
 * (default 20), -a s1 | s2 | a (default a: automatic), -i initial time
 * (default 0.5), -na / -nr bisection and deep-hole depths (35, 20), -d
 * directory; -p is accepted and ignored (grid.bin is always written
 * whole).  The table of S2 cells, dataS2.txt, is read from the working
 * directory when it is there, and never written.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/polgraw_gb300_host.h"

static double *read_all(const char *path, long long *count) {
  FILE *f = fopen(path, "rb");
  if (!f) return NULL;
  fseek(f, 0, SEEK_END);
  const long bytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  double *v = (double *)malloc((size_t)bytes + 8);
  const size_t got = v ? fread(v, 1, (size_t)bytes, f) : 0;
  fclose(f);
  if (!v || got != (size_t)bytes) {
    free(v);
    return NULL;
  }
  *count = bytes / (long)sizeof(double);
  return v;
}

static void print_matrix(const char *title, const double *m) {
  printf("%s\n", title);
  for (int i = 0; i < 16; i++) printf("%.12e%s", m[i], (i % 4 == 3) ? "\n" : "\t");
}

int main(int argc, char **argv) {
  pa_gridgen_opts o = {0.75 * 0.75, 0.5, 20, 0, 35, 20, NULL};
  const char *dir = "";
  for (int k = 1; k < argc; k++) {
    const char *a = argv[k];
    const char *v = k + 1 < argc ? argv[k + 1] : NULL;
    if (!strcmp(a, "-m") && v) {
      char buf[64];
      snprintf(buf, sizeof buf, "%f", atof(v) * atof(v)); /* main.cpp:172-190 */
      o.c0 = atof(buf);
      k++;
    } else if (!strcmp(a, "-c") && v) {
      o.c0 = atof(v);
      k++;
    } else if (!strcmp(a, "-n") && v) {
      o.nfft_exp = atoi(v) > 0 ? atoi(v) : 20;
      k++;
    } else if (!strcmp(a, "-a") && v) {
      o.method = !strcmp(v, "s1") ? 1 : !strcmp(v, "s2") ? 2 : 0;
      k++;
    } else if (!strcmp(a, "-i") && v) {
      o.xi = atof(v);
      k++;
    } else if (!strcmp(a, "-na") && v) {
      o.nalpha = atoi(v) > 0 ? atoi(v) : 35;
      k++;
    } else if (!strcmp(a, "-nr") && v) {
      o.nradius = atoi(v) > 0 ? atoi(v) : 20;
      k++;
    } else if (!strcmp(a, "-d") && v) {
      dir = v;
      k++;
    } else if (!strcmp(a, "-p") && v) {
      k++;
    } else {
      fprintf(stderr, "gridgen-gb300: unknown option %s\n", a);
      return 1;
    }
  }
  char p1[4096], p2[4096], p3[4096], pg[4096];
  snprintf(p1, sizeof p1, "%srSSB.bin", dir);
  snprintf(p2, sizeof p2, "%srDet.bin", dir);
  snprintf(p3, sizeof p3, "%sDetSSB.bin", dir);
  snprintf(pg, sizeof pg, "%sgrid.bin", dir);
  long long n1 = 0, n2 = 0, n3 = 0;
  double *ssb = read_all(p1, &n1), *det = read_all(p2, &n2), *dssb = read_all(p3, &n3);
  if (!ssb || !det || !dssb || n3 < 2) {
    fprintf(stderr, "gridgen-gb300: cannot read the ephemeris in '%s'\n", dir);
    return 1;
  }
  /* the obliquity: the last value of DetSSB.bin (ReadEphemeris.cpp:56-66) */
  const double epsm = dssb[n3 - 1];
  const long long n = n1 / 3 < n2 / 3 ? n1 / 3 : n2 / 3;
  FILE *t = fopen("dataS2.txt", "r");
  if (t) {
    fclose(t);
    o.table = "dataS2.txt";
  }
  pa_gridgen_out g;
  const int rc = pa_gridgen(ssb, det, n, epsm, &o, &g);
  free(ssb);
  free(det);
  free(dssb);
  if (rc) {
    fprintf(stderr, "gridgen-gb300: pa_gridgen failed (%d)\n", rc);
    return 1;
  }
  printf("grid.bin will be saved in %s\n", pg);
  printf("Method: S%d%s, density of covering: %.12f\n", g.method,
         g.method == 2 ? (g.alpha_from_table ? " (alpha from dataS2.txt)" : " (alpha computed)") : "", g.density);
  printf("fftpad: %d\n", g.fftpad);
  print_matrix("Normalized grid matrix:", g.M);
  print_matrix("Fisher matrix:", g.fisher);
  print_matrix("Grid matrix:", g.Mn);
  if (pa_gridgen_write(pg, &g)) {
    fprintf(stderr, "gridgen-gb300: cannot write %s\n", pg);
    return 1;
  }
  return 0;
}
