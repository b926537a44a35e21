/*
 * pa_grid.c -- input generation: the reduced Fisher matrix that the grid
 * generator writes into grid.bin (second 4x4 matrix) and that the
 * coincidence step diagonalises for its cells.
 *
 * Restates gridgen/src/ReadEphemeris.cpp:24-100 (ephemeris scaling),
 * gridgen/src/FisherRM.cpp:17-100 (prefisher integrals, postrmf) and the
 * composite Simpson rule of gridgen/src/num.cpp:20-119 with the same
 * arithmetic order, so that the matrix equals the grid generator's bit for
 * bit.  Host code: O(N) work once per segment.
 */
#include <math.h>
#include <stdlib.h>

#include "../../include/polgraw_gb300_host.h"

/* composite Simpson on [0, 1] over n samples of v1[i] * v2[i] (v2 NULL: 1);
 * an even n takes Simpson over the first n - 1 samples and the trapezoid on
 * the last interval */
static double simpson2(const double *v1, const double *v2, long long n) {
  const double dx = 1.0 / (double)(n - 1);
  double sum = 0.0, sum1 = 0.0, sum2 = 0.0;
  const double a = dx * (4.0 / 3.0), b = dx * (2.0 / 3.0), c = dx / 3.0;
#define PROD(i) (v2 ? v1[i] * v2[i] : v1[i])
  const long long last = (n % 2 == 1) ? n - 1 : n - 2; /* end point of the Simpson part */
  for (long long i = 1; i < last; i += 2) sum1 += PROD(i);
  for (long long i = 2; i < last - 1; i += 2) sum2 += PROD(i);
  sum1 *= a;
  sum2 *= b;
  sum += sum1;
  sum += sum2;
  if (v2) {
    sum += c * v1[0] * v2[0];
    sum += c * v1[last] * v2[last];
    if (n % 2 == 0) sum += (dx * 0.5) * (v1[n - 2] * v2[n - 2] + v1[n - 1] * v2[n - 1]);
  } else {
    sum += c * v1[0];
    sum += c * v1[last];
    if (n % 2 == 0) sum += (dx * 0.5) * (v1[n - 2] + v1[n - 1]);
  }
#undef PROD
  return sum;
}

int pa_fisher_reduced(const double *rSSB, const double *rDet, long long n, double epsm, double xi,
                      double *fisher) {
  if (!rSSB || !rDet || !fisher || n < 5) return PA_ERR_ARG;
  double *e1 = (double *)malloc(sizeof(double) * (size_t)n);
  double *e2 = (double *)malloc(sizeof(double) * (size_t)n);
  double *x = (double *)malloc(sizeof(double) * (size_t)n);
  double *x2 = (double *)malloc(sizeof(double) * (size_t)n);
  if (!e1 || !e2 || !x || !x2) {
    free(e1);
    free(e2);
    free(x);
    free(x2);
    return PA_ERR_NOMEM;
  }
  /* ReadEphemeris: the ecliptic y and the x coordinate, scaled by 1/n */
  const double ce = cos(epsm);
  const double ws = 1.0 / (double)n;
  for (long long j = 0; j < n; j++) {
    e1[j] = ws * (rSSB[3 * j + 1] / ce + rDet[3 * j + 1] * ce);
    e2[j] = ws * (rSSB[3 * j] + rDet[3 * j]);
  }
  for (long long i = 0; i < n; i++) {
    x[i] = ((double)i / (double)(n - 1)) - 0.5;
    x2[i] = x[i] * x[i];
  }
  double p[9];
  p[0] = simpson2(e1, NULL, n);
  p[1] = simpson2(e2, NULL, n);
  p[2] = simpson2(x, e1, n);
  p[3] = simpson2(x, e2, n);
  p[4] = simpson2(x2, e1, n);
  p[5] = simpson2(x2, e2, n);
  p[6] = simpson2(e1, e1, n);
  p[7] = simpson2(e1, e2, n);
  p[8] = simpson2(e2, e2, n);
  free(e1);
  free(e2);
  free(x);
  free(x2);
  /* postrmf(xi), row-major 4x4 */
  for (int k = 0; k < 16; k++) fisher[k] = 0.0;
  fisher[0] = 1.0 / 12.0;
  fisher[5] = 1.0 / 180.0 + (xi * xi) / 3.0;
  fisher[10] = -(p[0] * p[0]) + p[6];
  fisher[15] = -(p[1] * p[1]) + p[8];
  fisher[1] = fisher[4] = xi / 6.0;
  fisher[2] = fisher[8] = p[2];
  fisher[3] = fisher[12] = p[3];
  fisher[6] = fisher[9] = p[4] + (2.0 * xi * p[2]) - p[0] / 12.0;
  fisher[7] = fisher[13] = p[5] + (2.0 * xi * p[3]) - p[1] / 12.0;
  fisher[11] = fisher[14] = -(p[0] * p[1]) + p[7];
  return PA_OK;
}
