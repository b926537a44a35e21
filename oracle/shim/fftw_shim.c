/*
 * oracle/shim/fftw_shim.c -- implementation of the FFTW3-API shim.
 * TEST INFRASTRUCTURE ONLY; see fftw3.h.
 *
 * Plans are kept in a registry so that fftw_destroy_plan() on a handle that
 * was never created is a no-op: the reference's cleanup() destroys plan2,
 * pl_int2 and pl_inv2 (src-cpu/init.c:955-959), which plan_fftw() never
 * assigns (init.c:848-852) and which live in an uninitialised stack struct
 * (main.c:128).  Real FFTW would be handed garbage there as well.
 */
#include "fftw3.h"

#include <pthread.h>
#include <stdlib.h>

#include "../fft.h"

struct pa_shim_fftw_plan_s {
  oracle_fft_plan *fft;
  fftw_complex *in, *out;           /* arrays given at planning time */
  struct pa_shim_fftw_plan_s *next; /* registry link */
};

static struct pa_shim_fftw_plan_s *g_plans = NULL;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

fftw_plan fftw_plan_dft_1d(int n, fftw_complex *in, fftw_complex *out,
                           int sign, unsigned flags) {
  (void)flags;
  oracle_fft_plan *f = oracle_fft_plan_create(n, sign);
  if (!f) {
    fprintf(stderr, "fftw shim: length %d is not a power of two\n", n);
    return NULL;
  }
  struct pa_shim_fftw_plan_s *p =
      (struct pa_shim_fftw_plan_s *)calloc(1, sizeof(*p));
  p->fft = f;
  p->in = in;
  p->out = out;
  pthread_mutex_lock(&g_lock);
  p->next = g_plans;
  g_plans = p;
  pthread_mutex_unlock(&g_lock);
  return p;
}

void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
  oracle_fft_exec(p->fft, (const double complex *)in, (double complex *)out);
}

void fftw_execute(const fftw_plan p) { fftw_execute_dft(p, p->in, p->out); }

void fftw_destroy_plan(fftw_plan p) {
  pthread_mutex_lock(&g_lock);
  struct pa_shim_fftw_plan_s **pp = &g_plans;
  while (*pp && *pp != p) pp = &(*pp)->next;
  if (*pp) {
    *pp = p->next;
    oracle_fft_plan_destroy(p->fft);
    free(p);
  }
  pthread_mutex_unlock(&g_lock);
}

void *fftw_malloc(size_t n) {
  void *p = NULL;
  if (posix_memalign(&p, 64, n ? n : 1)) return NULL;
  return p;
}

void fftw_free(void *p) { free(p); }

int fftw_import_wisdom_from_file(FILE *input_file) {
  (void)input_file;
  return 1;
}

void fftw_export_wisdom_to_file(FILE *output_file) {
  if (output_file) fprintf(output_file, "(fftw shim: no wisdom)\n");
}

void fftw_forget_wisdom(void) {}
void fftw_cleanup(void) {}
int fftw_init_threads(void) { return 1; }
void fftw_plan_with_nthreads(int nthreads) { (void)nthreads; }
void fftw_cleanup_threads(void) {}
