/*
 * polgraw_gb300.h -- C-ABI of the GB300 coherent-search library
 * (libpolgraw_gb300.so).
 *
 * The library replaces the per-sky-point F-statistic search of the Polgraw
 * all-sky network search, i.e. job_core() of
 *   search/network/src-cpu/jobcore.h:22-34   (declaration)
 *   search/network/src-cpu/jobcore.c:189-785 (definition)
 * which the sky loop search() calls once per (pm, mm, nn) at
 *   search/network/src-cpu/jobcore.c:107-120.
 * All signatures use plain C types and pointers; no CUDA or torch types
 * cross this boundary.  Every entry point returns a pa_status code and never
 * calls exit().
 *
 * Structs mirror the fields of the reference structs that the hot path reads:
 *   pa_settings  <- Search_settings      (struct.h:100-140)
 *   pa_detector  <- Detector_settings/Signals (struct.h:36-56, 154-171)
 *   pa_opts      <- Command_line_opts    (struct.h:16-32; fields read by job_core)
 *   pa_range     <- Search_range         (struct.h:70-73)
 * Candidate records are NPAR = 5 doubles [f, s1, delta, alpha, snr], the
 * byte layout of the reference's trigger files (jobcore.c:671-687,141).
 */
#ifndef POLGRAW_GB300_H
#define POLGRAW_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PA_NPAR 5            /* settings.h:7 */
#define PA_MAX_DETECTORS 8   /* struct.h:7 */
#define PA_NAV 4096          /* settings.h:12: nmin/nmax edge width (x B) */
#define PA_NAVFSTAT 4096     /* auxi.h:8: F-statistic normalisation block */
#define PA_MAXL 2048         /* struct.h:13: maximum number of veto lines */

typedef enum pa_status {
  PA_OK = 0,
  PA_ERR_ARG = 1,       /* invalid argument or size */
  PA_ERR_CUDA = 2,      /* a CUDA call failed; see pa_last_error() */
  PA_ERR_CAPACITY = 3,  /* caller's candidate buffer too small; *needed set */
  PA_ERR_TIMEOUT = 4,   /* a bounded device wait gave up */
  PA_ERR_NOMEM = 5,     /* device or host allocation failed */
  PA_ERR_NODEV = 6      /* no CUDA device / library built without CUDA */
} pa_status;

/* Arithmetic form of the search kernels. */
typedef enum pa_precision {
  PA_PREC_MIXED = 0,   /* FP32 data, FFTs and F-statistic; FP64 where needed */
  PA_PREC_FP64 = 1     /* every stage in FP64 (the comparison form) */
} pa_precision;

/* How the spindown phase het1*i + s1*(i^2 + 2 i shft_i) is formed in the
 * mixed form (the FP64 form always evaluates it in FP64). */
typedef enum pa_phase_mode {
  PA_PHASE_F64 = 0,    /* FP64 per sample, reduced mod 2 pi, FP32 sincos */
  PA_PHASE_FIXED = 1,  /* 64-bit fixed-point turns from FP64 per-sky terms */
  PA_PHASE_FF = 2      /* compensated two-float (float-float) phase */
} pa_phase_mode;

/* Search_settings subset (struct.h:100-140), filled like search_settings()
 * (settings.c:16-81), read_grid() (init.c:287-321) and plan_fftw()
 * (init.c:835-844). */
typedef struct pa_settings {
  double fpo, dt, B, oms, omr, Smin, Smax, sepsm, cepsm;
  int nfft, nod, N, nfftf, nmax, nmin, s, nd, interpftpad, fftpad, Ninterp, nifo;
  double M[16];              /* grid generator, column-major as in grid.bin */
  int numlines_band;         /* veto intervals in band radians */
  const double *lines;       /* 2*numlines_band doubles: [lo, hi] pairs */
} pa_settings;

/* One detector (struct.h:36-56 Signals + 154-171 Detector_settings). */
typedef struct pa_detector {
  const double *xDat;        /* N samples (after any injection) */
  const double *DetSSB;      /* 3N: detector position, x y z interleaved */
  double sig2;               /* crf0 * var(xDat), init.c:367-370 */
  double sphir, cphir;       /* sin/cos(phir), init.c:408-409 */
  double amod[9];            /* c1..c9 from rogcvir(), settings.c:264-272 */
} pa_detector;

/* Command_line_opts fields read by job_core(). */
typedef struct pa_opts {
  double trl;                /* F-statistic threshold (default 20) */
  int white_flag;            /* --whitenoise: skip FStat normalisation */
  int s0_flag;               /* --nospindown */
  int use_range;             /* nonzero when -addsig or -range was given
                                (jobcore.c:424: spindown range from s_range) */
} pa_opts;

/* Search_range (struct.h:70-73). */
typedef struct pa_range {
  int pmr[2], mr[2], nr[2], spndr[2];
  int pst, mst, nst, sst;
} pa_range;

/* Index side channel for each candidate record (not in the reference's
 * trigger files; the reference prints them with -DVERBOSE, jobcore.c:689). */
typedef struct pa_cand_idx {
  int pm, mm, nn, ss, ii;
  float F;                   /* normalised F-statistic of the record */
} pa_cand_idx;

typedef struct pa_config {
  int precision;             /* pa_precision */
  int phase_mode;            /* pa_phase_mode (mixed form only) */
  int spindown_batch;        /* spindowns per fused launch; 0 = automatic */
  int device;                /* CUDA device ordinal */
} pa_config;

typedef struct pa_ctx pa_ctx;

/* One sky point of a batch. */
typedef struct pa_sky {
  int pm, mm, nn;
} pa_sky;

/* Library version string. */
const char *pa_version(void);

/* Number of CUDA devices visible (0 if none). */
int pa_device_count(void);

/* Creates a search context: validates sizes, uploads the detector data and
 * ephemerides (replaces init_arrays' per-detector arrays, init.c:339-455,
 * and plan_fftw, init.c:810-862).  Input arrays are copied; the caller may
 * free them afterwards.  On failure returns NULL and sets *status. */
pa_ctx *pa_create(const pa_settings *sett, const pa_detector *det, int nifo,
                  const pa_config *cfg, int *status);

/* Replaces the detector data (xDat, DetSSB, sig2, amod) of an existing
 * context with new host arrays of the same N and nifo. */
int pa_set_data(pa_ctx *ctx, const pa_detector *det, int nifo);

void pa_destroy(pa_ctx *ctx);

/* Last error message of the context (or of the last failed pa_create when
 * ctx is NULL). */
const char *pa_last_error(const pa_ctx *ctx);

/* Drop-in for job_core() (jobcore.c:189-785).
 *   pm, mm, nn     : hemisphere and sky-grid indices
 *   opts, s_range  : as in the reference; s_range->sst and s_range->spndr[1]
 *                    give the spindown range when opts->use_range is set
 *   sgnlc, sgnlv   : caller's candidate count and record buffer (PA_NPAR
 *                    doubles per candidate, capacity sgnlv_cap candidates);
 *                    records are appended in the reference's serial order
 *                    (ss ascending, then frequency bin ascending)
 *   idx            : optional (may be NULL), parallel to sgnlv
 *   FNum           : incremented once per spindown, like jobcore.c:632
 * Returns PA_OK, or PA_ERR_CAPACITY with *needed = total candidates the call
 * would have produced (nothing is appended then), or another error.
 * A sky point outside the grid disk (jobcore.c:248) returns PA_OK with no
 * work, like the reference. */
int pa_job_core(pa_ctx *ctx, int pm, int mm, int nn, const pa_opts *opts,
                const pa_range *s_range, int *sgnlc, double *sgnlv,
                int sgnlv_cap, pa_cand_idx *idx, int *FNum, int *needed);

/* Batched form of the sky loop body: runs job_core() for ntasks sky points
 * with the work of several sky points in flight, then appends all records in
 * task order (each task's records in serial order).  Same buffer contract
 * as pa_job_core().  The spindown range per task follows the same rules;
 * with opts->use_range the first task starts at s_range->sst and later
 * tasks at s_range->spndr[0], as the sky loop resets sst after each sky
 * point (jobcore.c:123). */
int pa_search_batch(pa_ctx *ctx, const pa_sky *tasks, int ntasks,
                    const pa_opts *opts, const pa_range *s_range, int *sgnlc,
                    double *sgnlv, int sgnlv_cap, pa_cand_idx *idx, int *FNum,
                    int *needed);

/* Diagnostics used by the parity tests. */

/* Per-sky prelude outputs for one sky point: the resampled, weighted
 * xDatma/xDatmb of every detector (jobcore.c:270-393) as interleaved
 * (re, im) doubles, nifo*N complex each, plus aa and bb (jobcore.c:375-393).
 * Returns PA_ERR_ARG when the point is outside the grid disk. */
int pa_debug_prelude(pa_ctx *ctx, int pm, int mm, int nn, double *xDatma,
                     double *xDatmb, double *aa, double *bb);

/* F-statistic after normalisation (jobcore.c:635-651) for one spindown ss
 * of one sky point: nmax-nmin doubles written to F. */
int pa_debug_fstat(pa_ctx *ctx, int pm, int mm, int nn, int ss,
                   const pa_opts *opts, double *F);

/* Normalised F-statistic of one template, like pa_debug_fstat() on a
 * mixed-precision, fixed-point-phase context, but without allocating
 * anything: for callers that cannot call cudaMalloc (a plugin inside a host
 * application that owns the GPU memory, code that must not grow its
 * footprint or synchronise the device with an allocation).  No counterpart
 * in the reference.  Inputs (settings, detector data) and the output F
 * (nmax-nmin doubles) are host memory; all device storage is one static
 * 16 MB array in the library, so sizes are limited to N <= 16384,
 * nfft <= 16384, nfftf <= 32768, nifo <= 3 (larger ones return PA_ERR_ARG
 * with the reason in pa_last_error(NULL)).  The first call on a device sets
 * up the array's device address and should come before any stream
 * capture.  Calls share the array: they are serialised on the host, and
 * calls that overlap on the same GPU race. */
int pa_fstat_noalloc(const pa_settings *sett, const pa_detector *det, int nifo,
                     int pm, int mm, int nn, int ss, const pa_opts *opts,
                     int device, double *F);

/* Number of CUDA kernel launches issued by this context so far. */
long long pa_kernel_launches(const pa_ctx *ctx);

/* Device time in milliseconds of the last pa_job_core/pa_search_batch call,
 * from CUDA events recorded on the context's stream before its first and
 * after its last kernel (the reference's analogue is the wall-clock
 * "Time elapsed" of jobcore.c:178-182). */
double pa_last_call_ms(const pa_ctx *ctx);

/* Per-kernel profile: when on, every kernel launch of the context is
 * bracketed by CUDA events on its stream and its duration accumulated per
 * kernel kind (adds a small overhead; off by default). */
int pa_set_profiling(pa_ctx *ctx, int on);
void pa_profile_reset(pa_ctx *ctx);
/* Totals of kernel kind `kind` (0, 1, ...); returns PA_ERR_ARG past the
 * last kind.  `items` counts the batch entries (spindowns or detectors)
 * the launches processed. */
int pa_profile_get(const pa_ctx *ctx, int kind, const char **name, double *total_ms,
                   long long *launches, long long *items);

#ifdef __cplusplus
}
#endif

#endif /* POLGRAW_GB300_H */
