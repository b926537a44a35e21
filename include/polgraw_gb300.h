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
/* settings.h:14,20: mean obliquity of the ecliptic, the epsm of ast2lin() */
#define PA_C_EPSMA (84381.448 / 3600. / (180 / M_PI))

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

/* Last error message of the context (or, with ctx NULL, of this thread's
 * last failed pa_create). */
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
 * with the reason in pa_last_error(NULL)).  The first call on a device --
 * and the first after that device's context was reset or replaced -- looks
 * up the array's device address and should come before any stream capture.
 * Calls share the array: they are serialised on the host (each waits for
 * its own GPU work, also when it fails), and calls that overlap on the same
 * GPU race.  The caller's current device is restored on return. */
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
 * kernel kind (adds a small overhead; off by default).  While it is on the
 * context runs its kernels one at a time (the preludes on the main stream,
 * one spindown lane, no graphs), so that each duration is that kernel's
 * own; the records are the same. */
int pa_set_profiling(pa_ctx *ctx, int on);
void pa_profile_reset(pa_ctx *ctx);
/* Totals of kernel kind `kind` (0, 1, ...); returns PA_ERR_ARG past the
 * last kind.  `items` counts the batch entries (spindowns or detectors)
 * the launches processed. */
int pa_profile_get(const pa_ctx *ctx, int kind, const char **name, double *total_ms,
                   long long *launches, long long *items);

/* Per-CTA trace of the context's kernels (a diagnostic of the launch
 * structure: gaps between kernels, partial waves).  dev_buf: device memory
 * for cap records of 48 bytes, {start %globaltimer ns, end %globaltimer ns,
 * start clock64, end clock64 (uint64 each), kernel kind, SM id, 2 x pad
 * (uint32 each)}, one per CTA, appended in completion order by the CTA's
 * thread 0; NULL switches the trace off (the default).  Setting it resets
 * the count.  pa_cta_trace_count: records written since (may exceed cap;
 * the excess is dropped).  Kernel kinds are those of pa_profile_get.
 * Only the diagnostic build of the library (compiled with -DPA_CTA_TRACE)
 * records the trace; the product build returns PA_ERR_CUDA with "operation
 * not supported". */
int pa_set_cta_trace(pa_ctx *ctx, void *dev_buf, unsigned int cap);
int pa_cta_trace_count(pa_ctx *ctx, unsigned int *n);

/* ------------------------------------------------------------------------
 * Launch schedule, CUDA graphs and the multi-segment front-end.  No
 * counterpart in the reference (one process per segment and sky range,
 * search/network/src-cpu/jobcore.c:51-184).
 * ------------------------------------------------------------------------ */

/* CUDA graphs on/off (default off): when on, each pa_search_batch /
 * pa_job_core call captures its launches (both streams) into a CUDA graph,
 * updated in place when the next call has the same launch structure, and
 * launches it once.  Results are identical either way. */
int pa_set_graphs(pa_ctx *ctx, int on);

/* Spindown-loop schedule: spindowns per fused launch (1 .. *max_sbatch, the
 * batch the buffers were sized for, four times the automatic default; a
 * batch above *max_sbatch / 2 selects one lane, see pa_set_lanes) and the
 * factor split of the spindown FFT (0: L1 = 2^ceil(m/2); 1: swapped
 * factors, different radix schedule of the two passes; for odd
 * m = log2(nfftf) only, ignored otherwise; default 0, except 1 for two
 * detectors in the FP32 forms with nfftf = 2^17, whose 256-point columns
 * take the radix-16 pass A). */
int pa_set_schedule(pa_ctx *ctx, int sbatch, int split);
int pa_get_schedule(const pa_ctx *ctx, int *sbatch, int *split, int *max_sbatch);

/* Spindown lanes: 1 (every spindown launch on the context's main stream) or
 * 2 (consecutive spindown launches alternate between two streams, each with
 * its own half of the FFT intermediate and F buffers, so that one launch's
 * FFT passes run beside the previous launch's).  Two lanes need a spindown
 * batch of at most *max_sbatch / 2 (PA_ERR_ARG otherwise: set the batch
 * first).  Default: 2 when the configured batch allows it, else 1.  Results
 * are identical either way; while the per-launch profile is on, one lane is
 * used. */
int pa_set_lanes(pa_ctx *ctx, int lanes);
int pa_get_lanes(const pa_ctx *ctx, int *lanes);

/* Times the candidate schedules (one lane with spindown batches of 1/4 ..
 * 4/4 of the maximum, two lanes with 1/4 and 1/2, each x the possible
 * splits) on the given sky points (each searched three times, the first as
 * warm-up, CUDA-event device time) and keeps the fastest; returns it in
 * *sbatch, *split (either may be NULL; the lane count it picked is read
 * with pa_get_lanes).  Results do not depend on sbatch or the lanes; the
 * split changes FFT rounding only. */
int pa_autotune(pa_ctx *ctx, const pa_sky *tasks, int ntasks, const pa_opts *opts, const pa_range *s_range,
                int *sbatch, int *split);

/* Several data segments searched together: one context per segment (own
 * N, FFT lengths, data), their batches enqueued at once on their own
 * streams, forked from one origin stream, so that the GPU runs them
 * concurrently; with the graph on (default) the whole multi-segment
 * workload is captured into one CUDA graph (updated in place on the next
 * call with the same launch structure) and launched once. */
typedef struct pa_segments pa_segments;

/* One segment's batch: the arguments of pa_search_batch() for context k. */
typedef struct pa_segment_job {
  const pa_sky *tasks;
  int ntasks;
  const pa_opts *opts;
  const pa_range *range;
  int *sgnlc;
  double *sgnlv;
  int cap;
  pa_cand_idx *idx;
  int *FNum;
  int *needed;
} pa_segment_job;

/* The contexts stay owned by the caller and must outlive the handle; all on
 * one device. */
pa_segments *pa_segments_create(pa_ctx *const *ctxs, int nseg, int *status);
void pa_segments_destroy(pa_segments *seg);
const char *pa_segments_last_error(const pa_segments *seg);
int pa_segments_set_graph(pa_segments *seg, int on);
/* jobs[k] runs on context k; status[k] (may be NULL) receives each
 * segment's result as pa_search_batch() would return it; the return value
 * is the first non-OK status.  Records are appended per segment exactly as
 * pa_search_batch() on that context would append them. */
int pa_segments_search(pa_segments *seg, const pa_segment_job *jobs, int *status);
/* Device time of the last pa_segments_search (CUDA events on the origin
 * stream around all segments). */
double pa_segments_last_call_ms(const pa_segments *seg);

/* ------------------------------------------------------------------------
 * Followup: the demodulated network F-statistic of followup/src/followup.c
 * at arbitrary (f, s, delta, alpha), its adjoint gradient, and maximisers.
 * A point is sgnlo = (f [rad/sample], s [rad/sample^2], delta, alpha [rad])
 * as in followup.c (sgnlo[0..3]).
 * ------------------------------------------------------------------------ */
typedef struct pa_followup pa_followup;

/* Options of pa_followup_ascent(). */
typedef struct pa_ascent_opts {
  double scale[4];   /* parameter scales of (f, s, delta, alpha): steps are
                        measured in these units (e.g. the peak widths
                        2pi/N, 2pi/N^2 and the sky widths); must be > 0 */
  double step0;      /* first step length in scale units (<= 0: 0.25) */
  double min_step;   /* a point stops when its step falls below this
                        (<= 0: 1e-3) */
  int max_iter;      /* iteration limit (<= 0: 100) */
} pa_ascent_opts;

/* Device copies of the data the followup program reads (xDat, DetSSB,
 * sig2, phir, c1..c9 per detector; followup init.c:326-460) and the
 * cos/sin(omr i) tables of its init_arrays() (followup init.c:464-475).
 * Uses sett->N, oms, omr; cfg->precision selects FP32 data with FP64 phase
 * (PA_PREC_MIXED) or every stage in FP64 (PA_PREC_FP64); cfg->device. */
pa_followup *pa_followup_create(const pa_settings *sett, const pa_detector *det, int nifo,
                                const pa_config *cfg, int *status);
void pa_followup_destroy(pa_followup *fu);
/* Last error of fu, or of the last failed pa_followup_create() of this
 * thread when fu is NULL. */
const char *pa_followup_last_error(const pa_followup *fu);

/* Fstatnet() (followup.c:413-535) with the sky set-up of evaluate_simplex()
 * (followup.c:986-1009) at n points sgnlo[n][4]; out[n][11] as the
 * reference's fstat_out: out[0..3] amplitude estimates, out[4] SNR
 * sqrt(2(F-2)), out[5] = -F, out[6..9] the point, out[10] SNR from the
 * amplitudes. */
int pa_fstatnet(pa_followup *fu, const double *sgnlo, int n, double *out);

/* F (= -out[5] of pa_fstatnet) and grad[n][4] = seed[k] dF/d(f, s, delta,
 * alpha) at n points, by a forward pass and an adjoint (reverse) pass that
 * recomputes the phase instead of storing it.  seed may be NULL (all 1).
 * No counterpart in the reference, whose followup maximises without
 * gradients (simplex, MADS). */
int pa_fstatnet_grad(pa_followup *fu, const double *sgnlo, int n, const double *seed, double *F,
                     double *grad);

/* Gradient ascent of F from n starting points sgnlo[n][4] (replaced by the
 * final points), all points in lockstep on the device: quasi-Newton (BFGS)
 * steps in scale units from the adjoint gradient, with a backtracking line
 * search (a step is accepted when F grows by at least 1e-4 of the predicted
 * gain, halved otherwise); the first step has length step0; a point stops
 * when its step falls below min_step.  out[n][11] as pa_fstatnet() at the
 * final points; iters[n] (may be NULL) the accepted steps.  No counterpart
 * in the reference: it refines followup candidates beside the simplex
 * (followup.c:1126-1174). */
int pa_followup_ascent(pa_followup *fu, double *sgnlo, int n, const pa_ascent_opts *opts,
                       double *out, int *iters);

/* The reference simplex amoeba() (followup.c:971-1174) for n starting
 * points at once, their F-statistic evaluations batched on the device:
 * initial steps pc2[4], relative tolerance tol (the reference program uses
 * 1e-7).  max_evals > 0 bounds the evaluations per point (the reference
 * loops until the tolerance holds).  sgnlo[n][4] is replaced by the best
 * vertex, out[n][11] is its fstat_out, nevals[n] (may be NULL) the
 * evaluations made. */
int pa_followup_simplex(pa_followup *fu, double *sgnlo, int n, const double *pc2, double tol,
                        int max_evals, double *out, int *nevals);

/* Device time of the last followup call (CUDA events on its stream), and
 * the number of kernel launches so far. */
double pa_followup_last_call_ms(const pa_followup *fu);
long long pa_followup_kernel_launches(const pa_followup *fu);

/* ------------------------------------------------------------------------
 * Coincidences among the trigger files of several time frames (segments):
 * the consumer of the search's trigger files, read_trigger_files() of
 * coincidences/src/coincidences.c:117-600, with the per-trigger cell
 * assignment, the per-frame duplicate removal and the coincidence count on
 * the device.  The trigger files themselves are read unchanged (5 doubles
 * f, s, delta, alpha, SNR per record: coincidences.c:229).
 * ------------------------------------------------------------------------ */

typedef struct pa_coinc pa_coinc;

typedef struct pa_coinc_cfg {
  int N;                   /* samples of a segment, search_settings() (settings.c:32) */
  double oms;              /* 2 pi fpo dt (settings.c:28) */
  double vedva[4][4];      /* eigenvectors x sqrt(eigenvalues) of the grid's
                              Fisher matrix (init.c:1195-1210); see pa_coinc_vedva */
  int shift[4];            /* cell shifts in f, s, delta, alpha (digits of -shift) */
  int scale[4];            /* cell scaling (digits of -scale; a 0 digit means 1) */
  int refr;                /* reference frame number (-refr) */
  double narrowdown;       /* half-width of the kept band around pi/2, radians
                              (-narrowdown times pi, init.c:1111) */
  double snrcutoff;        /* keep SNR > snrcutoff (-snrcutoff) */
  int mincoin;             /* minimal coincidence multiplicity (-mincoin, >= 1) */
  int device;              /* CUDA device ordinal */
} pa_coinc_cfg;

/* One coincidence as coincidences.c:488-541 writes it: multiplicity w, the
 * FP64 means of f, s, delta, alpha over the members and sqrt of the sum of
 * squared SNRs (the file stores them as float), and the offset of its w
 * members in the member arrays (frame numbers and record positions, in the
 * reference's order). */
typedef struct pa_coinc_rec {
  int w;
  int first;               /* index of the first member */
  double mean[5];
} pa_coinc_rec;

/* Sizes and per-frame counts after pa_coinc_run(). */
typedef struct pa_coinc_summary {
  int nframes;
  long long raw;           /* records read */
  long long inband;        /* records passing the band and SNR cuts */
  long long unique;        /* records left after the per-frame duplicate removal */
  int ncoin;               /* coincidence records to write (coincidences.c:488) */
  long long nmembers;      /* sum of their multiplicities */
  int maxcoin;             /* largest multiplicity (0: none) */
  int maxcoin_index;       /* record with maxcoin and the largest mean SNR */
  long long fp64_cells;    /* in-band records whose cells were recomputed in
                              FP64 (near a rounding edge of the fast path) */
} pa_coinc_summary;

/* Host: vedva[i][j] = eigvec[i][j] sqrt(eigval[j]) of the symmetric 4x4
 * matrix fisher[16] (row-major; the second matrix of grid.bin,
 * init.c:1167-1172), by cyclic Jacobi rotations (eigenvalues in the order
 * the rotations leave them, no sorting). */
int pa_coinc_vedva(const double *fisher, double *vedva);

pa_coinc *pa_coinc_create(const pa_coinc_cfg *cfg, int *status);
void pa_coinc_destroy(pa_coinc *cc);
/* Last error message of the handle (or, with cc NULL, of this thread's last
 * failed pa_coinc_create). */
const char *pa_coinc_last_error(const pa_coinc *cc);
/* Starts a new set of frames (keeps the device buffers). */
int pa_coinc_reset(pa_coinc *cc);
/* Appends one trigger file's records (host memory, n x 5 doubles) as frame
 * `frame` (the number parsed from the file name, coincidences.c:206-215);
 * frames are taken in the order they are added (the reference's directory
 * order).  At most 255 frames (Candidate_triggers.frameinfo[256]). */
int pa_coinc_add_frame(pa_coinc *cc, int frame, const double *records, long long n);
/* Cells, duplicate removal, coincidences.  Fills *sum. */
int pa_coinc_run(pa_coinc *cc, pa_coinc_summary *sum);
/* Results of the last run, each array optional (NULL): per-frame
 * frameinfo[nframes][3] = {frame, in-band, unique} (coincidences.c:305-421);
 * recs[ncoin]; member frame numbers fra[nmembers] and record positions
 * ops[nmembers] (position in the frame's trigger file). */
int pa_coinc_get(const pa_coinc *cc, int *frameinfo, pa_coinc_rec *recs, int *fra, int *ops);
/* The pre-binning itself: for the in-band records of the last run in read
 * order (frame by frame), cells[inband][4] (fi, si, di, ai of
 * coincidences.c:256-261) and keep[inband] = 1 for the record each
 * frame's duplicate removal keeps. */
int pa_coinc_cells(pa_coinc *cc, int *cells, unsigned char *keep);
double pa_coinc_last_call_ms(const pa_coinc *cc);
long long pa_coinc_kernel_launches(const pa_coinc *cc);
/* Per-kernel profile of the following runs (CUDA events around every
 * launch; resets the totals).  pa_coinc_profile_get: totals of kernel kind
 * `kind` (0, 1, ...), PA_ERR_ARG past the last kind. */
int pa_coinc_set_profiling(pa_coinc *cc, int on);
int pa_coinc_profile_get(const pa_coinc *cc, int kind, const char **name, double *total_ms, long long *launches);

#ifdef __cplusplus
}
#endif

#endif /* POLGRAW_GB300_H */
