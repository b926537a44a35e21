// pa_api.cu -- the C-ABI of libpolgraw_gb300.so (include/polgraw_gb300.h).
//
// Host logic of job_core() around the device engine: sky-point scalars
// (jobcore.c:243-299), spindown range (jobcore.c:424-444), candidate
// records and the line veto (jobcore.c:670-687).  All FP64 host arithmetic
// follows the reference expressions so that for the same (ss, ii) the
// f, s1, delta, alpha fields of a record are bit-identical to the
// reference's; this file is compiled with -ffp-contract=off for that.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/polgraw_gb300.h"
#include "pa_trace.h"
#include "pa_engine.h"

#define SQR(x) ((x) * (x))

namespace {

thread_local std::string g_create_error;

struct Twiddles {
  void* p[4] = {nullptr, nullptr, nullptr, nullptr};
};

}  // namespace

struct pa_ctx {
  pa_settings sett;
  std::vector<double> lines;
  int nifo = 0;
  pa_config cfg;
  bool fp64 = false;
  size_t rsz = 4;  // bytes of the Real type
  pa::DetConst dc[pa::kMaxDet];
  double det0[pa::kMaxDet][3];  // DetSSB of sample 0 (shft1)
  int dev = 0;
  cudaStream_t stream = nullptr;      // spindown loop, copies
  cudaStream_t stream_pre = nullptr;  // per-sky preludes
  cudaStream_t stream2 = nullptr;     // spindown lane 1
  cudaEvent_t ev_pre[2] = {nullptr, nullptr}, ev_spin[2] = {nullptr, nullptr};
  cudaEvent_t ev_spin2[2] = {nullptr, nullptr};  // lane 1's last reads of each prelude slot
  pa::Buffers b;
  std::vector<void*> allocs;
  Twiddles tw_fwd, tw_inv, tw_invh, tw_main;
  pa::Engine* eng = nullptr;
  pa::DevCand* h_cand = nullptr;  // pinned
  int* h_ncand = nullptr;          // pinned
  std::string err;
  long long extra_launches = 0;
  pa::Prof prof;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double last_ms = 0.;
  // CUDA graphs of a batch, one per part of the batch (captured launches,
  // updated in place when the next batch has the same launch structure)
  bool graphs = false;
  std::vector<cudaGraphExec_t> gexec_parts;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_join2 = nullptr;
  int sb_max = 0;  // spindown batch the buffers are sized for
  // spindown lanes: 1, or 2 (consecutive batches alternate between the main
  // stream and stream2, each with its own half of ybuf and F, so that one
  // batch's FFT passes run beside the previous batch's)
  int lanes = 2;
};

// Lanes used by the next enqueue, and the stream of the preludes: while the
// per-launch profile is on, one lane and the preludes on the main stream, so
// that every kernel runs alone and its events time that kernel only.
static int active_lanes(const pa_ctx* c) { return c->prof.on ? 1 : c->lanes; }
static cudaStream_t prelude_stream(const pa_ctx* c) { return c->prof.on ? c->stream : c->stream_pre; }

// sky points per captured part of a batch (launch_tasks): the first part
// kGraphFirst, each next one twice the previous, up to kGraphPart
constexpr size_t kGraphFirst = 16;
constexpr size_t kGraphPart = 256;

static void drop_graphs(pa_ctx* c) {
  for (auto& g : c->gexec_parts)
    if (g) cudaGraphExecDestroy(g);
  c->gexec_parts.clear();
}

namespace pa {
const char* kernel_kind_name(int k) {
  static const char* names[KK_COUNT] = {"prelude_mod", "resample_fft_fwd_a", "resample_fft_fwd_b",
                                        "resample_fft_inv_a", "resample_fft_inv_b", "spline_fwd",
                                        "spline_bwd", "splint", "spindown_pass_a", "spindown_pass_b_fstat",
                                        "threshold"};
  return (k >= 0 && k < KK_COUNT) ? names[k] : "";
}
}  // namespace pa

// Accumulates the recorded per-launch events after the stream finished.
static void prof_collect(pa_ctx* c) {
  pa::Prof& p = c->prof;
  for (int i = 0; i < p.n; i++) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.recs[i].a, p.recs[i].b) == cudaSuccess) {
      p.total_ms[p.recs[i].kind] += ms;
      p.launches[p.recs[i].kind] += 1;
      p.items[p.recs[i].kind] += p.recs[i].items;
    }
  }
  p.n = 0;
  cudaGetLastError();
}

static int fail(pa_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf;
  else g_create_error = buf;
  return code;
}

static int cuda_fail(pa_ctx* c, cudaError_t e, const char* what) {
  return fail(c, PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define CK(call, what)                               \
  do {                                               \
    cudaError_t e_ = (call);                         \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, what); \
  } while (0)

static int dalloc(pa_ctx* c, void** p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  c->allocs.push_back(*p);
  return PA_OK;
}

// exp(sign 2 pi i m / n) in FP64 with the angle folded to the first octant
static void host_twiddle(long m, long n, int sign, double* re, double* im) {
  long m8 = 8 * (m % n);
  long oct = m8 / n, rem = m8 - oct * n;
  double a = (oct & 1) ? (double)(n - rem) / (double)n * (M_PI / 4.0) : (double)rem / (double)n * (M_PI / 4.0);
  double ca = cos(a), sa = sin(a), co, si;
  switch (oct) {
    case 0: co = ca; si = sa; break;
    case 1: co = sa; si = ca; break;
    case 2: co = -sa; si = ca; break;
    case 3: co = -ca; si = sa; break;
    case 4: co = -ca; si = -sa; break;
    case 5: co = -sa; si = -ca; break;
    case 6: co = sa; si = -ca; break;
    default: co = ca; si = -sa; break;
  }
  *re = co;
  *im = sign * si;
}

static int upload_real(pa_ctx* c, void* dst, const std::vector<double>& v) {
  if (c->fp64) {
    CK(cudaMemcpy(dst, v.data(), v.size() * 8, cudaMemcpyHostToDevice), "upload");
  } else {
    std::vector<float> f(v.size());
    for (size_t i = 0; i < v.size(); i++) f[i] = (float)v[i];
    CK(cudaMemcpy(dst, f.data(), f.size() * 4, cudaMemcpyHostToDevice), "upload");
  }
  return PA_OK;
}

// tw1 (L1), tw2 (L2), twlo (1024), twhi (L/1024) for length L and sign
static int make_twiddles(pa_ctx* c, int L, int sign, Twiddles* t) {
  int m = 0;
  while ((1 << m) < L) ++m;
  const int L1 = 1 << ((m + 1) / 2), L2 = 1 << (m / 2);
  const int lens[4] = {L1, L2, 1024, L / 1024};
  for (int k = 0; k < 4; k++) {
    std::vector<double> v(2 * (size_t)lens[k]);
    for (int j = 0; j < lens[k]; j++) {
      long num, den;
      if (k == 0) { num = j; den = L1; }
      else if (k == 1) { num = j; den = L2; }
      else if (k == 2) { num = j; den = L; }
      else { num = (long)j * 1024; den = L; }
      host_twiddle(num, den, sign, &v[2 * j], &v[2 * j + 1]);
    }
    int rc = dalloc(c, &t->p[k], v.size() * c->rsz);
    if (rc) return rc;
    rc = upload_real(c, t->p[k], v);
    if (rc) return rc;
  }
  return PA_OK;
}

static void set_det_consts(pa_ctx* c, const pa_detector* det) {
  for (int n = 0; n < c->nifo; n++) {
    pa::DetConst& d = c->dc[n];
    memcpy(d.amod, det[n].amod, sizeof(d.amod));
    d.sig2 = det[n].sig2;
    d.inv_sig2 = 1.0 / det[n].sig2;
    d.sphir = det[n].sphir;
    d.cphir = det[n].cphir;
    for (int k = 0; k < 9; k++) d.amod_f[k] = (float)d.amod[k];
    d.inv_sig2_f = (float)d.inv_sig2;
    for (int k = 0; k < 3; k++) c->det0[n][k] = det[n].DetSSB[k];
  }
}

static int upload_data(pa_ctx* c, const pa_detector* det) {
  const int N = c->sett.N;
  for (int n = 0; n < c->nifo; n++) {
    CK(cudaMemcpyAsync((double*)c->b.xDat + (size_t)n * N, det[n].xDat, sizeof(double) * N,
                       cudaMemcpyHostToDevice, c->stream), "upload xDat");
    CK(cudaMemcpyAsync((double*)c->b.DetSSB + (size_t)n * 3 * N, det[n].DetSSB, sizeof(double) * 3 * N,
                       cudaMemcpyHostToDevice, c->stream), "upload DetSSB");
  }
  set_det_consts(c, det);
  CK(cudaMemcpyAsync((void*)c->b.dc, c->dc, sizeof(pa::DetConst) * c->nifo, cudaMemcpyHostToDevice,
                     c->stream), "upload detector constants");
  CK(cudaStreamSynchronize(c->stream), "upload sync");
  return PA_OK;
}

static int validate(const pa_settings* s, int nifo, const pa_config* cfg, char* why, size_t n) {
  auto ispow2 = [](int v) { return v > 0 && (v & (v - 1)) == 0; };
  if (nifo < 1 || nifo > PA_MAX_DETECTORS) return snprintf(why, n, "nifo=%d outside [1,%d]", nifo, PA_MAX_DETECTORS), 1;
  if (s->N < 2) return snprintf(why, n, "N=%d too small", s->N), 1;
  if (!ispow2(s->nfft) || s->nfft < 4096 || s->nfft > (1 << 19))
    return snprintf(why, n, "nfft=%d must be a power of two in [4096, 2^19]", s->nfft), 1;
  if (s->nfft < s->N) return snprintf(why, n, "nfft=%d < N=%d", s->nfft, s->N), 1;
  if (s->interpftpad != 2) return snprintf(why, n, "interpftpad=%d (only 2 is supported, as in settings.c:56)", s->interpftpad), 1;
  if (s->Ninterp != s->interpftpad * s->nfft) return snprintf(why, n, "Ninterp != interpftpad*nfft"), 1;
  if (s->fftpad < 1 || s->nfftf != s->fftpad * s->nfft || !ispow2(s->nfftf) || s->nfftf > (1 << 20))
    return snprintf(why, n, "nfftf=%d must be fftpad*nfft, a power of two <= 2^20", s->nfftf), 1;
  if (s->nmin < 0 || s->nmax > s->nfftf || s->nmax <= s->nmin)
    return snprintf(why, n, "bad F-statistic range [%d, %d)", s->nmin, s->nmax), 1;
  if (s->numlines_band < 0 || s->numlines_band > PA_MAXL || (s->numlines_band && !s->lines))
    return snprintf(why, n, "bad veto line list"), 1;
  if (cfg && (cfg->precision < 0 || cfg->precision > 1 || cfg->phase_mode < 0 || cfg->phase_mode > 2))
    return snprintf(why, n, "bad precision/phase_mode"), 1;
  if (cfg && (cfg->spindown_batch < 0 || cfg->spindown_batch > 4096))
    return snprintf(why, n, "spindown_batch outside [0, 4096]"), 1;
  return 0;
}

static int build_ctx(pa_ctx* c, const pa_detector* det) {
  const pa_settings& s = c->sett;
  const int N = s.N, nifo = c->nifo;
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking), "cudaStreamCreate");
  CK(cudaStreamCreateWithFlags(&c->stream_pre, cudaStreamNonBlocking), "cudaStreamCreate");
  CK(cudaStreamCreateWithFlags(&c->stream2, cudaStreamNonBlocking), "cudaStreamCreate");
  for (int k = 0; k < 2; k++) {
    CK(cudaEventCreateWithFlags(&c->ev_pre[k], cudaEventDisableTiming), "cudaEventCreate");
    CK(cudaEventCreateWithFlags(&c->ev_spin[k], cudaEventDisableTiming), "cudaEventCreate");
    CK(cudaEventCreateWithFlags(&c->ev_spin2[k], cudaEventDisableTiming), "cudaEventCreate");
  }
  pa::Buffers& b = c->b;
  memset(&b, 0, sizeof(b));
  b.N = N;
  b.nfft = s.nfft;
  b.Ninterp = s.Ninterp;
  b.nfftf = s.nfftf;
  b.nmin = s.nmin;
  b.nmax = s.nmax;
  b.bins = s.nmax - s.nmin;
  b.nblk = b.bins / PA_NAVFSTAT;
  b.nifo = nifo;
  b.fftpad = s.fftpad;
  int sb = c->cfg.spindown_batch;
  if (sb <= 0) {
    // keep the FFT intermediate of one batch near 64 MB (L2-sized)
    const size_t per = 2 * (size_t)s.nfftf * 2 * c->rsz;
    sb = (int)std::max<size_t>(1, std::min<size_t>(64, ((size_t)64 << 20) / per));
  }
  b.sbatch = sb;
  // buffers for up to four times the batch, for the schedule tuner: one lane
  // of up to sb_max spindowns, or two of up to sb_max / 2
  c->sb_max = std::min(128, 4 * sb);
  const int sbm = c->sb_max;
  b.lane_sb = sbm / 2;
  // two lanes by default (measured 3% faster than one on H1+L1 N=86164)
  c->lanes = sb <= b.lane_sb ? 2 : 1;
  const size_t rs = c->rsz, cs = 2 * c->rsz;
  int rc;
#define ALLOC(ptr, bytes)                              \
  do {                                                 \
    void* p_;                                          \
    if ((rc = dalloc(c, &p_, (bytes)))) return rc;     \
    ptr = decltype(ptr)(p_);                           \
  } while (0)
  ALLOC(b.xDat, sizeof(double) * nifo * (size_t)N);
  ALLOC(b.DetSSB, sizeof(double) * nifo * 3 * (size_t)N);
  ALLOC(b.cosmodf, rs * N);
  ALLOC(b.sinmodf, rs * N);
  ALLOC(b.dc, sizeof(pa::DetConst) * pa::kMaxDet);
  ALLOC(b.spline_invp, sizeof(double) * 64);
  ALLOC(b.spline_p, sizeof(double) * 64);
  ALLOC(b.xin, cs * nifo * 2 * (size_t)N);
  ALLOC(b.spec, cs * nifo * 2 * (size_t)s.nfft);
  ALLOC(b.yint, cs * nifo * 2 * (size_t)s.Ninterp);
  ALLOC(b.u, sizeof(double) * 2 * nifo * 2 * (size_t)(2 * N));
  ALLOC(b.y2, cs * nifo * 2 * (size_t)(2 * N));
  ALLOC(b.shftf, sizeof(double) * nifo * (size_t)N);
  for (int k = 0; k < 2; k++) {
    if (c->fp64) ALLOC(b.ph0[k], 8 * nifo * (size_t)N);  // tmp1 (FP32 forms keep it in xm)
    ALLOC(b.xm[k], 32 * nifo * (size_t)N);  // FP32: one 32-byte record; FP64: two double2
    ALLOC(b.sums[k], sizeof(double) * 8);
    ALLOC(b.sums_r[k], sizeof(double) * 4);
  }
  ALLOC(b.part, sizeof(double) * 2 * nifo * (size_t)((N + 255) / 256));
  ALLOC(b.ybuf_pre, cs * nifo * 2 * (size_t)s.Ninterp);
  ALLOC(b.counter, sizeof(unsigned int) * 4);
  CK(cudaMemset(b.counter, 0, sizeof(unsigned int) * 4), "cudaMemset");
  ALLOC(b.ybuf, (size_t)sbm * 2 * s.nfftf * cs);
  ALLOC(b.F, rs * (size_t)sbm * b.bins);
  ALLOC(b.mu, rs * (size_t)sbm * (b.nblk > 0 ? b.nblk : 1));
  b.cand_cap = 1 << 18;
  ALLOC(b.cand, sizeof(pa::DevCand) * (size_t)b.cand_cap);
  ALLOC(b.ncand, sizeof(int) * 4);
#undef ALLOC
  CK(cudaMallocHost((void**)&c->h_cand, sizeof(pa::DevCand) * (size_t)b.cand_cap), "cudaMallocHost");
  CK(cudaMallocHost((void**)&c->h_ncand, sizeof(int) * 4), "cudaMallocHost");
  // constant tables
  std::vector<double> cm(N), sm(N);
  for (int i = 0; i < N; i++) {
    double omrt = s.omr * i;  // init.c:450-455
    cm[i] = cos(omrt);
    sm[i] = sin(omrt);
  }
  if ((rc = upload_real(c, (void*)b.cosmodf, cm))) return rc;
  if ((rc = upload_real(c, (void*)b.sinmodf, sm))) return rc;
  double invp[64], p[64];
  p[0] = 0.;
  invp[0] = 0.;
  for (int i = 1; i < 64; i++) {  // auxi.c:71-72
    invp[i] = 2. / (p[i - 1] + 4.);
    p[i] = -.5 * invp[i];
  }
  CK(cudaMemcpy((void*)b.spline_invp, invp, sizeof(invp), cudaMemcpyHostToDevice), "upload spline");
  CK(cudaMemcpy((void*)b.spline_p, p, sizeof(p), cudaMemcpyHostToDevice), "upload spline");
  if ((rc = make_twiddles(c, s.nfft, -1, &c->tw_fwd))) return rc;
  if ((rc = make_twiddles(c, s.Ninterp, +1, &c->tw_inv))) return rc;
  if ((rc = make_twiddles(c, s.nfft, +1, &c->tw_invh))) return rc;
  if ((rc = make_twiddles(c, s.nfftf, -1, &c->tw_main))) return rc;
  if (!c->fp64) {  // inter-pass twiddle tables of the spindown transform, per split
    const long L = s.nfftf;
    int lg = 0;
    while ((1L << lg) < L) ++lg;
    for (int sp = 0; sp < 2; sp++) {
      if (sp == 1 && !(lg & 1)) {
        b.tw_pass[1] = b.tw_pass[0];
        break;
      }
      const int l1 = pa::pass_logl1(lg, sp);
      std::vector<double> v(2 * (size_t)L);
      for (long j = 0; j < L; j++) host_twiddle(pa::tw_pass_exp(j, L, l1), L, -1, &v[2 * j], &v[2 * j + 1]);
      void* p = nullptr;
      if ((rc = dalloc(c, &p, v.size() * c->rsz))) return rc;
      if ((rc = upload_real(c, p, v))) return rc;
      b.tw_pass[sp] = p;
    }
  }
  for (int k = 0; k < 4; k++) {
    b.tw_fwd[k] = c->tw_fwd.p[k];
    b.tw_inv[k] = c->tw_inv.p[k];
    b.tw_invh[k] = c->tw_invh.p[k];
    b.tw_main[k] = c->tw_main.p[k];
  }
  if ((rc = upload_data(c, det))) return rc;
  c->eng = c->fp64 ? pa::make_engine_f64(b) : pa::make_engine_f32(b, c->cfg.phase_mode);
  if (!c->eng) return fail(c, PA_ERR_NOMEM, "engine allocation failed");
  c->eng->prof = &c->prof;
  // default factor split: for two detectors in the FP32 forms, the one with
  // 256-point columns (the radix-16 spindown pass A): swapped for nfftf = 2^17
  if (!c->fp64 && nifo == 2 && s.nfftf == (1 << 17)) c->eng->set_split(1);
  CK(cudaEventCreate(&c->ev0), "cudaEventCreate");
  CK(cudaEventCreate(&c->ev1), "cudaEventCreate");
  CK(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming), "cudaEventCreate");
  CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming), "cudaEventCreate");
  CK(cudaEventCreateWithFlags(&c->ev_join2, cudaEventDisableTiming), "cudaEventCreate");
  return PA_OK;
}

extern "C" {

const char* pa_version(void) { return "polgraw-gb300 1.0 (sm_103a)"; }

int pa_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

const char* pa_last_error(const pa_ctx* ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

pa_ctx* pa_create(const pa_settings* sett, const pa_detector* det, int nifo, const pa_config* cfg,
                  int* status) {
  pa::TraceRange trace_("pa_create");
  char why[256];
  int st = PA_OK;
  if (!sett || !det) {
    fail(nullptr, PA_ERR_ARG, "null settings or detectors");
    if (status) *status = PA_ERR_ARG;
    return nullptr;
  }
  if (validate(sett, nifo, cfg, why, sizeof why)) {
    fail(nullptr, PA_ERR_ARG, "%s", why);
    if (status) *status = PA_ERR_ARG;
    return nullptr;
  }
  for (int n = 0; n < nifo; n++)
    if (!det[n].xDat || !det[n].DetSSB || !(det[n].sig2 > 0)) {
      fail(nullptr, PA_ERR_ARG, "detector %d: missing data or sig2 <= 0", n);
      if (status) *status = PA_ERR_ARG;
      return nullptr;
    }
  int ndev = pa_device_count();
  const int dev = cfg ? cfg->device : 0;
  if (ndev <= 0 || dev < 0 || dev >= ndev) {
    fail(nullptr, PA_ERR_NODEV, "no CUDA device %d (found %d)", dev, ndev);
    if (status) *status = PA_ERR_NODEV;
    return nullptr;
  }
  pa_ctx* c = new pa_ctx();
  c->sett = *sett;
  c->nifo = nifo;
  if (cfg) c->cfg = *cfg;
  else memset(&c->cfg, 0, sizeof(c->cfg));
  c->fp64 = c->cfg.precision == PA_PREC_FP64;
  c->rsz = c->fp64 ? 8 : 4;
  c->dev = dev;
  if (sett->numlines_band > 0) c->lines.assign(sett->lines, sett->lines + 2 * sett->numlines_band);
  c->sett.lines = c->lines.empty() ? nullptr : c->lines.data();
  st = build_ctx(c, det);
  if (st != PA_OK) {
    g_create_error = c->err;
    pa_destroy(c);
    if (status) *status = st;
    return nullptr;
  }
  if (status) *status = PA_OK;
  return c;
}

int pa_set_data(pa_ctx* c, const pa_detector* det, int nifo) {
  pa::TraceRange trace_("pa_set_data");
  if (!c || !det || nifo != c->nifo) return fail(c, PA_ERR_ARG, "pa_set_data: bad arguments");
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  for (int n = 0; n < nifo; n++)
    if (!det[n].xDat || !det[n].DetSSB || !(det[n].sig2 > 0))
      return fail(c, PA_ERR_ARG, "detector %d: missing data or sig2 <= 0", n);
  return upload_data(c, det);
}

void pa_destroy(pa_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->dev);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->stream_pre) cudaStreamSynchronize(c->stream_pre);
  if (c->stream2) cudaStreamSynchronize(c->stream2);
  delete c->eng;
  for (int i = 0; i < c->prof.cap; i++) {
    cudaEventDestroy(c->prof.recs[i].a);
    cudaEventDestroy(c->prof.recs[i].b);
  }
  delete[] c->prof.recs;
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  if (c->ev_join2) cudaEventDestroy(c->ev_join2);
  drop_graphs(c);
  for (void* p : c->allocs) cudaFree(p);
  if (c->h_cand) cudaFreeHost(c->h_cand);
  if (c->h_ncand) cudaFreeHost(c->h_ncand);
  if (c->stream) cudaStreamDestroy(c->stream);
  if (c->stream_pre) cudaStreamDestroy(c->stream_pre);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  for (int k = 0; k < 2; k++) {
    if (c->ev_pre[k]) cudaEventDestroy(c->ev_pre[k]);
    if (c->ev_spin[k]) cudaEventDestroy(c->ev_spin[k]);
    if (c->ev_spin2[k]) cudaEventDestroy(c->ev_spin2[k]);
  }
  delete c;
}

long long pa_kernel_launches(const pa_ctx* c) {
  if (!c) return 0;
  return (c->eng ? c->eng->launches() : 0) + c->extra_launches;
}

double pa_last_call_ms(const pa_ctx* c) { return c ? c->last_ms : 0.; }

int pa_set_profiling(pa_ctx* c, int on) {
  if (!c) return PA_ERR_ARG;
  if (on && !c->prof.recs) {
    CK(cudaSetDevice(c->dev), "cudaSetDevice");
    const int cap = 1 << 16;
    c->prof.recs = new pa::Prof::Rec[cap];
    for (int i = 0; i < cap; i++) {
      CK(cudaEventCreate(&c->prof.recs[i].a), "cudaEventCreate");
      CK(cudaEventCreate(&c->prof.recs[i].b), "cudaEventCreate");
      c->prof.cap = i + 1;
    }
  }
  c->prof.on = on != 0;
  return PA_OK;
}

int pa_set_cta_trace(pa_ctx* c, void* buf, unsigned int cap) {
  if (!c || !c->eng) return PA_ERR_ARG;
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  CK(c->eng->set_trace(buf, cap), "set trace");
  return PA_OK;
}

int pa_cta_trace_count(pa_ctx* c, unsigned int* n) {
  if (!c || !c->eng || !n) return PA_ERR_ARG;
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  CK(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
  CK(c->eng->trace_count(n), "trace count");
  return PA_OK;
}

void pa_profile_reset(pa_ctx* c) {
  if (!c) return;
  for (int k = 0; k < pa::KK_COUNT; k++) {
    c->prof.total_ms[k] = 0.;
    c->prof.launches[k] = 0;
    c->prof.items[k] = 0;
  }
  c->prof.n = 0;
}

int pa_profile_get(const pa_ctx* c, int kind, const char** name, double* total_ms, long long* launches,
                   long long* items) {
  if (!c || kind < 0 || kind >= pa::KK_COUNT) return PA_ERR_ARG;
  if (name) *name = pa::kernel_kind_name(kind);
  if (total_ms) *total_ms = c->prof.total_ms[kind];
  if (launches) *launches = c->prof.launches[kind];
  if (items) *items = c->prof.items[kind];
  return PA_OK;
}

}  // extern "C"

// ------------------------------------------------------------------
// job_core host logic

namespace {

struct SkyHost {
  int pm, mm, nn;
  int inside;
  double sgnlt2, sgnlt3, het0;
  int smin, smax, nss;
  pa::SkyArgs args;
};

// auxi.c:16-24
void lin2ast(double be1, double be2, int pm, double sepsm, double cepsm, double* sinal, double* cosal,
             double* sindel, double* cosdel) {
  *sindel = be1 * sepsm - (2 * pm - 3) * sqrt(1. - SQR(be1) - SQR(be2)) * cepsm;
  *cosdel = sqrt(1. - SQR(*sindel));
  *sinal = (be1 - sepsm * (*sindel)) / (cepsm * (*cosdel));
  *cosal = be2 / (*cosdel);
}

void sky_setup(const pa_ctx* c, int pm, int mm, int nn, const pa_opts* o, int sst, int spndr1,
               SkyHost* h) {
  const pa_settings& s = c->sett;
  const double* M = s.M;
  memset(h, 0, sizeof(*h));
  h->pm = pm;
  h->mm = mm;
  h->nn = nn;
  double al1 = nn * M[10] + mm * M[14];
  double al2 = nn * M[11] + mm * M[15];
  if ((SQR(al1) + SQR(al2)) / SQR(s.oms) > 1.) {  // jobcore.c:248
    h->inside = 0;
    return;
  }
  h->inside = 1;
  double sinalt, cosalt, sindelt, cosdelt;
  lin2ast(al1 / s.oms, al2 / s.oms, pm, s.sepsm, s.cepsm, &sinalt, &cosalt, &sindelt, &cosdelt);
  h->sgnlt2 = asin(sindelt);
  h->sgnlt3 = fmod(atan2(sinalt, cosalt) + 2. * M_PI, 2. * M_PI);
  h->het0 = fmod(nn * M[8] + mm * M[12], M[0]);
  // jobcore.c:424-444
  int smin = sst, smax = spndr1;
  if (!o->use_range) {
    smin = trunc((s.Smin - nn * M[9] - mm * M[13]) / M[5]);
    smax = trunc(-(nn * M[9] + mm * M[13] + s.Smax) / M[5]);
    if (smin > smax) std::swap(smin, smax);
  }
  if (o->s0_flag) smin = smax;
  h->smin = smin;
  h->smax = smax;
  h->nss = smax >= smin ? smax - smin + 1 : 0;
  pa::SkyArgs& a = h->args;
  a.het0 = h->het0;
  a.oms = s.oms;
  a.sinal = sinalt;
  a.cosal = cosalt;
  a.sindel = sindelt;
  a.cosdel = cosdelt;
  a.nS[0] = cosalt * cosdelt;
  a.nS[1] = sinalt * cosdelt;
  a.nS[2] = sindelt;
  for (int n = 0; n < c->nifo; n++) {
    a.shft1[n] = a.nS[0] * c->det0[n][0] + a.nS[1] * c->det0[n][1] + a.nS[2] * c->det0[n][2];
    a.cosalfr[n] = cosalt * c->dc[n].cphir + sinalt * c->dc[n].sphir;
    a.sinalfr[n] = sinalt * c->dc[n].cphir - cosalt * c->dc[n].sphir;
  }
  a.s1_0 = o->s0_flag ? 0. : nn * M[9] + mm * M[13];
  a.M5 = o->s0_flag ? 0. : M[5];
  a.M0 = M[0];
  a.M4 = M[4];
  a.task = 0;
}

// x mod 1 as a 64-bit fixed-point fraction (x 2^64 mod 2^64), exactly, from
// the bits of x (the same integer algorithm as the device's turns_fixed)
uint64_t host_turns_fixed(double x) {
  uint64_t bits;
  memcpy(&bits, &x, 8);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) return 0;
  const uint64_t m = (bits & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sh = e - 1011;
  uint64_t t;
  if (sh >= 64) t = 0;
  else if (sh >= 0) t = m << sh;
  else if (sh > -64) t = m >> (-sh);
  else t = 0;
  return (bits >> 63) ? (0 - t) : t;
}

// Kernel arguments of a sky point for this context's engine.
pa::SkyArgs sky_args(const pa_ctx* c, const SkyHost& h, int task) {
  pa::SkyArgs a = h.args;
  a.task = task;
  a.ss_base = 0;
  a.h0f = host_turns_fixed(a.het0 / (2. * M_PI));
  a.oms_t = a.oms / (2. * M_PI);
  for (int n = 0; n < pa::kMaxDet; n++) {
    a.cosalfr_f[n] = (float)a.cosalfr[n];
    a.sinalfr_f[n] = (float)a.sinalfr[n];
  }
  a.cosdel_f = (float)a.cosdel;
  a.sindel_f = (float)a.sindel;
  a.s1f = a.m5f = 0;
  if (!c->fp64 && c->cfg.phase_mode == PA_PHASE_FIXED) {
    // the fixed-point phase terms are formed in turns, relative to the
    // first spindown so that the per-spindown factor is non-negative
    a.ss_base = h.smin;
    a.s1_0 = (a.s1_0 + h.smin * a.M5) / (2. * M_PI);
    a.M5 = a.M5 / (2. * M_PI);
    a.s1f = host_turns_fixed(a.s1_0);
    a.m5f = host_turns_fixed(a.M5);
  }
  return a;
}

// Enqueues one sky point: its prelude on the prelude stream into slot
// task % 2 (after the spindowns that last read that slot), and its spindown
// batches after the prelude, on the main stream or, with two lanes,
// alternately on the main stream and stream2 (*lane: the lane of the next
// batch, carried over from sky point to sky point).
int enqueue_sky(pa_ctx* c, const SkyHost& h, const pa_opts* o, int task, void* Fdbg, int Fss,
                bool wait_slot = true, int* lane = nullptr) {
  const pa::SkyArgs a = sky_args(c, h, task);
  const int slot = task & 1;
  const int lanes = Fdbg ? 1 : active_lanes(c);
  cudaStream_t sp = prelude_stream(c);
  if (wait_slot) {
    CK(cudaStreamWaitEvent(sp, c->ev_spin[slot], 0), "cudaStreamWaitEvent");
    // (the debug path is never captured: it may wait on lane 1's reads of an
    // earlier call too)
    if (lanes == 2 || Fdbg) CK(cudaStreamWaitEvent(sp, c->ev_spin2[slot], 0), "cudaStreamWaitEvent");
  }
  cudaError_t e = c->eng->prelude(a, slot, sp);
  if (e != cudaSuccess) return cuda_fail(c, e, "prelude launch");
  CK(cudaEventRecord(c->ev_pre[slot], sp), "cudaEventRecord");
  CK(cudaStreamWaitEvent(c->stream, c->ev_pre[slot], 0), "cudaStreamWaitEvent");
  if (lanes == 2) CK(cudaStreamWaitEvent(c->stream2, c->ev_pre[slot], 0), "cudaStreamWaitEvent");
  if (Fdbg) {
    e = c->eng->spindowns(a, slot, 0, Fss, 1, o->trl, o->white_flag, o->s0_flag, c->stream, Fdbg);
    if (e != cudaSuccess) return cuda_fail(c, e, "spindown launch");
  } else {
    // full launches and one remainder: splitting into equal launches (200 as
    // 4 x 50 instead of 3 x 64 + 8) was measured 1.5% slower, as each
    // launch's last partial wave of CTAs costs a whole wave
    int l0 = 0;
    int* ln = lane ? lane : &l0;
    for (int ss = h.smin; ss <= h.smax; ss += c->b.sbatch) {
      const int nb = std::min(c->b.sbatch, h.smax - ss + 1);
      const int l = lanes == 2 ? *ln : 0;
      e = c->eng->spindowns(a, slot, l, ss, nb, o->trl, o->white_flag, o->s0_flag, l ? c->stream2 : c->stream,
                            nullptr);
      if (e != cudaSuccess) return cuda_fail(c, e, "spindown launch");
      if (lanes == 2) *ln ^= 1;
    }
  }
  CK(cudaEventRecord(c->ev_spin[slot], c->stream), "cudaEventRecord");
  if (lanes == 2) CK(cudaEventRecord(c->ev_spin2[slot], c->stream2), "cudaEventRecord");
  return PA_OK;
}

bool cand_less(const pa::DevCand& x, const pa::DevCand& y) {
  if (x.task != y.task) return x.task < y.task;
  if (x.ss != y.ss) return x.ss < y.ss;
  return x.ii < y.ii;
}

// Enqueues sky points [t0, t1) of a batch on the context's streams: the
// candidate counter reset (for the batch's first part), then every sky point
// (prelude on the prelude stream forked from the main stream, spindowns on
// the main stream), and the join of the prelude stream back into the main
// stream.  Slots are reused across sky points through their events; the
// first use of each slot in a part needs no wait (the work before it on the
// main stream -- the previous part or call -- has finished when the part
// starts).  Works unchanged under stream capture.
int enqueue_tasks(pa_ctx* c, const std::vector<SkyHost>& hs, const pa_opts* o, size_t t0, size_t t1,
                  bool reset) {
  const int lanes = active_lanes(c);
  if (reset) CK(cudaMemsetAsync(c->b.ncand, 0, sizeof(int), c->stream), "memset");
  CK(cudaEventRecord(c->ev_fork, c->stream), "cudaEventRecord");
  CK(cudaStreamWaitEvent(c->stream_pre, c->ev_fork, 0), "cudaStreamWaitEvent");
  if (lanes == 2) CK(cudaStreamWaitEvent(c->stream2, c->ev_fork, 0), "cudaStreamWaitEvent");
  bool used[2] = {false, false};
  int lane = 0;
  for (size_t t = t0; t < t1; t++) {
    if (!hs[t].inside || hs[t].nss == 0) continue;
    const int slot = (int)t & 1;
    int rc = enqueue_sky(c, hs[t], o, (int)t, nullptr, 0, used[slot], &lane);
    if (rc) return rc;
    used[slot] = true;
  }
  CK(cudaEventRecord(c->ev_join, c->stream_pre), "cudaEventRecord");
  CK(cudaStreamWaitEvent(c->stream, c->ev_join, 0), "cudaStreamWaitEvent");
  if (lanes == 2) {
    CK(cudaEventRecord(c->ev_join2, c->stream2), "cudaEventRecord");
    CK(cudaStreamWaitEvent(c->stream, c->ev_join2, 0), "cudaStreamWaitEvent");
  }
  return PA_OK;
}

int enqueue_tasks(pa_ctx* c, const std::vector<SkyHost>& hs, const pa_opts* o) {
  return enqueue_tasks(c, hs, o, 0, hs.size(), true);
}

// Replaces *exec by an executable graph of g: updated in place when the
// topology matches, instantiated anew otherwise.
int graph_exec_from(cudaGraph_t g, cudaGraphExec_t* exec, std::string* err) {
  if (*exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(*exec, g, &info) == cudaSuccess) return PA_OK;
    cudaGetLastError();
    cudaGraphExecDestroy(*exec);
    *exec = nullptr;
  }
  cudaError_t e = cudaGraphInstantiate(exec, g, 0);
  if (e != cudaSuccess) {
    *exec = nullptr;
    *err = std::string("cudaGraphInstantiate: ") + cudaGetErrorString(e);
    return PA_ERR_CUDA;
  }
  return PA_OK;
}

// Enqueues the batch directly, or captures it into the context's graph and
// launches that.  The timing event ev0 goes on the stream right before the
// work (after the capture and graph update, which are host work).
int launch_tasks(pa_ctx* c, const std::vector<SkyHost>& hs, const pa_opts* o) {
  pa::TraceRange trace_("launch (capture, graph launch)");
  const bool graph = c->graphs && !c->prof.on;
  if (!graph) {
    CK(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
    return enqueue_tasks(c, hs, o);
  }
  // The batch is captured in parts, each into its own executable graph
  // (updated in place when the part's launch structure repeats), and each
  // part is launched as soon as it is captured: the host captures part k + 1
  // while the device runs part k.  Only the first part's capture precedes
  // device work, so it is short (kGraphFirst sky points); the parts then
  // double, as capturing a sky point takes the host far less time than the
  // device takes to search it, up to kGraphPart.
  const size_t n = hs.size();
  std::vector<size_t> bound{0};
  for (size_t step = kGraphFirst; bound.back() < n; step = std::min(kGraphPart, 2 * step))
    bound.push_back(std::min(n, bound.back() + step));
  if (n == 0) bound.push_back(0);
  const size_t nparts = bound.size() - 1;
  if (c->gexec_parts.size() < nparts) c->gexec_parts.resize(nparts, nullptr);
  for (size_t k = 0; k < nparts; k++) {
    const size_t t0 = bound[k], t1 = bound[k + 1];
    CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    int rc = enqueue_tasks(c, hs, o, t0, t1, k == 0);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    rc = graph_exec_from(g, &c->gexec_parts[k], &c->err);
    cudaGraphDestroy(g);
    if (rc) return rc;
    if (k == 0) CK(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
    CK(cudaGraphLaunch(c->gexec_parts[k], c->stream), "cudaGraphLaunch");
  }
  return PA_OK;
}

// After the batch finished: the device candidates, sorted to the serial
// order, into `out`; returns PA_ERR_CAPACITY (with *n the count) when the
// device buffer overflowed.
int collect_tasks(pa_ctx* c, std::vector<pa::DevCand>* out, int* n_out) {
  pa::TraceRange trace_("collect candidates");
  CK(cudaMemcpyAsync(c->h_ncand, c->b.ncand, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "copy count");
  CK(cudaStreamSynchronize(c->stream), "search");
  const int n = *c->h_ncand;
  *n_out = n;
  if (n > c->b.cand_cap) return PA_ERR_CAPACITY;
  if (n > 0) {
    CK(cudaMemcpyAsync(c->h_cand, c->b.cand, sizeof(pa::DevCand) * (size_t)n, cudaMemcpyDeviceToHost,
                       c->stream), "copy candidates");
    CK(cudaStreamSynchronize(c->stream), "copy candidates");
  }
  out->assign(c->h_cand, c->h_cand + n);
  std::sort(out->begin(), out->end(), cand_less);
  return PA_OK;
}

// Grows the device candidate buffer to hold n (with margin); the engine is
// rebuilt on the new buffers (its schedule kept) and any graph dropped.
int grow_candidates(pa_ctx* c, int n) {
  const int ncap = n + n / 2;
  void* p = nullptr;
  CK(cudaMalloc(&p, sizeof(pa::DevCand) * (size_t)ncap), "cudaMalloc");
  c->allocs.push_back(p);
  c->b.cand = (pa::DevCand*)p;
  cudaFreeHost(c->h_cand);
  c->h_cand = nullptr;
  CK(cudaMallocHost((void**)&c->h_cand, sizeof(pa::DevCand) * (size_t)ncap), "cudaMallocHost");
  c->b.cand_cap = ncap;
  const long long before = c->eng->launches();
  const int split = c->eng->split();
  delete c->eng;
  c->eng = c->fp64 ? pa::make_engine_f64(c->b) : pa::make_engine_f32(c->b, c->cfg.phase_mode);
  c->eng->prof = &c->prof;
  c->eng->set_split(split);
  c->extra_launches += before;
  drop_graphs(c);
  return PA_OK;
}

// Runs the sky points, gathers the device candidates (sorted to the serial
// order) into `out`.  Grows the device candidate buffer and re-runs when it
// overflowed.
int run_tasks(pa_ctx* c, const std::vector<SkyHost>& hs, const pa_opts* o, std::vector<pa::DevCand>* out) {
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  for (int attempt = 0; attempt < 3; attempt++) {
    int rc = launch_tasks(c, hs, o);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
    int n = 0;
    rc = collect_tasks(c, out, &n);
    {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, c->ev0, c->ev1);
      c->last_ms = ms;
    }
    if (c->prof.on) prof_collect(c);
    if (rc == PA_OK) return PA_OK;
    if (rc != PA_ERR_CAPACITY) return rc;
    if ((rc = grow_candidates(c, n))) return rc;
  }
  return fail(c, PA_ERR_CAPACITY, "device candidate buffer overflow");
}

// jobcore.c:670-687 record for one candidate; returns 0 when vetoed
int make_record(const pa_ctx* c, const SkyHost& h, const pa_opts* o, const pa::DevCand& d, double rec[5]) {
  const pa_settings& s = c->sett;
  const double* M = s.M;
  const int ss = d.ss, nn = h.nn, mm = h.mm;
  double het1 = fmod(ss * M[4], M[0]);
  if (het1 < 0) het1 += M[0];
  const double sgnl0 = h.het0 + het1;
  rec[0] = 2. * M_PI * d.ii / ((double)s.fftpad * s.nfft) + sgnl0;
  rec[1] = o->s0_flag ? 0. : ss * M[5] + nn * M[9] + mm * M[13];
  rec[2] = h.sgnlt2;
  rec[3] = h.sgnlt3;
  rec[4] = sqrt(2. * (d.F - s.nd));
  for (int k = 0; k < s.numlines_band; k++)
    if (rec[0] >= s.lines[2 * k] && rec[0] <= s.lines[2 * k + 1]) return 0;
  return 1;
}

int append_records(pa_ctx* c, const std::vector<SkyHost>& hs, const pa_opts* o,
                   const std::vector<pa::DevCand>& cands, int* sgnlc, double* sgnlv, int cap,
                   pa_cand_idx* idx, int* FNum, int* needed) {
  std::vector<double> recs;
  std::vector<pa_cand_idx> ids;
  recs.reserve(cands.size() * PA_NPAR);
  for (const pa::DevCand& d : cands) {
    const SkyHost& h = hs[d.task];
    double rec[5];
    if (!make_record(c, h, o, d, rec)) continue;
    recs.insert(recs.end(), rec, rec + 5);
    pa_cand_idx x;
    x.pm = h.pm;
    x.mm = h.mm;
    x.nn = h.nn;
    x.ss = d.ss;
    x.ii = d.ii;
    x.F = (float)d.F;
    ids.push_back(x);
  }
  const int total = (int)ids.size();
  if (needed) *needed = *sgnlc + total;
  if (*sgnlc + total > cap) return fail(c, PA_ERR_CAPACITY, "candidate buffer too small: need %d", *sgnlc + total);
  memcpy(sgnlv + (size_t)PA_NPAR * (*sgnlc), recs.data(), sizeof(double) * recs.size());
  if (idx) memcpy(idx + *sgnlc, ids.data(), sizeof(pa_cand_idx) * ids.size());
  *sgnlc += total;
  int nss = 0;
  for (const SkyHost& h : hs)
    if (h.inside) nss += h.nss;
  *FNum += nss;
  return PA_OK;
}

}  // namespace

extern "C" {

int pa_job_core(pa_ctx* c, int pm, int mm, int nn, const pa_opts* o, const pa_range* r, int* sgnlc,
                double* sgnlv, int cap, pa_cand_idx* idx, int* FNum, int* needed) {
  pa::TraceRange trace_("pa_job_core");
  if (!c || !o || !r || !sgnlc || !sgnlv || !FNum || cap < 0) return fail(c, PA_ERR_ARG, "pa_job_core: bad arguments");
  pa_sky t{pm, mm, nn};
  return pa_search_batch(c, &t, 1, o, r, sgnlc, sgnlv, cap, idx, FNum, needed);
}

int pa_search_batch(pa_ctx* c, const pa_sky* tasks, int ntasks, const pa_opts* o, const pa_range* r,
                    int* sgnlc, double* sgnlv, int cap, pa_cand_idx* idx, int* FNum, int* needed) {
  pa::TraceRange trace_("pa_search_batch");
  if (!c || !tasks || ntasks < 0 || !o || !r || !sgnlc || !sgnlv || !FNum || cap < 0)
    return fail(c, PA_ERR_ARG, "pa_search_batch: bad arguments");
  if (needed) *needed = *sgnlc;
  std::vector<SkyHost> hs(ntasks);
  for (int t = 0; t < ntasks; t++) {
    // the sky loop resets sst to spndr[0] after each sky point (jobcore.c:123)
    const int sst = t == 0 ? r->sst : r->spndr[0];
    sky_setup(c, tasks[t].pm, tasks[t].mm, tasks[t].nn, o, sst, r->spndr[1], &hs[t]);
  }
  std::vector<pa::DevCand> cands;
  int rc = run_tasks(c, hs, o, &cands);
  if (rc) return rc;
  return append_records(c, hs, o, cands, sgnlc, sgnlv, cap, idx, FNum, needed);
}

int pa_set_graphs(pa_ctx* c, int on) {
  if (!c) return PA_ERR_ARG;
  c->graphs = on != 0;
  if (!c->graphs && !c->gexec_parts.empty()) {
    cudaSetDevice(c->dev);
    drop_graphs(c);
  }
  return PA_OK;
}

int pa_set_schedule(pa_ctx* c, int sbatch, int split) {
  if (!c || sbatch < 1 || sbatch > c->sb_max || split < 0 || split > 1)
    return fail(c, PA_ERR_ARG, "pa_set_schedule: sbatch must be in [1, %d], split 0 or 1", c ? c->sb_max : 0);
  c->b.sbatch = sbatch;
  c->eng->set_split(split);
  if (c->lanes == 2 && sbatch > c->b.lane_sb) {  // too large for a lane: one lane
    CK(cudaSetDevice(c->dev), "cudaSetDevice");
    drop_graphs(c);
    c->lanes = 1;
  }
  return PA_OK;
}

int pa_set_lanes(pa_ctx* c, int lanes) {
  if (!c || lanes < 1 || lanes > 2) return fail(c, PA_ERR_ARG, "pa_set_lanes: lanes must be 1 or 2");
  if (lanes == 2 && c->b.sbatch > c->b.lane_sb)
    return fail(c, PA_ERR_ARG, "pa_set_lanes: two lanes need a spindown batch of at most %d (now %d)",
                c->b.lane_sb, c->b.sbatch);
  if (lanes != c->lanes) {
    CK(cudaSetDevice(c->dev), "cudaSetDevice");
    drop_graphs(c);
  }
  c->lanes = lanes;
  return PA_OK;
}

int pa_get_lanes(const pa_ctx* c, int* lanes) {
  if (!c || !lanes) return PA_ERR_ARG;
  *lanes = c->lanes;
  return PA_OK;
}

int pa_get_schedule(const pa_ctx* c, int* sbatch, int* split, int* max_sbatch) {
  if (!c) return PA_ERR_ARG;
  if (sbatch) *sbatch = c->b.sbatch;
  if (split) *split = c->eng->split();
  if (max_sbatch) *max_sbatch = c->sb_max;
  return PA_OK;
}

int pa_autotune(pa_ctx* c, const pa_sky* tasks, int ntasks, const pa_opts* o, const pa_range* r, int* sbatch,
                int* split) {
  pa::TraceRange trace_("pa_autotune");
  if (!c || !tasks || ntasks < 1 || !o || !r) return fail(c, PA_ERR_ARG, "pa_autotune: bad arguments");
  std::vector<SkyHost> hs(ntasks);
  for (int t = 0; t < ntasks; t++)
    sky_setup(c, tasks[t].pm, tasks[t].mm, tasks[t].nn, o, t == 0 ? r->sst : r->spndr[0], r->spndr[1], &hs[t]);
  const int sb0 = c->b.sbatch, sp0 = c->eng->split(), ln0 = c->lanes;
  // (lanes, spindown batch) candidates: one lane with a quarter to all of the
  // buffers, two lanes with a quarter or half each
  const int m = c->sb_max;
  const int cands[6][2] = {{1, m / 4}, {1, m / 2}, {1, 3 * m / 4}, {1, m}, {2, m / 4}, {2, m / 2}};
  // the factor split is a choice only for odd log2(nfftf)
  const int nsplit = (c->sett.nfftf & 0xAAAAAAAA) ? 2 : 1;
  double best = 1e300;
  int bsb = sb0, bsp = sp0, bln = ln0;
  std::vector<pa::DevCand> out;
  for (int k = 0; k < 6; k++) {
    const int ln = cands[k][0], sb = std::max(1, cands[k][1]);
    bool seen = false;
    for (int q = 0; q < k; q++) seen = seen || (cands[q][0] == ln && std::max(1, cands[q][1]) == sb);
    if (seen) continue;
    for (int sp = 0; sp < nsplit; sp++) {
      c->lanes = ln;
      c->b.sbatch = sb;
      c->eng->set_split(sp);
      double t = 1e300;
      for (int rep = 0; rep < 4; rep++) {  // first run warms up; best of three
        int rc = run_tasks(c, hs, o, &out);
        if (rc) {
          c->lanes = ln0;
          c->b.sbatch = sb0;
          c->eng->set_split(sp0);
          return rc;
        }
        if (rep > 0) t = std::min(t, c->last_ms);
      }
      if (t < best) {
        best = t;
        bsb = sb;
        bsp = sp;
        bln = ln;
      }
    }
  }
  c->lanes = bln;
  c->b.sbatch = bsb;
  c->eng->set_split(bsp);
  drop_graphs(c);
  if (sbatch) *sbatch = bsb;
  if (split) *split = bsp;
  return PA_OK;
}

int pa_debug_prelude(pa_ctx* c, int pm, int mm, int nn, double* xa, double* xb, double* aa, double* bb) {
  if (!c) return PA_ERR_ARG;
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  pa_opts o;
  memset(&o, 0, sizeof(o));
  o.use_range = 1;
  SkyHost h;
  sky_setup(c, pm, mm, nn, &o, 0, 0, &h);
  if (!h.inside) return fail(c, PA_ERR_ARG, "sky point outside the grid disk");
  CK(cudaStreamSynchronize(c->stream), "sync");
  cudaError_t e = c->eng->prelude(sky_args(c, h, 0), 0, c->stream_pre);
  if (e != cudaSuccess) return cuda_fail(c, e, "prelude");
  const size_t n = (size_t)c->nifo * 2 * c->sett.N;
  std::vector<char> buf(n * 2 * 8);  // FP64 pairs or 32-byte FP32 records
  double sums[4];
  CK(cudaMemcpyAsync(buf.data(), c->b.xm[0], buf.size(), cudaMemcpyDeviceToHost, c->stream_pre), "copy");
  CK(cudaMemcpyAsync(sums, c->b.sums[0], sizeof(sums), cudaMemcpyDeviceToHost, c->stream_pre), "copy");
  CK(cudaStreamSynchronize(c->stream_pre), "prelude");
  const int N = c->sett.N;
  const int sw = c->eng->swapped_det();
  for (int d = 0; d < c->nifo; d++)
    for (int arr = 0; arr < 2; arr++) {
      double* dst = arr == 0 ? xa : xb;
      const int half = d == sw ? 1 - arr : arr;  // {xb, xa} records
      if (!dst) continue;
      for (int i = 0; i < N; i++) {
        double re, im;
        if (c->fp64) {
          const size_t src = ((size_t)d * 2 + arr) * N + i;
          re = ((double*)buf.data())[2 * src];
          im = ((double*)buf.data())[2 * src + 1];
        } else {
          // 32-byte records {xa.re, xa.im, xb.re, xb.im | phase terms}
          const size_t src = 8 * ((size_t)d * N + i) + 2 * half;
          re = ((float*)buf.data())[src];
          im = ((float*)buf.data())[src + 1];
        }
        dst[2 * ((size_t)d * N + i)] = re;
        dst[2 * ((size_t)d * N + i) + 1] = im;
      }
    }
  if (aa) *aa = sums[0];
  if (bb) *bb = sums[1];
  return PA_OK;
}

int pa_debug_fstat(pa_ctx* c, int pm, int mm, int nn, int ss, const pa_opts* o, double* F) {
  if (!c || !o || !F) return PA_ERR_ARG;
  CK(cudaSetDevice(c->dev), "cudaSetDevice");
  SkyHost h;
  sky_setup(c, pm, mm, nn, o, ss, ss, &h);
  if (!h.inside) return fail(c, PA_ERR_ARG, "sky point outside the grid disk");
  const int bins = c->b.bins;
  void* dF = nullptr;
  CK(cudaMalloc(&dF, c->rsz * (size_t)bins), "cudaMalloc");
  CK(cudaMemsetAsync(c->b.ncand, 0, sizeof(int), c->stream), "memset");
  int rc = enqueue_sky(c, h, o, 0, dF, ss);
  std::vector<char> buf(c->rsz * (size_t)bins);
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(buf.data(), dF, buf.size(), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(c, e, "debug fstat");
  }
  cudaFree(dF);
  if (rc) return rc;
  for (int i = 0; i < bins; i++) F[i] = c->fp64 ? ((double*)buf.data())[i] : ((float*)buf.data())[i];
  return PA_OK;
}

}  // extern "C"

// ------------------------------------------------------------------
// pa_fstat_noalloc: the normalised F-statistic of one template without any
// allocation.
//
// Some callers cannot allocate device memory: a plugin running inside a
// host application that owns the GPU memory budget, code that must not
// grow the process's footprint after start-up, or a caller that runs the
// search between other work where a cudaMalloc would synchronise the
// device.  For them this entry point computes what pa_debug_fstat computes
// for a mixed-precision, fixed-point-phase context -- the normalised F of
// one (sky point, spindown) -- with every device buffer carved out of one
// file-scope __device__ array of kNoAllocBytes (16 MB), which every GPU that
// loads the library holds until the process exits.  Host staging uses
// static arrays as well; the caller passes the inputs (settings, detector
// data) and the output array F, all in host memory.
//
// Limits: N <= 16384, nfft <= 16384, nfftf <= 32768, nifo <= 3; larger sizes
// are rejected with PA_ERR_ARG and a message in pa_last_error(NULL).
// The first call on a device looks up the array's device address
// (cudaGetSymbolAddress, with that device current) and caches it with the
// id of the device's current CUDA context; a later call in another context
// of that device (after a cudaDeviceReset, or when the application replaced
// the primary context) looks the address up again instead of using the
// stale one.  Make the first call on a device, and the first after such a
// reset, before any stream capture.  All calls share the array and it keeps
// the last call's contents: the call clears what must start at zero (the
// prelude's CTA counter and the candidate count) and overwrites the rest.
// Calls are serialised on the host by a mutex and every call, also one that
// fails part-way, waits for its own copies and kernels before it releases
// the mutex; calls that overlap on the GPU (e.g. from another process
// sharing the device through the same library instance) race on the shared
// array.  The caller's current device is restored on return.

namespace {

constexpr size_t kNoAllocBytes = (size_t)16 << 20;
constexpr int kNoAllocMaxN = 16384, kNoAllocMaxNfft = 16384, kNoAllocMaxNfftf = 32768, kNoAllocMaxNifo = 3;
constexpr int kNoAllocCandCap = 1024;
constexpr int kNoAllocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

std::mutex g_noalloc_mu;
// per device: the array's device address and the id of the context it was
// looked up in (0: not looked up)
void* g_noalloc_dev_ptr[kNoAllocMaxDevices];
unsigned long long g_noalloc_ctx_id[kNoAllocMaxDevices];

// The id of the calling thread's current CUDA context (cuCtxGetCurrent +
// cuCtxGetId, reached through the runtime's driver entry points so that the
// library needs no link to the driver library); 0 when unavailable, in
// which case every call looks the address up again.
unsigned long long noalloc_current_ctx_id() {
  typedef int (*GetCurrent)(void**);
  typedef int (*GetId)(void*, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      get_current = (GetCurrent)f1;
      get_id = (GetId)f2;
    }
  }
  void* ctx = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0ull;
  return id;
}

// On every return after the lock is taken: wait for what the call enqueued
// (so that the next call cannot start while this one's copies and kernels
// still write the array) and make the caller's device current again.
struct NoAllocExit {
  cudaStream_t st;
  int prev_dev;
  bool enqueued = false;
  ~NoAllocExit() {
    if (enqueued) cudaStreamSynchronize(st);
    if (prev_dev >= 0) cudaSetDevice(prev_dev);
  }
};
alignas(64) unsigned char g_noalloc_engine_mem[4096];
// host staging: the largest twiddle set (tw1 + tw2 + 1024 + L/1024 complex
// doubles for L <= 2^16) and one real array of N floats
double g_noalloc_tw[2 * (256 + 256 + 1024 + 64)];
float g_noalloc_tw_f[2 * (256 + 256 + 1024 + 64)];
float g_noalloc_real[kNoAllocMaxN];
float g_noalloc_F[kNoAllocMaxNfftf];
float g_noalloc_tw_pass[2 * kNoAllocMaxNfftf];  // host staging of Buffers::tw_pass

// 256-byte aligned bump layout inside the scratch array
struct Bump {
  char* base;
  size_t off = 0;
  void* take(size_t bytes) {
    off = (off + 255) & ~(size_t)255;
    void* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  }
};

int noalloc_fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_create_error = buf;
  return code;
}

// Lays the buffers of one search out in the scratch (or only sizes them
// when base == nullptr); returns the bytes used.
size_t noalloc_layout(char* base, const pa_settings& s, int nifo, pa::Buffers* b, void* tw[4][4], void** Fn) {
  Bump m{base};
  const size_t N = s.N, cs = 8;
  const int bins = s.nmax - s.nmin;
  memset(b, 0, sizeof(*b));
  b->xDat = (const double*)m.take(8 * nifo * N);
  b->DetSSB = (const double*)m.take(8 * nifo * 3 * N);
  b->cosmodf = m.take(4 * N);
  b->sinmodf = m.take(4 * N);
  b->dc = (const pa::DetConst*)m.take(sizeof(pa::DetConst) * pa::kMaxDet);
  b->spline_invp = (const double*)m.take(8 * 64);
  b->spline_p = (const double*)m.take(8 * 64);
  b->xin = m.take(cs * nifo * 2 * N);
  b->spec = m.take(cs * nifo * 2 * (size_t)s.nfft);
  b->yint = m.take(cs * nifo * 2 * (size_t)s.Ninterp);
  b->u = (double*)m.take(16 * nifo * 2 * 2 * N);
  b->y2 = m.take(cs * nifo * 2 * 2 * N);
  b->shftf = (double*)m.take(8 * nifo * N);
  b->xm[0] = b->xm[1] = m.take(32 * nifo * N);  // 32-byte records
  b->sums[0] = b->sums[1] = (double*)m.take(8 * 8);
  b->sums_r[0] = b->sums_r[1] = m.take(8 * 4);
  b->part = (double*)m.take(8 * 2 * nifo * ((N + 255) / 256));
  b->counter = (unsigned int*)m.take(16);
  b->ybuf_pre = m.take(cs * nifo * 2 * (size_t)s.Ninterp);
  b->ybuf = m.take(cs * 2 * (size_t)s.nfftf);
  b->F = m.take(4 * (size_t)bins);
  b->mu = m.take(16);
  *Fn = m.take(4 * (size_t)bins);  // normalised F (the output)
  b->cand = (pa::DevCand*)m.take(sizeof(pa::DevCand) * kNoAllocCandCap);
  b->ncand = (int*)m.take(16);
  b->tw_pass[0] = m.take(cs * (size_t)s.nfftf);
  b->tw_pass[1] = m.take(cs * (size_t)s.nfftf);
  const int lens[4] = {s.nfft, s.Ninterp, s.nfftf, s.nfft};
  for (int t = 0; t < 4; t++) {
    int lg = 0;
    while ((1 << lg) < lens[t]) ++lg;
    const int n4[4] = {1 << ((lg + 1) / 2), 1 << (lg / 2), 1024, lens[t] / 1024};
    for (int k = 0; k < 4; k++) tw[t][k] = m.take(cs * (size_t)n4[k]);
  }
  b->N = s.N;
  b->nfft = s.nfft;
  b->Ninterp = s.Ninterp;
  b->nfftf = s.nfftf;
  b->nmin = s.nmin;
  b->nmax = s.nmax;
  b->bins = bins;
  b->nblk = bins / PA_NAVFSTAT;
  b->nifo = nifo;
  b->fftpad = s.fftpad;
  b->sbatch = 1;
  b->lane_sb = 1;
  b->cand_cap = kNoAllocCandCap;
  for (int k = 0; k < 4; k++) {
    b->tw_fwd[k] = tw[0][k];
    b->tw_inv[k] = tw[1][k];
    b->tw_main[k] = tw[2][k];
    b->tw_invh[k] = tw[3][k];
  }
  return m.off;
}

// Twiddle tables of length L and sign into the device pointers t[0..3],
// through the static host staging arrays.
cudaError_t noalloc_twiddles(int L, int sign, void* const* t, cudaStream_t st) {
  int lg = 0;
  while ((1 << lg) < L) ++lg;
  const int L1 = 1 << ((lg + 1) / 2), L2 = 1 << (lg / 2);
  const int lens[4] = {L1, L2, 1024, L / 1024};
  for (int k = 0; k < 4; k++) {
    for (int j = 0; j < lens[k]; j++) {
      long num, den;
      if (k == 0) { num = j; den = L1; }
      else if (k == 1) { num = j; den = L2; }
      else if (k == 2) { num = j; den = L; }
      else { num = (long)j * 1024; den = L; }
      host_twiddle(num, den, sign, &g_noalloc_tw[2 * j], &g_noalloc_tw[2 * j + 1]);
      g_noalloc_tw_f[2 * j] = (float)g_noalloc_tw[2 * j];
      g_noalloc_tw_f[2 * j + 1] = (float)g_noalloc_tw[2 * j + 1];
    }
    cudaError_t e = cudaMemcpyAsync(t[k], g_noalloc_tw_f, sizeof(float) * 2 * lens[k], cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    e = cudaStreamSynchronize(st);  // the staging array is reused
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace

extern "C" int pa_fstat_noalloc(const pa_settings* sett, const pa_detector* det, int nifo, int pm, int mm,
                                int nn, int ss, const pa_opts* o, int device, double* F) {
  if (!sett || !det || !o || !F) return noalloc_fail(PA_ERR_ARG, "pa_fstat_noalloc: null argument");
  char why[256];
  pa_config cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.precision = PA_PREC_MIXED;
  cfg.phase_mode = PA_PHASE_FIXED;
  cfg.device = device;
  if (validate(sett, nifo, &cfg, why, sizeof why)) return noalloc_fail(PA_ERR_ARG, "pa_fstat_noalloc: %s", why);
  if (sett->N > kNoAllocMaxN || sett->nfft > kNoAllocMaxNfft || sett->nfftf > kNoAllocMaxNfftf ||
      nifo > kNoAllocMaxNifo)
    return noalloc_fail(PA_ERR_ARG,
                        "pa_fstat_noalloc: N=%d nfft=%d nfftf=%d nifo=%d beyond the no-allocation limits "
                        "(N <= %d, nfft <= %d, nfftf <= %d, nifo <= %d)",
                        sett->N, sett->nfft, sett->nfftf, nifo, kNoAllocMaxN, kNoAllocMaxNfft, kNoAllocMaxNfftf,
                        kNoAllocMaxNifo);
  for (int n = 0; n < nifo; n++)
    if (!det[n].xDat || !det[n].DetSSB || !(det[n].sig2 > 0))
      return noalloc_fail(PA_ERR_ARG, "pa_fstat_noalloc: detector %d: missing data or sig2 <= 0", n);
  if (device < 0 || device >= kNoAllocMaxDevices || device >= pa_device_count())
    return noalloc_fail(PA_ERR_NODEV, "pa_fstat_noalloc: no CUDA device %d", device);
  pa::Buffers b;
  void* tw[4][4];
  void* Fn = nullptr;
  const size_t need = noalloc_layout(nullptr, *sett, nifo, &b, tw, &Fn);
  if (need > kNoAllocBytes)
    return noalloc_fail(PA_ERR_ARG, "pa_fstat_noalloc: needs %zu bytes of scratch, the array holds %zu", need,
                        kNoAllocBytes);

  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  int prev_dev = -1;
  if (cudaGetDevice(&prev_dev) != cudaSuccess) prev_dev = -1;
  const cudaStream_t st = cudaStreamPerThread;
  NoAllocExit on_exit{st, prev_dev};
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return noalloc_fail(PA_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
  const unsigned long long ctx_id = noalloc_current_ctx_id();
  if (!g_noalloc_dev_ptr[device] || ctx_id == 0 || ctx_id != g_noalloc_ctx_id[device]) {
    // set-up on this device (or in a new context of it): the device address
    // of the array
    void* ptr = nullptr;
    g_noalloc_dev_ptr[device] = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr)
      return noalloc_fail(PA_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_noalloc_dev_ptr[device] = ptr;
    g_noalloc_ctx_id[device] = ctx_id;
  }
  noalloc_layout((char*)g_noalloc_dev_ptr[device], *sett, nifo, &b, tw, &Fn);

  // host-side scalars of the sky point, as job_core computes them
  pa_ctx c;
  c.sett = *sett;
  c.nifo = nifo;
  c.cfg = cfg;
  c.fp64 = false;
  c.rsz = 4;
  c.dev = device;
  set_det_consts(&c, det);
  SkyHost h;
  sky_setup(&c, pm, mm, nn, o, ss, ss, &h);
  if (!h.inside) return noalloc_fail(PA_ERR_ARG, "pa_fstat_noalloc: sky point outside the grid disk");

#define NCK(call, what)                                                                    \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return noalloc_fail(PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
  } while (0)
  const size_t N = sett->N;
  on_exit.enqueued = true;
  for (int n = 0; n < nifo; n++) {
    NCK(cudaMemcpyAsync((double*)b.xDat + n * N, det[n].xDat, 8 * N, cudaMemcpyHostToDevice, st), "upload");
    NCK(cudaMemcpyAsync((double*)b.DetSSB + n * 3 * N, det[n].DetSSB, 8 * 3 * N, cudaMemcpyHostToDevice, st),
        "upload");
  }
  NCK(cudaMemcpyAsync((void*)b.dc, c.dc, sizeof(pa::DetConst) * nifo, cudaMemcpyHostToDevice, st), "upload");
  for (int k = 0; k < 2; k++) {
    for (size_t i = 0; i < N; i++) {
      const double omrt = sett->omr * (double)i;  // init.c:450-455
      g_noalloc_real[i] = (float)(k == 0 ? cos(omrt) : sin(omrt));
    }
    NCK(cudaMemcpyAsync((void*)(k == 0 ? b.cosmodf : b.sinmodf), g_noalloc_real, 4 * N, cudaMemcpyHostToDevice,
                        st), "upload");
    NCK(cudaStreamSynchronize(st), "upload");  // the staging array is reused
  }
  double invp[64], p[64];
  p[0] = invp[0] = 0.;
  for (int i = 1; i < 64; i++) {  // auxi.c:71-72
    invp[i] = 2. / (p[i - 1] + 4.);
    p[i] = -.5 * invp[i];
  }
  NCK(cudaMemcpyAsync((void*)b.spline_invp, invp, sizeof(invp), cudaMemcpyHostToDevice, st), "upload");
  NCK(cudaMemcpyAsync((void*)b.spline_p, p, sizeof(p), cudaMemcpyHostToDevice, st), "upload");
  NCK(noalloc_twiddles(sett->nfft, -1, tw[0], st), "twiddles");
  NCK(noalloc_twiddles(sett->Ninterp, +1, tw[1], st), "twiddles");
  NCK(noalloc_twiddles(sett->nfftf, -1, tw[2], st), "twiddles");
  NCK(noalloc_twiddles(sett->nfft, +1, tw[3], st), "twiddles");
  for (int sp = 0; sp < 2; sp++) {
    const long L = sett->nfftf;
    int lg = 0;
    while ((1L << lg) < L) ++lg;
    const int l1 = pa::pass_logl1(lg, sp);
    for (long j = 0; j < L; j++) {
      double re, im;
      host_twiddle(pa::tw_pass_exp(j, L, l1), L, -1, &re, &im);
      g_noalloc_tw_pass[2 * j] = (float)re;
      g_noalloc_tw_pass[2 * j + 1] = (float)im;
    }
    NCK(cudaMemcpyAsync((void*)b.tw_pass[sp], g_noalloc_tw_pass, sizeof(float) * 2 * L, cudaMemcpyHostToDevice,
                        st), "twiddles");
    NCK(cudaStreamSynchronize(st), "twiddles");  // the staging array is reused
  }
  // what must start at zero
  NCK(cudaMemsetAsync(b.counter, 0, 16, st), "memset");
  NCK(cudaMemsetAsync(b.ncand, 0, 16, st), "memset");

  pa::Engine* eng = pa::make_engine_f32_fixed_at(g_noalloc_engine_mem, sizeof(g_noalloc_engine_mem), b);
  if (!eng) return noalloc_fail(PA_ERR_NOMEM, "pa_fstat_noalloc: engine storage too small");
  const pa::SkyArgs a = sky_args(&c, h, 0);
  e = eng->prelude(a, 0, st);
  if (e == cudaSuccess) e = eng->spindowns(a, 0, 0, ss, 1, o->trl, o->white_flag, o->s0_flag, st, Fn);
  const int bins = sett->nmax - sett->nmin;
  if (e == cudaSuccess) e = cudaMemcpyAsync(g_noalloc_F, Fn, 4 * (size_t)bins, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  eng->~Engine();
  if (e != cudaSuccess) return noalloc_fail(PA_ERR_CUDA, "pa_fstat_noalloc: %s", cudaGetErrorString(e));
  for (int i = 0; i < bins; i++) F[i] = g_noalloc_F[i];
#undef NCK
  return PA_OK;
}

// ------------------------------------------------------------------
// Multi-segment front-end: the batches of several contexts (one per data
// segment, each with its own N and FFT lengths) enqueued together, each on
// its own streams forked from one origin stream, optionally captured into
// one CUDA graph and launched once.

struct pa_segments {
  std::vector<pa_ctx*> ctx;
  int dev = 0;
  cudaStream_t origin = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> fork, join;
  bool graph = true;
  cudaGraphExec_t gexec = nullptr;
  double last_ms = 0.;
  std::string err;
};

namespace {
thread_local std::string g_seg_error;

int seg_fail(pa_segments* s, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (s) s->err = buf;
  else g_seg_error = buf;
  return code;
}

#define SCK(call, what)                                                                                   \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) return seg_fail(sg, PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_));      \
  } while (0)

// Enqueues every segment's batch, forked from and joined back into the
// origin stream.
int seg_enqueue(pa_segments* sg, const std::vector<std::vector<SkyHost>>& hs, const pa_segment_job* jobs) {
  for (size_t k = 0; k < sg->ctx.size(); k++) {
    pa_ctx* c = sg->ctx[k];
    SCK(cudaEventRecord(sg->fork[k], sg->origin), "cudaEventRecord");
    SCK(cudaStreamWaitEvent(c->stream, sg->fork[k], 0), "cudaStreamWaitEvent");
    int rc = enqueue_tasks(c, hs[k], jobs[k].opts);
    if (rc) return seg_fail(sg, rc, "segment %d: %s", (int)k, c->err.c_str());
    SCK(cudaEventRecord(sg->join[k], c->stream), "cudaEventRecord");
    SCK(cudaStreamWaitEvent(sg->origin, sg->join[k], 0), "cudaStreamWaitEvent");
  }
  return PA_OK;
}
}  // namespace

extern "C" {

pa_segments* pa_segments_create(pa_ctx* const* ctxs, int nseg, int* status) {
  if (!ctxs || nseg < 1) {
    seg_fail(nullptr, PA_ERR_ARG, "pa_segments_create: no contexts");
    if (status) *status = PA_ERR_ARG;
    return nullptr;
  }
  for (int k = 0; k < nseg; k++)
    if (!ctxs[k] || ctxs[k]->dev != ctxs[0]->dev) {
      seg_fail(nullptr, PA_ERR_ARG, "pa_segments_create: context %d missing or on another device", k);
      if (status) *status = PA_ERR_ARG;
      return nullptr;
    }
  pa_segments* sg = new pa_segments();
  sg->ctx.assign(ctxs, ctxs + nseg);
  sg->dev = ctxs[0]->dev;
  sg->fork.assign(nseg, nullptr);
  sg->join.assign(nseg, nullptr);
  auto bad = [&](cudaError_t e) {
    g_seg_error = std::string("pa_segments_create: ") + cudaGetErrorString(e);
    pa_segments_destroy(sg);
    if (status) *status = PA_ERR_CUDA;
    return (pa_segments*)nullptr;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(sg->dev)) != cudaSuccess) return bad(e);
  if ((e = cudaStreamCreateWithFlags(&sg->origin, cudaStreamNonBlocking)) != cudaSuccess) return bad(e);
  if ((e = cudaEventCreate(&sg->ev0)) != cudaSuccess) return bad(e);
  if ((e = cudaEventCreate(&sg->ev1)) != cudaSuccess) return bad(e);
  for (int k = 0; k < nseg; k++) {
    if ((e = cudaEventCreateWithFlags(&sg->fork[k], cudaEventDisableTiming)) != cudaSuccess) return bad(e);
    if ((e = cudaEventCreateWithFlags(&sg->join[k], cudaEventDisableTiming)) != cudaSuccess) return bad(e);
  }
  if (status) *status = PA_OK;
  return sg;
}

void pa_segments_destroy(pa_segments* sg) {
  if (!sg) return;
  cudaSetDevice(sg->dev);
  if (sg->origin) cudaStreamSynchronize(sg->origin);
  if (sg->gexec) cudaGraphExecDestroy(sg->gexec);
  for (cudaEvent_t e : sg->fork)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : sg->join)
    if (e) cudaEventDestroy(e);
  if (sg->ev0) cudaEventDestroy(sg->ev0);
  if (sg->ev1) cudaEventDestroy(sg->ev1);
  if (sg->origin) cudaStreamDestroy(sg->origin);
  delete sg;
}

const char* pa_segments_last_error(const pa_segments* sg) { return sg ? sg->err.c_str() : g_seg_error.c_str(); }

int pa_segments_set_graph(pa_segments* sg, int on) {
  if (!sg) return PA_ERR_ARG;
  sg->graph = on != 0;
  return PA_OK;
}

double pa_segments_last_call_ms(const pa_segments* sg) { return sg ? sg->last_ms : 0.; }

int pa_segments_search(pa_segments* sg, const pa_segment_job* jobs, int* status) {
  pa::TraceRange trace_("pa_segments_search");
  if (!sg || !jobs) return seg_fail(sg, PA_ERR_ARG, "pa_segments_search: bad arguments");
  const int ns = (int)sg->ctx.size();
  for (int k = 0; k < ns; k++) {
    const pa_segment_job& j = jobs[k];
    if ((j.ntasks > 0 && !j.tasks) || j.ntasks < 0 || !j.opts || !j.range || !j.sgnlc || !j.sgnlv || !j.FNum ||
        j.cap < 0)
      return seg_fail(sg, PA_ERR_ARG, "pa_segments_search: bad job %d", k);
  }
  SCK(cudaSetDevice(sg->dev), "cudaSetDevice");
  std::vector<std::vector<SkyHost>> hs(ns);
  bool profiling = false;
  for (int k = 0; k < ns; k++) {
    const pa_segment_job& j = jobs[k];
    hs[k].resize(j.ntasks);
    for (int t = 0; t < j.ntasks; t++)
      sky_setup(sg->ctx[k], j.tasks[t].pm, j.tasks[t].mm, j.tasks[t].nn, j.opts,
                t == 0 ? j.range->sst : j.range->spndr[0], j.range->spndr[1], &hs[k][t]);
    profiling |= sg->ctx[k]->prof.on;
  }
  int rc;
  if (sg->graph && !profiling) {
    SCK(cudaStreamBeginCapture(sg->origin, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    rc = seg_enqueue(sg, hs, jobs);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(sg->origin, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return seg_fail(sg, PA_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    rc = graph_exec_from(g, &sg->gexec, &sg->err);
    cudaGraphDestroy(g);
    if (rc) return rc;
    // timing starts at the launch (capture and update are host work)
    SCK(cudaEventRecord(sg->ev0, sg->origin), "cudaEventRecord");
    SCK(cudaGraphLaunch(sg->gexec, sg->origin), "cudaGraphLaunch");
  } else {
    SCK(cudaEventRecord(sg->ev0, sg->origin), "cudaEventRecord");
    if ((rc = seg_enqueue(sg, hs, jobs))) return rc;
  }
  SCK(cudaEventRecord(sg->ev1, sg->origin), "cudaEventRecord");
  SCK(cudaStreamSynchronize(sg->origin), "segments");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, sg->ev0, sg->ev1);
  sg->last_ms = ms;
  int worst = PA_OK;
  for (int k = 0; k < ns; k++) {
    pa_ctx* c = sg->ctx[k];
    const pa_segment_job& j = jobs[k];
    if (c->prof.on) prof_collect(c);
    std::vector<pa::DevCand> cands;
    int n = 0;
    rc = collect_tasks(c, &cands, &n);
    if (rc == PA_ERR_CAPACITY) {
      // device buffer overflow: grow and run this segment again on its own
      rc = grow_candidates(c, n);
      if (rc == PA_OK) rc = run_tasks(c, hs[k], j.opts, &cands);
    }
    if (rc == PA_OK)
      rc = append_records(c, hs[k], j.opts, cands, j.sgnlc, j.sgnlv, j.cap, j.idx, j.FNum, j.needed);
    if (status) status[k] = rc;
    if (rc && !worst) {
      worst = rc;
      sg->err = "segment " + std::to_string(k) + ": " + c->err;
    }
  }
  return worst;
}

}  // extern "C"
