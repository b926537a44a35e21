// pa_engine.h -- host-side interface between the C-ABI layer (pa_api.cu) and
// the templated device engines (pa_engine_f32.cu, pa_engine_f64.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pa {

// log2 of the pass-A column length L1 of a length 2^logL transform with
// factor split `split` (0: L1 = 2^ceil(logL/2); 1, odd logL only: 2^floor)
inline int pass_logl1(int logL, int split) { return (split && (logL & 1)) ? logL / 2 : (logL + 1) / 2; }
// exponent m of W_L^m at entry j of Buffers::tw_pass[split]: the inter-pass
// twiddle W_L^{n2 k1} at (n2 << logL1) + k1
inline long tw_pass_exp(long j, long L, int logL1) {
  return ((j >> logL1) * (j & ((1L << logL1) - 1))) % L;
}

constexpr int kMaxDet = 8;

// Per-context constants of one detector (uploaded once).
struct DetConst {
  double amod[9];
  double sig2, inv_sig2;
  double sphir, cphir;
  float amod_f[9], inv_sig2_f;  // FP32 copies (no per-thread conversions)
};

// Per-sky-point scalars, computed on the host in FP64 exactly as
// job_core() does (jobcore.c:243-299) and passed by value to the kernels.
struct SkyArgs {
  double het0;            // fmod(nn M8 + mm M12, M0)
  double oms;
  double sinal, cosal, sindel, cosdel;
  double nS[3];           // unit vector to the source
  double shft1[kMaxDet];  // nS . DetSSB[0..2] per detector
  double cosalfr[kMaxDet], sinalfr[kMaxDet];  // modvir rotated angles
  double s1_0;            // nn M9 + mm M13 (0 with --nospindown); over 2 pi
                          // in the fixed-point phase mode
  double M5;              // spindown step (0 with --nospindown); over 2 pi
                          // in the fixed-point phase mode
  double M0, M4;          // frequency step, het1 step
  // FP32 forms: the prelude and spindown phase terms as exact 64-bit
  // fixed-point turns of the FP64 values (turns_fixed)
  unsigned long long h0f; // het0 / 2 pi
  unsigned long long s1f; // s1_0 (already over 2 pi), fixed-point phase mode
  unsigned long long m5f; // M5 (already over 2 pi), fixed-point phase mode
  double oms_t;           // oms / 2 pi
  float cosalfr_f[kMaxDet], sinalfr_f[kMaxDet], cosdel_f, sindel_f;  // FP32 copies
  int ss_base;            // first spindown of the sky point (fixed-point form)
  int task;               // index of the sky point in the current batch
};

// One candidate found on the device (frequency bin ii is absolute).
struct DevCand {
  int task, ss, ii, pad;
  double F;
};

// Device buffers owned by the context and shared with the engine.
struct Buffers {
  int N, nfft, Ninterp, nfftf, nmin, nmax, bins, nblk, nifo, fftpad;
  int sbatch;                       // spindowns per fused launch
  const double* xDat;               // [nifo][N]
  const double* DetSSB;             // [nifo][3N]
  const void* cosmodf;              // [N] Real
  const void* sinmodf;              // [N] Real
  const DetConst* dc;               // [nifo]
  const double* spline_invp;        // [64] pivots 2/(p+4) of the spline solve
  const double* spline_p;           // [64] p_i
  void* xin;                        // [nifo][2][N] Real complex
  void* spec;                       // [nifo][2][nfft]
  void* yint;                       // [nifo][2][Ninterp]
  double* u;                        // [nifo][2][2N] double2
  void* y2;                         // [nifo][2][2N] Real complex
  double* shftf;                    // [nifo][N]
  // per-sky prelude outputs, double-buffered (slot 0/1) so that the prelude
  // of one sky point runs while the spindowns of the previous one read the
  // other slot
  void* ph0[2];                     // FP64 form: tmp1 [nifo][N]
  void* xm[2];                      // FP32 forms: [nifo][N] 32-byte records
                                    // {xa, xb | phase terms}; FP64 form:
                                    // [nifo][2][N] double complex
  double* sums[2];                  // aa, bb, 1/aa, 1/bb
  void* sums_r[2];                  // 1/aa, 1/bb in the working precision
  double* part;                     // partial sums of a^2, b^2
  void* ybuf_pre;                   // FFT intermediate of the prelude, nifo*2*Ninterp
  unsigned int* counter;            // CTA completion counter of the prelude (kept 0)
  void* ybuf;                       // FFT intermediate of the spindown loop, 2*lane_sb*2*nfftf
  void* F;                          // [2*lane_sb][bins] Real
  int lane_sb;                      // spindowns per lane of ybuf and F: lane 1 starts at
                                    // spindown lane_sb (two lanes run on two streams)
  void* mu;                         // [sbatch][nblk] Real
  DevCand* cand;
  int* ncand;
  int cand_cap;
  // twiddle tables (Real complex) per transform
  const void* tw_fwd[4];            // nfft forward: tw1, tw2, twlo, twhi
  const void* tw_inv[4];            // Ninterp backward (its twlo/twhi give e^{+i pi j/nfft})
  const void* tw_invh[4];           // nfft backward (the half-length resampling transform)
  const void* tw_main[4];           // nfftf forward
  // FP32 forms: the inter-pass twiddles W_L^{n2 k1} of the spindown
  // transform (L = nfftf) at (n2 << logL1) + k1 for each factor split
  // (pass_logl1), nfftf entries each; both pointers equal for even log2 L
  const void* tw_pass[2];
};

// Kernel kinds for the optional per-launch CUDA-event profile.
enum KernelKind {
  KK_PRELUDE_MOD = 0, KK_FFT_FWD_A, KK_FFT_FWD_B, KK_FFT_INV_A, KK_FFT_INV_B, KK_SPLINE_FWD, KK_SPLINE_BWD,
  KK_SPLINT, KK_SPIN_A, KK_SPIN_B, KK_THRESHOLD, KK_COUNT
};
const char* kernel_kind_name(int k);

// Event-bracketed launches recorded while profiling is on.
struct Prof {
  bool on = false;
  struct Rec {
    int kind, items;
    cudaEvent_t a, b;
  };
  Rec* recs = nullptr;
  int n = 0, cap = 0;
  double total_ms[KK_COUNT] = {0};
  long long launches[KK_COUNT] = {0};
  long long items[KK_COUNT] = {0};
};

class Engine {
 public:
  Prof* prof = nullptr;  // owned by the context
  virtual ~Engine() {}
  // Enqueues the per-sky prelude (jobcore.c:270-393) on `st`, outputs to
  // prelude slot `slot`.
  virtual cudaError_t prelude(const SkyArgs& sky, int slot, cudaStream_t st) = 0;
  // Enqueues spindowns ss0 .. ss0+nb-1 reading prelude slot `slot` into
  // lane `lane` of ybuf and F (lane 0: nb <= 2*lane_sb; lane 1, which starts
  // at spindown lane_sb of the buffers: nb <= lane_sb): phase modulation, FFT,
  // F-statistic, normalisation, threshold and candidate compaction.  Fdbg
  // (optional): normalised F of the batch, [nb][bins] Real.
  virtual cudaError_t spindowns(const SkyArgs& sky, int slot, int lane, int ss0, int nb, double trl, int white,
                                int s0_flag, cudaStream_t st, void* Fdbg) = 0;
  virtual long long launches() const = 0;
  virtual size_t real_size() const = 0;
  // Factor split of the spindown FFT (0: L1 = 2^ceil(m/2); 1: swapped, for
  // odd m only; ignored for even m).
  virtual void set_split(int split) = 0;
  virtual int split() const = 0;
  // Detector whose 32-byte records (FP32 forms) hold {xb, xa} instead of
  // {xa, xb}, as the prelude writes them for the current split; -1: none.
  virtual int swapped_det() const = 0;
  // Per-CTA trace of this engine's kernels into buf (cap records of 48
  // bytes: start/end %globaltimer, start/end clock64, kernel kind, SM id);
  // buf == nullptr switches it off.  trace_count: records written so far
  // (may exceed cap; the excess is dropped).
  virtual cudaError_t set_trace(void* buf, unsigned int cap) = 0;
  virtual cudaError_t trace_count(unsigned int* n) = 0;
};

// Factories (defined in the per-precision translation units).
Engine* make_engine_f32(const Buffers& b, int phase_mode);
Engine* make_engine_f32_fixed_at(void* mem, size_t bytes, const Buffers& b);
Engine* make_engine_f64(const Buffers& b);


}  // namespace pa
