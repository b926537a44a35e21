// pa_fft.cuh -- shared-memory Stockham FFT building blocks for sm_103a.
//
// A length-L (L = L1*L2 = 2^m, 4096 <= L <= 2^20) complex FFT runs as two
// fused passes of the four-step scheme:
//   x[n] with n = L2*n1 + n2, X[k] with k = k1 + L1*k2
//   pass A: per column n2, Y[k1,n2] = W_L^{n2 k1} * sum_n1 x[L2 n1 + n2] W_L1^{n1 k1}
//   pass B: per row k1,    X[k1 + L1 k2] = sum_n2 Y[k1,n2] W_L2^{n2 k2}
// Each CTA transforms a tile of E complex values held in shared memory:
// pass A takes C = E/(2 L1) columns of the two arrays (a, b) of one batch
// item, pass B takes Rr = E/(2 L2) rows.  The inner FFTs are mixed-radix
// Stockham autosort stages (one radix-2 or radix-4 stage, then radix-8),
// butterflies in registers, data exchanged through shared memory between
// stages.  The tile layout s[e * Q + q] (element e of sequence q, sequence
// index fastest) keeps every stage's shared-memory access contiguous across
// a warp.  The intermediate Y is stored as ybuf[batch][n2][k1][arr]: pass A
// writes the a|b values of one (n2, k1) as one 16-byte pair, consecutive
// lanes on consecutive k1, and a pass-B tile reads Rr consecutive k1 (Rr x
// 16 contiguous bytes) at every n2.
//
// Loaders (pass A input) and storers (pass B output) are functors, so the
// phase modulation of the spindown loop, the zero padding, the resampling
// spectrum remap and the F-statistic epilogue are fused into the FFT passes
// and never stored as separate arrays.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pa {

template <typename R> struct CT;
template <> struct CT<float> { typedef float2 T; };
template <> struct CT<double> { typedef double2 T; };

__device__ __forceinline__ float2 mk(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ double2 mk(double a, double b) { return make_double2(a, b); }
template <class T> __device__ __forceinline__ T cadd(T a, T b) { return mk(a.x + b.x, a.y + b.y); }
template <class T> __device__ __forceinline__ T csub(T a, T b) { return mk(a.x - b.x, a.y - b.y); }
template <class T> __device__ __forceinline__ T cmul(T a, T b) {
  return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class T, class S> __device__ __forceinline__ T cscale(T a, S s) { return mk(a.x * s, a.y * s); }
// (SIGN i) * a
template <int SIGN, class T> __device__ __forceinline__ T mulj(T a) {
  return SIGN > 0 ? mk(-a.y, a.x) : mk(a.y, -a.x);
}

// Tile geometry of one FFT length (host fills, kernels read by value).
struct Geom {
  int L, logL;       // transform length
  int L1, logL1;     // pass-A (column) FFT length
  int L2, logL2;     // pass-B (row) FFT length
  int C, logC;       // columns per pass-A tile
  int Rr, logRr;     // rows per pass-B tile
  int twlo_log;      // log2 of the low twiddle table length (10)
};

template <int SIGN, class T> __device__ __forceinline__ void dft2(T* v) {
  T a = v[0];
  v[0] = cadd(a, v[1]);
  v[1] = csub(a, v[1]);
}

template <int SIGN, class T> __device__ __forceinline__ void dft4(T& a, T& b, T& c, T& d) {
  T apc = cadd(a, c), amc = csub(a, c), bpd = cadd(b, d), jbmd = mulj<SIGN>(csub(b, d));
  a = cadd(apc, bpd);
  b = cadd(amc, jbmd);
  c = csub(apc, bpd);
  d = csub(amc, jbmd);
}

template <int SIGN, class T> __device__ __forceinline__ void dft4v(T* v) { dft4<SIGN>(v[0], v[1], v[2], v[3]); }

// 8-point DFT: X[q] = E[q mod 4] + W8^q O[q mod 4], W8 = exp(SIGN 2 pi i / 8)
template <int SIGN, class T> __device__ __forceinline__ void dft8(T* v) {
  typedef decltype(v[0].x) R;
  const R h = (R)0.70710678118654752440084436210485;
  T e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
  T o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
  dft4<SIGN>(e0, e1, e2, e3);
  dft4<SIGN>(o0, o1, o2, o3);
  // o1 *= (1 + SIGN i)/sqrt2 ; o2 *= SIGN i ; o3 *= (-1 + SIGN i)/sqrt2
  T t1 = SIGN > 0 ? mk((o1.x - o1.y) * h, (o1.y + o1.x) * h) : mk((o1.x + o1.y) * h, (o1.y - o1.x) * h);
  T t2 = mulj<SIGN>(o2);
  T t3 = SIGN > 0 ? mk((-o3.x - o3.y) * h, (-o3.y + o3.x) * h) : mk((-o3.x + o3.y) * h, (-o3.y - o3.x) * h);
  v[0] = cadd(e0, o0);
  v[4] = csub(e0, o0);
  v[1] = cadd(e1, t1);
  v[5] = csub(e1, t1);
  v[2] = cadd(e2, t2);
  v[6] = csub(e2, t2);
  v[3] = cadd(e3, t3);
  v[7] = csub(e3, t3);
}

// x * exp(SIGN 2 pi i e / 16) for a compile-time e in 1 .. 9
template <int SIGN, int e, class T> __device__ __forceinline__ T w16(T x) {
  typedef decltype(x.x) R;
  if (e == 4) return mulj<SIGN>(x);
  // cos and sin of 2 pi e / 16 for e = 0 .. 9
  constexpr double kc[10] = {1., 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173, 0.,
                             -0.38268343236508977173, -0.70710678118654752440, -0.92387953251128675613, -1.,
                             -0.92387953251128675613};
  constexpr double ks[10] = {0., 0.38268343236508977173, 0.70710678118654752440, 0.92387953251128675613, 1.,
                             0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173, 0.,
                             -0.38268343236508977173};
  const R c = (R)kc[e], s = (R)(SIGN * ks[e]);
  return mk(x.x * c - x.y * s, x.x * s + x.y * c);
}

// 16-point DFT in natural order, as 4 x 4: X[k1 + 4 k2] =
// sum_n2 W4^{n2 k2} W16^{n2 k1} sum_n1 x[4 n1 + n2] W4^{n1 k1}
template <int SIGN, class T> __device__ __forceinline__ void dft16(T* v) {
#pragma unroll
  for (int n2 = 0; n2 < 4; ++n2) dft4<SIGN>(v[n2], v[4 + n2], v[8 + n2], v[12 + n2]);
  // v[n2 + 4 k1] now holds the inner transform (n2, k1)
  v[5] = w16<SIGN, 1>(v[5]);
  v[6] = w16<SIGN, 2>(v[6]);
  v[7] = w16<SIGN, 3>(v[7]);
  v[9] = w16<SIGN, 2>(v[9]);
  v[10] = w16<SIGN, 4>(v[10]);
  v[11] = w16<SIGN, 6>(v[11]);
  v[13] = w16<SIGN, 3>(v[13]);
  v[14] = w16<SIGN, 6>(v[14]);
  v[15] = w16<SIGN, 9>(v[15]);
  T o[16];
#pragma unroll
  for (int k1 = 0; k1 < 4; ++k1) {
    T a = v[4 * k1], b = v[4 * k1 + 1], c = v[4 * k1 + 2], d = v[4 * k1 + 3];
    dft4<SIGN>(a, b, c, d);
    o[k1] = a;
    o[k1 + 4] = b;
    o[k1 + 8] = c;
    o[k1 + 12] = d;
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = o[k];
}

template <int SIGN, int RAD, class T> __device__ __forceinline__ void dftr(T* v) {
  if (RAD == 2) dft2<SIGN>(v);
  else if (RAD == 4) dft4v<SIGN>(v);
  else dft8<SIGN>(v);
}

// Shared-memory tile: Cs pair-sequences of length L; element e of
// pair-sequence c, array arr (0 = a, 1 = b) lives at s[e*P + 2c + arr] with
// row pitch P = 2*Cs + PADE.  The a/b values of one element are adjacent
// and moved as one 16-byte access, and the 16-byte row padding keeps both
// lane mappings conflict-free: consecutive c (rows of 2*Cs elements) and
// consecutive e (stride P*sizeof(T) = 16 bytes mod 128).
template <class T> struct Pair;
template <> struct Pair<float2> {
  static constexpr int PADE = 2;
  __device__ __forceinline__ static void ld(const float2* p, float2& a, float2& b) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
  }
  __device__ __forceinline__ static void ldg(const float2* p, float2& a, float2& b) {
    const float4 v = __ldg(reinterpret_cast<const float4*>(p));
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
  }
  // last read of the data: evict-first
  __device__ __forceinline__ static void ldlast(const float2* p, float2& a, float2& b) {
    const float4 v = __ldcs(reinterpret_cast<const float4*>(p));
    a = make_float2(v.x, v.y);
    b = make_float2(v.z, v.w);
  }
  __device__ __forceinline__ static void st(float2* p, float2 a, float2 b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.x, a.y, b.x, b.y);
  }
};
template <> struct Pair<double2> {
  static constexpr int PADE = 1;
  __device__ __forceinline__ static void ld(const double2* p, double2& a, double2& b) {
    a = p[0];
    b = p[1];
  }
  __device__ __forceinline__ static void ldg(const double2* p, double2& a, double2& b) {
    a = __ldg(p);
    b = __ldg(p + 1);
  }
  __device__ __forceinline__ static void ldlast(const double2* p, double2& a, double2& b) {
    a = __ldcs(p);
    b = __ldcs(p + 1);
  }
  __device__ __forceinline__ static void st(double2* p, double2 a, double2 b) {
    p[0] = a;
    p[1] = b;
  }
};

template <int RAD> struct LogR { static constexpr int v = RAD == 2 ? 1 : (RAD == 4 ? 2 : 3); };

// Reads the RAD inputs of one pair-butterfly of a Stockham stage from shared
// memory, applies the stage twiddles W_{Ns RAD}^{k r} and transforms both
// arrays.  Lane mapping: JFAST -> consecutive j, else consecutive c.  All
// geometry is compile-time (LOGL: log2 of the sequence length, LOGCS: log2
// of the number of pair-sequences, P: tile row pitch, LOGNS: log2 Ns).
template <int SIGN, int RAD, int NT, bool JFAST, int LOGL, int LOGCS, int P, int LOGNS, class T>
__device__ __forceinline__ void stage_load(const T* s, const T* tw, int it, int& j, int& c, T (&va)[RAD],
                                           T (&vb)[RAD]) {
  constexpr int lr = LogR<RAD>::v;
  constexpr int logLR = LOGL - lr;
  constexpr int Ns = 1 << LOGNS;
  const int b = threadIdx.x + it * NT;
  if (JFAST) {
    j = b & ((1 << logLR) - 1);
    c = b >> logLR;
  } else {
    c = b & ((1 << LOGCS) - 1);
    j = b >> LOGCS;
  }
#pragma unroll
  for (int r = 0; r < RAD; ++r) Pair<T>::ld(s + (j + (r << logLR)) * P + 2 * c, va[r], vb[r]);
  if (Ns > 1) {
    const int k = j & (Ns - 1);
    constexpr int twshift = LOGL - LOGNS - lr;
#pragma unroll
    for (int r = 1; r < RAD; ++r) {
      const T w = tw[(k * r) << twshift];
      va[r] = cmul(va[r], w);
      vb[r] = cmul(vb[r], w);
    }
  }
  dftr<SIGN, RAD>(va);
  dftr<SIGN, RAD>(vb);
}

// A middle radix-8 stage: shared memory -> registers -> shared memory.
template <int SIGN, int E, int NT, int LOGL, int LOGCS, int P, int LOGNS, class T>
__device__ __forceinline__ void stage_mid(T* s, const T* tw) {
  constexpr int RAD = 8;
  constexpr int PPT = E / (2 * RAD * NT);
  constexpr int Ns = 1 << LOGNS;
  T va[PPT][RAD], vb[PPT][RAD];
  int jj[PPT], cc[PPT];
#pragma unroll
  for (int it = 0; it < PPT; ++it)
    stage_load<SIGN, RAD, NT, false, LOGL, LOGCS, P, LOGNS>(s, tw, it, jj[it], cc[it], va[it], vb[it]);
  __syncthreads();
#pragma unroll
  for (int it = 0; it < PPT; ++it) {
    const int d = ((jj[it] >> LOGNS) << (LOGNS + 3)) + (jj[it] & (Ns - 1));
#pragma unroll
    for (int r = 0; r < RAD; ++r) Pair<T>::st(s + (d + r * Ns) * P + 2 * cc[it], va[it][r], vb[it][r]);
  }
  __syncthreads();
}

// First stage (Ns = 1, no twiddles) from values produced by `src(e, c, a, b)`
// in registers, written to shared memory (c-fastest mapping).
struct NoHook {
  __device__ __forceinline__ void operator()() const {}
};

// (hook: shared-memory stores of the caller that the later stages read,
// issued just before this stage's barrier)
template <int SIGN, int RAD, int E, int NT, int LOGL, int LOGCS, int P, class T, class Src, class Hook = NoHook>
__device__ __forceinline__ void stage_first(T* s, const Src& src, const Hook& hook = Hook()) {
  constexpr int PPT = E / (2 * RAD * NT);
  constexpr int logLR = LOGL - LogR<RAD>::v;
#pragma unroll
  for (int it = 0; it < PPT; ++it) {
    const int b = threadIdx.x + it * NT;
    const int c = b & ((1 << LOGCS) - 1), j = b >> LOGCS;
    T va[RAD], vb[RAD];
#pragma unroll
    for (int r = 0; r < RAD; ++r) src(j + (r << logLR), c, va[r], vb[r]);
    dftr<SIGN, RAD>(va);
    dftr<SIGN, RAD>(vb);
#pragma unroll
    for (int r = 0; r < RAD; ++r) Pair<T>::st(s + (j * RAD + r) * P + 2 * c, va[r], vb[r]);
  }
  hook();
  __syncthreads();
}

// Middle stages from log2 Ns = LOGNS up to the last one (recursion on LOGNS).
template <int SIGN, int E, int NT, int LOGL, int LOGCS, int P, int LOGNS, class T>
__device__ __forceinline__ void stages_mid(T* s, const T* tw) {
  if constexpr (LOGNS + 3 < LOGL) {
    stage_mid<SIGN, E, NT, LOGL, LOGCS, P, LOGNS>(s, tw);
    stages_mid<SIGN, E, NT, LOGL, LOGCS, P, LOGNS + 3>(s, tw);
  }
}

// Radix of the first stage: 2, 4 or 8 by log2(L) mod 3; the rest are radix 8
template <int LOGL> struct FirstRadix {
  static constexpr int rem = LOGL % 3;
  static constexpr int v = rem == 1 ? 2 : (rem == 2 ? 4 : 8);
  static constexpr int logv = rem == 1 ? 1 : (rem == 2 ? 2 : 3);
};

// First stage and middle stages; the last radix-8 stage has Ns = L/8.
template <int SIGN, int E, int NT, int LOGL, int LOGCS, int P, class T, class Src, class Hook = NoHook>
__device__ __forceinline__ void fft_front(T* s, const T* tw, const Src& src, const Hook& hook = Hook()) {
  stage_first<SIGN, FirstRadix<LOGL>::v, E, NT, LOGL, LOGCS, P>(s, src, hook);
  stages_mid<SIGN, E, NT, LOGL, LOGCS, P, FirstRadix<LOGL>::logv>(s, tw);
}

// Per-precision tile configuration.
template <typename R> struct TileCfg;
// (4096-element FP32 tiles with 256 threads and 4 CTAs per SM were measured
// 1% slower on the spindown passes)
template <> struct TileCfg<float> {
  static constexpr int E = 8192;   // complex elements per tile (64 KB)
  static constexpr int NT = 512;   // threads per CTA
  static constexpr int MINB = 2;   // resident CTAs per SM the registers are sized for
};
template <> struct TileCfg<double> {
  static constexpr int E = 4096;   // 64 KB
  static constexpr int NT = 256;
  static constexpr int MINB = 2;
};

template <typename R> __host__ __device__ constexpr int tile_pitch(int Cs) {
  return 2 * Cs + Pair<typename CT<R>::T>::PADE;
}

// Compile-time tile geometry of a length 2^LOGL transform.
// SPLIT 0: L1 = 2^ceil(m/2) (pass A has the longer columns); SPLIT 1 swaps
// the two factors for odd m (pass A shorter columns, more per tile; the
// radix schedules of the passes swap with them).
template <typename R, int LOGL, int SPLIT = 0> struct FftShape {
  static constexpr int E = TileCfg<R>::E, NT = TileCfg<R>::NT;
  static constexpr int logE = E == 8192 ? 13 : (E == 4096 ? 12 : 11);
  static constexpr int LOGL1 = SPLIT ? LOGL / 2 : (LOGL + 1) / 2, LOGL2 = LOGL - LOGL1;
  static constexpr int L1 = 1 << LOGL1, L2 = 1 << LOGL2;
  static constexpr int LOGC = logE - 1 - LOGL1, C = 1 << LOGC;      // pass-A columns per tile
  static constexpr int LOGRR = logE - 1 - LOGL2, RR = 1 << LOGRR;   // pass-B rows per tile
  static constexpr int PA = tile_pitch<R>(C), PB = tile_pitch<R>(RR);
  static constexpr int smem_a = (L1 * PA + L1) * (int)sizeof(typename CT<R>::T) + 128;
  static constexpr int smem_b = (L2 * PB + L2) * (int)sizeof(typename CT<R>::T);
  static_assert(C <= L2 && RR <= L1, "transform too short for the tile");
};

// Optional per-CTA trace, a diagnostic of the launch structure (gaps
// between kernels, partial waves): when a trace buffer is set
// (Engine::set_trace), thread 0 of every CTA of the engine's kernels
// fills one record {%globaltimer at start and end, clock64 at start and
// end, kernel kind, SM id}, in the order the CTAs start.  The variables are
// per translation unit (static): each engine sets those of its own unit.
struct CtaTraceRec {
  unsigned long long t0, t1, c0, c1;
  unsigned int kind, smid, pad0, pad1;
};
#ifdef PA_CTA_TRACE
static __constant__ CtaTraceRec* c_trace_buf;
static __constant__ unsigned int c_trace_cap;
static __device__ unsigned int g_trace_n;
#endif

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// The record's slot is taken when the CTA starts, so that only its index
// stays live in a register through the kernel.  Even that register can
// make a 64-register kernel spill, so the trace exists only in the
// diagnostic build (-DPA_CTA_TRACE, polgraw-allsky_gb300/build.py
// build(trace=True)); in the product build CtaTrace is empty.
#ifdef PA_CTA_TRACE
struct CtaTrace {
  unsigned int slot = 0xffffffffu;
  __device__ __forceinline__ explicit CtaTrace(int kind) {
    if (c_trace_buf && threadIdx.x == 0) {
      const unsigned long long t0 = global_ns(), c0 = clock64();
      const unsigned int i = atomicAdd(&g_trace_n, 1u);
      if (i < c_trace_cap) {
        unsigned int smid;
        asm volatile("mov.u32 %0, %%smid;" : "=r"(smid));
        c_trace_buf[i].t0 = t0;
        c_trace_buf[i].c0 = c0;
        c_trace_buf[i].kind = (unsigned int)kind;
        c_trace_buf[i].smid = smid;
        slot = i;
      }
    }
  }
  __device__ __forceinline__ ~CtaTrace() {
    if (slot != 0xffffffffu) {
      const unsigned long long c1 = clock64(), t1 = global_ns();
      c_trace_buf[slot].c1 = c1;
      c_trace_buf[slot].t1 = t1;
    }
  }
};
#else
struct CtaTrace {
  __device__ __forceinline__ explicit CtaTrace(int) {}
};
#endif

// Pass A: column FFTs of length L1 over C columns x 2 arrays of one batch
// item (blockIdx.y).  The first radix stage takes its inputs from the
// loader in registers; the last stage (lanes along k1) applies the
// inter-pass twiddle W_L^{n2 k1} and writes Y[n2][k1][a|b] straight to
// global memory, 16 contiguous bytes per lane.  The twiddle comes from the
// table twp of all of them at (n2 << LOGL1) + k1 when the loader's
// kTwiddleTable is set (the spindown transform of the FP32 forms), else as
// the product of the two tables twlo, twhi.
// Loader: prologue(batch, smem scratch) and load2(batch, n, a, b, scratch).
template <typename R, int SIGN, int LOGL, class Loader, int SPLIT = 0>
__global__ void __launch_bounds__(TileCfg<R>::NT, TileCfg<R>::MINB)
    k_pass_a(const __grid_constant__ Loader ld, const typename CT<R>::T* __restrict__ tw1,
             const typename CT<R>::T* __restrict__ twlo, const typename CT<R>::T* __restrict__ twhi,
             const typename CT<R>::T* __restrict__ twp, typename CT<R>::T* __restrict__ ybuf) {
  typedef typename CT<R>::T T;
  typedef FftShape<R, LOGL, SPLIT> G;
  constexpr int E = G::E, NT = G::NT, P = G::PA;
  CtaTrace trace_(Loader::kTraceKind);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  T* tws = s + G::L1 * P;
  char* lsm = reinterpret_cast<char*>(tws + G::L1);   // loader scratch
  const int batch = blockIdx.y;
  const int c0 = blockIdx.x << G::LOGC;
  auto src = [&](int n1, int c, T& a, T& b) { ld.load2(batch, (n1 << G::LOGL2) + c0 + c, a, b, lsm); };
  if constexpr (Loader::kEarlyLoads && G::L1 <= NT) {
    // no loader constants in shared memory: the column twiddles are stored
    // at the end of the first stage (as in pass B), no barrier before the
    // first loads
    const T twv = threadIdx.x < G::L1 ? tw1[threadIdx.x] : T();
    auto fill = [&]() {
      if (threadIdx.x < G::L1) tws[threadIdx.x] = twv;
    };
    fft_front<SIGN, E, NT, G::LOGL1, G::LOGC, P>(s, tws, src, fill);
  } else {
    for (int m = threadIdx.x; m < G::L1; m += NT) tws[m] = tw1[m];
    ld.prologue(batch, lsm);
    __syncthreads();
    fft_front<SIGN, E, NT, G::LOGL1, G::LOGC, P>(s, tws, src);
  }
  // last radix-8 stage, lanes along j (= k1 mod Ns)
  constexpr int LOGNS = G::LOGL1 - 3, Ns = 1 << LOGNS;
  constexpr int PPT = E / (2 * 8 * NT);
  constexpr int Lmask = (1 << LOGL) - 1;
  T* yb = ybuf + ((size_t)batch << (LOGL + 1));
#pragma unroll
  for (int it = 0; it < PPT; ++it) {
    int j, c;
    T va[8], vb[8];
    stage_load<SIGN, 8, NT, true, G::LOGL1, G::LOGC, P, LOGNS>(s, tws, it, j, c, va, vb);
    const int n2 = c0 + c;
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      const int k1 = j + r * Ns;
      T W;
      if constexpr (Loader::kTwiddleTable) {
        W = __ldg(&twp[((size_t)n2 << G::LOGL1) + k1]);
      } else {
        const int m = (n2 * k1) & Lmask;
        W = cmul(__ldg(&twlo[m & 1023]), __ldg(&twhi[m >> 10]));
      }
      Pair<T>::st(yb + (((size_t)n2 << G::LOGL1) + k1) * 2, cmul(va[r], W), cmul(vb[r], W));
    }
  }
}

// Pass B: row FFTs of length L2 over Rr rows (k1) x 2 arrays.  The first
// radix stage reads Y[n2][k1][a|b] from global memory (lanes along k1, 16
// contiguous bytes each); after the last stage every thread hands its
// outputs X[k1 + L1 k2] for both arrays to the storer:
//   Ctx begin() const   (per-thread constants, loaded when the CTA starts)
//   __device__ void put(const Ctx&, int batch, int k1, int k2, T a, T b, int logL1) const
// with consecutive lanes on consecutive k1.
template <typename R, int SIGN, int LOGL, class Storer, int SPLIT = 0>
__global__ void __launch_bounds__(TileCfg<R>::NT, TileCfg<R>::MINB)
    k_pass_b(const Storer st, const typename CT<R>::T* __restrict__ tw2,
             const typename CT<R>::T* __restrict__ ybuf) {
  typedef typename CT<R>::T T;
  typedef FftShape<R, LOGL, SPLIT> G;
  constexpr int E = G::E, NT = G::NT, P = G::PB;
  CtaTrace trace_(Storer::kTraceKind);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  T* tws = s + G::L2 * P;
  // batches in reverse launch order: pass A wrote the last batch items
  // last, so their intermediate is the likeliest to be still in L2
  const int batch = gridDim.y - 1 - blockIdx.y;
  const int k10 = blockIdx.x << G::LOGRR;
  const typename Storer::Ctx sctx = st.begin();
  const T* yb = ybuf + ((size_t)batch << (LOGL + 1));
  // the intermediate is read once, here: evict-first
  auto src = [&](int n2, int rr, T& a, T& b) {
    Pair<T>::ldlast(yb + (((size_t)n2 << G::LOGL1) + k10 + rr) * 2, a, b);
  };
  if constexpr (G::L2 <= NT) {
    // one twiddle per thread, loaded first and stored to shared memory at
    // the end of the first stage (which does not use it), so that the
    // intermediate's loads are not held behind a barrier
    const T twv = threadIdx.x < G::L2 ? tw2[threadIdx.x] : T();
    auto fill = [&]() {
      if (threadIdx.x < G::L2) tws[threadIdx.x] = twv;
    };
    fft_front<SIGN, E, NT, G::LOGL2, G::LOGRR, P>(s, tws, src, fill);
  } else {
    for (int m = threadIdx.x; m < G::L2; m += NT) tws[m] = tw2[m];
    __syncthreads();
    fft_front<SIGN, E, NT, G::LOGL2, G::LOGRR, P>(s, tws, src);
  }
  constexpr int LOGNS = G::LOGL2 - 3, Ns = 1 << LOGNS;
  constexpr int PPT = E / (2 * 8 * NT);
#pragma unroll
  for (int it = 0; it < PPT; ++it) {
    int j, rr;
    T va[8], vb[8];
    stage_load<SIGN, 8, NT, false, G::LOGL2, G::LOGRR, P, LOGNS>(s, tws, it, j, rr, va, vb);
#pragma unroll
    for (int r = 0; r < 8; ++r) st.put(sctx, batch, k10 + rr, j + r * Ns, va[r], vb[r], G::LOGL1);
  }
}

}  // namespace pa
