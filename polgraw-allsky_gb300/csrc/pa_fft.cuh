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
// a warp.  The intermediate Y is stored so that each pass-B tile is one
// contiguous block: ybuf[t][n2][arr][r] with t = k1 / Rr, r = k1 % Rr.
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

template <int SIGN, int RAD, class T> __device__ __forceinline__ void dftr(T* v) {
  if (RAD == 2) dft2<SIGN>(v);
  else if (RAD == 4) dft4v<SIGN>(v);
  else dft8<SIGN>(v);
}

// One Stockham stage of radix RAD over Q interleaved sequences of length L.
// PER butterflies per thread (PER * RAD * NT == Q * L).
template <int SIGN, int RAD, int PER, int NT, class T>
__device__ __forceinline__ void fft_stage(T* s, const T* tw, int L, int logL, int Ns, int logNs,
                                          int logQ) {
  const int Qmask = (1 << logQ) - 1;
  const int LR = L / RAD;
  const int logRAD = RAD == 2 ? 1 : (RAD == 4 ? 2 : 3);
  // twiddle index step L/(Ns*RAD)
  const int twshift = logL - logNs - logRAD;
  T v[PER][RAD];
  int jj[PER];
#pragma unroll
  for (int it = 0; it < PER; ++it) {
    const int b = threadIdx.x + it * NT;
    const int q = b & Qmask, j = b >> logQ;
    jj[it] = j;
#pragma unroll
    for (int r = 0; r < RAD; ++r) v[it][r] = s[((j + r * LR) << logQ) + q];
    if (Ns > 1) {
      const int k = j & (Ns - 1);
#pragma unroll
      for (int r = 1; r < RAD; ++r) v[it][r] = cmul(v[it][r], tw[(k * r) << twshift]);
    }
    dftr<SIGN, RAD>(v[it]);
  }
  __syncthreads();
#pragma unroll
  for (int it = 0; it < PER; ++it) {
    const int b = threadIdx.x + it * NT;
    const int q = b & Qmask, j = jj[it];
    const int idxD = ((j >> logNs) << (logNs + logRAD)) + (j & (Ns - 1));
#pragma unroll
    for (int r = 0; r < RAD; ++r) s[((idxD + r * Ns) << logQ) + q] = v[it][r];
  }
  __syncthreads();
}

// In-place FFT of 2^logQ interleaved sequences of length L = 2^logL held in
// shared memory (E = Q*L elements).  tw[m] = exp(SIGN 2 pi i m / L).
template <int SIGN, int E, int NT, class T>
__device__ __forceinline__ void cta_fft(T* s, const T* tw, int logL, int logQ) {
  const int L = 1 << logL;
  int Ns = 1, logNs = 0;
  const int rem = logL % 3;
  if (rem == 1) {
    fft_stage<SIGN, 2, E / (2 * NT), NT>(s, tw, L, logL, 1, 0, logQ);
    Ns = 2;
    logNs = 1;
  } else if (rem == 2) {
    fft_stage<SIGN, 4, E / (4 * NT), NT>(s, tw, L, logL, 1, 0, logQ);
    Ns = 4;
    logNs = 2;
  }
  for (; Ns < L; Ns <<= 3, logNs += 3) fft_stage<SIGN, 8, E / (8 * NT), NT>(s, tw, L, logL, Ns, logNs, logQ);
}

// Per-precision tile configuration.
template <typename R> struct TileCfg;
template <> struct TileCfg<float> {
  static constexpr int E = 8192;   // complex elements per tile (64 KB)
  static constexpr int NT = 512;   // threads per CTA
};
template <> struct TileCfg<double> {
  static constexpr int E = 4096;   // 64 KB
  static constexpr int NT = 256;
};

// Pass A: column FFTs of length L1 over C columns x 2 arrays of one batch
// item (blockIdx.y), twiddle W_L^{n2 k1}, store to the pass-B tile layout.
// Loader: __device__ void load2(int batch, int n, T& a, T& b) const, plus an
// optional per-CTA prologue  __device__ void prologue(int batch, char* smem) const.
template <typename R, int SIGN, class Loader>
__global__ void __launch_bounds__(TileCfg<R>::NT, 2)
    k_pass_a(const Loader ld, const Geom g, const typename CT<R>::T* __restrict__ tw1,
             const typename CT<R>::T* __restrict__ twlo, const typename CT<R>::T* __restrict__ twhi,
             typename CT<R>::T* __restrict__ ybuf) {
  typedef typename CT<R>::T T;
  constexpr int E = TileCfg<R>::E, NT = TileCfg<R>::NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  T* tws = s + E;
  char* lsm = reinterpret_cast<char*>(tws + g.L1);   // loader scratch
  const int batch = blockIdx.y;
  const int c0 = blockIdx.x << g.logC;
  const int logQ = g.logC + 1;
  for (int m = threadIdx.x; m < g.L1; m += NT) tws[m] = tw1[m];
  ld.prologue(batch, lsm);
  __syncthreads();
  const int cmask = g.C - 1;
  for (int e = threadIdx.x; e < (E >> 1); e += NT) {
    const int col = e & cmask, n1 = e >> g.logC;
    T va, vb;
    ld.load2(batch, (n1 << g.logL2) + c0 + col, va, vb, lsm);
    s[(n1 << logQ) + col] = va;
    s[(n1 << logQ) + g.C + col] = vb;
  }
  __syncthreads();
  cta_fft<SIGN, E, NT>(s, tws, g.logL1, logQ);
  // twiddle + store, V consecutive rows (32 bytes) per item
  constexpr int V = 32 / sizeof(T);
  constexpr int logV = V == 4 ? 2 : 1;
  const int Qmask = (1 << logQ) - 1;
  const int rgmask = (g.Rr >> logV) - 1, logRg = g.logRr - logV;
  const int Lmask = g.L - 1, lomask = (1 << g.twlo_log) - 1;
  T* yb = ybuf + ((size_t)batch << (g.logL + 1));
  for (int w = threadIdx.x; w < E / V; w += NT) {
    const int q = w & Qmask, rest = w >> logQ;
    const int rg = rest & rgmask, t = rest >> logRg;
    const int arr = q >> g.logC, col = q & cmask;
    const int n2 = c0 + col;
    __align__(16) T out[V];
#pragma unroll
    for (int v = 0; v < V; ++v) {
      const int k1 = (t << g.logRr) + (rg << logV) + v;
      const int m = (n2 * k1) & Lmask;
      const T W = cmul(__ldg(&twlo[m & lomask]), __ldg(&twhi[m >> g.twlo_log]));
      out[v] = cmul(s[(k1 << logQ) + q], W);
    }
    T* dst = yb + ((((size_t)t << g.logL2) + n2) * 2 + arr) * g.Rr + (rg << logV);
    float4* d4 = reinterpret_cast<float4*>(dst);
    const float4* o4 = reinterpret_cast<const float4*>(out);
    d4[0] = o4[0];
    d4[1] = o4[1];
  }
}

// Pass B: row FFTs of length L2 over Rr rows x 2 arrays; the storer writes
// the outputs.  Storer: __device__ void store(int batch, int t, const T* s,
// const Geom& g) const, called after the FFT with the tile in shared memory
// (element k2 of sequence q' = arr*Rr + r at s[k2*2Rr + q']).
template <typename R, int SIGN, class Storer>
__global__ void __launch_bounds__(TileCfg<R>::NT, 2)
    k_pass_b(const Storer st, const Geom g, const typename CT<R>::T* __restrict__ tw2,
             const typename CT<R>::T* __restrict__ ybuf) {
  typedef typename CT<R>::T T;
  constexpr int E = TileCfg<R>::E, NT = TileCfg<R>::NT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* s = reinterpret_cast<T*>(smem_raw);
  T* tws = s + E;
  const int batch = blockIdx.y, t = blockIdx.x;
  for (int m = threadIdx.x; m < g.L2; m += NT) tws[m] = tw2[m];
  const float4* src = reinterpret_cast<const float4*>(ybuf + ((size_t)batch << (g.logL + 1)) + (size_t)t * E);
  float4* dst = reinterpret_cast<float4*>(s);
  constexpr int NV = E * (int)sizeof(T) / 16;
  for (int i = threadIdx.x; i < NV; i += NT) dst[i] = __ldg(&src[i]);
  __syncthreads();
  cta_fft<SIGN, E, NT>(s, tws, g.logL2, g.logRr + 1);
  st.store(batch, t, s, g);
}

}  // namespace pa
