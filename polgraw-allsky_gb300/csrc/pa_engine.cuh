// pa_engine.cuh -- device kernels of the coherent-search hot path and the
// templated engine that enqueues them.  Included by the per-precision
// translation units only.
//
// Reference correspondence (search/network/src-cpu):
//   k_prelude_mod   modvir (settings.c:281-325), shft/shftf/_tmp1 and the
//                   prelude phase modulation (jobcore.c:277-313)
//   resample FFTs   jobcore.c:319-362 (pass A/B with PlainLoader; the
//                   interpolating inverse at half length: HalfShiftLoader,
//                   InterpStore)
//   k_spline_fwd/bwd spline() (auxi.c:56-81), FP64 chunked recurrences
//   k_splint        splint/splintpad (auxi.c:83-122) + 1/sig2 (jobcore.c:386-389)
//   (aa, bb: last-CTA reduction of k_prelude_mod, jobcore.c:375-393)
//   SpinLoader      spindown phase modulation (jobcore.c:455-623)
//   FstatStore      F = |Xa|^2/aa + |Xb|^2/bb (jobcore.c:635-638)
//   k_normthresh    FStat() block means and normalisation (auxi.c:214-240),
//                   threshold, run clustering, argmax (jobcore.c:659-669)
#pragma once
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>

#include "pa_engine.h"
#include "pa_fft.cuh"

namespace pa {

enum { PM_F64 = 0, PM_FIXED = 1, PM_FF = 2 };

constexpr double kTwoPiHi = 6.283185307179586232;       // 2 pi rounded to double
constexpr double kTwoPiLo = 2.4492935982947064e-16;      // 2 pi - kTwoPiHi
constexpr double kInvTwoPi = 0.15915494309189535;
constexpr double kTurnsPerRad64 = 2.9358905032820014e18;  // 2^64 / (2 pi)
// 2 pi as the sum of three floats with 12, 24 and 24 significant bits; k*A
// is exact for |k| < 2^12
constexpr float kTwoPiF_A = 6.28125f;
constexpr float kTwoPiF_B = 1.9353071693331003e-3f;
constexpr float kTwoPiF_C = 1.0253131677018246e-11f;
constexpr float kInvTwoPiF = 0.15915494309189533577f;

// x mod 1 as a 64-bit fixed-point fraction (t / 2^64), computed exactly
// from the bits of x with integer operations only: x = m 2^(e-1075) with the
// 53-bit integer significand m, so x 2^64 mod 2^64 = m << (e - 1011) (or
// >> for negative shifts), negated for x < 0.
__device__ __forceinline__ uint64_t turns_fixed(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) return 0ull;  // zero or subnormal: |x| < 2^-1022
  const unsigned long long m = (bits & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sh = e - 1011;
  unsigned long long t;
  if (sh >= 64) t = 0ull;
  else if (sh >= 0) t = m << sh;
  else if (sh > -64) t = m >> (-sh);
  else t = 0ull;
  return (bits >> 63) ? (0ull - t) : t;
}

// ------------------------------------------------------------------
// prelude: modvir + time shift + prelude phase modulation

// Sum of two values over a 256-thread block in a fixed order (xor tree in
// each warp, then warps in index order); the result is valid in every thread.
__device__ __forceinline__ void block_sum2(double& a, double& b, double (*red)[8]) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, off);
    b += __shfl_xor_sync(0xffffffffu, b, off);
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    red[0][w] = a;
    red[1][w] = b;
  }
  __syncthreads();
  double sa = 0., sb = 0.;
  for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
    sa += red[0][k];
    sb += red[1][k];
  }
  __syncthreads();
  a = sa;
  b = sb;
}

template <typename R, int PM>
__global__ void __launch_bounds__(256)
    k_prelude_mod(const double* __restrict__ xDat, const double* __restrict__ DetSSB,
                  const R* __restrict__ cosmodf, const R* __restrict__ sinmodf,
                  const DetConst* __restrict__ dc, const SkyArgs sky, int N,
                  typename CT<R>::T* __restrict__ xin, double* __restrict__ shftf, void* ph0,
                  double* __restrict__ part, double* __restrict__ sums, R* __restrict__ sums_r,
                  unsigned int* __restrict__ counter) {
  typedef typename CT<R>::T T;
  CtaTrace trace_(KK_PRELUDE_MOD);
  const int d = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  R a2r = 0, b2r = 0;
  // FP32 forms: shft at sample 0 of this detector, by the expression every
  // sample uses
  __shared__ double sh1[1];
  if (sizeof(R) == 4) {
    if (threadIdx.x == 0) {
      const double* D0 = DetSSB + 3 * (size_t)d * N;
      sh1[0] = fma(sky.nS[0], D0[0], fma(sky.nS[1], D0[1], __dmul_rn(sky.nS[2], D0[2])));
    }
    __syncthreads();
  }
  if (i < N) {
    const DetConst& k = dc[d];
    // modvir, settings.c:303-322
    // FP32 forms read the FP32 copies: no double-to-float conversion per
    // thread (conversions run on the FP64 pipe)
    const bool f32 = sizeof(R) == 4;
    const R cosalfr = f32 ? (R)sky.cosalfr_f[d] : (R)sky.cosalfr[d];
    const R sinalfr = f32 ? (R)sky.sinalfr_f[d] : (R)sky.sinalfr[d];
    const R cm = cosmodf[i], sm = sinmodf[i];
    const R c = cosalfr * cm + sinalfr * sm;
    const R s = sinalfr * cm - cosalfr * sm;
    const R cosdel = f32 ? (R)sky.cosdel_f : (R)sky.cosdel, sindel = f32 ? (R)sky.sindel_f : (R)sky.sindel;
    const R c2d = cosdel * cosdel, c2sd = sindel * cosdel;
    const R c2s = (R)2 * c * c, cs = c * s;
#define PA_AMOD(j) (f32 ? (R)k.amod_f[j] : (R)k.amod[j])
    const R k0 = PA_AMOD(0), k1 = PA_AMOD(1), k2 = PA_AMOD(2), k3 = PA_AMOD(3), k4 = PA_AMOD(4),
            k5 = PA_AMOD(5), k6 = PA_AMOD(6), k7 = PA_AMOD(7), k8 = PA_AMOD(8);
#undef PA_AMOD
    const R two_m = (R)2 - c2d;
    const R aa = k0 * two_m * c2s + k1 * two_m * (R)2 * cs + k2 * c2sd * c + k3 * c2sd * s -
                 k0 * two_m + k4 * c2d;
    const R bb = k5 * sindel * c2s + k6 * sindel * (R)2 * cs + k7 * cosdel * c + k8 * cosdel * s -
                 k5 * sindel;
    a2r = aa * aa;
    b2r = bb * bb;
    // shft, shftf, _tmp1 (jobcore.c:285-295)
    const double* D = DetSSB + 3 * ((size_t)d * N + i);
    const size_t o = (size_t)d * N + i;
    const double di = (double)i;
    R sp, cp;
    if (sizeof(R) == 8) {
      // FP64 form: the reference's rounding sequence (no FMA contraction):
      // shftf[0] must be exactly 0, as shft1 comes from the same expression
      // on the host; a contracted product would leave +-1 ulp there and push
      // the spline abscissa 2(i - shftf) below 0, where splint returns 0
      // (auxi.c:89).
      const double shft = __dadd_rn(__dadd_rn(__dmul_rn(sky.nS[0], D[0]), __dmul_rn(sky.nS[1], D[1])),
                                    __dmul_rn(sky.nS[2], D[2]));
      shftf[o] = shft - sky.shft1[d];
      const double tmp1 = __dadd_rn(__dmul_rn(di, di), __dmul_rn((double)(2 * i), shft));
      reinterpret_cast<double*>(ph0)[o] = tmp1;
      // prelude phase het0 i + oms shft (jobcore.c:299), FP64
      const double phase = __dadd_rn(__dmul_rn(sky.het0, di), __dmul_rn(sky.oms, shft));
      double sd, cd;
      sincos(phase, &sd, &cd);
      sp = (R)sd;
      cp = (R)cd;
    } else {
      // FP32 forms: shft with fused multiply-adds; shft1 is the same
      // expression at sample 0 (sh1, below), so shftf[0] is exactly 0
      const double shft = fma(sky.nS[0], D[0], fma(sky.nS[1], D[1], __dmul_rn(sky.nS[2], D[2])));
      shftf[o] = shft - sh1[0];
      // 2 i shft, the non-integer part of _tmp1 = i^2 + 2 i shft
      const double p2 = __dmul_rn(di + di, shft);
      const uint64_t ii2 = (uint64_t)i * (uint64_t)i;
      // the phase coefficients fill the upper half of the sample's 32-byte
      // record (the resampled data fill the lower half)
      uint4 hi16;
      if (PM == PM_FIXED) {
        // spindown phase s1(ss) tmp1 = s1(ss_base) tmp1 + (ss - ss_base) (M5 tmp1)
        // as 64-bit fixed-point turns: the i^2 part exactly in integers from
        // the fixed-point coefficients, the 2 i shft part from its FP64 value
        const uint64_t A = sky.s1f * ii2 + turns_fixed(sky.s1_0 * p2);
        const uint64_t B = sky.m5f * ii2 + turns_fixed(sky.M5 * p2);
        hi16 = make_uint4((unsigned)A, (unsigned)(A >> 32), (unsigned)B, (unsigned)(B >> 32));
      } else {
        const double tmp1 = (double)ii2 + p2;
        if (PM == PM_FF) {
          const float hi = (float)tmp1;
          hi16 = make_uint4(__float_as_uint(hi), __float_as_uint((float)(tmp1 - (double)hi)), 0u, 0u);
        } else {
          const unsigned long long tb = (unsigned long long)__double_as_longlong(tmp1);
          hi16 = make_uint4((unsigned)tb, (unsigned)(tb >> 32), 0u, 0u);
        }
      }
      reinterpret_cast<uint4*>(ph0)[2 * o + 1] = hi16;
      // prelude phase het0 i + oms shft (jobcore.c:299) in fixed-point
      // turns: het0/2pi exactly in integers, oms shft/2pi from its FP64 value
      const uint64_t t = sky.h0f * (uint64_t)i + turns_fixed(sky.oms_t * shft);
      float sf, cf;
      sincospif((float)(int)(t >> 32) * 4.656612873077393e-10f, &sf, &cf);
      sp = (R)sf;
      cp = (R)cf;
    }
    const R x = (R)xDat[(size_t)d * N + i];
    const R xa = x * aa, xb = x * bb;
    // x a exp(-i phase)
    xin[((size_t)d * 2 + 0) * N + i] = mk(xa * cp, -xa * sp);
    xin[((size_t)d * 2 + 1) * N + i] = mk(xb * cp, -xb * sp);
  }
  // deterministic block reduction of a^2, b^2: xor tree of each warp in the
  // working precision, warps summed in FP64 in index order
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    a2r += __shfl_xor_sync(0xffffffffu, a2r, off);
    b2r += __shfl_xor_sync(0xffffffffu, b2r, off);
  }
  __shared__ double red[2][8];
  __shared__ bool last;
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = (double)a2r;
    red[1][threadIdx.x >> 5] = (double)b2r;
  }
  __syncthreads();
  double a2 = 0., b2 = 0.;
  if (threadIdx.x == 0)
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      a2 += red[0][k];
      b2 += red[1][k];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    part[((size_t)d * gridDim.x + blockIdx.x) * 2 + 0] = a2;
    part[((size_t)d * gridDim.x + blockIdx.x) * 2 + 1] = b2;
    __threadfence();
    const unsigned int done = atomicAdd(counter, 1u);
    last = done == gridDim.x * gridDim.y - 1;
  }
  __syncthreads();
  if (!last) return;
  // the last CTA to finish: aa = sum_n (sum_i a^2)/sig2_n in detector order
  // (jobcore.c:375-393), partials summed in a fixed order
  double aa = 0., bb = 0.;
  for (int dd = 0; dd < (int)gridDim.y; ++dd) {
    double sa = 0., sb = 0.;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) {
      sa += __ldcg(&part[((size_t)dd * gridDim.x + k) * 2 + 0]);
      sb += __ldcg(&part[((size_t)dd * gridDim.x + k) * 2 + 1]);
    }
    __syncthreads();
    block_sum2(sa, sb, red);
    aa += sa / dc[dd].sig2;
    bb += sb / dc[dd].sig2;
  }
  if (threadIdx.x == 0) {
    sums[0] = aa;
    sums[1] = bb;
    sums[2] = 1.0 / aa;
    sums[3] = 1.0 / bb;
    sums_r[0] = (R)(1.0 / aa);
    sums_r[1] = (R)(1.0 / bb);
    *counter = 0u;
  }
}

// ------------------------------------------------------------------
// FFT loaders / storers

template <typename R> struct PlainLoader {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_FFT_FWD_A;
  static constexpr bool kEarlyLoads = true;  // no prologue: loads before any barrier
  static constexpr bool kTwiddleTable = false;
  const T* in;   // [batch][2][ld]
  int len, ld;
  __device__ __forceinline__ void prologue(int, char*) const {}
  __device__ __forceinline__ void load2(int batch, int n, T& a, T& b, const char*) const {
    if (n < len) {
      a = in[((size_t)batch * 2 + 0) * ld + n];
      b = in[((size_t)batch * 2 + 1) * ld + n];
    } else {
      a = b = mk((R)0, (R)0);
    }
  }
};

// The interpolating inverse transform of jobcore.c:338-362 at half length.
// The reference keeps bins [0, nyqst) of the length-nfft spectrum X, moves
// [nyqst, nfft) up by Ninterp - nfft = nfft and inverse-transforms at length
// Ninterp = 2 nfft with scale 2/Ninterp.  With that remap the output is
//   y[2m]   = x[m]                                  (the input itself)
//   y[2m+1] = (1/nfft) sum_j X[j] s_j e^{i pi j/nfft} e^{2 pi i j m/nfft}
// with s_j = +1 below nyqst and -1 from it (the moved bins pick up
// e^{i pi (2m+1)} = -1), i.e. an inverse FFT of length nfft of the
// phase-shifted spectrum: half the transform length, and no transform of the
// zero gap.  This loader feeds that transform; InterpStore interleaves.
template <typename R> struct HalfShiftLoader {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_FFT_INV_A;
  static constexpr bool kEarlyLoads = true;  // no prologue: loads before any barrier
  static constexpr bool kTwiddleTable = false;
  const T* spec;    // [batch][2][nfft]
  const T* twlo;    // e^{+2 pi i m/Ninterp}, m < 1024
  const T* twhi;    // e^{+2 pi i 1024 m/Ninterp}
  int nfft, nyqst;
  __device__ __forceinline__ void prologue(int, char*) const {}
  __device__ __forceinline__ void load2(int batch, int j, T& a, T& b, const char*) const {
    const T w0 = cmul(__ldg(&twlo[j & 1023]), __ldg(&twhi[j >> 10]));
    const T w = j < nyqst ? w0 : mk(-w0.x, -w0.y);
    a = cmul(spec[((size_t)batch * 2 + 0) * nfft + j], w);
    b = cmul(spec[((size_t)batch * 2 + 1) * nfft + j], w);
  }
};

struct SpinCta {
  double het1, s1;
  uint64_t H;
  unsigned ssr;  // ss - ss_base (>= 0), fixed-point form
  float s1h, s1l, h1h, h1l;
};

// Most spindowns in one launch of the spindown passes (the buffers are sized
// for at most 128).
constexpr int kSpinBatchMax = 128;

// het1 = fmod(ss M4, M0), wrapped into [0, M0) (jobcore.c:466-467), as
// 64-bit fixed-point turns: round-to-nearest-even of het1 2^64 / (2 pi),
// saturated as __double2ull_rn does.  fmod is exact and the two products
// are single roundings, so the host and the device give the same bits.
inline uint64_t het1_turns_fixed(int ss, double M4, double M0) {
  double het1 = fmod(ss * M4, M0);
  if (het1 < 0) het1 += M0;
  const double x = het1 * kTurnsPerRad64;
  if (!(x > 0.)) return 0;
  if (x >= 18446744073709551616.0) return ~0ull;
  // round half to even without depending on the host's rounding mode: below
  // 2^53, x - floor(x) is exact; from 2^53 on, x is an integer
  uint64_t r = (uint64_t)x;
  if (x < 9007199254740992.0) {
    const double fr = x - (double)r;
    if (fr > 0.5 || (fr == 0.5 && (r & 1))) ++r;
  }
  return r;
}

// Per-launch spindown constants passed by value with the loader.  The
// fixed-point form takes the het1 term of each batch item from the host
// (H[batch]), so that no CTA of pass A waits on a chain of FP64 operations
// before its first phase; the other forms form theirs per CTA (prologue).
template <typename R, int PM> struct SpinHet {
  static constexpr bool kHost = false;
};
template <> struct SpinHet<float, PM_FIXED> {
  static constexpr bool kHost = true;
  unsigned long long H[kSpinBatchMax];
};

// (a * b) mod 2^64 for a 64-bit a and a 32-bit b
__device__ __forceinline__ uint64_t mul64x32(uint64_t a, unsigned b) {
  return (uint64_t)(unsigned)a * b + ((uint64_t)((unsigned)(a >> 32) * b) << 32);
}

// Phase-modulated detector sum of the spindown loop (jobcore.c:455-623):
//   x_{a,b}[n] = sum_d xm_{a,b,d}[n] exp(-i (het1 n + s1 tmp1_d[n]))  (n < N)
template <typename R, int PM> struct SpinLoader {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_SPIN_A;
  // the fixed-point form needs no shared-memory constants (no barrier after
  // the prologue)
  static constexpr bool kPrologue = !SpinHet<R, PM>::kHost;
  // generic pass A: first loads before any barrier (no prologue to wait for)
  static constexpr bool kEarlyLoads = !kPrologue;
  // generic pass A: inter-pass twiddles from Buffers::tw_pass (FP32 forms)
  static constexpr bool kTwiddleTable = sizeof(R) == 4;
  const T* xm;       // [nifo][2][N]
  const void* ph0;   // FP64 form: tmp1 [nifo][N]; FP32 forms: unused
  int N, nifo, ss0, ss_base, s0_flag;
  double M0, M4, M5, s1_0;
  SpinHet<R, PM> het;

  // Spindown constants of batch item `batch`: the fixed-point form's from
  // the launch parameters (registers), the other forms' from the prologue's
  // shared-memory copy.
  __device__ __forceinline__ SpinCta consts(int batch, const char* sm) const {
    SpinCta k;
    if constexpr (SpinHet<R, PM>::kHost) {
      k.H = het.H[batch];
      k.ssr = s0_flag ? 0u : (unsigned)(ss0 + batch - ss_base);
    } else {
      k = *reinterpret_cast<const SpinCta*>(sm);
    }
    return k;
  }

  __device__ __forceinline__ void prologue(int batch, char* sm) const {
    if (kPrologue && threadIdx.x == 0) {
      SpinCta* p = reinterpret_cast<SpinCta*>(sm);
      const int ss = ss0 + batch;
      double het1 = fmod(ss * M4, M0);
      if (het1 < 0) het1 += M0;
      const double s1 = s0_flag ? 0. : ss * M5 + s1_0;
      p->het1 = het1;
      p->s1 = s1;
      p->H = (uint64_t)__double2ull_rn(het1 * kTurnsPerRad64);
      p->ssr = s0_flag ? 0u : (unsigned)(ss - ss_base);
      p->s1h = (float)s1;
      p->s1l = (float)(s1 - (double)p->s1h);
      p->h1h = (float)het1;
      p->h1l = (float)(het1 - (double)p->h1h);
    }
  }

  __device__ __forceinline__ void load2(int batch, int n, T& va, T& vb, const char* sm) const {
    va = vb = mk((R)0, (R)0);
    if (n >= N) return;
    const SpinCta pk = consts(batch, sm);
    const SpinCta* p = &pk;
    R accx = 0, accy = 0, bccx = 0, bccy = 0;
    double base = 0.;
    // fixed-point form: the high word of H n (the phase is formed from the
    // high words of its terms, as in mod1h)
    unsigned hn_hi = 0;
    if (PM == PM_FIXED) hn_hi = __umulhi((unsigned)p->H, (unsigned)n) + (unsigned)(p->H >> 32) * (unsigned)n;
    else if (PM == PM_F64) base = p->het1 * (double)n;
    for (int d = 0; d < nifo; ++d) {
      const size_t o = (size_t)d * N + n;
      R sn, cs;
      T xa, xb;
      uint4 hi16 = make_uint4(0u, 0u, 0u, 0u);
      if (sizeof(R) == 8) {
        xa = xm[((size_t)d * 2 + 0) * N + n];
        xb = xm[((size_t)d * 2 + 1) * N + n];
      } else {
        // one 32-byte record per detector and sample: xa, xb | phase terms
        const float4 lo16 = __ldg(reinterpret_cast<const float4*>(xm) + 2 * o);
        hi16 = __ldg(reinterpret_cast<const uint4*>(xm) + 2 * o + 1);
        xa = mk((R)lo16.x, (R)lo16.y);
        xb = mk((R)lo16.z, (R)lo16.w);
      }
      if (sizeof(R) == 8) {
        const double t1 = reinterpret_cast<const double*>(ph0)[o];
        // het1*i + s1*_tmp1 with the reference's rounding (jobcore.c:606)
        const double ph = __dadd_rn(__dmul_rn(p->het1, (double)n), __dmul_rn(p->s1, t1));
        double sd, cd;
        sincos(ph, &sd, &cd);
        sn = (R)sd;
        cs = (R)cd;
      } else if (PM == PM_F64) {
        const double t1 = __longlong_as_double((long long)(((unsigned long long)hi16.y << 32) | hi16.x));
        const double ph = fma(p->s1, t1, base);
        const double kk = rint(ph * kInvTwoPi);
        double r = fma(-kk, kTwoPiHi, ph);
        r = fma(-kk, kTwoPiLo, r);
        float sf, cf;
        sincosf((float)r, &sf, &cf);
        sn = (R)sf;
        cs = (R)cf;
      } else if (PM == PM_FIXED) {
        // top 32 bits of A + B ssr + H n (high words only, as mod1h) as a
        // signed fraction of half a turn: angle = pi * x, x in [-1, 1); the
        // hardware sine and cosine (absolute error <= 3.6e-7 there)
        const unsigned th = hi16.y + (__umulhi(hi16.z, p->ssr) + hi16.w * p->ssr) + hn_hi;
        float sf, cf;
        __sincosf((float)(int)th * 1.4629180792671596e-9f, &sf, &cf);  // pi 2^-31
        sn = (R)sf;
        cs = (R)cf;
      } else {
        // compensated float-float phase
        const float2 tt = make_float2(__uint_as_float(hi16.x), __uint_as_float(hi16.y));
        float p1 = p->s1h * tt.x;
        float e1 = fmaf(p->s1h, tt.x, -p1);
        e1 = fmaf(p->s1h, tt.y, e1);
        e1 = fmaf(p->s1l, tt.x, e1);
        const float nf = (float)n;
        float p2 = p->h1h * nf;
        float e2 = fmaf(p->h1h, nf, -p2);
        e2 = fmaf(p->h1l, nf, e2);
        const float s = p1 + p2;
        const float bb = s - p1;
        const float err = (p1 - (s - bb)) + (p2 - bb);
        const float e = err + e1 + e2;
        const float kk = rintf(s * kInvTwoPiF);
        float r = fmaf(-kk, kTwoPiF_A, s);
        r = fmaf(-kk, kTwoPiF_B, r);
        r = fmaf(-kk, kTwoPiF_C, r);
        r += e;
        float sf, cf;
        sincosf(r, &sf, &cf);
        sn = (R)sf;
        cs = (R)cf;
      }
      // x * (cos - i sin)
      accx += xa.x * cs + xa.y * sn;
      accy += xa.y * cs - xa.x * sn;
      bccx += xb.x * cs + xb.y * sn;
      bccy += xb.y * cs - xb.x * sn;
    }
    va = mk(accx, accy);
    vb = mk(bccx, bccy);
  }

  // The fixed-point form's term (FP32, n < N) with the high word of H n
  // given by the caller (hn_hi, carried from position to position): the
  // phase's high word is the sum of its three terms' high words.  The carries
  // of the low words that this drops lower it by at most 2 units of 2^-32
  // turns (3e-9 rad), far below the FP32 rounding of the angle that follows
  // (up to 2^-25 of a half turn, 9e-8 rad).  The angle, in [-pi, pi), goes
  // to the hardware sine and cosine (__sincosf: absolute error at most
  // 2^-21.41 = 3.6e-7 in that range), which the radix-16 pass A needs once
  // per detector and sample.  pa, pb as in mod1.
  __device__ __forceinline__ void mod1h(int d, int n, unsigned hn_hi, unsigned ssr, T& pa, T& pb) const {
    static_assert(sizeof(R) == 4 && PM == PM_FIXED, "fixed-point FP32 form only");
    const size_t o = (size_t)d * N + n;
    const float4 lo16 = __ldg(reinterpret_cast<const float4*>(xm) + 2 * o);
    const uint4 hi16 = __ldg(reinterpret_cast<const uint4*>(xm) + 2 * o + 1);
    const unsigned th = hi16.y + (__umulhi(hi16.z, ssr) + hi16.w * ssr) + hn_hi;
    float sn, cs;
    __sincosf((float)(int)th * 1.4629180792671596e-9f, &sn, &cs);  // pi 2^-31
    pa = mk(lo16.x * cs + lo16.y * sn, lo16.y * cs - lo16.x * sn);
    pb = mk(lo16.z * cs + lo16.w * sn, lo16.w * cs - lo16.z * sn);
  }

  // One detector's term of load2 (FP32 forms, n < N): xm_{a,b,d}[n] times
  // exp(-i phase_d(n)), with the phase evaluated as load2 does; pa and pb
  // follow the record's order (b first for the detector whose record
  // halves the prelude swapped, Engine::swapped_det).
  __device__ __forceinline__ void mod1(int d, int n, T& pa, T& pb, const SpinCta& pk) const {
    static_assert(sizeof(R) == 4, "FP32 forms only");
    const SpinCta* p = &pk;
    const size_t o = (size_t)d * N + n;
    const float4 lo16 = __ldg(reinterpret_cast<const float4*>(xm) + 2 * o);
    const uint4 hi16 = __ldg(reinterpret_cast<const uint4*>(xm) + 2 * o + 1);
    float sn, cs;
    if (PM == PM_FIXED) {
      const uint64_t A = ((uint64_t)hi16.y << 32) | hi16.x;
      const uint64_t B = ((uint64_t)hi16.w << 32) | hi16.z;
      const uint64_t t = A + mul64x32(B, p->ssr) + mul64x32(p->H, (unsigned)n);
      const float x = (float)(int)(t >> 32) * 4.656612873077393e-10f;  // 2^-31
      sincospif(x, &sn, &cs);
    } else if (PM == PM_F64) {
      const double t1 = __longlong_as_double((long long)(((unsigned long long)hi16.y << 32) | hi16.x));
      const double ph = fma(p->s1, t1, p->het1 * (double)n);
      const double kk = rint(ph * kInvTwoPi);
      double r = fma(-kk, kTwoPiHi, ph);
      r = fma(-kk, kTwoPiLo, r);
      sincosf((float)r, &sn, &cs);
    } else {
      const float2 tt = make_float2(__uint_as_float(hi16.x), __uint_as_float(hi16.y));
      float p1 = p->s1h * tt.x;
      float e1 = fmaf(p->s1h, tt.x, -p1);
      e1 = fmaf(p->s1h, tt.y, e1);
      e1 = fmaf(p->s1l, tt.x, e1);
      const float nf = (float)n;
      float p2 = p->h1h * nf;
      float e2 = fmaf(p->h1h, nf, -p2);
      e2 = fmaf(p->h1l, nf, e2);
      const float s = p1 + p2;
      const float bb = s - p1;
      const float err = (p1 - (s - bb)) + (p2 - bb);
      const float e = err + e1 + e2;
      const float kk = rintf(s * kInvTwoPiF);
      float r = fmaf(-kk, kTwoPiF_A, s);
      r = fmaf(-kk, kTwoPiF_B, r);
      r = fmaf(-kk, kTwoPiF_C, r);
      r += e;
      sincosf(r, &sn, &cs);
    }
    pa = mk(lo16.x * cs + lo16.y * sn, lo16.y * cs - lo16.x * sn);
    pb = mk(lo16.z * cs + lo16.w * sn, lo16.w * cs - lo16.z * sn);
  }
};

// Spindown pass A for two detectors and L1 = 256 = 16 x 16 (the FP32 forms):
// the column FFTs of k_pass_a as two radix-16 stages with one barrier
// between them, each thread holding 16 values of one array.
//   stage 1: warp w = b (n1 mod 16), lane = 2 col + arr.  At the 16 positions
//     n1 = 16 a + b of column col the thread evaluates detector arr's term
//     (mod1h in the fixed-point form, mod1 in the others) and swaps with its
//     partner lane (lane ^ 1) the term of the array the partner keeps, so
//     that it holds x_arr = term_0 + term_1: one sincos per detector and
//     position, as the paired loader.  Detector 1's records hold {xb, xa}
//     (k_splint swap_det), so the first term is always the one kept.
//     16-point DFT over a, store Z[c][b].
//   stage 2: warp = column, lane = 2 c + arr.  Twiddle W_256^{b c} (shared
//     table at c * 17 + b, stored after stage 1), 16-point DFT over b gives
//     Y[k1 = c + 16 d]; inter-pass twiddle W_L^{n2 k1} from a table of all
//     of them (Buffers::tw_pass, L entries); stored like k_pass_a
//     (the a|b values of one (n2, k1) adjacent, 256 contiguous bytes per warp).
// Shared tile: Z[c][b][lane] at c * 514 + b * 32 + lane (float2); the pad of
// 2 per c makes the stage-2 reads conflict-free (half-warp slots 2c + arr).
template <int SIGN, int LOGL, int PM>
__global__ void __launch_bounds__(512, 2)
    k_pass_a16(const __grid_constant__ SpinLoader<float, PM> ld, const float2* __restrict__ tw1,
               const float2* __restrict__ tw16, float2* __restrict__ ybuf) {
  constexpr int LOGL1 = 8, LOGL2 = LOGL - LOGL1, ZC = 16 * 32 + 2;
  CtaTrace trace_(KK_SPIN_A);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* z = reinterpret_cast<float2*>(smem_raw);
  // twiddles of the stage-1 outputs, applied in stage 2: W_256^{b c} at
  // c * 17 + b (the pitch of 17 makes the stage-2 reads conflict-free)
  float2* tws = z + 16 * ZC;
  char* lsm = reinterpret_cast<char*>(tws + 272);
  const int batch = blockIdx.y;
  const int c0 = blockIdx.x << 4;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  // loaded now, stored after stage 1: no barrier before the first record
  // loads (except for the forms whose prologue fills shared memory)
  float2 twv = make_float2(0.f, 0.f);
  if (threadIdx.x < 272) {
    const int tc = threadIdx.x / 17, tb = threadIdx.x - 17 * tc;
    twv = tw1[tb * tc];
  }
  if constexpr (SpinLoader<float, PM>::kPrologue) {
    ld.prologue(batch, lsm);
    __syncthreads();
  }
  const SpinCta pk = ld.consts(batch, lsm);
  float2 v[16];
  {
    const int arr = lane & 1;
    const int n2 = c0 + (lane >> 1);
    // fixed-point form: H n carried from position to position (exact, mod 2^64)
    uint64_t hn = mul64x32(pk.H, (unsigned)((w << LOGL2) + n2));
    const uint64_t hstep = pk.H << (4 + LOGL2);
#pragma unroll
    for (int a = 0; a < 16; ++a) {
      const int n = ((16 * a + w) << LOGL2) + n2;
      // detector 1's record holds {xb, xa} (k_splint swap_det): the first
      // term is the array this lane keeps, the second its partner's
      float2 mine = make_float2(0.f, 0.f), send = mine;
      if constexpr (PM == PM_FIXED) {
        if (n < ld.N) ld.mod1h(arr, n, (unsigned)(hn >> 32), pk.ssr, mine, send);
        hn += hstep;
      } else {
        if (n < ld.N) ld.mod1(arr, n, mine, send, pk);
      }
      const float rx = __shfl_xor_sync(0xffffffffu, send.x, 1);
      const float ry = __shfl_xor_sync(0xffffffffu, send.y, 1);
      v[a] = make_float2(mine.x + rx, mine.y + ry);
    }
    dft16<SIGN>(v);
#pragma unroll
    for (int c = 0; c < 16; ++c) z[c * ZC + w * 32 + lane] = v[c];
  }
  if (threadIdx.x < 272) tws[threadIdx.x] = twv;
  __syncthreads();
  {
    const int arr = lane & 1, c = lane >> 1;
    const int n2 = c0 + w;
    const float2* t2 = tws + c * 17;
    v[0] = z[c * ZC + 2 * w + arr];
#pragma unroll
    for (int b = 1; b < 16; ++b) v[b] = cmul(z[c * ZC + b * 32 + 2 * w + arr], t2[b]);
    dft16<SIGN>(v);
    float2* yb = ybuf + ((size_t)batch << (LOGL + 1)) + ((size_t)n2 << (LOGL1 + 1)) + arr;
    // inter-pass twiddle W_L^{n2 k1}, k1 = c + 16 d, from the table at
    // [n2][k1] (one load per output instead of two table loads, their
    // product and the exponent arithmetic)
    const float2* tw = tw16 + ((size_t)n2 << 8) + c;
#pragma unroll
    for (int d = 0; d < 16; ++d) yb[2 * (c + 16 * d)] = cmul(v[d], __ldg(&tw[16 * d]));
  }
}

template <class L> struct IsSpinF32 {
  static constexpr bool value = false;
  static constexpr int pm = 0;
};
template <int PM> struct IsSpinF32<SpinLoader<float, PM>> {
  static constexpr bool value = true;
  static constexpr int pm = PM;
};

// Complex output with a scale factor (resampling FFTs).
template <typename R> struct CStore {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_FFT_FWD_B;
  T* out;   // [batch][2][ldo]
  int ldo;
  R scale;
  struct Ctx {};
  __device__ __forceinline__ Ctx begin() const { return Ctx{}; }
  __device__ __forceinline__ void put(const Ctx&, int batch, int k1, int k2, T a, T b, int logL1) const {
    const size_t k = (size_t)k1 + ((size_t)k2 << logL1);
    out[((size_t)batch * 2 + 0) * ldo + k] = mk(a.x * scale, a.y * scale);
    out[((size_t)batch * 2 + 1) * ldo + k] = mk(b.x * scale, b.y * scale);
  }
};

// F-statistic epilogue: F[k] = |Xa[k]|^2 / aa + |Xb[k]|^2 / bb, k in [nmin, nmax)
template <typename R> struct FstatStore {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_SPIN_B;
  R* F;             // [batch][bins]
  const R* inv;     // 1/aa, 1/bb in the working precision
  int nmin, nmax, bins;
  // 1/aa and 1/bb, loaded when the CTA starts (beside the first loads of
  // the intermediate) rather than where the epilogue needs them
  struct Ctx {
    R ia, ib;
  };
  __device__ __forceinline__ Ctx begin() const { return Ctx{__ldg(&inv[0]), __ldg(&inv[1])}; }
  __device__ __forceinline__ void put(const Ctx& c, int batch, int k1, int k2, T a, T b, int logL1) const {
    const int k = k1 + (k2 << logL1);
    if (k >= nmin && k < nmax)
      F[(size_t)batch * bins + (k - nmin)] = (a.x * a.x + a.y * a.y) * c.ia + (b.x * b.x + b.y * b.y) * c.ib;
  }
};

// Output of the half-length interpolating transform: y[2m] = x[m] (zero
// past the N input samples), y[2m+1] = transform[m] / nfft, written as one
// 16-byte pair per (array, m) into yint [batch][2][Ninterp].
template <typename R> struct InterpStore {
  typedef typename CT<R>::T T;
  static constexpr int kTraceKind = KK_FFT_INV_B;
  T* yint;
  const T* xin;     // [batch][2][N]
  int N, Ninterp;
  R scale;          // 1/nfft
  struct Ctx {};
  __device__ __forceinline__ Ctx begin() const { return Ctx{}; }
  __device__ __forceinline__ void put(const Ctx&, int batch, int k1, int k2, T a, T b, int logL1) const {
    const int m = k1 + (k2 << logL1);
    const size_t qa = (size_t)batch * 2, qb = qa + 1;
    const T xa = m < N ? xin[qa * N + m] : mk((R)0, (R)0);
    const T xb = m < N ? xin[qb * N + m] : mk((R)0, (R)0);
    Pair<T>::st(yint + qa * Ninterp + 2 * (size_t)m, xa, mk(a.x * scale, a.y * scale));
    Pair<T>::st(yint + qb * Ninterp + 2 * (size_t)m, xb, mk(b.x * scale, b.y * scale));
  }
};

// ------------------------------------------------------------------
// Compensated two-float (float-float) arithmetic for the spline recurrences
// of the FP32 forms: a value is hi + lo with |lo| <= ulp(hi)/2 (about 48
// significant bits).  Products use fmaf for their exact error terms; the
// explicit __fmul_rn keeps the compiler from fusing a rounded product into
// the following sum.
struct FF {
  float hi, lo;
};

__device__ __forceinline__ FF ff_split(double x) {
  const float h = (float)x;
  return FF{h, (float)(x - (double)h)};
}

// a*x + t, a a float-float constant, t a float (Dekker/Knuth error-free
// transformations: the product error by fma, the sum error by TwoSum)
__device__ __forceinline__ FF ff_axpt(FF a, FF x, float t) {
  const float p = __fmul_rn(a.hi, x.hi);
  float e = __fmaf_rn(a.hi, x.hi, -p);
  e = __fmaf_rn(a.hi, x.lo, e);
  e = __fmaf_rn(a.lo, x.hi, e);
  const float s = __fadd_rn(p, t);
  const float bb = __fsub_rn(s, p);
  const float r = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(t, bb));
  const float c = __fadd_rn(r, e);
  const float hi = __fadd_rn(s, c);
  return FF{hi, __fsub_rn(c, __fsub_rn(hi, s))};
}

// a*x + y, a a float-float constant, x and y float-float
__device__ __forceinline__ FF ff_axpy(FF a, FF x, FF y) {
  const float p = __fmul_rn(a.hi, x.hi);
  float e = __fmaf_rn(a.hi, x.hi, -p);
  e = __fmaf_rn(a.hi, x.lo, e);
  e = __fmaf_rn(a.lo, x.hi, e);
  const float s = __fadd_rn(p, y.hi);
  const float bb = __fsub_rn(s, p);
  float r = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(y.hi, bb));
  r = __fadd_rn(r, __fadd_rn(e, y.lo));
  const float hi = __fadd_rn(s, r);
  return FF{hi, __fsub_rn(r, __fsub_rn(hi, s))};
}

// ------------------------------------------------------------------
// spline (auxi.c:56-81): chunked recurrences, FP64 in the FP64 form and
// compensated two-float in the FP32 forms (the FP64 pipe of a GB300 runs at
// 1/64 of the FP32 rate, and these sweeps are its largest user in the
// prelude).  The forward sweep
// u_i = (-u_{i-1}/2 + 3 d_i) invp_i has |dU_i/dU_{i-1}| -> 2 - sqrt(3) = 0.268
// and the back substitution y2_k = p_k y2_{k+1} + u_k likewise, so a chunk
// can start kWarm steps early from zero: the start error shrinks by
// 0.268^kWarm < 1e-18.  Chunks whose warm start reaches the array ends start
// from the exact boundary values u_0 = 0, y2_{n-1} = 0.
// Chunking per form: the warm start must bring the start error below the
// precision the result is stored in (y2 is stored in the working precision):
// 0.268^16 = 7e-10 is far below FP32 rounding, 0.268^32 = 5e-19 below FP64's.
// Shorter chunks in the FP32 forms also give twice the independent
// recurrences, which these latency-bound sweeps need.
template <typename R> struct SplineCfg;
template <> struct SplineCfg<float> {
  static constexpr int chunk = 32, warm = 16, log2chunk = 5;
};
template <> struct SplineCfg<double> {
  static constexpr int chunk = 64, warm = 32, log2chunk = 6;
};
constexpr int kSplineThreads = 256;                        // threads for staging loads/stores
constexpr int kSplineSeg = 4096;                           // elements per CTA

// Asynchronous global-to-shared copies (cp.async): every copy of a staging
// loop is in flight at once, with no registers held; an invalid element is
// zero-filled (source size 0, the source address is not read).
template <int BYTES>
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, bool valid) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if (BYTES == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(gmem), "r"(valid ? 16 : 0)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(s), "l"(gmem), "n"(BYTES),
                 "r"(valid ? BYTES : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared-memory slot of staged element k: one padding element per chunk, so
// that the recurrence threads (chunk starts one chunk apart) hit different
// banks.
template <typename R>
__device__ __forceinline__ int spad(int k) { return k + (k >> SplineCfg<R>::log2chunk); }
template <typename R>
__host__ __device__ constexpr int spad_len(int n) { return n + (n >> SplineCfg<R>::log2chunk) + 1; }

// Forward sweep.  A CTA owns one segment of kSplineSeg elements of one
// array; it stages y[seg - warm - 1, seg_end + 1) in shared memory with
// coalesced loads (as FP64), every thread runs its chunk's recurrence from
// shared memory, and the u values leave through shared memory again so the
// global stores are coalesced.
template <typename R>
__global__ void __launch_bounds__(kSplineThreads)
    k_spline_fwd(const typename CT<R>::T* __restrict__ y, int ldy, double2* __restrict__ u, int n, int nseg,
                 const double* __restrict__ invp) {
  typedef typename CT<R>::T T;
  CtaTrace trace_(KK_SPLINE_FWD);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  double2* us = reinterpret_cast<double2*>(sm_raw);                 // spad_len<R>(kSplineSeg)
  T* ys = reinterpret_cast<T*>(us + spad_len<R>(kSplineSeg));          // spad_len<R>(kSplineSeg + SplineCfg<R>::warm + 2)
  const int q = blockIdx.x / nseg, sg = blockIdx.x - q * nseg;
  const T* yq = y + (size_t)q * ldy;
  double2* uq = u + (size_t)q * n;
  const int seg0 = sg * kSplineSeg;
  const int y0 = seg0 - SplineCfg<R>::warm - 1;                       // first staged index
  const int ny = kSplineSeg + SplineCfg<R>::warm + 2;
  // the coefficients of the first 64 steps of the array, in shared memory
  // (the first chunks' recurrences read one per step): FP64 pivots for the
  // FP64 form, their float-float splits (formed here in parallel, keeping
  // FP64 work out of the sequential recurrence) for the FP32 forms
  __shared__ double tab[64];
  __shared__ float tal_h[64], tal_l[64], tbe[64];
  if (threadIdx.x < 64) {
    const double v = invp[threadIdx.x];
    tab[threadIdx.x] = v;
    const FF a = ff_split(-.5 * v);
    tal_h[threadIdx.x] = a.hi;
    tal_l[threadIdx.x] = a.lo;
    tbe[threadIdx.x] = (float)(3. * v);
  }
  for (int k = threadIdx.x; k < ny; k += kSplineThreads) {
    const int i = y0 + k;
    const bool ok = i >= 0 && i < n;
    cp_async<(int)sizeof(T)>(&ys[spad<R>(k)], ok ? (const void*)(yq + i) : (const void*)yq, ok);
  }
  cp_async_wait_all();
  __syncthreads();
  if (threadIdx.x < (kSplineSeg / SplineCfg<R>::chunk)) {
    const int lo = seg0 + threadIdx.x * SplineCfg<R>::chunk;
    const int hi = min(lo + SplineCfg<R>::chunk, n - 1);
    // u_i = (-u_{i-1}/2 + 3 d_i) invp_i = al_i u_{i-1} + be_i d_i; the
    // second difference d_i of the working-precision data is formed in that
    // precision (its rounding is below the data's own)
    int i = max(1, lo - SplineCfg<R>::warm);
    T p = ys[spad<R>(i - 1 - y0)], cc = ys[spad<R>(i - y0)];
    if (sizeof(R) == 8) {
      double ux = 0., uy = 0.;
      for (; i < hi; ++i) {
        const T nn = ys[spad<R>(i + 1 - y0)];
        const R dx = p.x - (R)2 * cc.x + nn.x, dy = p.y - (R)2 * cc.y + nn.y;
        const int ti = i < 64 ? i : 63;
        const double al = -.5 * tab[ti], be = 3. * tab[ti];
        ux = fma(al, ux, be * (double)dx);
        uy = fma(al, uy, be * (double)dy);
        if (i >= lo) us[spad<R>(i - seg0)] = make_double2(ux, uy);
        p = cc;
        cc = nn;
      }
    } else {
      FF ux{0.f, 0.f}, uy{0.f, 0.f};
      float4* us4 = reinterpret_cast<float4*>(us);
      auto step = [&](FF al, float be) {
        const T nn = ys[spad<R>(i + 1 - y0)];
        const float dx = (float)(p.x - (R)2 * cc.x + nn.x), dy = (float)(p.y - (R)2 * cc.y + nn.y);
        ux = ff_axpt(al, ux, __fmul_rn(be, dx));
        uy = ff_axpt(al, uy, __fmul_rn(be, dy));
        if (i >= lo) us4[spad<R>(i - seg0)] = make_float4(ux.hi, ux.lo, uy.hi, uy.lo);
        p = cc;
        cc = nn;
      };
      // the first 63 steps of the array have their own coefficients; from
      // i = 63 on they are constant (two loops keep the FP64 table reads out
      // of the main one)
      for (; i < hi && i < 63; ++i) step(FF{tal_h[i], tal_l[i]}, tbe[i]);
      const FF al{tal_h[63], tal_l[63]};
      const float be = tbe[63];
      for (; i < hi; ++i) step(al, be);
    }
    if (lo == 0) us[spad<R>(0)] = make_double2(0., 0.);
  }
  __syncthreads();
  const int cnt = min(kSplineSeg, n - 1 - seg0);
  for (int k = threadIdx.x; k < cnt; k += kSplineThreads) uq[seg0 + k] = us[spad<R>(k)];
}

// Back substitution, same staging: u[seg0, seg_end + warm) in shared memory,
// y2 of the segment written back through shared memory.
template <typename R>
__global__ void __launch_bounds__(kSplineThreads)
    k_spline_bwd(const double2* __restrict__ u, typename CT<R>::T* __restrict__ y2, int n, int nseg,
                 const double* __restrict__ ptab) {
  typedef typename CT<R>::T T;
  CtaTrace trace_(KK_SPLINE_BWD);
  extern __shared__ __align__(16) unsigned char sm_raw[];
  double2* us = reinterpret_cast<double2*>(sm_raw);                     // spad_len<R>(kSplineSeg + SplineCfg<R>::warm)
  T* ys = reinterpret_cast<T*>(us + spad_len<R>(kSplineSeg + SplineCfg<R>::warm));  // spad_len<R>(kSplineSeg)
  const int q = blockIdx.x / nseg, sg = blockIdx.x - q * nseg;
  const double2* uq = u + (size_t)q * n;
  T* yq = y2 + (size_t)q * n;
  const int seg0 = sg * kSplineSeg;
  const int nu = min(kSplineSeg + SplineCfg<R>::warm, n - 1 - seg0);  // u defined on [0, n-2]
  __shared__ double tab[64];
  __shared__ float tp_h[64], tp_l[64];
  if (threadIdx.x < 64) {
    const double v = ptab[threadIdx.x];
    tab[threadIdx.x] = v;
    const FF a = ff_split(v);
    tp_h[threadIdx.x] = a.hi;
    tp_l[threadIdx.x] = a.lo;
  }
  for (int k = threadIdx.x; k < nu; k += kSplineThreads) cp_async<16>(&us[spad<R>(k)], uq + seg0 + k, true);
  cp_async_wait_all();
  __syncthreads();
  const int lo = seg0 + threadIdx.x * SplineCfg<R>::chunk;
  const int hi = min(lo + SplineCfg<R>::chunk, n);
  if (threadIdx.x < (kSplineSeg / SplineCfg<R>::chunk) && lo < n) {
    const int kst = min(n - 2, hi - 1 + SplineCfg<R>::warm);
    if (sizeof(R) == 8) {
      double vx = 0., vy = 0.;
      for (int k = kst; k >= lo; --k) {
        const double p = tab[k < 64 ? k : 63];
        const double2 uk = us[spad<R>(k - seg0)];
        vx = p * vx + uk.x;
        vy = p * vy + uk.y;
        if (k < hi) ys[spad<R>(k - seg0)] = mk((R)vx, (R)vy);
      }
    } else {
      const float4* us4 = reinterpret_cast<const float4*>(us);
      FF vx{0.f, 0.f}, vy{0.f, 0.f};
      int k = kst;
      auto step = [&](FF pc) {
        const float4 uk = us4[spad<R>(k - seg0)];
        vx = ff_axpy(pc, vx, FF{uk.x, uk.y});
        vy = ff_axpy(pc, vy, FF{uk.z, uk.w});
        if (k < hi) ys[spad<R>(k - seg0)] = mk((R)vx.hi, (R)vy.hi);
      };
      // constant coefficient down to k = 64, then the table
      const FF pc63{tp_h[63], tp_l[63]};
      for (; k >= lo && k >= 64; --k) step(pc63);
      for (; k >= lo; --k) step(FF{tp_h[k], tp_l[k]});
    }
    if (hi == n) ys[spad<R>(n - 1 - seg0)] = mk((R)0, (R)0);
  }
  __syncthreads();
  const int cnt = min(kSplineSeg, n - seg0);
  for (int k = threadIdx.x; k < cnt; k += kSplineThreads) yq[seg0 + k] = ys[spad<R>(k)];
}

// splint at x = interpftpad (i - shftf_i) (auxi.c:83-122), then / sig2
template <typename R>
__global__ void __launch_bounds__(256)
    k_splint(const typename CT<R>::T* __restrict__ y, int ldy, const typename CT<R>::T* __restrict__ y2,
             const double* __restrict__ shftf, const DetConst* __restrict__ dc, int N,
             typename CT<R>::T* __restrict__ xm, int swap_det) {
  typedef typename CT<R>::T T;
  CtaTrace trace_(KK_SPLINT);
  const int d = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int n = 2 * N;
  const double x = __dmul_rn(2.0, __dsub_rn((double)i, shftf[(size_t)d * N + i]));
  const R is2 = sizeof(R) == 4 ? (R)dc[d].inv_sig2_f : (R)dc[d].inv_sig2;
  T out[2];
  for (int arr = 0; arr < 2; ++arr) {
    const size_t q = (size_t)d * 2 + arr;
    T v = mk((R)0, (R)0);
    if (!(x < 0 || x > n - 1)) {
      const int klo = (int)floor(x);
      const int khi = klo + 1;
      const int kh = khi < n ? khi : n - 1;
      const R a = (R)(khi - x), b = (R)(x - klo);
      const T ylo = y[q * ldy + klo], yhi = y[q * ldy + kh];
      const T zlo = y2[q * n + klo], zhi = y2[q * n + kh];
      const R ca = (a * a * a - a), cb = (b * b * b - b);
      v.x = a * ylo.x + b * yhi.x + (ca * zlo.x + cb * zhi.x) / (R)6;
      v.y = a * ylo.y + b * yhi.y + (ca * zlo.y + cb * zhi.y) / (R)6;
    }
    out[arr] = mk(v.x * is2, v.y * is2);
  }
  if (sizeof(R) == 8) {
    xm[((size_t)d * 2 + 0) * N + i] = out[0];
    xm[((size_t)d * 2 + 1) * N + i] = out[1];
  } else {
    // lower half of the sample's 32-byte record: {xa, xb}, or {xb, xa} for
    // detector swap_det (the radix-16 spindown pass A then needs no
    // lane-dependent selects, SpinLoader::mod1r)
    const int f = d == swap_det ? 1 : 0;
    reinterpret_cast<float4*>(xm)[2 * ((size_t)d * N + i)] =
        make_float4((float)out[f].x, (float)out[f].y, (float)out[1 - f].x, (float)out[1 - f].y);
  }
}

// ------------------------------------------------------------------
// FStat normalisation and thresholding

// FStat normalisation (auxi.c:214-240) and thresholding (jobcore.c:659-669)
// in one kernel.  One CTA per two 4096-bin chunks of one spindown: it loads
// the chunks, forms each block mean mu = sum/(2*4096) with a fixed reduction
// order (16 loads per thread at stride 256, xor tree per warp, warps in
// order), so a chunk's mu is bit-identical whichever CTA computes it; chunks
// beyond the last full block stay unnormalised.  When a bin is above trl,
// the normalised values go to shared memory, where runs of bins above trl
// are found; a run produces one candidate at its maximum, ties to the later
// bin.  The neighbour chunks' means are formed on demand (run starting at
// the chunk's first bin, or reaching its end), with all threads taking part.
__device__ __forceinline__ void emit_cand(DevCand* cand, int* ncand, int cap, int task, int ss, int ii,
                                          double F) {
  const int slot = atomicAdd(ncand, 1);
  if (slot < cap) {
    DevCand d;
    d.task = task;
    d.ss = ss;
    d.ii = ii;
    d.pad = 0;
    d.F = F;
    cand[slot] = d;
  }
}

template <typename R> __device__ __forceinline__ R chunk_sum(const R* f, int base, int cnt, R (*red)) {
  R v[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int i = k * 256 + threadIdx.x;
    v[k] = i < cnt ? f[base + i] : (R)0;
  }
  R acc = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) acc += v[k];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  R sum = 0;
  for (int k = 0; k < 8; ++k) sum += red[k];
  return sum;
}

// One chunk's normalised values v (this thread's 16, at k * 256 + tid),
// loaded as in load_chunk and scaled by its 1/mu: its runs above trl, their
// candidates, and a run reaching the chunk end followed into the next
// chunks.  Called by all threads of the CTA (it has barriers).
template <typename R>
__device__ __forceinline__ void chunk_runs(const R* f, R (&v)[16], unsigned above, int c, int bins, int nblk,
                                           int white, R trl, int nmin, int ss, int task, DevCand* cand,
                                           int* ncand, int cap, R* sv, R* red) {
  const int nchunk = (bins + 4095) >> 12;
  const int base = c * 4096;
  const int cnt = min(4096, bins - base);
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int i = k * 256 + threadIdx.x;
    if (i < cnt) sv[i + 1] = v[k];
  }
  __syncthreads();
  // value of the bin before the chunk, needed only when the chunk's first
  // bin is above the threshold
  if (c > 0 && sv[1] > trl) {
    const bool pn = !white && c - 1 < nblk;
    const R s = chunk_sum(f, base - 4096, 4096, red);
    if (threadIdx.x == 0) sv[0] = pn ? f[base - 1] * ((R)(2 * 4096) / s) : f[base - 1];
    __syncthreads();
  }
  int ii = -1;
  R Fc = 0;
  bool pend = false;  // this thread's run reaches the chunk end
  while (above) {
    const int k = __ffs(above) - 1;
    above &= above - 1;
    const int i = k * 256 + threadIdx.x;
    if (base + i != 0 && sv[i] > trl) continue;  // not the start of a run
    int iib = base + i;
    R Fcb = sv[i + 1];
    int jj = i + 1;
    for (; jj < cnt; ++jj) {
      const R w = sv[jj + 1];
      if (!(w > trl)) break;
      if (w >= Fcb) {
        iib = base + jj;
        Fcb = w;
      }
    }
    if (jj == cnt && c + 1 < nchunk) {
      ii = iib;  // continued below
      Fc = Fcb;
      pend = true;
    } else {
      emit_cand(cand, ncand, cap, task, ss, iib + nmin, Fcb);
    }
  }
  // follow a run across chunk ends; uniform loop, at most one thread active
  bool cont = pend;
  int cur = c;
  while (__syncthreads_or(cont)) {
    ++cur;
    if (cur >= nchunk) break;
    const int b2 = cur * 4096, n2 = min(4096, bins - b2);
    const bool pn = !white && cur < nblk;
    const R s = chunk_sum(f, b2, n2, red);
    if (cont) {
      const R im2 = pn ? (R)(2 * 4096) / s : (R)1;
      int j = 0;
      for (; j < n2; ++j) {
        const R w = f[b2 + j] * im2;
        if (!(w > trl)) break;
        if (w >= Fc) {
          ii = b2 + j;
          Fc = w;
        }
      }
      cont = (j == n2);
    }
  }
  if (pend) emit_cand(cand, ncand, cap, task, ss, ii + nmin, Fc);
  __syncthreads();  // sv is reused by the next chunk
}

// Two 4096-bin chunks per CTA (blockIdx.x: chunks 2x and 2x + 1 of the
// spindown blockIdx.y): both chunks' loads in flight together.
template <typename R>
__global__ void __launch_bounds__(256)
    k_normthresh(const R* __restrict__ F, int bins, int nblk, int white, R trl, int nmin, int ss0, int task,
                 DevCand* __restrict__ cand, int* __restrict__ ncand, int cap, R* __restrict__ Fdbg) {
  __shared__ R sv[4096 + 1];
  __shared__ R red[16];
  CtaTrace trace_(KK_THRESHOLD);
  const int sidx = blockIdx.y;
  const int nchunk = (bins + 4095) >> 12;
  const R* f = F + (size_t)sidx * bins;
  const int cA = 2 * blockIdx.x, cB = cA + 1;
  R va[16], vb[16];
  auto load = [&](int c, R (&v)[16]) {
    const int base = c * 4096, cnt = c < nchunk ? min(4096, bins - base) : 0;
    if (cnt == 4096) {
#pragma unroll
      for (int k = 0; k < 16; ++k) v[k] = f[base + k * 256 + threadIdx.x];
    } else {
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        const int i = k * 256 + threadIdx.x;
        v[k] = i < cnt ? f[base + i] : (R)0;
      }
    }
  };
  load(cA, va);
  load(cB, vb);
  // normalised value = F * (1/mu), mu = block sum / (2*4096); within one
  // ulp of F/mu.  The two chunks' sums in the same fixed order as one.
  R accA = 0, accB = 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    accA += va[k];
    accB += vb[k];
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    accA += __shfl_xor_sync(0xffffffffu, accA, off);
    accB += __shfl_xor_sync(0xffffffffu, accB, off);
  }
  if ((threadIdx.x & 31) == 0) {
    red[threadIdx.x >> 5] = accA;
    red[8 + (threadIdx.x >> 5)] = accB;
  }
  __syncthreads();
  R sumA = 0, sumB = 0;
  for (int k = 0; k < 8; ++k) {
    sumA += red[k];
    sumB += red[8 + k];
  }
  const R imA = (!white && cA < nblk) ? (R)(2 * 4096) / sumA : (R)1;
  const R imB = (!white && cB < nblk) ? (R)(2 * 4096) / sumB : (R)1;
  unsigned abA = 0, abB = 0;  // bit k: element k*256 + tid is above the threshold
  const int cntA = min(4096, bins - cA * 4096), cntB = cB < nchunk ? min(4096, bins - cB * 4096) : 0;
#pragma unroll
  for (int k = 0; k < 16; ++k) {
    const int i = k * 256 + threadIdx.x;
    va[k] *= imA;
    vb[k] *= imB;
    abA |= (i < cntA && va[k] > trl) ? (1u << k) : 0u;
    abB |= (i < cntB && vb[k] > trl) ? (1u << k) : 0u;
  }
  if (Fdbg) {
    for (int k = 0; k < 16; ++k) {
      const int i = k * 256 + threadIdx.x;
      if (i < cntA) Fdbg[(size_t)sidx * bins + cA * 4096 + i] = va[k];
      if (i < cntB) Fdbg[(size_t)sidx * bins + cB * 4096 + i] = vb[k];
    }
  }
  // no bin of either chunk above the threshold (the usual case): no run
  // starts here (a run from the previous chunk is followed by that chunk's
  // CTA)
  if (!__syncthreads_or((abA | abB) != 0u)) return;
  chunk_runs(f, va, abA, cA, bins, nblk, white, trl, nmin, ss0 + sidx, task, cand, ncand, cap, sv, red);
  if (cB < nchunk)
    chunk_runs(f, vb, abB, cB, bins, nblk, white, trl, nmin, ss0 + sidx, task, cand, ncand, cap, sv, red);
}

// ------------------------------------------------------------------
// engine

inline Geom make_geom(int L, int E) {
  Geom g;
  int m = 0;
  while ((1 << m) < L) ++m;
  g.L = L;
  g.logL = m;
  g.logL1 = (m + 1) / 2;
  g.logL2 = m / 2;
  g.L1 = 1 << g.logL1;
  g.L2 = 1 << g.logL2;
  int logE = 0;
  while ((1 << logE) < E) ++logE;
  g.logC = logE - 1 - g.logL1;
  g.C = 1 << g.logC;
  g.logRr = logE - 1 - g.logL2;
  g.Rr = 1 << g.logRr;
  g.twlo_log = 10;
  return g;
}

template <typename R, int PM> class EngineT : public Engine {
  typedef typename CT<R>::T T;
  Buffers b_;
  Geom gf_, gm_;
  long long launches_ = 0;
  int split_ = 0;
  int dev_ = 0;  // device the engine was made on (current at construction)
  // spindown pass A of two detectors with L1 = 256: the radix-16 kernel
  // (default) or the generic radix-4/8 one (environment PA_SPIN_PASS_A=radix8)
  bool a16_ = true;

  // The spindown pass A is the radix-16 kernel: FP32, two detectors, L1 =
  // 256 with the current split (the template condition of fft_l).
  bool use_a16() const {
    if (sizeof(R) != 4 || b_.nifo != 2 || !a16_ || !b_.tw_pass[split_]) return false;
    const int m = gm_.logL;
    return (split_ ? m / 2 : (m + 1) / 2) == 8;
  }
  // Detector whose record halves the prelude stores as {xb, xa}: detector 1
  // when the radix-16 pass A reads the records, else none (-1).
  int swapped_det() const override { return use_a16() ? 1 : -1; }

  // CUDA events around a launch when profiling is on
  void pre(int kind, int items, cudaStream_t st) {
    if (!prof || !prof->on) return;
    if (prof->n == prof->cap) return;  // pool exhausted: stop recording
    Prof::Rec& r = prof->recs[prof->n];
    r.kind = kind;
    r.items = items;
    cudaEventRecord(r.a, st);
  }
  void post(cudaStream_t st) {
    if (!prof || !prof->on) return;
    if (prof->n == prof->cap) return;
    cudaEventRecord(prof->recs[prof->n].b, st);
    prof->n++;
  }

  // opt-in above 48 KB of dynamic shared memory, once per kernel instance and
  // device (the attribute is set on the current device: the engine's own,
  // made current by every entry point); `done` holds one bit per device
  template <class K> void smem_attr(K kernel, int bytes, std::atomic<unsigned long long>& done) const {
    const unsigned long long bit = 1ull << (dev_ & 63);
    if (!(done.load(std::memory_order_acquire) & bit)) {
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
      done.fetch_or(bit, std::memory_order_release);
    }
  }

  // tw: W_L1 and W_L2 tables of the default split (L1 = 2^ceil(m/2)), then
  // the two halves of the inter-pass twiddle; SPLIT 1 swaps the factors and
  // so the first two tables.
  template <int SIGN, int LOGL, int SPLIT, class Loader, class Storer>
  cudaError_t fft_l(const void* const* tw, const Loader& ld, const Storer& st, int batch, cudaStream_t stream,
                    int kind_a, int kind_b, void* ybuf) {
    typedef FftShape<R, LOGL, SPLIT> G;
    constexpr int NT = TileCfg<R>::NT;
    const T* t1 = (const T*)tw[SPLIT ? 1 : 0];
    const T* t2 = (const T*)tw[SPLIT ? 0 : 1];
    const T* tlo = (const T*)tw[2];
    const T* thi = (const T*)tw[3];
    T* yb = (T*)ybuf;
    auto ka = k_pass_a<R, SIGN, LOGL, Loader, SPLIT>;
    auto kb = k_pass_b<R, SIGN, LOGL, Storer, SPLIT>;
    static std::atomic<unsigned long long> doneA{0}, doneB{0};
    smem_attr(ka, G::smem_a, doneA);
    smem_attr(kb, G::smem_b, doneB);
    dim3 ga(G::L2 >> G::LOGC, batch), gb(G::L1 >> G::LOGRR, batch);
    pre(kind_a, batch, stream);
    bool done = false;
    if constexpr (IsSpinF32<Loader>::value && G::LOGL1 == 8 && G::C == 16 && NT == 512) {
      // two detectors, L1 = 256: the two-stage radix-16 pass A
      if (use_a16()) {
        auto k16 = k_pass_a16<SIGN, LOGL, IsSpinF32<Loader>::pm>;
        constexpr int smem16 = (16 * (16 * 32 + 2) + 272) * (int)sizeof(float2) + 128;
        static std::atomic<unsigned long long> done16{0};
        smem_attr(k16, smem16, done16);
        k16<<<ga, 512, smem16, stream>>>(ld, t1, (const float2*)b_.tw_pass[SPLIT], yb);
        done = true;
      }
    }
    const T* twp = nullptr;
    if constexpr (Loader::kTwiddleTable) {
      twp = (const T*)b_.tw_pass[SPLIT];
      if (!twp) return cudaErrorInvalidValue;
    }
    if (!done) ka<<<ga, NT, G::smem_a, stream>>>(ld, t1, tlo, thi, twp, yb);
    post(stream);
    pre(kind_b, batch, stream);
    kb<<<gb, NT, G::smem_b, stream>>>(st, t2, yb);
    post(stream);
    launches_ += 2;
    return cudaGetLastError();
  }

  // Dispatch on the transform length (2^12 .. 2^20) to the compile-time
  // geometry of the passes; with SPLITS, odd lengths may take the swapped
  // split (split = 1).
  template <int SIGN, bool SPLITS = false, class Loader, class Storer>
  cudaError_t fft(const Geom& g, const void* const* tw, const Loader& ld, const Storer& st, int batch,
                  cudaStream_t stream, int kind_a, int kind_b, void* ybuf, int split = 0) {
    switch (g.logL) {
#define PA_FFT_CASE(M)                                                                              \
  case M:                                                                                           \
    if (SPLITS && (M & 1) && split)                                                                 \
      return fft_l<SIGN, M, SPLITS && (M & 1)>(tw, ld, st, batch, stream, kind_a, kind_b, ybuf);    \
    return fft_l<SIGN, M, 0>(tw, ld, st, batch, stream, kind_a, kind_b, ybuf);
      PA_FFT_CASE(12) PA_FFT_CASE(13) PA_FFT_CASE(14) PA_FFT_CASE(15) PA_FFT_CASE(16)
      PA_FFT_CASE(17) PA_FFT_CASE(18) PA_FFT_CASE(19) PA_FFT_CASE(20)
#undef PA_FFT_CASE
      default: return cudaErrorInvalidValue;
    }
  }

 public:
  explicit EngineT(const Buffers& b) : b_(b) {
    cudaGetDevice(&dev_);
    const char* pa = getenv("PA_SPIN_PASS_A");
    a16_ = !(pa && strcmp(pa, "radix8") == 0);
    gf_ = make_geom(b.nfft, TileCfg<R>::E);
    gm_ = make_geom(b.nfftf, TileCfg<R>::E);
  }

  long long launches() const override { return launches_; }
  size_t real_size() const override { return sizeof(R); }
  void set_split(int split) override { split_ = (gm_.logL & 1) ? split : 0; }
#ifdef PA_CTA_TRACE
  cudaError_t set_trace(void* buf, unsigned int cap) override {
    CtaTraceRec* p = static_cast<CtaTraceRec*>(buf);
    const unsigned int zero = 0, c = buf ? cap : 0u;
    cudaError_t e = cudaMemcpyToSymbol(c_trace_buf, &p, sizeof(p));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(c_trace_cap, &c, sizeof(c));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_trace_n, &zero, sizeof(zero));
    return e;
  }
  cudaError_t trace_count(unsigned int* n) override { return cudaMemcpyFromSymbol(n, g_trace_n, sizeof(*n)); }
#else
  cudaError_t set_trace(void*, unsigned int) override { return cudaErrorNotSupported; }
  cudaError_t trace_count(unsigned int*) override { return cudaErrorNotSupported; }
#endif
  int split() const override { return split_; }

  cudaError_t prelude(const SkyArgs& sky, int slot, cudaStream_t st) override {
    const int N = b_.N, nifo = b_.nifo;
    const int nbx = (N + 255) / 256;
    pre(KK_PRELUDE_MOD, nifo, st);
    k_prelude_mod<R, PM><<<dim3(nbx, nifo), 256, 0, st>>>(
        b_.xDat, b_.DetSSB, (const R*)b_.cosmodf, (const R*)b_.sinmodf, b_.dc, sky, N, (T*)b_.xin,
        b_.shftf, sizeof(R) == 8 ? b_.ph0[slot] : b_.xm[slot], b_.part, b_.sums[slot],
        (R*)b_.sums_r[slot], b_.counter);
    post(st);
    launches_ += 1;
    // forward FFT of the zero-padded series (length nfft)
    PlainLoader<R> pl{(const T*)b_.xin, N, N};
    CStore<R> cs1{(T*)b_.spec, b_.nfft, (R)1};
    cudaError_t e = fft<-1>(gf_, b_.tw_fwd, pl, cs1, nifo, st, KK_FFT_FWD_A, KK_FFT_FWD_B, b_.ybuf_pre);
    if (e != cudaSuccess) return e;
    // spectrum remap + backward FFT of length Ninterp, scale interpftpad/Ninterp
    // (jobcore.c:338-362), as a half-length transform (HalfShiftLoader)
    HalfShiftLoader<R> hl{(const T*)b_.spec, (const T*)b_.tw_inv[2], (const T*)b_.tw_inv[3], b_.nfft,
                          b_.nfft / 2 + 1};
    InterpStore<R> is{(T*)b_.yint, (const T*)b_.xin, N, b_.Ninterp, (R)(1.0 / b_.nfft)};
    e = fft<+1>(gf_, b_.tw_invh, hl, is, nifo, st, KK_FFT_INV_A, KK_FFT_INV_B, b_.ybuf_pre);
    if (e != cudaSuccess) return e;
    // spline through the first 2N points of each resampled array
    const int n = 2 * N;
    const int nseg = (n + kSplineSeg - 1) / kSplineSeg;
    constexpr int W = SplineCfg<R>::warm;
    const int smf = spad_len<R>(kSplineSeg) * (int)sizeof(double2) + spad_len<R>(kSplineSeg + W + 2) * (int)sizeof(T);
    const int smb = spad_len<R>(kSplineSeg + W) * (int)sizeof(double2) + spad_len<R>(kSplineSeg) * (int)sizeof(T);
    static std::atomic<unsigned long long> donef{0}, doneb{0};
    smem_attr(k_spline_fwd<R>, smf, donef);
    smem_attr(k_spline_bwd<R>, smb, doneb);
    pre(KK_SPLINE_FWD, nifo, st);
    k_spline_fwd<R><<<nseg * 2 * nifo, kSplineThreads, smf, st>>>((const T*)b_.yint, b_.Ninterp,
                                                                  (double2*)b_.u, n, nseg, b_.spline_invp);
    post(st);
    pre(KK_SPLINE_BWD, nifo, st);
    k_spline_bwd<R><<<nseg * 2 * nifo, kSplineThreads, smb, st>>>((const double2*)b_.u, (T*)b_.y2, n, nseg,
                                                                  b_.spline_p);
    post(st);
    pre(KK_SPLINT, nifo, st);
    k_splint<R><<<dim3(nbx, nifo), 256, 0, st>>>((const T*)b_.yint, b_.Ninterp, (const T*)b_.y2,
                                                 b_.shftf, b_.dc, N, (T*)b_.xm[slot], swapped_det());
    post(st);
    launches_ += 3;
    return cudaGetLastError();
  }

  cudaError_t spindowns(const SkyArgs& sky, int slot, int lane, int ss0, int nb, double trl, int white,
                        int s0_flag, cudaStream_t st, void* Fdbg) override {
    const size_t lo = (size_t)lane * b_.lane_sb;  // first spindown of the lane in ybuf and F
    T* const yb = (T*)b_.ybuf + lo * 2 * b_.nfftf;
    R* const Fl = (R*)b_.F + lo * b_.bins;
    SpinLoader<R, PM> sl;
    sl.xm = (const T*)b_.xm[slot];
    sl.ph0 = b_.ph0[slot];
    sl.ss_base = sky.ss_base;
    sl.N = b_.N;
    sl.nifo = b_.nifo;
    sl.ss0 = ss0;
    sl.s0_flag = s0_flag;
    sl.M0 = sky.M0;
    sl.M4 = sky.M4;
    sl.M5 = sky.M5;
    sl.s1_0 = sky.s1_0;
    if (nb > kSpinBatchMax) return cudaErrorInvalidValue;
    if constexpr (SpinHet<R, PM>::kHost) {
      for (int k = 0; k < nb; ++k) sl.het.H[k] = het1_turns_fixed(ss0 + k, sky.M4, sky.M0);
    }
    FstatStore<R> fs{Fl, (const R*)b_.sums_r[slot], b_.nmin, b_.nmax, b_.bins};
    cudaError_t e = fft<-1, true>(gm_, b_.tw_main, sl, fs, nb, st, KK_SPIN_A, KK_SPIN_B, yb, split_);
    if (e != cudaSuccess) return e;
    const int nchunk = (b_.bins + 4095) / 4096;
    pre(KK_THRESHOLD, nb, st);
    k_normthresh<R><<<dim3((nchunk + 1) / 2, nb), 256, 0, st>>>(Fl, b_.bins, b_.nblk, white, (R)trl,
                                                      b_.nmin, ss0, sky.task, b_.cand, b_.ncand,
                                                      b_.cand_cap, (R*)Fdbg);
    post(st);
    launches_ += 1;
    return cudaGetLastError();
  }
};

}  // namespace pa
