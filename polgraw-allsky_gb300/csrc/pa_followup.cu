// pa_followup.cu -- the followup path of libpolgraw_gb300.so: the
// demodulated network F-statistic of followup/src/followup.c (Fstatnet,
// :413-535, with the sky set-up of evaluate_simplex, :986-1009) at batches
// of arbitrary points (f, s, delta, alpha), its adjoint gradient, a batched
// gradient ascent, and the reference simplex amoeba (:971-1174) with its
// evaluations batched on the device.
//
// Device layout (per context):
//   xd  [nifo][N]      Real   xDat
//   pos [nifo][N][3]   double DetSSB (x y z interleaved, as the input file)
//   cm, sm [N]         Real   cos/sin(omr i), FP64-computed (init.c:464-475)
// Per evaluated point k:
//   cand[k]            scalars of the point (phase terms, seeds)
//   coef[k][d][20]     modvir factors of detector d and their sky derivatives
//   part[k][p][6|4]    FP64 partial sums of chunk p (fixed order)
//
// Work split: chunk p covers kChunk samples of one detector; a CTA stages
// its chunk in shared memory and each warp runs kCandPerWarp points over it
// (lanes stride the samples), then reduces across lanes and writes one
// FP64 partial per point and chunk.  A second kernel sums the partials of a
// point in a fixed order, so results do not depend on the batch.
//
// Phase: FP64 (the reference's expression, in turns for the mixed form so
// that the reduction mod 1 is exact), sin/cos in the working precision.
// Nothing here waits on another CTA or kernel.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/polgraw_gb300.h"
#include "pa_trace.h"

namespace {

constexpr int kChunk = 1024;      // samples per chunk (shared-memory stage)
constexpr int kThreads = 256;     // 8 warps
constexpr int kCandPerWarp = 4;   // points per warp per chunk
constexpr int kCandPerCta = 8 * kCandPerWarp;
constexpr int kCoef = 20;         // modvir factors per point and detector
constexpr double kInv2Pi = 0.15915494309189533577;  // 1/(2 pi), rounded to double

// x mod 1 as a 64-bit fixed-point fraction (x 2^64 mod 2^64), exactly, with
// integer operations on the bits of x: x = m 2^(e-1075), so the fraction is
// m shifted by e - 1011, negated for x < 0.
__device__ __forceinline__ unsigned long long fu_turns_fixed(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7ff);
  if (e == 0) return 0ull;
  const unsigned long long m = (bits & 0xfffffffffffffull) | 0x10000000000000ull;
  const int sh = e - 1011;
  unsigned long long t;
  if (sh >= 64) t = 0ull;
  else if (sh >= 0) t = m << sh;
  else if (sh > -64) t = m >> (-sh);
  else t = 0ull;
  return (bits >> 63) ? (0ull - t) : t;
}

thread_local std::string g_fu_create_error;

// Per-point scalars.  Phase terms in FP64; everything else in the working
// precision R.
template <typename R>
struct FuCand {
  double f, s;          // sgnlo[0], sgnlo[1] (radians)
  // mixed form, phase in turns: f i/2pi + s i^2/2pi as 64-bit fixed point
  // (exact integer products), (f + oms + 2 s i) shft/2pi from FP64
  unsigned long long ffx, sfx;  // f/2pi, s/2pi in fixed-point turns
  double fo_t, st2;     // (f + oms)/2pi, 2s/2pi
  double nS[3];         // source unit vector
  float nSf[3];         // FP32 copy (derivative factors); hi parts of nS
  float nSl[3];         // lo parts of nS (two-float phase)
  float foh, fol, s2h, s2l;  // (f + oms)/2pi and 2s/2pi as two floats
  R nD[3], nA[3];       // d nS / d delta, d nS / d alpha
  R om0, s2;            // f + oms, 2 s (d phase / d shft = om0 + s2 i)
  // adjoint seeds: conj(X) parts and the factors of dF/dX, dF/dA
  R xar, xai, xbr, xbi, ka, kb, qa, qb;
  int active;
  int pad;
};

// Per-detector inputs of the modvir() formula (settings.c:281-325).
struct FuDet {
  double amod[9];
  double cphir, sphir, inv_sig2;
};

struct FuDets {
  FuDet d[PA_MAX_DETECTORS];
};

// ---------------------------------------------------------------------
// Point set-up: sin/cos of the sky angles, source vector and derivatives,
// per-detector modvir factors.  One thread per point.
//   a = 2 A1 c^2 + A2 c s + A3 c + A4 s + A0      (modvir aa)
//   b = 2 B1 c^2 + B2 c s + B3 c + B4 s + B0      (modvir bb)
//   da/ddelta = D1 c^2 + D2 c s + D3 c + D4 s + D0, db/ddelta likewise (E)
// with c, s the rotated sidereal cos/sin of the sample; d/dalpha acts on
// (c, s) only: dc/dalpha = -s, ds/dalpha = c.
// ---------------------------------------------------------------------
template <typename R>
__global__ void k_fu_prep(const double* __restrict__ pts, int n, const unsigned char* __restrict__ mask,
                          FuCand<R>* __restrict__ cand, R* __restrict__ coef, FuDets dets, int nifo,
                          double oms) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  FuCand<R> c;
  c.active = mask ? (int)mask[k] : 1;
  const double f = pts[4 * k + 0], s = pts[4 * k + 1], de = pts[4 * k + 2], al = pts[4 * k + 3];
  double sa, ca, sd, cd;
  sincos(al, &sa, &ca);
  sincos(de, &sd, &cd);
  c.f = f;
  c.s = s;
  c.ffx = fu_turns_fixed(f * kInv2Pi);
  c.sfx = fu_turns_fixed(s * kInv2Pi);
  c.fo_t = (f + oms) * kInv2Pi;
  c.st2 = 2. * s * kInv2Pi;
  c.nS[0] = ca * cd;
  c.nS[1] = sa * cd;
  c.nS[2] = sd;
  for (int j = 0; j < 3; j++) {
    c.nSf[j] = (float)c.nS[j];
    c.nSl[j] = (float)(c.nS[j] - (double)c.nSf[j]);
  }
  c.foh = (float)c.fo_t;
  c.fol = (float)(c.fo_t - (double)c.foh);
  c.s2h = (float)c.st2;
  c.s2l = (float)(c.st2 - (double)c.s2h);
  c.nD[0] = (R)(-ca * sd);
  c.nD[1] = (R)(-sa * sd);
  c.nD[2] = (R)cd;
  c.nA[0] = (R)(-sa * cd);
  c.nA[1] = (R)(ca * cd);
  c.nA[2] = (R)0;
  c.om0 = (R)(f + oms);
  c.s2 = (R)(2. * s);
  c.xar = c.xai = c.xbr = c.xbi = c.ka = c.kb = c.qa = c.qb = (R)0;
  c.pad = 0;
  cand[k] = c;
  const double c2d = cd * cd, c2sd = sd * cd;
  const double dc2d = -2. * sd * cd, dc2sd = cd * cd - sd * sd;
  for (int d = 0; d < nifo; d++) {
    const double* K = dets.d[d].amod;
    const double cosalfr = ca * dets.d[d].cphir + sa * dets.d[d].sphir;
    const double sinalfr = sa * dets.d[d].cphir - ca * dets.d[d].sphir;
    R* q = coef + ((size_t)k * nifo + d) * kCoef;
    q[0] = (R)cosalfr;
    q[1] = (R)sinalfr;
    // a
    q[2] = (R)(K[0] * (2. - c2d));               // A1
    q[3] = (R)(2. * K[1] * (2. - c2d));          // A2
    q[4] = (R)(K[2] * c2sd);                     // A3
    q[5] = (R)(K[3] * c2sd);                     // A4
    q[6] = (R)(-K[0] * (2. - c2d) + K[4] * c2d); // A0
    // b
    q[7] = (R)(K[5] * sd);                       // B1
    q[8] = (R)(2. * K[6] * sd);                  // B2
    q[9] = (R)(K[7] * cd);                       // B3
    q[10] = (R)(K[8] * cd);                      // B4
    q[11] = (R)(-K[5] * sd);                     // B0
    // da/ddelta
    q[12] = (R)(-2. * K[0] * dc2d);              // D1 (c^2)
    q[13] = (R)(-2. * K[1] * dc2d);              // D2 (c s)
    q[14] = (R)(K[2] * dc2sd);                   // D3 (c)
    q[15] = (R)(K[3] * dc2sd);                   // D4 (s)
    q[16] = (R)((K[0] + K[4]) * dc2d);           // D0
    // db/ddelta = E1 c^2 + E2 c s + E3 c + E4 s + E0
    // (E3 = -K7 sd and E4 = -K8 sd are formed in the adjoint kernel)
    q[17] = (R)(2. * K[5] * cd);                 // E1
    q[18] = (R)(2. * K[6] * cd);                 // E2
    q[19] = (R)(-K[5] * cd);                     // E0
  }
}

// Makes the adjoint pass run for the points selected by need[] with the
// constants and seeds their last forward pass left in cand[].
template <typename R>
__global__ void k_fu_select(FuCand<R>* __restrict__ cand, int n, const unsigned char* __restrict__ need) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) cand[k].active = (int)need[k];
}

template <typename R>
struct Sample {
  R x, cm, sm;
  float r0f, r1f, r2f;   // FP32 copy of the position (derivative factors); hi parts
  float r0l, r1l, r2l;   // lo parts (two-float phase)
  double r0, r1, r2;
  double di;             // the sample index as FP64
};

// The phase of sample i for point c, returned as sin and cos in R.
//   FP64 form: phi = f (i + shft) + (s i) i + (oms + 2 s i) shft
//              (followup.c:460-462 order, no contraction)
//   mixed:     phi/2pi = [f i + s i^2]/2pi + (f + oms + 2 s i) shft/2pi with
//              the bracket in exact 64-bit fixed-point turns and the rest in
//              FP64 reduced to fixed point; sin/cos of the top 32 bits in
//              FP32 (sincospif).  Three FP64 operations besides shft.
template <typename R>
__device__ __forceinline__ void fu_phase(const FuCand<R>& c, double oms, int i, double di, double shft, R* sn,
                                         R* cs) {
  if (sizeof(R) == 8) {
    const double phi = __dadd_rn(__dadd_rn(__dmul_rn(c.f, __dadd_rn(di, shft)), __dmul_rn(__dmul_rn(c.s, di), di)),
                                 __dmul_rn(__dadd_rn(oms, __dmul_rn(__dmul_rn(2., c.s), di)), shft));
    double s_, c_;
    sincos(phi, &s_, &c_);
    *sn = (R)s_;
    *cs = (R)c_;
  } else {
    const unsigned long long ui = (unsigned long long)i;
    const unsigned long long t =
        c.ffx * ui + c.sfx * (ui * ui) + fu_turns_fixed(fma(c.st2, di, c.fo_t) * shft);
    float s_, c_;
    // (the hardware __sincosf measured no faster here, where the FP64 pipe
    // bounds the kernel, and doubles the error against the FP64 form)
    sincospif((float)(int)(t >> 32) * 4.656612873077393e-10f, &s_, &c_);
    *sn = (R)s_;
    *cs = (R)c_;
  }
}

// Two-float (compensated) form of the mixed phase: shft = nS.R, the factor
// (f + oms + 2 s i)/2pi and their product with float pairs (about 44
// significant bits; error-free products by fma, sums by TwoSum), the product
// reduced mod 1 exactly (Sterbenz) and added, as fixed point, to the exact
// integer part [f i + s i^2]/2pi.  No FP64 operation per (point, sample).
struct F2 {
  float h, l;
};
__device__ __forceinline__ F2 f2_mul(float ah, float al, float bh, float bl) {
  const float p = __fmul_rn(ah, bh);
  float e = __fmaf_rn(ah, bh, -p);
  e = __fmaf_rn(ah, bl, e);
  e = __fmaf_rn(al, bh, e);
  return F2{p, e};
}
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  const float r = __fadd_rn(__fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb)), __fadd_rn(a.l, b.l));
  const float h = __fadd_rn(s, r);
  return F2{h, __fsub_rn(r, __fsub_rn(h, s))};
}
template <typename R>
__device__ __forceinline__ void fu_phase_ff(const FuCand<R>& c, int i, const Sample<R>& v, R* sn, R* cs) {
  // shft = sum_k nS_k R_k
  F2 sh = f2_mul(c.nSf[0], c.nSl[0], v.r0f, v.r0l);
  sh = f2_add(sh, f2_mul(c.nSf[1], c.nSl[1], v.r1f, v.r1l));
  sh = f2_add(sh, f2_mul(c.nSf[2], c.nSl[2], v.r2f, v.r2l));
  // w = (f + oms)/2pi + (2s/2pi) i  (i < 2^24 is exact in FP32)
  const float fi = (float)i;
  const F2 w = f2_add(F2{c.foh, c.fol}, f2_mul(c.s2h, c.s2l, fi, 0.f));
  const F2 t = f2_mul(w.h, w.l, sh.h, sh.l);
  // t mod 1: h - rint(h) is exact
  const float fr = __fadd_rn(__fsub_rn(t.h, rintf(t.h)), t.l);
  const unsigned long long ui = (unsigned long long)i;
  const unsigned long long tt =
      c.ffx * ui + c.sfx * (ui * ui) + ((unsigned long long)(long long)__float2ll_rn(fr * 4294967296.f) << 32);
  // the top 32 bits as an angle in [-pi, pi); hardware sine and cosine
  // (absolute error <= 2^-21.41 = 3.6e-7 there): this form has no FP64
  // operation per (point, sample), and the accurate sincospif is its largest
  // instruction block
  float s_, c_;
  __sincosf((float)(int)(tt >> 32) * 1.4629180792671596e-9f, &s_, &c_);  // pi 2^-31
  *sn = (R)s_;
  *cs = (R)c_;
}

template <typename R>
__device__ __forceinline__ R warp_sum(R v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------
// Forward sums (ADJ = false): per point and chunk
//   sum x a e^{-i phi}, sum x b e^{-i phi}, sum a^2, sum b^2   (x 1/sig2)
// Adjoint sums (ADJ = true): per point and chunk, the four components of
//   dF/dtheta = sum [ dphi/dtheta x (ka a Im(conj(Xa)E) + kb b Im(conj(Xb)E))
//                   + da/dtheta (x ka Re(conj(Xa)E) + 2 qa a) + (b terms) ]
//   (x 1/sig2), with E = e^{-i phi}, ka = 2 seed/A, qa = -seed |Xa|^2/A^2.
// ---------------------------------------------------------------------
template <typename R, bool ADJ, bool FF = false>
__global__ void __launch_bounds__(kThreads) k_fu_sums(const R* __restrict__ xd, const double* __restrict__ pos,
                                                      const R* __restrict__ cmf, const R* __restrict__ smf,
                                                      const FuCand<R>* __restrict__ cand, const R* __restrict__ coef,
                                                      FuDets dets, int n, int N, int nifo, int nch, double oms,
                                                      double* __restrict__ part) {
  extern __shared__ __align__(16) unsigned char fu_smem[];
  Sample<R>* sh = reinterpret_cast<Sample<R>*>(fu_smem);
  const int P = nifo * nch;
  const int p = blockIdx.x;
  const int d = p / nch;
  const int base = (p - d * nch) * kChunk;
  const int cnt = min(kChunk, N - base);
  for (int j = threadIdx.x; j < cnt; j += kThreads) {
    const int i = base + j;
    Sample<R> v;
    v.x = xd[(size_t)d * N + i];
    v.cm = cmf[i];
    v.sm = smf[i];
    const double* r = pos + ((size_t)d * N + i) * 3;
    v.r0 = r[0];
    v.r1 = r[1];
    v.r2 = r[2];
    v.r0f = (float)v.r0;
    v.r1f = (float)v.r1;
    v.r2f = (float)v.r2;
    v.r0l = (float)(v.r0 - (double)v.r0f);
    v.r1l = (float)(v.r1 - (double)v.r1f);
    v.r2l = (float)(v.r2 - (double)v.r2f);
    v.di = (double)i;
    sh[j] = v;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const double is2 = dets.d[d].inv_sig2;
  const R k7 = (R)dets.d[d].amod[7], k8 = (R)dets.d[d].amod[8];
  for (int q = 0; q < kCandPerWarp; q++) {
    const int k = blockIdx.y * kCandPerCta + warp * kCandPerWarp + q;
    if (k >= n) break;
    const FuCand<R> c = cand[k];
    if (!c.active) continue;
    const R* cf = coef + ((size_t)k * nifo + d) * kCoef;
    R Q[kCoef];
#pragma unroll
    for (int t = 0; t < kCoef; t++) Q[t] = cf[t];
    const R cosalfr = Q[0], sinalfr = Q[1];
    R acc[6] = {(R)0, (R)0, (R)0, (R)0, (R)0, (R)0};
    const R sd_ = (R)c.nS[2];  // sin(delta), for E3 = -K7 sd, E4 = -K8 sd
    for (int j = lane; j < cnt; j += 32) {
      const Sample<R> v = sh[j];
      const int i = base + j;
      const R cc = cosalfr * v.cm + sinalfr * v.sm;
      const R ss = sinalfr * v.cm - cosalfr * v.sm;
      const R c2 = cc * cc, cs = cc * ss;
      const R a = (R)2 * Q[2] * c2 + Q[3] * cs + Q[4] * cc + Q[5] * ss + Q[6];
      const R b = (R)2 * Q[7] * c2 + Q[8] * cs + Q[9] * cc + Q[10] * ss + Q[11];
      R sn, co;
      double shft = 0.;
      if (FF) {
        fu_phase_ff<R>(c, i, v, &sn, &co);
      } else {
        shft = c.nS[0] * v.r0 + c.nS[1] * v.r1 + c.nS[2] * v.r2;
        fu_phase<R>(c, oms, i, v.di, shft, &sn, &co);
      }
      if (!ADJ) {
        const R xa = v.x * a, xb = v.x * b;
        acc[0] += xa * co;
        acc[1] -= xa * sn;
        acc[2] += xb * co;
        acc[3] -= xb * sn;
        acc[4] += a * a;
        acc[5] += b * b;
      } else {
        // conj(X) E with E = co - i sn
        const R rea = c.xar * co - c.xai * sn, ima = -(c.xar * sn + c.xai * co);
        const R reb = c.xbr * co - c.xbi * sn, imb = -(c.xbr * sn + c.xbi * co);
        const R gph = v.x * (c.ka * a * ima + c.kb * b * imb);
        const R ga = v.x * c.ka * rea + (R)2 * c.qa * a;
        const R gb = v.x * c.kb * reb + (R)2 * c.qb * b;
        const R fi = (R)i;
        // derivative factors in the working precision (FP32 copies of the
        // position in the mixed form: no per-sample conversions)
        const R r0 = sizeof(R) == 4 ? (R)v.r0f : (R)v.r0, r1 = sizeof(R) == 4 ? (R)v.r1f : (R)v.r1,
                r2 = sizeof(R) == 4 ? (R)v.r2f : (R)v.r2;
        const R sh_ = (sizeof(R) == 4 || FF) ? (R)(c.nSf[0] * v.r0f + c.nSf[1] * v.r1f + c.nSf[2] * v.r2f)
                                             : (R)shft;
        const R sh_de = c.nD[0] * r0 + c.nD[1] * r1 + c.nD[2] * r2;
        const R sh_al = c.nA[0] * r0 + c.nA[1] * r1;
        const R om = c.om0 + c.s2 * fi;
        // d a / d alpha, d b / d alpha
        const R a_al = -ss * ((R)4 * Q[2] * cc + Q[3] * ss + Q[4]) + cc * (Q[3] * cc + Q[5]);
        const R b_al = -ss * ((R)4 * Q[7] * cc + Q[8] * ss + Q[9]) + cc * (Q[8] * cc + Q[10]);
        // d a / d delta, d b / d delta
        const R a_de = Q[12] * c2 + Q[13] * cs + Q[14] * cc + Q[15] * ss + Q[16];
        const R b_de = Q[17] * c2 + Q[18] * cs - k7 * sd_ * cc - k8 * sd_ * ss + Q[19];
        acc[0] += gph * (fi + sh_);
        acc[1] += gph * (fi * fi + (R)2 * fi * sh_);
        acc[2] += gph * om * sh_de + ga * a_de + gb * b_de;
        acc[3] += gph * om * sh_al + ga * a_al + gb * b_al;
      }
    }
    constexpr int NA = ADJ ? 4 : 6;
    double* out = part + ((size_t)k * P + p) * NA;
#pragma unroll
    for (int t = 0; t < NA; t++) {
      const R v = warp_sum<R>(acc[t]);
      if (lane == 0) out[t] = (double)v * is2;
    }
  }
}

// Sum of the partials of one point in a fixed order (lane stride, then a
// fixed shuffle tree).
__device__ __forceinline__ double fixed_sum(const double* __restrict__ p, int P, int stride, int lane) {
  double s = 0.;
  for (int j = lane; j < P; j += 32) s += p[(size_t)j * stride];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// F and fstat_out (followup.c:508-529) per point; res[k] = {Xa, Xb, A, B}
// kept for the adjoint.  One warp per point.
template <typename R>
__global__ void k_fu_final(const double* __restrict__ part, const double* __restrict__ pts,
                           FuCand<R>* __restrict__ cand, int n, int P, double* __restrict__ res,
                           double* __restrict__ Fo, double* __restrict__ out, const double* __restrict__ seed) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= n) return;
  if (!cand[k].active) return;
  double v[6];
  for (int t = 0; t < 6; t++) v[t] = fixed_sum(part + (size_t)k * P * 6 + t, P, 6, lane);
  if (lane) return;
  const double xr = v[0], xi = v[1], yr = v[2], yi = v[3], A = v[4], B = v[5];
  const double F = ((xr * xr + xi * xi) / A) + ((yr * yr + yi * yi) / B);
  if (res)
    for (int t = 0; t < 6; t++) res[(size_t)k * 6 + t] = v[t];
  if (Fo) Fo[k] = F;
  if (out) {
    double* o = out + (size_t)k * 11;
    o[5] = -F;
    o[0] = 2 * xr / A;
    o[1] = 2 * yr / B;
    o[2] = -2 * xi / A;
    o[3] = -2 * yi / B;
    o[4] = sqrt(2 * (F - 2));
    for (int j = 0; j < 4; j++) o[6 + j] = pts[4 * k + j];
    o[10] = sqrt((2 * xr) * (2 * xr) + (2 * yr) * (2 * yr) + (2 * xi) * (2 * xi) + (2 * yi) * (2 * yi));
  }
  // seeds of the adjoint pass
  const double sd = seed ? seed[k] : 1.0;
  FuCand<R>& c = cand[k];
  c.xar = (R)xr;
  c.xai = (R)xi;
  c.xbr = (R)yr;
  c.xbi = (R)yi;
  c.ka = (R)(2. * sd / A);
  c.kb = (R)(2. * sd / B);
  c.qa = (R)(-sd * (xr * xr + xi * xi) / (A * A));
  c.qb = (R)(-sd * (yr * yr + yi * yi) / (B * B));
}

template <typename R>
__global__ void k_fu_final_adj(const double* __restrict__ part, const FuCand<R>* __restrict__ cand, int n, int P,
                               double* __restrict__ grad) {
  const int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (k >= n) return;
  if (!cand[k].active) return;
  double v[4];
  for (int t = 0; t < 4; t++) v[t] = fixed_sum(part + (size_t)k * P * 4 + t, P, 4, lane);
  if (lane) return;
  for (int t = 0; t < 4; t++) grad[(size_t)k * 4 + t] = v[t];
}

// ---------------------------------------------------------------------
// Gradient ascent state machine (one thread per point): BFGS on -F in
// scaled coordinates u = theta / scale (peak-width units), with a
// backtracking line search.
//   propose: trial u' = u + t p, p = H g_u (g_u = scale * grad; H the
//            inverse-Hessian estimate of -F, first H = (step0/|g_u|) I)
//   decide:  F(trial) >= F + 1e-4 t g_u.p -> accept (t = 1 next), need the
//            gradient there; otherwise t *= 0.5
//   take:    with s = u' - u, y = g_u(old) - g_u(new): when y.s > 0,
//            H <- (I - r s y^T) H (I - r y s^T) + r s s^T, r = 1/y.s
//   a point stops when its step |t p| falls below min_step, its gradient
//   vanishes, or the direction stops being an ascent direction.
// ---------------------------------------------------------------------
struct AscentState {
  double theta[4], grad[4], trial[4];
  double gold[4], sdir[4];   // g_u before the accepted step, the step s
  double H[16];              // inverse-Hessian estimate (row-major)
  double p[4];               // search direction
  double F, t;
  int active, iters;
};

__global__ void k_asc_propose(AscentState* __restrict__ st, int n, double s0, double s1, double s2, double s3,
                              double min_step, double* __restrict__ trial_pts, unsigned char* __restrict__ mask) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  AscentState& a = st[k];
  const double sc[4] = {s0, s1, s2, s3};
  if (a.active) {
    double gu[4], slope = 0., plen = 0.;
    for (int j = 0; j < 4; j++) gu[j] = sc[j] * a.grad[j];
    for (int i = 0; i < 4; i++) {
      double v = 0.;
      for (int j = 0; j < 4; j++) v += a.H[4 * i + j] * gu[j];
      a.p[i] = v;
      slope += v * gu[i];
      plen += v * v;
    }
    plen = sqrt(plen);
    if (!(slope > 0.) || !isfinite(slope) || a.t * plen < min_step) a.active = 0;
  }
  mask[k] = (unsigned char)a.active;
  for (int j = 0; j < 4; j++) {
    a.trial[j] = a.active ? a.theta[j] + sc[j] * a.t * a.p[j] : a.theta[j];
    trial_pts[4 * k + j] = a.trial[j];
  }
}

__global__ void k_asc_decide(AscentState* __restrict__ st, int n, double s0, double s1, double s2, double s3,
                             const double* __restrict__ Ftrial, unsigned char* __restrict__ need_grad,
                             int* __restrict__ nactive) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  AscentState& a = st[k];
  need_grad[k] = 0;
  if (!a.active) return;
  const double sc[4] = {s0, s1, s2, s3};
  double slope = 0.;
  for (int j = 0; j < 4; j++) slope += a.p[j] * sc[j] * a.grad[j];
  const double Ft = Ftrial[k];
  if (Ft >= a.F + 1e-4 * a.t * slope && Ft > a.F) {
    for (int j = 0; j < 4; j++) {
      a.gold[j] = sc[j] * a.grad[j];
      a.sdir[j] = a.t * a.p[j];
      a.theta[j] = a.trial[j];
    }
    a.F = Ft;
    a.t = 1.0;
    a.iters++;
    need_grad[k] = 1;
  } else {
    a.t *= 0.5;
  }
  atomicAdd(nactive, 1);
}

__global__ void k_asc_init(AscentState* __restrict__ st, int n, const double* __restrict__ pts,
                           const double* __restrict__ F, const double* __restrict__ grad, double s0, double s1,
                           double s2, double s3, double step0) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  AscentState& a = st[k];
  const double sc[4] = {s0, s1, s2, s3};
  double nrm = 0.;
  for (int j = 0; j < 4; j++) {
    a.theta[j] = pts[4 * k + j];
    a.grad[j] = grad[4 * k + j];
    a.trial[j] = a.theta[j];
    a.gold[j] = a.sdir[j] = a.p[j] = 0.;
    nrm += (sc[j] * a.grad[j]) * (sc[j] * a.grad[j]);
  }
  nrm = sqrt(nrm);
  const double h0 = nrm > 0. ? step0 / nrm : 0.;
  for (int j = 0; j < 16; j++) a.H[j] = (j % 5 == 0) ? h0 : 0.;
  a.F = F[k];
  a.t = 1.0;
  a.active = nrm > 0. && isfinite(nrm);
  a.iters = 0;
}

__global__ void k_asc_take_grad(AscentState* __restrict__ st, int n, double s0, double s1, double s2, double s3,
                                const unsigned char* __restrict__ need, const double* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n || !need[k]) return;
  AscentState& a = st[k];
  const double sc[4] = {s0, s1, s2, s3};
  double y[4], ys = 0.;
  for (int j = 0; j < 4; j++) {
    a.grad[j] = grad[4 * k + j];
    y[j] = a.gold[j] - sc[j] * a.grad[j];
    ys += y[j] * a.sdir[j];
  }
  if (!(ys > 0.) || !isfinite(ys)) return;  // keep H (curvature condition fails)
  const double r = 1. / ys;
  // H <- (I - r s y^T) H (I - r y s^T) + r s s^T
  double Hy[4], yHy = 0.;
  for (int i = 0; i < 4; i++) {
    double v = 0.;
    for (int j = 0; j < 4; j++) v += a.H[4 * i + j] * y[j];
    Hy[i] = v;
    yHy += y[i] * v;
  }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++)
      a.H[4 * i + j] += -r * (a.sdir[i] * Hy[j] + Hy[i] * a.sdir[j]) + (r * r * yHy + r) * a.sdir[i] * a.sdir[j];
}

__global__ void k_asc_export(const AscentState* __restrict__ st, int n, double* __restrict__ pts,
                             int* __restrict__ iters) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  for (int j = 0; j < 4; j++) pts[4 * k + j] = st[k].theta[j];
  iters[k] = st[k].iters;
}

}  // namespace

// ---------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------
struct pa_followup {
  int dev = 0;
  bool fp64 = false;
  bool ffphase = false;  // mixed form with the two-float phase
  int N = 0, nifo = 0, nch = 0;
  double oms = 0.;
  FuDets dets;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  void* xd = nullptr;
  double* pos = nullptr;
  void* cm = nullptr;
  void* sm = nullptr;
  // per-batch buffers (grown on demand)
  int cap = 0;
  double* pts = nullptr;
  void* cand = nullptr;
  void* coef = nullptr;
  double* part = nullptr;
  double* res = nullptr;
  double* F = nullptr;
  double* out = nullptr;
  double* grad = nullptr;
  double* seed = nullptr;
  unsigned char* mask = nullptr;
  unsigned char* need = nullptr;
  AscentState* asc = nullptr;
  int* iters = nullptr;
  int* counter = nullptr;
  double* trial = nullptr;
  std::string err;
  long long launches = 0;
  double last_ms = 0.;
};

static int fu_fail(pa_followup* f, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (f) f->err = buf;
  else g_fu_create_error = buf;
  return code;
}

#define FCK(call, what)                                                                             \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) return fu_fail(f, PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
  } while (0)

static size_t fu_rsz(const pa_followup* f) { return f->fp64 ? 8 : 4; }

static void fu_free_batch(pa_followup* f) {
  void* ps[] = {f->pts, f->cand, f->coef, f->part, f->res, f->F, f->out, f->grad, f->seed,
                f->mask, f->need, f->asc, f->iters, f->counter, f->trial};
  for (void* p : ps)
    if (p) cudaFree(p);
  f->pts = nullptr;
  f->cand = nullptr;
  f->coef = nullptr;
  f->part = nullptr;
  f->res = f->F = f->out = f->grad = f->seed = f->trial = nullptr;
  f->mask = f->need = nullptr;
  f->asc = nullptr;
  f->iters = f->counter = nullptr;
  f->cap = 0;
}

static int fu_reserve(pa_followup* f, int n) {
  if (n <= f->cap) return PA_OK;
  fu_free_batch(f);
  const int c = std::max(n, 64);
  const size_t P = (size_t)f->nifo * f->nch;
  const size_t candsz = f->fp64 ? sizeof(FuCand<double>) : sizeof(FuCand<float>);
#define FALLOC(ptr, bytes) FCK(cudaMalloc((void**)&(ptr), (bytes)), "cudaMalloc")
  FALLOC(f->pts, sizeof(double) * 4 * c);
  FALLOC(f->cand, candsz * c);
  FALLOC(f->coef, fu_rsz(f) * kCoef * f->nifo * (size_t)c);
  FALLOC(f->part, sizeof(double) * 6 * P * c);
  FALLOC(f->res, sizeof(double) * 6 * c);
  FALLOC(f->F, sizeof(double) * c);
  FALLOC(f->out, sizeof(double) * 11 * c);
  FALLOC(f->grad, sizeof(double) * 4 * c);
  FALLOC(f->seed, sizeof(double) * c);
  FALLOC(f->mask, c);
  FALLOC(f->need, c);
  FALLOC(f->asc, sizeof(AscentState) * c);
  FALLOC(f->iters, sizeof(int) * c);
  FALLOC(f->counter, sizeof(int));
  FALLOC(f->trial, sizeof(double) * 4 * c);
#undef FALLOC
  f->cap = c;
  return PA_OK;
}

template <typename R>
static size_t fu_smem() {
  return sizeof(Sample<R>) * kChunk;
}

// One launch of the sums kernel in the context's phase form.
template <typename R, bool ADJ>
static void fu_sums(pa_followup* f, int n, dim3 grid) {
  FuCand<R>* cand = (FuCand<R>*)f->cand;
  if (sizeof(R) == 4 && f->ffphase)
    k_fu_sums<R, ADJ, true><<<grid, kThreads, fu_smem<R>(), f->stream>>>(
        (const R*)f->xd, f->pos, (const R*)f->cm, (const R*)f->sm, cand, (const R*)f->coef, f->dets, n, f->N,
        f->nifo, f->nch, f->oms, f->part);
  else
    k_fu_sums<R, ADJ, false><<<grid, kThreads, fu_smem<R>(), f->stream>>>(
        (const R*)f->xd, f->pos, (const R*)f->cm, (const R*)f->sm, cand, (const R*)f->coef, f->dets, n, f->N,
        f->nifo, f->nch, f->oms, f->part);
}

// Forward (and optionally adjoint) evaluation of n points already in
// f->pts; mask (device, may be null) selects the active points.
template <typename R>
static int fu_eval_t(pa_followup* f, int n, const unsigned char* mask, bool want_out, bool adjoint,
                     const double* seed_dev) {
  const int P = f->nifo * f->nch;
  FuCand<R>* cand = (FuCand<R>*)f->cand;
  k_fu_prep<R><<<(n + 127) / 128, 128, 0, f->stream>>>(f->pts, n, mask, cand, (R*)f->coef, f->dets, f->nifo,
                                                          f->oms);
  dim3 grid(P, (n + kCandPerCta - 1) / kCandPerCta);
  fu_sums<R, false>(f, n, grid);
  k_fu_final<R><<<(n + 7) / 8, 256, 0, f->stream>>>(f->part, f->pts, cand, n, P, f->res, f->F,
                                                     want_out ? f->out : nullptr, seed_dev);
  f->launches += 3;
  if (adjoint) {
    fu_sums<R, true>(f, n, grid);
    k_fu_final_adj<R><<<(n + 7) / 8, 256, 0, f->stream>>>(f->part, cand, n, P, f->grad);
    f->launches += 2;
  }
  FCK(cudaGetLastError(), "followup launch");
  return PA_OK;
}

// Adjoint pass only, for the points selected by need[] (device).
template <typename R>
static int fu_adjoint_t(pa_followup* f, int n, const unsigned char* need) {
  const int P = f->nifo * f->nch;
  FuCand<R>* cand = (FuCand<R>*)f->cand;
  k_fu_select<R><<<(n + 255) / 256, 256, 0, f->stream>>>(cand, n, need);
  dim3 grid(P, (n + kCandPerCta - 1) / kCandPerCta);
  fu_sums<R, true>(f, n, grid);
  k_fu_final_adj<R><<<(n + 7) / 8, 256, 0, f->stream>>>(f->part, cand, n, P, f->grad);
  f->launches += 3;
  FCK(cudaGetLastError(), "followup adjoint launch");
  return PA_OK;
}

static int fu_eval(pa_followup* f, int n, const unsigned char* mask, bool want_out, bool adjoint,
                   const double* seed_dev) {
  return f->fp64 ? fu_eval_t<double>(f, n, mask, want_out, adjoint, seed_dev)
                 : fu_eval_t<float>(f, n, mask, want_out, adjoint, seed_dev);
}

static int fu_begin(pa_followup* f, int n) {
  FCK(cudaSetDevice(f->dev), "cudaSetDevice");
  int rc = fu_reserve(f, n);
  if (rc) return rc;
  FCK(cudaEventRecord(f->ev0, f->stream), "event");
  return PA_OK;
}

static int fu_end(pa_followup* f) {
  FCK(cudaEventRecord(f->ev1, f->stream), "event");
  FCK(cudaStreamSynchronize(f->stream), "followup");
  float ms = 0.f;
  FCK(cudaEventElapsedTime(&ms, f->ev0, f->ev1), "event time");
  f->last_ms += ms;
  return PA_OK;
}

extern "C" {

pa_followup* pa_followup_create(const pa_settings* sett, const pa_detector* det, int nifo, const pa_config* cfg,
                                int* status) {
  pa::TraceRange trace_("pa_followup_create");
  auto ret = [&](int st) {
    if (status) *status = st;
    return (pa_followup*)nullptr;
  };
  pa_followup* f = nullptr;
  if (!sett || !det || nifo < 1 || nifo > PA_MAX_DETECTORS || sett->N < 1)
    return fu_fail(f, PA_ERR_ARG, "pa_followup_create: invalid settings or detectors"), ret(PA_ERR_ARG);
  const pa_config dflt = {PA_PREC_MIXED, PA_PHASE_FIXED, 0, 0};
  const pa_config c = cfg ? *cfg : dflt;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return fu_fail(f, PA_ERR_NODEV, "pa_followup_create: no CUDA device"), ret(PA_ERR_NODEV);
  if (c.device < 0 || c.device >= ndev)
    return fu_fail(f, PA_ERR_ARG, "pa_followup_create: device %d out of range", c.device), ret(PA_ERR_ARG);
  f = new pa_followup();
  f->dev = c.device;
  f->fp64 = c.precision == PA_PREC_FP64;
  f->ffphase = !f->fp64 && c.phase_mode == PA_PHASE_FF;
  f->N = sett->N;
  f->nifo = nifo;
  f->nch = (sett->N + kChunk - 1) / kChunk;
  f->oms = sett->oms;
  memset(&f->dets, 0, sizeof(f->dets));
  for (int d = 0; d < nifo; d++) {
    memcpy(f->dets.d[d].amod, det[d].amod, sizeof(double) * 9);
    f->dets.d[d].cphir = det[d].cphir;
    f->dets.d[d].sphir = det[d].sphir;
    f->dets.d[d].inv_sig2 = 1. / det[d].sig2;
  }
  auto bail = [&](const char* what, cudaError_t e) {
    g_fu_create_error = std::string("pa_followup_create: ") + what + ": " + cudaGetErrorString(e);
    pa_followup_destroy(f);
    if (status) *status = PA_ERR_CUDA;
    return (pa_followup*)nullptr;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(f->dev)) != cudaSuccess) return bail("cudaSetDevice", e);
  if ((e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail("stream", e);
  if ((e = cudaEventCreate(&f->ev0)) != cudaSuccess) return bail("event", e);
  if ((e = cudaEventCreate(&f->ev1)) != cudaSuccess) return bail("event", e);
  const int N = sett->N;
  const size_t rs = f->fp64 ? 8 : 4;
  if ((e = cudaMalloc(&f->xd, rs * nifo * (size_t)N)) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMalloc((void**)&f->pos, sizeof(double) * 3 * nifo * (size_t)N)) != cudaSuccess)
    return bail("cudaMalloc", e);
  if ((e = cudaMalloc(&f->cm, rs * N)) != cudaSuccess) return bail("cudaMalloc", e);
  if ((e = cudaMalloc(&f->sm, rs * N)) != cudaSuccess) return bail("cudaMalloc", e);
  // host staging: xDat and cos/sin(omr i) (followup init.c:470-475) in the
  // working precision, DetSSB as is
  std::vector<double> xd64((size_t)nifo * N), c64(N), s64(N);
  for (int d = 0; d < nifo; d++) memcpy(&xd64[(size_t)d * N], det[d].xDat, sizeof(double) * N);
  for (int i = 0; i < N; i++) {
    const double omrt = sett->omr * i;
    c64[i] = cos(omrt);
    s64[i] = sin(omrt);
  }
  auto up = [&](void* dst, const std::vector<double>& src) -> cudaError_t {
    if (f->fp64) return cudaMemcpy(dst, src.data(), sizeof(double) * src.size(), cudaMemcpyHostToDevice);
    std::vector<float> t(src.size());
    for (size_t j = 0; j < src.size(); j++) t[j] = (float)src[j];
    return cudaMemcpy(dst, t.data(), sizeof(float) * t.size(), cudaMemcpyHostToDevice);
  };
  if ((e = up(f->xd, xd64)) != cudaSuccess) return bail("upload", e);
  if ((e = up(f->cm, c64)) != cudaSuccess) return bail("upload", e);
  if ((e = up(f->sm, s64)) != cudaSuccess) return bail("upload", e);
  for (int d = 0; d < nifo; d++)
    if ((e = cudaMemcpy(f->pos + (size_t)d * 3 * N, det[d].DetSSB, sizeof(double) * 3 * N,
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      return bail("upload", e);
  const size_t smem = f->fp64 ? fu_smem<double>() : fu_smem<float>();
  if (f->fp64) {
    cudaFuncSetAttribute(k_fu_sums<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_fu_sums<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  } else {
    cudaFuncSetAttribute(k_fu_sums<float, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_fu_sums<float, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_fu_sums<float, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(k_fu_sums<float, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return bail("set-up", e);
  if (status) *status = PA_OK;
  return f;
}

void pa_followup_destroy(pa_followup* f) {
  if (!f) return;
  cudaSetDevice(f->dev);
  if (f->stream) cudaStreamSynchronize(f->stream);
  fu_free_batch(f);
  void* ps[] = {f->xd, f->pos, f->cm, f->sm};
  for (void* p : ps)
    if (p) cudaFree(p);
  if (f->ev0) cudaEventDestroy(f->ev0);
  if (f->ev1) cudaEventDestroy(f->ev1);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
}

const char* pa_followup_last_error(const pa_followup* f) {
  return f ? f->err.c_str() : g_fu_create_error.c_str();
}

double pa_followup_last_call_ms(const pa_followup* f) { return f ? f->last_ms : 0.; }
long long pa_followup_kernel_launches(const pa_followup* f) { return f ? f->launches : 0; }

int pa_fstatnet(pa_followup* f, const double* sgnlo, int n, double* out) {
  pa::TraceRange trace_("pa_fstatnet");
  if (!f || !sgnlo || !out || n < 0) return fu_fail(f, PA_ERR_ARG, "pa_fstatnet: invalid arguments");
  if (n == 0) return PA_OK;
  f->last_ms = 0.;
  int rc = fu_begin(f, n);
  if (rc) return rc;
  FCK(cudaMemcpyAsync(f->pts, sgnlo, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, f->stream), "copy");
  if ((rc = fu_eval(f, n, nullptr, true, false, nullptr))) return rc;
  FCK(cudaMemcpyAsync(out, f->out, sizeof(double) * 11 * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  return fu_end(f);
}

int pa_fstatnet_grad(pa_followup* f, const double* sgnlo, int n, const double* seed, double* F, double* grad) {
  pa::TraceRange trace_("pa_fstatnet_grad");
  if (!f || !sgnlo || !F || !grad || n < 0) return fu_fail(f, PA_ERR_ARG, "pa_fstatnet_grad: invalid arguments");
  if (n == 0) return PA_OK;
  f->last_ms = 0.;
  int rc = fu_begin(f, n);
  if (rc) return rc;
  FCK(cudaMemcpyAsync(f->pts, sgnlo, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, f->stream), "copy");
  if (seed)
    FCK(cudaMemcpyAsync(f->seed, seed, sizeof(double) * n, cudaMemcpyHostToDevice, f->stream), "copy");
  if ((rc = fu_eval(f, n, nullptr, false, true, seed ? f->seed : nullptr))) return rc;
  FCK(cudaMemcpyAsync(F, f->F, sizeof(double) * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  FCK(cudaMemcpyAsync(grad, f->grad, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  return fu_end(f);
}

int pa_followup_ascent(pa_followup* f, double* sgnlo, int n, const pa_ascent_opts* opts, double* out, int* iters) {
  pa::TraceRange trace_("pa_followup_ascent");
  if (!f || !sgnlo || !out || !opts || n < 0) return fu_fail(f, PA_ERR_ARG, "pa_followup_ascent: invalid arguments");
  for (int j = 0; j < 4; j++)
    if (!(opts->scale[j] > 0.)) return fu_fail(f, PA_ERR_ARG, "pa_followup_ascent: scale[%d] must be > 0", j);
  if (n == 0) return PA_OK;
  const double step0 = opts->step0 > 0. ? opts->step0 : 0.25;
  const double min_step = opts->min_step > 0. ? opts->min_step : 1e-3;
  const int max_iter = opts->max_iter > 0 ? opts->max_iter : 100;
  f->last_ms = 0.;
  int rc = fu_begin(f, n);
  if (rc) return rc;
  const int nb = (n + 255) / 256;
  FCK(cudaMemcpyAsync(f->pts, sgnlo, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, f->stream), "copy");
  if ((rc = fu_eval(f, n, nullptr, false, true, nullptr))) return rc;
  const double* sc = opts->scale;
  k_asc_init<<<nb, 256, 0, f->stream>>>(f->asc, n, f->pts, f->F, f->grad, sc[0], sc[1], sc[2], sc[3], step0);
  f->launches++;
  int* h_active = nullptr;
  FCK(cudaMallocHost((void**)&h_active, sizeof(int)), "cudaMallocHost");
  for (int it = 0; it < max_iter; it++) {
    // trial points -> f->pts (the evaluation reads them from there)
    k_asc_propose<<<nb, 256, 0, f->stream>>>(f->asc, n, sc[0], sc[1], sc[2], sc[3], min_step, f->pts, f->mask);
    f->launches++;
    if ((rc = fu_eval(f, n, f->mask, false, false, nullptr))) break;
    cudaMemsetAsync(f->counter, 0, sizeof(int), f->stream);
    k_asc_decide<<<nb, 256, 0, f->stream>>>(f->asc, n, sc[0], sc[1], sc[2], sc[3], f->F, f->need, f->counter);
    f->launches++;
    // gradient at the accepted points: the trial evaluation left their
    // constants and adjoint seeds in cand[]; only the adjoint pass runs
    if ((rc = f->fp64 ? fu_adjoint_t<double>(f, n, f->need) : fu_adjoint_t<float>(f, n, f->need))) break;
    k_asc_take_grad<<<nb, 256, 0, f->stream>>>(f->asc, n, sc[0], sc[1], sc[2], sc[3], f->need, f->grad);
    f->launches++;
    if (cudaGetLastError() != cudaSuccess) {
      rc = fu_fail(f, PA_ERR_CUDA, "pa_followup_ascent: launch failed");
      break;
    }
    cudaMemcpyAsync(h_active, f->counter, sizeof(int), cudaMemcpyDeviceToHost, f->stream);
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) {
      rc = fu_fail(f, PA_ERR_CUDA, "pa_followup_ascent: %s", cudaGetErrorString(cudaGetLastError()));
      break;
    }
    if (*h_active == 0) break;
  }
  cudaFreeHost(h_active);
  if (rc) return rc;
  // final points and their fstat_out
  k_asc_export<<<nb, 256, 0, f->stream>>>(f->asc, n, f->pts, f->iters);
  f->launches++;
  if ((rc = fu_eval(f, n, nullptr, true, false, nullptr))) return rc;
  FCK(cudaMemcpyAsync(sgnlo, f->pts, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  FCK(cudaMemcpyAsync(out, f->out, sizeof(double) * 11 * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  if (iters) FCK(cudaMemcpyAsync(iters, f->iters, sizeof(int) * n, cudaMemcpyDeviceToHost, f->stream), "copy");
  return fu_end(f);
}

}  // extern "C"

// ---------------------------------------------------------------------
// The reference simplex as a resumable state machine per point, so that
// the evaluations of all points can be batched.  Mirrors amoeba()
// (followup.c:1126-1174) step for step: make_simplex (:971-984),
// evaluate_simplex (:986-1009), simplex_extremes (:1011-1040),
// simplex_bearings (:1042-1053), update_simplex (:1055-1087),
// contract_simplex (:1089-1118), check_tol (:1120-1124, ZEPS 1e-14).
// ---------------------------------------------------------------------
namespace {

enum SxState { SX_INIT, SX_REFLECT, SX_EXPAND, SX_CONTRACT, SX_SHRINK, SX_DONE };

struct Simplex {
  double sx[5][4];
  double fx[5][11];
  double mid[4], line[4], next[4];
  int ihi, ilo, inhi;
  int state;
  int nev;
};

void sx_extremes(Simplex& S) {
  int hi, lo, nhi;
  if (S.fx[0][5] > S.fx[1][5]) {
    hi = 0;
    lo = nhi = 1;
  } else {
    hi = 1;
    lo = nhi = 0;
  }
  for (int i = 2; i < 5; i++) {
    if (S.fx[i][5] <= S.fx[lo][5]) lo = i;
    else if (S.fx[i][5] > S.fx[hi][5]) {
      nhi = hi;
      hi = i;
    } else if (S.fx[i][5] > S.fx[nhi][5]) nhi = i;
  }
  S.ihi = hi;
  S.ilo = lo;
  S.inhi = nhi;
}

// Loop head of amoeba: extremes, bearings, tolerance; returns true when done.
bool sx_head(Simplex& S, double tol, int max_evals) {
  sx_extremes(S);
  for (int j = 0; j < 4; j++) S.mid[j] = 0.0;
  for (int i = 0; i < 5; i++)
    if (i != S.ihi)
      for (int j = 0; j < 4; j++) S.mid[j] += S.sx[i][j];
  for (int j = 0; j < 4; j++) {
    S.mid[j] /= 4;
    S.line[j] = S.sx[S.ihi][j] - S.mid[j];
  }
  const double fmax = S.fx[S.ihi][5], fmin = S.fx[S.ilo][5];
  if (fabs(fmax - fmin) < (fabs(fmax) + fabs(fmin)) * tol + 1e-14) return true;
  if (max_evals > 0 && S.nev >= max_evals) return true;
  return false;
}

void sx_propose(Simplex& S, double scale) {
  for (int j = 0; j < 4; j++) S.next[j] = S.mid[j] + scale * S.line[j];
}

}  // namespace

extern "C" int pa_followup_simplex(pa_followup* f, double* sgnlo, int n, const double* pc2, double tol,
                                   int max_evals, double* out, int* nevals) {
  pa::TraceRange trace_("pa_followup_simplex");
  if (!f || !sgnlo || !pc2 || !out || n < 0) return fu_fail(f, PA_ERR_ARG, "pa_followup_simplex: invalid arguments");
  if (n == 0) return PA_OK;
  std::vector<Simplex> S(n);
  for (int k = 0; k < n; k++) {
    Simplex& s = S[k];
    for (int i = 0; i < 5; i++)
      for (int j = 0; j < 4; j++) s.sx[i][j] = sgnlo[4 * k + j];
    for (int i = 0; i < 4; i++) s.sx[i][i] = s.sx[i][i] + pc2[i];
    s.state = SX_INIT;
    s.nev = 0;
  }
  std::vector<double> pts, res;
  std::vector<std::pair<int, int>> who;  // (point, vertex or -1 for next)
  double total_ms = 0.;
  int rc = PA_OK;
  for (;;) {
    pts.clear();
    who.clear();
    for (int k = 0; k < n; k++) {
      Simplex& s = S[k];
      if (s.state == SX_DONE) continue;
      if (s.state == SX_INIT) {
        for (int i = 0; i < 5; i++) {
          pts.insert(pts.end(), s.sx[i], s.sx[i] + 4);
          who.push_back({k, i});
        }
      } else if (s.state == SX_SHRINK) {
        for (int i = 0; i < 5; i++)
          if (i != s.ilo) {
            pts.insert(pts.end(), s.sx[i], s.sx[i] + 4);
            who.push_back({k, i});
          }
      } else {
        pts.insert(pts.end(), s.next, s.next + 4);
        who.push_back({k, -1});
      }
    }
    if (who.empty()) break;
    const int m = (int)who.size();
    res.resize((size_t)m * 11);
    if ((rc = pa_fstatnet(f, pts.data(), m, res.data()))) break;
    total_ms += f->last_ms;
    // feed the results back, in the order amoeba() would see them
    size_t r = 0;
    while (r < who.size()) {
      const int k = who[r].first;
      Simplex& s = S[k];
      if (s.state == SX_INIT || s.state == SX_SHRINK) {
        for (; r < who.size() && who[r].first == k; r++) {
          memcpy(s.fx[who[r].second], &res[r * 11], sizeof(double) * 11);
          s.nev++;
        }
        s.state = SX_REFLECT;  // to the loop head
        if (sx_head(s, tol, max_evals)) s.state = SX_DONE;
        else sx_propose(s, -1.0);
        continue;
      }
      const double* f2 = &res[r * 11];
      r++;
      s.nev++;
      const int st = s.state;
      // update_simplex: accept when better than the current worst
      const bool upd = f2[5] < s.fx[s.ihi][5];
      if (upd) {
        for (int j = 0; j < 4; j++) s.sx[s.ihi][j] = s.next[j];
        memcpy(s.fx[s.ihi], f2, sizeof(double) * 11);
      }
      bool head = false;
      if (st == SX_REFLECT) {
        if (s.fx[s.ihi][5] < s.fx[s.ilo][5]) {
          s.state = SX_EXPAND;
          sx_propose(s, -2.0);
        } else if (s.fx[s.ihi][5] > s.fx[s.inhi][5]) {
          s.state = SX_CONTRACT;
          sx_propose(s, 0.5);
        } else {
          head = true;
        }
      } else if (st == SX_EXPAND) {
        head = true;
      } else if (st == SX_CONTRACT) {
        if (upd) {
          head = true;
        } else {
          for (int i = 0; i < 5; i++)
            if (i != s.ilo)
              for (int j = 0; j < 4; j++) s.sx[i][j] = (s.sx[s.ilo][j] + s.sx[i][j]) * 0.5;
          s.state = SX_SHRINK;
        }
      }
      if (head) {
        s.state = SX_REFLECT;
        if (sx_head(s, tol, max_evals)) s.state = SX_DONE;
        else sx_propose(s, -1.0);
      }
    }
  }
  f->last_ms = total_ms;
  if (rc) return rc;
  for (int k = 0; k < n; k++) {
    const Simplex& s = S[k];
    for (int j = 0; j < 4; j++) sgnlo[4 * k + j] = s.sx[s.ilo][j];
    memcpy(out + (size_t)11 * k, s.fx[s.ilo], sizeof(double) * 11);
    if (nevals) nevals[k] = s.nev;
  }
  return PA_OK;
}
