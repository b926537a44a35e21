// pa_coinc.cu -- coincidences among the trigger files of several frames on
// the device: read_trigger_files() of coincidences/src/coincidences.c:117-600
// (cells, per-frame duplicate removal, coincidence count, records), plus the
// host-side transformation matrix of manage_grid_matrix (init.c:1142-1210).
//
// Data flow (one stream; arrays in HBM):
//   records [raw][5] f64 (uploaded per frame)
//   k_cells      band/frame-shift/SNR cuts and the 4 integer cells of each
//                record (FP64, no contraction: the reference's expression
//                order), per-block counts, per-column min/max
//   scan + k_inband   ordered compaction of the kept records (read order,
//                frame by frame), with a cell key: the 4 cells as unsigned
//                offsets from the column maxima (descending cells sort
//                ascending), packed to the bits their range needs
//   radix sort   LSD, 8-bit digits, stable: the order of the reference's two
//                qsort()s at once (cells descending; equal cells keep frame
//                then read order, which is what qsort's merge sort leaves)
//   frame ranks  per-block frame histograms + scan locate, for every frame,
//                its last sorted record and the record of an earlier frame
//                that the reference compares it with (the row left over at
//                that position of its candidate table)
//   k_dedup      runs of equal (cells, frame): the reference's highest-SNR
//                state machine per run (coincidences.c:317-413)
//   compaction   survivors in (cells desc, frame) order = the reference's
//                sorted allcandi
//   k_groups     runs of equal cells among survivors: multiplicity, stored
//                or not (coincidences.c:449-486)
//   radix pass   coincidences by multiplicity, descending, stable
//   k_means      FP64 means in the reference's member order (last to first)
//
// No kernel waits on another kernel or on a flag; every index is bounds
// checked against the sizes passed in.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/polgraw_gb300.h"
#include "pa_trace.h"

namespace {

constexpr int kMaxFrames = 255;
constexpr int kT = 256;                 // threads per block everywhere
constexpr int kIt = 8;                  // items per thread (tiles of 2048)
constexpr int kTile = kT * kIt;
constexpr int kRTile = 4096;            // radix tile (items per block)

struct FrameTab {
  int nframes;
  int frame_no[kMaxFrames];
  long long raw_start[kMaxFrames + 1];   // first raw record of each frame
  int blk_start[kMaxFrames + 1];         // first k_cells block of each frame
  long long in_start[kMaxFrames + 1];    // first in-band record of each frame
  int drop[kMaxFrames];                  // 1: the frame's last run is not written
  unsigned long long drop_lo[kMaxFrames], drop_hi[kMaxFrames];  // its cell key
};
__constant__ FrameTab c_ft;

struct CellArgs {
  double lo, hi;           // narrowdown band (pi/2 -+ narrowdown)
  double N, sqrN, omsN;    // coincidences.c:187-188
  double se, ce;           // sin/cos(C_EPSMA)
  double v[4][4];          // vedva / scale (coincidences.c:182-184)
  double half_shift[4];    // 0.5 shift[j]
  int refr;
  double snrcut;
  // FP32 sky terms: copies in float and, per cell column, the bound on
  // |cell value (FP64) - cell value (FP32 sky terms)|
  float omsN_f, se_f, ce_f, v2_f[4], v3_f[4], margin[4];
  // float-float (hi + lo) copies for the frequency and spindown terms
  float Nf, sqrN_h, sqrN_l, v0_h[4], v0_l[4], v1_h[4], v1_l[4], hs_f[4];
  int fast;                // N < 2^24 (exact in float): the FP32/float-float path is on
};

// float-float arithmetic (hi + lo, about 44 significant bits): error-free
// products by fmaf and sums by the two-sum of Knuth
struct FF {
  float h, l;
};
__device__ __forceinline__ FF ff_quick(float a, float b) {
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.h + b.h;
  const float bb = s - a.h;
  const float e = (a.h - (s - bb)) + (b.h - bb);
  return ff_quick(s, e + (a.l + b.l));
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.h * b.h;
  const float e = fmaf(a.h, b.h, -p);
  return ff_quick(p, fmaf(a.h, b.l, fmaf(a.l, b.h, e)));
}
__device__ __forceinline__ FF ff_of(double d) {
  const float h = (float)d;
  return {h, (float)(d - (double)h)};
}

struct KeyLayout {
  int maxc[4];             // column maxima
  int shift[4];            // bit position of each column's field
  int bits;                // total key bits
};

__device__ __forceinline__ int frame_of_block(int b) {
  int lo = 0, hi = c_ft.nframes;  // blk_start[lo] <= b < blk_start[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (c_ft.blk_start[mid] <= b) lo = mid; else hi = mid;
  }
  return lo;
}

// frame of in-band record v: the last frame whose first in-band record is
// <= v (empty frames share their successor's start); s_in = in_start in
// shared memory
__device__ __forceinline__ int frame_of_in(unsigned v, const unsigned* s_in, int nf) {
  int lo = 0, hi = nf;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (s_in[mid] <= v) lo = mid; else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void load_in_start(unsigned* s_in) {
  for (int k = threadIdx.x; k <= c_ft.nframes; k += blockDim.x) s_in[k] = (unsigned)c_ft.in_start[k];
  __syncthreads();
}

// coincidences.c:229-270 for one record in FP64, the reference's expression
// order without contraction; the cells of the kept record in *cl
__device__ __noinline__ void cells_f64(double c0s, double c1, double c2, double c3, const CellArgs& a, int4* cl) {
  double t[4];
  t[0] = __dmul_rn(c0s, a.N);
  t[1] = __dmul_rn(c1, a.sqrN);
  double sa, ca, sd, cd;
  sincos(c3, &sa, &ca);
  sincos(c2, &sd, &cd);
  const double be0 = __dadd_rn(__dmul_rn(__dmul_rn(a.ce, sa), cd), __dmul_rn(a.se, sd));
  const double be1 = __dmul_rn(ca, cd);
  t[2] = __dmul_rn(a.omsN, be0);
  t[3] = __dmul_rn(a.omsN, be1);
  int c[4];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    double s = __dmul_rn(t[0], a.v[0][j]);
    s = __dadd_rn(s, __dmul_rn(t[1], a.v[1][j]));
    s = __dadd_rn(s, __dmul_rn(t[2], a.v[2][j]));
    s = __dadd_rn(s, __dmul_rn(t[3], a.v[3][j]));
    s = __dadd_rn(s, a.half_shift[j]);
    c[j] = (int)round(s);
  }
  *cl = make_int4(c[0], c[1], c[2], c[3]);
}

// Returns 1 when the record is kept.  GB300 runs FP64 at 1/64 of the FP32
// rate, so only the frequency shift and the band/SNR tests (which must equal
// the reference's comparisons) run in FP64; the cell values are first formed
// with the frequency/spindown terms in float-float (about 44 bits) and the
// sky terms (two sincos, be0/be1 of ast2lin, auxi.c:34-35) in FP32.  Each
// column's value then lies within a.margin[j] + |value| 2^-36 of the FP64
// value (FP32 sincosf on |x| <= 8 with the argument rounded to float: <= 3.6e-7
// per sin/cos; the margin allows 8e-6 on be0 and be1).  When every column's
// fractional part is farther than that from 1/2, both round to the same
// integer; otherwise (or for |value| >= 2^22, or |delta|, |alpha| > 8) the
// record is recomputed in FP64.  The cells are therefore those of the FP64
// evaluation.
__device__ __forceinline__ int cell_of(const double* __restrict__ r, double fshift, const CellArgs& a,
                                      int4* cl, unsigned* nexact) {
  const double c0 = r[0], c1 = r[1], c2 = r[2], c3 = r[3], c4 = r[4];
  if (!((c0 > a.lo) && (c0 < a.hi))) return 0;
  const double c0s = __dadd_rn(c0, __dmul_rn(__dmul_rn(__dmul_rn(2., c1), a.N), fshift));
  if (!(((c0s > 0) && (c0s < M_PI)) && (c4 > a.snrcut))) return 0;
  const float x3 = (float)c3, x2 = (float)c2;
  bool exact = !a.fast || !(fabsf(x3) <= 8.f && fabsf(x2) <= 8.f);
  int c[4];
  if (!exact) {
    const FF t0 = ff_mul(ff_of(c0s), FF{a.Nf, 0.f});
    const FF t1 = ff_mul(ff_of(c1), FF{a.sqrN_h, a.sqrN_l});
    float sa, ca, sd, cd;
    sincosf(x3, &sa, &ca);
    sincosf(x2, &sd, &cd);
    const float be0 = fmaf(a.ce_f * sa, cd, a.se_f * sd);
    const float be1 = ca * cd;
    const float t2 = a.omsN_f * be0, t3 = a.omsN_f * be1;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      FF v = ff_add(ff_mul(t0, FF{a.v0_h[j], a.v0_l[j]}), ff_mul(t1, FF{a.v1_h[j], a.v1_l[j]}));
      v = ff_add(v, FF{a.hs_f[j], 0.f});
      v = ff_add(v, FF{fmaf(t2, a.v2_f[j], t3 * a.v3_f[j]), 0.f});
      float fl = floorf(v.h);
      float fr = (v.h - fl) + v.l;
      if (fr < 0.f) {
        fl -= 1.f;
        fr += 1.f;
      } else if (fr >= 1.f) {
        fl += 1.f;
        fr -= 1.f;
      }
      // float-float rounding: below 2^-40 of the terms' magnitudes
      const float av = fabsf(v.h);
      const float terms = fabsf(t0.h * a.v0_h[j]) + fabsf(t1.h * a.v1_h[j]) + av;
      exact |= !(av < 4194304.f) || fabsf(fr - 0.5f) <= a.margin[j] + terms * 1e-11f;
      c[j] = (int)fl + (fr > 0.5f ? 1 : 0);
    }
  }
  if (exact) {
    cells_f64(c0s, c1, c2, c3, a, cl);
    atomicAdd(nexact, 1u);
    return 1;
  }
  *cl = make_int4(c[0], c[1], c[2], c[3]);
  return 1;
}

__device__ __forceinline__ unsigned block_sum(unsigned v, unsigned* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  unsigned t = 0;
  for (int k = 0; k < kT / 32; k++) t += sh[k];
  return t;
}

// exclusive prefix of a 0/1 flag over the block (thread order); returns the
// thread's offset, *total the block's count
__device__ __forceinline__ unsigned block_flag_prefix(int flag, unsigned* sh, unsigned* total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, flag);
  const unsigned in_warp = __popc(bal & ((1u << lane) - 1u));
  __syncthreads();
  if (lane == 0) sh[w] = __popc(bal);
  __syncthreads();
  unsigned before = 0, tot = 0;
  for (int k = 0; k < kT / 32; k++) {
    const unsigned c = sh[k];
    if (k < w) before += c;
    tot += c;
  }
  *total = tot;
  return before + in_warp;
}

// ---- cells of every raw record ------------------------------------------

__global__ void __launch_bounds__(kT) k_cells(const double* __restrict__ rec, CellArgs a,
                                              int4* __restrict__ cells_raw, uint8_t* __restrict__ flag,
                                              unsigned* __restrict__ blk_cnt, int* __restrict__ minmax,
                                              unsigned* __restrict__ nexact, double* __restrict__ snr_raw) {
  __shared__ unsigned sh[kT / 32];
  __shared__ int smm[8];
  const int b = blockIdx.x;
  const int f = frame_of_block(b);
  const long long fend = c_ft.raw_start[f + 1];
  const long long tile0 = c_ft.raw_start[f] + (long long)(b - c_ft.blk_start[f]) * kTile;
  const double fshift = (double)(a.refr - c_ft.frame_no[f]);
  if (threadIdx.x < 4) smm[threadIdx.x] = INT_MAX;
  else if (threadIdx.x < 8) smm[threadIdx.x] = INT_MIN;
  __syncthreads();
  unsigned cnt = 0;
  int mn[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX}, mx[4] = {INT_MIN, INT_MIN, INT_MIN, INT_MIN};
  for (int it = 0; it < kIt; it++) {
    const long long r = tile0 + (long long)it * kT + threadIdx.x;
    if (r >= fend) break;
    int4 cl = make_int4(0, 0, 0, 0);
    const int ok = cell_of(rec + 5 * r, fshift, a, &cl, nexact);
    flag[r] = (uint8_t)ok;
    cells_raw[r] = cl;
    snr_raw[r] = rec[5 * r + 4];
    if (ok) {
      cnt++;
      mn[0] = min(mn[0], cl.x); mx[0] = max(mx[0], cl.x);
      mn[1] = min(mn[1], cl.y); mx[1] = max(mx[1], cl.y);
      mn[2] = min(mn[2], cl.z); mx[2] = max(mx[2], cl.z);
      mn[3] = min(mn[3], cl.w); mx[3] = max(mx[3], cl.w);
    }
  }
  const unsigned tot = block_sum(cnt, sh);
  if (threadIdx.x == 0) blk_cnt[b] = tot;
  if (cnt) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      atomicMin(&smm[j], mn[j]);
      atomicMax(&smm[4 + j], mx[j]);
    }
  }
  __syncthreads();
  if (tot && threadIdx.x < 4) {
    atomicMin(&minmax[threadIdx.x], smm[threadIdx.x]);
    atomicMax(&minmax[4 + threadIdx.x], smm[4 + threadIdx.x]);
  }
}

template <typename K>
__device__ __forceinline__ K make_key(int4 c, const KeyLayout& L);

template <>
__device__ __forceinline__ unsigned long long make_key<unsigned long long>(int4 c, const KeyLayout& L) {
  const int cc[4] = {c.x, c.y, c.z, c.w};
  unsigned long long k = 0;
#pragma unroll
  for (int j = 0; j < 4; j++)
    k |= (unsigned long long)(unsigned)(L.maxc[j] - cc[j]) << L.shift[j];
  return k;
}

struct U128 {
  unsigned long long lo, hi;
};
__device__ __forceinline__ bool operator==(const U128& a, const U128& b) { return a.lo == b.lo && a.hi == b.hi; }

template <>
__device__ __forceinline__ U128 make_key<U128>(int4 c, const KeyLayout& L) {
  // one 32-bit field per column: (maxc - c) < 2^32 always
  U128 k;
  k.hi = ((unsigned long long)(unsigned)(L.maxc[0] - c.x) << 32) | (unsigned)(L.maxc[1] - c.y);
  k.lo = ((unsigned long long)(unsigned)(L.maxc[2] - c.z) << 32) | (unsigned)(L.maxc[3] - c.w);
  return k;
}

__device__ __forceinline__ unsigned digit_of(unsigned long long k, int shift) { return (unsigned)(k >> shift) & 255u; }
__device__ __forceinline__ unsigned digit_of(const U128& k, int shift) {
  return shift < 64 ? (unsigned)(k.lo >> shift) & 255u : (unsigned)(k.hi >> (shift - 64)) & 255u;
}
__device__ __forceinline__ bool key_is(unsigned long long k, unsigned long long lo, unsigned long long hi) {
  return k == lo && hi == 0;
}
__device__ __forceinline__ bool key_is(const U128& k, unsigned long long lo, unsigned long long hi) {
  return k.lo == lo && k.hi == hi;
}
__device__ __forceinline__ void key_split(unsigned long long k, unsigned long long* lo, unsigned long long* hi) {
  *lo = k;
  *hi = 0;
}
__device__ __forceinline__ void key_split(const U128& k, unsigned long long* lo, unsigned long long* hi) {
  *lo = k.lo;
  *hi = k.hi;
}

// ordered compaction of the kept records, with their keys
template <typename K>
__global__ void __launch_bounds__(kT) k_inband(const uint8_t* __restrict__ flag, const int4* __restrict__ cells_raw,
                                               const unsigned* __restrict__ blk_off, KeyLayout L,
                                               unsigned* __restrict__ rawidx, int4* __restrict__ cells_in,
                                               K* __restrict__ key, unsigned* __restrict__ val,
                                               const double* __restrict__ snr_raw, double* __restrict__ snr_in) {
  __shared__ unsigned sh[kT / 32];
  const int b = blockIdx.x;
  const int f = frame_of_block(b);
  const long long fend = c_ft.raw_start[f + 1];
  const long long tile0 = c_ft.raw_start[f] + (long long)(b - c_ft.blk_start[f]) * kTile;
  unsigned base = blk_off[b];
  for (int it = 0; it < kIt; it++) {
    const long long r = tile0 + (long long)it * kT + threadIdx.x;
    // every thread takes part in the prefix (bounds folded into the flag)
    const int ok = (r < fend) ? flag[r] : 0;
    unsigned tot;
    const unsigned pre = block_flag_prefix(ok, sh, &tot);
    if (ok) {
      const unsigned o = base + pre;
      const int4 cl = cells_raw[r];
      rawidx[o] = (unsigned)r;
      cells_in[o] = cl;
      key[o] = make_key<K>(cl, L);
      val[o] = o;
      snr_in[o] = snr_raw[r];
    }
    base += tot;
  }
}

// ---- scan (exclusive, in place) ------------------------------------------

__global__ void __launch_bounds__(kT) k_scan_tiles(unsigned* __restrict__ d, long long n, unsigned* __restrict__ sums) {
  __shared__ unsigned sh[kT];
  const long long t0 = (long long)blockIdx.x * kTile + (long long)threadIdx.x * kIt;
  unsigned v[kIt], s = 0;
#pragma unroll
  for (int k = 0; k < kIt; k++) {
    v[k] = (t0 + k < n) ? d[t0 + k] : 0u;
    s += v[k];
  }
  // block exclusive scan of the thread sums
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned x = s;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned acc = 0;
    for (int k = 0; k < kT / 32; k++) {
      const unsigned c = sh[k];
      sh[k] = acc;
      acc += c;
    }
    sh[kT / 32] = acc;
  }
  __syncthreads();
  unsigned run = sh[w] + x - s;
  if (threadIdx.x == kT - 1 && sums) sums[blockIdx.x] = sh[kT / 32];
#pragma unroll
  for (int k = 0; k < kIt; k++) {
    if (t0 + k < n) d[t0 + k] = run;
    run += v[k];
  }
}

__global__ void __launch_bounds__(kT) k_scan_add(unsigned* __restrict__ d, long long n, const unsigned* __restrict__ sums) {
  const unsigned add = sums[blockIdx.x];
  const long long t0 = (long long)blockIdx.x * kTile;
  for (int k = threadIdx.x; k < kTile; k += kT)
    if (t0 + k < n) d[t0 + k] += add;
}

// ---- radix sort (LSD, 8-bit digits, stable) ------------------------------

template <typename K>
__global__ void __launch_bounds__(kT) k_radix_hist(const K* __restrict__ key, long long n, int shift, int nblk,
                                                   unsigned* __restrict__ hist, unsigned* __restrict__ cnt_local) {
  __shared__ unsigned h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const long long t0 = (long long)blockIdx.x * kRTile;
  for (int k = threadIdx.x; k < kRTile; k += kT) {
    const long long i = t0 + k;
    if (i < n) atomicAdd(&h[digit_of(key[i], shift)], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
  cnt_local[(long long)blockIdx.x * 256 + threadIdx.x] = h[threadIdx.x];
}

// digit = frame of the element (for the per-frame ranks of the sorted order)
__global__ void __launch_bounds__(kT) k_frame_hist(const unsigned* __restrict__ val, long long n, int nblk,
                                                   unsigned* __restrict__ hist) {
  __shared__ unsigned h[256];
  __shared__ unsigned s_in[kMaxFrames + 1];
  h[threadIdx.x] = 0;
  load_in_start(s_in);
  const int nf = c_ft.nframes;
  const long long t0 = (long long)blockIdx.x * kRTile;
  for (int k = threadIdx.x; k < kRTile; k += kT) {
    const long long i = t0 + k;
    if (i < n) atomicAdd(&h[frame_of_in(val[i], s_in, nf)], 1u);
  }
  __syncthreads();
  hist[(long long)threadIdx.x * nblk + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter of one 8-bit digit.  A tile of kRTile items is ranked in
// chunks of kT x kSub items (item j*kT + t of a chunk held by thread t):
// peers with the same digit in the warp (match_any), then an exclusive prefix
// per digit over the (item slot, warp) pairs in item order, carried across
// chunks.  Each item is staged in shared memory at its digit's place in the
// tile (tile base from the tile's own digit counts), and the tile is then
// written out digit run by digit run, so that consecutive threads store to
// consecutive addresses.
constexpr int kSub = 2;
constexpr int kChunk = kT * kSub;
constexpr int kSlots = kSub * (kT / 32);

template <typename K>
constexpr size_t scatter_smem() {
  return (size_t)kRTile * (sizeof(K) + sizeof(unsigned) + 1) + sizeof(unsigned) * 256 * (kSlots + 3);
}

__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned* scr) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) scr[w] = x;
  __syncthreads();
  unsigned before = 0;
  for (int k = 0; k < w; k++) before += scr[k];
  __syncthreads();
  return before + x - v;
}

template <typename K>
__global__ void __launch_bounds__(kT) k_radix_scatter(const K* __restrict__ kin, const unsigned* __restrict__ vin,
                                                      K* __restrict__ kout, unsigned* __restrict__ vout, long long n,
                                                      int shift, int nblk, const unsigned* __restrict__ off,
                                                      const unsigned* __restrict__ cnt_local) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ unsigned scr[kT / 32];
  K* st_k = (K*)smem;
  unsigned* st_v = (unsigned*)(st_k + kRTile);
  unsigned* wc = st_v + kRTile;              // [kSlots][256]
  unsigned* run = wc + kSlots * 256;
  unsigned* base = run + 256;
  unsigned* goff = base + 256;
  uint8_t* st_d = (uint8_t*)(goff + 256);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long long t0 = (long long)blockIdx.x * kRTile;
  const long long rem = n - t0;
  const int tn = rem < kRTile ? (int)rem : kRTile;
  const unsigned bt = block_excl_scan(cnt_local[(long long)blockIdx.x * 256 + threadIdx.x], scr);
  base[threadIdx.x] = bt;
  goff[threadIdx.x] = off[(long long)threadIdx.x * nblk + blockIdx.x];
  run[threadIdx.x] = 0;
  // the thread's items of the whole tile, loaded together
  constexpr int kCh = kRTile / kChunk;
  K kk[kCh][kSub];
  unsigned vv[kCh][kSub];
#pragma unroll
  for (int c = 0; c < kCh; c++)
#pragma unroll
    for (int j = 0; j < kSub; j++) {
      const int li = c * kChunk + j * kT + threadIdx.x;
      vv[c][j] = 0;
      if (li < tn) {
        kk[c][j] = kin[t0 + li];
        vv[c][j] = vin[t0 + li];
      }
    }
#pragma unroll
  for (int c = 0; c < kCh; c++) {
    unsigned d[kSub], rank[kSub];
#pragma unroll
    for (int j = 0; j < kSub; j++) {
      const int li = c * kChunk + j * kT + threadIdx.x;
      d[j] = li < tn ? digit_of(kk[c][j], shift) : 256u;
    }
    for (int k = 0; k < kSlots; k++) wc[k * 256 + threadIdx.x] = 0;
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSub; j++) {
      const unsigned peers = __match_any_sync(0xffffffffu, d[j]);
      rank[j] = __popc(peers & ((1u << lane) - 1u));
      if (d[j] < 256 && lane == __ffs(peers) - 1) wc[(j * (kT / 32) + w) * 256 + d[j]] = __popc(peers);
    }
    __syncthreads();
    {
      const int dg = threadIdx.x;
      unsigned p = run[dg];
      for (int k = 0; k < kSlots; k++) {
        const unsigned t = wc[k * 256 + dg];
        wc[k * 256 + dg] = p;
        p += t;
      }
      run[dg] = p;
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSub; j++)
      if (d[j] < 256) {
        const unsigned lp = base[d[j]] + wc[(j * (kT / 32) + w) * 256 + d[j]] + rank[j];
        st_k[lp] = kk[c][j];
        st_v[lp] = vv[c][j];
        st_d[lp] = (uint8_t)d[j];
      }
    __syncthreads();
  }
  for (int q = threadIdx.x; q < tn; q += kT) {
    const unsigned dq = st_d[q];
    const unsigned g = goff[dq] + ((unsigned)q - base[dq]);
    kout[g] = st_k[q];
    vout[g] = st_v[q];
  }
}

// ---- per-frame ranks: element p of frame g in sorted order -----------------

// req[r] = {frame, rank}; out[r] = sorted position (-1 if absent), with the
// element's cells and key.  One warp per request: binary search over the
// frame's block offsets, then a count through the block's tile.
template <typename K>
__global__ void k_frame_find(const int2* __restrict__ req, int nreq, const unsigned* __restrict__ hoff, int nblk,
                             const unsigned* __restrict__ val, long long n,
                             const K* __restrict__ key, const int4* __restrict__ cells_in,
                             long long* __restrict__ out, int4* __restrict__ out_cells,
                             unsigned long long* __restrict__ out_key) {
  __shared__ unsigned s_in[kMaxFrames + 1];
  load_in_start(s_in);
  const int nf = c_ft.nframes;
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nreq) return;
  const int g = req[r].x, p = req[r].y;
  const unsigned* o = hoff + (long long)g * nblk;
  const unsigned base = o[0];
  // last block b with o[b] - base <= p
  int lo = 0, hi = nblk;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (o[mid] - base <= (unsigned)p) lo = mid; else hi = mid;
  }
  unsigned need = (unsigned)p - (o[lo] - base);
  long long found = -1;
  const long long t0 = (long long)lo * kRTile;
  for (int k = 0; k < kRTile; k += 32) {
    const long long i = t0 + k + lane;
    const int hit = (i < n) && (frame_of_in(val[i], s_in, nf) == g);
    const unsigned bal = __ballot_sync(0xffffffffu, hit);
    const unsigned c = __popc(bal);
    if (need < c) {
      // the (need)-th set lane
      unsigned m = bal;
      for (unsigned q = 0; q < need; q++) m &= m - 1;
      found = t0 + k + (__ffs(m) - 1);
      break;
    }
    need -= c;
  }
  if (lane == 0) {
    out[r] = found;
    if (found >= 0) {
      out_cells[r] = cells_in[val[found]];
      key_split(key[found], &out_key[2 * r], &out_key[2 * r + 1]);
    }
  }
}

// ---- duplicate removal per (cells, frame) run ------------------------------

template <typename K>
__global__ void __launch_bounds__(kT) k_dedup(const K* __restrict__ key, const unsigned* __restrict__ val,
                                              const double* __restrict__ snr_in, long long n,
                                              uint8_t* __restrict__ keep, unsigned* __restrict__ uniq) {
  __shared__ unsigned hcount[256];
  __shared__ unsigned s_in[kMaxFrames + 1];
  hcount[threadIdx.x] = 0;
  load_in_start(s_in);
  const int nf = c_ft.nframes;
  const long long i = (long long)blockIdx.x * kT + threadIdx.x;
  if (i < n) {
    const K k0 = key[i];
    const unsigned v0 = val[i];
    const int f = frame_of_in(v0, s_in, nf);
    // the previous record's frame matters only when its cells are equal
    const bool start = (i == 0) || !(key[i - 1] == k0) || frame_of_in(val[i - 1], s_in, nf) != f;
    uint8_t kept = 0;
    if (start) {
      const long long fs = s_in[f];
      // walk the run [i, j]
      long long j = i;
      while (j + 1 < n && key[j + 1] == k0 && frame_of_in(val[j + 1], s_in, nf) == f) j++;
      // coincidences.c:317-413 over the pairs (t, t + 1) of the run
      long long maxsnridx = 0, maxi = i;
      double candsnr = 0;
      unsigned vt = v0;
      double s0 = j > i ? snr_in[vt] : 0.;
      for (long long t = i; t < j; t++) {
        const unsigned vt1 = val[t + 1];
        const double s1 = snr_in[vt1];
        const long long idx = (long long)vt - fs, idx1 = (long long)vt1 - fs;
        if (!maxsnridx) {
          maxsnridx = (s0 > s1) ? idx : idx1;
          maxi = (s0 > s1) ? t : t + 1;
          candsnr = (s0 > s1) ? s0 : s1;
        } else {
          if (s0 > candsnr) {
            maxsnridx = idx; maxi = t; candsnr = s0;
          } else if (s1 > candsnr) {
            maxsnridx = idx1; maxi = t + 1; candsnr = s1;
          }
        }
        vt = vt1;
        s0 = s1;
      }
      const bool dropped = c_ft.drop[f] && key_is(k0, c_ft.drop_lo[f], c_ft.drop_hi[f]);
      if (!dropped) {
        keep[maxsnridx ? maxi : j] = 1;
        kept = 1;
      }
    }
    if (kept) atomicAdd(&hcount[f], 1u);
  }
  __syncthreads();
  if (hcount[threadIdx.x]) atomicAdd(&uniq[threadIdx.x], hcount[threadIdx.x]);
}

// keep flags by in-band index, from the flags by sorted position
__global__ void k_keep_scatter(const uint8_t* __restrict__ keep, const unsigned* __restrict__ val, long long n,
                               uint8_t* __restrict__ keep_in) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) keep_in[val[i]] = keep[i];
}

// per-tile counts of a 0/1 array
__global__ void __launch_bounds__(kT) k_tile_count(const uint8_t* __restrict__ flag, long long n, unsigned* __restrict__ cnt) {
  __shared__ unsigned sh[kT / 32];
  const long long t0 = (long long)blockIdx.x * kTile;
  unsigned c = 0;
  for (int k = 0; k < kIt; k++) {
    const long long i = t0 + (long long)k * kT + threadIdx.x;
    if (i < n) c += flag[i];
  }
  const unsigned tot = block_sum(c, sh);
  if (threadIdx.x == 0) cnt[blockIdx.x] = tot;
}

// survivors in sorted order: key and in-band index
template <typename K>
__global__ void __launch_bounds__(kT) k_compact_surv(const uint8_t* __restrict__ keep, long long n,
                                                     const unsigned* __restrict__ off, const K* __restrict__ key,
                                                     const unsigned* __restrict__ val, K* __restrict__ skey,
                                                     unsigned* __restrict__ sval) {
  __shared__ unsigned sh[kT / 32];
  const long long t0 = (long long)blockIdx.x * kTile;
  unsigned base = off[blockIdx.x];
  for (int k = 0; k < kIt; k++) {
    const long long i = t0 + (long long)k * kT + threadIdx.x;
    const int ok = (i < n) ? keep[i] : 0;
    unsigned tot;
    const unsigned pre = block_flag_prefix(ok, sh, &tot);
    if (ok) {
      skey[base + pre] = key[i];
      sval[base + pre] = val[i];
    }
    base += tot;
  }
}

// runs of equal cells among the survivors (coincidences.c:449-486)
template <typename K>
__global__ void __launch_bounds__(kT) k_groups(const K* __restrict__ skey, long long G, int mincoin,
                                               uint8_t* __restrict__ gflag, unsigned* __restrict__ gend,
                                               unsigned* __restrict__ gw, int* __restrict__ last_unstored) {
  const long long i = (long long)blockIdx.x * kT + threadIdx.x;
  if (i >= G) return;
  const K k0 = skey[i];
  uint8_t fl = 0;
  if (i == 0 || !(skey[i - 1] == k0)) {
    long long j = i;
    while (j + 1 < G && skey[j + 1] == k0) j++;
    const long long w = j - i + 1;
    if (w >= mincoin) {
      if (j < G - 1) {
        fl = 1;
        gend[i] = (unsigned)j;
        gw[i] = (unsigned)w;
      } else {
        *last_unstored = 1;
      }
    }
  }
  gflag[i] = fl;
}

__global__ void __launch_bounds__(kT) k_compact_groups(const uint8_t* __restrict__ gflag, long long G,
                                                       const unsigned* __restrict__ off,
                                                       const unsigned* __restrict__ gend, const unsigned* __restrict__ gw,
                                                       unsigned long long* __restrict__ wkey,
                                                       unsigned* __restrict__ cend, unsigned* __restrict__ cw,
                                                       unsigned* __restrict__ cidx) {
  __shared__ unsigned sh[kT / 32];
  const long long t0 = (long long)blockIdx.x * kTile;
  unsigned base = off[blockIdx.x];
  for (int k = 0; k < kIt; k++) {
    const long long i = t0 + (long long)k * kT + threadIdx.x;
    const int ok = (i < G) ? gflag[i] : 0;
    unsigned tot;
    const unsigned pre = block_flag_prefix(ok, sh, &tot);
    if (ok) {
      const unsigned o = base + pre;
      cend[o] = gend[i];
      cw[o] = gw[i];
      wkey[o] = 255ull - gw[i];   // multiplicity <= frames <= 255: one digit
      cidx[o] = o;
    }
    base += tot;
  }
}

__global__ void k_gather_w(const unsigned* __restrict__ order, const unsigned* __restrict__ cw, int K,
                           unsigned* __restrict__ w_sorted) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < K) w_sorted[q] = cw[order[q]];
}

// coincidences.c:488-525: means over the members k = end, end - 1, ...
__global__ void k_means(const unsigned* __restrict__ order, const unsigned* __restrict__ cend,
                        const unsigned* __restrict__ cw, const unsigned* __restrict__ first, int K,
                        const unsigned* __restrict__ sval, const unsigned* __restrict__ rawidx,
                        const double* __restrict__ rec, double N, int refr,
                        pa_coinc_rec* __restrict__ out, int* __restrict__ fra, int* __restrict__ ops) {
  __shared__ unsigned s_in[kMaxFrames + 1];
  load_in_start(s_in);
  const int nf = c_ft.nframes;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= K) return;
  const unsigned g = order[q];
  const long long j = cend[g];
  const int w = (int)cw[g];
  const long long m0 = first[q];
  double m[5] = {0, 0, 0, 0, 0};
  for (int i = 0; i < w; i++) {
    const unsigned v = sval[j - i];
    const int f = frame_of_in(v, s_in, nf);
    const long long r = rawidx[v];
    const double* c = rec + 5 * r;
    const double fshift = (double)(refr - c_ft.frame_no[f]);
    const double c0s = __dadd_rn(c[0], __dmul_rn(__dmul_rn(__dmul_rn(2., c[1]), N), fshift));
    m[0] = __dadd_rn(m[0], c0s);
    m[1] = __dadd_rn(m[1], c[1]);
    m[2] = __dadd_rn(m[2], c[2]);
    m[3] = __dadd_rn(m[3], c[3]);
    m[4] = __dadd_rn(m[4], __dmul_rn(c[4], c[4]));
    ops[m0 + i] = (int)(r - c_ft.raw_start[f]);
    fra[m0 + i] = c_ft.frame_no[f];
  }
  const double dw = (double)w;
  pa_coinc_rec r;
  r.w = w;
  r.first = (int)m0;
  for (int l = 0; l < 4; l++) r.mean[l] = __ddiv_rn(m[l], dw);
  r.mean[4] = __dsqrt_rn(m[4]);
  out[q] = r;
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct pa_coinc {
  pa_coinc_cfg cfg;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;
  long long launches = 0;
  double last_ms = 0;
  FrameTab ft;
  std::vector<int> frames;
  std::vector<long long> raw_start;   // per frame, size nframes + 1
  long long nraw = 0;
  // device buffers (grow only)
  struct Buf {
    void* p = nullptr;
    size_t n = 0;
  };
  Buf rec, cells_raw, flag, snr_raw, blkcnt, scan_tmp, minmax, rawidx, cells_in, snr_in, cntl, keyA, keyB, valA, valB, hist,
      keep, keep_in, uniq, req, found, skey, sval, gflag, gend, gw, lastu, wkeyA, wkeyB, cend, cw, cidxA, cidxB,
      wsort, means, fra, ops;
  // optional per-kernel profile: events around each launch while on
  bool prof_on = false;
  struct Open {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Open> prof_open;
  double prof_ms[16] = {0};
  long long prof_n[16] = {0};
  // results
  pa_coinc_summary sum;
  std::vector<int> frameinfo;
  // results in page-locked host memory (grow only)
  pa_coinc_rec* h_recs = nullptr;
  int* h_fra = nullptr;
  int* h_ops = nullptr;
  size_t h_recs_cap = 0, h_mem_cap = 0;
  long long n_in = 0;
  const unsigned* val_sorted = nullptr;  // in-band index of each sorted position (last run)
  bool ev1_done = false;                 // the run's end event is already on the stream
};

thread_local std::string g_coinc_create_error;  // per host thread, as the other create errors

enum CoincKind { CK_CELLS = 0, CK_INBAND, CK_SORT_HIST, CK_SORT_SCATTER, CK_SCAN, CK_FRAME_RANK, CK_DEDUP,
                 CK_COMPACT, CK_GROUPS, CK_MEANS, CK_COUNT };
static const char* const kCoincKindName[CK_COUNT] = {
    "coinc_cells", "coinc_inband", "coinc_sort_hist", "coinc_sort_scatter", "coinc_scan",
    "coinc_frame_rank", "coinc_dedup", "coinc_compact", "coinc_groups", "coinc_means"};

// CUDA events around the launches of its scope, when profiling is on
struct Span {
  pa_coinc* c;
  int kind;
  cudaEvent_t a = nullptr, b = nullptr;
  Span(pa_coinc* c_, int k) : c(c_), kind(k) {
    if (c->prof_on && cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess)
      cudaEventRecord(a, c->stream);
  }
  ~Span() {
    if (a && b) {
      cudaEventRecord(b, c->stream);
      c->prof_open.push_back({kind, a, b});
    }
  }
};

static void prof_collect(pa_coinc* c) {
  for (auto& o : c->prof_open) {
    float ms = 0;
    if (cudaEventSynchronize(o.b) == cudaSuccess && cudaEventElapsedTime(&ms, o.a, o.b) == cudaSuccess) {
      c->prof_ms[o.kind] += ms;
      c->prof_n[o.kind]++;
    }
    cudaEventDestroy(o.a);
    cudaEventDestroy(o.b);
  }
  c->prof_open.clear();
}

static int cfail(pa_coinc* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  if (c) c->err = buf; else g_coinc_create_error = buf;
  return code;
}

#define CCK(call, what)                                                                  \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return cfail(c, PA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e_)); \
  } while (0)

static int ensure(pa_coinc* c, pa_coinc::Buf& b, size_t bytes) {
  if (bytes <= b.n && b.p) return PA_OK;
  size_t nb = bytes < 256 ? 256 : bytes;
  if (b.n) nb = nb > b.n + b.n / 2 ? nb : b.n + b.n / 2;
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, nb);
  if (e != cudaSuccess) return cfail(c, PA_ERR_NOMEM, "cudaMalloc(%zu): %s", nb, cudaGetErrorString(e));
  if (b.p) {
    // work queued on the stream may still read the old buffer
    cudaStreamSynchronize(c->stream);
    cudaFree(b.p);
  }
  b.p = p;
  b.n = nb;
  return PA_OK;
}
#define ENS(buf, bytes)                            \
  do {                                             \
    int rc_ = ensure(c, c->buf, (size_t)(bytes));  \
    if (rc_) return rc_;                           \
  } while (0)

template <typename T>
static T* P(pa_coinc::Buf& b) { return (T*)b.p; }

// exclusive scan of d[0..n) in place; tmp needs room for the block sums of
// every level
static int scan_excl(pa_coinc* c, unsigned* d, long long n, unsigned* tmp) {
  if (n <= 0) return PA_OK;
  const long long nb = (n + kTile - 1) / kTile;
  {
    Span sp_(c, CK_SCAN);
    k_scan_tiles<<<(unsigned)nb, kT, 0, c->stream>>>(d, n, nb > 1 ? tmp : nullptr);
  }
  c->launches++;
  if (nb > 1) {
    int rc = scan_excl(c, tmp, nb, tmp + nb);
    if (rc) return rc;
    {
      Span sp_(c, CK_SCAN);
      k_scan_add<<<(unsigned)nb, kT, 0, c->stream>>>(d, n, tmp);
    }
    c->launches++;
  }
  CCK(cudaGetLastError(), "scan");
  return PA_OK;
}

static long long scan_tmp_len(long long n) {
  long long t = 0;
  while (n > 1) {
    n = (n + kTile - 1) / kTile;
    t += n;
  }
  return t + 1;
}

template <typename K>
static int radix_sort(pa_coinc* c, K*& k, unsigned*& v, K* k2, unsigned* v2, long long n, int bits) {
  pa::TraceRange trace_("coinc radix sort");
  const int nblk = (int)((n + kRTile - 1) / kRTile);
  ENS(hist, sizeof(unsigned) * (256ll * nblk + 1));
  ENS(cntl, sizeof(unsigned) * 256ll * nblk);
  ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(256ll * nblk));
  // the staged scatter needs more than the default 48 KB of shared memory
  CCK(cudaFuncSetAttribute(k_radix_scatter<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)scatter_smem<K>()),
      "cudaFuncSetAttribute");
  K* ka = k;
  unsigned* va = v;
  K* kb = k2;
  unsigned* vb = v2;
  for (int s = 0; s < bits; s += 8) {
    {
      Span sp_(c, CK_SORT_HIST);
      k_radix_hist<K><<<nblk, kT, 0, c->stream>>>(ka, n, s, nblk, P<unsigned>(c->hist), P<unsigned>(c->cntl));
    }
    c->launches++;
    int rc = scan_excl(c, P<unsigned>(c->hist), 256ll * nblk, P<unsigned>(c->scan_tmp));
    if (rc) return rc;
    {
      Span sp_(c, CK_SORT_SCATTER);
      k_radix_scatter<K><<<nblk, kT, scatter_smem<K>(), c->stream>>>(ka, va, kb, vb, n, s, nblk,
                                                                      P<unsigned>(c->hist), P<unsigned>(c->cntl));
    }
    c->launches++;
    CCK(cudaGetLastError(), "radix pass");
    K* tk = ka; ka = kb; kb = tk;
    unsigned* tv = va; va = vb; vb = tv;
  }
  k = ka;
  v = va;
  return PA_OK;
}

extern "C" {

int pa_coinc_vedva(const double* fisher, double* vedva) {
  if (!fisher || !vedva) return PA_ERR_ARG;
  // cyclic Jacobi rotations on a copy (row-major), eigenvectors as columns
  double a[16], v[16];
  memcpy(a, fisher, sizeof(a));
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) v[4 * i + j] = (i == j);
  for (int sweep = 0; sweep < 64; sweep++) {
    double off = 0;
    for (int i = 0; i < 4; i++)
      for (int j = i + 1; j < 4; j++) off += a[4 * i + j] * a[4 * i + j];
    if (off < 1e-300) break;
    for (int p = 0; p < 4; p++)
      for (int q = p + 1; q < 4; q++) {
        const double apq = a[4 * p + q];
        if (apq == 0.0) continue;
        const double theta = (a[4 * q + q] - a[4 * p + p]) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
        for (int k = 0; k < 4; k++) {
          const double akp = a[4 * k + p], akq = a[4 * k + q];
          a[4 * k + p] = cs * akp - sn * akq;
          a[4 * k + q] = sn * akp + cs * akq;
        }
        for (int k = 0; k < 4; k++) {
          const double apk = a[4 * p + k], aqk = a[4 * q + k];
          a[4 * p + k] = cs * apk - sn * aqk;
          a[4 * q + k] = sn * apk + cs * aqk;
        }
        for (int k = 0; k < 4; k++) {
          const double vkp = v[4 * k + p], vkq = v[4 * k + q];
          v[4 * k + p] = cs * vkp - sn * vkq;
          v[4 * k + q] = sn * vkp + cs * vkq;
        }
      }
  }
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) vedva[4 * i + j] = v[4 * i + j] * sqrt(a[4 * j + j]);
  return PA_OK;
}

const char* pa_coinc_last_error(const pa_coinc* c) {
  return c ? c->err.c_str() : g_coinc_create_error.c_str();
}

pa_coinc* pa_coinc_create(const pa_coinc_cfg* cfg, int* status) {
  auto ret = [&](int st) {
    if (status) *status = st;
    return (pa_coinc*)nullptr;
  };
  pa_coinc* c = nullptr;
  if (!cfg || cfg->N < 1 || cfg->mincoin < 2)
    return cfail(c, PA_ERR_ARG, "pa_coinc_create: invalid configuration (N >= 1, mincoin >= 2)"), ret(PA_ERR_ARG);
  for (int j = 0; j < 4; j++)
    if (cfg->scale[j] == 0) return cfail(c, PA_ERR_ARG, "pa_coinc_create: scale digit 0"), ret(PA_ERR_ARG);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1)
    return cfail(c, PA_ERR_NODEV, "pa_coinc_create: no CUDA device"), ret(PA_ERR_NODEV);
  if (cfg->device < 0 || cfg->device >= ndev)
    return cfail(c, PA_ERR_ARG, "pa_coinc_create: device %d out of range", cfg->device), ret(PA_ERR_ARG);
  c = new pa_coinc();
  c->cfg = *cfg;
  cudaError_t e;
  if ((e = cudaSetDevice(cfg->device)) != cudaSuccess ||
      (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
      (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
    g_coinc_create_error = std::string("pa_coinc_create: ") + cudaGetErrorString(e);
    pa_coinc_destroy(c);
    if (status) *status = PA_ERR_CUDA;
    return nullptr;
  }
  pa_coinc_reset(c);
  if (status) *status = PA_OK;
  return c;
}

void pa_coinc_destroy(pa_coinc* c) {
  if (!c) return;
  cudaSetDevice(c->cfg.device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  pa_coinc::Buf* bufs[] = {&c->rec, &c->cells_raw, &c->flag, &c->snr_raw, &c->blkcnt, &c->scan_tmp, &c->minmax, &c->rawidx,
                           &c->cells_in, &c->snr_in, &c->cntl, &c->keyA, &c->keyB, &c->valA, &c->valB, &c->hist, &c->keep,
                           &c->keep_in, &c->uniq, &c->req, &c->found, &c->skey, &c->sval, &c->gflag, &c->gend,
                           &c->gw, &c->lastu, &c->wkeyA, &c->wkeyB, &c->cend, &c->cw, &c->cidxA, &c->cidxB,
                           &c->wsort, &c->means, &c->fra, &c->ops};
  for (auto* b : bufs)
    if (b->p) cudaFree(b->p);
  for (auto& o : c->prof_open) {
    cudaEventDestroy(o.a);
    cudaEventDestroy(o.b);
  }
  if (c->h_recs) cudaFreeHost(c->h_recs);
  if (c->h_fra) cudaFreeHost(c->h_fra);
  if (c->h_ops) cudaFreeHost(c->h_ops);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int pa_coinc_reset(pa_coinc* c) {
  if (!c) return PA_ERR_ARG;
  c->frames.clear();
  c->val_sorted = nullptr;
  c->raw_start.assign(1, 0);
  c->nraw = 0;
  c->n_in = 0;
  memset(&c->sum, 0, sizeof(c->sum));
  c->frameinfo.clear();

  return PA_OK;
}

int pa_coinc_add_frame(pa_coinc* c, int frame, const double* records, long long n) {
  pa::TraceRange trace_("pa_coinc_add_frame");
  if (!c || n < 0 || (n > 0 && !records)) return PA_ERR_ARG;
  if ((int)c->frames.size() >= kMaxFrames) return cfail(c, PA_ERR_ARG, "pa_coinc_add_frame: more than %d frames", kMaxFrames);
  if (c->nraw + n >= (1ll << 31)) return cfail(c, PA_ERR_ARG, "pa_coinc_add_frame: more than 2^31 records");
  CCK(cudaSetDevice(c->cfg.device), "cudaSetDevice");
  const size_t need = sizeof(double) * 5 * (size_t)(c->nraw + n);
  if (need > c->rec.n) {
    // grow keeping the frames already uploaded
    size_t nb = need + need / 2;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, nb);
    if (e != cudaSuccess) return cfail(c, PA_ERR_NOMEM, "cudaMalloc(%zu): %s", nb, cudaGetErrorString(e));
    if (c->rec.p) {
      CCK(cudaMemcpyAsync(p, c->rec.p, sizeof(double) * 5 * (size_t)c->nraw, cudaMemcpyDeviceToDevice, c->stream),
          "cudaMemcpyAsync");
      CCK(cudaStreamSynchronize(c->stream), "sync");
      cudaFree(c->rec.p);
    }
    c->rec.p = p;
    c->rec.n = nb;
  }
  if (n) {
    CCK(cudaMemcpyAsync((double*)c->rec.p + 5 * c->nraw, records, sizeof(double) * 5 * (size_t)n,
                        cudaMemcpyHostToDevice, c->stream),
        "cudaMemcpyAsync");
    // the caller's buffer is free again when the call returns
    CCK(cudaStreamSynchronize(c->stream), "sync");
  }
  c->frames.push_back(frame);
  c->nraw += n;
  c->raw_start.push_back(c->nraw);
  return PA_OK;
}

}  // extern "C"

template <typename K>
static int run_keyed(pa_coinc* c, const KeyLayout& L, int nblk1, std::vector<long long>& nin_f) {
  pa::TraceRange trace_("coinc sort, duplicates, coincidences");
  const int nf = (int)c->frames.size();
  const long long n = c->n_in;
  ENS(snr_in, sizeof(double) * n);
  ENS(keyA, sizeof(K) * n);
  ENS(keyB, sizeof(K) * n);
  ENS(valA, sizeof(unsigned) * n);
  ENS(valB, sizeof(unsigned) * n);
  {
    Span sp_(c, CK_INBAND);
    k_inband<K><<<nblk1, kT, 0, c->stream>>>(P<uint8_t>(c->flag), P<int4>(c->cells_raw), P<unsigned>(c->blkcnt), L,
                                             P<unsigned>(c->rawidx), P<int4>(c->cells_in),
                                             P<K>(c->keyA), P<unsigned>(c->valA), P<double>(c->snr_raw),
                                             P<double>(c->snr_in));
  }
  c->launches++;
  CCK(cudaGetLastError(), "k_inband");
  K* key = P<K>(c->keyA);
  unsigned* val = P<unsigned>(c->valA);
  int rc = radix_sort<K>(c, key, val, key == P<K>(c->keyA) ? P<K>(c->keyB) : P<K>(c->keyA),
                         val == P<unsigned>(c->valA) ? P<unsigned>(c->valB) : P<unsigned>(c->valA), n, L.bits);
  if (rc) return rc;

  // per-frame ranks of the sorted order: each frame's last record and the
  // record of an earlier frame at the position one past it
  const int nblkR = (int)((n + kRTile - 1) / kRTile);
  ENS(hist, sizeof(unsigned) * (256ll * nblkR + 1));
  ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(256ll * nblkR));
  {
    Span sp_(c, CK_FRAME_RANK);
    k_frame_hist<<<nblkR, kT, 0, c->stream>>>(val, n, nblkR, P<unsigned>(c->hist));
  }
  c->launches++;
  rc = scan_excl(c, P<unsigned>(c->hist), 256ll * nblkR, P<unsigned>(c->scan_tmp));
  if (rc) return rc;
  std::vector<int2> req;
  std::vector<int> req_last(nf, -1), req_stale(nf, -1);
  for (int f = 0; f < nf; f++) {
    if (nin_f[f] < 1) continue;
    req_last[f] = (int)req.size();
    req.push_back(make_int2(f, (int)(nin_f[f] - 1)));
    // latest earlier frame whose sorted rows reach position nin_f[f] (the
    // candidate table starts zeroed for its first 10485760 rows, struct.h:10)
    for (int g = f - 1; g >= 0; g--)
      if (nin_f[g] > nin_f[f]) {
        req_stale[f] = (int)req.size();
        req.push_back(make_int2(g, (int)nin_f[f]));
        break;
      }
  }
  std::vector<long long> pos(req.size(), -1);
  std::vector<int4> vcells(req.size());
  std::vector<unsigned long long> vkeys(2 * req.size(), 0);
  if (!req.empty()) {
    ENS(req, sizeof(int2) * req.size());
    // positions, then cells and keys on 16-byte boundaries
    const size_t nr = req.size(), pos_bytes = (sizeof(long long) * nr + 15) & ~(size_t)15;
    ENS(found, pos_bytes + (sizeof(int4) + 2 * sizeof(unsigned long long)) * nr);
    long long* d_pos = P<long long>(c->found);
    int4* d_cells = (int4*)((char*)c->found.p + pos_bytes);
    unsigned long long* d_keys = (unsigned long long*)(d_cells + nr);
    CCK(cudaMemcpyAsync(c->req.p, req.data(), sizeof(int2) * req.size(), cudaMemcpyHostToDevice, c->stream), "copy");
    const int wpb = kT / 32;
    {
      Span sp_(c, CK_FRAME_RANK);
      k_frame_find<K><<<(unsigned)((req.size() + wpb - 1) / wpb), kT, 0, c->stream>>>(
          P<int2>(c->req), (int)req.size(), P<unsigned>(c->hist), nblkR, val, n, key,
          P<int4>(c->cells_in), d_pos, d_cells, d_keys);
    }
    c->launches++;
    CCK(cudaGetLastError(), "k_frame_find");
    CCK(cudaMemcpyAsync(pos.data(), d_pos, sizeof(long long) * req.size(), cudaMemcpyDeviceToHost, c->stream), "copy");
    CCK(cudaMemcpyAsync(vcells.data(), d_cells, sizeof(int4) * req.size(), cudaMemcpyDeviceToHost, c->stream), "copy");
    CCK(cudaMemcpyAsync(vkeys.data(), d_keys, 2 * sizeof(unsigned long long) * req.size(), cudaMemcpyDeviceToHost,
                        c->stream),
        "copy");
    CCK(cudaStreamSynchronize(c->stream), "sync");
  }
  for (size_t r = 0; r < req.size(); r++)
    if (pos[r] < 0 || pos[r] >= n) return cfail(c, PA_ERR_CUDA, "pa_coinc_run: frame rank lookup failed");
  for (int f = 0; f < nf; f++) {
    c->ft.drop[f] = 0;
    if (req_last[f] < 0) continue;
    const int4 last = vcells[req_last[f]];
    int4 stale = make_int4(0, 0, 0, 0);
    if (req_stale[f] >= 0 && nin_f[f] < 10485760) stale = vcells[req_stale[f]];
    if (last.x == stale.x && last.y == stale.y && last.z == stale.z && last.w == stale.w) {
      c->ft.drop[f] = 1;
      c->ft.drop_lo[f] = vkeys[2 * req_last[f]];
      c->ft.drop_hi[f] = vkeys[2 * req_last[f] + 1];
    }
  }
  CCK(cudaMemcpyToSymbolAsync(c_ft, &c->ft, sizeof(FrameTab), 0, cudaMemcpyHostToDevice, c->stream), "symbol");

  // duplicate removal
  ENS(keep, n);
  ENS(uniq, sizeof(unsigned) * 256);
  CCK(cudaMemsetAsync(c->keep.p, 0, n, c->stream), "memset");
  CCK(cudaMemsetAsync(c->uniq.p, 0, sizeof(unsigned) * 256, c->stream), "memset");
  c->val_sorted = val;
  {
    Span sp_(c, CK_DEDUP);
    k_dedup<K><<<(unsigned)((n + kT - 1) / kT), kT, 0, c->stream>>>(key, val, P<double>(c->snr_in), n,
                                                                    P<uint8_t>(c->keep), P<unsigned>(c->uniq));
  }
  c->launches++;
  CCK(cudaGetLastError(), "k_dedup");
  // survivors in sorted order
  const long long nt = (n + kTile - 1) / kTile;
  ENS(blkcnt, sizeof(unsigned) * (nt + 1));
  ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(nt + 1));
  {
    Span sp_(c, CK_COMPACT);
    k_tile_count<<<(unsigned)nt, kT, 0, c->stream>>>(P<uint8_t>(c->keep), n, P<unsigned>(c->blkcnt));
  }
  c->launches++;
  CCK(cudaMemsetAsync(P<unsigned>(c->blkcnt) + nt, 0, sizeof(unsigned), c->stream), "memset");
  rc = scan_excl(c, P<unsigned>(c->blkcnt), nt + 1, P<unsigned>(c->scan_tmp));
  if (rc) return rc;
  unsigned G = 0;
  std::vector<unsigned> uniq(256, 0);
  CCK(cudaMemcpyAsync(&G, P<unsigned>(c->blkcnt) + nt, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "copy");
  CCK(cudaMemcpyAsync(uniq.data(), c->uniq.p, sizeof(unsigned) * 256, cudaMemcpyDeviceToHost, c->stream), "copy");
  CCK(cudaStreamSynchronize(c->stream), "sync");
  for (int f = 0; f < nf; f++) c->frameinfo[3 * f + 2] = (int)uniq[f];
  c->sum.unique = G;
  if (G == 0) return PA_OK;
  ENS(skey, sizeof(K) * G);
  ENS(sval, sizeof(unsigned) * G);
  {
    Span sp_(c, CK_COMPACT);
    k_compact_surv<K><<<(unsigned)nt, kT, 0, c->stream>>>(P<uint8_t>(c->keep), n, P<unsigned>(c->blkcnt), key, val,
                                                           P<K>(c->skey), P<unsigned>(c->sval));
  }
  c->launches++;
  CCK(cudaGetLastError(), "k_compact_surv");

  // coincidences: runs of equal cells
  ENS(gflag, G);
  ENS(gend, sizeof(unsigned) * G);
  ENS(gw, sizeof(unsigned) * G);
  ENS(lastu, sizeof(int));
  CCK(cudaMemsetAsync(c->lastu.p, 0, sizeof(int), c->stream), "memset");
  {
    Span sp_(c, CK_GROUPS);
    k_groups<K><<<(G + kT - 1) / kT, kT, 0, c->stream>>>(P<K>(c->skey), G, c->cfg.mincoin, P<uint8_t>(c->gflag),
                                                        P<unsigned>(c->gend), P<unsigned>(c->gw), P<int>(c->lastu));
  }
  c->launches++;
  CCK(cudaGetLastError(), "k_groups");
  const long long gt = ((long long)G + kTile - 1) / kTile;
  ENS(blkcnt, sizeof(unsigned) * (gt + 1));
  ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(gt + 1));
  {
    Span sp_(c, CK_GROUPS);
    k_tile_count<<<(unsigned)gt, kT, 0, c->stream>>>(P<uint8_t>(c->gflag), G, P<unsigned>(c->blkcnt));
  }
  c->launches++;
  CCK(cudaMemsetAsync(P<unsigned>(c->blkcnt) + gt, 0, sizeof(unsigned), c->stream), "memset");
  rc = scan_excl(c, P<unsigned>(c->blkcnt), gt + 1, P<unsigned>(c->scan_tmp));
  if (rc) return rc;
  unsigned Kc = 0;
  int lastu = 0;
  CCK(cudaMemcpyAsync(&Kc, P<unsigned>(c->blkcnt) + gt, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "copy");
  CCK(cudaMemcpyAsync(&lastu, c->lastu.p, sizeof(int), cudaMemcpyDeviceToHost, c->stream), "copy");
  CCK(cudaStreamSynchronize(c->stream), "sync");
  const int ncoin = (int)Kc + (lastu ? 1 : 0);
  if ((size_t)ncoin + 1 > c->h_recs_cap) {
    if (c->h_recs) cudaFreeHost(c->h_recs);
    c->h_recs = nullptr;
    c->h_recs_cap = 0;
    const size_t cap = (size_t)ncoin + 1 + ncoin / 2;
    CCK(cudaMallocHost((void**)&c->h_recs, sizeof(pa_coinc_rec) * cap), "cudaMallocHost");
    c->h_recs_cap = cap;
  }
  if (Kc > 0) {
    ENS(wkeyA, sizeof(unsigned long long) * Kc);
    ENS(wkeyB, sizeof(unsigned long long) * Kc);
    ENS(cend, sizeof(unsigned) * Kc);
    ENS(cw, sizeof(unsigned) * Kc);
    ENS(cidxA, sizeof(unsigned) * Kc);
    ENS(cidxB, sizeof(unsigned) * Kc);
    {
      Span sp_(c, CK_GROUPS);
      k_compact_groups<<<(unsigned)gt, kT, 0, c->stream>>>(P<uint8_t>(c->gflag), G, P<unsigned>(c->blkcnt),
                                                          P<unsigned>(c->gend), P<unsigned>(c->gw),
                                                          P<unsigned long long>(c->wkeyA), P<unsigned>(c->cend),
                                                          P<unsigned>(c->cw), P<unsigned>(c->cidxA));
    }
    c->launches++;
    CCK(cudaGetLastError(), "k_compact_groups");
    // multiplicity descending, stable (coincidences.c:486)
    unsigned long long* wk = P<unsigned long long>(c->wkeyA);
    unsigned* order = P<unsigned>(c->cidxA);
    rc = radix_sort<unsigned long long>(c, wk, order, P<unsigned long long>(c->wkeyB), P<unsigned>(c->cidxB), Kc, 8);
    if (rc) return rc;
    // member offsets
    ENS(wsort, sizeof(unsigned) * (Kc + 1));
    ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(Kc + 1));
    {
      Span sp_(c, CK_MEANS);
      k_gather_w<<<(Kc + kT - 1) / kT, kT, 0, c->stream>>>(order, P<unsigned>(c->cw), (int)Kc, P<unsigned>(c->wsort));
    }
    c->launches++;
    CCK(cudaMemsetAsync(P<unsigned>(c->wsort) + Kc, 0, sizeof(unsigned), c->stream), "memset");
    rc = scan_excl(c, P<unsigned>(c->wsort), (long long)Kc + 1, P<unsigned>(c->scan_tmp));
    if (rc) return rc;
    unsigned M = 0;
    CCK(cudaMemcpyAsync(&M, P<unsigned>(c->wsort) + Kc, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream), "copy");
    CCK(cudaStreamSynchronize(c->stream), "sync");
    ENS(means, sizeof(pa_coinc_rec) * Kc);
    ENS(fra, sizeof(int) * (M + 1));
    ENS(ops, sizeof(int) * (M + 1));
    {
      Span sp_(c, CK_MEANS);
      k_means<<<(Kc + 127) / 128, 128, 0, c->stream>>>(order, P<unsigned>(c->cend), P<unsigned>(c->cw),
                                                        P<unsigned>(c->wsort), (int)Kc, P<unsigned>(c->sval),
                                                        P<unsigned>(c->rawidx), P<double>(c->rec),
                                                        (double)c->cfg.N, c->cfg.refr, P<pa_coinc_rec>(c->means),
                                                        P<int>(c->fra), P<int>(c->ops));
    }
    c->launches++;
    CCK(cudaGetLastError(), "k_means");
    if ((size_t)M + 1 > c->h_mem_cap) {
      if (c->h_fra) cudaFreeHost(c->h_fra);
      if (c->h_ops) cudaFreeHost(c->h_ops);
      c->h_fra = c->h_ops = nullptr;
      c->h_mem_cap = 0;
      const size_t cap = (size_t)M + 1 + M / 2;
      CCK(cudaMallocHost((void**)&c->h_fra, sizeof(int) * cap), "cudaMallocHost");
      CCK(cudaMallocHost((void**)&c->h_ops, sizeof(int) * cap), "cudaMallocHost");
      c->h_mem_cap = cap;
    }
    CCK(cudaMemcpyAsync(c->h_recs, c->means.p, sizeof(pa_coinc_rec) * Kc, cudaMemcpyDeviceToHost, c->stream),
        "copy");
    if (M) {
      CCK(cudaMemcpyAsync(c->h_fra, c->fra.p, sizeof(int) * M, cudaMemcpyDeviceToHost, c->stream), "copy");
      CCK(cudaMemcpyAsync(c->h_ops, c->ops.p, sizeof(int) * M, cudaMemcpyDeviceToHost, c->stream), "copy");
    }
    // the device work ends here; what follows is host bookkeeping
    CCK(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
    c->ev1_done = true;
    CCK(cudaStreamSynchronize(c->stream), "sync");
    c->sum.nmembers = M;
  }
  if (lastu) {
    // the last group is counted but never stored: a record of multiplicity
    // 0 whose means are 0/0 (coincidences.c:504-512), computed at run time
    volatile double zero = 0.0;
    pa_coinc_rec& r = c->h_recs[ncoin - 1];
    r.w = 0;
    r.first = (int)c->sum.nmembers;
    for (int l = 0; l < 4; l++) r.mean[l] = zero / zero;
    r.mean[4] = sqrt(zero);
  }
  c->sum.ncoin = ncoin;
  // coincidences.c:535-541: the largest multiplicity with the largest SNR
  c->sum.maxcoin = Kc > 0 ? c->h_recs[0].w : 0;
  c->sum.maxcoin_index = 0;
  double maxsnr = 0;
  for (int q = 0; q < ncoin; q++) {
    if (!q) maxsnr = c->h_recs[q].mean[4];
    if (c->h_recs[q].w == c->sum.maxcoin && c->h_recs[q].mean[4] > maxsnr) {
      maxsnr = c->h_recs[q].mean[4];
      c->sum.maxcoin_index = q;
    }
  }
  return PA_OK;
}

extern "C" {

int pa_coinc_run(pa_coinc* c, pa_coinc_summary* sum) {
  pa::TraceRange trace_("pa_coinc_run");
  if (!c) return PA_ERR_ARG;
  CCK(cudaSetDevice(c->cfg.device), "cudaSetDevice");
  const int nf = (int)c->frames.size();
  memset(&c->sum, 0, sizeof(c->sum));

  c->frameinfo.assign(3 * (size_t)nf, 0);
  c->sum.nframes = nf;
  c->sum.raw = c->nraw;
  c->n_in = 0;
  c->val_sorted = nullptr;
  c->ev1_done = false;
  CCK(cudaEventRecord(c->ev0, c->stream), "cudaEventRecord");
  // frame table
  memset(&c->ft, 0, sizeof(c->ft));
  c->ft.nframes = nf;
  int nblk1 = 0;
  for (int f = 0; f < nf; f++) {
    c->ft.frame_no[f] = c->frames[f];
    c->ft.raw_start[f] = c->raw_start[f];
    c->ft.blk_start[f] = nblk1;
    nblk1 += (int)((c->raw_start[f + 1] - c->raw_start[f] + kTile - 1) / kTile);
    c->frameinfo[3 * f] = c->frames[f];
  }
  c->ft.raw_start[nf] = c->nraw;
  c->ft.blk_start[nf] = nblk1;
  int rc = PA_OK;
  if (nblk1 > 0) {
    CCK(cudaMemcpyToSymbolAsync(c_ft, &c->ft, sizeof(FrameTab), 0, cudaMemcpyHostToDevice, c->stream), "symbol");
    CellArgs a;
    a.lo = M_PI_2 - c->cfg.narrowdown;
    a.hi = M_PI_2 + c->cfg.narrowdown;
    a.N = (double)c->cfg.N;
    a.sqrN = pow(c->cfg.N, 2);
    a.omsN = c->cfg.oms * c->cfg.N;
    volatile double epsm = PA_C_EPSMA;
    a.se = sin(epsm);
    a.ce = cos(epsm);
    for (int j = 0; j < 4; j++) {
      for (int i = 0; i < 4; i++) a.v[i][j] = c->cfg.vedva[i][j] / c->cfg.scale[j];
      a.half_shift[j] = 0.5 * c->cfg.shift[j];
    }
    a.refr = c->cfg.refr;
    a.snrcut = c->cfg.snrcutoff;
    a.omsN_f = (float)a.omsN;
    a.se_f = (float)a.se;
    a.ce_f = (float)a.ce;
    auto split = [](double d, float* h, float* l) {
      *h = (float)d;
      *l = (float)(d - (double)*h);
    };
    a.fast = c->cfg.N < (1 << 24);
    a.Nf = (float)c->cfg.N;  // exact when fast
    split(a.sqrN, &a.sqrN_h, &a.sqrN_l);
    for (int j = 0; j < 4; j++) {
      split(a.v[0][j], &a.v0_h[j], &a.v0_l[j]);
      split(a.v[1][j], &a.v1_h[j], &a.v1_l[j]);
      a.hs_f[j] = (float)a.half_shift[j];  // exact: halves of digits
      a.v2_f[j] = (float)a.v[2][j];
      a.v3_f[j] = (float)a.v[3][j];
      // 8e-6 on be0 and be1 (their FP32 error is below 1.1e-6), plus the
      // FP32 products and the FP64 rounding differences
      const double m = fabs(a.omsN) * (fabs(a.v[2][j]) + fabs(a.v[3][j])) * 8e-6 + 2e-6;
      a.margin[j] = m < 1.0 ? (float)m : 1.0f;
    }
    ENS(cells_raw, sizeof(int4) * c->nraw);
    ENS(flag, c->nraw);
    ENS(snr_raw, sizeof(double) * c->nraw);
    ENS(blkcnt, sizeof(unsigned) * (nblk1 + 1));
    ENS(scan_tmp, sizeof(unsigned) * scan_tmp_len(nblk1 + 1));
    ENS(minmax, sizeof(int) * 9);
    const int mm0[9] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, INT_MIN, 0};
    CCK(cudaMemcpyAsync(c->minmax.p, mm0, sizeof(mm0), cudaMemcpyHostToDevice, c->stream), "copy");
    {
      Span sp_(c, CK_CELLS);
      k_cells<<<nblk1, kT, 0, c->stream>>>(P<double>(c->rec), a, P<int4>(c->cells_raw), P<uint8_t>(c->flag),
                                          P<unsigned>(c->blkcnt), P<int>(c->minmax),
                                          (unsigned*)(P<int>(c->minmax) + 8), P<double>(c->snr_raw));
    }
    c->launches++;
    CCK(cudaGetLastError(), "k_cells");
    CCK(cudaMemsetAsync(P<unsigned>(c->blkcnt) + nblk1, 0, sizeof(unsigned), c->stream), "memset");
    rc = scan_excl(c, P<unsigned>(c->blkcnt), nblk1 + 1, P<unsigned>(c->scan_tmp));
    if (rc) return rc;
    std::vector<unsigned> boff(nblk1 + 1);
    int mm[9];
    CCK(cudaMemcpyAsync(boff.data(), c->blkcnt.p, sizeof(unsigned) * (nblk1 + 1), cudaMemcpyDeviceToHost, c->stream),
        "copy");
    CCK(cudaMemcpyAsync(mm, c->minmax.p, sizeof(mm), cudaMemcpyDeviceToHost, c->stream), "copy");
    CCK(cudaStreamSynchronize(c->stream), "sync");
    c->n_in = boff[nblk1];
    std::vector<long long> nin_f(nf);
    for (int f = 0; f < nf; f++) {
      c->ft.in_start[f] = boff[c->ft.blk_start[f]];
      nin_f[f] = (long long)boff[c->ft.blk_start[f + 1]] - boff[c->ft.blk_start[f]];
      c->frameinfo[3 * f + 1] = (int)nin_f[f];
    }
    c->ft.in_start[nf] = c->n_in;
    c->sum.inband = c->n_in;
    c->sum.fp64_cells = (unsigned)mm[8];
    if (c->n_in > 0) {
      ENS(rawidx, sizeof(unsigned) * c->n_in);
      ENS(cells_in, sizeof(int4) * c->n_in);
      KeyLayout L;
      int bits[4], tot = 0;
      for (int j = 0; j < 4; j++) {
        const unsigned long long range = (unsigned long long)((long long)mm[4 + j] - (long long)mm[j]);
        int b = 0;
        while (b < 63 && (range >> b)) b++;
        bits[j] = b;
        tot += b;
        L.maxc[j] = mm[4 + j];
      }
      // column 0 is the most significant
      int sh = tot;
      for (int j = 0; j < 4; j++) {
        sh -= bits[j];
        L.shift[j] = sh;
      }
      CCK(cudaMemcpyToSymbolAsync(c_ft, &c->ft, sizeof(FrameTab), 0, cudaMemcpyHostToDevice, c->stream), "symbol");
      if (tot <= 64) {
        L.bits = tot;
        rc = run_keyed<unsigned long long>(c, L, nblk1, nin_f);
      } else {
        L.bits = 128;
        rc = run_keyed<U128>(c, L, nblk1, nin_f);
      }
      if (rc) return rc;
    }
  }
  if (!c->ev1_done) CCK(cudaEventRecord(c->ev1, c->stream), "cudaEventRecord");
  CCK(cudaEventSynchronize(c->ev1), "cudaEventSynchronize");
  float ms = 0;
  cudaEventElapsedTime(&ms, c->ev0, c->ev1);
  c->last_ms = ms;
  prof_collect(c);
  if (sum) *sum = c->sum;
  return PA_OK;
}

int pa_coinc_get(const pa_coinc* c, int* frameinfo, pa_coinc_rec* recs, int* fra, int* ops) {
  if (!c) return PA_ERR_ARG;
  if (frameinfo && !c->frameinfo.empty()) memcpy(frameinfo, c->frameinfo.data(), sizeof(int) * c->frameinfo.size());
  if (recs && c->sum.ncoin > 0) memcpy(recs, c->h_recs, sizeof(pa_coinc_rec) * c->sum.ncoin);
  if (fra && c->sum.nmembers > 0) memcpy(fra, c->h_fra, sizeof(int) * c->sum.nmembers);
  if (ops && c->sum.nmembers > 0) memcpy(ops, c->h_ops, sizeof(int) * c->sum.nmembers);
  return PA_OK;
}

int pa_coinc_cells(pa_coinc* c, int* cells, unsigned char* keep) {
  if (!c) return PA_ERR_ARG;
  if (c->n_in <= 0) return PA_OK;
  CCK(cudaSetDevice(c->cfg.device), "cudaSetDevice");
  if (cells)
    CCK(cudaMemcpyAsync(cells, c->cells_in.p, sizeof(int4) * c->n_in, cudaMemcpyDeviceToHost, c->stream), "copy");
  if (keep) {
    if (!c->val_sorted) return cfail(c, PA_ERR_ARG, "pa_coinc_cells: no completed run");
    // keep flags by in-band index, from those by sorted position
    int rc = ensure(c, c->keep_in, c->n_in);
    if (rc) return rc;
    k_keep_scatter<<<(unsigned)((c->n_in + kT - 1) / kT), kT, 0, c->stream>>>(P<uint8_t>(c->keep), c->val_sorted,
                                                                               c->n_in, P<uint8_t>(c->keep_in));
    c->launches++;
    CCK(cudaGetLastError(), "k_keep_scatter");
    CCK(cudaMemcpyAsync(keep, c->keep_in.p, c->n_in, cudaMemcpyDeviceToHost, c->stream), "copy");
  }
  CCK(cudaStreamSynchronize(c->stream), "sync");
  return PA_OK;
}

double pa_coinc_last_call_ms(const pa_coinc* c) { return c ? c->last_ms : 0.0; }

int pa_coinc_set_profiling(pa_coinc* c, int on) {
  if (!c) return PA_ERR_ARG;
  c->prof_on = on != 0;
  for (int k = 0; k < CK_COUNT; k++) {
    c->prof_ms[k] = 0;
    c->prof_n[k] = 0;
  }
  return PA_OK;
}

int pa_coinc_profile_get(const pa_coinc* c, int kind, const char** name, double* total_ms, long long* launches) {
  if (!c || kind < 0 || kind >= CK_COUNT) return PA_ERR_ARG;
  if (name) *name = kCoincKindName[kind];
  if (total_ms) *total_ms = c->prof_ms[kind];
  if (launches) *launches = c->prof_n[kind];
  return PA_OK;
}
long long pa_coinc_kernel_launches(const pa_coinc* c) { return c ? c->launches : 0; }

}  // extern "C"
