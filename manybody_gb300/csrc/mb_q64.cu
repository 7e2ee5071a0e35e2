// Block floating point ("Q64") path: FP64-class accuracy without the FP64 pipe.
//
// On GB300 the FP64 units run at 1/64 of the FP32 rate (a rate probe on the
// part measured 1.9 FP64 FMA per clock per SM against 109 FP32 FMA), so a
// matrix-free H|psi> that adds 33 complex128 terms per output element in
// FP64 is ALU-bound at ~2 % of HBM bandwidth.  Here a vector is stored as
// 64-bit integer mantissas (re, im) with ONE binary exponent per vector:
// value_i = q_i * 2^E.  The hopping part of H has integer weights (+-1, +-2
// times -t), so sum_j w_j q_j is an exact int64 sum (integer adders run at
// full rate); only the per-element products by -t*scale and by the diagonal
// U*n_double - shift are 64x64->128-bit integer multiplies, and one rounding
// shift produces the output mantissa.  Every vector keeps |q| < 2^qbits,
// qbits = 62 - ceil(log2(W)), W the largest sum of |hop weights| of a state,
// so the hop sums cannot overflow.  Accuracy: the quantum is 2^(E) with
// 2^(E+qbits) >~ max|x|, i.e. ~57 bits relative to the largest element;
// dot products are accumulated exactly in 128-bit integers.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mb_internal.h"
#include "mb_q64.h"

namespace mb {

// ---------------------------------------------------------------------------
// Exact conversions between FP64 and fixed point, integer operations only.
// ---------------------------------------------------------------------------
// round(x * 2^-E) for |x| < 2^(E+62); ties rounded away from zero.
__device__ __forceinline__ long long f64_to_fixed(double x, int E) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7FF);
  if (ex == 0) return 0;  // zero / subnormal: below any representable quantum here
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull;
  const int s = ex - 1075 - E;  // x = m * 2^(ex-1075) = (m * 2^s) * 2^E
  unsigned long long q;
  if (s >= 0) q = m << s;
  else if (s > -60) q = (m + (1ull << (-s - 1))) >> (-s);
  else q = 0;
  return (b >> 63) ? -(long long)q : (long long)q;
}

// q * 2^E rounded to nearest even (the exact value of the integer times the
// power of two), integer operations only.
__device__ __forceinline__ double fixed_to_f64(long long q, int E) {
  if (q == 0) return 0.0;
  const unsigned long long sign = q < 0 ? 0x8000000000000000ull : 0ull;
  unsigned long long a = q < 0 ? (unsigned long long)(-q) : (unsigned long long)q;
  const int lz = __clzll(a);
  a <<= lz;                                  // bit 63 set
  unsigned long long m = a >> 11;            // 53 bits
  const unsigned long long rem = a & 0x7FFull;
  int e2 = 63 - lz + E;                      // value = (a / 2^63) * 2^e2
  if (rem > 0x400ull || (rem == 0x400ull && (m & 1ull))) {
    m += 1;
    if (m == (1ull << 53)) {
      m >>= 1;
      e2 += 1;
    }
  }
  const int biased = e2 + 1023;
  if (biased <= 0) return 0.0;
  if (biased >= 2047) return __longlong_as_double((long long)(sign | 0x7FF0000000000000ull));
  const unsigned long long bits = sign | ((unsigned long long)biased << 52) | (m & 0xFFFFFFFFFFFFFull);
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ unsigned long long mag(long long q) {
  return q < 0 ? (unsigned long long)(-q) : (unsigned long long)q;
}

// 128-bit product accumulated with 32 low bits dropped (exact enough: each
// product loses < 2^32 units against sums of order 2^100+).
__device__ __forceinline__ __int128 prod_hi(long long a, long long b) {
  return ((__int128)a * (__int128)b) >> 32;
}

__device__ __forceinline__ double i128_to_f64(__int128 v) {
  const long long hi = (long long)(v >> 64);
  const unsigned long long lo = (unsigned long long)v;
  return (double)hi * 18446744073709551616.0 + (double)lo;
}

__device__ __forceinline__ long long round_shift(__int128 p, int sh) {
  if (sh <= 0) return (long long)(p << (-sh));
  if (sh >= 127) return 0;
  return (long long)((p + ((__int128)1 << (sh - 1))) >> sh);
}

template <int NC>
__device__ void q_block_reduce(double (&v)[NC], unsigned long long magor, double* partials,
                               unsigned long long* max_or) {
  __shared__ double red[32][NC];
  __shared__ unsigned long long mor[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    double a = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    v[k] = a;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) magor |= __shfl_down_sync(0xffffffffu, magor, o);
  __syncthreads();
  if (lane == 0) {
    for (int k = 0; k < NC; ++k) red[warp][k] = v[k];
    mor[warp] = magor;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    unsigned long long m = lane < nw ? mor[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m |= __shfl_down_sync(0xffffffffu, m, o);
    for (int k = 0; k < NC; ++k) {
      double a = lane < nw ? red[lane][k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0 && partials) partials[(size_t)blockIdx.x * NC + k] = a;
    }
    if (lane == 0 && max_or && m) atomicOr(max_or, m);
  }
}

// Exact block sums of the apply's two dot accumulators (128-bit integers):
// the block writes {xy_lo, xy_hi, yy_lo, yy_hi} to part128[4 * blockIdx.x]
// and ORs its max word into *max_or.  Integer sums are exact in any order, so
// the dot products do not depend on which block applied which rows.
__device__ __forceinline__ __int128 shfl_down_i128(__int128 v, int o) {
  const unsigned long long lo = __shfl_down_sync(0xffffffffu, (unsigned long long)v, o);
  const unsigned long long hi =
      __shfl_down_sync(0xffffffffu, (unsigned long long)((unsigned __int128)v >> 64), o);
  return (__int128)(((unsigned __int128)hi << 64) | lo);
}

__device__ void q_block_reduce_exact(__int128 xy, __int128 yy, unsigned long long magor,
                                     long long* part128, unsigned long long* max_or) {
  __shared__ __int128 red[32][2];
  __shared__ unsigned long long mor[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    xy += shfl_down_i128(xy, o);
    yy += shfl_down_i128(yy, o);
    magor |= __shfl_down_sync(0xffffffffu, magor, o);
  }
  __syncthreads();
  if (lane == 0) {
    red[warp][0] = xy;
    red[warp][1] = yy;
    mor[warp] = magor;
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    __int128 a = lane < nw ? red[lane][0] : 0, b = lane < nw ? red[lane][1] : 0;
    unsigned long long m = lane < nw ? mor[lane] : 0ull;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a += shfl_down_i128(a, o);
      b += shfl_down_i128(b, o);
      m |= __shfl_down_sync(0xffffffffu, m, o);
    }
    if (lane == 0) {
      if (part128) {
        long long* p = part128 + 4 * (size_t)blockIdx.x;
        p[0] = (long long)(unsigned long long)a;
        p[1] = (long long)(a >> 64);
        p[2] = (long long)(unsigned long long)b;
        p[3] = (long long)(b >> 64);
      }
      if (max_or && m) atomicOr(max_or, m);
    }
  }
}

// The exact sum of nblocks such partials, converted once to double: out[0]
// (xy), out[1] (yy).
__global__ void k_q_reduce128(const long long* __restrict__ part, int nblocks,
                              double* __restrict__ out) {
  __int128 a = 0, b = 0;
  for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    const long long* p = part + 4 * (size_t)i;
    a += (__int128)(((unsigned __int128)(unsigned long long)p[1] << 64) | (unsigned long long)p[0]);
    b += (__int128)(((unsigned __int128)(unsigned long long)p[3] << 64) | (unsigned long long)p[2]);
  }
  __shared__ __int128 red[32][2];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += shfl_down_i128(a, o);
    b += shfl_down_i128(b, o);
  }
  if (lane == 0) {
    red[warp][0] = a;
    red[warp][1] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    __int128 sa = 0, sb = 0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); ++w) {
      sa += red[w][0];
      sb += red[w][1];
    }
    out[0] = i128_to_f64(sa);
    out[1] = i128_to_f64(sb);
  }
}

void launch_q_reduce128(const void* part, int nblocks, double* out, cudaStream_t st) {
  k_q_reduce128<<<1, 256, 0, st>>>((const long long*)part, nblocks, out);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// The Q64 apply: y = scale (H - shift) x + beta z on mantissas.
//   P = c1 * S + cq[popc(up & down)] * x_q + c3 * z_q      (128-bit)
//   y_q = round(P / 2^sh)
// S = sum over hops of +-x_q (doubled bonds listed twice), exact in int64.
// dots (DOTS bit0): Re<x,y> and <y,y> as exact integer sums >> 32, written
// per block as 128-bit integers (partials: 4 words a block; k_q_reduce128
// sums them).
//
// One CTA of 1024 threads per SM walks the rows r_up in the row schedule's
// order (reverse Cuthill-McKee: rows in flight together share neighbour rows
// in L2).  Per row: the row x[r,:] and eight zero elements go to shared
// memory, then warp w takes the 32-column groups g = w, w + 32, ...:
//   down hops: sliced table, one coalesced 16-byte load per lane for four
//     slots; entry = neighbour index in the staged row | sign << 31, in an
//     order that keeps each quarter warp on distinct bank groups; padding
//     reads a zero element.  A negative hop adds v ^ -1 (= -v - 1); the
//     column's count of negative hops is added back once;
//   up hops: the row's sign-sorted target list (uniform across the CTA):
//     coalesced 16-byte loads x[r',c], summed then subtracted, no sign work;
//     with up_prefetch set, the warp asks L2 for its group's up-hop lines
//     before the down hops (an apply shape the autotuner may pick).
// Hops are summed in pairs (three-operand 64-bit adds).
// ---------------------------------------------------------------------------
constexpr int kQThreads = 1024;

// Sum of +-v over one warp group's sliced-table slots (down hops of a staged
// row, or up hops of a staged column).  `val` takes the neighbour's byte
// offset (index * 16).  A negative hop adds v ^ -1 (= -v - 1); the caller adds
// the state's count of negative hops back once.  The group's slot count k is
// the same for the whole warp, so the padding slots past k in the last word
// are skipped without divergence.
//  32-bit entries: index | negative << 31, four slots per 16-byte load;
//  16-bit entries: index | negative << 15, eight slots per 16-byte load.
template <typename Load>
__device__ __forceinline__ void hop_add(Load& val, uint32_t off, long long m, long long& sr,
                                        long long& si) {
  const longlong2 v = val(off);
  sr += v.x ^ m;
  si += v.y ^ m;
}

template <typename Load>
__device__ __forceinline__ void sliced_sum(const uint32_t* __restrict__ sell, int2 gi, int lane,
                                           Load&& val, long long& sr, long long& si) {
  const uint4* ep = reinterpret_cast<const uint4*>(sell + gi.x) + lane;
  const int k = gi.y;
  int j = 0;
  for (; j + 4 <= k; j += 4) {
    const uint4 e = __ldg(ep + 8 * j);
    const long long m0 = (int)e.x >> 31, m1 = (int)e.y >> 31;  // 0 or -1
    const long long m2 = (int)e.z >> 31, m3 = (int)e.w >> 31;
    const longlong2 v0 = val(e.x << 4), v1 = val(e.y << 4);  // the sign bit shifts out
    const longlong2 v2 = val(e.z << 4), v3 = val(e.w << 4);
    sr += (v0.x ^ m0) + (v1.x ^ m1);
    si += (v0.y ^ m0) + (v1.y ^ m1);
    sr += (v2.x ^ m2) + (v3.x ^ m3);
    si += (v2.y ^ m2) + (v3.y ^ m3);
  }
  if (j < k) {
    const uint4 e = __ldg(ep + 8 * j);
    hop_add(val, e.x << 4, (int)e.x >> 31, sr, si);
    if (j + 1 < k) hop_add(val, e.y << 4, (int)e.y >> 31, sr, si);
    if (j + 2 < k) hop_add(val, e.z << 4, (int)e.z >> 31, sr, si);
  }
}

// the two 16-bit entries of a word: byte offsets and sign masks
__device__ __forceinline__ uint32_t off_lo(uint32_t w) { return (w << 4) & 0x7FFF0u; }
__device__ __forceinline__ uint32_t off_hi(uint32_t w) { return (w >> 12) & 0x7FFF0u; }
__device__ __forceinline__ long long neg_lo(uint32_t w) { return (int)(w << 16) >> 31; }
__device__ __forceinline__ long long neg_hi(uint32_t w) { return (int)w >> 31; }

template <typename Load>
__device__ __forceinline__ void word_add(Load& val, uint32_t w, long long& sr, long long& si) {
  const longlong2 a = val(off_lo(w)), b = val(off_hi(w));
  const long long ma = neg_lo(w), mb = neg_hi(w);
  sr += (a.x ^ ma) + (b.x ^ mb);
  si += (a.y ^ ma) + (b.y ^ mb);
}

template <typename Load>
__device__ __forceinline__ void sliced_sum16(const uint16_t* __restrict__ sell, int2 gi, int lane,
                                             Load&& val, long long& sr, long long& si) {
  const uint4* ep = reinterpret_cast<const uint4*>(sell + gi.x) + lane;
  const int k = gi.y;
  int j = 0;
  for (; j + 8 <= k; j += 8) {
    const uint4 e = __ldg(ep + 4 * j);
    word_add(val, e.x, sr, si);
    word_add(val, e.y, sr, si);
    word_add(val, e.z, sr, si);
    word_add(val, e.w, sr, si);
  }
  if (j < k) {
    const uint4 e = __ldg(ep + 4 * j);
    const int rem = k - j;  // 1..7
    const uint32_t w[4] = {e.x, e.y, e.z, e.w};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      if (2 * q + 2 <= rem) word_add(val, w[q], sr, si);
      else if (2 * q + 1 == rem) hop_add(val, off_lo(w[q]), neg_lo(w[q]), sr, si);
    }
  }
}

// The same sum from a lane's words in a warp-private shared buffer (word w
// at ep[32 w]).
template <typename Load>
__device__ __forceinline__ void sliced_sum_words(const uint4* ep, int k, Load&& val, long long& sr,
                                                 long long& si) {
  int j = 0;
  for (; j + 4 <= k; j += 4) {
    const uint4 e = ep[8 * j];
    const long long m0 = (int)e.x >> 31, m1 = (int)e.y >> 31;
    const long long m2 = (int)e.z >> 31, m3 = (int)e.w >> 31;
    const longlong2 v0 = val(e.x << 4), v1 = val(e.y << 4);
    const longlong2 v2 = val(e.z << 4), v3 = val(e.w << 4);
    sr += (v0.x ^ m0) + (v1.x ^ m1);
    si += (v0.y ^ m0) + (v1.y ^ m1);
    sr += (v2.x ^ m2) + (v3.x ^ m3);
    si += (v2.y ^ m2) + (v3.y ^ m3);
  }
  if (j < k) {
    const uint4 e = ep[8 * j];
    hop_add(val, e.x << 4, (int)e.x >> 31, sr, si);
    if (j + 1 < k) hop_add(val, e.y << 4, (int)e.y >> 31, sr, si);
    if (j + 2 < k) hop_add(val, e.z << 4, (int)e.z >> 31, sr, si);
  }
}

template <int TB, typename Load>
__device__ __forceinline__ void sliced_sum_t(const uint32_t* sell, const uint16_t* sell16,
                                             int2 gi, int lane, Load&& val, long long& sr,
                                             long long& si) {
  if (TB == 16) sliced_sum16(sell16, gi, lane, val, sr, si);
  else sliced_sum(sell, gi, lane, val, sr, si);
}

// ---------------------------------------------------------------------------
// Column pass of the two-pass Q64 apply.  For every column c (down state) the
// column x[:, c] (Du elements, 16 bytes apart by the row length) and eight zero
// elements are staged in shared memory; warp w then takes the 32-row groups
// g = w, w + 32, ... and gathers each row's up hops from the staged column
// through the up sector's sliced table, exactly as the row pass gathers down
// hops from a staged row.  The exact int64 hop sum of (r, c) goes to
// ups[c * Du + r] (column-major: one warp's 32 rows are one 512-byte store).
// CTAs take consecutive columns, so the strided column loads of the CTAs in
// flight share their L2 sectors.
// ---------------------------------------------------------------------------
constexpr int kQColThreads = 1024;

template <int TB>
__global__ void __launch_bounds__(kQColThreads, 1)
k_upcol_q(OpView v, const longlong2* __restrict__ x, longlong2* __restrict__ ups) {
  extern __shared__ __align__(16) unsigned char smem[];
  longlong2* col = reinterpret_cast<longlong2*>(smem);
  const int64_t Dd = v.Dd, Du = v.dim / v.Dd;
  if (threadIdx.x < kSlicedPads) col[Du + threadIdx.x] = make_longlong2(0, 0);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int64_t ngroups = (Du + 31) >> 5;
  const int64_t nt = blockDim.x;
  const int2* sgrp = reinterpret_cast<const int2*>(TB == 16 ? v.up_sgrp16 : v.up_sgrp);
  auto val = [&](uint32_t off) -> longlong2 {
    return *reinterpret_cast<const longlong2*>(smem + off);
  };
  for (int64_t c = blockIdx.x; c < Dd; c += gridDim.x) {
    __syncthreads();
    for (int64_t r0 = threadIdx.x; r0 < Du; r0 += 8 * nt) {
      longlong2 t[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t r = r0 + k * nt;
        t[k] = r < Du ? __ldg(x + r * Dd + c) : make_longlong2(0, 0);
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t r = r0 + k * nt;
        if (r < Du) col[r] = t[k];
      }
    }
    __syncthreads();
    for (int64_t g = warp; g < ngroups; g += nwarps) {
      const int64_t r = (g << 5) + lane;
      long long sr = 0, si = 0;
      sliced_sum_t<TB>(v.up_sell, v.up_sell16, __ldg(sgrp + g), lane, val, sr, si);
      if (r < Du) {
        const int nneg = __ldg(&v.up_nneg[r]);
        ups[c * Du + r] = make_longlong2(sr + nneg, si + nneg);
      }
    }
  }
}

template <bool STAGED, int DOTS, bool HAS_Z, bool UPS, int TB, bool TS>
__global__ void __launch_bounds__(kQThreads, 1)
k_apply_q(OpView v, const longlong2* __restrict__ x, longlong2* y, const longlong2* z,
          const QParams* __restrict__ prm, double* __restrict__ partials,
          unsigned long long* __restrict__ max_or, const longlong2* __restrict__ ups) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t Dd = v.Dd;
  const int64_t Du_all = v.dim / v.Dd;
  const uint32_t row_bytes = (uint32_t)(16 * Dd);
  uint32_t* s_up = reinterpret_cast<uint32_t*>(smem + (STAGED ? row_bytes + 16 * kSlicedPads : 0));
  __shared__ long long s_cq[kMaxOrbitals + 1];
  __shared__ long long s_c1, s_c3;
  __shared__ int s_sh;
  if (threadIdx.x <= (unsigned)v.L) s_cq[threadIdx.x] = prm->cq[threadIdx.x];
  if (STAGED && threadIdx.x < kSlicedPads)
    reinterpret_cast<longlong2*>(smem + row_bytes)[threadIdx.x] = make_longlong2(0, 0);
  if (threadIdx.x == 0) {
    s_c1 = prm->c1;
    s_c3 = prm->c3;
    s_sh = prm->sh;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int64_t ngroups = (Dd + 31) >> 5;
  __int128 a_xy = 0, a_yy = 0;
  unsigned long long mor = 0;
  // a down neighbour by table entry: staged row, or the row in global memory
  auto dn_val = [&](const longlong2* xrow, uint32_t off) -> longlong2 {
    if (STAGED) return *reinterpret_cast<const longlong2*>(smem + off);
    return off < row_bytes
               ? __ldg(reinterpret_cast<const longlong2*>(reinterpret_cast<const char*>(xrow) + off))
               : make_longlong2(0, 0);
  };
  const int2* sgrp = reinterpret_cast<const int2*>(TB == 16 ? v.dn_sgrp16 : v.dn_sgrp);
  // row_split CTAs share a row (the grid is a multiple of it): each stages the
  // row and takes every split-th column group
  const int split = v.row_split > 1 ? v.row_split : 1;
  const int64_t g0 = (int64_t)(blockIdx.x % split) * nwarps, gstep = (int64_t)nwarps * split;
  const int64_t rstep = gridDim.x / split;
  // TS: a warp's down-table words of its next column group go to a
  // warp-private shared buffer (cp.async, one 16-byte word per lane and slot
  // quadruple) while it finishes the current group, so its down hops read them
  // from shared memory instead of waiting on L2 once per word.  A warp's groups
  // are the same in every row: after its last group of a row comes its first.
  uint4* tbuf = nullptr;
  int kcur = 0;
  auto ts_issue = [&](int64_t gg) -> int {
    const int2 gi = __ldg(sgrp + gg);
    const uint4* src = reinterpret_cast<const uint4*>(v.dn_sell + gi.x) + lane;
    const uint32_t dst = (uint32_t)__cvta_generic_to_shared(tbuf + lane);
    const int nw = (gi.y + 3) >> 2;
    for (int w = 0; w < nw; ++w)
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + 512u * (uint32_t)w),
                   "l"(src + 32 * w)
                   : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
    return gi.y;
  };
  if (TS) {
    const size_t lists = sizeof(uint32_t) * (size_t)((v.max_up_list + 3) & ~3);
    tbuf = reinterpret_cast<uint4*>(smem + row_bytes + 16 * kSlicedPads + lists) +
           (size_t)warp * v.dn_max_words * 32;
    if (g0 + warp < ngroups && blockIdx.x / split < v.Du) kcur = ts_issue(g0 + warp);
  }

  for (int64_t ri = blockIdx.x / split; ri < v.Du; ri += rstep) {
    const int64_t r = v.row_sched ? (int64_t)v.row_sched[ri] : ri;
    const longlong2* xrow = x + r * Dd;
    __syncthreads();
    const int u0 = UPS ? 0 : __ldg(&v.up_loff[r]);
    const int nu = UPS ? 0 : __ldg(&v.up_loff[r + 1]) - u0;
    const int npos = UPS ? 0 : __ldg(&v.up_lpos[r]);
    for (int j = threadIdx.x; j < nu; j += blockDim.x) s_up[j] = __ldg(&v.up_list[u0 + j]);
    if (STAGED)
      for (int64_t c = threadIdx.x; c < Dd; c += blockDim.x)
        reinterpret_cast<longlong2*>(smem)[c] = xrow[c];
    __syncthreads();
    const uint32_t um = v.up_mask[r];
    const long long c1 = s_c1, c3 = s_c3;
    const int sh = s_sh;
    for (int64_t g = g0 + warp; g < ngroups; g += gstep) {
      const int64_t c = (g << 5) + lane;
      const bool live = c < Dd;
      const int64_t cl = live ? c : Dd - 1;
      if (!UPS && v.up_prefetch) prefetch_up_group<16>(x, s_up, nu, g, lane, row_bytes);
      long long sr = 0, si = 0;
      if (TS) {
        asm volatile("cp.async.wait_all;" ::: "memory");  // this group's words
        sliced_sum_words(tbuf + lane, kcur, [&](uint32_t off) { return dn_val(xrow, off); }, sr,
                         si);
        int64_t gn = g + gstep;
        if (gn >= ngroups) gn = ri + rstep < v.Du ? g0 + warp : -1;
        if (gn >= 0) kcur = ts_issue(gn);
      } else {
        // four slots per 16-byte load; the last word's unused slots are padding
        sliced_sum_t<TB>(v.dn_sell, v.dn_sell16, __ldg(sgrp + g), lane,
                         [&](uint32_t off) { return dn_val(xrow, off); }, sr, si);
      }
      const int nneg = __ldg(&v.dn_nneg[cl]);
      sr += nneg;
      si += nneg;
      if (UPS) {
        // up hops: the column pass's exact sum for (r, c)
        const longlong2 uv = __ldg(ups + cl * Du_all + r);
        sr += uv.x;
        si += uv.y;
      }
      const char* xc = reinterpret_cast<const char*>(x + cl);
      auto up_val = [&](int k) {
        return __ldg(reinterpret_cast<const longlong2*>(xc + (uint64_t)s_up[k] * row_bytes));
      };
      int j = 0;
#pragma unroll 4
      for (; j + 2 <= npos; j += 2) {
        const longlong2 v0 = up_val(j), v1 = up_val(j + 1);
        sr += v0.x + v1.x;
        si += v0.y + v1.y;
      }
      if (j < npos) {
        const longlong2 v0 = up_val(j);
        sr += v0.x;
        si += v0.y;
      }
      j = npos;
#pragma unroll 4
      for (; j + 2 <= nu; j += 2) {
        const longlong2 v0 = up_val(j), v1 = up_val(j + 1);
        sr -= v0.x + v1.x;
        si -= v0.y + v1.y;
      }
      if (j < nu) {
        const longlong2 v0 = up_val(j);
        sr -= v0.x;
        si -= v0.y;
      }
      if (!live) continue;
      const longlong2 xv = STAGED ? reinterpret_cast<const longlong2*>(smem)[c] : xrow[c];
      const long long dq = s_cq[__popc(um & __ldg(&v.dn_mask[c]))];
      __int128 pr = (__int128)c1 * sr + (__int128)dq * xv.x;
      __int128 pi = (__int128)c1 * si + (__int128)dq * xv.y;
      const int64_t idx = r * Dd + c;
      if (HAS_Z) {
        const longlong2 zv = z[idx];
        pr += (__int128)c3 * zv.x;
        pi += (__int128)c3 * zv.y;
      }
      longlong2 out;
      out.x = round_shift(pr, sh);
      out.y = round_shift(pi, sh);
      y[idx] = out;
      if (DOTS & 1) a_xy += prod_hi(xv.x, out.x) + prod_hi(xv.y, out.y);
      if (DOTS & 2) a_yy += prod_hi(out.x, out.x) + prod_hi(out.y, out.y);
      if (DOTS & 4) mor |= mag(out.x) | mag(out.y);
    }
  }
  if (TS) asm volatile("cp.async.wait_all;" ::: "memory");
  if (DOTS) q_block_reduce_exact(a_xy, a_yy, mor, reinterpret_cast<long long*>(partials), max_or);
}

static int sm_count() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  return sms > 0 ? sms : 1;
}

static int smem_optin() {
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return v;
}

// ---------------------------------------------------------------------------
// The Q64 apply of a signed-column CSR operator (a momentum sector: every
// off-diagonal entry is +-off, the diagonal apart):
//   P = c1 S + dq x + c3 z   (128-bit),   y = round(P / 2^sh)
// with S the exact int64 sum of +-x over the row's entries (a negative entry
// adds x ^ -1 = -x - 1, its count added back once) and dq = round(2^G scale
// (diag - shift)) the row's fixed-point diagonal, formed here in FP64 once a
// row.  kQCsrLanes lanes a row, 256 threads a block, the fused exact dots as
// in k_apply_q.  The integer hop sums run on the integer pipe, where the
// complex128 kernel's adds wait on this GPU's FP64 pipe.
// ---------------------------------------------------------------------------
constexpr int kQCsrThreads = 256;
constexpr int kQCsrLanes = 8;  // lanes a row unless the operator's shape says otherwise

template <int DOTS, bool HAS_Z, int LPR>
__global__ void __launch_bounds__(kQCsrThreads)
k_csr_apply_q(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
              const double* __restrict__ diag, const longlong2* __restrict__ x, longlong2* y,
              const longlong2* __restrict__ z, const QParams* __restrict__ prm,
              double* __restrict__ partials, unsigned long long* __restrict__ max_or) {
  constexpr int RPW = 32 / LPR;
  const int lane = threadIdx.x & (LPR - 1);
  const int sub = (threadIdx.x & 31) / LPR;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const long long c1 = prm->c1, c3 = prm->c3;
  const int sh = prm->sh, G = prm->G;
  const double scale = prm->scale, shift = prm->shift;
  __int128 a_xy = 0, a_yy = 0;
  unsigned long long mor = 0;
  // the warp steps through its rows together (the shuffles need every lane)
  for (int64_t rb = w0 * RPW; rb < n; rb += nw * RPW) {
    const int64_t row = rb + sub;
    const bool live = row < n;
    long long sr = 0, si = 0;
    int neg = 0;
    if (live) {
      const int64_t k1 = rp[row + 1];
#pragma unroll 4
      for (int64_t k = rp[row] + lane; k < k1; k += LPR) {
        const uint32_t e = (uint32_t)__ldg(&ci[k]);
        const long long m = (int)e >> 31;  // 0 or -1
        const longlong2 v = __ldg(&x[e & 0x7FFFFFFFu]);
        sr += v.x ^ m;
        si += v.y ^ m;
        neg -= (int)m;
      }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
      neg += __shfl_xor_sync(0xffffffffu, neg, o);
    }
    if (live && lane == 0) {
      sr += neg;
      si += neg;
      const longlong2 xv = x[row];
      const long long dq = llrint(ldexp(scale * (diag[row] - shift), G));
      __int128 pr = (__int128)c1 * sr + (__int128)dq * xv.x;
      __int128 pi = (__int128)c1 * si + (__int128)dq * xv.y;
      if (HAS_Z) {
        const longlong2 zv = z[row];
        pr += (__int128)c3 * zv.x;
        pi += (__int128)c3 * zv.y;
      }
      longlong2 out;
      out.x = round_shift(pr, sh);
      out.y = round_shift(pi, sh);
      y[row] = out;
      if (DOTS & 1) a_xy += prod_hi(xv.x, out.x) + prod_hi(xv.y, out.y);
      if (DOTS & 2) a_yy += prod_hi(out.x, out.x) + prod_hi(out.y, out.y);
      if (DOTS & 4) mor |= mag(out.x) | mag(out.y);
    }
  }
  if (DOTS) q_block_reduce_exact(a_xy, a_yy, mor, reinterpret_cast<long long*>(partials), max_or);
}

static int q_csr_lanes(const OpView& v) { return v.csr_lanes ? v.csr_lanes : kQCsrLanes; }

static int q_csr_grid(const OpView& v) {
  const int64_t n = v.dim;
  const int64_t rows_per_block = kQCsrThreads / q_csr_lanes(v);
  int64_t g = (n + rows_per_block - 1) / rows_per_block;
  const int64_t cap = (int64_t)sm_count() * 16;
  if (g > cap) g = cap;
  return (int)(g > 0 ? g : 1);
}

template <int DOTS, bool HAS_Z, int LPR>
static void q_csr_l(const OpView& v, const void* x, void* y, const void* z, const QParams* prm,
                    double* partials, unsigned long long* max_or, cudaStream_t st) {
  k_csr_apply_q<DOTS, HAS_Z, LPR><<<q_csr_grid(v), kQCsrThreads, 0, st>>>(
      v.dim, v.csr_row, v.csr_col, v.csr_diag, (const longlong2*)x, (longlong2*)y,
      (const longlong2*)z, prm, partials, max_or);
  MB_CUDA(cudaGetLastError());
}

template <int DOTS, bool HAS_Z>
static void q_csr_t(const OpView& v, const void* x, void* y, const void* z, const QParams* prm,
                    double* partials, unsigned long long* max_or, cudaStream_t st) {
  switch (q_csr_lanes(v)) {
    case 4: q_csr_l<DOTS, HAS_Z, 4>(v, x, y, z, prm, partials, max_or, st); break;
    case 8: q_csr_l<DOTS, HAS_Z, 8>(v, x, y, z, prm, partials, max_or, st); break;
    case 16: q_csr_l<DOTS, HAS_Z, 16>(v, x, y, z, prm, partials, max_or, st); break;
    default: q_csr_l<DOTS, HAS_Z, 32>(v, x, y, z, prm, partials, max_or, st); break;
  }
}

static void launch_csr_apply_q(const OpView& v, const void* x, void* y, const void* z,
                               const QParams* prm, double* partials, unsigned long long* max_or,
                               int dots, cudaStream_t st) {
  MB_REQUIRE(!v.csr_val, MB_ERR_INVALID_ARG,
             "MB_PREC_Q64 takes only signed-column sparse operators (momentum sectors)");
  if (z) {
    if (dots) q_csr_t<7, true>(v, x, y, z, prm, partials, max_or, st);
    else q_csr_t<0, true>(v, x, y, z, prm, partials, max_or, st);
  } else {
    if (dots) q_csr_t<7, false>(v, x, y, z, prm, partials, max_or, st);
    else q_csr_t<0, false>(v, x, y, z, prm, partials, max_or, st);
  }
}

int q_apply_grid(const OpView& v) {
  if (v.csr_row) return q_csr_grid(v);
  const int split = v.row_split > 1 ? v.row_split : 1;
  int64_t g = sm_count();
  if (g > v.Du * split) g = v.Du * split;
  g -= g % split;
  return (int)std::max<int64_t>(g, split);
}

// the table width a launch uses: 16-bit where the view has the copies
static int q_table_bits(const OpView& v, bool rows) {
  if (v.table_bits != 16) return 32;
  return (rows ? v.dn_sell16 : v.up_sell16) ? 16 : 32;
}

// dynamic shared memory of a launch: the staged row and pads, the up list,
// and with TS the warps' table buffers
static size_t q_apply_smem(const OpView& v, bool staged, bool ups, bool ts) {
  size_t smem = ups ? 0 : sizeof(uint32_t) * (size_t)((v.max_up_list + 3) & ~3);
  if (staged) smem += sizeof(longlong2) * (size_t)(v.Dd + kSlicedPads);
  if (ts) smem += (size_t)(kQThreads / 32) * (size_t)v.dn_max_words * 512;
  return smem;
}

template <bool STAGED, int DOTS, bool HAS_Z, bool UPS, int TB, bool TS = false>
static void q_apply_t(const OpView& v, const void* x, void* y, const void* z, const QParams* prm,
                      double* partials, unsigned long long* max_or, const void* ups,
                      cudaStream_t st) {
  const size_t smem = q_apply_smem(v, STAGED, UPS, TS);
  auto kern = k_apply_q<STAGED, DOTS, HAS_Z, UPS, TB, TS>;
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<q_apply_grid(v), kQThreads, smem, st>>>(v, (const longlong2*)x, (longlong2*)y,
                                                   (const longlong2*)z, prm, partials, max_or,
                                                   (const longlong2*)ups);
  MB_CUDA(cudaGetLastError());
}

template <bool STAGED, bool UPS, int TB>
static void q_apply_sel(const OpView& v, const void* x, void* y, const void* z,
                        const QParams* prm, double* partials, unsigned long long* max_or,
                        int dots, const void* ups, cudaStream_t st) {
  if (z) {
    if (dots == 5) q_apply_t<STAGED, 5, true, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
    else if (dots) q_apply_t<STAGED, 7, true, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
    else q_apply_t<STAGED, 0, true, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
  } else {
    if (dots == 5) q_apply_t<STAGED, 5, false, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
    else if (dots) q_apply_t<STAGED, 7, false, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
    else q_apply_t<STAGED, 0, false, UPS, TB>(v, x, y, z, prm, partials, max_or, ups, st);
  }
}

// the table-staged one-pass apply: where the warps' buffers fit beside the row
bool q_table_stage_fits(const OpView& v) {
  return v.dn_max_words > 0 &&
         q_apply_smem(v, true, false, true) + 2048 <= (size_t)smem_optin();
}

static void q_apply_ts(const OpView& v, const void* x, void* y, const void* z,
                       const QParams* prm, double* partials, unsigned long long* max_or,
                       int dots, cudaStream_t st) {
  if (z) {
    if (dots) q_apply_t<true, 7, true, false, 32, true>(v, x, y, z, prm, partials, max_or, nullptr, st);
    else q_apply_t<true, 0, true, false, 32, true>(v, x, y, z, prm, partials, max_or, nullptr, st);
  } else {
    if (dots) q_apply_t<true, 7, false, false, 32, true>(v, x, y, z, prm, partials, max_or, nullptr, st);
    else q_apply_t<true, 0, false, false, 32, true>(v, x, y, z, prm, partials, max_or, nullptr, st);
  }
}

template <bool STAGED, bool UPS>
static void q_apply_tb(const OpView& v, const void* x, void* y, const void* z,
                       const QParams* prm, double* partials, unsigned long long* max_or,
                       int dots, const void* ups, cudaStream_t st) {
  if (STAGED && !UPS && v.table_stage && q_table_bits(v, true) == 32 && q_table_stage_fits(v)) {
    q_apply_ts(v, x, y, z, prm, partials, max_or, dots, st);
    return;
  }
  if (q_table_bits(v, true) == 16)
    q_apply_sel<STAGED, UPS, 16>(v, x, y, z, prm, partials, max_or, dots, ups, st);
  else q_apply_sel<STAGED, UPS, 32>(v, x, y, z, prm, partials, max_or, dots, ups, st);
}

bool q_upcol_fits(const OpView& v) {
  const int64_t Du = v.dim / v.Dd;
  return sizeof(longlong2) * (size_t)(Du + kSlicedPads) + 1024 <= (size_t)smem_optin() &&
         v.up_sell != nullptr;
}

template <int TB>
static void upcol_t(const OpView& v, const void* x, void* ups, cudaStream_t st) {
  const int64_t Du = v.dim / v.Dd;
  const size_t smem = sizeof(longlong2) * (size_t)(Du + kSlicedPads);
  MB_CUDA(cudaFuncSetAttribute(k_upcol_q<TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem));
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(sm_count(), v.Dd));
  k_upcol_q<TB><<<grid, kQColThreads, smem, st>>>(v, (const longlong2*)x, (longlong2*)ups);
  MB_CUDA(cudaGetLastError());
}

void launch_upcol_q(const OpView& v, const void* x, void* ups, cudaStream_t st) {
  if (q_table_bits(v, false) == 16) upcol_t<16>(v, x, ups, st);
  else upcol_t<32>(v, x, ups, st);
}

void launch_apply_q(const OpView& v, const void* x, void* y, const void* z, const QParams* prm,
                    double* partials, unsigned long long* max_or, int dots, cudaStream_t st,
                    const void* ups) {
  if (v.csr_row) {
    launch_csr_apply_q(v, x, y, z, prm, partials, max_or, dots, st);
    return;
  }
  const size_t row = sizeof(longlong2) * (size_t)(v.Dd + kSlicedPads) + 2048;
  const size_t lists = sizeof(uint32_t) * (size_t)((v.max_up_list + 3) & ~3);
  if (ups) {
    // the rows of the whole sector in index order (concurrent rows read
    // neighbouring elements of the column-major up sums); a row group keeps
    // its own schedule
    OpView w = v;
    if (w.Du == w.dim / w.Dd) w.row_sched = nullptr;
    if (row <= (size_t)smem_optin()) q_apply_tb<true, true>(w, x, y, z, prm, partials, max_or, dots, ups, st);
    else q_apply_tb<false, true>(w, x, y, z, prm, partials, max_or, dots, ups, st);
    return;
  }
  if (row + lists <= (size_t)smem_optin())
    q_apply_tb<true, false>(v, x, y, z, prm, partials, max_or, dots, nullptr, st);
  else q_apply_tb<false, false>(v, x, y, z, prm, partials, max_or, dots, nullptr, st);
}

// ---------------------------------------------------------------------------
// Parameter planning (host and device): fixed-point coefficients for
// y = scale (H - shift) x + beta z given the exponents of x and z.
// ---------------------------------------------------------------------------
__host__ __device__ static int ceil_log2_pos(double v) {
  // smallest k with v <= 2^k (v > 0)
  int e;
  const double m = frexp(v, &e);  // v = m * 2^e, m in [0.5, 1)
  return (m == 0.5) ? e - 1 : e;
}

__host__ __device__ void q_plan(QParams* p, const QPlanInput& in) {
  const double c1r = -in.t * in.scale;
  double maxcq = 0.0;
  for (int k = 0; k <= in.L; ++k) {
    const double cq = in.scale * (in.ufold[k] - in.shift);
    maxcq = fmax(maxcq, fabs(cq));
  }
  const double c3r = in.has_z ? in.beta * ldexp(1.0, in.ez - in.ex) : 0.0;
  const double maxc = fmax(fmax(fabs(c1r), maxcq), fabs(c3r));
  const double bound = (fabs(c1r) * in.w_max + maxcq) * in.x_frac + fabs(c3r) * in.z_frac;
  int G = 60;
  if (maxc > 0.0) G = 61 - ceil_log2_pos(maxc);
  int ey = in.ex;
  if (bound > 0.0) ey = in.ex + ceil_log2_pos(bound);
  p->c1 = llrint(ldexp(c1r, G));
  for (int k = 0; k <= in.L; ++k) p->cq[k] = llrint(ldexp(in.scale * (in.ufold[k] - in.shift), G));
  for (int k = in.L + 1; k <= kMaxOrbitals; ++k) p->cq[k] = 0;
  p->c3 = in.has_z ? llrint(ldexp(c3r, G)) : 0;
  p->G = G;
  p->scale = in.scale;
  p->shift = in.shift;
  p->ex = in.ex;
  p->ey = ey;
  p->ez = in.ez;
  p->sh = G + ey - in.ex;
}

// ---------------------------------------------------------------------------
// Conversions, with optional permutation (reference <-> tensor order).
// ---------------------------------------------------------------------------
constexpr int kQBlas = 256;

int q_blas_grid(int64_t n) {
  int64_t g = (n + kQBlas - 1) / kQBlas;
  const int64_t cap = (int64_t)sm_count() * 8;
  if (g > cap) g = cap;
  return (int)std::max<int64_t>(g, 1);
}

// max biased exponent over all components of a complex128 vector
__global__ void k_f64_maxexp(int64_t n, const double2* __restrict__ x, int* __restrict__ out) {
  int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = x[i];
    const int ea = (int)(((unsigned long long)__double_as_longlong(v.x) >> 52) & 0x7FF);
    const int eb = (int)(((unsigned long long)__double_as_longlong(v.y) >> 52) & 0x7FF);
    m = max(m, max(ea, eb));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// Ex from the max biased exponent: |x| < 2^(emax - 1022) -> Ex = that - qbits.
__global__ void k_exp_from_max(const int* __restrict__ emax, int qbits, int* __restrict__ ex) {
  const int e = *emax;
  *ex = (e == 0) ? -1074 : (e - 1022 - qbits);
}

__global__ void k_to_fixed(int64_t n, const double2* __restrict__ src, const int32_t* __restrict__ perm,
                           const int* __restrict__ ex, longlong2* __restrict__ dst) {
  const int E = *ex;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = src[perm ? (int64_t)perm[i] : i];
    dst[i] = make_longlong2(f64_to_fixed(v.x, E), f64_to_fixed(v.y, E));
  }
}

// dst[i] = value(src[iperm ? iperm[i] : i]) (iperm: reference -> tensor index)
__global__ void k_from_fixed(int64_t n, const longlong2* __restrict__ src,
                             const int32_t* __restrict__ iperm, const int* __restrict__ ey,
                             double2* __restrict__ dst) {
  const int E = *ey;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 q = src[iperm ? (int64_t)iperm[i] : i];
    dst[i] = make_double2(fixed_to_f64(q.x, E), fixed_to_f64(q.y, E));
  }
}

// Reference-order chunk -> tensor order (dst[iperm[i]] = src[i]), with the
// chunk's largest biased exponent folded into *emax: the landing step of a
// host-buffer apply, run on each chunk while the next one is in flight.
__global__ void k_scatter_maxexp(int64_t n, const double2* __restrict__ src,
                                 const int32_t* __restrict__ iperm, double2* __restrict__ dst,
                                 int* __restrict__ emax) {
  int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = src[i];
    dst[iperm[i]] = v;
    const int ea = (int)(((unsigned long long)__double_as_longlong(v.x) >> 52) & 0x7FF);
    const int eb = (int)(((unsigned long long)__double_as_longlong(v.y) >> 52) & 0x7FF);
    m = max(m, max(ea, eb));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(emax, m);
}

// complex128 -> Q64 in place (the same 16 bytes per element)
__global__ void k_to_fixed_inplace(int64_t n, void* buf, const int* __restrict__ ex) {
  const int E = *ex;
  double2* d = reinterpret_cast<double2*>(buf);
  longlong2* q = reinterpret_cast<longlong2*>(buf);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = d[i];
    q[i] = make_longlong2(f64_to_fixed(v.x, E), f64_to_fixed(v.y, E));
  }
}

// One-thread planner on the device (keeps mb_op_apply asynchronous).
__global__ void k_plan(QPlanInput in, const int* __restrict__ ex, QParams* __restrict__ p) {
  in.ex = *ex;
  in.ez = in.ex;
  q_plan(p, in);
}

void launch_f64_to_q(int64_t n, const void* src, const int32_t* perm, int qbits, int* scratch_int2,
                     void* dst, cudaStream_t st) {
  MB_CUDA(cudaMemsetAsync(scratch_int2, 0, sizeof(int), st));
  k_f64_maxexp<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const double2*)src, scratch_int2);
  k_exp_from_max<<<1, 1, 0, st>>>(scratch_int2, qbits, scratch_int2 + 1);
  k_to_fixed<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const double2*)src, perm, scratch_int2 + 1,
                                                 (longlong2*)dst);
  MB_CUDA(cudaGetLastError());
}

void launch_scatter_maxexp(int64_t n, const void* src, const int32_t* iperm, void* dst,
                           int* emax, cudaStream_t st) {
  if (n <= 0) return;
  k_scatter_maxexp<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const double2*)src, iperm,
                                                       (double2*)dst, emax);
  MB_CUDA(cudaGetLastError());
}

void launch_f64_to_q_inplace(int64_t n, void* buf, int qbits, int* scratch_int2, cudaStream_t st) {
  k_exp_from_max<<<1, 1, 0, st>>>(scratch_int2, qbits, scratch_int2 + 1);
  k_to_fixed_inplace<<<q_blas_grid(n), kQBlas, 0, st>>>(n, buf, scratch_int2 + 1);
  MB_CUDA(cudaGetLastError());
}

void launch_q_to_f64(int64_t n, const void* src, const int32_t* iperm, const int* e_dev, void* dst,
                     cudaStream_t st) {
  k_from_fixed<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const longlong2*)src, iperm, e_dev,
                                                   (double2*)dst);
  MB_CUDA(cudaGetLastError());
}

void launch_q_plan(const QPlanInput& in, const int* ex_dev, QParams* p_dev, cudaStream_t st) {
  k_plan<<<1, 1, 0, st>>>(in, ex_dev, p_dev);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Vector kernels on mantissas.
//   out = round((A a + B b) / 2^sh), A, B complex fixed-point (re, im), b optional;
//   partials: <out,out>>>32 ; max_or: OR of |out| components.
// ---------------------------------------------------------------------------
// REAL: both coefficients real (ai = bi = 0; the Lanczos recurrence), half
// the 128-bit products, the same integers
template <bool REAL>
__global__ void k_q_lincomb(int64_t n, const longlong2* a, long long ar, long long ai,
                            const longlong2* b, long long br, long long bi, int sh,
                            longlong2* out, double* __restrict__ partials,
                            unsigned long long* __restrict__ max_or) {
  __int128 nn = 0;
  unsigned long long mor = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 va = a ? a[i] : make_longlong2(0, 0);
    __int128 pr = (__int128)ar * va.x, pi = (__int128)ar * va.y;
    if (!REAL) {
      pr -= (__int128)ai * va.y;
      pi += (__int128)ai * va.x;
    }
    if (b) {
      const longlong2 vb = b[i];
      pr += (__int128)br * vb.x;
      pi += (__int128)br * vb.y;
      if (!REAL) {
        pr -= (__int128)bi * vb.y;
        pi += (__int128)bi * vb.x;
      }
    }
    longlong2 o;
    o.x = round_shift(pr, sh);
    o.y = round_shift(pi, sh);
    out[i] = o;
    nn += prod_hi(o.x, o.x) + prod_hi(o.y, o.y);
    mor |= mag(o.x) | mag(o.y);
  }
  if (partials || max_or) {
    double vals[2] = {i128_to_f64(nn), 0.0};
    q_block_reduce<2>(vals, mor, partials, max_or);
  }
}

void launch_q_lincomb(int64_t n, const void* a, long long ar, long long ai, const void* b,
                      long long br, long long bi, int sh, void* out, double* partials,
                      unsigned long long* max_or, cudaStream_t st) {
  if (ai == 0 && bi == 0)
    k_q_lincomb<true><<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const longlong2*)a, ar, ai,
                                                         (const longlong2*)b, br, bi, sh,
                                                         (longlong2*)out, partials, max_or);
  else
    k_q_lincomb<false><<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const longlong2*)a, ar, ai,
                                                          (const longlong2*)b, br, bi, sh,
                                                          (longlong2*)out, partials, max_or);
  MB_CUDA(cudaGetLastError());
}

// Re/Im <a, b> = sum conj(a) b as exact integer sums >> 32 -> partials[2].
__global__ void k_q_dot(int64_t n, const longlong2* __restrict__ a, const longlong2* __restrict__ b,
                        double* __restrict__ partials) {
  __int128 re = 0, im = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 u = a[i], w = b[i];
    re += prod_hi(u.x, w.x) + prod_hi(u.y, w.y);
    im += prod_hi(u.x, w.y) - prod_hi(u.y, w.x);
  }
  double vals[2] = {i128_to_f64(re), i128_to_f64(im)};
  q_block_reduce<2>(vals, 0ull, partials, nullptr);
}

void launch_q_dot(int64_t n, const void* a, const void* b, double* partials, cudaStream_t st) {
  k_q_dot<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const longlong2*)a, (const longlong2*)b, partials);
  MB_CUDA(cudaGetLastError());
}

// Re-orthogonalisation against a stored basis of Q64 vectors V_j (exponents
// per column).  c_j = <V_j, w> per block partials [blocks][2m].
constexpr int kQmdChunk = 512;
constexpr int kQmdThreads = 256;
constexpr int kQmdBatch = 8;  // loads in flight per lane in the multi-vector kernels

__global__ void __launch_bounds__(kQmdThreads)
k_q_multi_dot(int64_t n, const longlong2* __restrict__ V, int64_t ld, int m,
              const longlong2* __restrict__ w, double* __restrict__ partials) {
  __shared__ double acc[2 * kQMaxBasis];
  __shared__ longlong2 sw[kQmdChunk];
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) acc[j] = 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t base = (int64_t)blockIdx.x * kQmdChunk; base < n;
       base += (int64_t)gridDim.x * kQmdChunk) {
    const int len = (int)((n - base) < kQmdChunk ? (n - base) : kQmdChunk);
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x) sw[i] = w[base + i];
    __syncthreads();
    for (int j = warp; j < m; j += nwarps) {
      const longlong2* vj = V + (int64_t)j * ld + base;
      __int128 cr = 0, ci = 0;
      // kQmdBatch basis elements loaded before any is used: HBM loads in flight
      for (int i0 = lane; i0 < len; i0 += 32 * kQmdBatch) {
        longlong2 a[kQmdBatch];
#pragma unroll
        for (int u = 0; u < kQmdBatch; ++u)
          if (i0 + 32 * u < len) a[u] = vj[i0 + 32 * u];
#pragma unroll
        for (int u = 0; u < kQmdBatch; ++u) {
          if (i0 + 32 * u >= len) break;
          const longlong2 b = sw[i0 + 32 * u];
          cr += prod_hi(a[u].x, b.x) + prod_hi(a[u].y, b.y);
          ci += prod_hi(a[u].x, b.y) - prod_hi(a[u].y, b.x);
        }
      }
      double dr = i128_to_f64(cr), di = i128_to_f64(ci);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dr += __shfl_down_sync(0xffffffffu, dr, o);
        di += __shfl_down_sync(0xffffffffu, di, o);
      }
      if (lane == 0) {
        acc[2 * j] += dr;
        acc[2 * j + 1] += di;
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x)
    partials[(size_t)blockIdx.x * 2 * m + j] = acc[j];
}

int q_multi_dot_grid(int64_t n) {
  int64_t g = (n + kQmdChunk - 1) / kQmdChunk;
  const int64_t cap = (int64_t)sm_count() * 3;  // three CTAs per SM fit (80 registers)
  if (g > cap) g = cap;
  return (int)std::max<int64_t>(g, 1);
}

void launch_q_multi_dot(int64_t n, const void* V, int64_t ld, int m, const void* w,
                        double* partials, cudaStream_t st) {
  MB_REQUIRE(m <= kQMaxBasis, MB_ERR_CAPACITY, "re-orthogonalisation basis larger than 1024");
  k_q_multi_dot<<<q_multi_dot_grid(n), kQmdThreads, 0, st>>>(n, (const longlong2*)V, ld, m,
                                                             (const longlong2*)w, partials);
  MB_CUDA(cudaGetLastError());
}

// w = round((w - sum_j c_j V_j) / 2^shw), c_j fixed point (re, im) at scale
// 2^-G in w-mantissa units; the caller adds shw to w's exponent.
__global__ void __launch_bounds__(kQBlas)
k_q_multi_axpy(int64_t n, const longlong2* __restrict__ V, int64_t ld, int m,
               const long long* __restrict__ c, int G, int shw, longlong2* __restrict__ w,
               double* __restrict__ partials, unsigned long long* __restrict__ max_or) {
  __shared__ long long sc[2 * kQMaxBasis];
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) sc[j] = c[j];
  __syncthreads();
  __int128 nn = 0;
  unsigned long long mor = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const longlong2 wv = w[i];
    __int128 sr = (__int128)wv.x << G, si = (__int128)wv.y << G;
    for (int j0 = 0; j0 < m; j0 += kQmdBatch) {
      longlong2 a[kQmdBatch];
#pragma unroll
      for (int u = 0; u < kQmdBatch; ++u)
        if (j0 + u < m) a[u] = V[(int64_t)(j0 + u) * ld + i];
#pragma unroll
      for (int u = 0; u < kQmdBatch; ++u) {
        if (j0 + u >= m) break;
        const long long cr = sc[2 * (j0 + u)], ci = sc[2 * (j0 + u) + 1];
        sr -= (__int128)cr * a[u].x - (__int128)ci * a[u].y;
        si -= (__int128)cr * a[u].y + (__int128)ci * a[u].x;
      }
    }
    longlong2 o;
    o.x = round_shift(sr, G + shw);
    o.y = round_shift(si, G + shw);
    w[i] = o;
    nn += prod_hi(o.x, o.x) + prod_hi(o.y, o.y);
    mor |= mag(o.x) | mag(o.y);
  }
  double vals[2] = {i128_to_f64(nn), 0.0};
  q_block_reduce<2>(vals, mor, partials, max_or);
}

void launch_q_multi_axpy(int64_t n, const void* V, int64_t ld, int m, const long long* c, int G,
                         int shw, void* w, double* partials, unsigned long long* max_or,
                         cudaStream_t st) {
  MB_REQUIRE(m <= kQMaxBasis, MB_ERR_CAPACITY, "re-orthogonalisation basis larger than 1024");
  k_q_multi_axpy<<<q_blas_grid(n), kQBlas, 0, st>>>(n, (const longlong2*)V, ld, m, c, G, shw,
                                                    (longlong2*)w, partials, max_or);
  MB_CUDA(cudaGetLastError());
}

}  // namespace mb
