// Batched / served solver engine: many independent Hubbard sectors of uneven
// size advanced together, one Lanczos (or Chebyshev) step of every active
// slot per engine step.
//
// Layout.  A slot owns FP32 complex vectors (three rotating Lanczos buffers
// and a Ritz accumulator) and per-step FP64 alpha/beta arrays, all on the
// device; sector tables (masks, hop tables) are shared by every slot with the
// same lattice and filling.  A step is a fixed sequence of grouped kernels
// over a flat work list of (slot, row r_up) items -- one warp per item, so
// sectors from 3k to 12M states mix in one launch -- and per-slot fixed-order
// reductions (deterministic: a slot's result does not depend on what else
// runs).  alpha and beta never leave the device inside a step, so a fixed
// batch is captured once as a CUDA graph and replayed; the serving loop
// instead reads alpha/beta after each step to test convergence and to admit
// and retire requests.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "mb_internal.h"

namespace mb {

constexpr int kEngMaxK = 512;  // Lanczos steps a slot can record
// a slot's scalar table: alpha, beta, yk (kEngMaxK doubles each), the start
// vector's norm, then 1 / beta_k as floats (kEngMaxK)
constexpr int kEngNormAt = 3 * kEngMaxK;
constexpr size_t kEngIbAt = sizeof(double) * (size_t)(kEngNormAt + 1);
constexpr size_t kEngScalBytes = kEngIbAt + sizeof(float) * (size_t)kEngMaxK;

// Device descriptor of one slot (POD).
struct SlotDesc {
  const uint32_t* up_mask;
  const uint32_t* dn_mask;
  const int32_t* up_off;
  const uint32_t* up_ent;
  const int32_t* dn_off;
  const uint32_t* dn_ent;
  int64_t Du, Dd;
  float2* buf[3];   // Lanczos vectors: v_prev = buf[k%3], v = buf[(k+1)%3], w = buf[(k+2)%3]
  float2* xacc;     // Ritz vector accumulator (replay pass)
  double* alpha;    // [kEngMaxK]
  double* beta;     // [kEngMaxK]
  double* yk;       // Ritz coefficients for the replay pass [kEngMaxK]
  float* ib;        // (float)(1 / beta_k) [kEngMaxK]: the persistent step's deferred normalisation
  float ufold[kMaxOrbitals + 1];
  float t;
  float scale;      // Lanczos: -1 Negated H (ground state), +1 H
  float cheb_a;     // Chebyshev mode: Ht = (H - cheb_b) / cheb_a
  float cheb_b;
  int kmax;         // pass one: steps to run at most
  int k;            // this slot's step counter
  int mode;         // kModeIdle, kModeLanczos, kModeReplay
  int steps;        // pass-one steps taken (m)
  int item0, item1; // this slot's range of work items (partials at item0 + row)
  int fused;        // applied by the fused kernel (large sectors), not k_eng_apply
  // the sector's fused-apply tables (row-staged kernel): sign-sorted up
  // lists and the sliced down table
  const uint32_t* up_list;
  const int32_t* up_loff;
  const int32_t* up_lpos;
  const uint32_t* dn_sell;
  const int32_t* dn_sgrp;
  // diagonal self energies of lattices with a size-1 dimension (t times the
  // sector's t = 1 values, per up / down state), else nullptr
  const float* self_up;
  const float* self_dn;
  // the Lanczos vectors v_0, v_1, ... of pass one (kmax x dim), kept when the
  // request's basis fits the engine's limit: the Ritz vector is then summed
  // from them instead of replaying the recurrence; else nullptr
  float2* basis;
};

constexpr int kModeIdle = kEngIdle;
constexpr int kModeLanczos = kEngLanczos;
constexpr int kModeReplay = kEngReplay;
constexpr int kModeCheb = kEngCheb;   // T_{k+1} = 2 Ht T_k - T_{k-1} (T_1 = Ht T_0)

// ---------------------------------------------------------------------------
// Kernels.  One warp per (slot, row) item; lanes stride over the row.
// ---------------------------------------------------------------------------
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_eng_apply(const SlotDesc* __restrict__ slots, const int2* __restrict__ items, int n_items,
            double* __restrict__ part, double* __restrict__ part2) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < n_items; it += gridDim.x * WARPS) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    if (s.fused) continue;  // its partials come from the fused kernel
    const int k = s.k;
    const bool replay = s.mode == kModeReplay;
    const bool cheb = s.mode == kModeCheb;
    double dxy = 0.0, dyy = 0.0;
    if ((s.mode == kModeLanczos && k < s.kmax) || (replay && k + 1 < s.steps) ||
        (cheb && k < s.kmax)) {
      const int64_t r = item.y, Dd = s.Dd;
      const float2* v = s.buf[(k + 1) % 3] + r * Dd;
      const float2* x = s.buf[(k + 1) % 3];
      const float2* z = s.buf[k % 3] + r * Dd;
      float2* w = s.buf[(k + 2) % 3] + r * Dd;
      // Lanczos: w = scale (H v) - beta_{k-1} v_prev   (lanczos.h:25-31)
      // Chebyshev: w = c (H - b) v - [k > 0] v_prev, c = 1/a (k = 0) or 2/a (kpm.h:218-223)
      const double bprev = cheb ? 1.0 : (k > 0 ? s.beta[k - 1] : 0.0);
      const float beta = (float)(-bprev);
      const float sc = cheb ? (k == 0 ? 1.f : 2.f) / s.cheb_a : s.scale;
      const float shift = cheb ? s.cheb_b : 0.f;
      const float hop = -s.t * sc;
      float hi2 = 0.f, lo2 = 0.f;
      const uint32_t um = s.up_mask[r];
      const int u0 = s.up_off[r], u1 = s.up_off[r + 1];
      float hi = 0.f, lo = 0.f;
      for (int64_t c = lane; c < Dd; c += 32) {
        float ar = 0.f, ai = 0.f;
        for (int j = s.dn_off[c]; j < s.dn_off[c + 1]; ++j) {
          const uint32_t e = __ldg(&s.dn_ent[j]);
          const float2 val = v[e >> 8];
          float wgt = (e & 2u) ? 2.f : 1.f;
          if (e & 1u) wgt = -wgt;
          ar = fmaf(wgt, val.x, ar);
          ai = fmaf(wgt, val.y, ai);
        }
        for (int j = u0; j < u1; ++j) {
          const uint32_t e = __ldg(&s.up_ent[j]);
          const float2 val = x[(int64_t)(e >> 8) * Dd + c];
          float wgt = (e & 2u) ? 2.f : 1.f;
          if (e & 1u) wgt = -wgt;
          ar = fmaf(wgt, val.x, ar);
          ai = fmaf(wgt, val.y, ai);
        }
        const float2 xv = v[c];
        const float d = sc * (s.ufold[__popc(um & s.dn_mask[c])] +
                            (s.self_up ? s.self_up[r] + s.self_dn[c] : 0.f) - shift);
        float2 o;
        o.x = fmaf(hop, ar, d * xv.x);
        o.y = fmaf(hop, ai, d * xv.y);
        if (k > 0) {
          const float2 zv = z[c];
          o.x = fmaf(beta, zv.x, o.x);
          o.y = fmaf(beta, zv.y, o.y);
        }
        w[c] = o;
        if (!replay) {
          // compensated Re<v, w> (exact float products, TwoSum)
          float p = xv.x * o.x, pe = fmaf(xv.x, o.x, -p);
          float s1 = hi + p, bp = s1 - hi;
          lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
          hi = s1;
          p = xv.y * o.y;
          pe = fmaf(xv.y, o.y, -p);
          s1 = hi + p;
          bp = s1 - hi;
          lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
          hi = s1;
        }
        if (cheb) {  // <T_{k+1}, T_{k+1}>
          float p = o.x * o.x, pe = fmaf(o.x, o.x, -p);
          float s1 = hi2 + p, bp = s1 - hi2;
          lo2 += ((hi2 - (s1 - bp)) + (p - bp)) + pe;
          hi2 = s1;
          p = o.y * o.y;
          pe = fmaf(o.y, o.y, -p);
          s1 = hi2 + p;
          bp = s1 - hi2;
          lo2 += ((hi2 - (s1 - bp)) + (p - bp)) + pe;
          hi2 = s1;
        }
      }
      dxy = (double)hi + (double)lo;
      dyy = (double)hi2 + (double)lo2;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        dxy += __shfl_down_sync(0xffffffffu, dxy, o);
        dyy += __shfl_down_sync(0xffffffffu, dyy, o);
      }
    }
    if (lane == 0 && part) {
      part[s.item0 + item.y] = dxy;
      part2[s.item0 + item.y] = dyy;
    }
  }
}

// Rows of medium sectors, a block per (slot, row), as the operators' fused
// apply does it: the row of v (and the zero padding elements) and the row's
// sign-sorted up list staged in shared memory; warps take the row's 32-column
// groups; down hops gather from the staged row through the sliced table (four
// slots per 16-byte load), up hops are coalesced loads of the listed rows,
// added then subtracted; the step arithmetic and compensated partials of
// k_eng_apply.
constexpr int kEngRowWarps = 8;
constexpr int64_t kEngRowMinCols = 256;  // rows this wide and wider

__global__ void __launch_bounds__(kEngRowWarps * 32)
k_eng_apply_rows(const SlotDesc* __restrict__ slots, const int2* __restrict__ items, int n_items,
                 int max_cols, double* __restrict__ part, double* __restrict__ part2) {
  extern __shared__ __align__(16) unsigned char smem[];
  float2* srow = reinterpret_cast<float2*>(smem);
  uint32_t* s_up = reinterpret_cast<uint32_t*>(smem + sizeof(float2) * (max_cols + kSlicedPads));
  __shared__ double red[kEngRowWarps][2];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x; it < n_items; it += gridDim.x) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    const int k = s.k;
    const bool lanczos = s.mode == kModeLanczos && k < s.kmax;
    const bool replay = s.mode == kModeReplay && k + 1 < s.steps;
    const bool cheb = s.mode == kModeCheb && k < s.kmax;
    const int64_t pidx = s.item0 + item.y;
    if (!(lanczos || replay || cheb)) {  // uniform over the block
      if (threadIdx.x == 0) {
        part[pidx] = 0.0;
        part2[pidx] = 0.0;
      }
      continue;
    }
    const int64_t r = item.y, Dd = s.Dd;
    const uint64_t row_bytes = sizeof(float2) * (uint64_t)Dd;
    const float2* x = s.buf[(k + 1) % 3];
    const float2* v = x + r * Dd;
    const float2* z = s.buf[k % 3] + r * Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    const double bprev = cheb ? 1.0 : (k > 0 ? s.beta[k - 1] : 0.0);
    const float beta = (float)(-bprev);
    const float sc = cheb ? (k == 0 ? 1.f : 2.f) / s.cheb_a : s.scale;
    const float shift = cheb ? s.cheb_b : 0.f;
    const float hop = -s.t * sc;
    const uint32_t um = s.up_mask[r];
    const int u0 = __ldg(&s.up_loff[r]), nu = __ldg(&s.up_loff[r + 1]) - u0;
    const int npos = __ldg(&s.up_lpos[r]);
    __syncthreads();  // the previous item's readers are done with srow / s_up
    for (int64_t c = threadIdx.x; c < Dd; c += blockDim.x) srow[c] = v[c];
    if (threadIdx.x < kSlicedPads) srow[Dd + threadIdx.x] = make_float2(0.f, 0.f);
    for (int j = threadIdx.x; j < nu; j += blockDim.x) s_up[j] = __ldg(&s.up_list[u0 + j]);
    __syncthreads();
    float hi = 0.f, lo = 0.f, hi2 = 0.f, lo2 = 0.f;
    const int64_t ngroups = (Dd + 31) >> 5;
    for (int64_t g = warp; g < ngroups; g += kEngRowWarps) {
      const int64_t c = (g << 5) + lane;
      const bool live = c < Dd;
      const int64_t cl = live ? c : Dd - 1;
      float ar = 0.f, ai = 0.f;
      const int2 gi = __ldg(reinterpret_cast<const int2*>(s.dn_sgrp) + g);
      const uint4* ep = reinterpret_cast<const uint4*>(s.dn_sell + gi.x) + lane;
      auto dn = [&](uint32_t e) {
        const float2 val = srow[e & 0x7FFFFFFFu];
        const float wgt = __int_as_float((int)(0x3f800000u | (e & 0x80000000u)));
        ar = fmaf(wgt, val.x, ar);
        ai = fmaf(wgt, val.y, ai);
      };
      for (int j = 0; j < gi.y; j += 4) {
        const uint4 e = __ldg(ep + 8 * j);
        dn(e.x);
        dn(e.y);
        dn(e.z);
        dn(e.w);
      }
      const char* xc = reinterpret_cast<const char*>(x + cl);
      auto up = [&](int q) {
        return __ldg(reinterpret_cast<const float2*>(xc + (uint64_t)s_up[q] * row_bytes));
      };
      float pr = 0.f, pi = 0.f, nr = 0.f, ni = 0.f;
      int j = 0;
#pragma unroll 4
      for (; j < npos; ++j) {
        const float2 val = up(j);
        pr += val.x;
        pi += val.y;
      }
#pragma unroll 4
      for (; j < nu; ++j) {
        const float2 val = up(j);
        nr += val.x;
        ni += val.y;
      }
      ar += pr - nr;
      ai += pi - ni;
      if (!live) continue;
      const float2 xv = srow[c];
      const float d = sc * (s.ufold[__popc(um & s.dn_mask[c])] +
                            (s.self_up ? s.self_up[r] + s.self_dn[c] : 0.f) - shift);
      float2 o;
      o.x = fmaf(hop, ar, d * xv.x);
      o.y = fmaf(hop, ai, d * xv.y);
      if (k > 0) {
        const float2 zv = z[c];
        o.x = fmaf(beta, zv.x, o.x);
        o.y = fmaf(beta, zv.y, o.y);
      }
      w[c] = o;
      if (!replay) {  // compensated Re<v, w> (exact float products, TwoSum)
        float p = xv.x * o.x, pe = fmaf(xv.x, o.x, -p);
        float s1 = hi + p, bp = s1 - hi;
        lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
        hi = s1;
        p = xv.y * o.y;
        pe = fmaf(xv.y, o.y, -p);
        s1 = hi + p;
        bp = s1 - hi;
        lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
        hi = s1;
      }
      if (cheb) {  // <T_{k+1}, T_{k+1}>
        float p = o.x * o.x, pe = fmaf(o.x, o.x, -p);
        float s1 = hi2 + p, bp = s1 - hi2;
        lo2 += ((hi2 - (s1 - bp)) + (p - bp)) + pe;
        hi2 = s1;
        p = o.y * o.y;
        pe = fmaf(o.y, o.y, -p);
        s1 = hi2 + p;
        bp = s1 - hi2;
        lo2 += ((hi2 - (s1 - bp)) + (p - bp)) + pe;
        hi2 = s1;
      }
    }
    double dxy = (double)hi + (double)lo, dyy = (double)hi2 + (double)lo2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dxy += __shfl_down_sync(0xffffffffu, dxy, o);
      dyy += __shfl_down_sync(0xffffffffu, dyy, o);
    }
    if (lane == 0) {
      red[warp][0] = dxy;
      red[warp][1] = dyy;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // fixed order over the warps
      double a = 0.0, b = 0.0;
      for (int q = 0; q < kEngRowWarps; ++q) {
        a += red[q][0];
        b += red[q][1];
      }
      part[pidx] = a;
      part2[pidx] = b;
    }
  }
}

// Per-slot fixed-order sum of item partials into alpha[k] (what = 0) or
// beta[k] = sqrt(sum) (what = 1).
__global__ void k_eng_seg_reduce(SlotDesc* __restrict__ slots, int n_slots,
                                 const double* __restrict__ part, const double* __restrict__ part2,
                                 int what) {
  for (int si = blockIdx.x; si < n_slots; si += gridDim.x) {
    SlotDesc& s = slots[si];
    const int k = s.k;
    const bool cheb = s.mode == kModeCheb && what == 0;
    __shared__ double red[256], red2[256];
    double a = 0.0, b = 0.0;
    for (int it = s.item0 + threadIdx.x; it < s.item1; it += blockDim.x) {
      a += part[it];
      if (cheb) b += part2[it];
    }
    red[threadIdx.x] = a;
    red2[threadIdx.x] = b;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) {
        red[threadIdx.x] += red[threadIdx.x + w];
        red2[threadIdx.x] += red2[threadIdx.x + w];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0 && s.mode == kModeLanczos && k < s.kmax) {
      if (what == 0) s.alpha[k] = red[0];
      else s.beta[k] = sqrt(fmax(red[0], 0.0));
    }
    if (threadIdx.x == 0 && cheb && k < s.kmax) {
      s.alpha[k] = red[0];   // Re<T_k, T_{k+1}>
      s.beta[k] = red2[0];   // <T_{k+1}, T_{k+1}>
    }
    __syncthreads();
  }
}

// w -= alpha_k v ; partial ||w||^2 per item.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_eng_update(const SlotDesc* __restrict__ slots, const int2* __restrict__ items, int n_items,
             double* __restrict__ part) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < n_items; it += gridDim.x * WARPS) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    const int k = s.k;
    double nn = 0.0;
    if (s.mode == kModeLanczos && k < s.kmax) {
      const int64_t r = item.y, Dd = s.Dd;
      const float2* v = s.buf[(k + 1) % 3] + r * Dd;
      float2* w = s.buf[(k + 2) % 3] + r * Dd;
      const float a = (float)s.alpha[k];
      float hi = 0.f, lo = 0.f;
      for (int64_t c = lane; c < Dd; c += 32) {
        float2 o = w[c];
        const float2 xv = v[c];
        o.x = fmaf(-a, xv.x, o.x);
        o.y = fmaf(-a, xv.y, o.y);
        w[c] = o;
        float p = o.x * o.x, pe = fmaf(o.x, o.x, -p);
        float s1 = hi + p, bp = s1 - hi;
        lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
        hi = s1;
        p = o.y * o.y;
        pe = fmaf(o.y, o.y, -p);
        s1 = hi + p;
        bp = s1 - hi;
        lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
        hi = s1;
      }
      nn = (double)hi + (double)lo;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nn += __shfl_down_sync(0xffffffffu, nn, o);
    }
    if (lane == 0) part[it] = nn;
  }
}

// Replay pass: w = (w - alpha_k v) / beta_k ; x += y_{k+1} w.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_eng_replay_update(const SlotDesc* __restrict__ slots, const int2* __restrict__ items,
                    int n_items) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < n_items; it += gridDim.x * WARPS) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    const int k = s.k;
    if (!(s.mode == kModeReplay && k + 1 < s.steps)) continue;
    const int64_t r = item.y, Dd = s.Dd;
    const float2* v = s.buf[(k + 1) % 3] + r * Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    float2* x = s.xacc + r * Dd;
    const float a = (float)s.alpha[k], ib = (float)(1.0 / s.beta[k]);
    const float y = (float)s.yk[k + 1];
    for (int64_t c = lane; c < Dd; c += 32) {
      float2 o = w[c];
      const float2 xv = v[c];
      o.x = (o.x - a * xv.x) * ib;
      o.y = (o.y - a * xv.y) * ib;
      w[c] = o;
      float2 acc = x[c];
      acc.x = fmaf(y, o.x, acc.x);
      acc.y = fmaf(y, o.y, acc.y);
      x[c] = acc;
    }
  }
}

// v_{k+1} = w / beta_k (in place on w); marks breakdown / completion.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_eng_normalize(const SlotDesc* __restrict__ slots, const int2* __restrict__ items, int n_items) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < n_items; it += gridDim.x * WARPS) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    const int k = s.k;
    if (!(s.mode == kModeLanczos && k < s.kmax)) continue;
    const double b = s.beta[k];
    if (!(b > kTol)) continue;
    const int64_t r = item.y, Dd = s.Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    float2* vb = s.basis && k + 1 < s.kmax ? s.basis + (int64_t)(k + 1) * s.Du * Dd + r * Dd
                                           : nullptr;
    const float ib = (float)(1.0 / b);
    for (int64_t c = lane; c < Dd; c += 32) {
      float2 o = w[c];
      o.x *= ib;
      o.y *= ib;
      w[c] = o;
      if (vb) vb[c] = o;
    }
  }
}

// x = y_0 v_0 + y_1 v_1 + ... + y_(m-1) v_(m-1) from the kept Lanczos
// vectors, in the order and arithmetic of the replay (k_eng_replay_init, then
// one fmaf per replayed step), so the Ritz vector has the replay's bits.
__global__ void k_eng_combine(const float2* __restrict__ basis, int64_t dim, int m,
                              const double* __restrict__ yk, float2* __restrict__ x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < dim;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float y0 = (float)yk[0];
    const float2 a = basis[i];
    float2 acc = make_float2(y0 * a.x, y0 * a.y);
    for (int j = 1; j < m; ++j) {
      const float y = (float)yk[j];
      const float2 v = basis[(int64_t)j * dim + i];
      acc.x = fmaf(y, v.x, acc.x);
      acc.y = fmaf(y, v.y, acc.y);
    }
    x[i] = acc;
  }
}

// End of step: advance each slot's counter; a Lanczos slot that broke down
// (beta <= 1000 eps, lanczos.h:35) or reached kmax goes idle.
__global__ void k_eng_advance(SlotDesc* __restrict__ slots, int n_slots) {
  for (int si = threadIdx.x + blockIdx.x * blockDim.x; si < n_slots; si += blockDim.x * gridDim.x) {
    SlotDesc& s = slots[si];
    const int k = s.k;
    if (s.mode == kModeLanczos && k < s.kmax) {
      s.steps = k + 1;
      s.k = k + 1;
      if (!(s.beta[k] > kTol) || k + 1 >= s.kmax) s.mode = kModeIdle;
    } else if (s.mode == kModeReplay && k + 1 < s.steps) {
      s.k = k + 1;
      if (k + 2 >= s.steps) s.mode = kModeIdle;
    } else if (s.mode == kModeReplay) {
      s.mode = kModeIdle;
    } else if (s.mode == kModeCheb && k < s.kmax) {
      s.k = k + 1;
      s.steps = k + 1;
      if (k + 1 >= s.kmax) s.mode = kModeIdle;
    }
  }
}

__device__ __forceinline__ void eng_philox(uint32_t c[4], uint32_t k0, uint32_t k1);

// Random-phase probe exp(2 pi i u), u ~ U[0,1) from Philox (stream 1 + probe).
__global__ void k_eng_seed_phase(float2* __restrict__ v, int64_t n, uint64_t seed, uint32_t stream_id) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), stream_id, 0u};
    eng_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t m0 = ((((uint64_t)c[0]) << 32) | c[1]) >> 12;
    const double u = (__longlong_as_double((long long)(0x4000000000000000ull | m0)) - 3.0 + 1.0) * 0.5;
    float sn, cs;
    sincospif((float)(2.0 * u), &sn, &cs);
    v[i] = make_float2(cs, sn);
  }
}

// Replay start: v = b / ||b|| was kept in buf[1]; x = y_0 v.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32)
k_eng_replay_init(const SlotDesc* __restrict__ slots, const int2* __restrict__ items, int n_items) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int it = blockIdx.x * WARPS + warp; it < n_items; it += gridDim.x * WARPS) {
    const int2 item = items[it];
    const SlotDesc& s = slots[item.x];
    if (s.steps == 0) continue;
    const int64_t r = item.y, Dd = s.Dd;
    const float2* v = s.buf[1] + r * Dd;
    float2* x = s.xacc + r * Dd;
    float2* vp = s.buf[0] + r * Dd;
    const float y0 = (float)s.yk[0];
    for (int64_t c = lane; c < Dd; c += 32) {
      const float2 a = v[c];
      x[c] = make_float2(y0 * a.x, y0 * a.y);
      vp[c] = make_float2(0.f, 0.f);
    }
  }
}

// Start vectors: Philox4x32-10 uniform(-1,1) at counter = tensor index,
// normalised later (pass one scales by 1/||b||).
__device__ __forceinline__ void eng_philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

__global__ void k_eng_seed(float2* __restrict__ v, int64_t n, uint64_t seed, double inv_norm_hint) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), 0u, 0u};
    eng_philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    const uint64_t m0 = ((((uint64_t)c[0]) << 32) | c[1]) >> 12;
    const uint64_t m1 = ((((uint64_t)c[2]) << 32) | c[3]) >> 12;
    const double re = __longlong_as_double((long long)(0x4000000000000000ull | m0)) - 3.0;
    const double im = __longlong_as_double((long long)(0x4000000000000000ull | m1)) - 3.0;
    v[i] = make_float2((float)re, (float)im);
  }
}

// ||b||^2 of one slot's start vector (compensated): block b sums the
// elements [b * n / nb, (b + 1) * n / nb) into part[b], then k_eng_sum adds
// the nb partials in order (nb depends on n only: the same bits alone or in
// any mix of requests).
__global__ void k_eng_norm2(const float2* __restrict__ v, int64_t n, double* __restrict__ part) {
  __shared__ double red[256];
  const int64_t i0 = n * blockIdx.x / gridDim.x, i1 = n * (blockIdx.x + 1) / gridDim.x;
  float hi = 0.f, lo = 0.f;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const float2 a = v[i];
    float p = a.x * a.x, pe = fmaf(a.x, a.x, -p);
    float s1 = hi + p, bp = s1 - hi;
    lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
    hi = s1;
    p = a.y * a.y;
    pe = fmaf(a.y, a.y, -p);
    s1 = hi + p;
    bp = s1 - hi;
    lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
    hi = s1;
  }
  red[threadIdx.x] = (double)hi + (double)lo;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_eng_sum(const double* __restrict__ part, int nb, double* __restrict__ out) {
  double a = 0.0;
  for (int b = 0; b < nb; ++b) a += part[b];
  *out = a;
}

__global__ void k_eng_scale(float2* __restrict__ v, int64_t n, float s) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = v[i];
    v[i] = make_float2(a.x * s, a.y * s);
  }
}

// v /= sqrt(*n2), the norm's reciprocal rounded to float as the host would;
// the norm itself to *norm_out.
__global__ void k_eng_scale_by_norm(float2* __restrict__ v, int64_t n, const double* __restrict__ n2,
                                    double* __restrict__ norm_out) {
  const double nrm = sqrt(*n2);
  if (blockIdx.x == 0 && threadIdx.x == 0) *norm_out = nrm;
  const float s = (float)(1.0 / nrm);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 a = v[i];
    v[i] = make_float2(a.x * s, a.y * s);
  }
}

__global__ void k_f32_to_f64(const float2* __restrict__ a, double2* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float2 v = a[i];
    b[i] = make_double2((double)v.x, (double)v.y);
  }
}


// ===========================================================================
// The persistent engine step.  One cooperative launch runs `steps` engine
// steps of every active request, the phases of a step separated by a grid
// barrier:
//   A  apply: rows of staged sectors block per row (the row and its sign-
//      sorted up list in shared memory, the sliced down table), rows of small
//      sectors warp per row (the row staged in the warp's own shared memory,
//      CSR down table) -> per-row partials Re<v,w>, <w,w>;
//   B  per-request fixed-order sum of the partials -> alpha_k (Chebyshev:
//      Re<T_k,T_k+1> and <T_k+1,T_k+1>);
//   C  w -= alpha_k v and per-row ||w||^2 (Lanczos); w = (w - alpha v) / beta,
//      x += y w (replay);
//   D  per-request sum -> beta_k;
//   E  v_k+1 = w / beta_k;
//   F  step counters, breakdown (beta <= 1000 eps) and completion.
// The arithmetic of every phase is that of the grouped kernels above (same
// operation order, same fixed-order reductions over 256 threads), so a request
// gets the same bits alone, in any mix, and through either path.  Data that
// other CTAs of the launch write is read after a grid barrier (release fence
// and atomic arrival, gpu-scope acquire of the generation, then the block
// barrier) with ordinary loads, never through the read-only path; the step
// state (counters, alpha, beta, partials) through L2.  A barrier wait that runs past its clock64
// budget sets the status word, and every CTA then returns at its next barrier:
// the step fails with MB_ERR_TIMEOUT instead of hanging.
// ===========================================================================
struct EngGrid {
  unsigned int count;
  unsigned int gen;
  int status;   // 0: running; 1: a barrier wait ran out of its budget
  int pad;
};

struct EngPersistArgs {
  SlotDesc* slots;
  int n_slots;
  const int2* items;       // every (slot, row); item index = slot's item0 + row
  int n_items;
  const int2* items_rows;  // rows applied block per row (staged)
  int n_rows;
  const int2* items_warp;  // rows applied warp per row
  int n_warp;
  double* part;            // [n_items]
  double* part2;           // [n_items]
  int row_cols;            // widest staged row
  int steps;
  int apply_only;          // 1: phase A only (the autotuner's timing runs)
  EngGrid* grid;
  long long budget;        // clock64 cycles one barrier wait may take
};

constexpr int kEngPWarps = 8;             // 256 threads: the reductions' width
constexpr int kEngWarpRowCols = 256;      // widest row of the warp-per-row items

__device__ __forceinline__ unsigned eng_ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int eng_ld_relaxed(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void eng_st_release(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid barrier with a bounded wait; false once any CTA has given up.
__device__ bool eng_grid_sync(EngGrid* g, long long budget) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    const unsigned gen = eng_ld_acquire(&g->gen);
    if (atomicAdd(&g->count, 1u) == gridDim.x - 1) {
      atomicExch(&g->count, 0u);
      __threadfence();
      eng_st_release(&g->gen, gen + 1u);
    } else {
      const long long t0 = clock64();
      while (eng_ld_acquire(&g->gen) == gen) {
        if (eng_ld_relaxed(&g->status) != 0) {
          ok = 0;
          break;
        }
        if (clock64() - t0 > budget) {
          atomicExch(&g->status, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    if (ok && eng_ld_relaxed(&g->status) != 0) ok = 0;
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

struct SlotNow {
  int k, mode, kmax, steps;
};
__device__ __forceinline__ SlotNow slot_now(const SlotDesc& s) {
  SlotNow n;
  n.k = __ldcg(&s.k);
  n.mode = __ldcg(&s.mode);
  n.kmax = __ldcg(&s.kmax);
  n.steps = __ldcg(&s.steps);
  return n;
}

// compensated float accumulation of a * b (exact product, TwoSum)
__device__ __forceinline__ void eng_acc(float& hi, float& lo, float a, float b) {
  const float p = a * b, pe = fmaf(a, b, -p);
  const float s1 = hi + p, bp = s1 - hi;
  lo += ((hi - (s1 - bp)) + (p - bp)) + pe;
  hi = s1;
}

// Deferred normalisation within one launch of the persistent step.  At the
// end of step k a Lanczos request's v_k+1 = w_k / beta_k is not written back
// (except on the launch's last step): the later steps of the launch multiply
// what is stored by ib = (float)(1 / beta) as they load it, the same float
// product (no contraction) the normalisation would have stored, so every
// value, and every bit of the result, is the grouped kernels'.  `step` is the
// step's index in the launch: v_k is stored unnormalised when step >= 1
// (w_k-1), v_k-1 when step >= 2.
struct LazyScale {
  float v, prev;
};
__device__ __forceinline__ LazyScale lazy_scale(const SlotDesc& s, const SlotNow& n, int step) {
  LazyScale l{1.f, 1.f};
  if (n.mode == kModeLanczos && n.k < n.kmax) {
    if (step >= 1) l.v = __ldcg(&s.ib[n.k - 1]);
    if (step >= 2) l.prev = __ldcg(&s.ib[n.k - 2]);
  }
  return l;
}
__device__ __forceinline__ float2 lz(float2 a, float f) {
  return make_float2(__fmul_rn(a.x, f), __fmul_rn(a.y, f));
}

// Phase A, one staged row (block-level): the arithmetic of k_eng_apply_rows.
__device__ void p_apply_row(const SlotDesc& s, const SlotNow& n, int64_t r, int64_t pidx,
                            double* part, double* part2, float2* srow, uint32_t* s_up,
                            double (*red)[2], int step) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int k = n.k;
  const bool lanczos = n.mode == kModeLanczos && k < n.kmax;
  const bool replay = n.mode == kModeReplay && k + 1 < n.steps;
  const bool cheb = n.mode == kModeCheb && k < n.kmax;
  if (!(lanczos || replay || cheb)) {  // uniform over the block
    if (threadIdx.x == 0) {
      part[pidx] = 0.0;
      part2[pidx] = 0.0;
    }
    return;
  }
  const int64_t Dd = s.Dd;
  const uint64_t row_bytes = sizeof(float2) * (uint64_t)Dd;
  const float2* x = s.buf[(k + 1) % 3];
  const float2* v = x + r * Dd;
  const float2* z = s.buf[k % 3] + r * Dd;
  float2* w = s.buf[(k + 2) % 3] + r * Dd;
  const double bprev = cheb ? 1.0 : (k > 0 ? __ldcg(&s.beta[k - 1]) : 0.0);
  const float beta = (float)(-bprev);
  const float sc = cheb ? (k == 0 ? 1.f : 2.f) / s.cheb_a : s.scale;
  const float shift = cheb ? s.cheb_b : 0.f;
  const float hop = -s.t * sc;
  const uint32_t um = s.up_mask[r];
  const int u0 = __ldg(&s.up_loff[r]), nu = __ldg(&s.up_loff[r + 1]) - u0;
  const int npos = __ldg(&s.up_lpos[r]);
  const LazyScale ls = lazy_scale(s, n, step);
  // v_k in the kept basis: written here when this launch produced it
  float2* vb = lanczos && s.basis && step >= 1 ? s.basis + (int64_t)k * s.Du * Dd + r * Dd : nullptr;
  __syncthreads();  // the previous item's readers are done with srow / s_up
  for (int64_t c = threadIdx.x; c < Dd; c += blockDim.x) {
    const float2 t = lz(v[c], ls.v);
    srow[c] = t;
    if (vb) vb[c] = t;
  }
  if (threadIdx.x < kSlicedPads) srow[Dd + threadIdx.x] = make_float2(0.f, 0.f);
  for (int j = threadIdx.x; j < nu; j += blockDim.x) s_up[j] = __ldg(&s.up_list[u0 + j]);
  __syncthreads();
  float hi = 0.f, lo = 0.f, hi2 = 0.f, lo2 = 0.f;
  const int64_t ngroups = (Dd + 31) >> 5;
  for (int64_t g = warp; g < ngroups; g += kEngPWarps) {
    const int64_t c = (g << 5) + lane;
    const bool live = c < Dd;
    const int64_t cl = live ? c : Dd - 1;
    float ar = 0.f, ai = 0.f;
    const int2 gi = __ldg(reinterpret_cast<const int2*>(s.dn_sgrp) + g);
    const uint4* ep = reinterpret_cast<const uint4*>(s.dn_sell + gi.x) + lane;
    auto dn = [&](uint32_t e) {
      const float2 val = srow[e & 0x7FFFFFFFu];
      const float wgt = __int_as_float((int)(0x3f800000u | (e & 0x80000000u)));
      ar = fmaf(wgt, val.x, ar);
      ai = fmaf(wgt, val.y, ai);
    };
    for (int j = 0; j < gi.y; j += 4) {
      const uint4 e = __ldg(ep + 8 * j);
      dn(e.x);
      dn(e.y);
      dn(e.z);
      dn(e.w);
    }
    const char* xc = reinterpret_cast<const char*>(x + cl);
    auto up = [&](int q) {
      return lz(*reinterpret_cast<const float2*>(xc + (uint64_t)s_up[q] * row_bytes), ls.v);
    };
    float pr = 0.f, pi = 0.f, nr = 0.f, ni = 0.f;
    int j = 0;
#pragma unroll 4
    for (; j < npos; ++j) {
      const float2 val = up(j);
      pr += val.x;
      pi += val.y;
    }
#pragma unroll 4
    for (; j < nu; ++j) {
      const float2 val = up(j);
      nr += val.x;
      ni += val.y;
    }
    ar += pr - nr;
    ai += pi - ni;
    if (!live) continue;
    const float2 xv = srow[c];
    const float d = sc * (s.ufold[__popc(um & s.dn_mask[c])] +
                          (s.self_up ? s.self_up[r] + s.self_dn[c] : 0.f) - shift);
    float2 o;
    o.x = fmaf(hop, ar, d * xv.x);
    o.y = fmaf(hop, ai, d * xv.y);
    if (k > 0) {
      const float2 zv = lz(z[c], ls.prev);
      o.x = fmaf(beta, zv.x, o.x);
      o.y = fmaf(beta, zv.y, o.y);
    }
    w[c] = o;
    if (!replay) {
      eng_acc(hi, lo, xv.x, o.x);
      eng_acc(hi, lo, xv.y, o.y);
    }
    if (cheb) {
      eng_acc(hi2, lo2, o.x, o.x);
      eng_acc(hi2, lo2, o.y, o.y);
    }
  }
  double dxy = (double)hi + (double)lo, dyy = (double)hi2 + (double)lo2;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    dxy += __shfl_down_sync(0xffffffffu, dxy, o);
    dyy += __shfl_down_sync(0xffffffffu, dyy, o);
  }
  if (lane == 0) {
    red[warp][0] = dxy;
    red[warp][1] = dyy;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // fixed order over the warps
    double a = 0.0, b = 0.0;
    for (int q = 0; q < kEngPWarps; ++q) {
      a += red[q][0];
      b += red[q][1];
    }
    part[pidx] = a;
    part2[pidx] = b;
  }
}

// Phase A, one small row (warp-level, the row staged in the warp's shared
// memory): the arithmetic of k_eng_apply.
__device__ void p_apply_warp_row(const SlotDesc& s, const SlotNow& n, int64_t r, int64_t pidx,
                                 double* part, double* part2, float2* wrow, int step) {
  const int lane = threadIdx.x & 31;
  const int k = n.k;
  const bool replay = n.mode == kModeReplay;
  const bool cheb = n.mode == kModeCheb;
  double dxy = 0.0, dyy = 0.0;
  if ((n.mode == kModeLanczos && k < n.kmax) || (replay && k + 1 < n.steps) ||
      (cheb && k < n.kmax)) {
    const int64_t Dd = s.Dd;
    const float2* v = s.buf[(k + 1) % 3] + r * Dd;
    const float2* x = s.buf[(k + 1) % 3];
    const float2* z = s.buf[k % 3] + r * Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    const LazyScale ls = lazy_scale(s, n, step);
    float2* vb = n.mode == kModeLanczos && s.basis && step >= 1
                     ? s.basis + (int64_t)k * s.Du * Dd + r * Dd
                     : nullptr;
    __syncwarp();  // the warp's previous row is no longer read
    for (int64_t c = lane; c < Dd; c += 32) {
      const float2 t = lz(v[c], ls.v);
      wrow[c] = t;
      if (vb) vb[c] = t;
    }
    __syncwarp();
    const double bprev = cheb ? 1.0 : (k > 0 ? __ldcg(&s.beta[k - 1]) : 0.0);
    const float beta = (float)(-bprev);
    const float sc = cheb ? (k == 0 ? 1.f : 2.f) / s.cheb_a : s.scale;
    const float shift = cheb ? s.cheb_b : 0.f;
    const float hop = -s.t * sc;
    float hi2 = 0.f, lo2 = 0.f;
    const uint32_t um = s.up_mask[r];
    const int u0 = s.up_off[r], u1 = s.up_off[r + 1];
    float hi = 0.f, lo = 0.f;
    for (int64_t c = lane; c < Dd; c += 32) {
      float ar = 0.f, ai = 0.f;
      for (int j = s.dn_off[c]; j < s.dn_off[c + 1]; ++j) {
        const uint32_t e = __ldg(&s.dn_ent[j]);
        const float2 val = wrow[e >> 8];
        float wgt = (e & 2u) ? 2.f : 1.f;
        if (e & 1u) wgt = -wgt;
        ar = fmaf(wgt, val.x, ar);
        ai = fmaf(wgt, val.y, ai);
      }
      for (int j = u0; j < u1; ++j) {
        const uint32_t e = __ldg(&s.up_ent[j]);
        const float2 val = lz(x[(int64_t)(e >> 8) * Dd + c], ls.v);
        float wgt = (e & 2u) ? 2.f : 1.f;
        if (e & 1u) wgt = -wgt;
        ar = fmaf(wgt, val.x, ar);
        ai = fmaf(wgt, val.y, ai);
      }
      const float2 xv = wrow[c];
      const float d = sc * (s.ufold[__popc(um & s.dn_mask[c])] +
                            (s.self_up ? s.self_up[r] + s.self_dn[c] : 0.f) - shift);
      float2 o;
      o.x = fmaf(hop, ar, d * xv.x);
      o.y = fmaf(hop, ai, d * xv.y);
      if (k > 0) {
        const float2 zv = lz(z[c], ls.prev);
        o.x = fmaf(beta, zv.x, o.x);
        o.y = fmaf(beta, zv.y, o.y);
      }
      w[c] = o;
      if (!replay) {
        eng_acc(hi, lo, xv.x, o.x);
        eng_acc(hi, lo, xv.y, o.y);
      }
      if (cheb) {
        eng_acc(hi2, lo2, o.x, o.x);
        eng_acc(hi2, lo2, o.y, o.y);
      }
    }
    dxy = (double)hi + (double)lo;
    dyy = (double)hi2 + (double)lo2;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      dxy += __shfl_down_sync(0xffffffffu, dxy, o);
      dyy += __shfl_down_sync(0xffffffffu, dyy, o);
    }
  }
  if (lane == 0) {
    part[pidx] = dxy;
    part2[pidx] = dyy;
  }
}

// Phases B and D, one request (block-level): the sum of k_eng_seg_reduce.
__device__ void p_seg_reduce(SlotDesc& s, const double* part, const double* part2, int what,
                             double* red, double* red2) {
  const SlotNow n = slot_now(s);
  const int k = n.k;
  const bool cheb = n.mode == kModeCheb && what == 0;
  double a = 0.0, b = 0.0;
  for (int it = s.item0 + threadIdx.x; it < s.item1; it += blockDim.x) {
    a += __ldcg(part + it);
    if (cheb) b += __ldcg(part2 + it);
  }
  __syncthreads();  // the previous request's sums are read
  red[threadIdx.x] = a;
  red2[threadIdx.x] = b;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[threadIdx.x] += red[threadIdx.x + w];
      red2[threadIdx.x] += red2[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0 && n.mode == kModeLanczos && k < n.kmax) {
    if (what == 0) {
      s.alpha[k] = red[0];
    } else {
      const double b = sqrt(fmax(red[0], 0.0));
      s.beta[k] = b;
      s.ib[k] = (float)(1.0 / b);  // once a request, for the deferred normalisation
    }
  }
  if (threadIdx.x == 0 && cheb && k < n.kmax) {
    s.alpha[k] = red[0];
    s.beta[k] = red2[0];
  }
}

// Phase C, one row (warp-level): k_eng_update and k_eng_replay_update.
__device__ void p_update_row(const SlotDesc& s, const SlotNow& n, int64_t r, int it, double* part,
                             int step) {
  const int lane = threadIdx.x & 31;
  const int k = n.k;
  const int64_t Dd = s.Dd;
  if (n.mode == kModeLanczos && k < n.kmax) {
    const float2* v = s.buf[(k + 1) % 3] + r * Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    const float a = (float)__ldcg(&s.alpha[k]);
    const float lv = lazy_scale(s, n, step).v;
    float hi = 0.f, lo = 0.f;
    // four elements a lane in flight (half the threads of the grouped
    // kernels run here), summed in the same order
    int64_t c = lane;
    for (; c + 96 < Dd; c += 128) {
      float2 o[4], xv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        o[q] = w[c + 32 * q];
        xv[q] = lz(v[c + 32 * q], lv);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        o[q].x = fmaf(-a, xv[q].x, o[q].x);
        o[q].y = fmaf(-a, xv[q].y, o[q].y);
        w[c + 32 * q] = o[q];
        eng_acc(hi, lo, o[q].x, o[q].x);
        eng_acc(hi, lo, o[q].y, o[q].y);
      }
    }
    for (; c < Dd; c += 32) {
      float2 o = w[c];
      const float2 xv = lz(v[c], lv);
      o.x = fmaf(-a, xv.x, o.x);
      o.y = fmaf(-a, xv.y, o.y);
      w[c] = o;
      eng_acc(hi, lo, o.x, o.x);
      eng_acc(hi, lo, o.y, o.y);
    }
    double nn = (double)hi + (double)lo;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nn += __shfl_down_sync(0xffffffffu, nn, o);
    if (lane == 0) part[it] = nn;
    return;
  }
  if (lane == 0) part[it] = 0.0;
  if (n.mode == kModeReplay && k + 1 < n.steps) {
    const float2* v = s.buf[(k + 1) % 3] + r * Dd;
    float2* w = s.buf[(k + 2) % 3] + r * Dd;
    float2* xa = s.xacc + r * Dd;
    const float a = (float)__ldcg(&s.alpha[k]), ib = (float)(1.0 / __ldcg(&s.beta[k]));
    const float y = (float)s.yk[k + 1];
    for (int64_t c = lane; c < Dd; c += 32) {
      float2 o = w[c];
      const float2 xv = v[c];
      o.x = (o.x - a * xv.x) * ib;
      o.y = (o.y - a * xv.y) * ib;
      w[c] = o;
      float2 acc = xa[c];
      acc.x = fmaf(y, o.x, acc.x);
      acc.y = fmaf(y, o.y, acc.y);
      xa[c] = acc;
    }
  }
}

// Phase E, one row (warp-level): k_eng_normalize.  Runs on the launch's last
// step only; v_k, when this launch left it unnormalised, is normalised in
// place too, so every launch ends with the grouped kernels' vectors.
__device__ void p_normalize_row(const SlotDesc& s, const SlotNow& n, int64_t r, int step) {
  const int lane = threadIdx.x & 31;
  const int k = n.k;
  if (!(n.mode == kModeLanczos && k < n.kmax)) return;
  const int64_t Dd = s.Dd;
  const float lv = lazy_scale(s, n, step).v;
  if (step >= 1) {
    float2* v = s.buf[(k + 1) % 3] + r * Dd;
    for (int64_t c = lane; c < Dd; c += 32) v[c] = lz(v[c], lv);
  }
  const double b = __ldcg(&s.beta[k]);
  if (!(b > kTol)) return;
  float2* w = s.buf[(k + 2) % 3] + r * Dd;
  float2* vb = s.basis && k + 1 < n.kmax ? s.basis + (int64_t)(k + 1) * s.Du * Dd + r * Dd
                                         : nullptr;
  const float ib = (float)(1.0 / b);
  int64_t c = lane;
  for (; c + 96 < Dd; c += 128) {
    float2 o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) o[q] = w[c + 32 * q];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      o[q] = make_float2(o[q].x * ib, o[q].y * ib);
      w[c + 32 * q] = o[q];
      if (vb) vb[c + 32 * q] = o[q];
    }
  }
  for (; c < Dd; c += 32) {
    float2 o = w[c];
    o.x *= ib;
    o.y *= ib;
    w[c] = o;
    if (vb) vb[c] = o;
  }
}

// Phase F, one request: k_eng_advance.
__device__ void p_advance(SlotDesc& s) {
  const SlotNow n = slot_now(s);
  const int k = n.k;
  if (n.mode == kModeLanczos && k < n.kmax) {
    s.steps = k + 1;
    s.k = k + 1;
    if (!(__ldcg(&s.beta[k]) > kTol) || k + 1 >= n.kmax) s.mode = kModeIdle;
  } else if (n.mode == kModeReplay && k + 1 < n.steps) {
    s.k = k + 1;
    if (k + 2 >= n.steps) s.mode = kModeIdle;
  } else if (n.mode == kModeReplay) {
    s.mode = kModeIdle;
  } else if (n.mode == kModeCheb && k < n.kmax) {
    s.k = k + 1;
    s.steps = k + 1;
    if (k + 1 >= n.kmax) s.mode = kModeIdle;
  }
}

// four co-resident blocks an SM (64 registers a thread): the occupancy the
// apply phase's gathers need
__global__ void __launch_bounds__(kEngPWarps * 32, 4)
k_eng_persistent(EngPersistArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[kEngPWarps][2];
  __shared__ double sred[kEngPWarps * 32], sred2[kEngPWarps * 32];
  const int warp = threadIdx.x >> 5;
  float2* srow = reinterpret_cast<float2*>(smem);
  uint32_t* s_up = reinterpret_cast<uint32_t*>(smem + sizeof(float2) * (a.row_cols + kSlicedPads));
  float2* wrow = reinterpret_cast<float2*>(smem) + (size_t)warp * kEngWarpRowCols;
  const int gw = blockIdx.x * kEngPWarps + warp, nw = gridDim.x * kEngPWarps;
  for (int step = 0; step < a.steps; ++step) {
    const bool last = step + 1 == a.steps;
    // A: apply
    for (int it = blockIdx.x; it < a.n_rows; it += gridDim.x) {
      const int2 item = a.items_rows[it];
      const SlotDesc& s = a.slots[item.x];
      p_apply_row(s, slot_now(s), item.y, s.item0 + item.y, a.part, a.part2, srow, s_up, red,
                  step);
    }
    __syncthreads();  // the row items' shared memory becomes the warps' rows
    for (int it = gw; it < a.n_warp; it += nw) {
      const int2 item = a.items_warp[it];
      const SlotDesc& s = a.slots[item.x];
      p_apply_warp_row(s, slot_now(s), item.y, s.item0 + item.y, a.part, a.part2, wrow, step);
    }
    if (a.apply_only) return;
    if (!eng_grid_sync(a.grid, a.budget)) return;
    // B: alpha
    for (int si = blockIdx.x; si < a.n_slots; si += gridDim.x)
      p_seg_reduce(a.slots[si], a.part, a.part2, 0, sred, sred2);
    if (!eng_grid_sync(a.grid, a.budget)) return;
    // C: update (and the replay accumulation)
    for (int it = gw; it < a.n_items; it += nw) {
      const int2 item = a.items[it];
      const SlotDesc& s = a.slots[item.x];
      p_update_row(s, slot_now(s), item.y, it, a.part, step);
    }
    if (!eng_grid_sync(a.grid, a.budget)) return;
    // D: beta; before the last step, F (advance) right after it by the same
    // block (no normalisation pass between them: it is deferred)
    for (int si = blockIdx.x; si < a.n_slots; si += gridDim.x) {
      p_seg_reduce(a.slots[si], a.part, a.part2, 1, sred, sred2);
      if (!last) {
        __syncthreads();
        if (threadIdx.x == 0) p_advance(a.slots[si]);
      }
    }
    if (!last) {
      if (!eng_grid_sync(a.grid, a.budget)) return;
      continue;
    }
    if (!eng_grid_sync(a.grid, a.budget)) return;
    // E: normalise (the last step)
    for (int it = gw; it < a.n_items; it += nw) {
      const int2 item = a.items[it];
      const SlotDesc& s = a.slots[item.x];
      p_normalize_row(s, slot_now(s), item.y, step);
    }
    if (!eng_grid_sync(a.grid, a.budget)) return;
    // F: advance
    for (int si = blockIdx.x * blockDim.x + threadIdx.x; si < a.n_slots;
         si += gridDim.x * blockDim.x)
      p_advance(a.slots[si]);
  }
}

}  // namespace mb

// ===========================================================================
// Host side.
// ===========================================================================
namespace mb {

// Device buffer: cudaMalloc, or (with a pool) stream-ordered from the
// engine's memory pool, so that admitting and retiring requests neither
// maps nor unmaps device memory nor waits for the device.
struct EngBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaMemPool_t pool = nullptr;
  cudaStream_t ps = nullptr;
  EngBuf() = default;
  explicit EngBuf(size_t b) : bytes(b) {
    if (b) MB_CUDA(cudaMalloc(&p, b));
  }
  EngBuf(size_t b, cudaMemPool_t mp, cudaStream_t st) : bytes(b), pool(mp), ps(st) {
    if (b) MB_CUDA(cudaMallocFromPoolAsync(&p, b, mp, st));
  }
  ~EngBuf() {
    if (!p) return;
    if (pool) cudaFreeAsync(p, ps);
    else cudaFree(p);
  }
  EngBuf(const EngBuf&) = delete;
  EngBuf& operator=(const EngBuf&) = delete;
};

// Sector tables shared by all slots with the same lattice and filling.
struct TableSet {
  mb_basis_s basis;
  mb_model_s model;  // bonds only; t and U come per slot
  std::vector<std::unique_ptr<EngBuf>> bufs;
  const uint32_t *up_mask = nullptr, *dn_mask = nullptr, *up_ent = nullptr, *dn_ent = nullptr;
  const int32_t *up_off = nullptr, *dn_off = nullptr;
  int max_up_deg = 0, max_dn_deg = 0;
  OpView fused{};  // tables of the fused FP64 apply (refinement)
  // self energies at t = 1 (lattices with a size-1 dimension): per up state,
  // per down state; empty otherwise
  std::vector<double> self_up1, self_dn1;
  int64_t bytes = 0;
  int refs = 0;
};

template <typename T>
const T* tupload(TableSet& ts, const std::vector<T>& h) {
  auto b = std::make_unique<EngBuf>(sizeof(T) * std::max<size_t>(h.size(), 1));
  if (!h.empty()) MB_CUDA(cudaMemcpy(b->p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  ts.bytes += (int64_t)b->bytes;
  const T* p = (const T*)b->p;
  ts.bufs.push_back(std::move(b));
  return p;
}

using SectorKey = std::tuple<std::vector<int64_t>, int, int>;

struct EngineSlot {
  int64_t id = -1;
  std::shared_ptr<TableSet> tables;
  double t = 1.0, u = 0.0;
  uint64_t seed = 0;
  int64_t kmax = 0;
  double rel_tol = 0.0;
  int check_every = 10;
  int refine = 1;
  std::unique_ptr<EngBuf> vecs;   // 4 vectors: buf0..2, xacc (complex64)
  std::unique_ptr<EngBuf> scal;   // alpha, beta, yk (double x kEngMaxK each), the start norm
  std::unique_ptr<EngBuf> selfe;  // self energies times t, float: [Du] up, [Dd] down (or none)
  std::unique_ptr<EngBuf> basis;  // pass one's Lanczos vectors (kmax x dim complex64), or none
  int64_t dim = 0, Du = 0, Dd = 0;
  int64_t bytes = 0;
  int phase = 0;                  // 0 pass one, 1 replay, 2 done, 10 DOS bounds, 11 DOS Chebyshev
  int kind = 0;                   // 0 ground state, 1 DOS moments
  float scale = -1.f;             // Lanczos scale (-1: ground state; +1: spectral bounds)
  int n_moments = 0, n_probes = 0, probe = 0;
  double padding = 0.01, emin = 0.0, emax = 0.0, mu0 = 0.0;
  std::vector<double> mu;         // accumulated DOS moments
  double b_norm = 0.0;
  double last_ritz = 0.0;
  bool have_ritz = false;
  int m = 0;                      // pass-one steps
  int m_ritz = 0;                 // steps replayed for the Ritz vector
  double e_raw = 0.0, e0 = 0.0;
  std::chrono::steady_clock::time_point t_submit, t_done;
};

}  // namespace mb

struct mb_engine_s {
  int64_t budget = 0, in_use = 0;
  int warps = 8;                  // chosen by the autotuner
  bool tuned = false;
  std::map<mb::SectorKey, std::shared_ptr<mb::TableSet>> tables;
  std::vector<std::unique_ptr<mb::EngineSlot>> slots;   // active (phases 0, 1)
  std::map<int64_t, std::unique_ptr<mb::EngineSlot>> done;
  int64_t next_id = 1;
  // device work lists
  std::unique_ptr<mb::EngBuf> d_slots, d_items, d_part;
  std::unique_ptr<mb::EngBuf> d_norm;  // start-vector norm partials (stream-ordered reuse)
  // the apply's work lists: rows of small sectors (warp per row) and rows of
  // medium ones (block per row, staged); large sectors use the fused kernel
  std::unique_ptr<mb::EngBuf> d_items_warp, d_items_rows;
  int n_warp = 0, n_rows = 0;
  int row_cols = 0;     // widest staged row
  size_t row_smem = 0;  // its row plus the longest up list
  int row_grid = 1;
  std::vector<mb::SlotDesc> h_slots;
  int n_items = 0;
  bool dirty = true;
  // slots of at least fused_min states step through the fused complex64
  // apply (staged rows, sliced tables) instead of the warp-per-row kernel
  int64_t fused_min = 1048576;
  std::vector<std::pair<mb::OpView, mb::EngFusedArgs>> fused;
  std::vector<std::unique_ptr<mb::EngBuf>> fused_scratch;
  cudaStream_t st = nullptr;
  // The persistent step (k_eng_persistent, cooperative launch): on by
  // default; rows of at least p_row_min_cols columns (and every row of a
  // sector of fused_min states or more) are applied block per row, the others
  // warp per row; p_ctas_per_sm CTAs per SM (0: as many as fit).
  bool persistent = true;
  int p_row_min_cols = 256;
  int p_ctas_per_sm = 0;
  // the persistent shape the autotuner chose for a mix of requests, keyed by
  // the mix's sorted (Du, Dd, kind) list: the same mix again is not re-timed
  std::vector<std::tuple<int64_t, int64_t, int>> tuned_mix;
  int tuned_cols = 256, tuned_ctas = 0;
  double tuned_ms = 0.0;
  int p_grid = 1;
  int p_bps = 1, p_sms = 1;  // co-resident blocks per SM of the last launch shape, SMs
  size_t p_smem = 0;
  long long wait_budget = 1LL << 32;  // clock64 cycles one barrier wait may take
  std::unique_ptr<mb::EngBuf> d_grid;  // barrier state and status (mb::EngGrid)
  bool broken = false;                 // a barrier wait ran out: requests are lost
  // a ground-state request keeps its pass-one Lanczos vectors (kmax x dim
  // complex64) when they take at most this many bytes (0: never)
  int64_t basis_limit = int64_t(2) << 30;
  // ids retired since the last mb_engine_completed call
  std::vector<int64_t> newly_done;
  // step statistics: steps run, wall time of the step calls, device time of
  // the step kernels (events around each step's launches)
  int64_t stat_steps = 0;
  double stat_wall_ms = 0.0, stat_dev_ms = 0.0;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  // the requests' vectors and scalars: stream-ordered on st, memory kept by
  // the pool between requests (returned to the device when the engine goes)
  cudaMemPool_t pool = nullptr;
  ~mb_engine_s() {
    slots.clear();  // their pool buffers are freed on st
    if (st) cudaStreamSynchronize(st);
    if (pool) cudaMemPoolDestroy(pool);
    for (cudaEvent_t x : ev)
      if (x) cudaEventDestroy(x);
    if (st) cudaStreamDestroy(st);
  }
};

namespace mb {
namespace {

std::shared_ptr<TableSet> get_tables(mb_engine_s* e, const mb_sector_desc& d) {
  std::vector<int64_t> dims(d.dims, d.dims + d.ndim);
  SectorKey key(dims, d.n_up, d.n_down);
  auto it = e->tables.find(key);
  if (it != e->tables.end()) return it->second;
  auto ts = std::make_shared<TableSet>();
  mb_basis_t b = nullptr;
  mb_model_t m = nullptr;
  int64_t L = 1;
  for (int i = 0; i < d.ndim; ++i) L *= d.dims[i];
  int rc = mb_basis_create_fixed_spin(L, d.n_up + d.n_down, d.n_up - d.n_down, &b);
  if (rc) throw Error(rc, mb_last_error());
  rc = mb_hubbard_create(d.dims, d.ndim, 1.0, 1.0, &m);
  if (rc) {
    mb_basis_destroy(b);
    throw Error(rc, mb_last_error());
  }
  ts->basis = *b;
  ts->model = *m;
  mb_basis_destroy(b);
  mb_model_destroy(m);
  const HopTable tu = build_hop_table(ts->basis.up, ts->model);
  const HopTable td = build_hop_table(ts->basis.down, ts->model);
  // a size-1 dimension: hopping(i, i) self bonds, a diagonal term per spin
  // (HubbardModel2D/3D with a size-1 side, hubbard_model.h:61-129)
  if (tu.has_self || td.has_self) {
    ts->self_up1 = tu.has_self ? tu.self_energy : std::vector<double>((size_t)ts->basis.up.D, 0.0);
    ts->self_dn1 = td.has_self ? td.self_energy : std::vector<double>((size_t)ts->basis.down.D, 0.0);
  }
  ts->up_mask = tupload(*ts, ts->basis.up.masks);
  ts->dn_mask = tupload(*ts, ts->basis.down.masks);
  ts->up_off = tupload(*ts, tu.off);
  ts->up_ent = tupload(*ts, tu.ent);
  ts->dn_off = tupload(*ts, td.off);
  ts->dn_ent = tupload(*ts, td.ent);
  ts->max_up_deg = tu.max_degree;
  ts->max_dn_deg = td.max_degree;
  TableSet* tsp = ts.get();
  fill_fused_tables(ts->fused, tu, td, ts->basis.up.D, ts->basis.down.D,
                    [tsp](const void* h, size_t bytes) -> const void* {
                      auto b = std::make_unique<EngBuf>(std::max<size_t>(bytes, 16));
                      if (bytes) MB_CUDA(cudaMemcpy(b->p, h, bytes, cudaMemcpyHostToDevice));
                      tsp->bytes += (int64_t)b->bytes;
                      const void* p = b->p;
                      tsp->bufs.push_back(std::move(b));
                      return p;
                    });
  e->tables[key] = ts;
  return ts;
}

// Device bytes of one slot: 4 complex64 vectors plus 3 x kEngMaxK doubles.
int64_t slot_bytes(int64_t dim) { return 4 * 8 * dim + (int64_t)kEngScalBytes; }

// The fused-apply view of a slot's sector (tables shared by its TableSet).
// The slot's self energies (t times the sector's t = 1 values) as float.
void upload_self_energies(mb_engine_s* e, EngineSlot& s) {
  const TableSet& ts = *s.tables;
  if (ts.self_up1.empty()) return;
  std::vector<float> h;
  h.reserve(ts.self_up1.size() + ts.self_dn1.size());
  for (double x : ts.self_up1) h.push_back((float)(s.t * x));
  for (double x : ts.self_dn1) h.push_back((float)(s.t * x));
  s.selfe = std::make_unique<EngBuf>(sizeof(float) * h.size(), e->pool, e->st);
  // on st, after the pool hands the block over (pageable source: staged
  // before the call returns)
  MB_CUDA(cudaMemcpyAsync(s.selfe->p, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice,
                          e->st));
}

OpView slot_view(const EngineSlot& s) {
  const TableSet& ts = *s.tables;
  OpView v = ts.fused;
  v.Du = s.Du;
  v.Dd = s.Dd;
  v.dim = s.dim;
  v.L = ts.basis.L;
  v.up_mask = ts.up_mask;
  v.dn_mask = ts.dn_mask;
  v.up_off = ts.up_off;
  v.up_ent = ts.up_ent;
  v.dn_off = ts.dn_off;
  v.dn_ent = ts.dn_ent;
  v.max_up_degree = ts.max_up_deg;
  v.max_dn_degree = ts.max_dn_deg;
  v.t = s.t;
  return v;
}

// Work-list buffers only grow (by half again), so admissions and
// retirements do not free and reallocate device memory every time.
void reserve(std::unique_ptr<EngBuf>& b, size_t bytes) {
  if (b && b->bytes >= bytes) return;
  const size_t want = b ? std::max(bytes, b->bytes + b->bytes / 2) : bytes;
  b.reset();
  b = std::make_unique<EngBuf>(want);
}

void rebuild(mb_engine_s* e) {
  if (!e->dirty) return;
  // h_slots holds the device state of the previous list (fetched after the
  // last step, host edits since): keep each surviving slot's progress
  std::map<const float2*, SlotDesc> old;
  for (const SlotDesc& od : e->h_slots) old[od.buf[0]] = od;
  e->h_slots.clear();
  std::vector<int2> items, items_warp, items_rows;
  int max_list = 0;
  e->row_cols = 0;
  for (auto& sp : e->slots) {
    EngineSlot& s = *sp;
    SlotDesc d{};
    const TableSet& ts = *s.tables;
    d.up_mask = ts.up_mask;
    d.dn_mask = ts.dn_mask;
    d.up_off = ts.up_off;
    d.up_ent = ts.up_ent;
    d.dn_off = ts.dn_off;
    d.dn_ent = ts.dn_ent;
    d.Du = s.Du;
    d.Dd = s.Dd;
    float2* base = (float2*)s.vecs->p;
    for (int q = 0; q < 3; ++q) d.buf[q] = base + (size_t)q * (size_t)s.dim;
    d.xacc = base + 3 * (size_t)s.dim;
    double* sc = (double*)s.scal->p;
    d.alpha = sc;
    d.beta = sc + kEngMaxK;
    d.yk = sc + 2 * kEngMaxK;
    d.ib = reinterpret_cast<float*>(reinterpret_cast<char*>(sc) + kEngIbAt);
    const std::vector<double> uf = u_fold_table(s.u, !(s.u * s.u < kTol * kTol), ts.basis.L);
    for (int kk = 0; kk <= kMaxOrbitals; ++kk) d.ufold[kk] = kk < (int)uf.size() ? (float)uf[(size_t)kk] : 0.f;
    d.t = (float)s.t;
    d.scale = s.scale;
    d.kmax = (int)s.kmax;
    d.item0 = (int)items.size();
    for (int64_t r = 0; r < s.Du; ++r) items.push_back(make_int2((int)e->h_slots.size(), (int)r));
    d.item1 = (int)items.size();
    d.fused = s.dim >= e->fused_min ? 1 : 0;
    d.up_list = ts.fused.up_list;
    d.up_loff = ts.fused.up_loff;
    d.up_lpos = ts.fused.up_lpos;
    d.dn_sell = ts.fused.dn_sell;
    d.dn_sgrp = ts.fused.dn_sgrp;
    d.self_up = s.selfe ? (const float*)s.selfe->p : nullptr;
    d.self_dn = s.selfe ? (const float*)s.selfe->p + s.Du : nullptr;
    d.basis = s.basis ? (float2*)s.basis->p : nullptr;
    if (e->persistent) {
      // the persistent step applies a sector's rows block per row when they
      // are wide (or the sector is large), else warp per row
      const bool rows = d.fused || s.Dd >= e->p_row_min_cols;
      auto& list = rows ? items_rows : items_warp;
      for (int64_t r = 0; r < s.Du; ++r) list.push_back(make_int2((int)e->h_slots.size(), (int)r));
      if (rows) {
        e->row_cols = std::max(e->row_cols, (int)s.Dd);
        max_list = std::max(max_list, ts.fused.max_up_list);
      }
      d.fused = 0;
    } else if (!d.fused) {
      const bool rows = s.Dd >= kEngRowMinCols;
      auto& list = rows ? items_rows : items_warp;
      for (int64_t r = 0; r < s.Du; ++r) list.push_back(make_int2((int)e->h_slots.size(), (int)r));
      if (rows) {
        e->row_cols = std::max(e->row_cols, (int)s.Dd);
        max_list = std::max(max_list, ts.fused.max_up_list);
      }
    }
    auto o = old.find(d.buf[0]);
    if (o != old.end()) {
      d.k = o->second.k;
      d.mode = o->second.mode;
      d.steps = o->second.steps;
      d.kmax = o->second.kmax;
      d.cheb_a = o->second.cheb_a;
      d.cheb_b = o->second.cheb_b;
    } else {  // admitted since: its vectors were seeded at submission
      d.k = 0;
      d.mode = kModeLanczos;
      d.steps = 0;
    }
    e->h_slots.push_back(d);
  }
  e->n_items = (int)items.size();
  reserve(e->d_slots, sizeof(SlotDesc) * std::max<size_t>(e->h_slots.size(), 1));
  reserve(e->d_items, sizeof(int2) * std::max<size_t>(items.size(), 1));
  reserve(e->d_part, 2 * sizeof(double) * std::max<size_t>(items.size(), 1));
  // fused slots: device addresses of their step state in the new slot array
  e->fused.clear();
  e->fused_scratch.clear();
  SlotDesc* dsl = (SlotDesc*)e->d_slots->p;
  double* part = (double*)e->d_part->p;
  for (size_t i = 0; i < e->h_slots.size(); ++i) {
    const SlotDesc& d = e->h_slots[i];
    if (!d.fused) continue;
    const OpView v = slot_view(*e->slots[i]);
    EngFusedArgs a{};
    a.k = &dsl[i].k;
    a.mode = &dsl[i].mode;
    a.kmax = &dsl[i].kmax;
    a.steps = &dsl[i].steps;
    a.beta = d.beta;
    a.ufold = dsl[i].ufold;
    a.self_up = d.self_up;
    a.self_dn = d.self_dn;
    for (int q = 0; q < 3; ++q) a.buf[q] = d.buf[q];
    a.t = d.t;
    a.scale = d.scale;
    a.cheb_a = &dsl[i].cheb_a;
    a.cheb_b = &dsl[i].cheb_b;
    a.part = part;
    a.part2 = part + items.size();  // the second half of d_part, as step_kernels uses it
    a.item0 = d.item0;
    a.n_items = d.item1 - d.item0;
    e->fused_scratch.push_back(
        std::make_unique<EngBuf>(3 * sizeof(double) * (size_t)std::max(eng_fused_blocks(v), 1)));
    a.scratch = (double*)e->fused_scratch.back()->p;
    e->fused.push_back({v, a});
  }
  if (!e->fused.empty()) prepare_eng_fused();
  if (!e->h_slots.empty())
    MB_CUDA(cudaMemcpyAsync(e->d_slots->p, e->h_slots.data(), sizeof(SlotDesc) * e->h_slots.size(),
                            cudaMemcpyHostToDevice, e->st));
  if (!items.empty())
    MB_CUDA(cudaMemcpyAsync(e->d_items->p, items.data(), sizeof(int2) * items.size(),
                            cudaMemcpyHostToDevice, e->st));
  e->n_warp = (int)items_warp.size();
  e->n_rows = (int)items_rows.size();
  reserve(e->d_items_warp, sizeof(int2) * std::max<size_t>(items_warp.size(), 1));
  reserve(e->d_items_rows, sizeof(int2) * std::max<size_t>(items_rows.size(), 1));
  if (!items_warp.empty())
    MB_CUDA(cudaMemcpyAsync(e->d_items_warp->p, items_warp.data(),
                            sizeof(int2) * items_warp.size(), cudaMemcpyHostToDevice, e->st));
  if (e->persistent) {
    if (!items_rows.empty())
      MB_CUDA(cudaMemcpyAsync(e->d_items_rows->p, items_rows.data(),
                              sizeof(int2) * items_rows.size(), cudaMemcpyHostToDevice, e->st));
    // launch shape, set outside any capture: the staged row and its up list,
    // or the warps' rows, in dynamic shared memory; co-resident blocks
    const size_t rows_smem = sizeof(float2) * (size_t)(e->row_cols + kSlicedPads) +
                             sizeof(uint32_t) * (size_t)((max_list + 3) & ~3);
    const size_t warps_smem = sizeof(float2) * (size_t)kEngPWarps * kEngWarpRowCols;
    e->p_smem = std::max(rows_smem, warps_smem);
    MB_CUDA(cudaFuncSetAttribute(k_eng_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)e->p_smem));
    int bps = 0, sms = 0, dev = 0;
    MB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_eng_persistent,
                                                          kEngPWarps * 32, e->p_smem));
    MB_REQUIRE(bps >= 1, MB_ERR_CAPACITY, "the persistent engine step does not fit on an SM");
    MB_CUDA(cudaGetDevice(&dev));
    MB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    e->p_bps = bps;
    e->p_sms = sms;
    const int per_sm = e->p_ctas_per_sm > 0 ? std::min(e->p_ctas_per_sm, bps) : bps;
    e->p_grid = std::max(1, per_sm * sms);
    if (!e->d_grid) e->d_grid = std::make_unique<EngBuf>(sizeof(EngGrid));
  } else if (!items_rows.empty()) {
    MB_CUDA(cudaMemcpyAsync(e->d_items_rows->p, items_rows.data(),
                            sizeof(int2) * items_rows.size(), cudaMemcpyHostToDevice, e->st));
    // launch shape, set outside any capture: shared memory and resident blocks
    e->row_smem = sizeof(float2) * (size_t)(e->row_cols + kSlicedPads) +
                  sizeof(uint32_t) * (size_t)((max_list + 3) & ~3);
    MB_CUDA(cudaFuncSetAttribute(k_eng_apply_rows, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)e->row_smem));
    int bps = 0, sms = 0, dev = 0;
    MB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, k_eng_apply_rows,
                                                          kEngRowWarps * 32, e->row_smem));
    MB_CUDA(cudaGetDevice(&dev));
    MB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    e->row_grid = std::max(1, std::min(e->n_rows, std::max(bps, 1) * sms));
  }
  MB_CUDA(cudaStreamSynchronize(e->st));
  e->dirty = false;
}

// Pull the per-slot mode/k/steps fields back after a step.
void fetch_slots(mb_engine_s* e) {
  if (e->h_slots.empty()) return;
  MB_CUDA(cudaMemcpyAsync(e->h_slots.data(), e->d_slots->p, sizeof(SlotDesc) * e->h_slots.size(),
                          cudaMemcpyDeviceToHost, e->st));
  MB_CUDA(cudaStreamSynchronize(e->st));
}

void push_slots(mb_engine_s* e) {
  if (e->h_slots.empty()) return;
  MB_CUDA(cudaMemcpyAsync(e->d_slots->p, e->h_slots.data(), sizeof(SlotDesc) * e->h_slots.size(),
                          cudaMemcpyHostToDevice, e->st));
  MB_CUDA(cudaStreamSynchronize(e->st));
}

int eng_grid(int n_items, int warps) {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  }
  int g = (n_items + warps - 1) / warps;
  const int cap = sms * (2048 / (32 * warps));
  return std::max(1, std::min(g, cap));
}

template <int W>
void step_kernels(mb_engine_s* e) {
  const SlotDesc* ds = (const SlotDesc*)e->d_slots->p;
  SlotDesc* dsm = (SlotDesc*)e->d_slots->p;
  const int2* it = (const int2*)e->d_items->p;
  double* part = (double*)e->d_part->p;
  const int n = e->n_items, ns = (int)e->h_slots.size();
  double* part2 = part + n;
  const int g = eng_grid(n, W);
  if (e->n_warp)
    k_eng_apply<W><<<eng_grid(e->n_warp, W), W * 32, 0, e->st>>>(
        ds, (const int2*)e->d_items_warp->p, e->n_warp, part, part2);
  if (e->n_rows)
    k_eng_apply_rows<<<e->row_grid, kEngRowWarps * 32, e->row_smem, e->st>>>(
        ds, (const int2*)e->d_items_rows->p, e->n_rows, e->row_cols, part, part2);
  for (const auto& [v, a] : e->fused) launch_eng_fused(v, a, e->st);
  k_eng_seg_reduce<<<std::min(ns, 1024), 256, 0, e->st>>>(dsm, ns, part, part2, 0);
  k_eng_update<W><<<g, W * 32, 0, e->st>>>(ds, it, n, part);
  k_eng_replay_update<W><<<g, W * 32, 0, e->st>>>(ds, it, n);
  k_eng_seg_reduce<<<std::min(ns, 1024), 256, 0, e->st>>>(dsm, ns, part, part2, 1);
  k_eng_normalize<W><<<g, W * 32, 0, e->st>>>(ds, it, n);
  k_eng_advance<<<(ns + 255) / 256, 256, 0, e->st>>>(dsm, ns);
}

// The persistent step: the barrier state cleared, then one cooperative
// launch of `steps` engine steps (graph-capturable).
void launch_persistent(mb_engine_s* e, int steps, bool apply_only = false) {
  EngPersistArgs a{};
  a.slots = (SlotDesc*)e->d_slots->p;
  a.n_slots = (int)e->h_slots.size();
  a.items = (const int2*)e->d_items->p;
  a.n_items = e->n_items;
  a.items_rows = (const int2*)e->d_items_rows->p;
  a.n_rows = e->n_rows;
  a.items_warp = (const int2*)e->d_items_warp->p;
  a.n_warp = e->n_warp;
  a.part = (double*)e->d_part->p;
  a.part2 = a.part + e->n_items;
  a.row_cols = e->row_cols;
  a.steps = steps;
  a.apply_only = apply_only ? 1 : 0;
  a.grid = (EngGrid*)e->d_grid->p;
  a.budget = e->wait_budget;
  MB_CUDA(cudaMemsetAsync(e->d_grid->p, 0, sizeof(EngGrid), e->st));
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)e->p_grid);
  cfg.blockDim = dim3(kEngPWarps * 32);
  cfg.dynamicSmemBytes = e->p_smem;
  cfg.stream = e->st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  MB_CUDA(cudaLaunchKernelEx(&cfg, k_eng_persistent, a));
}

// MB_ERR_TIMEOUT once a barrier wait of the persistent step ran out (the
// engine's requests are then lost: a step stopped part-way).
void check_grid(mb_engine_s* e) {
  if (!e->persistent || !e->d_grid) return;
  EngGrid g{};
  MB_CUDA(cudaMemcpyAsync(&g, e->d_grid->p, sizeof(EngGrid), cudaMemcpyDeviceToHost, e->st));
  MB_CUDA(cudaStreamSynchronize(e->st));
  if (g.status != 0) {
    e->broken = true;
    throw Error(MB_ERR_TIMEOUT,
                "a grid barrier of the persistent engine step waited past its budget; "
                "the engine's requests are lost (destroy the engine)");
  }
}

void launch_step(mb_engine_s* e) {
  if (e->persistent) {
    launch_persistent(e, 1);
    return;
  }
  switch (e->warps) {
    case 2: step_kernels<2>(e); break;
    case 4: step_kernels<4>(e); break;
    case 16: step_kernels<16>(e); break;
    default: step_kernels<8>(e); break;
  }
  MB_CUDA(cudaGetLastError());
}

// Seed, normalise and arm a slot for pass one (or replay).
// ||v||^2 into out[0] (out holds kEngNormBlocks + 1 doubles of scratch).
constexpr int kEngNormBlocks = 128;
void eng_norm2(mb_engine_s* e, const float2* v, int64_t n, double* out) {
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(kEngNormBlocks, (n + 8191) / 8192));
  k_eng_norm2<<<nb, 256, 0, e->st>>>(v, n, out + 1);
  k_eng_sum<<<1, 1, 0, e->st>>>(out + 1, nb, out);
}

// Seeds v = buf[1] (normalised start vector) and zeroes v_prev = buf[0],
// all on the device (no host wait): the norm goes to the slot's scalar table
// (kEngNormAt), which the host reads with alpha and beta once pass one ends.
// A Philox uniform(-1, 1) vector is never zero (its entries are never all 0).
void seed_vectors(mb_engine_s* e, EngineSlot& s, float2* b0, float2* b1) {
  if (!e->d_norm) e->d_norm = std::make_unique<EngBuf>(sizeof(double) * (kEngNormBlocks + 1));
  double* nb = (double*)e->d_norm->p;
  k_eng_seed<<<256, 256, 0, e->st>>>(b1, s.dim, s.seed, 1.0);
  eng_norm2(e, b1, s.dim, nb);
  k_eng_scale_by_norm<<<256, 256, 0, e->st>>>(b1, s.dim, nb, (double*)s.scal->p + kEngNormAt);
  MB_CUDA(cudaGetLastError());
  MB_CUDA(cudaMemsetAsync(b0, 0, 8 * (size_t)s.dim, e->st));
}

void arm_slot(mb_engine_s* e, EngineSlot& s, SlotDesc& d, bool replay) {
  seed_vectors(e, s, d.buf[0], d.buf[1]);
  d.k = 0;
  if (replay) {
    d.mode = kModeReplay;
    d.steps = s.m_ritz;
  } else {
    d.mode = kModeLanczos;
    d.steps = 0;
  }
}

double ritz_min(const std::vector<double>& a, const std::vector<double>& b, int m,
                std::vector<double>* vec) {
  std::vector<double> d(a.begin(), a.begin() + m), z, ee(b.begin(), b.begin() + std::max(m - 1, 0));
  MB_REQUIRE(tridiag_eig(m, d, ee, vec ? &z : nullptr), MB_ERR_EIG_FAILED,
             "Eigenvalue decomposition of T_k failed");
  if (vec) {
    vec->assign((size_t)m, 0.0);
    for (int i = 0; i < m; ++i) (*vec)[(size_t)i] = z[(size_t)(m - 1) * m + i];
  }
  return d[(size_t)m - 1];  // largest of -T: -E0
}

// FP64 refinement of finished ground-state requests, all at once: each
// slot's FP64 operator view (the engine's tables, its U fold and self
// energies in FP64) and its Ritz vector in FP64 go to fp64_refine_many,
// which advances them in lockstep (one host wait per Krylov step for all).
// The start vectors of a call stay under kEngRefineBytes; more requests run
// in further calls.
constexpr size_t kEngRefineBytes = (size_t)4 << 30;

void refine_slots(mb_engine_s* e, const std::vector<size_t>& idx) {
  size_t i0 = 0;
  while (i0 < idx.size()) {
    size_t xbytes = 0, i1 = i0;
    while (i1 < idx.size()) {
      const EngineSlot& s = *e->slots[idx[i1]];
      const size_t b = 16 * (size_t)s.dim;
      if (i1 > i0 && xbytes + b > kEngRefineBytes) break;
      xbytes += b;
      ++i1;
    }
    const size_t n = i1 - i0;
    std::vector<double> tab;
    std::vector<size_t> uoff(n), soff(n, SIZE_MAX);
    for (size_t j = 0; j < n; ++j) {
      const EngineSlot& s = *e->slots[idx[i0 + j]];
      const TableSet& ts = *s.tables;
      const std::vector<double> uf = u_fold_table(s.u, !(s.u * s.u < kTol * kTol), ts.basis.L);
      uoff[j] = tab.size();
      tab.insert(tab.end(), uf.begin(), uf.end());
      if (!ts.self_up1.empty()) {
        soff[j] = tab.size();
        for (double x : ts.self_up1) tab.push_back(s.t * x);
        for (double x : ts.self_dn1) tab.push_back(s.t * x);
      }
    }
    EngBuf dtab(sizeof(double) * tab.size(), e->pool, e->st), xs(xbytes, e->pool, e->st);
    MB_CUDA(cudaMemcpyAsync(dtab.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice,
                            e->st));
    std::vector<RefineProblem> probs(n);
    char* xp = (char*)xs.p;
    for (size_t j = 0; j < n; ++j) {
      const EngineSlot& s = *e->slots[idx[i0 + j]];
      const SlotDesc& d = e->h_slots[idx[i0 + j]];
      RefineProblem& p = probs[j];
      p.v = slot_view(s);
      p.v.u_fold = (const double*)dtab.p + uoff[j];
      p.v.self_up = p.v.self_dn = nullptr;
      if (soff[j] != SIZE_MAX) {
        p.v.self_up = (const double*)dtab.p + soff[j];
        p.v.self_dn = p.v.self_up + s.Du;
      }
      k_f32_to_f64<<<256, 256, 0, e->st>>>(d.xacc, (double2*)xp, s.dim);
      MB_CUDA(cudaGetLastError());
      p.x = xp;
      xp += 16 * (size_t)s.dim;
    }
    // Rayleigh-Ritz on span{x, Hx, ...} in FP64 (its first step is the
    // Rayleigh quotient of the Ritz vector)
    fp64_refine_many(probs.data(), (int)n, e->st);
    for (size_t j = 0; j < n; ++j) {
      EngineSlot& s = *e->slots[idx[i0 + j]];
      s.e0 = probs[j].e0;
      s.phase = 2;
    }
    i0 = i1;
  }
}

// Seed probe `p` of a DOS request into buf[1] and arm Chebyshev mode.
void arm_probe(mb_engine_s* e, EngineSlot& s, SlotDesc& d) {
  k_eng_seed_phase<<<256, 256, 0, e->st>>>(d.buf[1], s.dim, s.seed, (uint32_t)(1 + s.probe));
  EngBuf nb(sizeof(double) * (kEngNormBlocks + 1));
  eng_norm2(e, d.buf[1], s.dim, (double*)nb.p);
  MB_CUDA(cudaMemcpyAsync(&s.mu0, nb.p, sizeof(double), cudaMemcpyDeviceToHost, e->st));
  MB_CUDA(cudaMemsetAsync(d.buf[0], 0, 8 * (size_t)s.dim, e->st));
  MB_CUDA(cudaStreamSynchronize(e->st));
  const double a = (s.emax - s.emin) / 2.0 * (1.0 + s.padding);  // rescaling.h:33-38
  const double b = (s.emax + s.emin) / 2.0;
  d.cheb_a = (float)a;
  d.cheb_b = (float)b;
  d.mode = kModeCheb;
  d.k = 0;
  d.steps = 0;
  d.kmax = std::max(s.n_moments / 2, 1);
}

// DOS bookkeeping when a slot's device phase went idle.
void dos_transition(mb_engine_s* e, EngineSlot& s, SlotDesc& d, bool& changed) {
  if (s.phase == 10) {
    // spectral bounds: extremal Ritz values of pass one on H, widened by
    // their residual bounds beta_m |z_m|
    const int m = d.steps;
    std::vector<double> a((size_t)m), b((size_t)m);
    MB_CUDA(cudaMemcpy(a.data(), d.alpha, sizeof(double) * m, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(b.data(), d.beta, sizeof(double) * m, cudaMemcpyDeviceToHost));
    std::vector<double> dd(a), z, ee(b.begin(), b.begin() + std::max(m - 1, 0));
    MB_REQUIRE(tridiag_eig(m, dd, ee, &z), MB_ERR_EIG_FAILED, "Eigenvalue decomposition of T_k failed");
    const double bm = b[(size_t)m - 1];
    const double rlo = bm * std::fabs(z[(size_t)0 * m + (m - 1)]);
    const double rhi = bm * std::fabs(z[(size_t)(m - 1) * m + (m - 1)]);
    s.emin = dd[0] - rlo;
    s.emax = dd[(size_t)m - 1] + rhi;
    if (!(s.emax > s.emin)) s.emax = s.emin + 1.0;
    s.mu.assign((size_t)s.n_moments, 0.0);
    s.probe = 0;
    arm_probe(e, s, d);
    s.phase = 11;
    changed = true;
  } else if (s.phase == 11) {
    const int ns = d.steps;
    std::vector<double> a((size_t)ns), b((size_t)ns);
    MB_CUDA(cudaMemcpy(a.data(), d.alpha, sizeof(double) * ns, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(b.data(), d.beta, sizeof(double) * ns, cudaMemcpyDeviceToHost));
    // mu_0 = <T0,T0>, mu_1 = <T0,T1>, mu_2n = 2<Tn,Tn> - mu_0, mu_2n+1 = 2<Tn+1,Tn> - mu_1
    const double mu0 = s.mu0, mu1 = ns > 0 ? a[0] : 0.0;
    s.mu[0] += mu0;
    if (s.n_moments > 1) s.mu[1] += mu1;
    for (int n = 1; 2 * n < s.n_moments; ++n) {
      s.mu[(size_t)(2 * n)] += 2.0 * b[(size_t)n - 1] - mu0;
      if (2 * n + 1 < s.n_moments) s.mu[(size_t)(2 * n + 1)] += 2.0 * a[(size_t)n] - mu1;
    }
    s.probe += 1;
    if (s.probe < s.n_probes) {
      arm_probe(e, s, d);
    } else {
      const double norm = 1.0 / ((double)s.n_probes * (double)s.dim);
      for (auto& v : s.mu) v *= norm;
      s.phase = 2;
    }
    changed = true;
  }
}

// Host bookkeeping after a step: convergence, replay, refinement, retirement.
void after_step(mb_engine_s* e) {
  check_grid(e);
  fetch_slots(e);
  bool changed = false;
  std::vector<size_t> to_refine;  // slots whose Ritz vectors are ready
  for (size_t i = 0; i < e->slots.size(); ++i) {
    EngineSlot& s = *e->slots[i];
    SlotDesc& d = e->h_slots[i];
    if (s.phase == 0 && s.kind == 0) {
      const int m = d.steps;
      bool finished = d.mode == kModeIdle, converged = false;
      if (!finished && s.rel_tol > 0.0 && m >= 2 && (m % s.check_every) == 0) {
        // alpha and beta sit kEngMaxK apart in one buffer: one copy; the
        // extreme Ritz value by Sturm bisection (O(m) a sweep), not a full
        // eigensolve of T_m
        std::vector<double> ab((size_t)(kEngMaxK + m));
        MB_CUDA(cudaMemcpy(ab.data(), d.alpha, sizeof(double) * ab.size(), cudaMemcpyDeviceToHost));
        const double r = tridiag_max_eig(ab.data(), ab.data() + kEngMaxK, m);
        if (s.have_ritz && std::fabs(r - s.last_ritz) <= s.rel_tol * std::fabs(r)) finished = converged = true;
        s.last_ritz = r;
        s.have_ritz = true;
      }
      if (finished) {
        s.m = m;
        std::vector<double> a((size_t)m), b((size_t)m), y;
        MB_CUDA(cudaMemcpy(a.data(), d.alpha, sizeof(double) * m, cudaMemcpyDeviceToHost));
        MB_CUDA(cudaMemcpy(b.data(), d.beta, sizeof(double) * m, cudaMemcpyDeviceToHost));
        MB_CUDA(cudaMemcpy(&s.b_norm, (const double*)s.scal->p + kEngNormAt, sizeof(double),
                           cudaMemcpyDeviceToHost));
        s.e_raw = -ritz_min(a, b, m, nullptr);
        s.e0 = s.e_raw;
        if (s.refine && m > 0) {
          // a run that stopped on its convergence test ends before a ghost
          // copy of the ground state can enter T_m; one that ran to kmax
          // takes its Ritz vector from the first converged checkpoint
          s.m_ritz = converged ? m : ritz_vector_steps(a, b, m, s.check_every, 1e-9);
          ritz_min(a, b, s.m_ritz, &y);
          for (auto& yv : y) yv *= s.b_norm;
          MB_CUDA(cudaMemcpy(d.yk, y.data(), sizeof(double) * s.m_ritz, cudaMemcpyHostToDevice));
          if (s.basis) {
            // the Ritz vector from the kept Lanczos vectors (the replay's
            // bits); the FP64 refinement after this pass over the slots
            const int64_t nb = std::max<int64_t>(1, std::min<int64_t>((s.dim + 255) / 256, 4096));
            k_eng_combine<<<(unsigned)nb, 256, 0, e->st>>>((const float2*)s.basis->p, s.dim,
                                                          s.m_ritz, d.yk, d.xacc);
            MB_CUDA(cudaGetLastError());
            to_refine.push_back(i);
          } else {
            arm_slot(e, s, d, true);
            // x = y_0 v_0, v_prev = 0
            const int2* it = (const int2*)e->d_items->p;
            push_slots(e);
            k_eng_replay_init<8><<<eng_grid(d.item1 - d.item0, 8), 256, 0, e->st>>>(
                (const SlotDesc*)e->d_slots->p, it + d.item0, d.item1 - d.item0);
            s.phase = 1;
          }
        } else {
          s.phase = 2;
        }
        changed = true;
      }
    } else if (s.phase == 1 && d.mode == kModeIdle) {
      to_refine.push_back(i);
      changed = true;
    } else if ((s.phase == 10 || s.phase == 11) && d.mode == kModeIdle) {
      dos_transition(e, s, d, changed);
    }
  }
  if (!to_refine.empty()) refine_slots(e, to_refine);
  // retire finished slots
  for (size_t i = 0; i < e->slots.size();) {
    if (e->slots[i]->phase == 2) {
      auto sp = std::move(e->slots[i]);
      sp->t_done = std::chrono::steady_clock::now();
      e->in_use -= sp->bytes;
      sp->vecs.reset();
      sp->scal.reset();
      sp->basis.reset();
      sp->selfe.reset();
      sp->tables.reset();
      e->newly_done.push_back(sp->id);
      e->done[sp->id] = std::move(sp);
      e->slots.erase(e->slots.begin() + (long)i);
      changed = true;
    } else {
      ++i;
    }
  }
  if (changed) {  // new work lists; rebuild keeps the survivors' progress
    e->dirty = true;
    rebuild(e);
  }
}

}  // namespace
}  // namespace mb

using namespace mb;

extern "C" {

int mb_engine_create(int64_t device_bytes_budget, mb_engine_t* out) {
  return guard([&] {
    MB_REQUIRE(out, MB_ERR_INVALID_ARG, "NULL argument");
    int n = 0;
    MB_REQUIRE(cudaGetDeviceCount(&n) == cudaSuccess && n > 0, MB_ERR_NO_DEVICE,
               "no CUDA device available");
    auto e = std::make_unique<mb_engine_s>();
    size_t free_b = 0, total_b = 0;
    MB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    e->budget = device_bytes_budget > 0 ? device_bytes_budget : (int64_t)(free_b * 0.8);
    MB_CUDA(cudaStreamCreateWithFlags(&e->st, cudaStreamNonBlocking));
    for (cudaEvent_t& x : e->ev) MB_CUDA(cudaEventCreate(&x));
    int dev = 0;
    MB_CUDA(cudaGetDevice(&dev));
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    MB_CUDA(cudaMemPoolCreate(&e->pool, &props));
    uint64_t keep = UINT64_MAX;  // freed blocks stay in the pool for the next requests
    MB_CUDA(cudaMemPoolSetAttribute(e->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    *out = (mb_engine_t)e.release();
  });
}

int mb_engine_destroy(mb_engine_t eng) {
  auto* e = (mb_engine_s*)eng;
  if (e) {
    cudaStreamSynchronize(e->st);
    delete e;
  }
  return MB_OK;
}

int mb_engine_footprint(const mb_sector_desc* d, int64_t* bytes) {
  return guard([&] {
    MB_REQUIRE(d && bytes, MB_ERR_INVALID_ARG, "NULL argument");
    int64_t L = 1;
    for (int i = 0; i < d->ndim; ++i) L *= d->dims[i];
    MB_REQUIRE(L >= 1 && L <= kMaxOrbitals, MB_ERR_CAPACITY, "orbitals must be in [1, 32]");
    const int64_t dim = binom_at(binom_table(), (int)L, d->n_up) * binom_at(binom_table(), (int)L, d->n_down);
    *bytes = slot_bytes(dim);
  });
}

int mb_engine_submit_ground_state(mb_engine_t eng, const mb_sector_desc* desc, uint64_t seed,
                                  int64_t kmax, double rel_tol, int refine, int64_t* request_id) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && desc && request_id, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    MB_REQUIRE(kmax >= 1 && kmax <= kEngMaxK, MB_ERR_INVALID_ARG, "kmax must be in [1, 512]");
    MB_REQUIRE(desc->ndim >= 1 && desc->ndim <= 3, MB_ERR_INVALID_ARG, "ndim must be 1..3");
    MB_REQUIRE(!(desc->t * desc->t < kTol * kTol), MB_ERR_INVALID_ARG, "t must be non-zero");
    int64_t need = 0;
    int rc = mb_engine_footprint(desc, &need);
    if (rc) throw Error(rc, mb_last_error());
    MB_REQUIRE(e->in_use + need <= e->budget, MB_ERR_CAPACITY,
               "device-memory budget full: retry after a step retires requests");
    auto s = std::make_unique<EngineSlot>();
    s->tables = get_tables(e, *desc);
    s->t = desc->t;
    s->u = desc->u;
    s->seed = seed;
    s->kmax = std::min<int64_t>(kmax, s->tables->basis.dim);
    s->rel_tol = rel_tol;
    s->refine = refine;
    s->Du = s->tables->basis.up.D;
    s->Dd = s->tables->basis.down.D;
    s->dim = s->tables->basis.dim;
    s->bytes = need;
    s->vecs = std::make_unique<EngBuf>(4 * 8 * (size_t)s->dim, e->pool, e->st);
    s->scal = std::make_unique<EngBuf>(kEngScalBytes, e->pool, e->st);
    upload_self_energies(e, *s);
    const int64_t basis_bytes = 8 * s->kmax * s->dim;
    if (refine && basis_bytes <= e->basis_limit && e->in_use + need + basis_bytes <= e->budget) {
      // every vector the Ritz sum reads is written by pass one first
      s->basis = std::make_unique<EngBuf>((size_t)basis_bytes, e->pool, e->st);
      need += basis_bytes;
      s->bytes = need;
    }
    s->id = e->next_id++;
    s->t_submit = std::chrono::steady_clock::now();
    float2* base = (float2*)s->vecs->p;
    seed_vectors(e, *s, base, base + s->dim);
    if (s->basis)  // v_0, the normalised start vector
      MB_CUDA(cudaMemcpyAsync(s->basis->p, base + s->dim, 8 * (size_t)s->dim,
                              cudaMemcpyDeviceToDevice, e->st));
    e->in_use += need;
    *request_id = s->id;
    // joins at the next step (rebuild keeps the others' progress)
    e->slots.push_back(std::move(s));
    e->dirty = true;
  });
}

int mb_engine_submit_dos(mb_engine_t eng, const mb_sector_desc* desc, int64_t n_moments,
                         int64_t n_probes, uint64_t seed, double padding, int64_t* request_id) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && desc && request_id, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    MB_REQUIRE(n_moments >= 2 && n_moments <= 2 * kEngMaxK, MB_ERR_INVALID_ARG,
               "n_moments must be in [2, 1024]");
    MB_REQUIRE(n_probes >= 1, MB_ERR_INVALID_ARG, "n_probes must be >= 1");
    MB_REQUIRE(desc->ndim >= 1 && desc->ndim <= 3, MB_ERR_INVALID_ARG, "ndim must be 1..3");
    MB_REQUIRE(!(desc->t * desc->t < kTol * kTol), MB_ERR_INVALID_ARG, "t must be non-zero");
    int64_t need = 0;
    int rc = mb_engine_footprint(desc, &need);
    if (rc) throw Error(rc, mb_last_error());
    MB_REQUIRE(e->in_use + need <= e->budget, MB_ERR_CAPACITY,
               "device-memory budget full: retry after a step retires requests");
    auto s = std::make_unique<EngineSlot>();
    s->tables = get_tables(e, *desc);
    s->kind = 1;
    s->scale = 1.f;
    s->t = desc->t;
    s->u = desc->u;
    s->seed = seed;
    s->Du = s->tables->basis.up.D;
    s->Dd = s->tables->basis.down.D;
    s->dim = s->tables->basis.dim;
    s->kmax = std::min<int64_t>(40, s->dim);  // Lanczos steps for the spectral bounds
    s->n_moments = (int)n_moments;
    s->n_probes = (int)n_probes;
    s->padding = padding;
    s->bytes = need;
    s->vecs = std::make_unique<EngBuf>(4 * 8 * (size_t)s->dim, e->pool, e->st);
    s->scal = std::make_unique<EngBuf>(kEngScalBytes, e->pool, e->st);
    upload_self_energies(e, *s);
    s->id = e->next_id++;
    s->t_submit = std::chrono::steady_clock::now();
    s->phase = 10;
    float2* base = (float2*)s->vecs->p;
    seed_vectors(e, *s, base, base + s->dim);
    e->in_use += need;
    *request_id = s->id;
    e->slots.push_back(std::move(s));
    e->dirty = true;
  });
}

int mb_engine_poll_dos(mb_engine_t eng, int64_t id, int* done, double* mu, double* e_min,
                       double* e_max, double* latency_s) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && done, MB_ERR_INVALID_ARG, "NULL argument");
    auto it = e->done.find(id);
    if (it == e->done.end()) {
      *done = 0;
      return;
    }
    const EngineSlot& s = *it->second;
    MB_REQUIRE(s.kind == 1, MB_ERR_INVALID_ARG, "request is not a DOS request");
    *done = 1;
    if (mu) std::copy(s.mu.begin(), s.mu.end(), mu);
    if (e_min) *e_min = s.emin;
    if (e_max) *e_max = s.emax;
    if (latency_s) *latency_s = std::chrono::duration<double>(s.t_done - s.t_submit).count();
  });
}

int mb_engine_step(mb_engine_t eng, int n_steps, int* n_active) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && n_steps >= 0, MB_ERR_INVALID_ARG, "bad argument");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    for (int i = 0; i < n_steps && !e->slots.empty(); ++i) {
      const auto t0 = std::chrono::steady_clock::now();
      rebuild(e);
      MB_CUDA(cudaEventRecord(e->ev[0], e->st));
      launch_step(e);
      MB_CUDA(cudaEventRecord(e->ev[1], e->st));
      after_step(e);  // waits on the stream: both events have completed
      float ms = 0.f;
      MB_CUDA(cudaEventElapsedTime(&ms, e->ev[0], e->ev[1]));
      e->stat_dev_ms += ms;
      e->stat_wall_ms +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
      ++e->stat_steps;
    }
    if (n_active) *n_active = (int)e->slots.size();
  });
}

int mb_engine_poll(mb_engine_t eng, int64_t id, int* done, double* e0, double* e0_raw,
                   int64_t* steps, double* latency_s) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && done, MB_ERR_INVALID_ARG, "NULL argument");
    auto it = e->done.find(id);
    if (it == e->done.end()) {
      *done = 0;
      return;
    }
    const EngineSlot& s = *it->second;
    *done = 1;
    if (e0) *e0 = s.e0;
    if (e0_raw) *e0_raw = s.e_raw;
    if (steps) *steps = s.m;
    if (latency_s) *latency_s = std::chrono::duration<double>(s.t_done - s.t_submit).count();
  });
}

int mb_engine_completed(mb_engine_t eng, int64_t* ids, int64_t capacity, int64_t* n) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && n && (ids || capacity == 0) && capacity >= 0, MB_ERR_INVALID_ARG,
               "NULL argument or negative capacity");
    const int64_t k = std::min<int64_t>(capacity, (int64_t)e->newly_done.size());
    std::copy(e->newly_done.begin(), e->newly_done.begin() + k, ids);
    e->newly_done.erase(e->newly_done.begin(), e->newly_done.begin() + k);
    *n = k;
  });
}

int mb_engine_stats(mb_engine_t eng, int64_t* steps, double* step_wall_ms, double* step_device_ms) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e, MB_ERR_INVALID_ARG, "NULL engine");
    if (steps) *steps = e->stat_steps;
    if (step_wall_ms) *step_wall_ms = e->stat_wall_ms;
    if (step_device_ms) *step_device_ms = e->stat_dev_ms;
  });
}

int mb_engine_set_fused_threshold(mb_engine_t eng, int64_t min_states) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && min_states >= 1, MB_ERR_INVALID_ARG, "NULL engine or threshold below 1");
    // mid-run changes keep each slot's progress: only the kernel that applies it changes
    e->fused_min = min_states;
    e->dirty = true;
    rebuild(e);
  });
}

int mb_engine_set_warps(mb_engine_t eng, int warps_per_block) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e, MB_ERR_INVALID_ARG, "NULL engine");
    MB_REQUIRE(warps_per_block == 2 || warps_per_block == 4 || warps_per_block == 8 ||
                   warps_per_block == 16,
               MB_ERR_INVALID_ARG, "warps per block must be 2, 4, 8 or 16");
    e->warps = warps_per_block;
  });
}

}  // extern "C"

extern "C" {

// n_steps engine steps without host round trips (no convergence checks in
// between), optionally as one captured CUDA graph replayed n_steps times;
// then one round of bookkeeping.  For fixed-length batches.
int mb_engine_step_fixed(mb_engine_t eng, int n_steps, int use_graph, int* n_active) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && n_steps >= 0, MB_ERR_INVALID_ARG, "bad argument");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    if (!e->slots.empty() && n_steps > 0) {
      rebuild(e);
      if (e->persistent) {
        // all n steps in one persistent launch, captured as a graph or not
        if (use_graph) {
          cudaGraph_t g = nullptr;
          cudaGraphExec_t ge = nullptr;
          MB_CUDA(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
          try {
            launch_persistent(e, n_steps);
          } catch (...) {
            cudaStreamEndCapture(e->st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
          }
          MB_CUDA(cudaStreamEndCapture(e->st, &g));
          MB_CUDA(cudaGraphInstantiate(&ge, g, 0));
          MB_CUDA(cudaGraphLaunch(ge, e->st));
          MB_CUDA(cudaStreamSynchronize(e->st));
          cudaGraphExecDestroy(ge);
          cudaGraphDestroy(g);
        } else {
          launch_persistent(e, n_steps);
        }
      } else if (use_graph) {
        cudaGraph_t g = nullptr;
        cudaGraphExec_t ge = nullptr;
        MB_CUDA(cudaStreamBeginCapture(e->st, cudaStreamCaptureModeThreadLocal));
        launch_step(e);
        MB_CUDA(cudaStreamEndCapture(e->st, &g));
        MB_CUDA(cudaGraphInstantiate(&ge, g, 0));
        for (int i = 0; i < n_steps; ++i) MB_CUDA(cudaGraphLaunch(ge, e->st));
        MB_CUDA(cudaStreamSynchronize(e->st));
        cudaGraphExecDestroy(ge);
        cudaGraphDestroy(g);
      } else {
        for (int i = 0; i < n_steps; ++i) launch_step(e);
      }
      after_step(e);
    }
    if (n_active) *n_active = (int)e->slots.size();
  });
}

// Autotuner: times the grouped apply kernel at 2, 4, 8 and 16 warps per
// block on the current set of requests and keeps the fastest.  The timed
// launches write only the w buffers, which the next real step overwrites.
int mb_engine_set_persistent(mb_engine_t eng, int on) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e, MB_ERR_INVALID_ARG, "NULL engine");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    e->persistent = on != 0;
    e->dirty = true;  // new work lists; every request keeps its progress
    rebuild(e);
  });
}

int mb_engine_set_basis_limit(mb_engine_t eng, int64_t bytes) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && bytes >= 0, MB_ERR_INVALID_ARG, "NULL engine or negative limit");
    e->basis_limit = bytes;
  });
}

int mb_engine_set_wait_budget(mb_engine_t eng, int64_t cycles) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && cycles >= 0, MB_ERR_INVALID_ARG, "NULL engine or negative budget");
    e->wait_budget = cycles;
  });
}

int mb_engine_get_shape(mb_engine_t eng, mb_engine_shape* shape) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && shape, MB_ERR_INVALID_ARG, "NULL argument");
    *shape = mb_engine_shape{};
    shape->persistent = e->persistent ? 1 : 0;
    shape->row_min_cols = e->p_row_min_cols;
    shape->ctas_per_sm = e->p_ctas_per_sm;
    shape->grid = e->p_grid;
    shape->warps = e->warps;
  });
}

int mb_engine_set_shape(mb_engine_t eng, const mb_engine_shape* shape) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e && shape, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    MB_REQUIRE(shape->row_min_cols >= 32 && shape->row_min_cols <= 1 << 20, MB_ERR_INVALID_ARG,
               "row_min_cols must be in [32, 2^20]");
    MB_REQUIRE(shape->ctas_per_sm >= 0 && shape->ctas_per_sm <= 32, MB_ERR_INVALID_ARG,
               "ctas_per_sm must be in [0, 32]");
    MB_REQUIRE(shape->warps == 2 || shape->warps == 4 || shape->warps == 8 || shape->warps == 16,
               MB_ERR_INVALID_ARG, "warps must be 2, 4, 8 or 16");
    e->persistent = shape->persistent != 0;
    e->p_row_min_cols = std::min(shape->row_min_cols, kEngWarpRowCols);
    e->p_ctas_per_sm = shape->ctas_per_sm;
    e->warps = shape->warps;
    e->dirty = true;
    rebuild(e);
  });
}

int mb_engine_autotune(mb_engine_t eng, int* chosen, double* ms) {
  return guard([&] {
    auto* e = (mb_engine_s*)eng;
    MB_REQUIRE(e, MB_ERR_INVALID_ARG, "NULL engine");
    MB_REQUIRE(!e->broken, MB_ERR_TIMEOUT, "the engine stopped after a barrier timeout");
    if (e->slots.empty()) {
      if (chosen) *chosen = e->warps;
      return;
    }
    if (e->persistent) {
      // the persistent step's shapes, timed on the live requests with
      // apply-only launches (they write only w and the partials, which the
      // next step rewrites): rows below row_min_cols columns warp per row,
      // ctas_per_sm co-resident blocks (0: all that fit).  A mix of requests
      // the engine has tuned for before takes that shape without timing.
      std::vector<std::tuple<int64_t, int64_t, int>> mix;
      mix.reserve(e->slots.size());
      for (const auto& sl : e->slots) mix.emplace_back(sl->Du, sl->Dd, sl->kind);
      std::sort(mix.begin(), mix.end());
      if (!e->tuned_mix.empty() && mix == e->tuned_mix) {
        e->p_row_min_cols = e->tuned_cols;
        e->p_ctas_per_sm = e->tuned_ctas;
        e->dirty = true;
        rebuild(e);
        if (chosen) *chosen = e->warps;
        if (ms) *ms = e->tuned_ms;
        return;
      }
      cudaEvent_t a, b;
      MB_CUDA(cudaEventCreate(&a));
      MB_CUDA(cudaEventCreate(&b));
      double best = 1e300;
      int best_cols = e->p_row_min_cols, best_ctas = e->p_ctas_per_sm;
      try {
        // one CTA per SM never won on the measured mixes and costs the most to
        // time; one warm-up and two timed launches a candidate
        for (int cols : {64, 128, 256}) {
          e->p_row_min_cols = cols;
          e->dirty = true;
          rebuild(e);  // new work lists; the block count below needs none
          for (int ctas : {0, 2}) {
            e->p_ctas_per_sm = ctas;
            e->p_grid = std::max(1, (ctas > 0 ? std::min(ctas, e->p_bps) : e->p_bps) * e->p_sms);
            launch_persistent(e, 1, true);
            MB_CUDA(cudaEventRecord(a, e->st));
            for (int rep = 0; rep < 2; ++rep) launch_persistent(e, 1, true);
            MB_CUDA(cudaEventRecord(b, e->st));
            MB_CUDA(cudaEventSynchronize(b));
            float t = 0.f;
            MB_CUDA(cudaEventElapsedTime(&t, a, b));
            if (t < best) {
              best = t;
              best_cols = cols;
              best_ctas = ctas;
            }
          }
        }
      } catch (...) {
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        throw;
      }
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      e->p_row_min_cols = best_cols;
      e->p_ctas_per_sm = best_ctas;
      e->dirty = true;
      rebuild(e);
      e->tuned_mix = std::move(mix);
      e->tuned_cols = best_cols;
      e->tuned_ctas = best_ctas;
      e->tuned_ms = best / 2.0;
      if (chosen) *chosen = e->warps;
      if (ms) *ms = best / 2.0;
      return;
    }
    rebuild(e);
    const SlotDesc* ds = (const SlotDesc*)e->d_slots->p;
    const int2* it = (const int2*)e->d_items_warp->p;
    double* part = (double*)e->d_part->p;
    double* part2 = part + e->n_items;
    const int n = e->n_warp;
    if (n == 0) {  // every request runs through the row-staged or fused kernels
      if (chosen) *chosen = e->warps;
      if (ms) *ms = 0.0;
      return;
    }
    cudaEvent_t a, b;
    MB_CUDA(cudaEventCreate(&a));
    MB_CUDA(cudaEventCreate(&b));
    int best = e->warps;
    float best_ms = 1e30f;
    const int cand[4] = {2, 4, 8, 16};
    for (int ci = 0; ci < 4; ++ci) {
      const int W = cand[ci];
      auto run = [&] {
        const int g = eng_grid(n, W);
        switch (W) {
          case 2: k_eng_apply<2><<<g, 64, 0, e->st>>>(ds, it, n, part, part2); break;
          case 4: k_eng_apply<4><<<g, 128, 0, e->st>>>(ds, it, n, part, part2); break;
          case 8: k_eng_apply<8><<<g, 256, 0, e->st>>>(ds, it, n, part, part2); break;
          default: k_eng_apply<16><<<g, 512, 0, e->st>>>(ds, it, n, part, part2); break;
        }
      };
      run();
      MB_CUDA(cudaEventRecord(a, e->st));
      for (int rep = 0; rep < 3; ++rep) run();
      MB_CUDA(cudaEventRecord(b, e->st));
      MB_CUDA(cudaEventSynchronize(b));
      float t = 0.f;
      MB_CUDA(cudaEventElapsedTime(&t, a, b));
      if (t < best_ms) {
        best_ms = t;
        best = W;
      }
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    MB_CUDA(cudaGetLastError());
    e->warps = best;
    if (chosen) *chosen = best;
    if (ms) *ms = best_ms / 3.0;
  });
}

}  // extern "C"
