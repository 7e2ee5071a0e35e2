// CUDA kernels of the matrix-free Hubbard operator and the Krylov drivers.
//
// Layout in HBM: a state vector is X[r_up * D_down + r_down] (tensor order),
// interleaved complex (double2 / float2), r_up / r_down the colex ranks of the
// up / down occupation masks.  H = H_up (x) 1 + 1 (x) H_down + diag, where the
// per-spin hopping matrices come from hop tables (CSR over ranks, see
// mb_internal.h) and diag = U * popcount(up & down) (+ self-bond energies).
#include <cuda_runtime.h>

#include "mb_internal.h"

namespace mb {

template <typename T> struct C2;
template <> struct C2<double> { using type = double2; };
template <> struct C2<float> { using type = float2; };

size_t elem_bytes(int precision) { return precision == MB_PREC_F32 ? 8 : 16; }

// ---------------------------------------------------------------------------
// Dot-product accumulators.  FP64 dots on this GPU's FP64 pipe for double
// vectors; for float vectors a compensated float pair (TwoSum on exact
// TwoProd terms, Knuth / Ogita-Rump-Oishi) so no FP64 instruction runs per
// element.
// ---------------------------------------------------------------------------
template <typename T> struct DotAcc;
template <> struct DotAcc<double> {
  double s = 0.0;
  __device__ void add_prod(double a, double b) { s = fma(a, b, s); }
  __device__ double value() const { return s; }
};
template <> struct DotAcc<float> {
  float hi = 0.f, lo = 0.f;
  __device__ void add_prod(float a, float b) {
    const float p = a * b;
    const float pe = fmaf(a, b, -p);
    const float s = hi + p;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (p - bp);
    hi = s;
    lo += e + pe;
  }
  __device__ double value() const { return (double)hi + (double)lo; }
};

// Block reduction of NC doubles; thread 0 writes partials[blockIdx.x*NC + k].
template <int NC>
__device__ void block_reduce_store(double (&v)[NC], double* partials) {
  __shared__ double red[32][NC > 0 ? NC : 1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NC; ++k) {
    double a = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    v[k] = a;
  }
  __syncthreads();
  if (lane == 0)
    for (int k = 0; k < NC; ++k) red[warp][k] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    for (int k = 0; k < NC; ++k) {
      double a = lane < nw ? red[lane][k] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0) partials[(size_t)blockIdx.x * NC + k] = a;
    }
  }
}

// Fixed-order final reduction: out[k] = sum_b partials[b*ncomp + k].  Warp w
// takes the components w, w + 32, ...; lane l sums the partials l, l + 32, ...
// in four chains (partial l + 128 i + 32 q into chain q, then the chains in
// order), and the lanes meet in a shuffle tree: no block barrier, and the
// chains keep four loads in flight a lane.
__global__ void __launch_bounds__(1024)
k_reduce(const double* __restrict__ partials, int nblocks, int ncomp, double* __restrict__ out) {
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int k = threadIdx.x >> 5; k < ncomp; k += nw) {
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    int b = lane;
    for (; b + 96 < nblocks; b += 128) {
      a0 += partials[(size_t)b * ncomp + k];
      a1 += partials[(size_t)(b + 32) * ncomp + k];
      a2 += partials[(size_t)(b + 64) * ncomp + k];
      a3 += partials[(size_t)(b + 96) * ncomp + k];
    }
    for (; b < nblocks; b += 32) a0 += partials[(size_t)b * ncomp + k];
    double a = (a0 + a1) + (a2 + a3);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) out[k] = a;
  }
}

void launch_reduce(const double* partials, int nblocks, int ncomp, double* out, cudaStream_t st) {
  const int warps = ncomp < 1 ? 1 : (ncomp > 32 ? 32 : ncomp);
  k_reduce<<<1, 32 * warps, 0, st>>>(partials, nblocks, ncomp, out);
  MB_CUDA(cudaGetLastError());
}

static int num_sms() {
  static int sms = -1;
  if (sms < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
  return sms;
}

static int max_smem_optin() {
  static int v = -1;
  if (v < 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  }
  return v;
}

// ---------------------------------------------------------------------------
// The matrix-free apply:  y = scale * (H - shift) x + beta * z
// with optional fused dot products (dot_mode bit0: Re<x,y>, bit1: <y,y>,
// bit2: <x,x>).  One CTA per SM (two for complex64) walks the rows r_up in
// the row schedule's order; it stages the row X[r_up, :] (and eight zero elements) in shared
// memory when it fits, so the down hops, which stay inside the row, gather
// from shared memory through the sliced table (one coalesced 16-byte load
// per lane for four slots: neighbour index | sign << 31, padding = one of the
// zero elements past the row), while the up hops read the neighbour rows X[r_up', c] from
// L2/HBM with coalesced 8/16-byte loads, the row's sign-sorted target list
// in shared memory (added, then subtracted).  Warp w takes the 32-column
// groups w, w + 32, ... (with up_prefetch set it asks L2 for the group's
// up-hop lines before its down hops).
// ---------------------------------------------------------------------------
constexpr int kApplyThreads = 1024;
// CTAs per SM: complex64 rows are half the size, and two CTAs per SM (32
// registers a thread) beat one with 64 registers (measured 2.03 -> 1.75 ms at
// 4x4 6+6, 3.41 -> 2.98 ms at 1D L=16 8+8); complex128 keeps one.
template <typename T> constexpr int kApplyCtasPerSm = sizeof(T) == 4 ? 2 : 1;

// +-1 from the sign bit of a table entry
__device__ __forceinline__ double unit_sign(uint32_t e, double) {
  return __hiloint2double((int)(0x3ff00000u | (e & 0x80000000u)), 0);
}
__device__ __forceinline__ float unit_sign(uint32_t e, float) {
  return __int_as_float((int)(0x3f800000u | (e & 0x80000000u)));
}

template <typename T, bool STAGED, int DOTS>
__device__ __forceinline__ void apply_rows(
    const OpView& v, const typename C2<T>::type* __restrict__ x, typename C2<T>::type* y,
    T hop_coef, T dscale, T shift, T beta, const typename C2<T>::type* z,
    const T* __restrict__ ufold, const T* __restrict__ self_up, const T* __restrict__ self_dn,
    double* __restrict__ partials) {
  using V2 = typename C2<T>::type;
  constexpr int kShift = sizeof(V2) == 16 ? 4 : 3;
  extern __shared__ __align__(16) unsigned char smem[];
  const int64_t Dd = v.Dd;
  const uint32_t row_bytes = (uint32_t)(sizeof(V2) * Dd);
  uint32_t* s_up =
      reinterpret_cast<uint32_t*>(smem + (STAGED ? row_bytes + sizeof(V2) * kSlicedPads : 0));
  if (STAGED && threadIdx.x < kSlicedPads) {
    V2 zero;
    zero.x = T(0);
    zero.y = T(0);
    reinterpret_cast<V2*>(smem + row_bytes)[threadIdx.x] = zero;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int64_t ngroups = (Dd + 31) >> 5;
  DotAcc<T> a_xy, a_yy, a_xx;

  for (int64_t ri = blockIdx.x; ri < v.Du; ri += gridDim.x) {
    const int64_t r = v.row_sched ? (int64_t)v.row_sched[ri] : ri;
    const V2* xrow = x + r * Dd;
    __syncthreads();
    const int u0 = __ldg(&v.up_loff[r]), nu = __ldg(&v.up_loff[r + 1]) - u0;
    const int npos = __ldg(&v.up_lpos[r]);
    for (int j = threadIdx.x; j < nu; j += blockDim.x) s_up[j] = __ldg(&v.up_list[u0 + j]);
    if (STAGED)
      for (int64_t c = threadIdx.x; c < Dd; c += blockDim.x)
        reinterpret_cast<V2*>(smem)[c] = xrow[c];
    __syncthreads();
    const uint32_t um = v.up_mask[r];
    const T su = self_up ? self_up[r] : T(0);
    for (int64_t g = warp; g < ngroups; g += nwarps) {
      const int64_t c = (g << 5) + lane;
      const bool live = c < Dd;
      const int64_t cl = live ? c : Dd - 1;
      if (v.up_prefetch) prefetch_up_group<(int)sizeof(V2)>(x, s_up, nu, g, lane, row_bytes);
      T ar = T(0), ai = T(0);
      const int2 gi = __ldg(reinterpret_cast<const int2*>(v.dn_sgrp) + g);
      auto hop = [&](uint32_t e) {
        const uint32_t off = e << kShift;  // the sign bit shifts out
        V2 val;
        if (STAGED) {
          val = *reinterpret_cast<const V2*>(smem + off);
        } else if (off < row_bytes) {
          val = __ldg(reinterpret_cast<const V2*>(reinterpret_cast<const char*>(xrow) + off));
        } else {
          val.x = T(0);
          val.y = T(0);
        }
        const T w = unit_sign(e, T(0));
        ar = fma(w, val.x, ar);
        ai = fma(w, val.y, ai);
      };
      // four slots per 16-byte load; the last word's unused slots are padding
      const uint4* ep = reinterpret_cast<const uint4*>(v.dn_sell + gi.x) + lane;
      for (int j = 0; j < gi.y; j += 4) {
        const uint4 e = __ldg(ep + 8 * j);
        hop(e.x);
        hop(e.y);
        hop(e.z);
        hop(e.w);
      }
      const char* xc = reinterpret_cast<const char*>(x + cl);
#pragma unroll 4
      for (int j = 0; j < npos; ++j) {
        const V2 val = __ldg(reinterpret_cast<const V2*>(xc + (uint64_t)s_up[j] * row_bytes));
        ar += val.x;
        ai += val.y;
      }
#pragma unroll 4
      for (int j = npos; j < nu; ++j) {
        const V2 val = __ldg(reinterpret_cast<const V2*>(xc + (uint64_t)s_up[j] * row_bytes));
        ar -= val.x;
        ai -= val.y;
      }
      if (!live) continue;
      const V2 xv = STAGED ? reinterpret_cast<const V2*>(smem)[c] : xrow[c];
      T dv = ufold[__popc(um & v.dn_mask[c])] + su;
      if (self_dn) dv += self_dn[c];
      const T ds = dscale * (dv - shift);
      V2 out;
      out.x = fma(hop_coef, ar, ds * xv.x);
      out.y = fma(hop_coef, ai, ds * xv.y);
      const int64_t idx = r * Dd + c;
      if (z) {
        const V2 zv = z[idx];
        out.x = fma(beta, zv.x, out.x);
        out.y = fma(beta, zv.y, out.y);
      }
      y[idx] = out;
      if (DOTS & 1) { a_xy.add_prod(xv.x, out.x); a_xy.add_prod(xv.y, out.y); }
      if (DOTS & 2) { a_yy.add_prod(out.x, out.x); a_yy.add_prod(out.y, out.y); }
      if (DOTS & 4) { a_xx.add_prod(xv.x, xv.x); a_xx.add_prod(xv.y, xv.y); }
    }
  }
  if (DOTS) {
    double vals[3] = {a_xy.value(), a_yy.value(), a_xx.value()};
    block_reduce_store<3>(vals, partials);
  }
}

template <typename T, bool STAGED, int DOTS>
__global__ void __launch_bounds__(kApplyThreads, kApplyCtasPerSm<T>)
k_apply(OpView v, const typename C2<T>::type* __restrict__ x, typename C2<T>::type* y,
        T hop_coef, T dscale, T shift, T beta, const typename C2<T>::type* z,
        const T* __restrict__ ufold, const T* __restrict__ self_up, const T* __restrict__ self_dn,
        double* __restrict__ partials) {
  apply_rows<T, STAGED, DOTS>(v, x, y, hop_coef, dscale, shift, beta, z, ufold, self_up, self_dn,
                              partials);
}

// One engine step of a large slot through the fused complex64 apply: the
// slot's mode and step counter are read on the device, so the launch can sit
// in a captured graph.  Lanczos / replay: w = scale H v - beta_{k-1} v_prev;
// Chebyshev: w = c (H - b) v - [k > 0] T_{k-1}, c = (k ? 2 : 1) / a.
// Block partials (Re<v,w>, <w,w>) go to a.scratch.
template <bool STAGED>
__global__ void __launch_bounds__(kApplyThreads, kApplyCtasPerSm<float>)
k_eng_fused(OpView v, EngFusedArgs a) {
  const int k = *a.k, mode = *a.mode;
  float sc, shift = 0.f, beta = 0.f;
  if ((mode == kEngLanczos && k < *a.kmax) || (mode == kEngReplay && k + 1 < *a.steps)) {
    sc = a.scale;
    if (k > 0) beta = -(float)a.beta[k - 1];
  } else if (mode == kEngCheb && k < *a.kmax) {
    sc = (k == 0 ? 1.f : 2.f) / *a.cheb_a;
    shift = *a.cheb_b;
    if (k > 0) beta = -1.f;
  } else {
    return;  // idle this step: k_eng_fused_place writes zero partials
  }
  apply_rows<float, STAGED, 3>(v, a.buf[(k + 1) % 3], a.buf[(k + 2) % 3], -a.t * sc, sc, shift,
                               beta, k > 0 ? a.buf[k % 3] : nullptr, a.ufold, a.self_up,
                               a.self_dn, a.scratch);
}

// The fused slot's block partials into the engine's per-item partial arrays
// (its items [item0, item0 + n_items)), zeros where there is no block.
__global__ void k_eng_fused_place(EngFusedArgs a, int nblocks) {
  const int k = *a.k, mode = *a.mode;
  const bool ran = (mode == kEngLanczos && k < *a.kmax) || (mode == kEngReplay && k + 1 < *a.steps) ||
                   (mode == kEngCheb && k < *a.kmax);
  for (int i = threadIdx.x; i < a.n_items; i += blockDim.x) {
    const bool b = ran && i < nblocks;
    a.part[a.item0 + i] = b ? a.scratch[3 * i] : 0.0;
    a.part2[a.item0 + i] = b ? a.scratch[3 * i + 1] : 0.0;
  }
}

static size_t apply_smem(const OpView& v, int precision, bool staged) {
  const int up_words = (v.max_up_list + 3) & ~3;
  size_t s = sizeof(uint32_t) * (size_t)up_words;
  if (staged) s += elem_bytes(precision) * (size_t)(v.Dd + kSlicedPads);
  return s;
}

static bool apply_staged(const OpView& v, int precision) {
  return apply_smem(v, precision, true) + 1024 <= (size_t)max_smem_optin();
}

static int csr_grid(const OpView& v, int precision);

int apply_grid(const OpView& v, int precision) {
  if (v.n_blocks) {
    int g = 0;
    for (int b = 0; b < v.n_blocks; ++b) g += apply_grid(v.sub[b], precision);
    return g;
  }
  if (v.csr_row) return csr_grid(v, precision);
  int64_t g = (int64_t)num_sms() * (precision == MB_PREC_F32 ? kApplyCtasPerSm<float> : 1);
  if (g > v.Du) g = v.Du;
  return (int)(g > 0 ? g : 1);
}

template <typename T, bool STAGED, int DOTS>
static void apply_t(const OpView& v, const void* x, void* y, double scale, double shift,
                    double beta, const void* z, double* partials, cudaStream_t st) {
  using V2 = typename C2<T>::type;
  const size_t smem = apply_smem(v, sizeof(T) == 8 ? MB_PREC_F64 : MB_PREC_F32, STAGED);
  auto kern = k_apply<T, STAGED, DOTS>;
  MB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const T* uf = sizeof(T) == 8 ? (const T*)v.u_fold : (const T*)v.u_fold_f;
  const T* su = sizeof(T) == 8 ? (const T*)v.self_up : (const T*)v.self_up_f;
  const T* sd = sizeof(T) == 8 ? (const T*)v.self_dn : (const T*)v.self_dn_f;
  const int grid = apply_grid(v, sizeof(T) == 4 ? MB_PREC_F32 : MB_PREC_F64);
  kern<<<grid, kApplyThreads, smem, st>>>(v, (const V2*)x, (V2*)y, (T)(-v.t * scale), (T)scale,
                                          (T)shift, (T)beta, (const V2*)z, uf, su, sd, partials);
  MB_CUDA(cudaGetLastError());
}

template <typename T, bool STAGED>
static void apply_dots(const OpView& v, const void* x, void* y, double scale, double shift,
                       double beta, const void* z, double* partials, int dot_mode,
                       cudaStream_t st) {
  switch (dot_mode) {
    case 0: apply_t<T, STAGED, 0>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 1: apply_t<T, STAGED, 1>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 2: apply_t<T, STAGED, 2>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 3: apply_t<T, STAGED, 3>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 5: apply_t<T, STAGED, 5>(v, x, y, scale, shift, beta, z, partials, st); break;
    default: apply_t<T, STAGED, 7>(v, x, y, scale, shift, beta, z, partials, st); break;
  }
}

// ---------------------------------------------------------------------------
// The same contract for an operator given as a sparse matrix (CSR): one warp
// per row (rows grid-strided over a fixed grid), lanes over the row's
// entries, complex products, a fixed-order shuffle sum, then the affine
// epilogue and the fused dots in lane 0.  Deterministic.  In the signed-
// column form (no values) every entry is +-off and the diagonal comes apart.
// ---------------------------------------------------------------------------
constexpr int kCsrThreads = 256;
// Lanes per CSR row: a row's partial sums meet in a log2(lanes)-step shuffle
// reduction, which on this GPU's slow FP64 pipe cost as much as the row's own
// adds at 32 lanes.  Measured at 4x4 6+6, K = (0,0) (~210 entries a row):
// complex128 10.85 / 6.72 / 5.11 / 4.47 ms at 32 / 16 / 8 / 4 lanes,
// complex64 2.95 / 2.32 / 2.02 / 2.07 ms.
template <typename T> constexpr int csr_lanes() { return sizeof(T) == 8 ? 4 : 8; }

// v with its sign flipped when bit 31 of e is set
__device__ __forceinline__ double flip_sign(double v, uint32_t e) {
  return __longlong_as_double(__double_as_longlong(v) ^ ((long long)(e >> 31) << 63));
}
__device__ __forceinline__ float flip_sign(float v, uint32_t e) {
  return __int_as_float(__float_as_int(v) ^ (int)(e & 0x80000000u));
}

template <typename T, int DOTS, int LPR>
__global__ void __launch_bounds__(kCsrThreads)
k_csr_apply(int64_t n, const int64_t* __restrict__ rp, const int32_t* __restrict__ ci,
            const typename C2<T>::type* __restrict__ val, const double* __restrict__ diag, T off,
            const typename C2<T>::type* __restrict__ x, typename C2<T>::type* y, T scale, T shift,
            T beta, const typename C2<T>::type* z, double* __restrict__ partials) {
  using V2 = typename C2<T>::type;
  // LPR lanes per row, 32 / LPR rows per warp; the warp steps through its rows
  // together (the shuffles need every lane), groups past the last row idle
  constexpr int RPW = 32 / LPR;
  const int lane = threadIdx.x & (LPR - 1);
  const int sub = (threadIdx.x & 31) / LPR;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  DotAcc<T> a_xy, a_yy, a_xx;
  for (int64_t rb = w0 * RPW; rb < n; rb += nw * RPW) {
    const int64_t row = rb + sub;
    const bool live = row < n;
    T ar = T(0), ai = T(0);
    if (!live) {
    } else if (val) {
      for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += LPR) {
        const V2 a = val[k], b = x[ci[k]];
        ar = fma(a.x, b.x, fma(-a.y, b.y, ar));
        ai = fma(a.x, b.y, fma(a.y, b.x, ai));
      }
    } else {  // signed columns: entries +-1 (times off below), diagonal apart
      // the sign goes onto the sign bit, so no lane branches per entry; for
      // complex64 two independent sums (even / odd strides) halve the add
      // chains (measured at 4x4 6+6, K=0, 32 lanes a row: 3.19 -> 2.81 ms),
      // for complex128 one (9.1 ms, against 12.9 ms with two)
      T br = T(0), bi = T(0);
      const int64_t k1 = rp[row + 1];
      int64_t k = rp[row] + lane;
#pragma unroll 4
      for (; sizeof(T) == 4 && k + LPR < k1; k += 2 * LPR) {
        const uint32_t e0 = (uint32_t)__ldg(&ci[k]), e1 = (uint32_t)__ldg(&ci[k + LPR]);
        const V2 b0 = __ldg(&x[e0 & 0x7FFFFFFFu]), b1 = __ldg(&x[e1 & 0x7FFFFFFFu]);
        ar += flip_sign(b0.x, e0);
        ai += flip_sign(b0.y, e0);
        br += flip_sign(b1.x, e1);
        bi += flip_sign(b1.y, e1);
      }
#pragma unroll 4
      for (; k < k1; k += LPR) {
        const uint32_t e0 = (uint32_t)__ldg(&ci[k]);
        const V2 b0 = __ldg(&x[e0 & 0x7FFFFFFFu]);
        ar += flip_sign(b0.x, e0);
        ai += flip_sign(b0.y, e0);
      }
      ar += br;
      ai += bi;
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o);
      ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (live && lane == 0) {
      const V2 xv = x[row];
      if (!val) {
        const T d = (T)diag[row];
        ar = fma(off, ar, d * xv.x);
        ai = fma(off, ai, d * xv.y);
      }
      V2 out;
      out.x = scale * (ar - shift * xv.x);
      out.y = scale * (ai - shift * xv.y);
      if (z) {
        const V2 zv = z[row];
        out.x = fma(beta, zv.x, out.x);
        out.y = fma(beta, zv.y, out.y);
      }
      y[row] = out;
      if (DOTS & 1) { a_xy.add_prod(xv.x, out.x); a_xy.add_prod(xv.y, out.y); }
      if (DOTS & 2) { a_yy.add_prod(out.x, out.x); a_yy.add_prod(out.y, out.y); }
      if (DOTS & 4) { a_xx.add_prod(xv.x, xv.x); a_xx.add_prod(xv.y, xv.y); }
    }
  }
  if (DOTS) {
    double vals[3] = {a_xy.value(), a_yy.value(), a_xx.value()};
    block_reduce_store<3>(vals, partials);
  }
}

// the lanes a row of this operator's CSR apply takes
static int csr_lanes_of(const OpView& v, int precision) {
  if (v.csr_lanes) return v.csr_lanes;
  return precision == MB_PREC_F32 ? csr_lanes<float>() : csr_lanes<double>();
}

static int csr_grid(const OpView& v, int precision) {
  const int64_t n = v.dim;
  const int64_t rows_per_block = kCsrThreads / csr_lanes_of(v, precision);
  int64_t g = (n + rows_per_block - 1) / rows_per_block;
  const int64_t cap = (int64_t)num_sms() * 16;
  if (g > cap) g = cap;
  return (int)(g > 0 ? g : 1);
}

template <typename T, int DOTS, int LPR>
static void csr_apply_l(const OpView& v, const void* x, void* y, double scale, double shift,
                        double beta, const void* z, double* partials, cudaStream_t st) {
  using V2 = typename C2<T>::type;
  const V2* val = sizeof(T) == 8 ? (const V2*)v.csr_val : (const V2*)v.csr_val_f;
  k_csr_apply<T, DOTS, LPR><<<csr_grid(v, sizeof(T) == 4 ? MB_PREC_F32 : MB_PREC_F64),
                              kCsrThreads, 0, st>>>(
      v.dim, v.csr_row, v.csr_col, val, v.csr_diag, (T)v.csr_off, (const V2*)x, (V2*)y,
      (T)scale, (T)shift, (T)beta, (const V2*)z, partials);
  MB_CUDA(cudaGetLastError());
}

template <typename T, int DOTS>
static void csr_apply_t(const OpView& v, const void* x, void* y, double scale, double shift,
                        double beta, const void* z, double* partials, cudaStream_t st) {
  switch (csr_lanes_of(v, sizeof(T) == 4 ? MB_PREC_F32 : MB_PREC_F64)) {
    case 4: csr_apply_l<T, DOTS, 4>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 8: csr_apply_l<T, DOTS, 8>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 16: csr_apply_l<T, DOTS, 16>(v, x, y, scale, shift, beta, z, partials, st); break;
    default: csr_apply_l<T, DOTS, 32>(v, x, y, scale, shift, beta, z, partials, st); break;
  }
}

template <typename T>
static void csr_apply_dots(const OpView& v, const void* x, void* y, double scale, double shift,
                           double beta, const void* z, double* partials, int dot_mode,
                           cudaStream_t st) {
  switch (dot_mode) {
    case 0: csr_apply_t<T, 0>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 1: csr_apply_t<T, 1>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 2: csr_apply_t<T, 2>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 3: csr_apply_t<T, 3>(v, x, y, scale, shift, beta, z, partials, st); break;
    case 5: csr_apply_t<T, 5>(v, x, y, scale, shift, beta, z, partials, st); break;
    default: csr_apply_t<T, 7>(v, x, y, scale, shift, beta, z, partials, st); break;
  }
}

void launch_apply(const OpView& v, int precision, const void* x, void* y, double scale,
                  double shift, double beta, const void* z, double* partials, int dot_mode,
                  cudaStream_t st) {
  if (v.n_blocks) {  // block-diagonal: each block on its slice, partials one after another
    const size_t es = elem_bytes(precision);
    int64_t first = 0;
    for (int b = 0; b < v.n_blocks; ++b) {
      const size_t off = es * (size_t)v.sub_off[b];
      launch_apply(v.sub[b], precision, (const char*)x + off, (char*)y + off, scale, shift, beta,
                   z ? (const char*)z + off : nullptr, partials ? partials + 3 * first : nullptr,
                   dot_mode, st);
      first += apply_grid(v.sub[b], precision);
    }
    return;
  }
  if (v.csr_row) {
    if (precision == MB_PREC_F32) csr_apply_dots<float>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
    else csr_apply_dots<double>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
    return;
  }
  const bool staged = apply_staged(v, precision);
  if (precision == MB_PREC_F32) {
    if (staged) apply_dots<float, true>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
    else apply_dots<float, false>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
  } else {
    if (staged) apply_dots<double, true>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
    else apply_dots<double, false>(v, x, y, scale, shift, beta, z, partials, dot_mode, st);
  }
}

int eng_fused_blocks(const OpView& v) { return apply_grid(v, MB_PREC_F32); }

void prepare_eng_fused() {
  // the launch limit on dynamic shared memory, set outside any stream capture
  static bool done = false;
  if (done) return;
  // the opt-in maximum less each kernel's static shared memory
  auto allow = [](const void* f) {
    cudaFuncAttributes fa{};
    MB_CUDA(cudaFuncGetAttributes(&fa, f));
    MB_CUDA(cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 max_smem_optin() - (int)fa.sharedSizeBytes));
  };
  allow((const void*)k_eng_fused<true>);
  allow((const void*)k_eng_fused<false>);
  done = true;
}

void launch_eng_fused(const OpView& v, const EngFusedArgs& a, cudaStream_t st) {
  const bool staged = apply_staged(v, MB_PREC_F32);
  const size_t smem = apply_smem(v, MB_PREC_F32, staged);
  const int grid = apply_grid(v, MB_PREC_F32);
  if (staged) k_eng_fused<true><<<grid, kApplyThreads, smem, st>>>(v, a);
  else k_eng_fused<false><<<grid, kApplyThreads, smem, st>>>(v, a);
  k_eng_fused_place<<<1, 256, 0, st>>>(a, grid);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Vector kernels (grid-stride, one complex element per step).
// ---------------------------------------------------------------------------
constexpr int kBlasThreads = 256;

int blas_grid(int64_t n) {
  int64_t g = (n + kBlasThreads - 1) / kBlasThreads;
  const int64_t cap = (int64_t)num_sms() * 8;
  if (g > cap) g = cap;
  return (int)(g > 0 ? g : 1);
}

// y = a*x + b*y, complex a, b; dot_mode bit1: <y,y> of the result.
template <typename T, int DOTS>
__global__ void k_axpby(int64_t n, T ar, T ai, const typename C2<T>::type* __restrict__ x, T br,
                        T bi, typename C2<T>::type* __restrict__ y, double* __restrict__ partials) {
  using V2 = typename C2<T>::type;
  DotAcc<T> acc;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const V2 xv = x ? x[i] : V2{T(0), T(0)};
    const V2 yv = (br != T(0) || bi != T(0)) ? y[i] : V2{T(0), T(0)};
    V2 o;
    o.x = ar * xv.x - ai * xv.y + br * yv.x - bi * yv.y;
    o.y = ar * xv.y + ai * xv.x + br * yv.y + bi * yv.x;
    y[i] = o;
    if (DOTS & 2) { acc.add_prod(o.x, o.x); acc.add_prod(o.y, o.y); }
  }
  if (DOTS) {
    double vals[3] = {0.0, acc.value(), 0.0};
    block_reduce_store<3>(vals, partials);
  }
}

void launch_axpby(int precision, int64_t n, double ar, double ai, const void* x, double br,
                  double bi, void* y, double* partials, int dot_mode, cudaStream_t st) {
  const int g = blas_grid(n);
  if (precision == MB_PREC_F32) {
    if (dot_mode) k_axpby<float, 2><<<g, kBlasThreads, 0, st>>>(n, (float)ar, (float)ai, (const float2*)x, (float)br, (float)bi, (float2*)y, partials);
    else k_axpby<float, 0><<<g, kBlasThreads, 0, st>>>(n, (float)ar, (float)ai, (const float2*)x, (float)br, (float)bi, (float2*)y, partials);
  } else {
    if (dot_mode) k_axpby<double, 2><<<g, kBlasThreads, 0, st>>>(n, ar, ai, (const double2*)x, br, bi, (double2*)y, partials);
    else k_axpby<double, 0><<<g, kBlasThreads, 0, st>>>(n, ar, ai, (const double2*)x, br, bi, (double2*)y, partials);
  }
  MB_CUDA(cudaGetLastError());
}

// Re<x,y>, Im<x,y>, <y,y> with <x,y> = sum conj(x_i) y_i (arma::cdot).
template <typename T>
__global__ void k_dot(int64_t n, const typename C2<T>::type* __restrict__ x,
                      const typename C2<T>::type* __restrict__ y, double* __restrict__ partials) {
  using V2 = typename C2<T>::type;
  DotAcc<T> re, im, yy;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const V2 a = x[i], b = y[i];
    re.add_prod(a.x, b.x);
    re.add_prod(a.y, b.y);
    im.add_prod(a.x, b.y);
    im.add_prod(-a.y, b.x);
    yy.add_prod(b.x, b.x);
    yy.add_prod(b.y, b.y);
  }
  double vals[3] = {re.value(), im.value(), yy.value()};
  block_reduce_store<3>(vals, partials);
}

void launch_dot(int precision, int64_t n, const void* x, const void* y, double* partials,
                cudaStream_t st) {
  const int g = blas_grid(n);
  if (precision == MB_PREC_F32)
    k_dot<float><<<g, kBlasThreads, 0, st>>>(n, (const float2*)x, (const float2*)y, partials);
  else
    k_dot<double><<<g, kBlasThreads, 0, st>>>(n, (const double2*)x, (const double2*)y, partials);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Re-orthogonalisation against a stored basis V (columns V_j, leading
// dimension ld elements), V in FP64 or FP32, w in FP64 or FP32.
// multi_dot: c_j = <V_j, w>; each block keeps per-j sums in shared memory
// over the chunks it owns and writes one partial per j.
// ---------------------------------------------------------------------------
constexpr int kMdChunk = 1024;
constexpr int kMdThreads = 256;
constexpr int kMdBatch = 8;  // loads in flight per lane in the multi-vector kernels
constexpr int kMaxBasis = 1024;

template <typename TV, typename TW>
__global__ void __launch_bounds__(kMdThreads)
k_multi_dot(int64_t n, const typename C2<TV>::type* __restrict__ V, int64_t ld, int m,
            const typename C2<TW>::type* __restrict__ w, double* __restrict__ partials) {
  using VV = typename C2<TV>::type;
  using VW = typename C2<TW>::type;
  __shared__ double acc[2 * kMaxBasis];
  __shared__ double2 sw[kMdChunk];
  // a complex64 basis: w split into float hi + lo parts (lo = 0 for a
  // complex64 w), products on the FP32 pipe (exact products, compensated
  // sums), FP64 per chunk; the FP64 pipe runs at 1/57 of the FP32 rate here
  constexpr bool kSplit = sizeof(TV) == 4;
  __shared__ float4 swf[kSplit ? kMdChunk : 1];
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) acc[j] = 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int64_t base = (int64_t)blockIdx.x * kMdChunk; base < n; base += (int64_t)gridDim.x * kMdChunk) {
    const int len = (int)((n - base) < kMdChunk ? (n - base) : kMdChunk);
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      const VW a = w[base + i];
      if constexpr (kSplit) {
        const float hx = (float)a.x, hy = (float)a.y;
        swf[i] = make_float4(hx, hy, (float)((double)a.x - (double)hx),
                             (float)((double)a.y - (double)hy));
      } else {
        sw[i] = make_double2((double)a.x, (double)a.y);
      }
    }
    __syncthreads();
    for (int j = warp; j < m; j += nwarps) {
      const VV* vj = V + (int64_t)j * ld + base;
      double cr = 0.0, ci = 0.0;
      // the basis elements of kMdBatch iterations are loaded before any is
      // used, so a warp has that many HBM loads in flight instead of one
      if constexpr (kSplit) {
        DotAcc<float> pr, pi;
        float lr = 0.f, li = 0.f;
        for (int i0 = lane; i0 < len; i0 += 32 * kMdBatch) {
          VV a[kMdBatch];
#pragma unroll
          for (int u = 0; u < kMdBatch; ++u)
            if (i0 + 32 * u < len) a[u] = vj[i0 + 32 * u];
#pragma unroll
          for (int u = 0; u < kMdBatch; ++u) {
            if (i0 + 32 * u >= len) break;
            const float4 b = swf[i0 + 32 * u];
            pr.add_prod(a[u].x, b.x);
            pr.add_prod(a[u].y, b.y);
            pi.add_prod(a[u].x, b.y);
            pi.add_prod(-a[u].y, b.x);
            lr = fmaf(a[u].x, b.z, fmaf(a[u].y, b.w, lr));
            li = fmaf(a[u].x, b.w, fmaf(-a[u].y, b.z, li));
          }
        }
        cr = pr.value() + (double)lr;
        ci = pi.value() + (double)li;
      } else {
        for (int i0 = lane; i0 < len; i0 += 32 * kMdBatch) {
          VV a[kMdBatch];
#pragma unroll
          for (int u = 0; u < kMdBatch; ++u)
            if (i0 + 32 * u < len) a[u] = vj[i0 + 32 * u];
#pragma unroll
          for (int u = 0; u < kMdBatch; ++u) {
            if (i0 + 32 * u >= len) break;
            const double ar = (double)a[u].x, ai = (double)a[u].y;
            const double2 b = sw[i0 + 32 * u];
            cr = fma(ar, b.x, cr);
            cr = fma(ai, b.y, cr);
            ci = fma(ar, b.y, ci);
            ci = fma(-ai, b.x, ci);
          }
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        cr += __shfl_down_sync(0xffffffffu, cr, o);
        ci += __shfl_down_sync(0xffffffffu, ci, o);
      }
      if (lane == 0) { acc[2 * j] += cr; acc[2 * j + 1] += ci; }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x)
    partials[(size_t)blockIdx.x * 2 * m + j] = acc[j];
}

static int md_grid(int64_t n) {
  int64_t g = (n + kMdChunk - 1) / kMdChunk;
  // four CTAs per SM fit (64 registers x 256 threads, 32 KB of shared memory
  // each): twice the loads in flight of two
  const int64_t cap = (int64_t)num_sms() * 4;
  if (g > cap) g = cap;
  return (int)(g > 0 ? g : 1);
}

int multi_dot_grid(int64_t n) { return md_grid(n); }

void launch_multi_dot(int vprec, int wprec, int64_t n, const void* V, int64_t ld, int m,
                      const void* w, double* partials, cudaStream_t st) {
  MB_REQUIRE(m <= kMaxBasis, MB_ERR_CAPACITY, "re-orthogonalisation basis larger than 1024");
  const int g = md_grid(n);
  if (vprec == MB_PREC_F32 && wprec == MB_PREC_F32)
    k_multi_dot<float, float><<<g, kMdThreads, 0, st>>>(n, (const float2*)V, ld, m, (const float2*)w, partials);
  else if (vprec == MB_PREC_F32)
    k_multi_dot<float, double><<<g, kMdThreads, 0, st>>>(n, (const float2*)V, ld, m, (const double2*)w, partials);
  else if (wprec == MB_PREC_F32)
    k_multi_dot<double, float><<<g, kMdThreads, 0, st>>>(n, (const double2*)V, ld, m, (const float2*)w, partials);
  else
    k_multi_dot<double, double><<<g, kMdThreads, 0, st>>>(n, (const double2*)V, ld, m, (const double2*)w, partials);
  MB_CUDA(cudaGetLastError());
}

// w -= sum_j c_j V_j (c complex, on device), then <w,w> partials.
template <typename TV, typename TW>
__global__ void __launch_bounds__(kBlasThreads)
k_multi_axpy(int64_t n, const typename C2<TV>::type* __restrict__ V, int64_t ld, int m,
             const double* __restrict__ c, typename C2<TW>::type* __restrict__ w,
             double* __restrict__ partials) {
  using VV = typename C2<TV>::type;
  using VW = typename C2<TW>::type;
  __shared__ double sc[2 * kMaxBasis];
  for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) sc[j] = c[j];
  __syncthreads();
  // a complex64 basis: the correction sum_j c_j V_j on the FP32 pipe (it is
  // small next to w: the projections measure lost orthogonality), subtracted
  // in FP64
  constexpr bool kSplit = sizeof(TV) == 4;
  __shared__ float scf[kSplit ? 2 * kMaxBasis : 1];
  if constexpr (kSplit)
    for (int j = threadIdx.x; j < 2 * m; j += blockDim.x) scf[j] = (float)c[j];
  __syncthreads();
  DotAcc<double> ww;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const VW wv = w[i];
    double sr = (double)wv.x, si = (double)wv.y;
    // kMdBatch basis vectors' elements are loaded before any is used (HBM
    // loads in flight); the sums run in the same order as one at a time
    if constexpr (kSplit) {
      float fr = 0.f, fi = 0.f;
      for (int j0 = 0; j0 < m; j0 += kMdBatch) {
        VV a[kMdBatch];
#pragma unroll
        for (int u = 0; u < kMdBatch; ++u)
          if (j0 + u < m) a[u] = V[(int64_t)(j0 + u) * ld + i];
#pragma unroll
        for (int u = 0; u < kMdBatch; ++u) {
          if (j0 + u >= m) break;
          const float cr = scf[2 * (j0 + u)], ci = scf[2 * (j0 + u) + 1];
          fr = fmaf(cr, a[u].x, fmaf(-ci, a[u].y, fr));
          fi = fmaf(cr, a[u].y, fmaf(ci, a[u].x, fi));
        }
      }
      sr -= (double)fr;
      si -= (double)fi;
    } else {
      for (int j0 = 0; j0 < m; j0 += kMdBatch) {
        VV a[kMdBatch];
#pragma unroll
        for (int u = 0; u < kMdBatch; ++u)
          if (j0 + u < m) a[u] = V[(int64_t)(j0 + u) * ld + i];
#pragma unroll
        for (int u = 0; u < kMdBatch; ++u) {
          if (j0 + u >= m) break;
          const double cr = sc[2 * (j0 + u)], ci = sc[2 * (j0 + u) + 1];
          sr -= cr * (double)a[u].x - ci * (double)a[u].y;
          si -= cr * (double)a[u].y + ci * (double)a[u].x;
        }
      }
    }
    VW o;
    o.x = (decltype(o.x))sr;
    o.y = (decltype(o.y))si;
    w[i] = o;
    ww.add_prod((double)o.x, (double)o.x);
    ww.add_prod((double)o.y, (double)o.y);
  }
  double vals[3] = {0.0, ww.value(), 0.0};
  block_reduce_store<3>(vals, partials);
}

void launch_multi_axpy(int vprec, int wprec, int64_t n, const void* V, int64_t ld, int m,
                       const double* c, void* w, double* partials, cudaStream_t st) {
  MB_REQUIRE(m <= kMaxBasis, MB_ERR_CAPACITY, "re-orthogonalisation basis larger than 1024");
  const int g = blas_grid(n);
  if (vprec == MB_PREC_F32 && wprec == MB_PREC_F32)
    k_multi_axpy<float, float><<<g, kBlasThreads, 0, st>>>(n, (const float2*)V, ld, m, c, (float2*)w, partials);
  else if (vprec == MB_PREC_F32)
    k_multi_axpy<float, double><<<g, kBlasThreads, 0, st>>>(n, (const float2*)V, ld, m, c, (double2*)w, partials);
  else if (wprec == MB_PREC_F32)
    k_multi_axpy<double, float><<<g, kBlasThreads, 0, st>>>(n, (const double2*)V, ld, m, c, (float2*)w, partials);
  else
    k_multi_axpy<double, double><<<g, kBlasThreads, 0, st>>>(n, (const double2*)V, ld, m, c, (double2*)w, partials);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Precision conversion and permutations.
// ---------------------------------------------------------------------------
template <typename TA, typename TB>
__global__ void k_convert(int64_t n, const typename C2<TA>::type* __restrict__ a,
                          typename C2<TB>::type* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const auto v = a[i];
    typename C2<TB>::type o;
    o.x = (TB)v.x;
    o.y = (TB)v.y;
    b[i] = o;
  }
}

void launch_convert(int from_prec, int to_prec, int64_t n, const void* x, void* y,
                    cudaStream_t st) {
  const int g = blas_grid(n);
  const bool f32a = from_prec == MB_PREC_F32, f32b = to_prec == MB_PREC_F32;
  if (f32a == f32b) {
    MB_CUDA(cudaMemcpyAsync(y, x, elem_bytes(from_prec) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    return;
  }
  if (f32a) k_convert<float, double><<<g, kBlasThreads, 0, st>>>(n, (const float2*)x, (double2*)y);
  else k_convert<double, float><<<g, kBlasThreads, 0, st>>>(n, (const double2*)x, (float2*)y);
  MB_CUDA(cudaGetLastError());
}

template <typename V2, bool SCATTER>
__global__ void k_permute(int64_t n, const int32_t* __restrict__ perm, const V2* __restrict__ src,
                          V2* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = perm[i];
    if (SCATTER) dst[p] = src[i];
    else dst[i] = src[p];
  }
}

void launch_gather(int precision, int64_t n, const int32_t* perm, const void* src, void* dst,
                   cudaStream_t st) {
  const int g = blas_grid(n);
  if (precision == MB_PREC_F32) k_permute<float2, false><<<g, kBlasThreads, 0, st>>>(n, perm, (const float2*)src, (float2*)dst);
  else k_permute<double2, false><<<g, kBlasThreads, 0, st>>>(n, perm, (const double2*)src, (double2*)dst);
  MB_CUDA(cudaGetLastError());
}

void launch_scatter(int precision, int64_t n, const int32_t* perm, const void* src, void* dst,
                    cudaStream_t st) {
  const int g = blas_grid(n);
  if (precision == MB_PREC_F32) k_permute<float2, true><<<g, kBlasThreads, 0, st>>>(n, perm, (const float2*)src, (float2*)dst);
  else k_permute<double2, true><<<g, kBlasThreads, 0, st>>>(n, perm, (const double2*)src, (double2*)dst);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror & Shaw, SC'11).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox10(uint32_t c[4], uint32_t k0, uint32_t k1) {
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

// 52 random bits placed in [2,4), minus 3: uniform on [-1, 1), exact.
__device__ __forceinline__ double u52_pm1(uint32_t hi, uint32_t lo) {
  const uint64_t m = ((((uint64_t)hi) << 32) | lo) >> 12;
  return __longlong_as_double((long long)(0x4000000000000000ull | m)) - 3.0;
}

template <typename V2>
__global__ void k_fill_rng(int64_t n, uint64_t seed, uint32_t stream_id, int phase,
                           V2* __restrict__ dst) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), stream_id, 0u};
    philox10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    double re, im;
    if (phase) {
      const double u = (u52_pm1(c[0], c[1]) + 1.0) * 0.5;
      sincospi(2.0 * u, &im, &re);
    } else {
      re = u52_pm1(c[0], c[1]);
      im = u52_pm1(c[2], c[3]);
    }
    V2 o;
    o.x = (decltype(o.x))re;
    o.y = (decltype(o.y))im;
    dst[i] = o;
  }
}

void launch_fill_rng(int precision, int64_t Du, int64_t Dd, uint64_t seed, uint32_t stream_id,
                     int phase, void* dst, cudaStream_t st) {
  const int64_t n = Du * Dd;
  const int g = blas_grid(n);
  if (precision == MB_PREC_F32) k_fill_rng<float2><<<g, kBlasThreads, 0, st>>>(n, seed, stream_id, phase, (float2*)dst);
  else k_fill_rng<double2><<<g, kBlasThreads, 0, st>>>(n, seed, stream_id, phase, (double2*)dst);
  MB_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// Tensor index -> reference index, and the reference-order CSR export.
// ---------------------------------------------------------------------------
__constant__ Binom c_binom;

void upload_binomials(cudaStream_t st) {
  MB_CUDA(cudaMemcpyToSymbolAsync(c_binom, &binom_table(), sizeof(Binom), 0,
                                  cudaMemcpyHostToDevice, st));
}

__global__ void k_perm(OpView v, int32_t* __restrict__ perm) {
  __shared__ Binom sb;
  for (int i = threadIdx.x; i < (int)(sizeof(Binom) / sizeof(int64_t)); i += blockDim.x)
    (&sb.c[0][0])[i] = (&c_binom.c[0][0])[i];
  __syncthreads();
  const int64_t n = v.dim;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ru = i / v.Dd, rd = i - ru * v.Dd;
    perm[i] = (int32_t)reference_rank(sb, v.up_mask[ru], v.dn_mask[rd], v.L);
  }
}

__global__ void k_invert_perm(int64_t n, const int32_t* __restrict__ perm, int32_t* __restrict__ iperm) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    iperm[perm[i]] = (int32_t)i;
}

void launch_invert_perm(int64_t n, const int32_t* perm, int32_t* iperm, cudaStream_t st) {
  k_invert_perm<<<blas_grid(n), kBlasThreads, 0, st>>>(n, perm, iperm);
  MB_CUDA(cudaGetLastError());
}

void launch_perm(const OpView& v, int32_t* perm, cudaStream_t st) {
  k_perm<<<blas_grid(v.dim), kBlasThreads, 0, st>>>(v, perm);
  MB_CUDA(cudaGetLastError());
}

// first[r] = the smallest reference index among the states of tensor row r
// (min of perm over the row's Dd columns); one block per row.
__global__ void k_row_first(int64_t Du, int64_t Dd, const int32_t* __restrict__ perm,
                            int32_t* __restrict__ first) {
  __shared__ int32_t s_min[kBlasThreads / 32];
  for (int64_t r = blockIdx.x; r < Du; r += gridDim.x) {
    int32_t m = INT32_MAX;
    for (int64_t c = threadIdx.x; c < Dd; c += blockDim.x) m = min(m, perm[r * Dd + c]);
    for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = threadIdx.x < blockDim.x / 32 ? s_min[threadIdx.x] : INT32_MAX;
      for (int o = 16; o > 0; o >>= 1) m = min(m, __shfl_xor_sync(0xffffffffu, m, o));
      if (threadIdx.x == 0) first[r] = m;
    }
    __syncthreads();
  }
}

void launch_row_first(int64_t Du, int64_t Dd, const int32_t* perm, int32_t* first,
                      cudaStream_t st) {
  const int grid = (int)std::min<int64_t>(std::max<int64_t>(Du, 1), 65535);
  k_row_first<<<grid, kBlasThreads, 0, st>>>(Du, Dd, perm, first);
  MB_CUDA(cudaGetLastError());
}

constexpr int kMaxRowNnz = 256;

__device__ __forceinline__ double diag_value(const OpView& v, int64_t ru, int64_t rd) {
  double d = v.u_fold[__popc(v.up_mask[ru] & v.dn_mask[rd])];
  if (v.self_up) d += v.self_up[ru];
  if (v.self_dn) d += v.self_dn[rd];
  return d;
}

// Row of the reference-order CSR for tensor state i: hops from both spin
// tables (value -t * weight), plus the diagonal unless |d| < 1000*eps (the
// reference drops such coefficients, expression_base.h:79-97).
// ---------------------------------------------------------------------------
// Momentum-sector Hamiltonian (HubbardModelMomentum on one total momentum,
// src/algebra/fermion/model/hubbard_model_momentum.h:19-180):
//   H = sum_{k,s} eps(k) n_{k,s} + (U/N) sum_q rho_{q,up} rho_{-q,down},
//   rho_{q,s} = sum_k c+_{k+q,s} c_{k,s}
// (the reference's term c+_{k1+q,up} c+_{k2-q,dn} c_{k2,dn} c_{k1,up} equals
// (c+_{k1+q,up} c_{k1,up})(c+_{k2-q,dn} c_{k2,dn}) with sign +1).  Per row:
// diagonal = sum of eps over the occupied orbitals + (U/N) N_up N_down
// (the q = 0 terms), dropped below 1000 eps as the reference's expression
// does; off-diagonal = (U/N) * hop sign (up) * hop sign (down) for every
// q != 0, up electron k1 -> k1+q and down electron k2 -> k2-q into empty
// orbitals.  A column is the row of (up', down') in the sector: its
// full-sector reference rank, then a binary search in the sector's ranks.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int64_t mom_find(const MomTables& m, const Binom& b, uint32_t up,
                                            uint32_t dn) {
  const int64_t r = reference_rank(b, up, dn, m.L);
  int64_t lo = 0, hi = m.n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (m.full[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  return (lo < m.n && m.full[lo] == r) ? lo : -1;
}

__device__ __forceinline__ uint32_t between_bits(int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  return ((1u << hi) - 1u) & ~((2u << lo) - 1u);
}

template <bool FILL>
__global__ void k_mom_rows(MomTables m, int32_t* __restrict__ cnt, double* __restrict__ diag,
                           const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col) {
  __shared__ Binom sb;
  for (int i = threadIdx.x; i < (int)(sizeof(Binom) / sizeof(int64_t)); i += blockDim.x)
    (&sb.c[0][0])[i] = (&c_binom.c[0][0])[i];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m.n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t up = m.up[i], dn = m.dn[i];
    if (!FILL) {
      double d = 0.0;
      for (uint32_t b = up; b; b &= b - 1) d += m.eps[__ffs(b) - 1];
      for (uint32_t b = dn; b; b &= b - 1) d += m.eps[__ffs(b) - 1];
      if (m.u_over_n != 0.0) d += m.u_over_n * (double)(m.n_up * m.n_down);
      diag[i] = (d * d < kTol * kTol) ? 0.0 : d;
    }
    int c = 0;
    int64_t out = FILL ? row_ptr[i] : 0;
    if (m.u_over_n != 0.0) {
      for (int q = 1; q < m.L; ++q) {
        for (uint32_t bu = up; bu; bu &= bu - 1) {
          const int k1 = __ffs(bu) - 1, a = m.kadd[k1 * m.L + q];
          if ((up >> a) & 1u) continue;
          const uint32_t up2 = up ^ (1u << k1) ^ (1u << a);
          const uint32_t su = __popc(up & between_bits(k1, a)) & 1u;
          for (uint32_t bd = dn; bd; bd &= bd - 1) {
            const int k2 = __ffs(bd) - 1, b = m.ksub[k2 * m.L + q];
            if ((dn >> b) & 1u) continue;
            const uint32_t dn2 = dn ^ (1u << k2) ^ (1u << b);
            const int64_t j = mom_find(m, sb, up2, dn2);
            if (j < 0) continue;  // not in the sector (cannot happen: momentum is conserved)
            if (FILL) {
              const uint32_t sd = __popc(dn & between_bits(k2, b)) & 1u;
              col[out++] = (int32_t)((uint32_t)j | ((su ^ sd) << 31));
            }
            ++c;
          }
        }
      }
    }
    if (!FILL) cnt[i] = c;
  }
}

void launch_mom_count(const MomTables& m, int32_t* count, double* diag, cudaStream_t st) {
  k_mom_rows<false><<<blas_grid(m.n), kBlasThreads, 0, st>>>(m, count, diag, nullptr, nullptr);
  MB_CUDA(cudaGetLastError());
}

void launch_mom_fill(const MomTables& m, const int64_t* row_ptr, int32_t* col, cudaStream_t st) {
  k_mom_rows<true><<<blas_grid(m.n), kBlasThreads, 0, st>>>(m, nullptr, nullptr, row_ptr, col);
  MB_CUDA(cudaGetLastError());
}

__global__ void k_csr_count(OpView v, const int32_t* __restrict__ perm, int32_t* __restrict__ cnt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.dim;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ru = i / v.Dd, rd = i - ru * v.Dd;
    int c = (v.up_off[ru + 1] - v.up_off[ru]) + (v.dn_off[rd + 1] - v.dn_off[rd]);
    const double d = diag_value(v, ru, rd);
    if (!(d * d < kTol * kTol)) c += 1;
    cnt[perm[i]] = c;
  }
}

void launch_csr_count(const OpView& v, const int32_t* perm, int32_t* row_count, cudaStream_t st) {
  k_csr_count<<<blas_grid(v.dim), kBlasThreads, 0, st>>>(v, perm, row_count);
  MB_CUDA(cudaGetLastError());
}

__global__ void k_csr_fill(OpView v, const int32_t* __restrict__ perm, const int64_t* __restrict__ row_ptr,
                           int64_t* __restrict__ col_idx, double* __restrict__ values,
                           int* __restrict__ overflow) {
  int64_t cols[kMaxRowNnz];
  double vals[kMaxRowNnz];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < v.dim;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ru = i / v.Dd, rd = i - ru * v.Dd;
    int m = 0;
    const double d = diag_value(v, ru, rd);
    if (!(d * d < kTol * kTol)) { cols[m] = perm[i]; vals[m] = d; ++m; }
    for (int j = v.up_off[ru]; j < v.up_off[ru + 1]; ++j) {
      const uint32_t e = v.up_ent[j];
      if (m >= kMaxRowNnz) { atomicExch(overflow, 1); break; }
      cols[m] = perm[(int64_t)(e >> 8) * v.Dd + rd];
      vals[m] = -v.t * ((e & 2u) ? 2.0 : 1.0) * ((e & 1u) ? -1.0 : 1.0);
      ++m;
    }
    for (int j = v.dn_off[rd]; j < v.dn_off[rd + 1]; ++j) {
      const uint32_t e = v.dn_ent[j];
      if (m >= kMaxRowNnz) { atomicExch(overflow, 1); break; }
      cols[m] = perm[ru * v.Dd + (e >> 8)];
      vals[m] = -v.t * ((e & 2u) ? 2.0 : 1.0) * ((e & 1u) ? -1.0 : 1.0);
      ++m;
    }
    for (int a = 1; a < m; ++a) {
      const int64_t kc = cols[a];
      const double kv = vals[a];
      int b = a - 1;
      while (b >= 0 && cols[b] > kc) { cols[b + 1] = cols[b]; vals[b + 1] = vals[b]; --b; }
      cols[b + 1] = kc;
      vals[b + 1] = kv;
    }
    const int64_t base = row_ptr[perm[i]];
    for (int a = 0; a < m; ++a) {
      col_idx[base + a] = cols[a];
      values[2 * (base + a)] = vals[a];
      values[2 * (base + a) + 1] = 0.0;
    }
  }
}

void launch_csr_fill(const OpView& v, const int32_t* perm, const int64_t* row_ptr,
                     int64_t* col_idx, double* values, cudaStream_t st) {
  int* overflow = nullptr;
  MB_CUDA(cudaMallocAsync(&overflow, sizeof(int), st));
  MB_CUDA(cudaMemsetAsync(overflow, 0, sizeof(int), st));
  k_csr_fill<<<blas_grid(v.dim), 128, 0, st>>>(v, perm, row_ptr, col_idx, values, overflow);
  MB_CUDA(cudaGetLastError());
  int h = 0;
  MB_CUDA(cudaMemcpyAsync(&h, overflow, sizeof(int), cudaMemcpyDeviceToHost, st));
  MB_CUDA(cudaStreamSynchronize(st));
  MB_CUDA(cudaFreeAsync(overflow, st));
  MB_REQUIRE(!h, MB_ERR_CAPACITY, "a Hamiltonian row has more than 256 entries");
}

}  // namespace mb
