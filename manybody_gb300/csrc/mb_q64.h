// Block-floating-point (Q64) vectors: declarations shared by the Q64 kernels
// and the drivers.  value_i = q_i * 2^E with q_i a 64-bit integer and E one
// exponent per vector (see mb_q64.cu for the arithmetic).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mb_internal.h"

namespace mb {

constexpr int kQMaxBasis = 1024;

// Fixed-point coefficients of one y = scale (H - shift) x + beta z launch:
//   P = c1 * S + cq[k] * x_q + c3 * z_q,   y_q = round(P / 2^sh)
// with S the exact hop sum and k = popcount(up & down).
struct QParams {
  long long c1;
  long long c3;
  long long cq[kMaxOrbitals + 1];
  int sh;
  int G;
  int ex, ey, ez;
  int pad;
  // the plan's scale and shift: a sparse-matrix operator's per-row diagonal
  // coefficient round(2^G scale (diag - shift)) is formed in its kernel
  double scale, shift;
};

struct QPlanInput {
  double t, scale, shift, beta;
  double ufold[kMaxOrbitals + 1];
  double w_max;  // largest sum of |hop weights| of one state (both spins)
  // bounds on max |x_q|, max |z_q| as fractions of 2^qbits (1 when unknown);
  // the output exponent follows them, so chained applies keep their bits
  double x_frac, z_frac;
  int L;
  int ex, ez;
  int has_z;
};

__host__ __device__ void q_plan(QParams* p, const QPlanInput& in);
// The plan input of y = H x (scale 1, no shift, no z) on an MB_PREC_Q64
// operator, the exponent of x read on the device.
QPlanInput q_plain_plan_input(const mb_op_s* op);

// The fused apply (see mb_q64.cu).  y must not alias x or z.  With ups (the
// column pass's up-hop sums of x, launch_upcol_q) the up hops are read from
// it; without, they are gathered from x in the same pass.  dots: 0 none;
// 5 Re<x,y> and max |y| (<y,y> left 0); any other non-zero value all three.
void launch_apply_q(const OpView& v, const void* x, void* y, const void* z, const QParams* prm_dev,
                    double* partials, unsigned long long* max_or, int dots, cudaStream_t st,
                    const void* ups = nullptr);
// The exact sum of an apply's per-block dot partials (4 words a block:
// 128-bit Re<x,y> and <y,y>) -> out[0], out[1] as double.
void launch_q_reduce128(const void* part, int nblocks, double* out, cudaStream_t st);
// Column pass of the two-pass apply: ups[c * Du + r] = exact sum of the up
// hops of (r, c) on x's mantissas (dim longlong2 elements of scratch).
void launch_upcol_q(const OpView& v, const void* x, void* ups, cudaStream_t st);
// whether a column of the sector fits in shared memory (the column pass)
bool q_upcol_fits(const OpView& v);
// whether the warps' table buffers fit beside the staged row (table_stage)
bool q_table_stage_fits(const OpView& v);
// blocks that write dot partials for an apply
int q_apply_grid(const OpView& v);
int q_blas_grid(int64_t n);
int q_multi_dot_grid(int64_t n);

// FP64 (tensor or, through perm, reference order) -> Q64 with the exponent
// chosen from the vector's largest magnitude; scratch_int2 = 2 device ints
// (max biased exponent, resulting E).
void launch_f64_to_q(int64_t n, const void* src, const int32_t* perm, int qbits, int* scratch_int2,
                     void* dst, cudaStream_t st);
// dst[iperm[i]] = src[i] for a reference-order complex128 chunk, its largest
// biased exponent folded into *emax (atomic max; zero it before the first).
void launch_scatter_maxexp(int64_t n, const void* src, const int32_t* iperm, void* dst,
                           int* emax, cudaStream_t st);
// complex128 -> Q64 in place, the exponent from scratch_int2[0] (the largest
// biased exponent) written to scratch_int2[1].
void launch_f64_to_q_inplace(int64_t n, void* buf, int qbits, int* scratch_int2, cudaStream_t st);
// Q64 (tensor order) -> FP64; with iperm (reference -> tensor index) the
// output is in reference order.
void launch_q_to_f64(int64_t n, const void* src, const int32_t* iperm, const int* e_dev, void* dst,
                     cudaStream_t st);
void launch_q_plan(const QPlanInput& in, const int* ex_dev, QParams* p_dev, cudaStream_t st);
void launch_q_lincomb(int64_t n, const void* a, long long ar, long long ai, const void* b,
                      long long br, long long bi, int sh, void* out, double* partials,
                      unsigned long long* max_or, cudaStream_t st);
void launch_q_dot(int64_t n, const void* a, const void* b, double* partials, cudaStream_t st);
void launch_q_multi_dot(int64_t n, const void* V, int64_t ld, int m, const void* w,
                        double* partials, cudaStream_t st);
void launch_q_multi_axpy(int64_t n, const void* V, int64_t ld, int m, const long long* c, int G,
                         int shw, void* w, double* partials, unsigned long long* max_or,
                         cudaStream_t st);

}  // namespace mb
