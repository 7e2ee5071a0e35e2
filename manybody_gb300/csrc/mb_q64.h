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
};

struct QPlanInput {
  double t, scale, shift, beta;
  double ufold[kMaxOrbitals + 1];
  double w_max;  // largest sum of |hop weights| of one state (both spins)
  int L;
  int ex, ez;
  int has_z;
};

__host__ __device__ void q_plan(QParams* p, const QPlanInput& in);

void launch_apply_q(const OpView& v, bool has_double_bonds, const void* x, void* y, const void* z,
                    const QParams* prm_dev, double* partials, unsigned long long* max_or, int dots,
                    cudaStream_t st);
int q_apply_grid(const OpView& v);
// Two-pass apply (down hops by rows, up hops by L2-resident column blocks)
// for sectors of >= 2^22 states when s_scratch (one Q64 vector) is given;
// otherwise the fused single-pass kernel.
void launch_apply_q2(const OpView& v, bool has_double_bonds, const void* x, void* y,
                     const void* z, void* s_scratch, const QParams* prm_dev, double* partials,
                     unsigned long long* max_or, int dots, cudaStream_t st);
bool q_use_split(const OpView& v);
// blocks that write dot partials for an apply (split or fused)
int q_apply_grid_for(const OpView& v, bool split);
int q_blas_grid(int64_t n);
int q_multi_dot_grid(int64_t n);

// FP64 (tensor or, through perm, reference order) -> Q64 with the exponent
// chosen from the vector's largest magnitude; scratch_int2 = 2 device ints
// (max biased exponent, resulting E).
void launch_f64_to_q(int64_t n, const void* src, const int32_t* perm, int qbits, int* scratch_int2,
                     void* dst, cudaStream_t st);
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
