// Operators between two momentum sectors and the current-current correlator.
//
// The current operator J_d(Q) = sum_{k,s} v_d(k) c+_{k+Q,s} c_{k,s},
// v_d(k) = 2t (2 pi / L_d) sin(2 pi k_d / L_d)
// (src/algebra/fermion/model/hubbard_model_momentum.h:38-90), maps the sector
// of total momentum K to K+Q.  The reference builds it with
// compute_rectangular_matrix_elements (src/algebra/matrix_elements.h:107-167)
// and uses it in the stochastic optical-conductivity driver
// (examples/hubbard_momentum_optical_conductivity.cpp:340-410).  Here J and
// its adjoint are built on the GPU as real-valued CSR (one electron moves per
// entry, so every entry is one v_d(k) times a hop sign), applied to complex
// vectors, and the correlator runs on the device.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "mb_internal.h"

struct mb_rect_op_s {
  int device = 0;
  int precision = MB_PREC_F64;
  int64_t n_rows = 0, n_cols = 0;
  // J (rows: sector K+Q) and its adjoint (rows: sector K): CSR on the device
  int64_t* rp[2] = {nullptr, nullptr};
  int32_t* col[2] = {nullptr, nullptr};
  double* val[2] = {nullptr, nullptr};
  std::vector<void*> allocations;
};

namespace mb {
namespace {

__constant__ Binom c_rect_binom;  // binomials for the rank lookups of this file

struct Dev {
  std::vector<void*>& owner;
  template <typename T>
  T* put(const std::vector<T>& h) {
    void* p = nullptr;
    MB_CUDA(cudaMalloc(&p, std::max<size_t>(sizeof(T) * h.size(), 16)));
    owner.push_back(p);
    if (!h.empty()) MB_CUDA(cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
    return (T*)p;
  }
  template <typename T>
  T* make(size_t n) {
    void* p = nullptr;
    MB_CUDA(cudaMalloc(&p, std::max<size_t>(sizeof(T) * n, 16)));
    owner.push_back(p);
    return (T*)p;
  }
};

// Rows of a one-electron operator between two sectors: for each row state
// and spin, each occupied orbital a whose target b = move[a] is empty gives
// the column state with a -> b and the value wt[a] * hop sign (0 weights
// are skipped); with Q = 0 the terms are number operators and merge into
// one diagonal entry (dropped below 1000 eps, as the reference's expression
// does).  Columns are found by full-sector reference rank and a binary
// search in the column sector's ranks.
struct MoveTables {
  int64_t n_rows, n_cols;
  int L;
  int diagonal;             // Q = 0: every move is the identity (J = sum v(k) n_k)
  const uint32_t* row_up;
  const uint32_t* row_dn;
  const int64_t* col_full;  // ascending
  const uint8_t* move;      // [L]
  const double* wt;         // [L]
};

__device__ __forceinline__ int64_t find_col(const MoveTables& m, const Binom& b, uint32_t up,
                                            uint32_t dn) {
  const int64_t r = reference_rank(b, up, dn, m.L);
  int64_t lo = 0, hi = m.n_cols;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (m.col_full[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  return (lo < m.n_cols && m.col_full[lo] == r) ? lo : -1;
}

__device__ __forceinline__ uint32_t strictly_between(int a, int b) {
  const int lo = min(a, b), hi = max(a, b);
  return ((1u << hi) - 1u) & ~((2u << lo) - 1u);
}

template <bool FILL>
__global__ void k_move_rows(MoveTables m, int32_t* __restrict__ cnt,
                            const int64_t* __restrict__ rp, int32_t* __restrict__ col,
                            double* __restrict__ val) {
  __shared__ Binom sb;
  for (int i = threadIdx.x; i < (int)(sizeof(Binom) / sizeof(int64_t)); i += blockDim.x)
    (&sb.c[0][0])[i] = (&c_rect_binom.c[0][0])[i];
  __syncthreads();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m.n_rows;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t up = m.row_up[i], dn = m.row_dn[i];
    int c = 0;
    int64_t o = FILL ? rp[i] : 0;
    if (m.diagonal) {  // one merged entry: sum of v(k) over the occupied orbitals
      double d = 0.0;
      for (uint32_t b = up; b; b &= b - 1) d += m.wt[__ffs(b) - 1];
      for (uint32_t b = dn; b; b &= b - 1) d += m.wt[__ffs(b) - 1];
      const int64_t j = find_col(m, sb, up, dn);
      if (!(d * d < kTol * kTol) && j >= 0) {
        if (FILL) {
          col[o] = (int32_t)j;
          val[o] = d;
        }
        c = 1;
      }
      if (!FILL) cnt[i] = c;
      continue;
    }
    for (int spin = 0; spin < 2; ++spin) {
      const uint32_t mine = spin ? dn : up;
      for (uint32_t bits = mine; bits; bits &= bits - 1) {
        const int a = __ffs(bits) - 1, b = m.move[a];
        const double w = m.wt[a];
        if (w == 0.0 || (a != b && ((mine >> b) & 1u))) continue;
        const uint32_t moved = a == b ? mine : (mine ^ (1u << a) ^ (1u << b));
        const int64_t j = spin ? find_col(m, sb, up, moved) : find_col(m, sb, moved, dn);
        if (j < 0) continue;
        if (FILL) {
          const int neg = a == b ? 0 : (__popc(mine & strictly_between(a, b)) & 1);
          col[o] = (int32_t)j;
          val[o] = neg ? -w : w;
          ++o;
        }
        ++c;
      }
    }
    if (!FILL) cnt[i] = c;
  }
}

constexpr int kThreads = 256;

int grid_for(int64_t n) {
  int64_t g = (n + kThreads - 1) / kThreads;
  if (g > 152 * 32) g = 152 * 32;
  return (int)std::max<int64_t>(g, 1);
}

// Builds the CSR of one direction; returns nnz.
int64_t build_rows(mb_rect_op_s* op, int which, const MoveTables& m) {
  Dev dev{op->allocations};
  std::vector<int64_t> rp((size_t)m.n_rows + 1, 0);
  if (m.n_rows > 0) {
    int32_t* cnt = dev.make<int32_t>((size_t)m.n_rows);
    k_move_rows<false><<<grid_for(m.n_rows), kThreads>>>(m, cnt, nullptr, nullptr, nullptr);
    MB_CUDA(cudaGetLastError());
    std::vector<int32_t> hc((size_t)m.n_rows);
    MB_CUDA(cudaMemcpy(hc.data(), cnt, sizeof(int32_t) * hc.size(), cudaMemcpyDeviceToHost));
    for (int64_t i = 0; i < m.n_rows; ++i) rp[(size_t)i + 1] = rp[(size_t)i] + hc[(size_t)i];
  }
  const int64_t nnz = rp.back();
  op->rp[which] = dev.put(rp);
  op->col[which] = dev.make<int32_t>((size_t)nnz);
  op->val[which] = dev.make<double>((size_t)nnz);
  if (m.n_rows > 0) {
    k_move_rows<true><<<grid_for(m.n_rows), kThreads>>>(m, nullptr, op->rp[which],
                                                         op->col[which], op->val[which]);
    MB_CUDA(cudaGetLastError());
  }
  MB_CUDA(cudaDeviceSynchronize());
  return nnz;
}

// y[row] = sum val * x[col] (real values, complex vectors).  A row of the
// current operator has about one entry per electron, so kRowLanes lanes take
// a row (32 / kRowLanes rows a warp): the partial sums meet in a two-step
// shuffle instead of five FP64 steps at a warp per row.  The warp steps
// through its rows together (the shuffles need every lane).
constexpr int kRowLanes = 4;

template <typename V2>
__global__ void k_real_csr_apply(int64_t n, const int64_t* __restrict__ rp,
                                 const int32_t* __restrict__ ci, const double* __restrict__ val,
                                 const V2* __restrict__ x, V2* __restrict__ y) {
  constexpr int RPW = 32 / kRowLanes;
  const int lane = threadIdx.x & (kRowLanes - 1);
  const int sub = (threadIdx.x & 31) / kRowLanes;
  const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t rb = w0 * RPW; rb < n; rb += nw * RPW) {
    const int64_t row = rb + sub;
    const bool live = row < n;
    double ar = 0.0, ai = 0.0;
    if (live)
      for (int64_t k = rp[row] + lane; k < rp[row + 1]; k += kRowLanes) {
        const V2 b = x[ci[k]];
        ar = fma(val[k], (double)b.x, ar);
        ai = fma(val[k], (double)b.y, ai);
      }
#pragma unroll
    for (int o = kRowLanes / 2; o > 0; o >>= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o);
      ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    if (live && lane == 0) {
      V2 out;
      out.x = (decltype(out.x))ar;
      out.y = (decltype(out.y))ai;
      y[row] = out;
    }
  }
}

// <a, b> = sum conj(a) b as per-block partials (re, im), fixed order.
template <typename V2>
__global__ void k_cdot(int64_t n, const V2* __restrict__ a, const V2* __restrict__ b,
                       double* __restrict__ partials) {
  __shared__ double sr[kThreads], si[kThreads];
  double re = 0.0, im = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const V2 u = a[i], v = b[i];
    re += (double)u.x * v.x + (double)u.y * v.y;
    im += (double)u.x * v.y - (double)u.y * v.x;
  }
  sr[threadIdx.x] = re;
  si[threadIdx.x] = im;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      sr[threadIdx.x] += sr[threadIdx.x + w];
      si[threadIdx.x] += si[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sr[0];
    partials[2 * blockIdx.x + 1] = si[0];
  }
}

void rect_apply(const mb_rect_op_s* op, const void* x, void* y, int adjoint, cudaStream_t st) {
  const int w = adjoint ? 1 : 0;
  const int64_t n = adjoint ? op->n_cols : op->n_rows;
  const int64_t rows_per_block = kThreads / kRowLanes;
  const int g = (int)std::min<int64_t>(
      std::max<int64_t>((n + rows_per_block - 1) / rows_per_block, 1), 152 * 16);
  if (op->precision == MB_PREC_F32)
    k_real_csr_apply<float2><<<g, kThreads, 0, st>>>(n, op->rp[w], op->col[w], op->val[w],
                                                     (const float2*)x, (float2*)y);
  else
    k_real_csr_apply<double2><<<g, kThreads, 0, st>>>(n, op->rp[w], op->col[w], op->val[w],
                                                       (const double2*)x, (double2*)y);
  MB_CUDA(cudaGetLastError());
}

std::complex<double> cdot(int precision, int64_t n, const void* a, const void* b, double* part,
                          int grid, cudaStream_t st) {
  if (precision == MB_PREC_F32)
    k_cdot<float2><<<grid, kThreads, 0, st>>>(n, (const float2*)a, (const float2*)b, part);
  else
    k_cdot<double2><<<grid, kThreads, 0, st>>>(n, (const double2*)a, (const double2*)b, part);
  MB_CUDA(cudaGetLastError());
  std::vector<double> h(2 * (size_t)grid);
  MB_CUDA(cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
  MB_CUDA(cudaStreamSynchronize(st));
  double re = 0.0, im = 0.0;
  for (int i = 0; i < grid; ++i) {
    re += h[2 * (size_t)i];
    im += h[2 * (size_t)i + 1];
  }
  return {re, im};
}

}  // namespace

// v_d(k) = 2t (2 pi / L_d) sin(2 pi k_d / L_d) per orbital, as the reference
// computes it (hubbard_model_momentum.h:38-48); 0 where it is 0 or below the
// expression's 1000 eps drop.
std::vector<double> current_velocity(const std::vector<int64_t>& dims, double t, int direction) {
  int64_t L = 1;
  for (int64_t d : dims) L *= d;
  std::vector<double> v((size_t)L, 0.0);
  for (int64_t k = 0; k < L; ++k) {
    int64_t rest = k, kd = 0;
    for (int d = 0; d <= direction; ++d) {
      kd = rest % dims[(size_t)d];
      rest /= dims[(size_t)d];
    }
    const double pi = 3.14159265358979323846;
    const double phase = 2.0 * pi * (double)kd / (double)dims[(size_t)direction];
    const double vel = 2.0 * t * (2.0 * pi / (double)dims[(size_t)direction]) * std::sin(phase);
    v[(size_t)k] = (vel == 0.0 || vel * vel < kTol * kTol) ? 0.0 : vel;
  }
  return v;
}

}  // namespace mb

using namespace mb;

extern "C" {

int mb_current_create(const int64_t* dims, int ndim, double t, const int64_t* transfer,
                      int direction, mb_model_t* out) {
  return guard([&] {
    MB_REQUIRE(dims && transfer && out && ndim >= 1 && ndim <= 3, MB_ERR_INVALID_ARG,
               "NULL argument or ndim outside 1..3");
    MB_REQUIRE(direction >= 0 && direction < ndim, MB_ERR_INVALID_ARG, "direction out of bounds");
    *out = nullptr;
    int64_t L = 1;
    for (int d = 0; d < ndim; ++d) {
      MB_REQUIRE(dims[d] >= 1 && transfer[d] >= 0 && transfer[d] < dims[d], MB_ERR_INVALID_ARG,
                 "bad lattice size or transfer");
      L *= dims[d];
      MB_REQUIRE(L <= kMaxOrbitals, MB_ERR_CAPACITY, "more than 32 orbitals");
    }
    MB_REQUIRE(std::isfinite(t), MB_ERR_INVALID_ARG, "t must be finite");
    auto m = std::make_unique<mb_model_s>();
    m->dims.assign(dims, dims + ndim);
    m->L = (int)L;
    m->t = t;
    m->current = true;
    m->transfer.assign(transfer, transfer + ndim);
    m->direction = direction;
    m->eps = current_velocity(m->dims, t, direction);
    int64_t terms = 0;
    for (double v : m->eps) terms += v != 0.0 ? 2 : 0;
    m->n_terms = terms;
    *out = m.release();
  });
}

int mb_rect_op_create(mb_basis_t row_basis, mb_basis_t col_basis, mb_model_t model, int precision,
                      mb_rect_op_t* out) {
  return guard([&] {
    MB_REQUIRE(row_basis && col_basis && model && out, MB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    MB_REQUIRE(model->current, MB_ERR_INVALID_ARG, "the model must be a current operator");
    MB_REQUIRE(precision == MB_PREC_F64 || precision == MB_PREC_F32, MB_ERR_INVALID_ARG,
               "precision must be MB_PREC_F64 or MB_PREC_F32");
    MB_REQUIRE(row_basis->momentum() && col_basis->momentum(), MB_ERR_INVALID_ARG,
               "both bases must be momentum sectors");
    MB_REQUIRE(row_basis->kdims == model->dims && col_basis->kdims == model->dims &&
                   row_basis->n_up == col_basis->n_up && row_basis->n_down == col_basis->n_down,
               MB_ERR_DIM_MISMATCH, "bases and operator differ in lattice or particle numbers");
    for (size_t d = 0; d < model->dims.size(); ++d)
      MB_REQUIRE((col_basis->kvec[d] + model->transfer[d]) % model->dims[d] == row_basis->kvec[d],
                 MB_ERR_DIM_MISMATCH, "the row sector must be the column sector's K + Q");
    int dev = 0;
    MB_CUDA(cudaGetDevice(&dev));
    auto op = std::make_unique<mb_rect_op_s>();
    op->device = dev;
    op->precision = precision;
    op->n_rows = row_basis->dim;
    op->n_cols = col_basis->dim;
    try {
      const int L = model->L;
      Dev d{op->allocations};
      MB_CUDA(cudaMemcpyToSymbol(c_rect_binom, &binom_table(), sizeof(Binom)));
      std::vector<uint8_t> minus_q((size_t)L), plus_q((size_t)L);
      std::vector<double> w_minus((size_t)L);
      int64_t q = 0, stride = 1;
      for (size_t i = 0; i < model->dims.size(); ++i) {
        q += model->transfer[i] * stride;
        stride *= model->dims[i];
      }
      for (int k = 0; k < L; ++k) {
        minus_q[(size_t)k] = (uint8_t)momentum_add(k, q, -1, model->dims);
        plus_q[(size_t)k] = (uint8_t)momentum_add(k, q, +1, model->dims);
        w_minus[(size_t)k] = model->eps[minus_q[(size_t)k]];  // J rows: k' -> k'-Q, weight v(k'-Q)
      }
      // J: rows in sector K+Q, an occupied k' moves back to k' - Q
      MoveTables j{row_basis->dim, col_basis->dim, L, q == 0, d.put(row_basis->kup),
                   d.put(row_basis->kdown), d.put(col_basis->kfull), d.put(minus_q), d.put(w_minus)};
      build_rows(op.get(), 0, j);
      // J+: rows in sector K, an occupied k moves to k + Q, weight v(k)
      MoveTables jt{col_basis->dim, row_basis->dim, L, q == 0, d.put(col_basis->kup),
                    d.put(col_basis->kdown), d.put(row_basis->kfull), d.put(plus_q),
                    d.put(model->eps)};
      build_rows(op.get(), 1, jt);
    } catch (...) {
      for (void* p : op->allocations) cudaFree(p);
      throw;
    }
    *out = op.release();
  });
}

int mb_rect_op_destroy(mb_rect_op_t op) {
  if (!op) return MB_OK;
  cudaSetDevice(op->device);
  cudaDeviceSynchronize();
  for (void* p : op->allocations) cudaFree(p);
  delete op;
  return MB_OK;
}

int mb_rect_op_dims(mb_rect_op_t op, int64_t* n_rows, int64_t* n_cols) {
  return guard([&] {
    MB_REQUIRE(op && n_rows && n_cols, MB_ERR_INVALID_ARG, "NULL argument");
    *n_rows = op->n_rows;
    *n_cols = op->n_cols;
  });
}

int mb_rect_op_apply(mb_rect_op_t op, const void* x_dev, void* y_dev, int adjoint, void* stream) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && y_dev, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(x_dev != y_dev, MB_ERR_INVALID_ARG, "x and y must not overlap");
    rect_apply(op, x_dev, y_dev, adjoint, (cudaStream_t)stream);
  });
}

int mb_compute_rectangular_matrix_elements_csr(mb_basis_t row_basis, mb_basis_t col_basis,
                                               mb_model_t model, int64_t* nnz, int64_t* row_ptr,
                                               int64_t* col_idx, double* values) {
  return guard([&] {
    MB_REQUIRE(nnz, MB_ERR_INVALID_ARG, "NULL argument");
    mb_rect_op_t op = nullptr;
    const int rc = mb_rect_op_create(row_basis, col_basis, model, MB_PREC_F64, &op);
    if (rc) throw Error(rc, mb_last_error());
    std::unique_ptr<mb_rect_op_s, int (*)(mb_rect_op_t)> hold(op, mb_rect_op_destroy);
    const int64_t n = op->n_rows;
    std::vector<int64_t> rp((size_t)n + 1);
    MB_CUDA(cudaMemcpy(rp.data(), op->rp[0], sizeof(int64_t) * rp.size(), cudaMemcpyDeviceToHost));
    const int64_t total = rp[(size_t)n];
    if (!col_idx) {
      *nnz = total;
      if (row_ptr) std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
      return;
    }
    MB_REQUIRE(*nnz >= total, MB_ERR_CAPACITY, "nnz capacity smaller than the matrix");
    MB_REQUIRE(row_ptr && values, MB_ERR_INVALID_ARG, "NULL row_ptr or values");
    std::vector<int32_t> hc((size_t)std::max<int64_t>(total, 1));
    std::vector<double> hv((size_t)std::max<int64_t>(total, 1));
    if (total) {
      MB_CUDA(cudaMemcpy(hc.data(), op->col[0], sizeof(int32_t) * (size_t)total, cudaMemcpyDeviceToHost));
      MB_CUDA(cudaMemcpy(hv.data(), op->val[0], sizeof(double) * (size_t)total, cudaMemcpyDeviceToHost));
    }
    for (int64_t i = 0; i < n; ++i) {
      std::vector<std::pair<int64_t, double>> row;
      for (int64_t k = rp[(size_t)i]; k < rp[(size_t)i + 1]; ++k) row.push_back({hc[(size_t)k], hv[(size_t)k]});
      std::sort(row.begin(), row.end());
      int64_t o = rp[(size_t)i];
      for (const auto& [c, v] : row) {
        col_idx[o] = c;
        values[2 * o] = v;
        values[2 * o + 1] = 0.0;
        ++o;
      }
    }
    std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
    *nnz = total;
  });
}

int mb_current_correlator(mb_op_t op_k, mb_op_t op_kq, mb_rect_op_t current, int64_t n_samples,
                          uint64_t seed, double beta, double dt, int64_t steps,
                          int64_t krylov_steps, double* correlator) {
  return guard([&] {
    MB_REQUIRE(op_k && op_kq && current && correlator, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(n_samples >= 1 && steps >= 1, MB_ERR_INVALID_ARG, "need samples and steps");
    int64_t nk = 0, nkq = 0;
    int prec_k = 0, prec_kq = 0;
    mb_op_dimension(op_k, &nk);
    mb_op_dimension(op_kq, &nkq);
    mb_op_precision(op_k, &prec_k);
    mb_op_precision(op_kq, &prec_kq);
    MB_REQUIRE(nk == current->n_cols && nkq == current->n_rows, MB_ERR_DIM_MISMATCH,
               "operators and current do not share sectors");
    MB_REQUIRE(prec_k == current->precision && prec_kq == current->precision, MB_ERR_INVALID_ARG,
               "operators and current must share the precision");
    const int prec = current->precision;
    const size_t es = prec == MB_PREC_F32 ? 8 : 16;
    std::vector<void*> bufs;
    auto alloc = [&](size_t bytes) {
      void* p = nullptr;
      MB_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
      bufs.push_back(p);
      return p;
    };
    struct Free {
      std::vector<void*>& b;
      ~Free() {
        for (void* p : b) cudaFree(p);
      }
    } release{bufs};
    void* v = alloc(es * (size_t)nk);
    void* phi1 = alloc(es * (size_t)nk);
    void* phi2 = alloc(es * (size_t)nkq);
    void* tmp_k = alloc(es * (size_t)nk);
    void* tmp_kq = alloc(es * (size_t)nkq);
    const int grid = grid_for(std::max(nk, nkq)) > 1024 ? 1024 : grid_for(std::max(nk, nkq));
    double* part = (double*)alloc(sizeof(double) * 2 * (size_t)grid);
    std::vector<std::complex<double>> acc((size_t)steps, 0.0);
    auto check = [](int rc) {
      if (rc) throw Error(rc, mb_last_error());
    };
    for (int64_t s = 0; s < n_samples; ++s) {
      // random-phase probe in sector K (Philox stream 1 + s)
      check(mb_fill_phase(op_k, seed, (uint32_t)(1 + s), v, MB_ORDER_REFERENCE, nullptr));
      // |v_beta> = exp(-beta H / 2) |v>; the correlator is a ratio of two
      // forms quadratic in v, so v needs no normalisation
      check(mb_time_evolve(op_k, v, MB_ORDER_REFERENCE, 0.5 * beta, krylov_steps, 1, phi1));
      const double z = cdot(prec, nk, phi1, phi1, part, grid, 0).real();
      MB_REQUIRE(z > 0.0, MB_ERR_ZERO_NORM, "thermal probe vanished");
      rect_apply(current, phi1, phi2, 0, 0);  // J |v_beta> in K + Q
      for (int64_t i = 0; i < steps; ++i) {
        rect_apply(current, phi2, tmp_k, 1, 0);  // J+ |phi_2> in K
        acc[(size_t)i] += cdot(prec, nk, phi1, tmp_k, part, grid, 0) / z;
        check(mb_time_evolve(op_k, phi1, MB_ORDER_REFERENCE, dt, krylov_steps, 0, tmp_k));
        std::swap(phi1, tmp_k);
        check(mb_time_evolve(op_kq, phi2, MB_ORDER_REFERENCE, dt, krylov_steps, 0, tmp_kq));
        std::swap(phi2, tmp_kq);
      }
    }
    for (int64_t i = 0; i < steps; ++i) {
      correlator[2 * i] = acc[(size_t)i].real() / (double)n_samples;
      correlator[2 * i + 1] = acc[(size_t)i].imag() / (double)n_samples;
    }
  });
}

}  // extern "C"
