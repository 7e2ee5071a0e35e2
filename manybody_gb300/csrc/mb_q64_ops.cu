// Drivers of block-floating-point (MB_PREC_Q64) operators: the FP64-in /
// FP64-out apply, native Q64 entry points, and Lanczos / Krylov evolution
// on Q64 vectors.  Exponent bookkeeping happens on the host between kernel
// launches (the Lanczos loop reads alpha and beta every step anyway); the
// stand-alone apply plans on the device so it stays asynchronous.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "mb_internal.h"
#include "mb_q64.h"

namespace mb {

namespace {

struct QBuf {
  void* p = nullptr;
  QBuf() = default;
  explicit QBuf(size_t b) {
    if (b) MB_CUDA(cudaMalloc(&p, b));
  }
  ~QBuf() {
    if (p) cudaFree(p);
  }
  QBuf(const QBuf&) = delete;
  QBuf& operator=(const QBuf&) = delete;
  QBuf(QBuf&& o) noexcept : p(o.p) { o.p = nullptr; }
  QBuf& operator=(QBuf&& o) noexcept {
    std::swap(p, o.p);
    return *this;
  }
};

int ceil_log2(double v) {  // smallest k with v <= 2^k, v > 0
  int e;
  const double m = std::frexp(v, &e);
  return m == 0.5 ? e - 1 : e;
}

}  // namespace

void q_op_prepare(mb_op_s* op, const mb_model_s* m, const HopTable& tu, const HopTable& td) {
  MB_REQUIRE(!tu.has_self && !td.has_self, MB_ERR_INVALID_ARG,
             "MB_PREC_Q64 operators need a lattice without size-1 dimensions (self bonds); "
             "use MB_PREC_F64");
  auto wsum = [](const HopTable& t, int64_t D) {
    double best = 0.0;
    for (int64_t r = 0; r < D; ++r) {
      double s = 0.0;
      for (int32_t j = t.off[(size_t)r]; j < t.off[(size_t)r + 1]; ++j) s += (t.ent[(size_t)j] & 2u) ? 2.0 : 1.0;
      best = std::max(best, s);
    }
    return best;
  };
  op->q_wmax = wsum(tu, op->Du) + wsum(td, op->Dd);
  op->q_qbits = 62 - (op->q_wmax > 1.0 ? ceil_log2(op->q_wmax) : 0);
  op->q_has_double = false;
  for (const auto& b : m->bonds) op->q_has_double = op->q_has_double || b.mult == 2;
  op->ufold_host = u_fold_table(m->u, m->has_u, op->L);
  op->q_t = op->t;
  op->q_L = op->L;
}

void q_op_prepare_csr(mb_op_s* op, int64_t max_row_entries, double diag_min, double diag_max,
                      double off) {
  op->q_wmax = (double)std::max<int64_t>(max_row_entries, 1);
  op->q_qbits = 62 - (op->q_wmax > 1.0 ? ceil_log2(op->q_wmax) : 0);
  op->q_has_double = false;
  op->ufold_host = {diag_min, diag_max};
  op->q_t = -off;
  op->q_L = 1;
}

void q_op_release(mb_op_s* op) {
  for (auto& kv : op->qscratch) {
    for (void* p : {kv.second.xq, kv.second.yq, kv.second.prm, (void*)kv.second.ints})
      if (p) cudaFree(p);
  }
  op->qscratch.clear();
  for (auto& kv : op->ups_scratch)
    if (kv.second) cudaFree(kv.second);
  op->ups_scratch.clear();
}

static QPlanInput plan_input(const mb_op_s* op, double scale, double shift, double beta, int ex,
                             int ez, bool has_z, double x_frac = 1.0, double z_frac = 1.0) {
  QPlanInput in{};
  in.x_frac = std::min(x_frac, 1.0);
  in.z_frac = std::min(z_frac, 1.0);
  in.t = op->q_t;
  in.scale = scale;
  in.shift = shift;
  in.beta = beta;
  for (int k = 0; k <= op->q_L; ++k) in.ufold[k] = op->ufold_host[(size_t)k];
  in.w_max = op->q_wmax;
  in.L = op->q_L;
  in.ex = ex;
  in.ez = ez;
  in.has_z = has_z ? 1 : 0;
  return in;
}

QPlanInput q_plain_plan_input(const mb_op_s* op) {
  return plan_input(op, 1.0, 0.0, 0.0, 0, 0, false);
}

static mb_op_s::QScratch& qscratch_for(mb_op_s* op, cudaStream_t st) {
  std::lock_guard<std::mutex> lk(op->mu);
  auto& s = op->qscratch[st];
  if (!s.xq) {
    const size_t vb = sizeof(longlong2) * (size_t)op->dim;
    MB_CUDA(cudaMalloc(&s.xq, vb));
    MB_CUDA(cudaMalloc(&s.yq, vb));
    MB_CUDA(cudaMalloc(&s.prm, sizeof(QParams)));
    MB_CUDA(cudaMalloc((void**)&s.ints, 4 * sizeof(int)));
  }
  return s;
}

// The up-hop scratch of `st` when the operator's apply runs in two passes
// (allocated on first use), else nullptr.
static void* q_ups_for(mb_op_s* op, cudaStream_t st) {
  if (op->apply_passes != 2 || !q_upcol_fits(op->view)) return nullptr;
  std::lock_guard<std::mutex> lk(op->mu);
  void*& p = op->ups_scratch[st];
  if (!p) MB_CUDA(cudaMalloc(&p, sizeof(longlong2) * (size_t)op->dim));
  return p;
}

// The Q64 apply of the whole sector in the operator's shape.
static void q_apply_whole(mb_op_s* op, const void* xq, void* yq, const void* zq,
                          const QParams* prm, double* partials, unsigned long long* max_or,
                          int dots, cudaStream_t st) {
  void* ups = q_ups_for(op, st);
  if (ups) launch_upcol_q(op->view, xq, ups, st);
  launch_apply_q(op->view, xq, yq, zq, prm, partials, max_or, dots, st, ups);
}

// The autotuner's Q64 vectors: a seeded vector's mantissas (tensor order), an
// output and its planned parameters (y = H x).
void q_tune_prepare(mb_op_s* op, void** xq, void** yq, void** prm, cudaStream_t st) {
  const size_t vb = sizeof(longlong2) * (size_t)op->dim;
  QBuf x64(vb), ints(4 * sizeof(int));
  void *a = nullptr, *b = nullptr, *p = nullptr;
  try {
    MB_CUDA(cudaMalloc(&a, vb));
    MB_CUDA(cudaMalloc(&b, vb));
    MB_CUDA(cudaMalloc(&p, sizeof(QParams)));
    launch_fill_rng(MB_PREC_F64, op->Du, op->Dd, 12345, 0, 0, x64.p, st);
    launch_f64_to_q(op->dim, x64.p, nullptr, op->q_qbits, (int*)ints.p, a, st);
    launch_q_plan(q_plain_plan_input(op), (const int*)ints.p + 1, (QParams*)p, st);
    MB_CUDA(cudaStreamSynchronize(st));
  } catch (...) {
    for (void* q : {a, b, p})
      if (q) cudaFree(q);
    throw;
  }
  *xq = a;
  *yq = b;
  *prm = p;
}

void q_tune_apply(mb_op_s* op, const void* xq, void* yq, const void* prm, cudaStream_t st) {
  q_apply_whole(op, xq, yq, nullptr, (const QParams*)prm, nullptr, nullptr, 0, st);
}

// y = scale (H - shift) x + beta z on complex128 vectors through Q64.
// z, when used, is folded in FP64 after the Q64 apply (z keeps its own
// magnitude): y = Q64[scale (H - shift) x] + beta z.
void q_apply_affine(mb_op_s* op, const void* x, void* y, double scale, double shift, double beta,
                    const void* z, int order, cudaStream_t st) {
  auto& s = qscratch_for(op, st);
  int32_t* perm = order == MB_ORDER_REFERENCE ? op_perm(op) : nullptr;
  int32_t* iperm = order == MB_ORDER_REFERENCE ? op_iperm(op) : nullptr;
  launch_f64_to_q(op->dim, x, perm, op->q_qbits, s.ints, s.xq, st);
  launch_q_plan(plan_input(op, scale, shift, 0.0, 0, 0, false), s.ints + 1, (QParams*)s.prm, st);
  q_apply_whole(op, s.xq, s.yq, nullptr, (const QParams*)s.prm, nullptr, nullptr, 0, st);
  // the output exponent sits in the planned QParams (field ey)
  const int* ey = (const int*)((const char*)s.prm + offsetof(QParams, ey));
  if (!z) {
    launch_q_to_f64(op->dim, s.yq, iperm, ey, y, st);
    return;
  }
  // y = beta z + (Q64 result): z may alias y; convert into a tensor-order
  // temporary, then combine with the FP64 vector kernel.
  QBuf tmp(sizeof(double2) * (size_t)op->dim);
  launch_q_to_f64(op->dim, s.yq, iperm, ey, tmp.p, st);
  launch_axpby(MB_PREC_F64, op->dim, beta, 0.0, z, 1.0, 0.0, tmp.p, nullptr, 0, st);
  MB_CUDA(cudaMemcpyAsync(y, tmp.p, sizeof(double2) * (size_t)op->dim, cudaMemcpyDeviceToDevice, st));
  MB_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------------------
// The host-buffer apply in reference order, pipelined over the host link.
//
// On the way in, a page-locked x is read over the link by the kernel that
// scatters it to tensor order (with its largest exponent); a pageable x
// arrives in chunks, each scattered while the next one is in flight.  The
// vector is converted to Q64 in place once all of it has landed.  On the way
// out, the rows are applied in groups ordered by the first reference index
// among their states, so each group finishes a prefix of the reference order,
// which is converted back and downloaded on the copy engine while the later
// groups run (host_groups_run).  The arithmetic is that of mb_op_apply (same
// exponent, same kernel per row), so the result is bit-identical to the
// device-buffer call.
// ---------------------------------------------------------------------------

static void q_apply_host_pipeline(mb_op_s* op, const mb_op_s::HostLane& lane, const void* x_host,
                                  const void* x_mapped, void* y_host, void* x_stage,
                                  void* y_stage);

void q_apply_host_reference(mb_op_s* op, const mb_op_s::HostLane& lane, const void* x_host,
                            const void* x_mapped, void* y_host, void* x_stage, void* y_stage) {
  try {
    q_apply_host_pipeline(op, lane, x_host, x_mapped, y_host, x_stage, y_stage);
  } catch (...) {
    // nothing may still read or write the caller's buffers once it sees the error
    cudaStreamSynchronize(lane.copy);
    cudaStreamSynchronize(lane.comp);
    throw;
  }
}

static void q_apply_host_pipeline(mb_op_s* op, const mb_op_s::HostLane& lane, const void* x_host,
                                  const void* x_mapped, void* y_host, void* x_stage,
                                  void* y_stage) {
  cudaStream_t comp = lane.comp;
  auto& q = qscratch_for(op, comp);
  int32_t* iperm = op_iperm(op);
  const int64_t n = op->dim;
  constexpr size_t es = sizeof(double2);
  MB_CUDA(cudaMemsetAsync(q.ints, 0, sizeof(int), comp));
  if (x_mapped) {
    // page-locked x: the scatter kernel reads it over the link directly
    launch_scatter_maxexp(n, x_mapped, iperm, q.xq, q.ints, comp);
  } else {
    // pageable x: through the lane's bounce buffers, each chunk scattered once landed
    lane_upload(lane, x_stage, x_host, es * (size_t)n, es, [&](size_t off, size_t len, cudaEvent_t e) {
      MB_CUDA(cudaStreamWaitEvent(comp, e, 0));
      const int64_t i0 = (int64_t)(off / es);
      launch_scatter_maxexp((int64_t)(len / es), (const char*)x_stage + off, iperm + i0, q.xq,
                            q.ints, comp);
    });
  }
  launch_f64_to_q_inplace(n, q.xq, op->q_qbits, q.ints, comp);
  launch_q_plan(plan_input(op, 1.0, 0.0, 0.0, 0, 0, false), q.ints + 1, (QParams*)q.prm, comp);
  const int* ey = (const int*)((const char*)q.prm + offsetof(QParams, ey));
  // two passes: the column pass covers the whole sector before the first group
  void* ups = q_ups_for(op, comp);
  if (ups) launch_upcol_q(op->view, q.xq, ups, comp);
  host_groups_run(
      op, lane, es, y_host, y_stage,
      [&](const OpView& v) {
        launch_apply_q(v, q.xq, q.yq, nullptr, (const QParams*)q.prm, nullptr, nullptr, 0, comp,
                       ups);
      },
      [&](int64_t i0, int64_t i1, void* dst) {
        launch_q_to_f64(i1 - i0, q.yq, iperm + i0, ey, dst, comp);
      });
}

// ---------------------------------------------------------------------------
// Q64 Krylov machinery.
// ---------------------------------------------------------------------------
namespace {

// Non-owning view of a Q64 vector: mantissas, exponent, bound on max |q|.
struct QRef {
  void* p = nullptr;
  int E = 0;
  double maxq = 0.0;
  // the vector is m times its mantissas' value: a normalisation not yet
  // applied to them (the plain Lanczos recurrence folds 1 / beta into the
  // coefficients of the next apply and combination instead of a pass)
  double m = 1.0;
};

struct QVec {
  QBuf buf;
  QRef r;
  explicit QVec(int64_t n) : buf(sizeof(longlong2) * (size_t)n) { r.p = buf.p; }
};

struct QKrylov {
  mb_op_s* op;
  cudaStream_t st;
  int64_t n;
  int qbits;
  QBuf partials, red_out, maxor, prm;
  double* host = nullptr;      // pinned: reduce outputs, then the max word
  QParams* hprm = nullptr;     // pinned
  int grid_apply, grid_blas, grid_md;
  QBuf basis;                  // reorth basis: columns of n mantissas
  int64_t basis_cap = 0;
  std::vector<int> basis_E;
  std::vector<double> basis_max;
  QBuf coef;
  long long* hcoef = nullptr;  // pinned
  // Kept Lanczos vectors (plain runs that need their Ritz vector): the
  // mantissas of the vectors pass one applies, with their exponents, bounds
  // and pending normalisations, in chunks of kQKeepChunk columns while a
  // tenth of the device memory stays free.  The Ritz vector is summed from
  // them by pass two's combination sequence (the same bits) without
  // re-running the recurrence.
  static constexpr int64_t kQKeepChunk = 16;
  std::vector<QBuf> keep;
  std::vector<QRef> kept;

  QKrylov(mb_op_s* o, cudaStream_t s)
      : op(o), st(s), n(o->dim), qbits(o->q_qbits),
        partials(sizeof(double) *
                 (size_t)std::max(q_apply_grid(o->view) * 4,
                                  std::max(q_blas_grid(o->dim) * 2,
                                           q_multi_dot_grid(o->dim) * 2 * kQMaxBasis))),
        red_out(sizeof(double) * 2 * kQMaxBasis), maxor(sizeof(unsigned long long)),
        prm(sizeof(QParams)),
        grid_apply(q_apply_grid(o->view)), grid_blas(q_blas_grid(o->dim)),
        grid_md(q_multi_dot_grid(o->dim)), coef(sizeof(long long) * 2 * kQMaxBasis) {
    MB_CUDA(cudaMallocHost((void**)&host, sizeof(double) * (2 * kQMaxBasis + 8)));
    MB_CUDA(cudaMallocHost((void**)&hprm, sizeof(QParams)));
    MB_CUDA(cudaMallocHost((void**)&hcoef, sizeof(long long) * 2 * kQMaxBasis));
  }
  ~QKrylov() {
    if (host) cudaFreeHost(host);
    if (hprm) cudaFreeHost(hprm);
    if (hcoef) cudaFreeHost(hcoef);
  }

  double* part() { return (double*)partials.p; }
  unsigned long long* mor() { return (unsigned long long*)maxor.p; }
  void zero_max() { MB_CUDA(cudaMemsetAsync(maxor.p, 0, sizeof(unsigned long long), st)); }

  // Reduce partials (nblocks x ncomp) plus the max word; waits on the stream.
  const double* fetch(int nblocks, int ncomp, double* maxq_out) {
    launch_reduce(part(), nblocks, ncomp, (double*)red_out.p, st);
    MB_CUDA(cudaMemcpyAsync(host, red_out.p, sizeof(double) * ncomp, cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaMemcpyAsync(host + ncomp, maxor.p, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
    if (maxq_out) {
      unsigned long long m;
      std::memcpy(&m, host + ncomp, sizeof(m));
      *maxq_out = m ? std::ldexp(1.0, 64 - __builtin_clzll(m)) : 0.0;  // max < 2^bitlen(OR)
    }
    return host;
  }

  // The apply's exact dot partials (128-bit, 4 words a block), summed and
  // converted once, plus the max word; waits on the stream.
  const double* fetch_apply(double* maxq_out) {
    launch_q_reduce128(part(), grid_apply, (double*)red_out.p, st);
    MB_CUDA(cudaMemcpyAsync(host, red_out.p, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaMemcpyAsync(host + 2, maxor.p, sizeof(unsigned long long),
                            cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
    unsigned long long m;
    std::memcpy(&m, host + 2, sizeof(m));
    *maxq_out = m ? std::ldexp(1.0, 64 - __builtin_clzll(m)) : 0.0;  // max < 2^bitlen(OR)
    return host;
  }

  // out = ca a + cb b (complex coefficients; out may alias a or b).  The
  // output exponent comes from the bound |ca| max|a| + |cb| max|b|.
  // Returns ||out||^2.
  double lincomb(QRef& out, const QRef* a, std::complex<double> ca, const QRef* b,
                 std::complex<double> cb) {
    if (a) ca *= a->m;
    if (b) cb *= b->m;
    out.m = 1.0;
    const double ba = a ? std::abs(ca) * std::ldexp(a->maxq, a->E) : 0.0;
    const double bb = b ? std::abs(cb) * std::ldexp(b->maxq, b->E) : 0.0;
    const double bound = (ba + bb) * (1.0 + 1e-12);
    const int Eo = bound > 0.0 ? ceil_log2(bound) - qbits : (a ? a->E : (b ? b->E : 0));
    double cmax = 0.0;
    if (a) cmax = std::max(cmax, std::abs(ca) * std::ldexp(1.0, a->E - Eo));
    if (b) cmax = std::max(cmax, std::abs(cb) * std::ldexp(1.0, b->E - Eo));
    const int Gs = cmax > 0.0 ? std::min(61 - ceil_log2(cmax), 120) : 0;
    auto fx = [&](double c, int E) -> long long { return std::llrint(std::ldexp(c, E - Eo + Gs)); };
    long long ar = 0, ai = 0, br = 0, bi = 0;
    if (a) { ar = fx(ca.real(), a->E); ai = fx(ca.imag(), a->E); }
    if (b) { br = fx(cb.real(), b->E); bi = fx(cb.imag(), b->E); }
    zero_max();
    launch_q_lincomb(n, a ? a->p : nullptr, ar, ai, b ? b->p : nullptr, br, bi, Gs, out.p, part(),
                     mor(), st);
    double mq = 0.0;
    const double* h = fetch(grid_blas, 2, &mq);
    out.E = Eo;
    out.maxq = std::max(mq, 1.0);
    return h[0] * std::ldexp(1.0, 2 * Eo + 32);
  }

  // w = scale H v - beta_prev v_prev; returns (Re<v,w>, ||w||^2).
  std::pair<double, double> apply(QRef& w, const QRef& v, double scale, double beta_prev,
                                  const QRef* v_prev) {
    // the recurrence reads Re<v,w> only: ||w||^2 comes from w -= alpha v
    return apply_affine(w, v, scale, 0.0, -beta_prev, v_prev, 5);
  }

  // w = scale (H - shift) v + beta z; returns (Re<v,w>, ||w||^2) (dots 5: the
  // second is left 0, saving its 128-bit products).
  std::pair<double, double> apply_affine(QRef& w, const QRef& v, double scale, double shift,
                                         double beta, const QRef* z, int dots = 1) {
    // scale (H - shift)(m v) = (scale m)(H - shift) v
    scale *= v.m;
    if (z) beta *= z->m;
    w.m = 1.0;
    const bool hz = z && beta != 0.0;
    const double full = std::ldexp(1.0, qbits);
    q_plan(hprm, plan_input(op, scale, shift, beta, v.E, hz ? z->E : v.E, hz, v.maxq / full,
                            hz ? z->maxq / full : 1.0));
    MB_CUDA(cudaMemcpyAsync(prm.p, hprm, sizeof(QParams), cudaMemcpyHostToDevice, st));
    zero_max();
    q_apply_whole(op, v.p, w.p, hz ? z->p : nullptr, (const QParams*)prm.p, part(), mor(), dots, st);
    double mq = 0.0;
    const double* h = fetch_apply(&mq);
    w.E = hprm->ey;
    w.maxq = std::max(mq, 1.0);
    return {v.m * h[0] * std::ldexp(1.0, v.E + w.E + 32), h[1] * std::ldexp(1.0, 2 * w.E + 32)};
  }

  void reserve_basis(int64_t k) {
    size_t free_b = 0, total_b = 0;
    MB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t need = (size_t)k * sizeof(longlong2) * (size_t)n;
    MB_REQUIRE(need + (size_t)(512u << 20) < free_b, MB_ERR_OOM,
               "Krylov basis for full re-orthogonalisation does not fit in device memory");
    MB_REQUIRE(k <= kQMaxBasis, MB_ERR_CAPACITY, "re-orthogonalisation basis larger than 1024");
    basis = QBuf(need);
    basis_cap = k;
  }

  QRef column(int64_t j) const {
    QRef r;
    r.p = (char*)basis.p + sizeof(longlong2) * (size_t)n * (size_t)j;
    r.E = basis_E[(size_t)j];
    r.maxq = basis_max[(size_t)j];
    return r;
  }

  void store_basis(const QRef& v) {
    MB_REQUIRE(v.m == 1.0, MB_ERR_INVALID_ARG, "basis vector with a pending normalisation");
    const int64_t j = (int64_t)basis_E.size();
    MB_REQUIRE(j < basis_cap, MB_ERR_CAPACITY, "basis full");
    MB_CUDA(cudaMemcpyAsync((char*)basis.p + sizeof(longlong2) * (size_t)n * (size_t)j, v.p,
                            sizeof(longlong2) * (size_t)n, cudaMemcpyDeviceToDevice, st));
    basis_E.push_back(v.E);
    basis_max.push_back(v.maxq);
  }

  // Classical Gram-Schmidt, w -= V (V^H w), with the DGKS test (a second
  // pass only when the first took w below 1/sqrt(2) of its norm, nrm2 on
  // entry).  Returns ||w||^2.
  double reorth(QRef& w, double nrm2) {
    const int m = (int)basis_E.size();
    for (int pass = 0; pass < 2; ++pass) {
      const double before = nrm2;
      launch_q_multi_dot(n, basis.p, n, m, w.p, part(), st);
      const double* h = fetch(grid_md, 2 * m, nullptr);
      std::vector<std::complex<double>> c((size_t)m);
      double bmant = w.maxq;  // bound of the result in w-mantissa units
      for (int j = 0; j < m; ++j) {
        const double s = std::ldexp(1.0, basis_E[(size_t)j] + w.E + 32);
        c[(size_t)j] = {h[2 * j] * s, h[2 * j + 1] * s};
        bmant += std::abs(c[(size_t)j]) * std::ldexp(basis_max[(size_t)j], basis_E[(size_t)j] - w.E);
      }
      const int shw = std::max(0, ceil_log2(bmant * (1.0 + 1e-12)) - qbits);
      const int G = std::max(0, std::min(62, 124 - ceil_log2(std::max(bmant, 1.0))));
      for (int j = 0; j < m; ++j) {
        hcoef[2 * j] = std::llrint(std::ldexp(c[(size_t)j].real(), basis_E[(size_t)j] - w.E + G));
        hcoef[2 * j + 1] = std::llrint(std::ldexp(c[(size_t)j].imag(), basis_E[(size_t)j] - w.E + G));
      }
      MB_CUDA(cudaMemcpyAsync(coef.p, hcoef, sizeof(long long) * 2 * (size_t)m,
                              cudaMemcpyHostToDevice, st));
      zero_max();
      launch_q_multi_axpy(n, basis.p, n, m, (const long long*)coef.p, G, shw, w.p, part(), mor(), st);
      double mq = 0.0;
      const double* h2 = fetch(grid_blas, 2, &mq);
      w.E += shw;
      w.maxq = std::max(mq, 1.0);
      nrm2 = h2[0] * std::ldexp(1.0, 2 * w.E + 32);
      if (nrm2 >= 0.5 * before) break;
    }
    return nrm2;
  }

  // Pass one from b (Q64, tensor order) (lanczos.h:130-175).
  int64_t pass_one(const QRef& b, double b_norm, int64_t k, double scale,
                   std::vector<double>& alphas, std::vector<double>& betas, bool reorth_on,
                   double conv_tol, int check_every, QRef* vp, QRef* vc, QRef* ww,
                   bool keep_vectors = false) {
    alphas.clear();
    betas.clear();
    kept.clear();
    if (k == 0) return 0;
    lincomb(*vc, &b, 1.0 / b_norm, nullptr, 0.0);
    double beta_prev = 0.0;
    int64_t steps = 0;
    double last_ritz = 0.0;
    bool have_ritz = false;
    for (int64_t it = 0; it < k; ++it) {
      if (reorth_on) store_basis(*vc);
      if (keep_vectors && (int64_t)kept.size() == it && keep_room(it)) keep_vector(*vc);
      const double alpha = apply(*ww, *vc, scale, beta_prev, beta_prev != 0.0 ? vp : nullptr).first;
      QRef wv = *ww;
      double nrm2 = lincomb(*ww, vc, -alpha, &wv, 1.0);  // w -= alpha v
      if (reorth_on) nrm2 = reorth(*ww, nrm2);
      const double beta = std::sqrt(nrm2);
      alphas.push_back(alpha);
      steps += 1;
      if (beta <= kTol) break;
      if (it + 1 < k) betas.push_back(beta);
      std::swap(vp, vc);  // v_prev <- v
      std::swap(vc, ww);  // v <- w / beta
      if (reorth_on) {  // the basis stores normalised mantissas
        QRef cur = *vc;
        lincomb(*vc, &cur, 1.0 / beta, nullptr, 0.0);
      } else {  // folded into the next apply and combination
        vc->m = 1.0 / beta;
      }
      beta_prev = beta;
      if (conv_tol > 0.0 && check_every > 0 && (steps % check_every) == 0 && it + 1 < k) {
        std::vector<double> d(alphas), e(betas);
        e.resize(d.size() - 1);
        if (tridiag_eig((int)d.size(), d, e, nullptr)) {
          const double ritz = d.back();
          if (have_ritz && std::fabs(ritz - last_ritz) <= conv_tol * std::fabs(ritz)) {
            betas.resize((size_t)steps - 1);
            break;
          }
          last_ritz = ritz;
          have_ritz = true;
        }
      }
    }
    if ((int64_t)betas.size() > std::max<int64_t>(steps - 1, 0)) betas.resize((size_t)steps - 1);
    return steps;
  }

  // x = sum_j y_j v_j by re-running the recurrence (lanczos.h:177-218) with
  // pass one's operations and coefficients (the same apply, w -= alpha v, the
  // 1/beta folded into the next vector), so the replayed vectors are pass
  // one's mantissas and exponents.
  void pass_two(const QRef& b, double b_norm, int64_t steps, double scale,
                const std::vector<double>& alphas, const std::vector<double>& betas,
                const std::vector<std::complex<double>>& y, QRef& x, QRef* vp, QRef* vc,
                QRef* ww) {
    lincomb(*vc, &b, 1.0 / b_norm, nullptr, 0.0);
    lincomb(x, vc, y[0], nullptr, 0.0);
    for (int64_t j = 0; j + 1 < steps; ++j) {
      const double beta_prev = j == 0 ? 0.0 : betas[(size_t)j - 1];
      apply(*ww, *vc, scale, beta_prev, beta_prev != 0.0 ? vp : nullptr);
      QRef wv = *ww;
      lincomb(*ww, vc, -alphas[(size_t)j], &wv, 1.0);
      std::swap(vp, vc);
      std::swap(vc, ww);
      vc->m = 1.0 / betas[(size_t)j];
      QRef xv = x;
      lincomb(x, &xv, 1.0, vc, y[(size_t)j + 1]);
    }
  }

  bool keep_room(int64_t j) {
    if ((size_t)(j / kQKeepChunk) < keep.size()) return true;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const size_t need = sizeof(longlong2) * (size_t)n * (size_t)kQKeepChunk;
    if (need + total_b / 10 > free_b) return false;
    try {
      keep.emplace_back(need);
    } catch (const Error&) {
      cudaGetLastError();
      return false;
    }
    return true;
  }

  void keep_vector(const QRef& v) {
    const int64_t j = (int64_t)kept.size();
    QRef c = v;
    c.p = (char*)keep[(size_t)(j / kQKeepChunk)].p +
          sizeof(longlong2) * (size_t)n * (size_t)(j % kQKeepChunk);
    MB_CUDA(cudaMemcpyAsync(c.p, v.p, sizeof(longlong2) * (size_t)n, cudaMemcpyDeviceToDevice,
                            st));
    kept.push_back(c);
  }

  // x = sum_(j < steps) y_j v_j from the kept vectors, in pass two's order.
  void combine_kept(int64_t steps, const std::vector<std::complex<double>>& y, QRef& x) {
    lincomb(x, &kept[0], y[0], nullptr, 0.0);
    for (int64_t j = 1; j < steps; ++j) {
      QRef xv = x;
      lincomb(x, &xv, 1.0, &kept[(size_t)j], y[(size_t)j]);
    }
  }

  // x = sum_j y_j V_j from the stored basis.
  void combine_basis(int64_t steps, const std::vector<std::complex<double>>& y, QRef& x) {
    for (int64_t j = 0; j < steps; ++j) {
      const QRef vj = column(j);
      if (j == 0) {
        lincomb(x, &vj, y[0], nullptr, 0.0);
      } else {
        QRef xv = x;
        lincomb(x, &xv, 1.0, &vj, y[(size_t)j]);
      }
    }
  }

  // complex128 (order) -> Q64 tensor order; returns ||b||.
  double load(const void* src, int order, QRef& out) {
    int32_t* perm = order == MB_ORDER_REFERENCE ? op_perm(op) : nullptr;
    QBuf ints(4 * sizeof(int));
    launch_f64_to_q(n, src, perm, qbits, (int*)ints.p, out.p, st);
    int hE[2];
    MB_CUDA(cudaMemcpyAsync(hE, ints.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
    out.E = hE[1];
    out.maxq = std::ldexp(1.0, qbits);
    launch_q_dot(n, out.p, out.p, part(), st);
    const double* h = fetch(grid_blas, 2, nullptr);
    return std::sqrt(h[0] * std::ldexp(1.0, 2 * out.E + 32));
  }

  void store(const QRef& x, int order, void* dst) {
    int32_t* iperm = order == MB_ORDER_REFERENCE ? op_iperm(op) : nullptr;
    QBuf e(sizeof(int));
    MB_CUDA(cudaMemcpyAsync(e.p, &x.E, sizeof(int), cudaMemcpyHostToDevice, st));
    launch_q_to_f64(n, x.p, iperm, (const int*)e.p, dst, st);
    MB_CUDA(cudaStreamSynchronize(st));
  }
};

}  // namespace

void q_eigenpair(mb_op_s* op, int64_t k, const void* seed, int order, const mb_lanczos_opts* opts,
                 double sign, double* e_out, void* vec, int64_t* steps_out) {
  MB_REQUIRE(k >= 0, MB_ERR_INVALID_ARG, "k must be >= 0");
  mb_lanczos_opts o{};
  o.basis_precision = -1;
  o.check_every = 10;
  if (opts) o = *opts;
  if (o.check_every <= 0) o.check_every = 10;
  cudaStream_t st = 0;
  QKrylov kr(op, st);
  const int64_t n = op->dim;
  QVec b(n), vp(n), vc(n), w(n);
  const double b_norm = kr.load(seed, order, b.r);
  MB_REQUIRE(b_norm > kTol, MB_ERR_ZERO_NORM, "Input vector has zero norm");
  const bool reorth = o.reorth != 0 && k > 0;
  if (reorth) kr.reserve_basis(k);
  std::vector<double> alphas, betas;
  const int64_t m = kr.pass_one(b.r, b_norm, k, sign, alphas, betas, reorth, o.conv_tol,
                                o.check_every, &vp.r, &vc.r, &w.r, vec && !reorth);
  if (steps_out) *steps_out = m;
  if (m == 0) {
    *e_out = 0.0;
    if (vec) MB_CUDA(cudaMemset(vec, 0, sizeof(double2) * (size_t)n));
    return;
  }
  std::vector<double> d(alphas), z, e(betas);
  e.resize((size_t)m - 1);
  MB_REQUIRE(tridiag_eig((int)m, d, e, &z), MB_ERR_EIG_FAILED,
             "Eigenvalue decomposition of T_k failed");
  *e_out = sign * d[(size_t)m - 1];
  if (vec) {
    std::vector<std::complex<double>> y((size_t)m);
    for (int64_t i = 0; i < m; ++i) y[(size_t)i] = z[(size_t)(m - 1) * m + i] * b_norm;
    QVec x(n);
    if (reorth) kr.combine_basis(m, y, x.r);
    else if (m <= (int64_t)kr.kept.size()) kr.combine_kept(m, y, x.r);
    else kr.pass_two(b.r, b_norm, m, sign, alphas, betas, y, x.r, &vp.r, &vc.r, &w.r);
    kr.store(x.r, order, vec);
  }
}

// DOS Chebyshev moments on Q64 vectors: per probe (random phases, Philox
// stream 1 + p, tensor order) T_0 = r, T_1 = Ht T_0, T_{s+1} = 2 Ht T_s -
// T_{s-1} with Ht = (H - b) / a, each step one fused apply whose exact dots
// give <T_s, T_{s+1}> and <T_{s+1}, T_{s+1}>; moments by the doubling
// identities mu_2s = 2<T_s,T_s> - mu_0, mu_2s+1 = 2<T_s,T_{s+1}> - mu_1.
void q_kpm_dos_moments(mb_op_s* op, int64_t n_moments, int64_t n_probes, uint64_t seed, double a,
                       double b, double* mu) {
  cudaStream_t st = 0;
  QKrylov kr(op, st);
  const int64_t n = op->dim;
  QVec v0(n), v1(n), v2(n);
  QBuf probe(sizeof(double2) * (size_t)n);
  const int64_t nsteps = std::max<int64_t>(n_moments / 2, 1);
  std::vector<double> acc((size_t)n_moments, 0.0), self((size_t)nsteps + 1), cross((size_t)nsteps);
  for (int64_t p = 0; p < n_probes; ++p) {
    launch_fill_rng(MB_PREC_F64, op->Du, op->Dd, seed, (uint32_t)(1 + p), 1, probe.p, st);
    const double nrm = kr.load(probe.p, MB_ORDER_TENSOR, v0.r);
    QRef* prev = &v0.r;
    QRef* cur = &v1.r;
    QRef* nxt = &v2.r;
    const double mu0 = nrm * nrm;
    const auto first = kr.apply_affine(*cur, *prev, 1.0 / a, b, 0.0, nullptr);
    cross[0] = first.first;
    self[1] = first.second;
    for (int64_t s = 1; s < nsteps; ++s) {
      const auto r = kr.apply_affine(*nxt, *cur, 2.0 / a, b, -1.0, prev);
      cross[(size_t)s] = r.first;
      self[(size_t)s + 1] = r.second;
      QRef* old = prev;
      prev = cur;
      cur = nxt;
      nxt = old;
    }
    const double mu1 = cross[0];
    acc[0] += mu0;
    if (n_moments > 1) acc[1] += mu1;
    for (int64_t s = 1; 2 * s < n_moments; ++s) {
      acc[(size_t)(2 * s)] += 2.0 * self[(size_t)s] - mu0;
      if (2 * s + 1 < n_moments) acc[(size_t)(2 * s + 1)] += 2.0 * cross[(size_t)s] - mu1;
    }
  }
  const double norm = 1.0 / ((double)n_probes * (double)n);
  for (int64_t i = 0; i < n_moments; ++i) mu[i] = acc[(size_t)i] * norm;
}

void q_evolve(mb_op_s* op, const void* psi0, int order, double t, int64_t krylov_steps,
              int imaginary, void* out) {
  cudaStream_t st = 0;
  QKrylov kr(op, st);
  const int64_t n = op->dim;
  QVec b(n), vp(n), vc(n), w(n);
  const double psi_norm = kr.load(psi0, order, b.r);
  if (psi_norm <= kTol) {
    if (out != psi0) MB_CUDA(cudaMemcpy(out, psi0, sizeof(double2) * (size_t)n, cudaMemcpyDeviceToDevice));
    return;
  }
  int64_t k = krylov_steps <= 0 ? 30 : krylov_steps;
  if (k > n) k = n;
  std::vector<double> alphas, betas;
  const int64_t m = kr.pass_one(b.r, psi_norm, k, 1.0, alphas, betas, false, 0.0, 0, &vp.r,
                                &vc.r, &w.r, true);
  std::vector<double> d(alphas), z, e(betas);
  e.resize((size_t)std::max<int64_t>(m - 1, 0));
  MB_REQUIRE(tridiag_eig((int)m, d, e, &z), MB_ERR_EIG_FAILED,
             "Eigenvalue decomposition of T_k failed");
  std::vector<std::complex<double>> y((size_t)m);
  for (int64_t i = 0; i < m; ++i) {
    std::complex<double> s = 0.0;
    for (int64_t j = 0; j < m; ++j) {
      const std::complex<double> ex =
          imaginary ? std::complex<double>(std::exp(-t * d[(size_t)j]), 0.0)
                    : std::exp(std::complex<double>(0.0, -t * d[(size_t)j]));
      s += z[(size_t)j * m + i] * ex * z[(size_t)j * m + 0];
    }
    y[(size_t)i] = s * psi_norm;
  }
  QVec x(n);
  if (m <= (int64_t)kr.kept.size()) kr.combine_kept(m, y, x.r);
  else kr.pass_two(b.r, psi_norm, m, 1.0, alphas, betas, y, x.r, &vp.r, &vc.r, &w.r);
  kr.store(x.r, order, out);
}

}  // namespace mb

using namespace mb;

extern "C" {

int mb_q64_from_f64(mb_op_t op, const void* x_dev, int order, void* xq_dev, int* exponent,
                    void* stream) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && xq_dev && exponent, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(op->precision == MB_PREC_Q64, MB_ERR_INVALID_ARG, "operator is not MB_PREC_Q64");
    MB_REQUIRE(order == MB_ORDER_REFERENCE || order == MB_ORDER_TENSOR, MB_ERR_INVALID_ARG,
               "bad order");
    cudaStream_t st = (cudaStream_t)stream;
    int32_t* perm = order == MB_ORDER_REFERENCE ? op_perm(op) : nullptr;
    QBuf ints(4 * sizeof(int));
    launch_f64_to_q(op->dim, x_dev, perm, op->q_qbits, (int*)ints.p, xq_dev, st);
    int h[2];
    MB_CUDA(cudaMemcpyAsync(h, ints.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
    *exponent = h[1];
  });
}

int mb_q64_to_f64(mb_op_t op, const void* xq_dev, int exponent, int order, void* x_dev,
                  void* stream) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && xq_dev, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(order == MB_ORDER_REFERENCE || order == MB_ORDER_TENSOR, MB_ERR_INVALID_ARG,
               "bad order");
    cudaStream_t st = (cudaStream_t)stream;
    int32_t* iperm = order == MB_ORDER_REFERENCE ? op_iperm(op) : nullptr;
    QBuf e(sizeof(int));
    MB_CUDA(cudaMemcpyAsync(e.p, &exponent, sizeof(int), cudaMemcpyHostToDevice, st));
    launch_q_to_f64(op->dim, xq_dev, iperm, (const int*)e.p, x_dev, st);
    MB_CUDA(cudaStreamSynchronize(st));
  });
}

int mb_op_apply_q64(mb_op_t op, const void* xq_dev, int x_exponent, void* yq_dev,
                    int* y_exponent, void* stream) {
  return guard([&] {
    MB_REQUIRE(op && xq_dev && yq_dev && y_exponent, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(op->precision == MB_PREC_Q64, MB_ERR_INVALID_ARG, "operator is not MB_PREC_Q64");
    MB_REQUIRE(xq_dev != yq_dev, MB_ERR_INVALID_ARG, "x and y must not overlap");
    cudaStream_t st = (cudaStream_t)stream;
    auto& s = qscratch_for(op, st);
    QParams p{};
    q_plan(&p, plan_input(op, 1.0, 0.0, 0.0, x_exponent, x_exponent, false));
    // a plan per call: the parameter block lives in per-stream scratch, and
    // the copy is ordered before the kernel on the same stream.
    MB_CUDA(cudaMemcpyAsync(s.prm, &p, sizeof(QParams), cudaMemcpyHostToDevice, st));
    q_apply_whole(op, xq_dev, yq_dev, nullptr, (const QParams*)s.prm, nullptr, nullptr, 0, st);
    *y_exponent = p.ey;
  });
}

int mb_q64_mantissa_bits(mb_op_t op, int* bits) {
  return guard([&] {
    MB_REQUIRE(op && bits, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(op->precision == MB_PREC_Q64, MB_ERR_INVALID_ARG, "operator is not MB_PREC_Q64");
    *bits = op->q_qbits;
  });
}

}  // extern "C"
