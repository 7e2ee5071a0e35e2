// Operator handle and the device-resident Krylov drivers behind the C ABI.
//
// Every solver keeps its vectors on the device in tensor order and in the
// operator's precision; only alpha/beta scalars (and the small tridiagonal
// problems) touch the host.  Reference-order arguments are permuted on the
// device at entry and exit.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "mb_internal.h"
#include "mb_q64.h"

namespace mb {

// Q64 hooks (mb_q64_ops.cu)
void q_op_prepare(mb_op_s* op, const mb_model_s* m, const HopTable& tu, const HopTable& td);
void q_op_release(mb_op_s* op);
void q_op_prepare_csr(mb_op_s* op, int64_t max_row_entries, double diag_min, double diag_max,
                      double off);
void q_apply_host_reference(mb_op_s* op, const mb_op_s::HostLane& lane, const void* x_host,
                            const void* x_mapped, void* y_host, void* x_stage, void* y_stage);
int q_apply_grid(const OpView& v);
void q_apply_affine(mb_op_s* op, const void* x, void* y, double scale, double shift, double beta,
                    const void* z, int order, cudaStream_t st);
void q_eigenpair(mb_op_s* op, int64_t k, const void* seed, int order, const mb_lanczos_opts* opts,
                 double sign, double* e_out, void* vec, int64_t* steps_out);
void q_evolve(mb_op_s* op, const void* psi0, int order, double t, int64_t krylov_steps,
              int imaginary, void* out);
void q_kpm_dos_moments(mb_op_s* op, int64_t n_moments, int64_t n_probes, uint64_t seed, double a,
                       double b, double* mu);
int32_t* op_perm(mb_op_s* op);

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  explicit DevBuf(size_t b) : bytes(b) {
    if (b) MB_CUDA(cudaMalloc(&p, b));
  }
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes) { o.p = nullptr; o.bytes = 0; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    std::swap(p, o.p);
    std::swap(bytes, o.bytes);
    return *this;
  }
};

template <typename T>
T* upload(mb_op_s* op, const std::vector<T>& h) {
  if (h.empty()) return nullptr;
  void* p = nullptr;
  MB_CUDA(cudaMalloc(&p, sizeof(T) * h.size()));
  op->allocations.push_back(p);
  MB_CUDA(cudaMemcpy(p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
  return (T*)p;
}

int g_binom_uploaded_dev = -1;
std::mutex g_binom_mu;

void ensure_binomials() {
  int dev = 0;
  MB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_binom_mu);
  if (g_binom_uploaded_dev != dev) {
    upload_binomials(0);
    MB_CUDA(cudaStreamSynchronize(0));
    g_binom_uploaded_dev = dev;
  }
}

void require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  MB_REQUIRE(e == cudaSuccess && n > 0, MB_ERR_NO_DEVICE, "no CUDA device available");
}

// Reduction helper: partials -> device result -> host (pinned) values.
struct Reducer {
  DevBuf partials, out;
  double* host = nullptr;
  int cap_blocks, cap_comp;
  Reducer(int blocks, int comps) : partials(sizeof(double) * (size_t)blocks * comps),
                                   out(sizeof(double) * (size_t)comps), cap_blocks(blocks),
                                   cap_comp(comps) {
    MB_CUDA(cudaMallocHost(&host, sizeof(double) * (size_t)comps));
  }
  ~Reducer() {
    if (host) cudaFreeHost(host);
  }
  double* p() { return (double*)partials.p; }
  // Reduce `nblocks` x `ncomp` partials and copy to host; waits on st.
  const double* fetch(int nblocks, int ncomp, cudaStream_t st) {
    launch_reduce(p(), nblocks, ncomp, (double*)out.p, st);
    MB_CUDA(cudaMemcpyAsync(host, out.p, sizeof(double) * ncomp, cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
    return host;
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// Operator construction.
// ---------------------------------------------------------------------------
static void build_op(mb_op_s* op, const mb_basis_s* b, const mb_model_s* m) {
  MB_CUDA(cudaGetDevice(&op->device));
  op->L = b->L;
  op->n_up = b->n_up;
  op->n_down = b->n_down;
  op->Du = b->up.D;
  op->Dd = b->down.D;
  op->dim = b->dim;
  op->t = m->t;
  op->u = m->u;
  op->tune_key = "lattice";
  for (int64_t d : m->dims) op->tune_key += "_" + std::to_string(d);
  op->tune_key += " n" + std::to_string(b->n_up) + "+" + std::to_string(b->n_down) + " prec" +
                  std::to_string(op->precision);
  const HopTable tu = build_hop_table(b->up, *m);
  const bool same = b->n_up == b->n_down;
  HopTable td_store;
  if (!same) td_store = build_hop_table(b->down, *m);
  const HopTable& td = same ? tu : td_store;
  OpView& v = op->view;
  v.Du = op->Du;
  v.Dd = op->Dd;
  v.dim = op->dim;
  v.L = op->L;
  v.t = m->t;
  v.up_mask = upload(op, b->up.masks);
  v.up_off = upload(op, tu.off);
  v.up_ent = upload(op, tu.ent.empty() ? std::vector<uint32_t>{0u} : tu.ent);
  if (same) {
    v.dn_mask = v.up_mask;
    v.dn_off = v.up_off;
    v.dn_ent = v.up_ent;
  } else {
    v.dn_mask = upload(op, b->down.masks);
    v.dn_off = upload(op, td.off);
    v.dn_ent = upload(op, td.ent.empty() ? std::vector<uint32_t>{0u} : td.ent);
  }
  v.max_up_degree = tu.max_degree;
  v.max_dn_degree = td.max_degree;
  fill_fused_tables(v, tu, td, op->Du, op->Dd, [op](const void* h, size_t bytes) -> const void* {
    void* p = nullptr;
    MB_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 16)));
    op->allocations.push_back(p);
    if (bytes) MB_CUDA(cudaMemcpy(p, h, bytes, cudaMemcpyHostToDevice));
    return p;
  });
  const std::vector<double> uf = u_fold_table(m->u, m->has_u, op->L);
  v.u_fold = upload(op, uf);
  v.u_fold_f = upload(op, std::vector<float>(uf.begin(), uf.end()));
  if (tu.has_self) {
    v.self_up = upload(op, tu.self_energy);
    v.self_up_f = upload(op, std::vector<float>(tu.self_energy.begin(), tu.self_energy.end()));
  }
  if (td.has_self) {
    if (same) {
      v.self_dn = v.self_up;
      v.self_dn_f = v.self_up_f;
    } else {
      v.self_dn = upload(op, td.self_energy);
      v.self_dn_f = upload(op, std::vector<float>(td.self_energy.begin(), td.self_energy.end()));
    }
  }
  ensure_binomials();
  if (op->precision == MB_PREC_Q64) q_op_prepare(op, m, tu, td);
}

// One (N_up, N_down) block of an all-spin-projection basis as a basis.
static mb_basis_s sector_of(const mb_basis_s* b, size_t blk) {
  mb_basis_s s;
  s.L = b->L;
  s.n_up = b->sz_nup[blk];
  s.n_down = b->particles - s.n_up;
  s.up = make_spin_sector(s.L, s.n_up);
  s.down = make_spin_sector(s.L, s.n_down);
  s.dim = s.up.D * s.down.D;
  return s;
}

// Reference indices (all spin projections) of one block's tensor order.
static std::vector<int32_t> block_perm(const mb_basis_s& s) {
  std::vector<int32_t> p((size_t)s.dim);
  const Binom& B = binom_table();
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < s.dim; ++i)
    p[(size_t)i] = (int32_t)reference_rank_all(B, s.up.masks[(size_t)(i / s.down.D)],
                                               s.down.masks[(size_t)(i % s.down.D)], s.L);
  return p;
}

static void free_op_memory(mb_op_s* op) {
  for (auto& lane : op->host_lanes) {
    if (lane->comp) cudaStreamDestroy(lane->comp);
    if (lane->copy) cudaStreamDestroy(lane->copy);
    for (int b = 0; b < 2; ++b) {
      if (lane->bounce[b]) cudaFreeHost(lane->bounce[b]);
      if (lane->bev[b]) cudaEventDestroy(lane->bev[b]);
    }
  }
  op->host_lanes.clear();
  op->host_idle.clear();
  for (auto& kv : op->scratch) {
    for (void* p : {kv.second.a, kv.second.b, kv.second.hx, kv.second.hy})
      if (p) cudaFree(p);
  }
  op->scratch.clear();
  for (auto& sub : op->subs) free_op_memory(sub.get());
  for (void* p : op->allocations) cudaFree(p);
  op->allocations.clear();
}

// The block-diagonal operator of an all-spin-projection basis: one lattice
// operator per (N_up, N_down) block on consecutive slices, the permutation
// to the reference order (reference_rank_all) computed here.
static void build_all_sz(mb_op_s* op, const mb_basis_s* b, const mb_model_s* m) {
  MB_REQUIRE(!m->momentum && !m->current, MB_ERR_INVALID_ARG,
             "an all-spin-projection basis takes the real-space model");
  MB_REQUIRE(op->precision != MB_PREC_Q64, MB_ERR_INVALID_ARG,
             "all-spin-projection operators take MB_PREC_F64 or MB_PREC_F32");
  MB_CUDA(cudaGetDevice(&op->device));
  op->L = b->L;
  op->n_up = -1;
  op->n_down = -1;
  op->dim = b->dim;
  op->Du = b->dim;
  op->Dd = 1;
  op->t = m->t;
  op->u = m->u;
  std::vector<int32_t> perm((size_t)b->dim);
  for (size_t blk = 0; blk < b->sz_nup.size(); ++blk) {
    const mb_basis_s s = sector_of(b, blk);
    auto sub = std::make_unique<mb_op_s>();
    sub->precision = op->precision;
    try {
      build_op(sub.get(), &s, m);
    } catch (...) {
      free_op_memory(sub.get());
      throw;
    }
    op->sub_views.push_back(sub->view);
    op->subs.push_back(std::move(sub));
    const std::vector<int32_t> p = block_perm(s);
    std::copy(p.begin(), p.end(), perm.begin() + b->sz_off[blk]);
  }
  op->sub_offsets = b->sz_off;
  OpView& v = op->view;
  v.Du = b->dim;
  v.Dd = 1;
  v.dim = b->dim;
  v.L = b->L;
  v.n_blocks = (int)op->subs.size();
  v.sub = op->sub_views.data();
  v.sub_off = op->sub_offsets.data();
  op->perm = upload(op, perm.empty() ? std::vector<int32_t>{0} : perm);
}

// A momentum-sector operator: the sector's Hamiltonian built on the device
// in signed-column form (row_ptr, column | sign << 31, diagonal, U/N); its
// rows are the sector's reference order.
struct MomBuild {
  int64_t n = 0, nnz = 0;
  std::vector<int64_t> row_ptr;
  int32_t* col = nullptr;  // device
  double* diag = nullptr;  // device
};

static void build_momentum(mb_op_s* op, const mb_basis_s* b, const mb_model_s* m, MomBuild& out) {
  MB_REQUIRE(b->momentum() && m->momentum, MB_ERR_INVALID_ARG,
             "a momentum-sector basis needs the momentum-space model (and the reverse)");
  MB_REQUIRE(b->kdims == m->dims, MB_ERR_DIM_MISMATCH, "basis and model lattices differ");
  const int L = b->L;
  std::vector<uint8_t> kadd((size_t)L * L), ksub((size_t)L * L);
  for (int k = 0; k < L; ++k)
    for (int q = 0; q < L; ++q) {
      kadd[(size_t)k * L + q] = (uint8_t)momentum_add(k, q, +1, b->kdims);
      ksub[(size_t)k * L + q] = (uint8_t)momentum_add(k, q, -1, b->kdims);
    }
  MomTables t{};
  t.n = b->dim;
  t.L = L;
  t.n_up = b->n_up;
  t.n_down = b->n_down;
  t.up = upload(op, b->kup.empty() ? std::vector<uint32_t>{0u} : b->kup);
  t.dn = upload(op, b->kdown.empty() ? std::vector<uint32_t>{0u} : b->kdown);
  t.full = upload(op, b->kfull.empty() ? std::vector<int64_t>{0} : b->kfull);
  t.eps = upload(op, m->eps);
  t.kadd = upload(op, kadd);
  t.ksub = upload(op, ksub);
  t.u_over_n = m->u_over_n;
  ensure_binomials();
  cudaStream_t st = 0;
  out.n = b->dim;
  out.row_ptr.assign((size_t)out.n + 1, 0);
  if (out.n == 0) return;
  DevBuf cnt(sizeof(int32_t) * (size_t)out.n);
  void* dg = nullptr;
  MB_CUDA(cudaMalloc(&dg, sizeof(double) * (size_t)out.n));
  op->allocations.push_back(dg);
  out.diag = (double*)dg;
  launch_mom_count(t, (int32_t*)cnt.p, out.diag, st);
  std::vector<int32_t> hc((size_t)out.n);
  MB_CUDA(cudaMemcpy(hc.data(), cnt.p, sizeof(int32_t) * (size_t)out.n, cudaMemcpyDeviceToHost));
  for (int64_t i = 0; i < out.n; ++i) out.row_ptr[(size_t)i + 1] = out.row_ptr[(size_t)i] + hc[(size_t)i];
  out.nnz = out.row_ptr[(size_t)out.n];
  const int64_t* drp = upload(op, out.row_ptr);
  void* dc = nullptr;
  MB_CUDA(cudaMalloc(&dc, sizeof(int32_t) * (size_t)std::max<int64_t>(out.nnz, 1)));
  op->allocations.push_back(dc);
  out.col = (int32_t*)dc;
  launch_mom_fill(t, drp, out.col, st);
  MB_CUDA(cudaStreamSynchronize(st));
  OpView& v = op->view;
  v.csr_row = drp;
  v.csr_col = out.col;
  v.csr_val = nullptr;
  v.csr_diag = out.diag;
  v.csr_off = m->u_over_n;
}

// A momentum-sector operator: natural (sector reference) order, signed-column
// CSR on the device.
static void build_momentum_op(mb_op_s* op, const mb_basis_s* basis, const mb_model_s* model) {
  MB_CUDA(cudaGetDevice(&op->device));
  op->L = basis->L;
  op->n_up = basis->n_up;
  op->n_down = basis->n_down;
  op->Du = basis->dim;
  op->Dd = 1;
  op->dim = basis->dim;
  op->t = model->t;
  op->u = model->u;
  op->natural_order = true;
  op->view.Du = basis->dim;
  op->view.Dd = 1;
  op->view.dim = basis->dim;
  op->view.L = basis->L;
  MomBuild mbld;
  build_momentum(op, basis, model, mbld);
  // the apply autotuner's cache key: the sector (lattice, fillings, momentum)
  op->tune_key = "momentum";
  for (int64_t d : model->dims) op->tune_key += "_" + std::to_string(d);
  op->tune_key += " n" + std::to_string(basis->n_up) + "+" + std::to_string(basis->n_down) + " K";
  for (int64_t k : basis->kvec) op->tune_key += "_" + std::to_string(k);
  op->tune_key += " prec" + std::to_string(op->precision);
  if (op->precision == MB_PREC_Q64) {
    // the block-floating-point plan: the longest row bounds the hop sums, the
    // diagonal's range bounds its coefficients
    int64_t longest = 0;
    for (int64_t i = 0; i < mbld.n; ++i)
      longest = std::max(longest, mbld.row_ptr[(size_t)i + 1] - mbld.row_ptr[(size_t)i]);
    std::vector<double> d((size_t)mbld.n);
    if (mbld.n)
      MB_CUDA(cudaMemcpy(d.data(), mbld.diag, sizeof(double) * (size_t)mbld.n, cudaMemcpyDeviceToHost));
    const auto mm = std::minmax_element(d.begin(), d.end());
    q_op_prepare_csr(op, longest, d.empty() ? 0.0 : *mm.first, d.empty() ? 0.0 : *mm.second,
                     model->u_over_n);
  }
}

// The total-momentum sectors of a whole (N_up, N_down) basis on the model's
// lattice, K in flat order (first dimension fastest); empty sectors skipped.
static std::vector<std::unique_ptr<mb_basis_s>> momentum_sectors(const mb_basis_s* b,
                                                                 const mb_model_s* m) {
  const int ndim = (int)m->dims.size();
  std::vector<std::unique_ptr<mb_basis_s>> out;
  for (int64_t K = 0; K < b->L; ++K) {
    int64_t kv[3] = {0, 0, 0}, rest = K;
    for (int d = 0; d < ndim; ++d) {
      kv[d] = rest % m->dims[(size_t)d];
      rest /= m->dims[(size_t)d];
    }
    mb_basis_t h = nullptr;
    const int rc = mb_basis_create_momentum(m->dims.data(), ndim, b->n_up + b->n_down,
                                            b->n_up - b->n_down, kv, &h);
    if (rc) throw Error(rc, mb_last_error());
    std::unique_ptr<mb_basis_s> sec(h);
    if (sec->dim > 0) out.push_back(std::move(sec));
  }
  return out;
}

// The momentum-space model on a whole (N_up, N_down) basis: the matrix the
// reference's HubbardMomentumFactorized applies
// (src/numerics/hubbard_momentum_factorized.h:32-249), H = t sum eps(k) n_k +
// (U/N) sum_q rho_{q,up} rho_{-q,down}.  H conserves the total momentum, so
// the operator is block diagonal: one sector operator per K on consecutive
// slices, and the permutation to the whole basis's reference order is each
// sector's list of full-basis reference ranks.
static void build_momentum_all(mb_op_s* op, const mb_basis_s* b, const mb_model_s* m) {
  MB_REQUIRE(op->precision != MB_PREC_Q64, MB_ERR_INVALID_ARG,
             "momentum-space operators take MB_PREC_F64 or MB_PREC_F32");
  MB_CUDA(cudaGetDevice(&op->device));
  op->L = b->L;
  op->n_up = b->n_up;
  op->n_down = b->n_down;
  op->dim = b->dim;
  op->Du = b->dim;
  op->Dd = 1;
  op->t = m->t;
  op->u = m->u;
  std::vector<int32_t> perm((size_t)b->dim);
  int64_t off = 0;
  for (auto& sec : momentum_sectors(b, m)) {
    auto sub = std::make_unique<mb_op_s>();
    sub->precision = op->precision;
    try {
      build_momentum_op(sub.get(), sec.get(), m);
    } catch (...) {
      free_op_memory(sub.get());
      throw;
    }
    op->sub_views.push_back(sub->view);
    op->subs.push_back(std::move(sub));
    op->sub_offsets.push_back(off);
    for (int64_t i = 0; i < sec->dim; ++i) perm[(size_t)(off + i)] = (int32_t)sec->kfull[(size_t)i];
    off += sec->dim;
  }
  MB_REQUIRE(off == b->dim, MB_ERR_INVALID_ARG, "momentum sectors do not cover the basis");
  OpView& v = op->view;
  v.Du = b->dim;
  v.Dd = 1;
  v.dim = b->dim;
  v.L = b->L;
  v.n_blocks = (int)op->subs.size();
  v.sub = op->sub_views.data();
  v.sub_off = op->sub_offsets.data();
  op->perm = upload(op, perm.empty() ? std::vector<int32_t>{0} : perm);
}

// Per-stream scratch vectors: nvec = 1 gives a, 2 gives a and b; staging
// adds the host-buffer staging pair hx, hy.  Each is allocated on first use.
static mb_op_s::Scratch& scratch_for(mb_op_s* op, cudaStream_t st, int nvec, bool staging = false) {
  std::lock_guard<std::mutex> lk(op->mu);
  auto& s = op->scratch[st];
  const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
  if (nvec >= 1 && !s.a) {
    MB_CUDA(cudaMalloc(&s.a, vb));
  }
  if (nvec >= 2 && !s.b) {
    MB_CUDA(cudaMalloc(&s.b, vb));
  }
  if (staging && !s.hx) {
    MB_CUDA(cudaMalloc(&s.hx, vb));
    MB_CUDA(cudaMalloc(&s.hy, vb));
  }
  return s;
}

static void ensure_perm(mb_op_s* op) {
  std::lock_guard<std::mutex> lk(op->mu);
  if (op->perm) return;
  void* p = nullptr;
  MB_CUDA(cudaMalloc(&p, sizeof(int32_t) * (size_t)op->dim));
  op->allocations.push_back(p);
  launch_perm(op->view, (int32_t*)p, 0);
  MB_CUDA(cudaStreamSynchronize(0));
  op->perm = (int32_t*)p;
}

// the permutation tensor -> reference order (nullptr: the operator's own index
// is the reference order)
int32_t* op_perm(mb_op_s* op) {
  if (op->natural_order) return nullptr;
  ensure_perm(op);
  return op->perm;
}

int32_t* op_iperm(mb_op_s* op) {
  if (op->natural_order) return nullptr;
  ensure_perm(op);
  std::lock_guard<std::mutex> lk(op->mu);
  if (!op->iperm) {
    void* p = nullptr;
    MB_CUDA(cudaMalloc(&p, sizeof(int32_t) * (size_t)op->dim));
    op->allocations.push_back(p);
    launch_invert_perm(op->dim, op->perm, (int32_t*)p, 0);
    MB_CUDA(cudaStreamSynchronize(0));
    op->iperm = (int32_t*)p;
  }
  return op->iperm;
}

static void to_tensor(mb_op_s* op, const void* src, void* dst, int order, cudaStream_t st) {
  if (order == MB_ORDER_TENSOR || op->natural_order) {
    if (src != dst)
      MB_CUDA(cudaMemcpyAsync(dst, src, elem_bytes(op->precision) * (size_t)op->dim,
                              cudaMemcpyDeviceToDevice, st));
    return;
  }
  ensure_perm(op);
  launch_gather(op->precision, op->dim, op->perm, src, dst, st);
}

static void from_tensor(mb_op_s* op, const void* src, void* dst, int order, cudaStream_t st) {
  if (order == MB_ORDER_TENSOR || op->natural_order) {
    if (src != dst)
      MB_CUDA(cudaMemcpyAsync(dst, src, elem_bytes(op->precision) * (size_t)op->dim,
                              cudaMemcpyDeviceToDevice, st));
    return;
  }
  // y_ref[i] = y_tensor[iperm[i]]: coalesced writes, random reads
  launch_gather(op->precision, op->dim, op_iperm(op), src, dst, st);
}

// The row groups of the pipelined host-buffer applies.  Rows are ordered by
// the first reference index among their states and cut into at most
// kHostGroups groups; once groups 0..g are applied, every reference index
// below the first one of a later group's rows is final, so that prefix can go
// back while the later groups run.  Group sizes are whole multiples of the
// apply's grid (each CTA takes one row per wave), so the groups together run
// no more waves than one launch over every row.  Within a group the rows keep
// the row schedule's order (its L2 locality).  Built on the first host-buffer
// call.
constexpr int64_t kHostGroups = 8;

void ensure_host_groups(mb_op_s* op) {
  {
    std::lock_guard<std::mutex> lk(op->mu);
    if (op->host_sched) return;
  }
  const int32_t* perm = op_perm(op);
  const int64_t Du = op->Du;
  std::vector<int32_t> first((size_t)Du), sched((size_t)Du);
  {
    DevBuf d_first(sizeof(int32_t) * (size_t)Du);
    launch_row_first(Du, op->Dd, perm, (int32_t*)d_first.p, 0);
    MB_CUDA(cudaMemcpy(first.data(), d_first.p, sizeof(int32_t) * (size_t)Du,
                       cudaMemcpyDeviceToHost));
  }
  if (op->view.row_sched) {
    MB_CUDA(cudaMemcpy(sched.data(), op->view.row_sched, sizeof(int32_t) * (size_t)Du,
                       cudaMemcpyDeviceToHost));
  } else {
    for (int64_t r = 0; r < Du; ++r) sched[(size_t)r] = (int32_t)r;
  }
  std::vector<int64_t> pos((size_t)Du);
  for (int64_t i = 0; i < Du; ++i) pos[(size_t)sched[(size_t)i]] = i;
  std::vector<int32_t> order((size_t)Du);
  for (int64_t r = 0; r < Du; ++r) order[(size_t)r] = (int32_t)r;
  std::sort(order.begin(), order.end(),
            [&](int32_t a, int32_t b) { return first[(size_t)a] < first[(size_t)b]; });
  const int64_t wave =
      op->precision == MB_PREC_Q64 ? q_apply_grid(op->view) : apply_grid(op->view, op->precision);
  const int64_t waves = (Du + wave - 1) / wave;
  const int64_t G = std::min<int64_t>(kHostGroups, waves);
  std::vector<int64_t> row0((size_t)G + 1), ready((size_t)G);
  for (int64_t g = 0; g <= G; ++g)
    row0[(size_t)g] = std::min<int64_t>(Du, (g * waves + G / 2) / G * wave);
  row0[(size_t)G] = Du;
  for (int64_t g = 0; g < G; ++g)
    ready[(size_t)g] = g + 1 < G ? (int64_t)first[(size_t)order[(size_t)row0[(size_t)g + 1]]]
                                 : op->dim;
  for (int64_t g = 0; g < G; ++g)
    std::sort(order.begin() + row0[(size_t)g], order.begin() + row0[(size_t)g + 1],
              [&](int32_t a, int32_t b) { return pos[(size_t)a] < pos[(size_t)b]; });
  // callers hold host_mu, so no other thread builds the groups meanwhile
  std::lock_guard<std::mutex> lk(op->mu);
  void* p = nullptr;
  MB_CUDA(cudaMalloc(&p, sizeof(int32_t) * (size_t)std::max<int64_t>(Du, 1)));
  op->allocations.push_back(p);
  MB_CUDA(cudaMemcpy(p, order.data(), sizeof(int32_t) * (size_t)Du, cudaMemcpyHostToDevice));
  op->host_row0 = std::move(row0);
  op->host_ready = std::move(ready);
  op->host_sched = (int32_t*)p;
}

bool host_pinned(const void* p) {
  cudaPointerAttributes at{};
  const bool pinned = cudaPointerGetAttributes(&at, p) == cudaSuccess &&
                      at.type == cudaMemoryTypeHost && at.devicePointer != nullptr;
  if (!pinned) cudaGetLastError();  // clear a failed query on pageable memory
  return pinned;
}

constexpr size_t kBounceBytes = size_t(16) << 20;

static void lane_bounce(const mb_op_s::HostLane& lane_c) {
  auto& lane = const_cast<mb_op_s::HostLane&>(lane_c);  // the calling thread owns the lane
  for (int b = 0; b < 2; ++b) {
    if (!lane.bounce[b]) MB_CUDA(cudaHostAlloc(&lane.bounce[b], kBounceBytes, cudaHostAllocDefault));
    if (!lane.bev[b]) MB_CUDA(cudaEventCreateWithFlags(&lane.bev[b], cudaEventDisableTiming));
  }
}

void lane_upload(const mb_op_s::HostLane& lane, void* dst_dev, const void* src_host, size_t bytes,
                 size_t chunk_align,
                 const std::function<void(size_t, size_t, cudaEvent_t)>& on_chunk) {
  if (bytes == 0) return;
  lane_bounce(lane);
  const size_t chunk = kBounceBytes - kBounceBytes % chunk_align;
  size_t off = 0;
  for (int c = 0; off < bytes; ++c) {
    const int b = c & 1;
    const size_t len = std::min(chunk, bytes - off);
    // the buffer's previous transfer (two chunks back) is done before refilling it
    if (c >= 2) MB_CUDA(cudaEventSynchronize(lane.bev[b]));
    std::memcpy(lane.bounce[b], (const char*)src_host + off, len);
    MB_CUDA(cudaMemcpyAsync((char*)dst_dev + off, lane.bounce[b], len, cudaMemcpyHostToDevice,
                            lane.copy));
    MB_CUDA(cudaEventRecord(lane.bev[b], lane.copy));
    on_chunk(off, len, lane.bev[b]);
    off += len;
  }
}

void lane_download(const mb_op_s::HostLane& lane, void* dst_host, const void* src_dev,
                   size_t bytes) {
  if (bytes == 0) return;
  lane_bounce(lane);
  const size_t n = (bytes + kBounceBytes - 1) / kBounceBytes;
  size_t issued = 0, done = 0;
  while (done < n) {
    while (issued < n && issued - done < 2) {
      const int b = (int)(issued & 1);
      const size_t off = issued * kBounceBytes, len = std::min(kBounceBytes, bytes - off);
      MB_CUDA(cudaMemcpyAsync(lane.bounce[b], (const char*)src_dev + off, len,
                              cudaMemcpyDeviceToHost, lane.copy));
      MB_CUDA(cudaEventRecord(lane.bev[b], lane.copy));
      ++issued;
    }
    const int b = (int)(done & 1);
    const size_t off = done * kBounceBytes, len = std::min(kBounceBytes, bytes - off);
    MB_CUDA(cudaEventSynchronize(lane.bev[b]));
    std::memcpy((char*)dst_host + off, lane.bounce[b], len);
    ++done;
  }
}

void host_groups_run(mb_op_s* op, const mb_op_s::HostLane& lane, size_t elem, void* y_host,
                     void* y_stage, const std::function<void(const OpView&)>& apply_rows,
                     const std::function<void(int64_t, int64_t, void*)>& gather) {
  cudaStream_t comp = lane.comp, copy = lane.copy;
  const int64_t G = (int64_t)op->host_ready.size();
  Events ev((int)G);
  int64_t done = 0;
  for (int64_t g = 0; g < G; ++g) {
    OpView v = op->view;
    v.row_sched = op->host_sched + op->host_row0[(size_t)g];
    v.Du = op->host_row0[(size_t)g + 1] - op->host_row0[(size_t)g];
    apply_rows(v);
    const int64_t ready = op->host_ready[(size_t)g];
    if (ready > done) gather(done, ready, (char*)y_stage + elem * (size_t)done);
    MB_CUDA(cudaEventRecord(ev[(int)g], comp));
    done = ready;
  }
  // every compute launch is queued before the first download: a download to
  // pageable memory returns only when it has finished (through the lane's
  // bounce buffers)
  const bool pinned = host_pinned(y_host);
  done = 0;
  for (int64_t g = 0; g < G; ++g) {
    const int64_t ready = op->host_ready[(size_t)g];
    if (ready > done) {
      MB_CUDA(cudaStreamWaitEvent(copy, ev[(int)g], 0));
      if (pinned)
        MB_CUDA(cudaMemcpyAsync((char*)y_host + elem * (size_t)done,
                                (const char*)y_stage + elem * (size_t)done,
                                elem * (size_t)(ready - done), cudaMemcpyDeviceToHost, copy));
      else
        lane_download(lane, (char*)y_host + elem * (size_t)done,
                      (const char*)y_stage + elem * (size_t)done, elem * (size_t)(ready - done));
    }
    done = ready;
  }
  MB_CUDA(cudaStreamSynchronize(copy));
  MB_CUDA(cudaStreamSynchronize(comp));
}

static void check_order(int order) {
  MB_REQUIRE(order == MB_ORDER_REFERENCE || order == MB_ORDER_TENSOR, MB_ERR_INVALID_ARG,
             "order must be MB_ORDER_REFERENCE or MB_ORDER_TENSOR");
}

// y = scale*(H - shift) x + beta z in `order`.
static void apply_affine(mb_op_s* op, const void* x, void* y, double scale, double shift,
                         double beta, const void* z, int order, cudaStream_t st) {
  check_order(order);
  MB_REQUIRE(x && y, MB_ERR_INVALID_ARG, "NULL vector");
  MB_REQUIRE(x != y, MB_ERR_INVALID_ARG, "x and y must not overlap");
  if (beta != 0.0) MB_REQUIRE(z, MB_ERR_INVALID_ARG, "z is NULL with beta != 0");
  if (op->precision == MB_PREC_Q64) {
    q_apply_affine(op, x, y, scale, shift, beta, beta != 0.0 ? z : nullptr, order, st);
    return;
  }
  if (order == MB_ORDER_TENSOR) {
    launch_apply(op->view, op->precision, x, y, scale, shift, beta, beta != 0.0 ? z : nullptr,
                 nullptr, 0, st);
    return;
  }
  auto& s = scratch_for(op, st, 2);
  to_tensor(op, x, s.a, order, st);
  const void* zt = nullptr;
  if (beta != 0.0) {
    // z gathered into y's slot would clobber z when z == y; use b then swap roles.
    to_tensor(op, z, s.b, order, st);
    zt = s.b;
  }
  // In-place on s.b when z is used: each element reads z[i] before writing y[i].
  launch_apply(op->view, op->precision, s.a, s.b, scale, shift, beta, zt, nullptr, 0, st);
  from_tensor(op, s.b, y, order, st);
}

// ---------------------------------------------------------------------------
// Lanczos (src/numerics/lanczos.h) on scale*H, device-resident.
// ---------------------------------------------------------------------------
struct Krylov {
  mb_op_s* op;
  cudaStream_t st;
  int64_t n;
  int prec;
  size_t vb;
  DevBuf v_prev, v_curr, w, basis, coef;
  int basis_prec = MB_PREC_F64;
  int64_t basis_cap = 0;
  Reducer red;
  int grid_apply, grid_blas;

  Krylov(mb_op_s* o, cudaStream_t s)
      : op(o), st(s), n(o->dim), prec(o->precision), vb(elem_bytes(o->precision) * (size_t)o->dim),
        v_prev(vb), v_curr(vb), w(vb),
        red(std::max(std::max(apply_grid(o->view, o->precision), blas_grid(o->dim)), 1024) , 2 * 1024 + 8),
        grid_apply(apply_grid(o->view, o->precision)), grid_blas(blas_grid(o->dim)) {}

  double norm_of(const void* x) {
    launch_dot(prec, n, x, x, red.p(), st);
    const double* h = red.fetch(grid_blas, 3, st);
    return std::sqrt(h[2]);
  }

  void reserve_basis(int64_t k, int want_prec) {
    size_t free_b = 0, total_b = 0;
    MB_CUDA(cudaMemGetInfo(&free_b, &total_b));
    int p = want_prec;
    const size_t need64 = (size_t)k * 16 * (size_t)n, need32 = (size_t)k * 8 * (size_t)n;
    if (p < 0) p = (need64 + (size_t)(1u << 30) < free_b) ? MB_PREC_F64 : MB_PREC_F32;
    if (prec == MB_PREC_F32) p = MB_PREC_F32;
    const size_t need = p == MB_PREC_F64 ? need64 : need32;
    MB_REQUIRE(need + (size_t)(256u << 20) < free_b, MB_ERR_OOM,
               "Krylov basis for full re-orthogonalisation does not fit in device memory");
    basis = DevBuf(need);
    basis_prec = p;
    basis_cap = k;
    coef = DevBuf(sizeof(double) * 2 * (size_t)std::max<int64_t>(k, 1));
  }

  void* basis_col(int64_t j) {
    return (char*)basis.p + elem_bytes(basis_prec) * (size_t)n * (size_t)j;
  }

  // Kept Lanczos vectors: a run without re-orthogonalisation that needs its
  // Ritz vector keeps the vectors pass one applies (u_0, u_1, ..., in chunks
  // of kKeepChunk) while a tenth of the device memory stays free, and sums
  // the Ritz vector from them instead of replaying the recurrence; pass two
  // remains for a run whose Ritz vector needs more vectors than it kept.
  static constexpr int64_t kKeepChunk = 16;
  std::vector<DevBuf> keep;
  DevBuf keep_coef;
  int64_t kept = 0;  // u_0 .. u_(kept-1) are kept

  void* keep_col(int64_t j) {
    return (char*)keep[(size_t)(j / kKeepChunk)].p + vb * (size_t)(j % kKeepChunk);
  }

  bool keep_room(int64_t j) {
    if ((size_t)(j / kKeepChunk) < keep.size()) return true;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    const size_t need = vb * (size_t)kKeepChunk;
    if (need + total_b / 10 > free_b) return false;
    try {
      keep.emplace_back(need);
    } catch (const Error&) {
      cudaGetLastError();
      return false;
    }
    return true;
  }

  // x = sum_(j < m) y_j v_j from the kept vectors, v_j = u_j / s_j (s_j =
  // beta_(j-1) for pass one's unnormalised FP32 vectors, 1 otherwise).
  void combine_kept(int64_t m, const std::vector<double>& betas,
                    const std::vector<std::complex<double>>& y, void* x) {
    const bool fold = prec == MB_PREC_F32;
    std::vector<double> c(2 * (size_t)m);
    for (int64_t j = 0; j < m; ++j) {
      const double sj = fold && j > 0 ? betas[(size_t)j - 1] : 1.0;
      c[2 * (size_t)j] = -y[(size_t)j].real() / sj;  // multi_axpy subtracts
      c[2 * (size_t)j + 1] = -y[(size_t)j].imag() / sj;
    }
    if (keep_coef.bytes < sizeof(double) * c.size()) keep_coef = DevBuf(sizeof(double) * c.size());
    MB_CUDA(cudaMemcpyAsync(keep_coef.p, c.data(), sizeof(double) * c.size(),
                            cudaMemcpyHostToDevice, st));
    MB_CUDA(cudaMemsetAsync(x, 0, vb, st));
    for (int64_t j0 = 0; j0 < m; j0 += kKeepChunk) {
      const int cnt = (int)std::min<int64_t>(kKeepChunk, m - j0);
      launch_multi_axpy(prec, prec, n, keep_col(j0), n, cnt, (const double*)keep_coef.p + 2 * j0,
                        x, red.p(), st);
    }
  }

  // Full re-orthogonalisation of w (squared norm nrm2) against the m stored
  // vectors: classical Gram-Schmidt, w -= V (V^H w), with the DGKS test
  // (Daniel, Gragg, Kaufman and Stewart, Math. Comp. 30 (1976); Parlett's
  // "twice is enough"): a second pass runs only when the first one took w
  // below 1/sqrt(2) of its norm, where cancellation can leave components
  // along V.  A Lanczos vector is already nearly orthogonal to V, so one pass
  // is the rule.  Returns ||w||^2 after the last pass.
  double reorth(int m, double nrm2) {
    for (int pass = 0; pass < 2; ++pass) {
      const double before = nrm2;
      launch_multi_dot(basis_prec, prec, n, basis.p, n, m, w.p, red.p(), st);
      launch_reduce(red.p(), multi_dot_grid(n), 2 * m, (double*)coef.p, st);
      launch_multi_axpy(basis_prec, prec, n, basis.p, n, m, (const double*)coef.p, w.p, red.p(),
                        st);
      nrm2 = red.fetch(grid_blas, 3, st)[1];
      if (nrm2 >= 0.5 * before) break;
    }
    return nrm2;
  }

  // Pass one from b (tensor order, op precision).  Returns steps taken.
  int64_t pass_one(const void* b, int64_t k, double scale, std::vector<double>& alphas,
                   std::vector<double>& betas, double& b_norm, bool reorth, double conv_tol,
                   int check_every, std::vector<double>* ritz_trace = nullptr,
                   bool keep_vectors = false) {
    b_norm = norm_of(b);
    MB_REQUIRE(b_norm > kTol, MB_ERR_ZERO_NORM, "Input vector has zero norm");
    alphas.clear();
    betas.clear();
    if (k == 0) return 0;
    // v_curr = b / ||b||, v_prev = 0
    launch_axpby(prec, n, 1.0 / b_norm, 0.0, b, 0.0, 0.0, v_curr.p, nullptr, 0, st);
    MB_CUDA(cudaMemsetAsync(v_prev.p, 0, vb, st));
    double beta_prev = 0.0;
    int64_t steps = 0;
    double last_ritz = 0.0;
    bool have_ritz = false;
    // FP32 runs without re-orthogonalisation keep their Lanczos vectors
    // unnormalised, u_j = s_j v_j with s_j = beta_(j-1): the next apply and
    // the combination take 1/s_j in their coefficients, so a step is two
    // vector passes (apply, combination) instead of three.  Other runs keep
    // s_j = 1 and normalise as the reference does.
    const bool fold = prec == MB_PREC_F32 && !reorth;
    double s_curr = 1.0, s_prev = 1.0;
    kept = 0;
    for (int64_t it = 0; it < k; ++it) {
      if (reorth) launch_convert(prec, basis_prec, n, v_curr.p, basis_col(it), st);
      if (keep_vectors && kept == it && keep_room(it)) {
        MB_CUDA(cudaMemcpyAsync(keep_col(it), v_curr.p, vb, cudaMemcpyDeviceToDevice, st));
        kept = it + 1;
      }
      // w = scale*H v - beta_prev v_prev ; alpha = Re<v, w>   (lanczos.h:25-33)
      launch_apply(op->view, prec, v_curr.p, w.p, scale / s_curr, 0.0, -beta_prev / s_prev,
                   beta_prev != 0.0 ? v_prev.p : nullptr, red.p(), 1, st);
      const double alpha = red.fetch(grid_apply, 3, st)[0] / s_curr;
      // w -= alpha v ; beta = ||w||                             (lanczos.h:34-36)
      launch_axpby(prec, n, -alpha / s_curr, 0.0, v_curr.p, 1.0, 0.0, w.p, red.p(), 1, st);
      double nrm2 = red.fetch(grid_blas, 3, st)[1];
      if (reorth) nrm2 = this->reorth((int)(it + 1), nrm2);
      const double beta = std::sqrt(nrm2);
      alphas.push_back(alpha);
      steps += 1;
      if (beta <= kTol) break;
      if (it + 1 < k) betas.push_back(beta);
      // v_prev <- v, v <- w / beta                               (lanczos.h:113-121)
      std::swap(v_prev.p, v_curr.p);
      std::swap(v_curr.p, w.p);
      if (fold) {
        s_prev = s_curr;
        s_curr = beta;
      } else {
        launch_axpby(prec, n, 0.0, 0.0, nullptr, 1.0 / beta, 0.0, v_curr.p, nullptr, 0, st);
      }
      beta_prev = beta;
      if (conv_tol > 0.0 && check_every > 0 && (steps % check_every) == 0 && it + 1 < k) {
        std::vector<double> d(alphas), e(betas);
        e.resize(d.size() > 0 ? d.size() - 1 : 0);
        if (tridiag_eig((int)d.size(), d, e, nullptr)) {
          const double ritz = d.back();
          if (ritz_trace) ritz_trace->push_back(ritz);
          if (have_ritz && std::fabs(ritz - last_ritz) <= conv_tol * std::fabs(ritz)) {
            betas.resize(steps > 0 ? steps - 1 : 0);
            break;
          }
          last_ritz = ritz;
          have_ritz = true;
        }
      }
    }
    if ((int64_t)betas.size() > std::max<int64_t>(steps - 1, 0)) betas.resize(steps - 1);
    return steps;
  }

  // Pass two (lanczos.h:177-218): x = sum_j y_j v_j by re-running the
  // recurrence; y complex.  x in tensor order, op precision.  Each step runs
  // pass one's kernels with pass one's coefficients (the apply, the update,
  // the normalisation of an FP64 run), so the replayed vectors are pass one's
  // bits: after a Ritz pair converges the recurrence amplifies any rounding
  // difference, and a replay in other arithmetic drifted from the vectors
  // whose T_m gave y (an FP32 Ritz vector 6 % off the ground state of a
  // 49-state sector).
  void pass_two(const void* b, int64_t steps, double scale, const std::vector<double>& alphas,
                const std::vector<double>& betas, double b_norm,
                const std::vector<std::complex<double>>& y, void* x) {
    MB_REQUIRE(b_norm > kTol, MB_ERR_ZERO_NORM, "Input vector has zero norm");
    MB_REQUIRE((int64_t)y.size() == steps, MB_ERR_DIM_MISMATCH,
               "Dimension mismatch: y_k size must match decomposition steps");
    if (steps == 0) {
      MB_CUDA(cudaMemsetAsync(x, 0, vb, st));
      return;
    }
    launch_axpby(prec, n, 1.0 / b_norm, 0.0, b, 0.0, 0.0, v_curr.p, nullptr, 0, st);
    MB_CUDA(cudaMemsetAsync(v_prev.p, 0, vb, st));
    launch_axpby(prec, n, y[0].real(), y[0].imag(), v_curr.p, 0.0, 0.0, x, nullptr, 0, st);
    const bool fold = prec == MB_PREC_F32;  // pass one's unnormalised FP32 vectors
    double s_curr = 1.0, s_prev = 1.0;
    for (int64_t j = 0; j + 1 < steps; ++j) {
      const double alpha_j = alphas[(size_t)j], beta_j = betas[(size_t)j];
      const double beta_prev = j == 0 ? 0.0 : betas[(size_t)j - 1];
      launch_apply(op->view, prec, v_curr.p, w.p, scale / s_curr, 0.0, -beta_prev / s_prev,
                   beta_prev != 0.0 ? v_prev.p : nullptr, red.p(), 1, st);
      launch_axpby(prec, n, -alpha_j / s_curr, 0.0, v_curr.p, 1.0, 0.0, w.p, red.p(), 1, st);
      std::swap(v_prev.p, v_curr.p);
      std::swap(v_curr.p, w.p);
      if (fold) {
        s_prev = s_curr;
        s_curr = beta_j;
      } else {
        launch_axpby(prec, n, 0.0, 0.0, nullptr, 1.0 / beta_j, 0.0, v_curr.p, nullptr, 0, st);
      }
      // x += y_(j+1) v_(j+1), v_(j+1) = u_(j+1) / s_(j+1)
      launch_axpby(prec, n, y[(size_t)j + 1].real() / s_curr, y[(size_t)j + 1].imag() / s_curr,
                   v_curr.p, 1.0, 0.0, x, nullptr, 0, st);
    }
  }

  // x = sum_j y_j V_j from the stored basis (full re-orthogonalisation runs).
  void combine_basis(int64_t steps, const std::vector<std::complex<double>>& y, void* x) {
    std::vector<double> c(2 * (size_t)steps);
    for (int64_t j = 0; j < steps; ++j) {
      c[2 * (size_t)j] = -y[(size_t)j].real();
      c[2 * (size_t)j + 1] = -y[(size_t)j].imag();
    }
    MB_CUDA(cudaMemcpyAsync(coef.p, c.data(), sizeof(double) * c.size(), cudaMemcpyHostToDevice, st));
    MB_CUDA(cudaMemsetAsync(x, 0, vb, st));
    launch_multi_axpy(basis_prec, prec, n, basis.p, n, (int)steps, (const double*)coef.p, x,
                      red.p(), st);
    MB_CUDA(cudaStreamSynchronize(st));
  }
};

// ---------------------------------------------------------------------------
// FP64 Rayleigh-Ritz refinement of ground-state estimates, many at once.  A
// problem is an operator view and a start vector x (complex128, tensor
// order).  Its Krylov space span{x, Hx, H^2 x, ...} is built with FP64
// vectors and arithmetic: Lanczos with full re-orthogonalisation (w = H q_j
// orthogonalised against q_0..q_j by classical Gram-Schmidt, kRefinePasses
// passes; alpha_j is w's total coefficient on q_j, beta_j the norm of what
// remains).  Two passes (CGS2): with one, orthogonality decays by about
// |theta| / beta a step, and a start vector close to an eigenvector of an
// operator far from zero (beta_0 ~ 1e-5, |E0| ~ 100: 1D L=14 13+13 at U=9.2)
// lost it within six steps, its lowest Ritz value falling 7 % below E0; the
// second pass holds it at ~1e-17.  After each step the lowest
// eigenvalue of T_(j+1) is the estimate; steps continue until it settles to
// kRefineSettle relative (at least kRefineMinSteps), the space breaks down,
// or the problem's step budget (kRefineMaxSteps, fewer where the basis would
// pass kRefineBasisBytes).  The problems advance in lockstep: their kernels
// queue on kRefineLanes streams and the host waits once per step for all of
// them.
// ---------------------------------------------------------------------------
namespace {
constexpr int kRefinePasses = 2;
constexpr size_t kRefineBasisBytes = (size_t)24 << 30;  // one problem's basis at most
constexpr size_t kRefineChunkBytes = (size_t)4 << 30;   // bases of problems run together

struct RefineRun {
  RefineProblem* p;
  int64_t n;
  size_t vb;
  int steps, cap;
  char* q = nullptr;     // cap vectors
  double* dc = nullptr;  // device: 2 passes x 2 cap coefficients, then 3 reduced norms
  double* hc = nullptr;  // host mirror
  std::vector<double> alpha, beta;
  double theta = 0.0;
  bool done = false;
  char* col(int k) const { return q + vb * (size_t)k; }
};
}  // namespace

// The buffers of a group of problems run together, sized for the largest
// group of a call and reused by each group (one allocation a call).
struct RefineSizes {
  size_t qbytes = 0, cwords = 0;
  int pblocks = 1, pcomps = 3;
  void add(const RefineRun& r) {
    qbytes += r.vb * (size_t)r.cap;
    cwords += 4 * (size_t)r.cap + 4;
    pblocks = std::max({pblocks, apply_grid(r.p->v, MB_PREC_F64), blas_grid(r.n),
                        multi_dot_grid(r.n)});
    pcomps = std::max(pcomps, 2 * r.cap);
  }
  void widen(const RefineSizes& o) {
    qbytes = std::max(qbytes, o.qbytes);
    cwords = std::max(cwords, o.cwords);
    pblocks = std::max(pblocks, o.pblocks);
    pcomps = std::max(pcomps, o.pcomps);
  }
};
// The problems of a group spread over kRefineLanes streams (problem i on
// lane i mod kRefineLanes, each lane with its own partial sums), so the small
// sectors' latency-bound kernels overlap on the device; every problem's
// kernels and their order are the same as on one stream, so are its bits.
constexpr int kRefineLanes = 8;
struct RefineBufs {
  DevBuf q, c, part;
  size_t pstride = 0;  // doubles of partial sums a lane
  double* host = nullptr;
  cudaStream_t lane[kRefineLanes] = {};
  cudaEvent_t fork = nullptr, done[kRefineLanes] = {};
  explicit RefineBufs(const RefineSizes& z)
      : q(z.qbytes), c(sizeof(double) * z.cwords),
        part(sizeof(double) * kRefineLanes * (size_t)z.pblocks * z.pcomps),
        pstride((size_t)z.pblocks * z.pcomps) {
    MB_CUDA(cudaMallocHost(&host, sizeof(double) * z.cwords));
    MB_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    for (int k = 0; k < kRefineLanes; ++k) {
      MB_CUDA(cudaStreamCreateWithFlags(&lane[k], cudaStreamNonBlocking));
      MB_CUDA(cudaEventCreateWithFlags(&done[k], cudaEventDisableTiming));
    }
  }
  ~RefineBufs() {
    for (int k = 0; k < kRefineLanes; ++k) {
      if (lane[k]) cudaStreamDestroy(lane[k]);
      if (done[k]) cudaEventDestroy(done[k]);
    }
    if (fork) cudaEventDestroy(fork);
    if (host) cudaFreeHost(host);
  }
  RefineBufs(const RefineBufs&) = delete;
  RefineBufs& operator=(const RefineBufs&) = delete;
};

static void refine_chunk(std::vector<RefineRun>& runs, RefineBufs& bufs, cudaStream_t st) {
  RefineSizes z;
  for (auto& r : runs) z.add(r);
  const size_t cwords = z.cwords;
  DevBuf& qbuf = bufs.q;
  DevBuf& cbuf = bufs.c;
  double* host = bufs.host;
  {
    size_t qo = 0, co = 0;
    for (auto& r : runs) {
      r.q = (char*)qbuf.p + qo;
      r.dc = (double*)cbuf.p + co;
      r.hc = host + co;
      qo += r.vb * (size_t)r.cap;
      co += 4 * (size_t)r.cap + 4;
    }
  }
  const int nl = std::min<int>(kRefineLanes, (int)runs.size());
  auto ls = [&](size_t i) { return bufs.lane[i % kRefineLanes]; };
  auto pp = [&](size_t i) { return (double*)bufs.part.p + bufs.pstride * (i % kRefineLanes); };
  // the lanes start after the caller's stream (the start vectors), and the
  // caller's stream waits for every lane before it reads the coefficients
  MB_CUDA(cudaEventRecord(bufs.fork, st));
  for (int k = 0; k < nl; ++k) MB_CUDA(cudaStreamWaitEvent(bufs.lane[k], bufs.fork, 0));
  auto sync_all = [&] {
    for (int k = 0; k < nl; ++k) {
      MB_CUDA(cudaEventRecord(bufs.done[k], bufs.lane[k]));
      MB_CUDA(cudaStreamWaitEvent(st, bufs.done[k], 0));
    }
    MB_CUDA(cudaMemcpyAsync(host, cbuf.p, sizeof(double) * cwords, cudaMemcpyDeviceToHost, st));
    MB_CUDA(cudaStreamSynchronize(st));
  };
  auto nn_off = [](const RefineRun& r) { return 4 * (size_t)r.cap; };
  // q_0 = x / |x|
  for (size_t i = 0; i < runs.size(); ++i) {
    RefineRun& r = runs[i];
    MB_CUDA(cudaMemcpyAsync(r.col(0), r.p->x, r.vb, cudaMemcpyDeviceToDevice, ls(i)));
    launch_dot(MB_PREC_F64, r.n, r.col(0), r.col(0), pp(i), ls(i));
    launch_reduce(pp(i), blas_grid(r.n), 3, r.dc + nn_off(r), ls(i));
  }
  sync_all();
  for (size_t i = 0; i < runs.size(); ++i) {
    RefineRun& r = runs[i];
    const double nx = std::sqrt(r.hc[nn_off(r) + 2]);
    MB_REQUIRE(nx > 0.0, MB_ERR_ZERO_NORM, "refinement start vector has zero norm");
    launch_axpby(MB_PREC_F64, r.n, 1.0 / nx, 0.0, r.col(0), 0.0, 0.0, r.col(0), nullptr, 0, ls(i));
  }
  for (int j = 0;; ++j) {
    bool any = false;
    for (size_t i = 0; i < runs.size(); ++i) {
      RefineRun& r = runs[i];
      if (r.done) continue;
      any = true;
      // w = H q_j in the next basis slot, then w -= Q Q^H w twice against
      // q_0..q_j: the passes' coefficients at dc[0..) and dc[2 cap..), the
      // norm of the rest at dc[4 cap + 1]
      void* w = r.col(j + 1);
      launch_apply(r.p->v, MB_PREC_F64, r.col(j), w, 1.0, 0.0, 0.0, nullptr, nullptr, 0, ls(i));
      for (int pass = 0; pass < kRefinePasses; ++pass) {
        double* c = r.dc + 2 * (size_t)r.cap * pass;
        launch_multi_dot(MB_PREC_F64, MB_PREC_F64, r.n, r.q, r.n, j + 1, w, pp(i), ls(i));
        launch_reduce(pp(i), multi_dot_grid(r.n), 2 * (j + 1), c, ls(i));
        launch_multi_axpy(MB_PREC_F64, MB_PREC_F64, r.n, r.q, r.n, j + 1, c, w, pp(i), ls(i));
      }
      launch_reduce(pp(i), blas_grid(r.n), 3, r.dc + nn_off(r), ls(i));
    }
    if (!any) break;
    sync_all();
    for (size_t i = 0; i < runs.size(); ++i) {
      RefineRun& r = runs[i];
      if (r.done) continue;
      double a = 0.0;
      for (int pass = 0; pass < kRefinePasses; ++pass) a += r.hc[2 * (size_t)r.cap * pass + 2 * j];
      r.alpha.push_back(a);
      const double b = std::sqrt(r.hc[nn_off(r) + 1]);
      std::vector<double> d(r.alpha), e(r.beta);
      MB_REQUIRE(tridiag_eig((int)d.size(), d, e, nullptr), MB_ERR_EIG_FAILED,
                 "Eigenvalue decomposition of T_k failed");
      const bool settled = j + 1 >= kRefineMinSteps &&
                           std::fabs(d[0] - r.theta) <= kRefineSettle * std::fabs(d[0]);
      r.theta = d[0];
      if (settled || j + 1 >= r.steps || !(b > kTol)) {
        r.done = true;
        r.p->e0 = r.theta;
        continue;
      }
      r.beta.push_back(b);
      launch_axpby(MB_PREC_F64, r.n, 1.0 / b, 0.0, r.col(j + 1), 0.0, 0.0, r.col(j + 1), nullptr,
                   0, ls(i));
    }
  }
}

void fp64_refine_many(RefineProblem* probs, int count, cudaStream_t st) {
  if (count <= 0) return;
  // group the problems (consecutive, bases under kRefineChunkBytes a group)
  std::vector<std::vector<RefineRun>> groups(1);
  std::vector<RefineSizes> sizes(1);
  size_t group_bytes = 0;
  for (int i = 0; i < count; ++i) {
    RefineRun r{};
    RefineProblem& p = probs[i];
    r.p = &p;
    r.n = p.v.dim;
    r.vb = 16 * (size_t)r.n;
    const int64_t fit = (int64_t)(kRefineBasisBytes / std::max<size_t>(r.vb, 1)) - 1;
    r.steps = (int)std::max<int64_t>(kRefineMinSteps, std::min<int64_t>(kRefineMaxSteps, fit));
    r.cap = r.steps + 1;
    const size_t rb = r.vb * (size_t)r.cap;
    if (!groups.back().empty() && group_bytes + rb > kRefineChunkBytes) {
      groups.emplace_back();
      sizes.emplace_back();
      group_bytes = 0;
    }
    sizes.back().add(r);
    groups.back().push_back(std::move(r));
    group_bytes += rb;
  }
  RefineSizes most;
  for (const auto& z : sizes) most.widen(z);
  RefineBufs bufs(most);
  for (auto& g : groups) refine_chunk(g, bufs, st);
}

double fp64_ritz_refine(const OpView& v, const void* x64, cudaStream_t st) {
  RefineProblem p{};
  p.v = v;
  p.x = x64;
  fp64_refine_many(&p, 1, st);
  return p.e0;
}

static void eigenpair(mb_op_s* op, int64_t k, const void* seed, int order,
                      const mb_lanczos_opts* opts, double sign, double* e_out, void* vec,
                      int64_t* steps_out) {
  check_order(order);
  if (op->precision == MB_PREC_Q64) {
    MB_REQUIRE(seed && e_out, MB_ERR_INVALID_ARG, "NULL argument");
    q_eigenpair(op, k, seed, order, opts, sign, e_out, vec, steps_out);
    return;
  }
  MB_REQUIRE(seed && e_out, MB_ERR_INVALID_ARG, "NULL argument");
  MB_REQUIRE(k >= 0, MB_ERR_INVALID_ARG, "k must be >= 0");
  mb_lanczos_opts o{};
  o.basis_precision = -1;
  o.check_every = 10;
  if (opts) o = *opts;
  if (o.check_every <= 0) o.check_every = 10;
  cudaStream_t st = 0;
  Krylov kr(op, st);
  DevBuf bt(kr.vb);
  to_tensor(op, seed, bt.p, order, st);
  const bool reorth = o.reorth != 0 && k > 0;
  if (reorth) kr.reserve_basis(k, o.basis_precision);
  std::vector<double> alphas, betas;
  double b_norm = 0.0;
  const bool refine = o.refine && op->precision == MB_PREC_F32;
  // find_min_eigenpair runs find_max_eigenpair on Negated<Op> (lanczos.h:283-290).
  const int64_t m = kr.pass_one(bt.p, k, sign, alphas, betas, b_norm, reorth, o.conv_tol,
                                o.check_every, nullptr, !reorth && (vec || refine));
  if (steps_out) *steps_out = m;
  if (m == 0) {
    *e_out = 0.0;
    if (vec) MB_CUDA(cudaMemsetAsync(vec, 0, kr.vb, st));
    MB_CUDA(cudaStreamSynchronize(st));
    return;
  }
  std::vector<double> d(alphas), z;
  std::vector<double> e(betas);
  e.resize((size_t)m - 1);
  MB_REQUIRE(tridiag_eig((int)m, d, e, &z), MB_ERR_EIG_FAILED,
             "Eigenvalue decomposition of T_k failed");
  *e_out = sign * d[(size_t)m - 1];
  if (vec || refine) {
    // An FP32 run without re-orthogonalisation that ran all k steps takes
    // its Ritz vector from the first converged checkpoint, before a ghost
    // copy of the eigenvalue can enter T_m; every other run (including one
    // that stopped on its convergence test) from T_m as the reference does.
    int64_t mv = m;
    if (refine && !reorth && m == k) {
      mv = ritz_vector_steps(alphas, betas, (int)m, o.check_every, 1e-9);
      if (mv != m) {
        d.assign(alphas.begin(), alphas.begin() + mv);
        e.assign(betas.begin(), betas.begin() + (mv - 1));
        MB_REQUIRE(tridiag_eig((int)mv, d, e, &z), MB_ERR_EIG_FAILED,
                   "Eigenvalue decomposition of T_k failed");
      }
    }
    std::vector<std::complex<double>> y((size_t)mv);
    for (int64_t i = 0; i < mv; ++i) y[(size_t)i] = z[(size_t)(mv - 1) * mv + i] * b_norm;
    DevBuf xt(kr.vb);
    if (reorth) {
      kr.combine_basis(m, y, xt.p);
    } else if (mv <= kr.kept) {
      kr.combine_kept(mv, betas, y, xt.p);
    } else {
      kr.pass_two(bt.p, mv, sign, alphas, betas, b_norm, y, xt.p);
    }
    if (refine) {
      // FP64 refinement of the FP32 Ritz vector x: Rayleigh-Ritz on
      // span{x, Hx, ..., H^(j-1) x} with FP64 vectors and arithmetic (its
      // first step is the Rayleigh quotient <x,Hx>/<x,x>; further Krylov
      // directions, 3 to 8 until the lowest Ritz value settles, remove the
      // FP32 error of x).
      DevBuf x64(16 * (size_t)op->dim);
      launch_convert(MB_PREC_F32, MB_PREC_F64, op->dim, xt.p, x64.p, st);
      *e_out = fp64_ritz_refine(op->view, x64.p, st);
    }
    if (vec) from_tensor(op, xt.p, vec, order, st);
  }
  MB_CUDA(cudaStreamSynchronize(st));
}

// Krylov expmv (evolve_state.h:120-151).
static void evolve(mb_op_s* op, const void* psi0, int order, double t, int64_t krylov_steps,
                   int imaginary, void* out) {
  check_order(order);
  MB_REQUIRE(psi0 && out, MB_ERR_INVALID_ARG, "NULL vector");
  if (op->precision == MB_PREC_Q64) {
    q_evolve(op, psi0, order, t, krylov_steps, imaginary, out);
    return;
  }
  cudaStream_t st = 0;
  Krylov kr(op, st);
  DevBuf bt(kr.vb);
  to_tensor(op, psi0, bt.p, order, st);
  const double psi_norm = kr.norm_of(bt.p);
  if (psi_norm <= kTol) {  // evolve_state returns psi0 unchanged (:130-133)
    if (out != psi0) MB_CUDA(cudaMemcpyAsync(out, psi0, kr.vb, cudaMemcpyDeviceToDevice, st));
    MB_CUDA(cudaStreamSynchronize(st));
    return;
  }
  int64_t k = krylov_steps <= 0 ? 30 : krylov_steps;
  if (k > op->dim) k = op->dim;
  std::vector<double> alphas, betas;
  double b_norm = 0.0;
  const int64_t m = kr.pass_one(bt.p, k, 1.0, alphas, betas, b_norm, false, 0.0, 0, nullptr, true);
  // expm_tridiagonal_first_column_{unitary,imaginary} (evolve_state.h:22-106)
  std::vector<double> d(alphas), z, e(betas);
  e.resize((size_t)std::max<int64_t>(m - 1, 0));
  MB_REQUIRE(tridiag_eig((int)m, d, e, &z), MB_ERR_EIG_FAILED,
             "Eigenvalue decomposition of T_k failed");
  std::vector<std::complex<double>> y((size_t)m);
  for (int64_t i = 0; i < m; ++i) {
    std::complex<double> s = 0.0;
    for (int64_t j = 0; j < m; ++j) {
      const double wj = z[(size_t)j * m + 0];
      const std::complex<double> ex =
          imaginary ? std::complex<double>(std::exp(-t * d[(size_t)j]), 0.0)
                    : std::exp(std::complex<double>(0.0, -t * d[(size_t)j]));
      s += z[(size_t)j * m + i] * ex * wj;
    }
    y[(size_t)i] = s * b_norm;  // solve() scales y by ||b|| (lanczos.h:231-233)
  }
  DevBuf xt(kr.vb);
  if (m <= kr.kept) kr.combine_kept(m, betas, y, xt.p);
  else kr.pass_two(bt.p, m, 1.0, alphas, betas, b_norm, y, xt.p);
  from_tensor(op, xt.p, out, order, st);
  MB_CUDA(cudaStreamSynchronize(st));
}

}  // namespace mb

using namespace mb;

extern "C" {

int mb_device_count(int* count) {
  if (!count) return MB_ERR_INVALID_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  *count = n;
  return MB_OK;
}

int mb_alloc(void** dev_ptr, size_t bytes) {
  return guard([&] {
    MB_REQUIRE(dev_ptr, MB_ERR_INVALID_ARG, "NULL argument");
    require_device();
    MB_CUDA(cudaMalloc(dev_ptr, bytes));
  });
}

int mb_free(void* dev_ptr) {
  return guard([&] { MB_CUDA(cudaFree(dev_ptr)); });
}

int mb_memcpy(void* dst, const void* src, size_t bytes, int kind) {
  return guard([&] {
    MB_REQUIRE(kind >= 0 && kind <= 2, MB_ERR_INVALID_ARG, "kind must be 0, 1 or 2");
    const cudaMemcpyKind k = kind == 0 ? cudaMemcpyHostToDevice
                             : kind == 1 ? cudaMemcpyDeviceToHost
                                         : cudaMemcpyDeviceToDevice;
    MB_CUDA(cudaMemcpy(dst, src, bytes, k));
  });
}

int mb_synchronize(void) {
  return guard([&] { MB_CUDA(cudaDeviceSynchronize()); });
}

int mb_op_create(mb_basis_t basis, mb_model_t model, int precision, mb_op_t* out) {
  return guard([&] {
    MB_REQUIRE(basis && model && out, MB_ERR_INVALID_ARG, "NULL argument");
    *out = nullptr;
    MB_REQUIRE(precision == MB_PREC_F64 || precision == MB_PREC_F32 || precision == MB_PREC_Q64,
               MB_ERR_INVALID_ARG, "precision must be MB_PREC_F64, MB_PREC_F32 or MB_PREC_Q64");
    MB_REQUIRE(model->L == basis->L, MB_ERR_DIM_MISMATCH,
               "model sites and basis orbitals differ");
    require_device();
    auto op = std::make_unique<mb_op_s>();
    op->precision = precision;
    try {
      if (basis->all_sz()) {
        build_all_sz(op.get(), basis, model);
      } else if (model->momentum && !model->current && !basis->momentum()) {
        build_momentum_all(op.get(), basis, model);
      } else if (basis->momentum() || model->momentum) {
        build_momentum_op(op.get(), basis, model);
      } else {
        build_op(op.get(), basis, model);
      }
    } catch (...) {
      free_op_memory(op.get());
      throw;
    }
    *out = op.release();
  });
}

int mb_op_create_csr(int64_t n, const int64_t* row_ptr, const int64_t* col_idx,
                     const double* values, int precision, mb_op_t* out) {
  return guard([&] {
    MB_REQUIRE(row_ptr && out && n > 0, MB_ERR_INVALID_ARG, "NULL argument or empty matrix");
    *out = nullptr;
    MB_REQUIRE(precision == MB_PREC_F64 || precision == MB_PREC_F32, MB_ERR_INVALID_ARG,
               "a sparse-matrix operator takes MB_PREC_F64 or MB_PREC_F32");
    MB_REQUIRE(n < (int64_t(1) << 31), MB_ERR_CAPACITY, "matrix dimension above 2^31 - 1");
    MB_REQUIRE(row_ptr[0] == 0, MB_ERR_INVALID_ARG, "row_ptr[0] must be 0");
    for (int64_t i = 0; i < n; ++i)
      MB_REQUIRE(row_ptr[i + 1] >= row_ptr[i], MB_ERR_INVALID_ARG, "row_ptr must not decrease");
    const int64_t nnz = row_ptr[n];
    MB_REQUIRE(nnz == 0 || (col_idx && values), MB_ERR_INVALID_ARG, "NULL col_idx or values");
    std::vector<int32_t> col((size_t)std::max<int64_t>(nnz, 1), 0);
    for (int64_t k = 0; k < nnz; ++k) {
      MB_REQUIRE(col_idx[k] >= 0 && col_idx[k] < n, MB_ERR_INVALID_ARG, "column index out of range");
      col[(size_t)k] = (int32_t)col_idx[k];
    }
    require_device();
    auto op = std::make_unique<mb_op_s>();
    op->precision = precision;
    op->natural_order = true;
    try {
      MB_CUDA(cudaGetDevice(&op->device));
      op->Du = n;
      op->Dd = 1;
      op->dim = n;
      OpView& v = op->view;
      v.Du = n;
      v.Dd = 1;
      v.dim = n;
      v.csr_row = upload(op.get(), std::vector<int64_t>(row_ptr, row_ptr + n + 1));
      v.csr_col = upload(op.get(), col);
      std::vector<double2> val((size_t)std::max<int64_t>(nnz, 1), make_double2(0.0, 0.0));
      for (int64_t k = 0; k < nnz; ++k) val[(size_t)k] = make_double2(values[2 * k], values[2 * k + 1]);
      v.csr_val = upload(op.get(), val);
      if (precision == MB_PREC_F32) {
        std::vector<float2> vf(val.size());
        for (size_t k = 0; k < val.size(); ++k) vf[k] = make_float2((float)val[k].x, (float)val[k].y);
        v.csr_val_f = upload(op.get(), vf);
      }
    } catch (...) {
      for (void* p : op->allocations) cudaFree(p);
      throw;
    }
    *out = op.release();
  });
}

int mb_op_destroy(mb_op_t op) {
  if (!op) return MB_OK;
  cudaSetDevice(op->device);
  cudaDeviceSynchronize();
  q_op_release(op);
  free_op_memory(op);
  delete op;
  return MB_OK;
}

int mb_op_dimension(mb_op_t op, int64_t* dim) {
  return guard([&] {
    MB_REQUIRE(op && dim, MB_ERR_INVALID_ARG, "NULL argument");
    *dim = op->dim;
  });
}

int mb_op_precision(mb_op_t op, int* precision) {
  return guard([&] {
    MB_REQUIRE(op && precision, MB_ERR_INVALID_ARG, "NULL argument");
    *precision = op->precision;
  });
}

int mb_op_get_apply_shape(mb_op_t op, mb_apply_shape* shape) {
  return guard([&] {
    MB_REQUIRE(op && shape, MB_ERR_INVALID_ARG, "NULL argument");
    *shape = mb_apply_shape{};
    shape->passes = op->apply_passes;
    shape->row_split = std::max(1, op->view.row_split);
    shape->table_bits = op->view.table_bits == 16 ? 16 : 32;
    shape->prefetch = op->view.up_prefetch;
    shape->table_stage = op->view.table_stage ? 1 : 0;
    shape->csr_lanes = op->view.csr_lanes;
  });
}

int mb_op_set_apply_shape(mb_op_t op, const mb_apply_shape* shape) {
  return guard([&] {
    MB_REQUIRE(op && shape, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(shape->passes == 1 || shape->passes == 2, MB_ERR_INVALID_ARG,
               "passes must be 1 or 2");
    MB_REQUIRE(shape->row_split == 1 || shape->row_split == 2 || shape->row_split == 4,
               MB_ERR_INVALID_ARG, "row_split must be 1, 2 or 4");
    MB_REQUIRE(shape->table_bits == 32 || shape->table_bits == 16, MB_ERR_INVALID_ARG,
               "table_bits must be 32 or 16");
    MB_REQUIRE(shape->prefetch == 0 || shape->prefetch == 1, MB_ERR_INVALID_ARG,
               "prefetch must be 0 or 1");
    MB_REQUIRE(shape->table_stage == 0 || shape->table_stage == 1, MB_ERR_INVALID_ARG,
               "table_stage must be 0 or 1");
    MB_REQUIRE(shape->csr_lanes == 0 || shape->csr_lanes == 4 || shape->csr_lanes == 8 ||
                   shape->csr_lanes == 16 || shape->csr_lanes == 32,
               MB_ERR_INVALID_ARG, "csr_lanes must be 0, 4, 8, 16 or 32");
    MB_REQUIRE(shape->csr_lanes == 0 || (op->view.csr_row && !op->view.n_blocks),
               MB_ERR_INVALID_ARG, "csr_lanes applies to operators held as one sparse matrix");
    const bool lattice = !op->view.csr_row && !op->view.n_blocks && op->view.dn_sell;
    const bool tuned = shape->passes != 1 || shape->row_split != 1 || shape->table_bits != 32;
    if (tuned)
      MB_REQUIRE(op->precision == MB_PREC_Q64 && lattice, MB_ERR_INVALID_ARG,
                 "passes, row_split and table_bits other than 1, 1, 32 need an MB_PREC_Q64 "
                 "lattice operator");
    if (shape->prefetch)
      MB_REQUIRE(lattice, MB_ERR_INVALID_ARG, "prefetch needs a lattice operator");
    if (shape->table_stage) {
      MB_REQUIRE(op->precision == MB_PREC_Q64 && lattice && shape->passes == 1 &&
                     shape->table_bits == 32,
                 MB_ERR_INVALID_ARG,
                 "table_stage needs a one-pass MB_PREC_Q64 lattice apply with 32-bit entries");
      MB_REQUIRE(q_table_stage_fits(op->view), MB_ERR_CAPACITY,
                 "the warps' table buffers do not fit beside the staged row");
    }
    if (shape->passes == 2)
      MB_REQUIRE(q_upcol_fits(op->view), MB_ERR_CAPACITY,
                 "a column of the sector does not fit in shared memory");
    if (shape->table_bits == 16)
      MB_REQUIRE(op->view.dn_sell16 && op->view.up_sell16, MB_ERR_CAPACITY,
                 "16-bit table entries need sectors below 32760 states per spin");
    std::lock_guard<std::mutex> lk(op->mu);
    op->apply_passes = shape->passes;
    op->view.row_split = shape->row_split;
    op->view.table_bits = shape->table_bits;
    op->view.up_prefetch = shape->prefetch;
    op->view.table_stage = shape->table_stage;
    op->view.csr_lanes = shape->csr_lanes;
  });
}

// ---------------------------------------------------------------------------
// The apply autotuner: every candidate shape of a lattice operator timed on
// the live GPU (CUDA events, tensor-order device vectors, median of 7 after
// 2 warm-up applies); the fastest is kept, and cached per (lattice, N_up,
// N_down, precision) for the process, so later operators of the same sector
// take it without timing.
// ---------------------------------------------------------------------------
static std::mutex g_tune_mu;
static std::map<std::string, std::pair<mb_apply_shape, double>> g_tune_cache;

static std::vector<mb_apply_shape> tune_candidates(const mb_op_s* op) {
  std::vector<mb_apply_shape> out;
  if (op->view.csr_row) {  // one sparse matrix: the lanes a row
    for (int lanes : {4, 8, 16, 32}) {
      mb_apply_shape s{};
      s.passes = 1;
      s.row_split = 1;
      s.table_bits = 32;
      s.csr_lanes = lanes;
      out.push_back(s);
    }
    return out;
  }
  for (int pf = 0; pf <= 1; ++pf) {
    if (op->precision != MB_PREC_Q64) {
      mb_apply_shape s{};
      s.passes = 1;
      s.row_split = 1;
      s.table_bits = 32;
      s.prefetch = pf;
      out.push_back(s);
      continue;
    }
    for (int passes = 1; passes <= 2; ++passes) {
      if (passes == 2 && !q_upcol_fits(op->view)) continue;
      for (int split : {1, 2})
        for (int tb : {32, 16}) {
          if (tb == 16 && !(op->view.dn_sell16 && op->view.up_sell16)) continue;
          if (passes == 2 && pf) continue;  // the row pass of two has no up-hop loads
          for (int ts = 0; ts <= 1; ++ts) {
            if (ts && !(passes == 1 && tb == 32 && q_table_stage_fits(op->view))) continue;
            mb_apply_shape s{};
            s.passes = passes;
            s.row_split = split;
            s.table_bits = tb;
            s.prefetch = pf;
            s.table_stage = ts;
            out.push_back(s);
          }
        }
    }
  }
  return out;
}

}  // extern "C"

namespace mb {
void q_tune_prepare(mb_op_s* op, void** xq, void** yq, void** prm, cudaStream_t st);
void q_tune_apply(mb_op_s* op, const void* xq, void* yq, const void* prm, cudaStream_t st);
}  // namespace mb

extern "C" {

int mb_op_autotune(mb_op_t op, void* stream, mb_apply_shape* chosen, double* best_ms) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    cudaStream_t st = (cudaStream_t)stream;
    mb_apply_shape best{};
    double best_t = 0.0;
    bool cached = false;
    if (!op->tune_key.empty()) {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune_cache.find(op->tune_key);
      if (it != g_tune_cache.end()) {
        best = it->second.first;
        best_t = it->second.second;
        cached = true;
      }
    }
    if (!cached && !op->tune_key.empty()) {
      const auto cands = tune_candidates(op);
      // device vectors in tensor order: complex128 / complex64, or Q64 mantissas
      void *x = nullptr, *y = nullptr, *prm = nullptr;
      std::vector<void*> own;
      if (op->precision == MB_PREC_Q64) {
        q_tune_prepare(op, &x, &y, &prm, st);
        own = {x, y, prm};
      } else {
        const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
        MB_CUDA(cudaMalloc(&x, vb));
        own.push_back(x);
        MB_CUDA(cudaMalloc(&y, vb));
        own.push_back(y);
        launch_fill_rng(op->precision, op->Du, op->Dd, 12345, 0, 0, x, st);
      }
      struct TimingEvents {  // Events (no timing) will not do for elapsed times
        cudaEvent_t e[2] = {nullptr, nullptr};
        TimingEvents() {
          for (auto& x : e) MB_CUDA(cudaEventCreate(&x));
        }
        ~TimingEvents() {
          for (auto x : e)
            if (x) cudaEventDestroy(x);
        }
        cudaEvent_t operator[](int i) const { return e[i]; }
      } ev;
      const mb_apply_shape keep = [&] {
        mb_apply_shape k{};
        k.passes = op->apply_passes;
        k.row_split = std::max(1, op->view.row_split);
        k.table_bits = op->view.table_bits == 16 ? 16 : 32;
        k.prefetch = op->view.up_prefetch;
        k.table_stage = op->view.table_stage;
        k.csr_lanes = op->view.csr_lanes;
        return k;
      }();
      try {
        for (const auto& c : cands) {
          op->apply_passes = c.passes;
          op->view.row_split = c.row_split;
          op->view.table_bits = c.table_bits;
          op->view.up_prefetch = c.prefetch;
          op->view.table_stage = c.table_stage;
          op->view.csr_lanes = c.csr_lanes;
          auto run = [&] {
            if (op->precision == MB_PREC_Q64) q_tune_apply(op, x, y, prm, st);
            else launch_apply(op->view, op->precision, x, y, 1.0, 0.0, 0.0, nullptr, nullptr, 0, st);
          };
          run();
          run();
          std::vector<float> ts;
          for (int i = 0; i < 7; ++i) {
            MB_CUDA(cudaEventRecord(ev[0], st));
            run();
            MB_CUDA(cudaEventRecord(ev[1], st));
            MB_CUDA(cudaEventSynchronize(ev[1]));
            float ms = 0.f;
            MB_CUDA(cudaEventElapsedTime(&ms, ev[0], ev[1]));
            ts.push_back(ms);
          }
          std::sort(ts.begin(), ts.end());
          const double t = ts[ts.size() / 2];
          if (best_t == 0.0 || t < best_t) {
            best_t = t;
            best = c;
          }
        }
      } catch (...) {
        op->apply_passes = keep.passes;
        op->view.row_split = keep.row_split;
        op->view.table_bits = keep.table_bits;
        op->view.up_prefetch = keep.prefetch;
        op->view.table_stage = keep.table_stage;
        op->view.csr_lanes = keep.csr_lanes;
        for (void* p : own) cudaFree(p);
        throw;
      }
      for (void* p : own) cudaFree(p);
      std::lock_guard<std::mutex> lk(g_tune_mu);
      g_tune_cache[op->tune_key] = {best, best_t};
    }
    if (op->tune_key.empty()) {  // operators without shapes keep the default
      best = mb_apply_shape{};
      best.passes = 1;
      best.row_split = 1;
      best.table_bits = 32;
    } else {
      std::lock_guard<std::mutex> lk(op->mu);
      op->apply_passes = best.passes;
      op->view.row_split = best.row_split;
      op->view.table_bits = best.table_bits;
      op->view.up_prefetch = best.prefetch;
      op->view.table_stage = best.table_stage;
      op->view.csr_lanes = best.csr_lanes;
    }
    if (chosen) *chosen = best;
    if (best_ms) *best_ms = best_t;
  });
}

int mb_op_apply(mb_op_t op, const void* x_dev, void* y_dev, int order, void* stream) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    apply_affine(op, x_dev, y_dev, 1.0, 0.0, 0.0, nullptr, order, (cudaStream_t)stream);
  });
}

int mb_op_apply_affine(mb_op_t op, const void* x_dev, void* y_dev, double scale, double shift,
                       double beta, const void* z_dev, int order, void* stream) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    apply_affine(op, x_dev, y_dev, scale, shift, beta, z_dev, order, (cudaStream_t)stream);
  });
}

// The host-buffer apply of a complex128 / complex64 lattice operator in
// reference order, pipelined over the host link as the Q64 one is: x lands
// scattered to tensor order (a page-locked x read over the link by the
// scatter kernel, a pageable one in chunks, each scattered while the next is
// in flight), then the rows are applied group by group and each finished
// prefix of the reference order goes back on the copy engine while the later
// groups run.  Same kernels and arithmetic as mb_op_apply, so the same bits.
static void host_apply_pipeline(mb_op_s* op, const mb_op_s::HostLane& lane, const void* x_host,
                                const void* x_mapped, void* y_host, mb_op_s::Scratch& s) {
  cudaStream_t comp = lane.comp;
  int32_t* iperm = op_iperm(op);
  const int prec = op->precision;
  const size_t es = elem_bytes(prec);
  const int64_t n = op->dim;
  char* xt = (char*)s.a;  // tensor order
  char* yt = (char*)s.b;
  char* xs = (char*)s.hx;  // landing, reference order
  if (x_mapped) {
    launch_scatter(prec, n, iperm, x_mapped, xt, comp);
  } else {
    // pageable x: through the lane's bounce buffers, each chunk scattered to
    // tensor order once it has landed
    lane_upload(lane, xs, x_host, es * (size_t)n, es, [&](size_t off, size_t len, cudaEvent_t e) {
      MB_CUDA(cudaStreamWaitEvent(comp, e, 0));
      const int64_t i0 = (int64_t)(off / es);
      launch_scatter(prec, (int64_t)(len / es), iperm + i0, xs + off, xt, comp);
    });
  }
  host_groups_run(
      op, lane, es, y_host, s.hy,
      [&](const OpView& v) {
        launch_apply(v, prec, xt, yt, 1.0, 0.0, 0.0, nullptr, nullptr, 0, comp);
      },
      [&](int64_t i0, int64_t i1, void* dst) {
        launch_gather(prec, i1 - i0, iperm + i0, yt, dst, comp);
      });
}

// A lane of the operator's host-buffer pool for the length of one call.
class LaneLease {
 public:
  explicit LaneLease(mb_op_s* op) : op_(op) {
    std::unique_lock<std::mutex> lk(op->host_mu);
    op->host_cv.wait(lk, [&] {
      return !op->host_idle.empty() || (int)op->host_lanes.size() < mb_op_s::kMaxHostLanes;
    });
    if (op->host_idle.empty()) {
      auto lane = std::make_unique<mb_op_s::HostLane>();
      MB_CUDA(cudaStreamCreateWithFlags(&lane->comp, cudaStreamNonBlocking));
      MB_CUDA(cudaStreamCreateWithFlags(&lane->copy, cudaStreamNonBlocking));
      op->host_idle.push_back(lane.get());
      op->host_lanes.push_back(std::move(lane));
    }
    lane_ = op->host_idle.back();
    op->host_idle.pop_back();
  }
  ~LaneLease() {
    {
      std::lock_guard<std::mutex> lk(op_->host_mu);
      op_->host_idle.push_back(lane_);
    }
    op_->host_cv.notify_one();
  }
  LaneLease(const LaneLease&) = delete;
  LaneLease& operator=(const LaneLease&) = delete;
  const mb_op_s::HostLane& lane() const { return *lane_; }

 private:
  mb_op_s* op_;
  mb_op_s::HostLane* lane_;
};

int mb_op_apply_host(mb_op_t op, const void* x_host, void* y_host, int order) {
  return guard([&] {
    MB_REQUIRE(op && x_host && y_host, MB_ERR_INVALID_ARG, "NULL argument");
    check_order(order);
    const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
    const bool pipelined = order == MB_ORDER_REFERENCE && !op->natural_order &&
                           !op->view.n_blocks && !op->view.csr_row;
    if (pipelined) {
      // the row groups are built once, before any lane uses them
      std::lock_guard<std::mutex> lk(op->host_mu);
      ensure_host_groups(op);
    }
    // each concurrent call runs on its own lane: its streams key its own
    // staging and scratch buffers.  A call on page-locked vectors moves them
    // over the host link at its full rate by itself; such calls take turns
    // (overlapping them only splits the link and slows each one).
    const bool link_bound = host_pinned(x_host) || host_pinned(y_host);
    std::unique_lock<std::mutex> link_lock(op->host_link_mu, std::defer_lock);
    if (link_bound) link_lock.lock();
    LaneLease lease(op);
    const mb_op_s::HostLane& lane = lease.lane();
    cudaStream_t st = lane.comp;
    auto& s = scratch_for(op, st, 0, true);  // the staging pair; a, b where a path needs them
    // A page-locked y (cudaHostAlloc / cudaHostRegister) is written in place by
    // the last kernel (the order / format change), so the result crosses the
    // host link once, while it is produced, instead of after a device copy.
    void* y_dev = s.hy;
    cudaPointerAttributes at{};
    const bool direct = cudaPointerGetAttributes(&at, y_host) == cudaSuccess &&
                        at.type == cudaMemoryTypeHost && at.devicePointer != nullptr;
    if (!direct) cudaGetLastError();  // clear a failed query on pageable memory
    if (direct) y_dev = at.devicePointer;
    if (pipelined) {
      // x lands scattered to tensor order as it arrives; each finished prefix
      // of the result (reference order) goes back while later rows run
      cudaPointerAttributes ax{};
      const bool x_locked = cudaPointerGetAttributes(&ax, x_host) == cudaSuccess &&
                            ax.type == cudaMemoryTypeHost && ax.devicePointer != nullptr;
      if (!x_locked) cudaGetLastError();
      const void* x_mapped = x_locked ? ax.devicePointer : nullptr;
      if (op->precision == MB_PREC_Q64) {
        q_apply_host_reference(op, lane, x_host, x_mapped, y_host, s.hx, s.hy);
        return;
      }
      scratch_for(op, st, 2);  // a, b: x and y in tensor order
      try {
        host_apply_pipeline(op, lane, x_host, x_mapped, y_host, s);
      } catch (...) {
        // nothing may still read or write the caller's buffers once it sees the error
        cudaStreamSynchronize(lane.copy);
        cudaStreamSynchronize(lane.comp);
        throw;
      }
      return;
    }
    try {
      if (host_pinned(x_host)) {
        MB_CUDA(cudaMemcpyAsync(s.hx, x_host, vb, cudaMemcpyHostToDevice, st));
      } else {
        lane_upload(lane, s.hx, x_host, vb, 16, [&](size_t, size_t, cudaEvent_t e) {
          MB_CUDA(cudaStreamWaitEvent(st, e, 0));
        });
      }
      apply_affine(op, s.hx, y_dev, 1.0, 0.0, 0.0, nullptr, order, st);
      if (!direct) {  // pageable y: through the lane's bounce buffers
        Events ev(1);
        MB_CUDA(cudaEventRecord(ev[0], st));
        MB_CUDA(cudaStreamWaitEvent(lane.copy, ev[0], 0));
        lane_download(lane, y_host, s.hy, vb);
      }
      MB_CUDA(cudaStreamSynchronize(st));
    } catch (...) {
      cudaStreamSynchronize(lane.copy);
      cudaStreamSynchronize(st);
      throw;
    }
  });
}

int mb_fill_uniform(mb_op_t op, uint64_t seed, uint32_t stream_id, void* v_dev, int order,
                    void* stream) {
  return guard([&] {
    MB_REQUIRE(op && v_dev, MB_ERR_INVALID_ARG, "NULL argument");
    check_order(order);
    cudaStream_t st = (cudaStream_t)stream;
    if (order == MB_ORDER_TENSOR) {
      launch_fill_rng(op->precision, op->Du, op->Dd, seed, stream_id, 0, v_dev, st);
    } else {
      auto& s = scratch_for(op, st, 1);
      launch_fill_rng(op->precision, op->Du, op->Dd, seed, stream_id, 0, s.a, st);
      from_tensor(op, s.a, v_dev, order, st);
    }
  });
}

int mb_fill_phase(mb_op_t op, uint64_t seed, uint32_t stream_id, void* v_dev, int order,
                  void* stream) {
  return guard([&] {
    MB_REQUIRE(op && v_dev, MB_ERR_INVALID_ARG, "NULL argument");
    check_order(order);
    cudaStream_t st = (cudaStream_t)stream;
    if (order == MB_ORDER_TENSOR) {
      launch_fill_rng(op->precision, op->Du, op->Dd, seed, stream_id, 1, v_dev, st);
    } else {
      auto& s = scratch_for(op, st, 1);
      launch_fill_rng(op->precision, op->Du, op->Dd, seed, stream_id, 1, s.a, st);
      from_tensor(op, s.a, v_dev, order, st);
    }
  });
}

// One momentum sector's H as CSR in the sector's reference order, each row's
// columns ascending (off-diagonals +-U/N, the diagonal where non-zero).
static void momentum_csr(const mb_basis_s* b, const mb_model_s* m, std::vector<int64_t>& rp,
                         std::vector<int64_t>& cols, std::vector<double>& vals) {
  mb_op_s tmp;
  tmp.precision = MB_PREC_F64;
  struct Cleanup {
    mb_op_s& o;
    ~Cleanup() {
      for (void* p : o.allocations) cudaFree(p);
    }
  } cleanup{tmp};
  MomBuild mb;
  build_momentum(&tmp, b, m, mb);
  const int64_t n = mb.n;
  std::vector<int32_t> hcol((size_t)std::max<int64_t>(mb.nnz, 1));
  std::vector<double> hdiag((size_t)std::max<int64_t>(n, 1));
  if (mb.nnz) MB_CUDA(cudaMemcpy(hcol.data(), mb.col, sizeof(int32_t) * (size_t)mb.nnz, cudaMemcpyDeviceToHost));
  if (n) MB_CUDA(cudaMemcpy(hdiag.data(), mb.diag, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost));
  rp.assign((size_t)n + 1, 0);
  for (int64_t i = 0; i < n; ++i)
    rp[(size_t)i + 1] = rp[(size_t)i] + (mb.row_ptr[(size_t)i + 1] - mb.row_ptr[(size_t)i]) +
                        (hdiag[(size_t)i] != 0.0 ? 1 : 0);
  cols.resize((size_t)rp[(size_t)n]);
  vals.resize((size_t)rp[(size_t)n]);
  const double off = tmp.view.csr_off;
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; ++i) {
    std::vector<std::pair<int64_t, double>> row;
    for (int64_t k = mb.row_ptr[(size_t)i]; k < mb.row_ptr[(size_t)i + 1]; ++k) {
      const uint32_t e = (uint32_t)hcol[(size_t)k];
      row.push_back({(int64_t)(e & 0x7FFFFFFFu), (e >> 31) ? -off : off});
    }
    if (hdiag[(size_t)i] != 0.0) row.push_back({i, hdiag[(size_t)i]});
    std::sort(row.begin(), row.end());
    int64_t o = rp[(size_t)i];
    for (const auto& [c, v] : row) {
      cols[(size_t)o] = c;
      vals[(size_t)o] = v;
      ++o;
    }
  }
}

int mb_compute_matrix_elements_csr(mb_basis_t basis, mb_model_t model, int64_t* nnz,
                                   int64_t* row_ptr, int64_t* col_idx, double* values) {
  return guard([&] {
    MB_REQUIRE(basis && model && nnz, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(model->L == basis->L, MB_ERR_DIM_MISMATCH, "model sites and basis orbitals differ");
    require_device();
    mb_op_s tmp;
    tmp.precision = MB_PREC_F64;
    struct Cleanup {
      mb_op_s& o;
      ~Cleanup() {
        for (void* p : o.allocations) cudaFree(p);
      }
    } cleanup{tmp};
    if (basis->all_sz()) {
      MB_REQUIRE(!model->momentum && !model->current, MB_ERR_INVALID_ARG,
                 "an all-spin-projection basis takes the real-space model");
      cudaStream_t st = 0;
      const int64_t dim = basis->dim;
      DevBuf cnt(sizeof(int32_t) * (size_t)std::max<int64_t>(dim, 1));
      std::vector<mb_basis_s> secs;
      std::vector<std::unique_ptr<mb_op_s>> ops;
      std::vector<int32_t*> perms;
      for (size_t blk = 0; blk < basis->sz_nup.size(); ++blk) {
        secs.push_back(sector_of(basis, blk));
        ops.push_back(std::make_unique<mb_op_s>());
        ops.back()->precision = MB_PREC_F64;
        build_op(ops.back().get(), &secs.back(), model);
        perms.push_back(upload(&tmp, block_perm(secs.back())));
        launch_csr_count(ops.back()->view, perms.back(), (int32_t*)cnt.p, st);
      }
      struct FreeOps {
        std::vector<std::unique_ptr<mb_op_s>>& o;
        ~FreeOps() {
          for (auto& p : o) free_op_memory(p.get());
        }
      } free_ops{ops};
      std::vector<int32_t> hc((size_t)dim);
      if (dim) MB_CUDA(cudaMemcpy(hc.data(), cnt.p, sizeof(int32_t) * (size_t)dim, cudaMemcpyDeviceToHost));
      std::vector<int64_t> rp((size_t)dim + 1, 0);
      for (int64_t i = 0; i < dim; ++i) rp[(size_t)i + 1] = rp[(size_t)i] + hc[(size_t)i];
      const int64_t total = rp[(size_t)dim];
      if (!col_idx) {
        *nnz = total;
        if (row_ptr) std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
        return;
      }
      MB_REQUIRE(*nnz >= total, MB_ERR_CAPACITY, "nnz capacity smaller than the matrix");
      MB_REQUIRE(row_ptr && values, MB_ERR_INVALID_ARG, "NULL row_ptr or values");
      DevBuf drp(sizeof(int64_t) * rp.size()), dci(sizeof(int64_t) * (size_t)std::max<int64_t>(total, 1)),
          dv(sizeof(double) * 2 * (size_t)std::max<int64_t>(total, 1));
      MB_CUDA(cudaMemcpy(drp.p, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice));
      for (size_t blk = 0; blk < ops.size(); ++blk)
        launch_csr_fill(ops[blk]->view, perms[blk], (const int64_t*)drp.p, (int64_t*)dci.p,
                        (double*)dv.p, st);
      std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
      MB_CUDA(cudaMemcpy(col_idx, dci.p, sizeof(int64_t) * (size_t)total, cudaMemcpyDeviceToHost));
      MB_CUDA(cudaMemcpy(values, dv.p, sizeof(double) * 2 * (size_t)total, cudaMemcpyDeviceToHost));
      *nnz = total;
      return;
    }
    if (basis->momentum() || model->momentum) {
      // a momentum sector, or the whole basis as the union of its sectors
      // (rows and columns mapped to the whole basis's reference ranks)
      MB_REQUIRE(basis->momentum() || !model->current, MB_ERR_INVALID_ARG,
                 "the current operator maps between sectors: use "
                 "mb_compute_rectangular_matrix_elements_csr");
      std::vector<int64_t> rp, cols;
      std::vector<double> vals;
      if (basis->momentum()) {
        momentum_csr(basis, model, rp, cols, vals);
      } else {
        const int64_t dim = basis->dim;
        std::vector<std::vector<std::pair<int64_t, double>>> rows((size_t)dim);
        for (auto& sec : momentum_sectors(basis, model)) {
          std::vector<int64_t> srp, scol;
          std::vector<double> sval;
          momentum_csr(sec.get(), model, srp, scol, sval);
          for (int64_t i = 0; i < sec->dim; ++i) {
            auto& row = rows[(size_t)sec->kfull[(size_t)i]];
            for (int64_t k = srp[(size_t)i]; k < srp[(size_t)i + 1]; ++k)
              row.push_back({sec->kfull[(size_t)scol[(size_t)k]], sval[(size_t)k]});
          }
        }
        rp.assign((size_t)dim + 1, 0);
        for (int64_t i = 0; i < dim; ++i) {
          auto& row = rows[(size_t)i];
          std::sort(row.begin(), row.end());
          rp[(size_t)i + 1] = rp[(size_t)i] + (int64_t)row.size();
        }
        cols.resize((size_t)rp[(size_t)dim]);
        vals.resize((size_t)rp[(size_t)dim]);
        for (int64_t i = 0; i < dim; ++i) {
          int64_t o = rp[(size_t)i];
          for (const auto& [c, v] : rows[(size_t)i]) {
            cols[(size_t)o] = c;
            vals[(size_t)o] = v;
            ++o;
          }
        }
      }
      const int64_t total = rp.back();
      if (!col_idx) {
        *nnz = total;
        if (row_ptr) std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
        return;
      }
      MB_REQUIRE(*nnz >= total, MB_ERR_CAPACITY, "nnz capacity smaller than the matrix");
      MB_REQUIRE(row_ptr && values, MB_ERR_INVALID_ARG, "NULL row_ptr or values");
      for (int64_t k = 0; k < total; ++k) {
        col_idx[k] = cols[(size_t)k];
        values[2 * k] = vals[(size_t)k];
        values[2 * k + 1] = 0.0;
      }
      std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
      *nnz = total;
      return;
    }
    build_op(&tmp, basis, model);
    ensure_perm(&tmp);
    const int64_t dim = tmp.dim;
    cudaStream_t st = 0;
    DevBuf cnt(sizeof(int32_t) * (size_t)dim);
    launch_csr_count(tmp.view, tmp.perm, (int32_t*)cnt.p, st);
    std::vector<int32_t> hc((size_t)dim);
    MB_CUDA(cudaMemcpy(hc.data(), cnt.p, sizeof(int32_t) * (size_t)dim, cudaMemcpyDeviceToHost));
    std::vector<int64_t> rp((size_t)dim + 1, 0);
    for (int64_t i = 0; i < dim; ++i) rp[(size_t)i + 1] = rp[(size_t)i] + hc[(size_t)i];
    const int64_t total = rp[(size_t)dim];
    if (!col_idx) {
      *nnz = total;
      if (row_ptr) std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
      return;
    }
    MB_REQUIRE(*nnz >= total, MB_ERR_CAPACITY, "nnz capacity smaller than the matrix");
    MB_REQUIRE(row_ptr && values, MB_ERR_INVALID_ARG, "NULL row_ptr or values");
    DevBuf drp(sizeof(int64_t) * rp.size()), dci(sizeof(int64_t) * (size_t)std::max<int64_t>(total, 1)),
        dv(sizeof(double) * 2 * (size_t)std::max<int64_t>(total, 1));
    MB_CUDA(cudaMemcpy(drp.p, rp.data(), sizeof(int64_t) * rp.size(), cudaMemcpyHostToDevice));
    launch_csr_fill(tmp.view, tmp.perm, (const int64_t*)drp.p, (int64_t*)dci.p, (double*)dv.p, st);
    std::memcpy(row_ptr, rp.data(), sizeof(int64_t) * rp.size());
    MB_CUDA(cudaMemcpy(col_idx, dci.p, sizeof(int64_t) * (size_t)total, cudaMemcpyDeviceToHost));
    MB_CUDA(cudaMemcpy(values, dv.p, sizeof(double) * 2 * (size_t)total, cudaMemcpyDeviceToHost));
    *nnz = total;
  });
}

int mb_lanczos_pass_one(mb_op_t op, const void* b_dev, int order, int64_t k, double scale,
                        double* alphas, double* betas, int64_t* steps, double* b_norm) {
  return guard([&] {
    MB_REQUIRE(op && b_dev && alphas && steps && b_norm, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(k >= 0, MB_ERR_INVALID_ARG, "k must be >= 0");
    check_order(order);
    cudaStream_t st = 0;
    Krylov kr(op, st);
    DevBuf bt(kr.vb);
    to_tensor(op, b_dev, bt.p, order, st);
    std::vector<double> a, b;
    const int64_t m = kr.pass_one(bt.p, k, scale, a, b, *b_norm, false, 0.0, 0);
    std::copy(a.begin(), a.end(), alphas);
    if (betas) std::copy(b.begin(), b.end(), betas);
    *steps = m;
  });
}

int mb_lanczos_pass_two(mb_op_t op, const void* b_dev, int order, double scale,
                        const double* alphas, const double* betas, int64_t steps, double b_norm,
                        const double* y, void* x_dev) {
  return guard([&] {
    MB_REQUIRE(op && b_dev && x_dev, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(steps == 0 || (alphas && y), MB_ERR_INVALID_ARG, "NULL coefficients");
    MB_REQUIRE(steps <= 1 || betas, MB_ERR_INVALID_ARG, "NULL betas");
    check_order(order);
    cudaStream_t st = 0;
    Krylov kr(op, st);
    DevBuf bt(kr.vb), xt(kr.vb);
    to_tensor(op, b_dev, bt.p, order, st);
    std::vector<double> a(alphas, alphas + steps), b;
    if (steps > 1) b.assign(betas, betas + steps - 1);
    std::vector<std::complex<double>> yy((size_t)steps);
    for (int64_t i = 0; i < steps; ++i) yy[(size_t)i] = {y[2 * i], y[2 * i + 1]};
    kr.pass_two(bt.p, steps, scale, a, b, b_norm, yy, xt.p);
    from_tensor(op, xt.p, x_dev, order, st);
    MB_CUDA(cudaStreamSynchronize(st));
  });
}

int mb_find_min_eigenpair(mb_op_t op, int64_t k, const void* seed_dev, int order,
                          const mb_lanczos_opts* opts, double* e0, void* vec_dev,
                          int64_t* steps_out) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    eigenpair(op, k, seed_dev, order, opts, -1.0, e0, vec_dev, steps_out);
  });
}

int mb_find_max_eigenpair(mb_op_t op, int64_t k, const void* seed_dev, int order,
                          const mb_lanczos_opts* opts, double* e_max, void* vec_dev,
                          int64_t* steps_out) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    eigenpair(op, k, seed_dev, order, opts, 1.0, e_max, vec_dev, steps_out);
  });
}

int mb_time_evolve(mb_op_t op, const void* psi0_dev, int order, double t, int64_t krylov_steps,
                   int imaginary, void* out_dev) {
  return guard([&] {
    MB_REQUIRE(op, MB_ERR_INVALID_ARG, "NULL operator");
    evolve(op, psi0_dev, order, t, krylov_steps, imaginary, out_dev);
  });
}

int mb_time_evolve_steps(mb_op_t op, void* psi_dev, int order, double t0, double t1, double dt,
                         int64_t krylov_steps) {
  return guard([&] {
    MB_REQUIRE(op && psi_dev, MB_ERR_INVALID_ARG, "NULL argument");
    if (dt == 0.0 || (t1 - t0) == 0.0) return;
    const double direction = (t1 >= t0) ? 1.0 : -1.0;
    dt = std::fabs(dt) * direction;
    double t = t0;
    DevBuf tmp(elem_bytes(op->precision) * (size_t)op->dim);
    while ((direction > 0 && t < t1) || (direction < 0 && t > t1)) {
      const double step = direction > 0 ? std::min(dt, t1 - t) : std::max(dt, t1 - t);
      evolve(op, psi_dev, order, step, krylov_steps, 0, tmp.p);
      MB_CUDA(cudaMemcpy(psi_dev, tmp.p, tmp.bytes, cudaMemcpyDeviceToDevice));
      t += step;
    }
  });
}

int mb_kpm_dos_moments(mb_op_t op, int64_t n_moments, int64_t n_probes, uint64_t seed,
                       double e_min, double e_max, double padding, double* mu) {
  return guard([&] {
    MB_REQUIRE(op && mu, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(n_moments >= 1 && n_probes >= 1, MB_ERR_INVALID_ARG,
               "need at least one moment and one probe");
    MB_REQUIRE(e_max > e_min, MB_ERR_INVALID_ARG, "e_max must exceed e_min");
    const double a = (e_max - e_min) / 2.0 * (1.0 + padding);  // rescaling.h:33-38
    const double b = (e_max + e_min) / 2.0;
    if (op->precision == MB_PREC_Q64) {
      q_kpm_dos_moments(op, n_moments, n_probes, seed, a, b, mu);
      return;
    }
    cudaStream_t st = 0;
    const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
    DevBuf t0(vb), t1(vb);
    const int ga = apply_grid(op->view, op->precision), gb = blas_grid(op->dim);
    Reducer red(std::max(ga, gb), 3);
    // Device-side moment sums per step, read once per probe.  Step s produces
    // T_{s+1}; moments up to n_moments-1 need T_j for j <= n_moments/2.
    const int64_t nsteps = std::max<int64_t>(n_moments / 2, 1);
    DevBuf dots(sizeof(double) * 3 * (size_t)nsteps);
    std::vector<double> acc((size_t)n_moments, 0.0), hd(3 * (size_t)nsteps);
    for (int64_t p = 0; p < n_probes; ++p) {
      void* cur = t0.p;   // T_n
      void* oth = t1.p;   // T_{n-1}, then T_{n+1}
      launch_fill_rng(op->precision, op->Du, op->Dd, seed, (uint32_t)(1 + p), 1, cur, st);
      // step 0: T1 = Ht T0 into oth; dots <T0,T1>, <T1,T1>, <T0,T0>
      launch_apply(op->view, op->precision, cur, oth, 1.0 / a, b, 0.0, nullptr, red.p(), 7, st);
      launch_reduce(red.p(), ga, 3, (double*)dots.p, st);
      std::swap(cur, oth);  // cur = T1, oth = T0
      for (int64_t s = 1; s < nsteps; ++s) {
        // T_{s+1} = 2 Ht T_s - T_{s-1}, written over T_{s-1}
        launch_apply(op->view, op->precision, cur, oth, 2.0 / a, b, -1.0, oth, red.p(), 3, st);
        launch_reduce(red.p(), ga, 3, (double*)dots.p + 3 * s, st);
        std::swap(cur, oth);
      }
      MB_CUDA(cudaMemcpyAsync(hd.data(), dots.p, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, st));
      MB_CUDA(cudaStreamSynchronize(st));
      // s=0: hd[0]=<T0,T1>=mu1, hd[1]=<T1,T1>, hd[2]=<T0,T0>=mu0
      // s>=1: hd[3s]=<T_s,T_{s+1}>, hd[3s+1]=<T_{s+1},T_{s+1}>
      const double mu0 = hd[2], mu1 = hd[0];
      std::vector<double> m((size_t)n_moments, 0.0);
      m[0] = mu0;
      if (n_moments > 1) m[1] = mu1;
      for (int64_t s = 1; 2 * s < n_moments; ++s) {
        m[(size_t)(2 * s)] = 2.0 * hd[3 * (size_t)(s - 1) + 1] - mu0;  // <T_s, T_s>
        if (2 * s + 1 < n_moments) m[(size_t)(2 * s + 1)] = 2.0 * hd[3 * (size_t)s] - mu1;
      }
      for (int64_t i = 0; i < n_moments; ++i) acc[(size_t)i] += m[(size_t)i];
    }
    const double norm = 1.0 / ((double)n_probes * (double)op->dim);
    for (int64_t i = 0; i < n_moments; ++i) mu[i] = acc[(size_t)i] * norm;
  });
}

int mb_kpm_projector_apply(mb_op_t op, int64_t expansion_order, double e_min, double e_max,
                           double e_fermi, double padding, const void* v_dev, int order,
                           void* out_dev) {
  return guard([&] {
    MB_REQUIRE(op && v_dev && out_dev, MB_ERR_INVALID_ARG, "NULL argument");
    MB_REQUIRE(expansion_order >= 0, MB_ERR_INVALID_ARG, "negative expansion order");
    check_order(order);
    const int64_t M = expansion_order;
    const double a = (e_max - e_min) / 2.0 * (1.0 + padding);
    const double b = (e_max + e_min) / 2.0;
    const double eps = (e_fermi - b) / a;
    const double pi = 3.14159265358979323846;
    std::vector<double> g((size_t)M + 1), mu((size_t)M + 1);
    mb_kpm_jackson_kernel(M, g.data());
    const double ac = std::acos(eps);  // projector_moments (kpm.h:51-61)
    mu[0] = 1.0 - ac / pi;
    for (int64_t m = 1; m <= M; ++m) mu[(size_t)m] = -2.0 * std::sin((double)m * ac) / ((double)m * pi);
    cudaStream_t st = 0;
    const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
    DevBuf tp(vb), tc(vb), res(vb);
    to_tensor(op, v_dev, tp.p, order, st);
    launch_axpby(op->precision, op->dim, g[0] * mu[0], 0.0, tp.p, 0.0, 0.0, res.p, nullptr, 0, st);
    if (M > 0) {
      launch_apply(op->view, op->precision, tp.p, tc.p, 1.0 / a, b, 0.0, nullptr, nullptr, 0, st);
      launch_axpby(op->precision, op->dim, g[1] * mu[1], 0.0, tc.p, 1.0, 0.0, res.p, nullptr, 0, st);
      void* prev = tp.p;
      void* cur = tc.p;
      for (int64_t m = 2; m <= M; ++m) {
        launch_apply(op->view, op->precision, cur, prev, 2.0 / a, b, -1.0, prev, nullptr, 0, st);
        std::swap(prev, cur);
        launch_axpby(op->precision, op->dim, g[(size_t)m] * mu[(size_t)m], 0.0, cur, 1.0, 0.0,
                     res.p, nullptr, 0, st);
      }
    }
    from_tensor(op, res.p, out_dev, order, st);
    MB_CUDA(cudaStreamSynchronize(st));
  });
}

int mb_estimate_bounds(mb_op_t op, int64_t power_iterations, double spectral_padding,
                       uint64_t seed, double* lower, double* upper) {
  return guard([&] {
    MB_REQUIRE(op && lower && upper, MB_ERR_INVALID_ARG, "NULL argument");
    cudaStream_t st = 0;
    const size_t vb = elem_bytes(op->precision) * (size_t)op->dim;
    DevBuf s0(vb), v(vb), w(vb);
    launch_fill_rng(op->precision, op->Du, op->Dd, seed, 0, 0, s0.p, st);
    const int ga = apply_grid(op->view, op->precision), gb = blas_grid(op->dim);
    Reducer red(std::max(ga, gb), 3);
    // power_method (linear_operator_utils.h:18-51) on scale*(H - shift)
    auto power = [&](double scale, double shift) -> double {
      if (power_iterations == 0) return 0.0;
      launch_dot(op->precision, op->dim, s0.p, s0.p, red.p(), st);
      double nrm = std::sqrt(red.fetch(gb, 3, st)[2]);
      if (nrm == 0.0) return 0.0;
      launch_axpby(op->precision, op->dim, 1.0 / nrm, 0.0, s0.p, 0.0, 0.0, v.p, nullptr, 0, st);
      double eig = 0.0;
      for (int64_t i = 0; i < power_iterations; ++i) {
        launch_apply(op->view, op->precision, v.p, w.p, scale, shift, 0.0, nullptr, red.p(), 7, st);
        const double* h = red.fetch(ga, 3, st);
        const double num = h[0], den = h[2], wn = std::sqrt(h[1]);
        if (den == 0.0) return 0.0;
        eig = num / den;
        if (wn == 0.0) return 0.0;
        launch_axpby(op->precision, op->dim, 1.0 / wn, 0.0, w.p, 0.0, 0.0, v.p, nullptr, 0, st);
      }
      return eig;
    };
    const double dominant = std::fabs(power(1.0, 0.0));
    if (dominant == 0.0) {
      *lower = *upper = 0.0;
      return;
    }
    const double shift = dominant * (1.0 + spectral_padding) + 2.220446049250313e-16;
    // Shifted: H + shift ; NegShift: -H + shift  (linear_operator.h:124-151)
    const double beta = power(1.0, -shift) - shift;
    const double alpha = shift - power(-1.0, shift);
    *lower = std::min(alpha, beta);
    *upper = std::max(alpha, beta);
  });
}

int mb_dot_re(mb_op_t op, const void* x_dev, const void* y_dev, double* out) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && y_dev && out, MB_ERR_INVALID_ARG, "NULL argument");
    const int gb = blas_grid(op->dim);
    Reducer red(gb, 3);
    launch_dot(op->precision, op->dim, x_dev, y_dev, red.p(), 0);
    *out = red.fetch(gb, 3, 0)[0];
  });
}

int mb_norm(mb_op_t op, const void* x_dev, double* out) {
  return guard([&] {
    MB_REQUIRE(op && x_dev && out, MB_ERR_INVALID_ARG, "NULL argument");
    const int gb = blas_grid(op->dim);
    Reducer red(gb, 3);
    launch_dot(op->precision, op->dim, x_dev, x_dev, red.p(), 0);
    *out = std::sqrt(red.fetch(gb, 3, 0)[2]);
  });
}

}  // extern "C"
