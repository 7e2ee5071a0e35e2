// Internal declarations shared by the engine's host and CUDA sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <condition_variable>
#include <cstdio>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/manybody_gb300.h"

namespace mb {

// ---------------------------------------------------------------------------
// Errors: internal code throws mb::Error; the C ABI converts it to a status
// and stores the message in the thread-local last-error string.
// ---------------------------------------------------------------------------
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& msg) : std::runtime_error(msg), status(s) {}
};

void set_last_error(const std::string& msg);

#define MB_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t mb_err_ = (call);                                                      \
    if (mb_err_ != cudaSuccess) {                                                      \
      int mb_code_ = mb_err_ == cudaErrorMemoryAllocation ? MB_ERR_OOM : MB_ERR_CUDA;  \
      throw ::mb::Error(mb_code_, std::string(#call) + ": " + cudaGetErrorString(mb_err_)); \
    }                                                                                  \
  } while (0)

#define MB_REQUIRE(cond, status, msg)                 \
  do {                                                \
    if (!(cond)) throw ::mb::Error((status), (msg));  \
  } while (0)

// Tolerance 1000 * eps (src/utils/tolerances.h:7-10).
constexpr double kTol = 1000.0 * 2.220446049250313e-16;
constexpr int kMaxOrbitals = 32;
constexpr int64_t kMaxSectorDim = int64_t(1) << 23;  // per spin; hop entries keep 24 bits

// ---------------------------------------------------------------------------
// Binomials and ranks (host + device).
// ---------------------------------------------------------------------------
struct Binom {
  int64_t c[kMaxOrbitals + 2][kMaxOrbitals + 2];
};
const Binom& binom_table();

__host__ __device__ inline int64_t binom_at(const Binom& B, int n, int k) {
  return (k < 0 || n < 0 || k > n) ? 0 : B.c[n][k];
}

// Colex rank of an n-bit combination: sum_i C(p_i, i), p_1 < ... < p_n the
// set bit positions.  Increasing integers with n bits set enumerate ranks
// 0, 1, 2, ... in order (Gosper's hack order).
__host__ __device__ inline int64_t colex_rank(const Binom& B, uint32_t m) {
  int64_t r = 0;
  int i = 1;
  while (m) {
#ifdef __CUDA_ARCH__
    int p = __ffs(m) - 1;
#else
    int p = __builtin_ctz(m);
#endif
    r += B.c[p][i];
    ++i;
    m &= m - 1;
  }
  return r;
}

// Reference index of the state (up, down) on L orbitals.  The reference
// enumerates states depth-first (src/algebra/basis.cpp:267-302): each level
// appends one occupied slot, slots taken orbital-major with Up before Down on
// the same orbital, children visited in (spin, orbital) order.  The index of a
// state is therefore the number of complete sequences that are
// lexicographically smaller under the element order (spin, orbital): at each
// position, every valid smaller alternative e' contributes
// C(#Up slots after e', Up left) * C(#Down slots after e', Down left).
__host__ __device__ inline int64_t reference_rank(const Binom& B, uint32_t up, uint32_t down,
                                                  int L) {
#ifdef __CUDA_ARCH__
  int ul = __popc(up), dl = __popc(down);
#else
  int ul = __builtin_popcount(up), dl = __builtin_popcount(down);
#endif
  int back_orb = -1, back_spin = 1;
  int64_t r = 0;
  for (int o = 0; o < L; ++o) {
    for (int s = 0; s < 2; ++s) {
      if (!(((s ? down : up) >> o) & 1u)) continue;
      if (ul > 0) {
        const int hi = (s == 0) ? o : L;
        for (int op = back_orb + 1; op < hi; ++op)
          r += binom_at(B, L - 1 - op, ul - 1) * binom_at(B, L - op, dl);
      }
      if (s == 1) {
        for (int op = back_orb + (back_spin == 1 ? 1 : 0); op < o; ++op)
          r += binom_at(B, L - 1 - op, ul) * binom_at(B, L - 1 - op, dl - 1);
      }
      if (s == 0) --ul; else --dl;
      back_orb = o;
      back_spin = s;
    }
  }
  return r;
}

// Reference index of the state (up, down) in the basis of all spin
// projections, with_fixed_particle_number (src/algebra/basis.cpp:69-89,
// 248-266): the same depth-first enumeration without the per-spin counts, so
// the index counts the sequences of occupied slots (orbital-major, Up before
// Down) that are lexicographically smaller under the element order (spin,
// orbital).  At each position every valid smaller alternative e' contributes
// C(#slots after e', particles left), where the slots after (o', Up) are
// 1 + 2 (L-1-o') and after (o', Down) are 2 (L-1-o').
__host__ __device__ inline int64_t reference_rank_all(const Binom& B, uint32_t up, uint32_t down,
                                                      int L) {
#ifdef __CUDA_ARCH__
  const int n = __popc(up) + __popc(down);
#else
  const int n = __builtin_popcount(up) + __builtin_popcount(down);
#endif
  int64_t r = 0;
  int t = 0, last_o = -1, last_s = 1;
  for (int o = 0; o < L; ++o) {
    for (int s = 0; s < 2; ++s) {
      if (!(((s ? down : up) >> o) & 1u)) continue;
      const int rem = n - t - 1;
      for (int s2 = 0; s2 <= s; ++s2) {
        const int hi = s2 < s ? L : o;
        for (int o2 = 0; o2 < hi; ++o2) {
          if (!(o2 > last_o || (o2 == last_o && s2 > last_s))) continue;
          r += binom_at(B, (s2 == 0 ? 1 : 0) + 2 * (L - 1 - o2), rem);
        }
      }
      ++t;
      last_o = o;
      last_s = s;
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// Host objects behind the opaque handles.
// ---------------------------------------------------------------------------
struct SpinSector {
  int L = 0, n = 0;
  int64_t D = 0;
  std::vector<uint32_t> masks;  // colex rank -> occupation mask
};

}  // namespace mb

struct mb_basis_s {
  int L = 0, n_up = 0, n_down = 0;
  int64_t dim = 0;
  mb::SpinSector up, down;
  // A total-momentum sector (with_fixed_particle_number_spin_momentum): its
  // states' masks in reference order, their full-(N_up, N_down)-sector
  // reference ranks (ascending), the lattice and the momentum.
  std::vector<int64_t> kdims, kvec;
  std::vector<uint32_t> kup, kdown;
  std::vector<int64_t> kfull;
  bool momentum() const { return !kdims.empty(); }
  // All spin projections (with_fixed_particle_number): the sectors N_up =
  // sz_nup[b], N_down = particles - N_up, concatenated in the tensor layout
  // (block b at sz_off[b], its own r_up * D_down + r_down inside).
  int particles = 0;
  std::vector<int> sz_nup;
  std::vector<int64_t> sz_off;
  bool all_sz() const { return !sz_nup.empty(); }
};

struct mb_model_s {
  std::vector<int64_t> dims;
  int L = 0;
  double t = 0.0, u = 0.0;
  bool has_hop = false, has_u = false;
  // Undirected bonds a < b with their multiplicity (1, or 2 when a lattice
  // dimension of size 2 lists the pair twice).
  struct Bond { int a, b, mult; };
  std::vector<Bond> bonds;
  // self_mult[i] = number of hopping(i, i) calls (a dimension of size 1).
  std::vector<int> self_mult;
  int64_t n_terms = 0;
  // The momentum-space model (HubbardModelMomentum): dispersion per orbital
  // and U/N, each 0 where the expression's 1000 eps zero drop removes it.
  // For a current operator J_d(Q) (current = true) eps holds the velocity
  // v_d(k) per orbital instead, with the transfer Q and the direction d.
  bool momentum = false;
  std::vector<double> eps;
  double u_over_n = 0.0;
  bool current = false;
  std::vector<int64_t> transfer;
  int direction = 0;
};

namespace mb {

// Hop table of one spin sector: CSR over colex ranks.  Entry =
// (target_rank << 8) | code; code bit0 = negative sign, bit1 = doubled bond.
// The element <target|c+_x c_y|source> of one bond is
// (-1)^popcount(source & bits strictly between x and y).
struct HopTable {
  std::vector<int32_t> off;
  std::vector<uint32_t> ent;
  int max_degree = 0;
  std::vector<double> self_energy;  // per state: sum over self bonds of -2t*mult*occupation
  bool has_self = false;
};
HopTable build_hop_table(const SpinSector& s, const mb_model_s& m);

// The masks of one spin sector (n of L orbitals) in colex order.
SpinSector make_spin_sector(int L, int n);

// Reverse Cuthill-McKee order of the states of a hop table (BFS from a
// low-degree state, neighbours by increasing degree, reversed).
std::vector<int32_t> rcm_order(const HopTable& t, int64_t D);

// Largest eigenvalue of the symmetric tridiagonal matrix (a[0..m), b[0..m-1)).
double tridiag_max_eig(const double* a, const double* b, int m);

// Steps of a finished Lanczos run (on an operator whose extremal eigenvalue
// sought is the largest) to build the Ritz vector from.  Without full re-
// orthogonalisation, and with FP32 vectors early, the recurrence loses
// orthogonality once that Ritz value has converged, and some steps later a
// second copy of it appears in T_m; a Ritz vector from T_m past that point
// can be a near-cancelling mix of the two copies.  Returns the first
// checkpoint k (multiples of `every`) whose largest Ritz value moved by at
// most tol * |value| since the previous checkpoint, else the first that
// moved by at most 1e-7 * |value|, else m.
int ritz_vector_steps(const std::vector<double>& a, const std::vector<double>& b, int m,
                      int every, double tol);

// Hop lists of the fused block-floating-point apply, signs resolved ahead:
// per state the target ranks with the positive hops first and doubled bonds
// listed twice (so the kernel needs neither a sign nor a weight per hop).
struct SignedLists {
  std::vector<uint32_t> list;  // target ranks
  std::vector<int32_t> off;    // [D+1]
  std::vector<int32_t> pos;    // [D] number of positive hops
  int max_len = 0;
};
SignedLists signed_lists(const HopTable& t, int64_t D);

// Sliced-ELL copy of a hop table over groups of 32 consecutive states:
// group g's slot j for lane l is ent[grp[2g] + 128 (j / 4) + 4 l + j % 4] =
// target | (negative << 31) (a lane loads four slots as one 16-byte word, a
// warp 512 contiguous bytes), doubled bonds listed twice, padding D + k (one
// of kSlicedPads zero elements past the row); grp[2g+1] = slots of group g,
// stored rounded up to a multiple of 4 with padding.
// Within a group each lane's entries are ordered (the hop sum does not
// depend on the order) so that in every slot the eight lanes of a quarter
// warp read distinct 16-byte shared-memory bank groups (index mod 8): a
// warp's 16-byte gather from the staged row then takes 4 wavefronts, not
// the ~8 of the hop order.  Padding takes a zero element in a free group.
constexpr int kSlicedPads = 8;

#ifdef __CUDACC__
// Apply shape prefetch = 1: before its down hops, a warp asks L2 for the
// up-hop operands of its column group g, the segments X[s_up[k], 32g .. 32g+31]
// (ES-byte elements, 32·ES bytes each), so they are on their way while the
// down hops run from shared memory.  Each lane takes one 128-byte line, so one
// instruction covers 32·128/(32·ES) segments; lines past the row's end are
// skipped, so every address stays inside the neighbour's row.
template <int ES>
__device__ __forceinline__ void prefetch_up_group(const void* x, const uint32_t* s_up, int nu,
                                                  int64_t g, int lane, uint32_t row_bytes) {
  constexpr int kLines = ES / 4;     // lines of one segment
  constexpr int kPer = 32 / kLines;  // segments one instruction covers
  const uint32_t lo = (uint32_t)g * (32u * ES) + (uint32_t)(lane % kLines) * 128u;
  if (lo >= row_bytes) return;
  const char* xg = static_cast<const char*>(x) + lo;
  for (int k = lane / kLines; k < nu; k += kPer)
    asm volatile("prefetch.global.L2 [%0];" ::"l"(xg + (uint64_t)s_up[k] * row_bytes));
}
#endif
struct SlicedTable {
  std::vector<uint32_t> ent;
  std::vector<int32_t> grp;
  std::vector<uint8_t> nneg;  // [D] negative entries per state
};
SlicedTable sliced_table(const HopTable& t, int64_t D);
// The same table with 16-bit entries (index | negative << 15; D + kSlicedPads
// must stay below 2^15), a lane's slots 8i..8i+7 in one 16-byte word.
struct SlicedTable16 {
  std::vector<uint16_t> ent;
  std::vector<int32_t> grp;
};
constexpr int64_t kSliced16MaxD = (int64_t(1) << 15) - kSlicedPads;
SlicedTable16 sliced_table16(const SlicedTable& s, int64_t D);

// Left fold U + U + ... (k terms), the order-independent value the reference
// accumulates for k doubly occupied sites (matrix_elements.h:85-96).
std::vector<double> u_fold_table(double u, bool has_u, int L);

// Device-side view of an operator (POD; passed to kernels by value).
struct OpView {
  int64_t Du, Dd, dim;
  int L;
  const uint32_t* up_mask;
  const uint32_t* dn_mask;
  const int32_t* up_off;
  const uint32_t* up_ent;
  const int32_t* dn_off;
  const uint32_t* dn_ent;
  const double* u_fold;     // [L+1]
  const double* self_up;    // [Du] or nullptr
  const double* self_dn;    // [Dd] or nullptr
  const float* u_fold_f;    // float copies for complex64 operators
  const float* self_up_f;
  const float* self_dn_f;
  // Row processing order of the fused applies (reverse Cuthill-McKee of the
  // up-hop graph): rows in flight together share more neighbour rows in L2.
  const int32_t* row_sched;
  // Sign-resolved hop lists of the fused block-floating-point apply (see
  // SignedLists / SlicedTable): up hops by row, down hops sliced by column.
  const uint32_t* up_list;
  const int32_t* up_loff;
  const int32_t* up_lpos;
  const uint32_t* dn_sell;
  const int32_t* dn_sgrp;
  const uint8_t* dn_nneg;  // per down state: number of negative hops (doubled twice)
  // The same sliced table for the up sector (the column pass of the two-pass
  // applies gathers up hops from a staged column); shares the down table's
  // memory when the two sectors are the same.
  const uint32_t* up_sell;
  const int32_t* up_sgrp;
  const uint8_t* up_nneg;
  // 16-bit copies of the two sliced tables (sectors below 32760 states; else
  // nullptr): entry = index | negative << 15, a lane's slots 8i..8i+7 in one
  // 16-byte word, group g at sgrp16[2g] with sgrp16[2g+1] slots.
  const uint16_t* dn_sell16;
  const int32_t* dn_sgrp16;
  const uint16_t* up_sell16;
  const int32_t* up_sgrp16;
  // Kernel shape of the fused applies (mb_apply_shape): CTAs sharing one row
  // (each stages the row and takes every split-th column group) and the
  // sliced-table entry width (32 or 16 bits).
  int row_split;
  int table_bits;
  // 1: before its down hops, each warp prefetches the up-hop lines of its
  // column group into L2 (prefetch_up_group)
  int up_prefetch;
  // 1: each warp copies its next column group's down-table words into a
  // warp-private shared buffer (cp.async) while it finishes the current one
  // (MB_PREC_Q64 row-staged applies where it fits); dn_max_words = the most
  // 16-byte words (four 32-bit slots each) of one group.
  int table_stage;
  int dn_max_words;
  int max_up_list;
  // Operators made from a sparse matrix instead of a lattice (mb_op_create_csr):
  // CSR on the device, values complex128 (and complex64 copies for MB_PREC_F32).
  const int64_t* csr_row;
  const int32_t* csr_col;
  const double2* csr_val;
  const float2* csr_val_f;
  // Signed-column form (csr_val == nullptr): an entry is +-csr_off by bit 31
  // of its column, plus a separate diagonal (the momentum-sector operators).
  const double* csr_diag;
  double csr_off;
  // lanes a CSR row (4, 8, 16 or 32; 0: the precision's default), chosen by
  // the apply autotuner
  int csr_lanes;
  // Block-diagonal operators (all spin projections): n_blocks sub-views on
  // consecutive slices of the vector, sub_off[b] their element offsets (host
  // arrays; launch_apply loops over them).
  int n_blocks;
  const OpView* sub;
  const int64_t* sub_off;
  double t;
  int max_up_degree;
  int max_dn_degree;
};

// Fills the tables of the fused applies (row schedule, sign-sorted up lists,
// sliced down table) into v; `upload` copies host bytes to the device and
// returns the device address.
// Engine slot modes (device side of mb_engine.cu's batched solves).
enum EngMode { kEngIdle = 0, kEngLanczos = 1, kEngReplay = 2, kEngCheb = 3 };

// One large engine slot applied by the fused complex64 kernel: device
// addresses of the slot's step state (read every step) and its fixed data.
struct EngFusedArgs {
  const int* k;
  const int* mode;
  const int* kmax;
  const int* steps;
  const double* beta;   // beta[k - 1] scales v_prev
  const float* ufold;   // [L + 1] U fold of the slot
  const float* self_up; // self energies of a size-1 dimension (t-scaled), or nullptr
  const float* self_dn;
  float2* buf[3];       // v_prev = buf[k % 3], v = buf[(k + 1) % 3], w = buf[(k + 2) % 3]
  const float* cheb_a;  // Chebyshev rescaling (H - b) / a of the current probe
  const float* cheb_b;
  float t, scale;
  double* part;         // per-item partials of the engine (Re<v,w>)
  double* part2;        // (<w,w>)
  int item0, n_items;   // the slot's item range
  double* scratch;      // [blocks * 3] block partials
};
// Launches the slot's step (apply + partial placement) on `st`; graph-safe
// once prepare_eng_fused() has run (outside any capture).
void prepare_eng_fused();
void launch_eng_fused(const OpView& v, const EngFusedArgs& a, cudaStream_t st);
int eng_fused_blocks(const OpView& v);

using TableUpload = std::function<const void*(const void* host, size_t bytes)>;
void fill_fused_tables(OpView& v, const HopTable& tu, const HopTable& td, int64_t Du, int64_t Dd,
                       const TableUpload& upload);

}  // namespace mb

struct mb_op_s {
  int device = 0;
  int precision = MB_PREC_F64;
  int L = 0, n_up = 0, n_down = 0;
  int64_t Du = 0, Dd = 0, dim = 0;
  double t = 0.0, u = 0.0;
  mb::OpView view{};
  bool natural_order = false;      // a sparse-matrix operator: reference order = its own index
  std::vector<std::unique_ptr<mb_op_s>> subs;  // blocks of an all-spin-projection operator
  std::vector<mb::OpView> sub_views;
  std::vector<int64_t> sub_offsets;
  std::vector<void*> allocations;  // device buffers owned by the op
  int32_t* perm = nullptr;         // tensor -> reference index (lazy)
  int32_t* iperm = nullptr;        // reference -> tensor index (lazy)
  std::mutex mu;
  std::mutex host_mu;  // host-buffer calls: the lane pool and the row groups
  std::mutex host_link_mu;  // host-buffer calls on page-locked vectors take turns
  // Pipelined host-buffer apply (lattice operators, reference order): the
  // rows in groups by the first reference index among their states, each
  // group in the row schedule's order, so that once groups 0..g are applied
  // the reference indices [0, host_ready[g]) are final; group g is
  // host_sched[host_row0[g], host_row0[g+1]).  Two non-blocking streams.
  int32_t* host_sched = nullptr;
  std::vector<int64_t> host_row0;
  std::vector<int64_t> host_ready;
  // Host-buffer calls run on lanes: a lane is a pair of non-blocking streams
  // (compute, copy) whose compute stream keys its own staging and scratch
  // buffers, so calls from several host threads overlap.  A call takes an
  // idle lane or makes one (at most kMaxHostLanes; more callers wait).
  struct HostLane {
    cudaStream_t comp = nullptr, copy = nullptr;
    // two page-locked bounce buffers for pageable host vectors (made on first
    // use): the calling thread copies one chunk while the copy engine moves
    // the other, so pageable transfers of concurrent calls do not queue
    // behind each other in the driver's own staging
    void* bounce[2] = {nullptr, nullptr};
    cudaEvent_t bev[2] = {nullptr, nullptr};
  };
  static constexpr int kMaxHostLanes = 8;
  std::vector<std::unique_ptr<HostLane>> host_lanes;
  std::vector<HostLane*> host_idle;
  std::condition_variable host_cv;
  struct Scratch {
    void* a = nullptr;  // tensor-order copies for reference-order calls
    void* b = nullptr;
    void* hx = nullptr;  // device staging for host-buffer calls
    void* hy = nullptr;
  };
  std::map<cudaStream_t, Scratch> scratch;
  // Block-floating-point (MB_PREC_Q64) operators.
  double q_wmax = 0.0;              // largest sum of |hop weights| of one state
  int q_qbits = 62;                 // mantissas kept below 2^q_qbits
  bool q_has_double = false;        // any bond of multiplicity 2
  std::vector<double> ufold_host;   // U fold table (host copy)
  // the plan's hop coefficient -q_t (lattice: t; signed-column CSR: -off) and
  // diagonal table ufold_host[0..q_L] (lattice: the U fold by double
  // occupancy; CSR: the diagonal's least and largest entries)
  double q_t = 0.0;
  int q_L = 0;
  struct QScratch {
    void* xq = nullptr;
    void* yq = nullptr;
    void* prm = nullptr;   // QParams
    int* ints = nullptr;   // [max exp, Ex, unused, unused]
  };
  // per stream: the up-hop sums of the two-pass apply (dim elements)
  std::map<cudaStream_t, void*> ups_scratch;
  // Kernel shape of the lattice apply (mb_op_set_apply_shape / the autotuner):
  // 1 = one pass, 2 = column pass for the up hops, then the row pass.
  int apply_passes = 1;
  // (lattice, N_up, N_down, precision) of a lattice operator: the autotuner's
  // cache key ("" for operators it does not tune)
  std::string tune_key;
  std::map<cudaStream_t, QScratch> qscratch;
};

namespace mb {

// Flat orbital index of momentum k + sign * q on a periodic lattice (first
// dimension fastest).
int64_t momentum_add(int64_t k, int64_t q, int sign, const std::vector<int64_t>& dims);

// A momentum sector's Hamiltonian on the device (see mb_kernels.cu): the
// states, the momentum arithmetic of the lattice and the model's numbers.
struct MomTables {
  int64_t n;
  int L, n_up, n_down;
  const uint32_t* up;     // masks, reference order
  const uint32_t* dn;
  const int64_t* full;    // full-sector reference ranks, ascending
  const double* eps;      // [L]
  const uint8_t* kadd;    // [L*L]: orbital of momentum k + q
  const uint8_t* ksub;    // [L*L]: orbital of momentum k - q
  double u_over_n;
};
// Per row: the diagonal (0 when dropped) and the number of off-diagonal
// entries; then the off-diagonal columns (index | negative << 31).
void launch_mom_count(const MomTables& m, int32_t* count, double* diag, cudaStream_t st);
void launch_mom_fill(const MomTables& m, const int64_t* row_ptr, int32_t* col, cudaStream_t st);

// Kernel launchers (mb_kernels.cu).  All asynchronous on `st`.
size_t elem_bytes(int precision);
void launch_apply(const OpView& v, int precision, const void* x, void* y, double scale,
                  double shift, double beta, const void* z, double* partials, int dot_mode,
                  cudaStream_t st);
int apply_grid(const OpView& v, int precision);
void launch_reduce(const double* partials, int nblocks, int ncomp, double* out, cudaStream_t st);
int blas_grid(int64_t n);
// y = a*x + b*y (complex coefficients); dots of the result if dot_mode.
void launch_axpby(int precision, int64_t n, double ar, double ai, const void* x, double br,
                  double bi, void* y, double* partials, int dot_mode, cudaStream_t st);
// partials for Re<x,y> (comp 0), Im<x,y> (comp 1), <y,y> (comp 2).
void launch_dot(int precision, int64_t n, const void* x, const void* y, double* partials,
                cudaStream_t st);
int multi_dot_grid(int64_t n);
// c[j] = <V_j, w> for j < m (complex, 2 comps each) -> partials [blocks][2m]
void launch_multi_dot(int vprec, int wprec, int64_t n, const void* V, int64_t ld, int m,
                      const void* w, double* partials, cudaStream_t st);
// w -= sum_j c[j] V_j ; c on device (interleaved complex), then <w,w> partials
void launch_multi_axpy(int vprec, int wprec, int64_t n, const void* V, int64_t ld, int m,
                       const double* c, void* w, double* partials, cudaStream_t st);
void launch_convert(int from_prec, int to_prec, int64_t n, const void* x, void* y,
                    cudaStream_t st);
void launch_gather(int precision, int64_t n, const int32_t* perm, const void* src, void* dst,
                   cudaStream_t st);   // dst[i] = src[perm[i]]
void launch_scatter(int precision, int64_t n, const int32_t* perm, const void* src, void* dst,
                    cudaStream_t st);  // dst[perm[i]] = src[i]
void launch_fill_rng(int precision, int64_t Du, int64_t Dd, uint64_t seed, uint32_t stream_id,
                     int phase, void* dst, cudaStream_t st);
void launch_perm(const OpView& v, int32_t* perm, cudaStream_t st);
void launch_csr_count(const OpView& v, const int32_t* perm, int32_t* row_count, cudaStream_t st);
void launch_csr_fill(const OpView& v, const int32_t* perm, const int64_t* row_ptr,
                     int64_t* col_idx, double* values, cudaStream_t st);
void upload_binomials(cudaStream_t st);
// tensor -> reference index table of an operator, built on first use
int32_t* op_perm(mb_op_s* op);
// reference -> tensor index table (inverse of op_perm), built on first use
int32_t* op_iperm(mb_op_s* op);
// first[r] = the smallest reference index of tensor row r's states
void launch_row_first(int64_t Du, int64_t Dd, const int32_t* perm, int32_t* first,
                      cudaStream_t st);
// row groups and streams of the pipelined host-buffer applies
void ensure_host_groups(mb_op_s* op);
// The result side of a pipelined host-buffer apply, on the operator's host
// streams: per row group, apply_rows(view of the group's rows) and
// gather(i0, i1, dst) (reference indices [i0, i1) of the result to dst) on the
// compute stream; each finished reference range goes from y_stage to y_host on
// the copy stream while later groups run.  Returns once y_host is written.
// Host <-> device copies of one lane: page-locked host memory by the copy
// engine directly; pageable memory chunk by chunk through the lane's bounce
// buffers.  lane_upload calls on_chunk(offset, length, event) once each chunk
// is queued (event: its transfer done, on the copy stream) and returns once
// the last chunk is queued; lane_download returns once dst holds the bytes
// (the copy stream must already wait for their producer).
bool host_pinned(const void* p);
void lane_upload(const mb_op_s::HostLane& lane, void* dst_dev, const void* src_host, size_t bytes,
                 size_t chunk_align,
                 const std::function<void(size_t, size_t, cudaEvent_t)>& on_chunk);
void lane_download(const mb_op_s::HostLane& lane, void* dst_host, const void* src_dev,
                   size_t bytes);
void host_groups_run(mb_op_s* op, const mb_op_s::HostLane& lane, size_t elem, void* y_host,
                     void* y_stage,
                     const std::function<void(const OpView&)>& apply_rows,
                     const std::function<void(int64_t, int64_t, void*)>& gather);

// CUDA events without timing, destroyed with the owner.
struct Events {
  std::vector<cudaEvent_t> ev;
  explicit Events(int n) : ev((size_t)n, nullptr) {
    for (auto& e : ev) MB_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  ~Events() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
  }
  Events(const Events&) = delete;
  Events& operator=(const Events&) = delete;
  cudaEvent_t operator[](int i) const { return ev[(size_t)i]; }
};
void launch_invert_perm(int64_t n, const int32_t* perm, int32_t* iperm, cudaStream_t st);

// FP64 refinement of ground-state estimates: Rayleigh-Ritz on the Krylov
// space span{x, Hx, H^2 x, ...} with FP64 vectors and arithmetic (Lanczos with
// full re-orthogonalisation), x complex128 in tensor order.  fp64_refine_many
// runs many problems in lockstep (one host wait per step for all) and writes
// each one's lowest Ritz value to e0.
struct RefineProblem {
  OpView v;
  const void* x;
  double e0;  // out
};
void fp64_refine_many(RefineProblem* probs, int count, cudaStream_t st);
double fp64_ritz_refine(const OpView& v, const void* x64, cudaStream_t st);
// the refinement's Krylov steps: at least kRefineMinSteps, then until the
// lowest Ritz value moves by at most kRefineSettle relative (the convergence
// level of the plain FP64 solver, well above the rounding of FP64 dot products
// over a sector), at most kRefineMaxSteps
constexpr int kRefineMinSteps = 3;
constexpr int kRefineMaxSteps = 8;
constexpr double kRefineSettle = 1e-12;

// Host tridiagonal eigensolver (implicit QL, mb_tridiag.cpp).
bool tridiag_eig(int n, std::vector<double>& d, const std::vector<double>& e,
                 std::vector<double>* z);

}  // namespace mb

namespace mb {

// Runs f and converts exceptions to an mb_status + thread-local message.
template <typename F>
int guard(F&& f) {
  try {
    f();
    return MB_OK;
  } catch (const Error& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return MB_ERR_OOM;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return MB_ERR_INVALID_ARG;
  }
}

}  // namespace mb
