/*
 * manybody_gb300.h -- C ABI of the GB300 exact-diagonalisation engine for the
 * fixed-(N_up, N_down) Hubbard model.
 *
 * The calling surface mirrors keyehzy/manybody's Basis / HubbardModel /
 * compute_matrix_elements / LinearOperator + Lanczos path.  Each entry point
 * names the reference interface it replaces (file:line within that project).
 *
 * Conventions
 *  - Every function returns an mb_status (MB_OK == 0).  On failure the
 *    calling thread's last-error string (mb_last_error) says why.  No C++
 *    exception crosses this boundary.
 *  - Vectors are interleaved complex numbers: complex128 ({double re, im})
 *    for MB_PREC_F64 / MB_PREC_Q64, complex64 ({float re, im}) for
 *    MB_PREC_F32.  "_dev" pointers are device memory on the current CUDA
 *    device, "_host" pointers host memory.  Buffers are owned by the caller.
 *  - Vector order: MB_ORDER_REFERENCE indexes a vector by the reference
 *    basis index (the order of FermionBasis::set); MB_ORDER_TENSOR indexes it
 *    by r_up * D_down + r_down, the engine's native layout (colex ranks of
 *    the up and down occupation masks).
 *  - Streams: a `stream` argument is a cudaStream_t passed as void* (NULL =
 *    the legacy default stream).  mb_op_apply may be called concurrently on
 *    one operator from several host threads with distinct streams and
 *    buffers (the reference calls LinearOperator::apply concurrently from
 *    OpenMP sample loops, examples/hubbard_momentum_optical_conductivity.cpp:351-400).
 */
#ifndef MANYBODY_GB300_H
#define MANYBODY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  MB_OK = 0,
  MB_ERR_INVALID_ARG = 1,  /* replaces the reference's assert()s (UB in Release) */
  MB_ERR_CAPACITY = 2,     /* sector or lattice larger than the engine supports */
  MB_ERR_ZERO_NORM = 3,    /* lanczos.h:92,138-144 "Input vector has zero norm" */
  MB_ERR_DIM_MISMATCH = 4, /* lanczos.h:138,186 dimension mismatch */
  MB_ERR_EIG_FAILED = 5,   /* lanczos.h:270, evolve_state.h:46 eig_sym failure */
  MB_ERR_OOM = 6,          /* device or host allocation failed */
  MB_ERR_TIMEOUT = 7,      /* a bounded device wait ran out */
  MB_ERR_CUDA = 8,         /* a CUDA runtime call failed */
  MB_ERR_NO_DEVICE = 9     /* no CUDA device / extension unusable */
} mb_status;

typedef enum { MB_ORDER_REFERENCE = 0, MB_ORDER_TENSOR = 1 } mb_order;

typedef enum {
  MB_PREC_F64 = 0, /* complex128 vectors, FP64 arithmetic */
  MB_PREC_F32 = 1, /* complex64 vectors, FP32 arithmetic */
  MB_PREC_Q64 = 2  /* complex128 at the boundary; block floating point with
                      64-bit integer mantissas and one exponent per vector
                      inside (exact integer hopping sums) */
} mb_precision;

typedef struct mb_basis_s* mb_basis_t;
typedef struct mb_model_s* mb_model_t;
typedef struct mb_op_s* mb_op_t;

/* ---- library ------------------------------------------------------------ */
int mb_version(void);
/* Thread-local text of the last error raised on this thread ("" if none). */
const char* mb_last_error(void);
/* Number of visible CUDA devices (0 without a GPU); never fails. */
int mb_device_count(int* count);
/* cudaMalloc / cudaFree / cudaMemcpy helpers for callers without the CUDA
 * runtime headers.  kind: 0 host->device, 1 device->host, 2 device->device. */
int mb_alloc(void** dev_ptr, size_t bytes);
int mb_free(void* dev_ptr);
int mb_memcpy(void* dst, const void* src, size_t bytes, int kind);
int mb_synchronize(void);

/* ---- basis: FermionBasis (src/algebra/fermion/basis.h, src/algebra/basis.h:12-76)
 * mb_basis_create_fixed_spin replaces
 *   BasisImpl::with_fixed_particle_number_and_spin (src/algebra/basis.cpp:91-126).
 * Same arguments; invalid combinations (odd N+Sz, |Sz|>N, more particles than
 * orbitals) return MB_ERR_INVALID_ARG where the reference asserts.  Orbitals
 * <= 32 and C(L,N_up), C(L,N_down) <= 2^23. */
int mb_basis_create_fixed_spin(int64_t orbitals, int64_t particles, int spin_projection,
                               mb_basis_t* out);
/* BasisImpl::with_fixed_particle_number (src/algebra/basis.cpp:69-89,248-266):
 * all spin projections for `particles` fermions, in the reference's index
 * order (its depth-first enumeration without per-spin counts).  Operators on
 * it (mb_op_create with a real-space model; MB_PREC_F64 / MB_PREC_F32) are
 * block diagonal: one (N_up, N_down) block per spin projection, each the
 * matrix-free kernel on its slice of the tensor layout (blocks by N_up
 * ascending).  mb_basis_sector reports n_up = n_down = -1. */
int mb_basis_create_fixed_number(int64_t orbitals, int64_t particles, mb_basis_t* out);
/* BasisImpl::with_fixed_particle_number_spin_momentum (src/algebra/basis.cpp:128-185,
 * 304-356): the states of one total momentum K on a periodic lattice of sizes
 * dims[0..ndim) (orbital k has coordinates k_d, first dimension fastest;
 * total momentum = sum of the occupied orbitals' coordinates mod the sizes),
 * in the reference's index order (its depth-first order filtered by K).
 * mb_basis_size / export / index_of work as for the full sector; the
 * permutation is the identity (operators on it use reference order). */
int mb_basis_create_momentum(const int64_t* dims, int ndim, int64_t particles,
                             int spin_projection, const int64_t* momentum, mb_basis_t* out);
int mb_basis_destroy(mb_basis_t basis);
/* basis.set.size() (compute_basis_size_spin, src/algebra/basis.cpp:39-50). */
int mb_basis_size(mb_basis_t basis, int64_t* dim);
int mb_basis_sector(mb_basis_t basis, int64_t* orbitals, int64_t* n_up, int64_t* n_down,
                    int64_t* dim_up, int64_t* dim_down);
/* The keys of basis.set in reference index order, as occupation bit masks
 * (bit o of up_masks[i] set <=> key i holds creation(Up, o)).  Host arrays of
 * mb_basis_size entries.  Replaces iterating FermionBasis::set. */
int mb_basis_export_reference_order(mb_basis_t basis, uint64_t* up_masks, uint64_t* down_masks);
/* IndexedHashSet::index_of (src/utils/indexed_hash_set.h:158-164) for the key
 * with these masks; MB_ERR_INVALID_ARG if the key is not in the basis
 * (IndexedHashSet::contains is false). */
int mb_basis_index_of(mb_basis_t basis, uint64_t up_mask, uint64_t down_mask, int64_t* index);
/* ref_of_tensor[r_up * D_down + r_down] = reference index (host array). */
int mb_basis_permutation(mb_basis_t basis, int64_t* ref_of_tensor);

/* ---- model: HubbardModel / 2D / 3D (src/algebra/fermion/model/hubbard_model.h:10-212)
 * dims = {L} (HubbardModel(t,u,L)), {Lx,Ly} (HubbardModel2D) or {Lx,Ly,Lz}
 * (HubbardModel3D); periodic, sites x + Lx*y + Lx*Ly*z (src/utils/index.h:69-88).
 * A lattice dimension of size 2 lists each bond twice and so hops with -2t,
 * as the reference's merged expression does (tests/algebra/test_model.cpp:58-74).
 * Coefficients with |c| < 1000*eps are dropped (src/utils/tolerances.h:7-10). */
int mb_hubbard_create(const int64_t* dims, int ndim, double t, double u, mb_model_t* out);
/* HubbardModelMomentum (src/algebra/fermion/model/hubbard_model_momentum.h:19-180):
 * H = sum_{k,s} eps(k) n_{k,s} + (U/N) sum_{k1,k2,q} c+_{k1+q,up} c+_{k2-q,dn}
 * c_{k2,dn} c_{k1,up}, eps(k) = -2t sum_d cos(2 pi k_d / L_d), on momentum
 * orbitals (same lattice indexing).  With a momentum-sector basis it gives
 * the sector's H: mb_compute_matrix_elements_csr (built on the GPU) and
 * mb_op_create (the sector's H kept on the device in signed-column sparse
 * form; reference order; MB_PREC_F64, MB_PREC_F32, or MB_PREC_Q64 with the
 * +-U/N entries summed exactly as integers and the diagonal as a per-row
 * fixed-point coefficient).  With a whole (N_up,
 * N_down) basis (mb_basis_create_fixed_spin) it gives the operator of the
 * reference's HubbardMomentumFactorized (src/numerics/
 * hubbard_momentum_factorized.h:32-249, t sum eps(k) n_k + (U/N) sum_q
 * rho_{q,up} rho_{-q,down}): block diagonal over the total momentum, one
 * sector operator per K, in the whole basis's reference order. */
int mb_hubbard_momentum_create(const int64_t* dims, int ndim, double t, double u,
                               mb_model_t* out);
int mb_model_destroy(mb_model_t model);
/* FermionExpression::size() of hamiltonian(): number of distinct terms. */
int mb_model_term_count(mb_model_t model, int64_t* n_terms);

/* ---- compute_matrix_elements<sp_cx_mat> (src/algebra/matrix_elements.h:74-105)
 * Builds H on the GPU as CSR in reference order (row i = basis key i; column
 * indices ascending), bit-identical to the reference's entries.  Two calls:
 * first with col_idx == NULL to get *nnz, then with arrays of that size
 * (row_ptr: dim+1 entries; values: interleaved complex128).  Host arrays. */
int mb_compute_matrix_elements_csr(mb_basis_t basis, mb_model_t model, int64_t* nnz,
                                   int64_t* row_ptr, int64_t* col_idx, double* values);

/* ---- the reference's sparse-matrix cache format ---------------------------- *
 * Hamiltonian caches are cereal binary archives of arma::sp_cx_mat
 * (src/utils/arma_cereal.h:9-30; written and read by
 * examples/hubbard_momentum_optical_conductivity.cpp:185-203): uint32 version
 * 0, uint64 n_rows, n_cols, n_nonzero, then per non-zero in column-major order
 * uint64 row, uint64 col and the value as two float64, little-endian.
 * CSR here: row_ptr n_rows+1 entries, col_idx and values (interleaved
 * complex128) nnz entries, host arrays.
 * Write: entries go out in column-major order.  Read: two calls, first with
 * row_ptr == NULL for the sizes; loading follows arma's t(row, col) = value
 * (a later duplicate wins, an explicit zero stores nothing), rows sorted by
 * column. */
int mb_cereal_write_csr(const char* path, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr,
                        const int64_t* col_idx, const double* values);
int mb_cereal_read_csr(const char* path, int64_t* n_rows, int64_t* n_cols, int64_t* nnz,
                       int64_t* row_ptr, int64_t* col_idx, double* values);

/* ---- operator: SparseComplexMatrixOperator (src/numerics/linear_operator.h:81-91)
 * replaced by a matrix-free operator on the GPU.  The operator holds the
 * sector tables on the device; it never stores H. */
int mb_op_create(mb_basis_t basis, mb_model_t model, int precision, mb_op_t* out);
/* SparseComplexMatrixOperator itself (src/numerics/linear_operator.h:81-91):
 * an operator from any square complex sparse matrix in CSR (host arrays, as
 * mb_cereal_read_csr gives them), applied on the GPU by a CSR kernel, for
 * Hamiltonians built elsewhere (the reference's cached momentum-space or
 * correlator matrices).  MB_PREC_F64 or MB_PREC_F32; its index order is the
 * matrix's own, so MB_ORDER_REFERENCE and MB_ORDER_TENSOR coincide.  Every
 * driver below takes it (apply, Lanczos, KPM, evolution); the Q64 and
 * allocation-free entry points take lattice operators only. */
int mb_op_create_csr(int64_t n, const int64_t* row_ptr, const int64_t* col_idx,
                     const double* values, int precision, mb_op_t* out);
int mb_op_destroy(mb_op_t op);
/* LinearOperator::dimension() (linear_operator.h:42). */
int mb_op_dimension(mb_op_t op, int64_t* dim);
int mb_op_precision(mb_op_t op, int* precision);
/* LinearOperator::apply (linear_operator.h:41): y = H x on device buffers.
 * Asynchronous on `stream`.  x and y must not overlap. */
int mb_op_apply(mb_op_t op, const void* x_dev, void* y_dev, int order, void* stream);
/* y = scale * (H - shift) x + beta * z, fused (z may be NULL when beta == 0).
 * Covers Negated (scale -1, linear_operator.h:93-105), Scaled, Shifted and
 * the Chebyshev step 2*Ht*T_n - T_{n-1} (kpm.h:222) in one pass. */
int mb_op_apply_affine(mb_op_t op, const void* x_dev, void* y_dev, double scale, double shift,
                       double beta, const void* z_dev, int order, void* stream);
/* apply() with host buffers: copies x in, applies, copies y out, then waits.
 * In reference order on a lattice operator the copies overlap the apply: rows
 * run in groups ordered by where their states first appear in the reference
 * order, and each finished prefix of y goes back while later groups run; a
 * page-locked x is read over the link by the kernel that scatters it.
 * Calls on one operator from several host threads overlap: each runs on its
 * own lane (two streams and its own staging buffers, about four vectors of
 * device memory, made on first use and kept with the operator; at most 8
 * lanes, further callers wait for one), with the bits a call alone gets.
 * Pageable vectors (an Armadillo vector's memory) pass through the lane's own
 * two 16 MiB page-locked bounce buffers; calls on page-locked vectors, each of
 * which runs the host link at its full rate alone, take turns. */
int mb_op_apply_host(mb_op_t op, const void* x_host, void* y_host, int order);

/* y = H x on device buffers in REFERENCE order, without allocating: no
 * cudaMalloc/cudaFree, no allocating library call.  No counterpart in the
 * reference.  For callers that cannot let the library allocate device memory
 * (a host framework that owns all device memory through its own pool, a
 * latency-critical loop that cannot afford cudaMalloc's implicit device
 * synchronisation).  mb_op_apply's permutation scratch comes instead from one
 * fixed 32 MiB array inside the library (two vectors of up to 1,048,576
 * complex128 elements); larger sectors return MB_ERR_CAPACITY.  The array is
 * part of the library's device code, which CUDA loads into a device lazily
 * (the default since CUDA 12.2): the first call on a device loads it there,
 * taking the 32 MiB on that device until the process exits, looks up the
 * array's address and uploads a small table, with the operator's device
 * current.  Make that first call during set-up, before any stream capture;
 * later calls allocate nothing.  MB_PREC_F64, MB_PREC_F32 and MB_PREC_Q64
 * operators (Q64 takes the steps of mb_op_apply on it: the same bits).  All
 * calls on a device share the array: calls that overlap on the GPU race;
 * serialise them. */
int mb_op_apply_noalloc(mb_op_t op, const void* x_dev, void* y_dev, void* stream);

/* ---- apply kernel shapes ------------------------------------------------- *
 * No counterpart in the reference.  How a lattice operator's H|psi> runs on
 * the GPU.  Every shape gives the same result bits on an MB_PREC_Q64
 * operator (its hop sums are exact integers in any order).  Shapes other than
 * the default {1, 1, 32} apply to MB_PREC_Q64 lattice operators.
 *  passes     1: one pass over the rows r_up; each row staged in shared
 *                memory for the down hops, the up hops read from x in global
 *                memory;
 *             2: first a column pass (each column r_down staged in shared
 *                memory, the up hops gathered there, their exact sums written
 *                to scratch: one vector per stream, allocated on first use),
 *                then the row pass adds them (sectors whose column fits);
 *  row_split  1, 2 or 4 CTAs share a row (each stages it and takes every
 *             row_split-th column group): fewer rows in flight, so the up-hop
 *             rows they read stay in L2;
 *  table_bits 32 or 16: width of the down/up hop-table entries (16 needs
 *             sectors below 32760 states per spin). */
typedef struct {
  int passes;
  int row_split;
  int table_bits;
  int prefetch;   /* 1: before its down hops, each warp asks L2 for the
                     up-hop lines of its column group, one 128-byte line a
                     lane (any lattice operator) */
  int table_stage; /* 1: each warp copies its next column group's down-table
                      words into its own shared buffer (cp.async) while it
                      finishes the current one (MB_PREC_Q64, one pass, 32-bit
                      entries, where the buffers fit beside the row) */
  int csr_lanes;  /* operators held as a sparse matrix (momentum sectors,
                     mb_op_create_csr): lanes a row, 4, 8, 16 or 32 (0: the
                     precision's default, 4 complex128 / 8 otherwise); must be
                     0 for lattice operators */
  int reserved[2];
} mb_apply_shape;
int mb_op_get_apply_shape(mb_op_t op, mb_apply_shape* shape);
int mb_op_set_apply_shape(mb_op_t op, const mb_apply_shape* shape);
/* The apply autotuner: times every candidate shape of the operator on the
 * live GPU (tensor-order device vectors, CUDA events on `stream`, median of 7
 * applies after 2 warm-up ones), keeps the fastest and returns it with its
 * time.  Choices are cached per (lattice, N_up, N_down, precision) for the
 * process: a later operator of the same sector takes the cached shape without
 * timing.  Operators without shapes (sparse matrix, block diagonal) keep the
 * default and report 0 ms.  Allocates two (Q64: three) vectors while it runs. */
int mb_op_autotune(mb_op_t op, void* stream, mb_apply_shape* chosen, double* best_ms);

/* ---- seeded start vectors ----------------------------------------------- *
 * v[i] = (u1, u2), u ~ U[-1,1) from Philox4x32-10 (Salmon et al., SC'11) with
 * key = seed and counter (i_lo, i_hi, stream, 0), where i is the TENSOR index
 * of the element; written in `order`.  Identical bits to the CPU oracle. */
int mb_fill_uniform(mb_op_t op, uint64_t seed, uint32_t stream_id, void* v_dev, int order,
                    void* stream);
/* v[i] = exp(i*2*pi*u), u ~ U[0,1) from the same generator (random phases). */
int mb_fill_phase(mb_op_t op, uint64_t seed, uint32_t stream_id, void* v_dev, int order,
                  void* stream);

/* ---- Lanczos (src/numerics/lanczos.h) ------------------------------------ */
typedef struct {
  int reorth;           /* 0: plain three-term recurrence (the reference's); 1: full
                           re-orthogonalisation (classical Gram-Schmidt against every
                           stored vector; a second pass when the first one takes ||w||
                           below 1/sqrt(2) of its norm, the DGKS test) */
  int basis_precision;  /* storage of the Krylov basis for reorth: MB_PREC_F64 or MB_PREC_F32;
                           -1 = F64 when it fits in free device memory, else F32 */
  double conv_tol;      /* > 0: stop early once the extremal Ritz value changes by
                           less than conv_tol * |E| between checks (0 = run k steps) */
  int check_every;      /* Ritz check period in steps when conv_tol > 0 (default 10) */
  int refine;           /* MB_PREC_F32 operators: 1 = finish with an FP64 Rayleigh-Ritz
                           refinement (FP64 Lanczos from the Ritz vector, each step
                           orthogonalised against all earlier ones by two Gram-Schmidt
                           passes: at least 3 steps, then until the lowest Ritz value
                           moves by at most 1e-12 relative, at most 8; a plain run that
                           used all k steps takes the vector from its first settled
                           checkpoint, before ghost copies of E0 form) */
} mb_lanczos_opts;

/* lanczos_pass_one (lanczos.h:130-175) on the operator scaled by `scale`
 * (1: H, -1: Negated<H> as find_min_eigenpair uses).  alphas[k], betas[k-1]
 * host arrays; *steps = decomposition steps taken. */
int mb_lanczos_pass_one(mb_op_t op, const void* b_dev, int order, int64_t k, double scale,
                        double* alphas, double* betas, int64_t* steps, double* b_norm);
/* lanczos_pass_two (lanczos.h:177-218): x = sum_j y_j v_j by re-running the
 * recurrence.  y is complex (interleaved re, im; `steps` entries). */
int mb_lanczos_pass_two(mb_op_t op, const void* b_dev, int order, double scale,
                        const double* alphas, const double* betas, int64_t steps, double b_norm,
                        const double* y, void* x_dev);
/* find_min_eigenpair (lanczos.h:283-290): Lanczos on Negated<H> from the given
 * seed vector (the reference draws an unseeded arma::randu seed,
 * linear_operator.h:26-32), eig of T, the Ritz vector.  Without
 * re-orthogonalisation pass one keeps its vectors while a tenth of the
 * device memory stays free and the Ritz vector is summed from them; pass two
 * replays the recurrence otherwise.  vec_dev
 * may be NULL.  steps_out (may be NULL) receives the Lanczos steps taken. */
int mb_find_min_eigenpair(mb_op_t op, int64_t k, const void* seed_dev, int order,
                          const mb_lanczos_opts* opts, double* e0, void* vec_dev,
                          int64_t* steps_out);
/* find_max_eigenpair (lanczos.h:246-281). */
int mb_find_max_eigenpair(mb_op_t op, int64_t k, const void* seed_dev, int order,
                          const mb_lanczos_opts* opts, double* e_max, void* vec_dev,
                          int64_t* steps_out);

/* ---- Krylov time evolution (src/numerics/evolve_state.h) ----------------- *
 * imaginary = 0: time_evolve_state, psi(t) = exp(-i t H) psi0 (:164-178);
 * imaginary = 1: imaginary_time_evolve_state, exp(-t H) psi0 (:186-195).
 * krylov_steps 0 means the reference default (30, EvolutionOptions :110-112). */
int mb_time_evolve(mb_op_t op, const void* psi0_dev, int order, double t, int64_t krylov_steps,
                   int imaginary, void* out_dev);
/* time_evolve_state_steps (evolve_state.h:204-231) from t0 to t1 by dt,
 * in place on psi_dev. */
int mb_time_evolve_steps(mb_op_t op, void* psi_dev, int order, double t0, double t1, double dt,
                         int64_t krylov_steps);

/* ---- KPM (src/numerics/kpm.h, src/numerics/rescaling.h) ------------------ *
 * Density-of-states Chebyshev moments mu[n] = (1/R) sum_r <r|T_n(Ht)|r> / D,
 * Ht = (H - b)/a with (a, b) = rescaling::from_bounds(e_min, e_max, padding)
 * (rescaling.h:33-38), R = n_probes random-phase vectors from
 * mb_fill_phase(seed, stream_id = 1 + probe).  Uses the doubling identities
 * mu_2n = 2<T_n|T_n> - mu_0, mu_2n+1 = 2<T_n+1|T_n> - mu_1 (n_moments/2
 * matvecs per probe).  The reference implements only the Fermi projector;
 * the DOS moments restate its Chebyshev recurrence (kpm.h:212-229). */
int mb_kpm_dos_moments(mb_op_t op, int64_t n_moments, int64_t n_probes, uint64_t seed,
                       double e_min, double e_max, double padding, double* mu);
/* jackson_kernel (kpm.h:19-30), lorentz_kernel (kpm.h:34-44). */
int mb_kpm_jackson_kernel(int64_t n, double* g);
int mb_kpm_lorentz_kernel(int64_t n, double lambda, double* g);
/* SparseKPMProjector(H, M, e_min, e_max, e_fermi, padding).apply(v)
 * (kpm.h:184-241) on a complex vector. */
int mb_kpm_projector_apply(mb_op_t op, int64_t expansion_order, double e_min, double e_max,
                           double e_fermi, double padding, const void* v_dev, int order,
                           void* out_dev);
/* estimate_bounds (src/numerics/linear_operator_utils.h:53-77) by power
 * iterations from the seeded vector (seed, stream_id 0). */
int mb_estimate_bounds(mb_op_t op, int64_t power_iterations, double spectral_padding,
                       uint64_t seed, double* lower, double* upper);

/* ---- block-floating-point vectors (MB_PREC_Q64 operators) ---------------- *
 * A Q64 vector is n pairs of int64 mantissas {re, im} (16 bytes per element,
 * like complex128) plus one int exponent E: element = (re + i im) * 2^E.
 * Mantissas stay below 2^bits (mb_q64_mantissa_bits), which leaves room for
 * the exact integer hop sums.  These entry points expose the engine's
 * internal vector format to drivers that keep many applies on the device;
 * they have no counterpart in the reference. */
int mb_q64_mantissa_bits(mb_op_t op, int* bits);
/* complex128 (order) -> Q64 in tensor order; *exponent receives E.  Waits. */
int mb_q64_from_f64(mb_op_t op, const void* x_dev, int order, void* xq_dev, int* exponent,
                    void* stream);
/* Q64 (tensor order) -> complex128 in `order` (correctly rounded).  Waits. */
int mb_q64_to_f64(mb_op_t op, const void* xq_dev, int exponent, int order, void* x_dev,
                  void* stream);
/* yq = H xq on Q64 vectors in tensor order; *y_exponent receives the output
 * exponent (known before the kernel runs).  Asynchronous on `stream`. */
int mb_op_apply_q64(mb_op_t op, const void* xq_dev, int x_exponent, void* yq_dev,
                    int* y_exponent, void* stream);

/* ---- operators between momentum sectors; the current correlator ---------- *
 * The current operator J_d(Q) = sum_{k,s} v_d(k) c+_{k+Q,s} c_{k,s},
 * v_d(k) = 2t (2 pi / L_d) sin(2 pi k_d / L_d)
 * (HubbardModelMomentum::current, src/algebra/fermion/model/
 * hubbard_model_momentum.h:38-90), maps the sector of momentum K to K+Q. */
int mb_current_create(const int64_t* dims, int ndim, double t, const int64_t* transfer,
                      int direction, mb_model_t* out);
/* compute_rectangular_matrix_elements (src/algebra/matrix_elements.h:107-167):
 * rows in row_basis (sector K+Q), columns in col_basis (sector K), built on
 * the GPU; two calls as mb_compute_matrix_elements_csr. */
int mb_compute_rectangular_matrix_elements_csr(mb_basis_t row_basis, mb_basis_t col_basis,
                                               mb_model_t model, int64_t* nnz, int64_t* row_ptr,
                                               int64_t* col_idx, double* values);
/* J and J+ on the device (MB_PREC_F64 / MB_PREC_F32 vectors, reference
 * order): y = J x (x in sector K, y in K+Q), or with adjoint = 1 y = J+ x. */
typedef struct mb_rect_op_s* mb_rect_op_t;
int mb_rect_op_create(mb_basis_t row_basis, mb_basis_t col_basis, mb_model_t model, int precision,
                      mb_rect_op_t* out);
int mb_rect_op_destroy(mb_rect_op_t op);
int mb_rect_op_dims(mb_rect_op_t op, int64_t* n_rows, int64_t* n_cols);
int mb_rect_op_apply(mb_rect_op_t op, const void* x_dev, void* y_dev, int adjoint, void* stream);
/* The stochastic current-current correlator of the reference's optical-
 * conductivity driver (examples/hubbard_momentum_optical_conductivity.cpp:
 * 340-410), on the device: per sample a probe |v> in sector K (random phases,
 * Philox stream 1 + s; the example draws complex Gaussians), |v_b> =
 * exp(-beta H_K / 2)|v>, Z = <v_b|v_b>, phi1 = v_b, phi2 = J v_b, then for
 * each step C[i] += <phi1| J+ |phi2> / Z, phi1 <- exp(-i H_K dt) phi1,
 * phi2 <- exp(-i H_{K+Q} dt) phi2 (Krylov, krylov_steps); C averaged over the
 * samples.  correlator: 2 * steps doubles (re, im). */
int mb_current_correlator(mb_op_t op_k, mb_op_t op_kq, mb_rect_op_t current, int64_t n_samples,
                          uint64_t seed, double beta, double dt, int64_t steps,
                          int64_t krylov_steps, double* correlator);

/* ---- batched / served solves ------------------------------------------------ *
 * An engine advances many independent sectors of uneven size together: one
 * Lanczos step of every active request per engine step, complex64 vectors with
 * FP64 alpha/beta, an optional replay pass that rebuilds the Ritz vector and
 * an FP64 Rayleigh-Ritz refinement of the energy.  Requests are admitted
 * while the device-memory budget allows and retire when converged, so new
 * requests join while others run.  No counterpart in the reference (its
 * closest analogue are the OpenMP sample loops over independent vectors,
 * examples/hubbard_momentum_optical_conductivity.cpp:351-400). */
typedef struct mb_engine_s* mb_engine_t;
typedef struct {
  int64_t dims[3]; /* lattice sizes (periodic), as mb_hubbard_create */
  int ndim;
  int n_up, n_down;
  double t, u;
} mb_sector_desc;
/* device_bytes_budget <= 0: 80 % of the free device memory. */
int mb_engine_create(int64_t device_bytes_budget, mb_engine_t* out);
int mb_engine_destroy(mb_engine_t engine);
/* Device bytes a request of this sector holds while active. */
int mb_engine_footprint(const mb_sector_desc* desc, int64_t* bytes);
/* Ground state of one sector: Lanczos on -H from the Philox start vector of
 * `seed` (tensor order), until the lowest Ritz value changes by less than
 * rel_tol * |E| between checks (every 10 steps; rel_tol 0: run kmax steps),
 * at most kmax <= 512 steps; refine = 1 adds the pass that rebuilds the
 * Ritz vector (from T_m; for a run that reached kmax, from its first
 * checkpoint whose Ritz value had settled to 1e-9, before ghost copies of E0
 * form: summed from the kept Lanczos vectors, or by replaying the
 * recurrence) and an FP64 Rayleigh-Ritz refinement of the energy (3 to 8
 * FP64 Lanczos steps from that vector, until the lowest Ritz value settles).
 * The requests finishing in one step are refined together.  MB_ERR_CAPACITY
 * when the budget is full (retry after mb_engine_step retires requests). */
int mb_engine_submit_ground_state(mb_engine_t engine, const mb_sector_desc* desc, uint64_t seed,
                                  int64_t kmax, double rel_tol, int refine, int64_t* request_id);
/* Density-of-states moments of one sector: spectral bounds from 40 Lanczos
 * steps on H (extremal Ritz values widened by their residual bounds), then
 * (H - b)/a with (a, b) = rescaling::from_bounds(E_min, E_max, padding)
 * (rescaling.h:33-38) and n_probes random-phase probes (Philox stream
 * 1 + probe), n_moments/2 Chebyshev steps each with the doubling identities.
 * The result is mu[n] = (1/R) sum_r <r|T_n|r> / D. */
int mb_engine_submit_dos(mb_engine_t engine, const mb_sector_desc* desc, int64_t n_moments,
                         int64_t n_probes, uint64_t seed, double padding, int64_t* request_id);
/* *done = 1 once finished; mu receives n_moments values; the bounds used. */
int mb_engine_poll_dos(mb_engine_t engine, int64_t request_id, int* done, double* mu,
                       double* e_min, double* e_max, double* latency_s);
/* Run up to n_steps engine steps; *n_active = requests still running. */
int mb_engine_step(mb_engine_t engine, int n_steps, int* n_active);
/* *done = 1 once the request finished: energy (refined if asked), the
 * unrefined Ritz value, Lanczos steps and submit-to-finish seconds. */
int mb_engine_poll(mb_engine_t engine, int64_t request_id, int* done, double* e0, double* e0_raw,
                   int64_t* steps, double* latency_s);
/* Ids of the requests (ground state or DOS) that finished since the last
 * call, oldest first, at most `capacity` of them (the rest stay queued);
 * *n = how many were written.  Lets a serving loop poll only those. */
int mb_engine_completed(mb_engine_t engine, int64_t* ids, int64_t capacity, int64_t* n);
/* Totals over mb_engine_step calls: steps run, their wall time and the
 * device time of their kernels (ms), for the host / device split. */
int mb_engine_stats(mb_engine_t engine, int64_t* steps, double* step_wall_ms,
                    double* step_device_ms);
/* Warps per block of the grouped kernels (2, 4, 8, 16): the autotuner's knob. */
int mb_engine_set_warps(mb_engine_t engine, int warps_per_block);
/* Requests on sectors of at least min_states states step through the fused
 * complex64 apply (rows staged in shared memory, sliced tables), one launch
 * per such request; smaller ones share the grouped warp-per-row kernels.
 * Default 1,048,576 (a launch per large request pays off; many medium
 * requests run faster together); 1 sends every request through it. */
int mb_engine_set_fused_threshold(mb_engine_t engine, int64_t min_states);
/* Times the step's apply at each shape on the current requests and keeps the
 * fastest; *ms = its time per apply.  Persistent step: row_min_cols in
 * {64, 128, 256} x ctas_per_sm in {all that fit, 2} (set_shape takes any
 * ctas_per_sm), timed with apply-only launches (they change no request's
 * progress); a mix of requests (their sectors' shapes and kinds) that this
 * engine has tuned for before takes the shape found then, untimed.  Grouped
 * kernels: warps per block in {2, 4, 8, 16}.  *chosen = the grouped kernels'
 * warps per block. */
int mb_engine_autotune(mb_engine_t engine, int* chosen, double* ms);
/* n_steps steps with no host round trip between them (fixed-length batches).
 * Persistent step (the default): ONE cooperative launch of the fused kernel
 * runs all n_steps (with use_graph, captured as a CUDA graph and launched);
 * grouped kernels: the step's launches captured once and the graph replayed
 * n_steps times. */
int mb_engine_step_fixed(mb_engine_t engine, int n_steps, int use_graph, int* n_active);

/* The persistent step (default on): one cooperative launch runs whole engine
 * steps of every request, the apply (rows of wide or large sectors block per
 * row, staged in shared memory with the sliced tables; the others warp per
 * row), the per-request fixed-order alpha and beta reductions, the update, the
 * normalisation and the step counters, its phases separated by grid barriers.
 * Off: each step is the grouped kernels (apply, reduce, update, reduce,
 * normalise, advance).  Requests keep their progress across a switch, and get
 * the same bits through both for sectors applied warp per row or row-staged
 * in both; a large sector (>= the fused threshold) runs its rows through the
 * block-per-row body here and the fused kernel there. */
int mb_engine_set_persistent(mb_engine_t engine, int on);
/* A ground-state request (with refinement) keeps its pass-one Lanczos
 * vectors (kmax x dim complex64) when they take at most `bytes` (default
 * 2 GiB; 0: never) and fit the device-memory budget: its Ritz vector is then
 * summed from them (the replay's order and arithmetic: the same bits) instead
 * of re-running the recurrence for up to kmax more steps.  Applies to
 * requests submitted afterwards. */
int mb_engine_set_basis_limit(mb_engine_t engine, int64_t bytes);
/* Budget in clock64 cycles of one grid-barrier wait of the persistent step
 * (default 2^32, about two seconds).  A wait that runs past it sets the
 * step's status word; every block then returns at its next barrier and the
 * step fails with MB_ERR_TIMEOUT.  The requests in flight are lost then: the
 * step stopped part-way, and the engine refuses further work (destroy it). */
int mb_engine_set_wait_budget(mb_engine_t engine, int64_t cycles);
typedef struct {
  int persistent;    /* 1: the persistent step; 0: the grouped kernels */
  int row_min_cols;  /* persistent: rows this wide or wider block per row (<= 256) */
  int ctas_per_sm;   /* persistent: co-resident blocks per SM (0: all that fit) */
  int grid;          /* persistent: blocks of the last launch shape (read only) */
  int warps;         /* grouped kernels: warps per block (2, 4, 8, 16) */
  int reserved[3];
} mb_engine_shape;
int mb_engine_get_shape(mb_engine_t engine, mb_engine_shape* shape);
int mb_engine_set_shape(mb_engine_t engine, const mb_engine_shape* shape);

/* ---- block reductions on device vectors (for drivers above this ABI) ---- */
/* *out = Re <x, y> (arma::cdot real part), FP64 accumulation, deterministic. */
int mb_dot_re(mb_op_t op, const void* x_dev, const void* y_dev, double* out);
int mb_norm(mb_op_t op, const void* x_dev, double* out);

#ifdef __cplusplus
}
#endif

#endif /* MANYBODY_GB300_H */
