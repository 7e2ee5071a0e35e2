/*
 * oracle.c -- CPU restatement of the reference library's Hubbard hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py load this library, and only to
 * verify results or as the timed CPU baseline.  The GPU product never calls it.
 *
 * Parity pins: the basis order and the sparse Hamiltonian produced here are
 * compared bit-for-bit against outputs of the reference's own code
 * (oracle/build_ref.sh -> oracle/_ref/ref_dump), committed as fixtures under
 * tests/golden/.  The numerics (Lanczos, KPM, Krylov evolution) restate
 * reference headers that need Armadillo, which is absent here.  Lanczos
 * (find_min_eigenpair, pass one), Krylov evolution, the KPM kernels, the
 * projector moments and the sparse KPM projector are pinned against the
 * reference's own lanczos.h, evolve_state.h and kpm.h, run unchanged on the
 * CPU with a minimal Armadillo stand-in (oracle/ref_numerics_pin.cpp); the
 * DOS moments, which the reference does not implement, against the
 * reference's own test expectations (tests/numerics/); all of them against
 * numpy dense solves, within stated tolerances.
 *
 * Every function cites the reference file:line it follows.  Operator packing
 * follows src/algebra/operator.h:15-110: bit 15 = type (0 creation,
 * 1 annihilation), bit 14 = spin (0 up, 1 down), bits 0-13 = orbital.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_TYPE_BIT 0x8000u
#define OR_SPIN_BIT 0x4000u
#define OR_VALUE_MASK 0x3FFFu
#define OR_MAX_OPS 64
#define OR_TOL (1000.0 * 2.220446049250313e-16) /* src/utils/tolerances.h:7-10 */
#define OR_PI 3.14159265358979323846

typedef uint16_t or_op;

static or_op op_make(int annihilation, int spin, int orbital) {
  return (or_op)((annihilation ? OR_TYPE_BIT : 0) | (spin ? OR_SPIN_BIT : 0) |
                 ((unsigned)orbital & OR_VALUE_MASK));
}
static int op_type(or_op a) { return (a >> 15) & 1; }
static int op_spin(or_op a) { return (a >> 14) & 1; }
static int op_value(or_op a) { return a & OR_VALUE_MASK; }

/* operator< (src/algebra/operator.h:69-79). */
static int op_less(or_op a, or_op b) {
  const int other_is_creation = op_type(b) == 0;
  if (op_type(a) != op_type(b)) return op_type(a) < op_type(b);
  if (op_spin(a) != op_spin(b))
    return other_is_creation ? (op_spin(a) < op_spin(b)) : (op_spin(a) > op_spin(b));
  return other_is_creation ? (op_value(a) < op_value(b)) : (op_value(a) > op_value(b));
}
/* commutes(): true unless the two differ only in the type bit (operator.h:87-89). */
static int op_commutes(or_op a, or_op b) { return (uint16_t)(a ^ b) != OR_TYPE_BIT; }

/* ------------------------------------------------------------------------ */
/* A tiny expression: list of (operator string, complex coefficient).       */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n;
  or_op ops[OR_MAX_OPS];
  double re, im;
} or_term;

typedef struct {
  or_term* t;
  int n, cap;
} or_expr;

static void expr_init(or_expr* e) { e->t = NULL; e->n = 0; e->cap = 0; }
static void expr_free(or_expr* e) { free(e->t); e->t = NULL; e->n = e->cap = 0; }
static int is_zero(double re, double im) { return re * re + im * im < OR_TOL * OR_TOL; }

static int key_equal(const or_term* a, int n, const or_op* ops) {
  return a->n == n && (n == 0 || memcmp(a->ops, ops, sizeof(or_op) * (size_t)n) == 0);
}

/* ExpressionBase::add_to (src/algebra/expression_base.h:85-97): skip zero
 * coefficients, merge equal keys, erase a key whose sum becomes zero. */
static void expr_add(or_expr* e, int n, const or_op* ops, double re, double im) {
  if (is_zero(re, im)) return;
  for (int i = 0; i < e->n; ++i) {
    if (key_equal(&e->t[i], n, ops)) {
      e->t[i].re += re;
      e->t[i].im += im;
      if (is_zero(e->t[i].re, e->t[i].im)) {
        e->t[i] = e->t[e->n - 1];
        e->n -= 1;
      }
      return;
    }
  }
  if (e->n == e->cap) {
    e->cap = e->cap ? 2 * e->cap : 8;
    e->t = (or_term*)realloc(e->t, sizeof(or_term) * (size_t)e->cap);
  }
  or_term* t = &e->t[e->n++];
  t->n = n;
  if (n) memcpy(t->ops, ops, sizeof(or_op) * (size_t)n);
  t->re = re;
  t->im = im;
}

static int has_consecutive_elements(int n, const or_op* ops) { /* utils/static_vector.h:150-152 */
  for (int i = 0; i + 1 < n; ++i)
    if (ops[i] == ops[i + 1]) return 1;
  return 0;
}

static void canonicalize_recursive(int n, const or_op* in, double pre, double pim, or_expr* out);

/* handle_non_commuting (src/algebra/canonicalize.h:63-78): ops[idx], ops[idx+1]
 * are c_a c+_a; c_a c+_a = 1 - c+_a c_a for fermions. */
static void handle_non_commuting(int n, or_op* ops, int idx, double pre, double pim, or_expr* out) {
  or_op contracted[OR_MAX_OPS];
  int m = 0;
  for (int i = 0; i < n; ++i)
    if (i != idx && i != idx + 1) contracted[m++] = ops[i];
  or_op tmp = ops[idx];
  ops[idx] = ops[idx + 1];
  ops[idx + 1] = tmp;
  canonicalize_recursive(m, contracted, pre, pim, out);
  canonicalize_recursive(n, ops, -pre, -pim, out);
}

/* canonicalize_recursive (src/algebra/canonicalize.h:20-60): insertion sort
 * by operator<, a -1 per swap of commuting operators, contraction on a
 * non-commuting pair, Pauli zero on repeated operators.  Results are scaled
 * by (pre_re, pre_im) and accumulated into out. */
static void canonicalize_recursive(int n, const or_op* in, double pre_re, double pre_im,
                                   or_expr* out) {
  or_op ops[OR_MAX_OPS];
  if (n) memcpy(ops, in, sizeof(or_op) * (size_t)n);
  if (n < 2) {
    expr_add(out, n, ops, pre_re, pre_im);
    return;
  }
  if (has_consecutive_elements(n, ops)) return;
  double phase = 1.0;
  for (int i = 1; i < n; ++i) {
    int j = i;
    while (j > 0 && op_less(ops[j], ops[j - 1])) {
      if (op_commutes(ops[j], ops[j - 1])) {
        or_op tmp = ops[j];
        ops[j] = ops[j - 1];
        ops[j - 1] = tmp;
        phase = -phase;
        --j;
      } else {
        handle_non_commuting(n, ops, j - 1, pre_re * phase, pre_im * phase, out);
        return;
      }
    }
  }
  if (has_consecutive_elements(n, ops)) return;
  expr_add(out, n, ops, pre_re * phase, pre_im * phase);
}

/* ------------------------------------------------------------------------ */
/* Hubbard Hamiltonian terms (src/algebra/fermion/model/hubbard_model.h).   */
/* ------------------------------------------------------------------------ */

/* hopping_generic (src/algebra/expression_base.h:394-403) scaled by -t and
 * added into h: c+_from c_to (coeff) + c+_to c_from (conj coeff). */
static void add_hopping(or_expr* h, double t, int from, int to, int spin) {
  or_expr one;
  expr_init(&one);
  or_op a[2] = {op_make(0, spin, from), op_make(1, spin, to)};
  or_op b[2] = {op_make(0, spin, to), op_make(1, spin, from)};
  expr_add(&one, 2, a, 1.0, 0.0);
  expr_add(&one, 2, b, 1.0, -0.0);
  for (int i = 0; i < one.n; ++i)
    expr_add(h, one.t[i].n, one.t[i].ops, -t * one.t[i].re, -t * one.t[i].im);
  expr_free(&one);
}

/* HubbardModel{,2D,3D}::hamiltonian(): kinetic() then interaction().
 * Sites are x + Lx*y + Lx*Ly*z (src/utils/index.h:69-88). */
static void hubbard_terms(const int* dims, int ndim, double t, double U, or_expr* h) {
  int Lx = dims[0], Ly = ndim > 1 ? dims[1] : 1, Lz = ndim > 2 ? dims[2] : 1;
  for (int x = 0; x < Lx; ++x)
    for (int y = 0; y < Ly; ++y)
      for (int z = 0; z < Lz; ++z) {
        int site = x + Lx * (y + Ly * z);
        int nb[3] = {((x + 1) % Lx) + Lx * (y + Ly * z), x + Lx * (((y + 1) % Ly) + Ly * z),
                     x + Lx * (y + Ly * ((z + 1) % Lz))};
        for (int d = 0; d < ndim; ++d) {
          add_hopping(h, t, site, nb[d], 0);
          add_hopping(h, t, site, nb[d], 1);
        }
      }
  int L = Lx * Ly * Lz;
  for (int i = 0; i < L; ++i) {
    /* density_density(Up,i,Down,i) = c+_up c_up c+_dn c_dn (fermion/term.h:45-48) */
    or_op k[4] = {op_make(0, 0, i), op_make(1, 0, i), op_make(0, 1, i), op_make(1, 1, i)};
    expr_add(h, 4, k, U, 0.0);
  }
}

int or_hubbard_term_count(const int* dims, int ndim, double t, double U) {
  or_expr h;
  expr_init(&h);
  hubbard_terms(dims, ndim, t, U, &h);
  int n = h.n;
  expr_free(&h);
  return n;
}

/* ------------------------------------------------------------------------ */
/* Basis (src/algebra/basis.cpp).                                           */
/* ------------------------------------------------------------------------ */

static uint64_t choose_u64(uint64_t n, uint64_t m) { /* basis.cpp:13-26 */
  if (m > n) return 0;
  if (m == 0 || m == n) return 1;
  if (m > n - m) m = n - m;
  uint64_t r = 1;
  for (uint64_t i = 0; i < m; ++i) {
    r *= (n - i);
    r /= (i + 1);
  }
  return r;
}

int64_t or_basis_size(int L, int nup, int ndn) { /* compute_basis_size_spin, basis.cpp:39-50 */
  if (L < 0 || nup < 0 || ndn < 0 || nup > L || ndn > L) return 0;
  return (int64_t)(choose_u64((uint64_t)L, (uint64_t)nup) * choose_u64((uint64_t)L, (uint64_t)ndn));
}

typedef struct {
  int L;
  uint64_t *up, *dn;
  int64_t count;
} dfs_ctx;

/* generate_restrict_combinations_with_spin (basis.cpp:267-302): the
 * current sequence is kept as occupation masks; "back" is the last slot. */
static void dfs(dfs_ctx* c, int size, int back_orb, int back_spin, int first, int up_left,
                int dn_left, uint64_t um, uint64_t dm, int particles) {
  if (up_left == 0 && dn_left == 0) {
    c->up[c->count] = um;
    c->dn[c->count] = dm;
    c->count += 1;
    return;
  }
  if (size >= particles) return;
  for (int s = 0; s < 2; ++s) {
    for (int i = first; i < c->L; ++i) {
      if ((s == 0 && up_left == 0) || (s == 1 && dn_left == 0)) continue;
      int ok = size == 0 || back_orb < i || (back_orb == i && s > back_spin);
      if (ok) {
        dfs(c, size + 1, i, s, i, up_left - (s == 0), dn_left - (s == 1),
            s == 0 ? (um | (1ull << i)) : um, s == 1 ? (dm | (1ull << i)) : dm, particles);
      }
    }
  }
}

/* with_fixed_particle_number_and_spin (basis.cpp:91-126), written as the
 * (up, down) counts; fills masks in reference index order. */
int64_t or_basis_enumerate(int L, int nup, int ndn, uint64_t* up, uint64_t* dn) {
  if (L < 0 || L > 63 || nup < 0 || ndn < 0 || nup > L || ndn > L) return -1;
  dfs_ctx c = {L, up, dn, 0};
  dfs(&c, 0, -1, -1, 0, nup, ndn, 0, 0, nup + ndn);
  return c.count;
}

/* Sorted key (operator<): all Up creators ascending, then Down ascending. */
static int state_key(int L, uint64_t um, uint64_t dm, or_op* ops) {
  int n = 0;
  for (int i = 0; i < L; ++i)
    if (um >> i & 1) ops[n++] = op_make(0, 0, i);
  for (int i = 0; i < L; ++i)
    if (dm >> i & 1) ops[n++] = op_make(0, 1, i);
  return n;
}

typedef struct {
  uint64_t up, dn;
  int64_t idx;
} key_idx;

static int key_cmp(const void* a, const void* b) {
  const key_idx* x = (const key_idx*)a;
  const key_idx* y = (const key_idx*)b;
  if (x->up != y->up) return x->up < y->up ? -1 : 1;
  if (x->dn != y->dn) return x->dn < y->dn ? -1 : 1;
  return 0;
}

/* ------------------------------------------------------------------------ */
/* compute_matrix_elements (src/algebra/matrix_elements.h:74-105).          */
/* ------------------------------------------------------------------------ */

typedef struct {
  int64_t row;
  double re, im;
} col_entry;

static int col_entry_cmp(const void* a, const void* b) {
  const col_entry* x = (const col_entry*)a;
  const col_entry* y = (const col_entry*)b;
  return x->row < y->row ? -1 : (x->row > y->row ? 1 : 0);
}

/* Entries of column j of H (compute_matrix_elements, matrix_elements.h:80-104):
 * canonicalize(H * key_j) (ExpressionBase::operator*=, expression_base.h:175-193,
 * then canonicalize again at matrix_elements.h:85 -- the identity on
 * normal-ordered terms), keep the pure creator strings of the sector
 * (set.contains), look up their index, sort by row.  Returns the count. */
static int column_entries(const or_expr* h, int L, int nup, int ndn, uint64_t um_j, uint64_t dm_j,
                          const key_idx* lookup, int64_t dim, col_entry* col, int col_cap) {
  or_op key[OR_MAX_OPS];
  int kn = state_key(L, um_j, dm_j, key);
  or_expr prod;
  expr_init(&prod);
  for (int a = 0; a < h->n; ++a) {
    if (h->t[a].n + kn > OR_MAX_OPS) continue;
    if (is_zero(h->t[a].re, h->t[a].im)) continue;
    or_op cat[OR_MAX_OPS];
    memcpy(cat, h->t[a].ops, sizeof(or_op) * (size_t)h->t[a].n);
    memcpy(cat + h->t[a].n, key, sizeof(or_op) * (size_t)kn);
    canonicalize_recursive(h->t[a].n + kn, cat, h->t[a].re, h->t[a].im, &prod);
  }
  int m = 0;
  for (int p = 0; p < prod.n; ++p) {
    const or_term* tm = &prod.t[p];
    if (tm->n != nup + ndn) continue;
    uint64_t um = 0, dm = 0;
    int ok = 1;
    for (int q = 0; q < tm->n; ++q) {
      if (op_type(tm->ops[q]) != 0) { ok = 0; break; }
      if (op_spin(tm->ops[q]) == 0) um |= 1ull << op_value(tm->ops[q]);
      else dm |= 1ull << op_value(tm->ops[q]);
    }
    if (!ok) continue;
    or_op chk[OR_MAX_OPS];
    int cn = state_key(L, um, dm, chk);
    if (!key_equal(tm, cn, chk)) continue;
    key_idx probe = {um, dm, 0};
    key_idx* hit = (key_idx*)bsearch(&probe, lookup, (size_t)dim, sizeof(key_idx), key_cmp);
    if (!hit) continue;
    if (m < col_cap) {
      col[m].row = hit->idx;
      col[m].re = tm->re;
      col[m].im = tm->im;
    }
    ++m;
  }
  expr_free(&prod);
  if (m <= col_cap) qsort(col, (size_t)m, sizeof(col_entry), col_entry_cmp);
  return m;
}

#define OR_COL_CAP 1024

/*
 * H(i,j) = coefficient of basis key i in canonicalize(H * key_j), written as
 * CSC (column j's rows ascending); for the Hermitian real-space Hubbard H the
 * same arrays read as CSR of H^T = H.  Two calls: with row_idx == NULL it
 * fills col_ptr (dim+1 entries) and returns nnz; then with row_idx/re/im of
 * that capacity and the same col_ptr it fills the entries.  Columns are
 * processed in parallel (OpenMP, as the reference's #pragma omp parallel for
 * schedule(dynamic), matrix_elements.h:80-82).  Returns nnz or -1.
 */
int64_t or_matrix_elements_csc(const int* dims, int ndim, double t, double U, int nup, int ndn,
                               int64_t* col_ptr, int64_t* row_idx, double* re, double* im,
                               int64_t cap) {
  int L = 1;
  for (int d = 0; d < ndim; ++d) L *= dims[d];
  if (ndim < 1 || ndim > 3 || L > 60 || !col_ptr) return -1;
  int64_t dim = or_basis_size(L, nup, ndn);
  if (dim <= 0) return -1;
  uint64_t* up = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)dim);
  uint64_t* dn = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)dim);
  or_basis_enumerate(L, nup, ndn, up, dn);
  key_idx* lookup = (key_idx*)malloc(sizeof(key_idx) * (size_t)dim);
  for (int64_t i = 0; i < dim; ++i) {
    lookup[i].up = up[i];
    lookup[i].dn = dn[i];
    lookup[i].idx = i;
  }
  qsort(lookup, (size_t)dim, sizeof(key_idx), key_cmp);
  or_expr h;
  expr_init(&h);
  hubbard_terms(dims, ndim, t, U, &h);
  int64_t nnz = 0;
  int failed = 0;
  if (!row_idx) {
#pragma omp parallel
    {
      col_entry* col = (col_entry*)malloc(sizeof(col_entry) * OR_COL_CAP);
#pragma omp for schedule(dynamic, 64)
      for (int64_t j = 0; j < dim; ++j)
        col_ptr[j + 1] = column_entries(&h, L, nup, ndn, up[j], dn[j], lookup, dim, col, OR_COL_CAP);
      free(col);
    }
    col_ptr[0] = 0;
    for (int64_t j = 0; j < dim; ++j) col_ptr[j + 1] += col_ptr[j];
    nnz = col_ptr[dim];
  } else {
    if (col_ptr[dim] > cap) failed = 1;
#pragma omp parallel
    {
      col_entry* col = (col_entry*)malloc(sizeof(col_entry) * OR_COL_CAP);
#pragma omp for schedule(dynamic, 64)
      for (int64_t j = 0; j < dim; ++j) {
        if (failed) continue;
        int m = column_entries(&h, L, nup, ndn, up[j], dn[j], lookup, dim, col, OR_COL_CAP);
        if (m > OR_COL_CAP || col_ptr[j] + m != col_ptr[j + 1]) {
          failed = 1;
          continue;
        }
        for (int p = 0; p < m; ++p) {
          row_idx[col_ptr[j] + p] = col[p].row;
          re[col_ptr[j] + p] = col[p].re;
          im[col_ptr[j] + p] = col[p].im;
        }
      }
      free(col);
    }
    nnz = failed ? -1 : col_ptr[dim];
  }
  expr_free(&h);
  free(lookup);
  free(up);
  free(dn);
  return nnz;
}

/* ------------------------------------------------------------------------ */
/* Sparse apply: Armadillo sp_cx_mat * cx_vec, serial column scatter         */
/* (src/numerics/linear_operator.h:81-91; ARMA_OPENMP_THREADS=1 per          */
/* src/CMakeLists.txt:20).  Vectors are interleaved (re, im).                */
/* ------------------------------------------------------------------------ */
void or_csc_apply(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx, const double* re,
                  const double* im, const double* x, double* y) {
  memset(y, 0, sizeof(double) * 2 * (size_t)dim);
  for (int64_t j = 0; j < dim; ++j) {
    const double xr = x[2 * j], xi = x[2 * j + 1];
    for (int64_t p = col_ptr[j]; p < col_ptr[j + 1]; ++p) {
      const int64_t i = row_idx[p];
      y[2 * i] += re[p] * xr - im[p] * xi;
      y[2 * i + 1] += re[p] * xi + im[p] * xr;
    }
  }
}

/* Best-effort multi-core y = H x for a Hermitian H held as CSC: column i of H
 * is the conjugate of row i, so y_i = sum_p conj(H_{row(p), i}) x_{row(p)}
 * over column i's entries, a gather that splits over rows with no write
 * conflicts.  Not the reference's algorithm (Armadillo's serial column
 * scatter, or_csc_apply above); a multi-core CPU figure for context. */
void or_csc_apply_hermitian_parallel(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx,
                                     const double* re, const double* im, const double* x,
                                     double* y) {
#pragma omp parallel for schedule(static, 1024)
  for (int64_t i = 0; i < dim; ++i) {
    double yr = 0.0, yi = 0.0;
    for (int64_t p = col_ptr[i]; p < col_ptr[i + 1]; ++p) {
      const int64_t j = row_idx[p];
      const double xr = x[2 * j], xi = x[2 * j + 1];
      yr += re[p] * xr + im[p] * xi;
      yi += re[p] * xi - im[p] * xr;
    }
    y[2 * i] = yr;
    y[2 * i + 1] = yi;
  }
}

int or_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Counter-based RNG: Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).     */
/* ------------------------------------------------------------------------ */
static void philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1) {
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

/* Uniform [-1, 1): 52 random bits placed in [2, 4), minus 3 (exact). */
static double u52_to_pm1(uint32_t hi, uint32_t lo) {
  uint64_t m = (((uint64_t)hi << 32) | lo) >> 12;
  uint64_t bits = 0x4000000000000000ull | m;
  double v;
  memcpy(&v, &bits, 8);
  return v - 3.0;
}

/* Element with tensor index i of stream `stream` and seed `seed`: counter
 * (i_lo, i_hi, stream, 0), key (seed_lo, seed_hi). */
void or_philox_uniform_pm1(uint64_t seed, uint32_t stream, int64_t n, double* out_interleaved) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), stream, 0};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    out_interleaved[2 * i] = u52_to_pm1(c[0], c[1]);
    out_interleaved[2 * i + 1] = u52_to_pm1(c[2], c[3]);
  }
}

/* Random phases: phi = 2*pi*u, u in [0,1) from 52 bits of (c0, c1). */
void or_philox_phase(uint64_t seed, uint32_t stream, int64_t n, double* out_interleaved) {
  for (int64_t i = 0; i < n; ++i) {
    uint32_t c[4] = {(uint32_t)i, (uint32_t)((uint64_t)i >> 32), stream, 0};
    philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    double u = (u52_to_pm1(c[0], c[1]) + 1.0) * 0.5;
    out_interleaved[2 * i] = cos(2.0 * OR_PI * u);
    out_interleaved[2 * i + 1] = sin(2.0 * OR_PI * u);
  }
}

/* ------------------------------------------------------------------------ */
/* Symmetric tridiagonal eigensolver: implicit QL with Wilkinson shifts      */
/* (Bowdler, Martin, Reinsch & Wilkinson 1968, EISPACK tql2).  d[n]          */
/* diagonal, e[n-1] off-diagonal; on return d ascending and z (n x n,        */
/* column-major) the orthonormal eigenvectors.  Stands in for               */
/* arma::eig_sym on T (src/numerics/lanczos.h:258-270).  Returns 0 or -1.    */
/* ------------------------------------------------------------------------ */
int or_tridiag_eig(int n, double* d, const double* e_in, double* z) {
  if (n <= 0) return 0;
  double* e = (double*)calloc((size_t)n, sizeof(double));
  for (int i = 0; i + 1 < n; ++i) e[i] = e_in[i];
  for (int i = 0; i < n * n; ++i) z[i] = 0.0;
  for (int i = 0; i < n; ++i) z[i + (size_t)n * i] = 1.0;
  int status = 0;
  for (int l = 0; l < n; ++l) {
    int iter = 0;
    int m;
    do {
      for (m = l; m < n - 1; ++m) {
        double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) <= 2.220446049250313e-16 * dd) break;
      }
      if (m != l) {
        if (++iter > 60) { status = -1; break; }
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = hypot(g, 1.0);
        g = d[m] - d[l] + e[l] / (g + (g >= 0 ? fabs(r) : -fabs(r)));
        double s = 1.0, c = 1.0, p = 0.0;
        int i;
        for (i = m - 1; i >= l; --i) {
          double f = s * e[i], b = c * e[i];
          r = hypot(f, g);
          e[i + 1] = r;
          if (r == 0.0) {
            d[i + 1] -= p;
            e[m] = 0.0;
            break;
          }
          s = f / r;
          c = g / r;
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          for (int k = 0; k < n; ++k) {
            double zf = z[k + (size_t)n * (i + 1)];
            z[k + (size_t)n * (i + 1)] = s * z[k + (size_t)n * i] + c * zf;
            z[k + (size_t)n * i] = c * z[k + (size_t)n * i] - s * zf;
          }
        }
        if (r == 0.0 && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
    if (status) break;
  }
  /* sort ascending with vectors */
  for (int i = 0; i < n - 1; ++i) {
    int k = i;
    for (int j = i + 1; j < n; ++j)
      if (d[j] < d[k]) k = j;
    if (k != i) {
      double tmp = d[i];
      d[i] = d[k];
      d[k] = tmp;
      for (int r = 0; r < n; ++r) {
        double zz = z[r + (size_t)n * i];
        z[r + (size_t)n * i] = z[r + (size_t)n * k];
        z[r + (size_t)n * k] = zz;
      }
    }
  }
  free(e);
  return status;
}

/* ------------------------------------------------------------------------ */
/* Generic complex-vector numerics over a CSC operator.                     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int64_t dim;
  const int64_t *col_ptr, *row_idx;
  const double *re, *im;
  double scale;  /* apply returns scale*(H - shift) v: +1 plain, -1 Negated */
  double shift;
} or_op_ctx;

static void op_apply(const or_op_ctx* op, const double* x, double* y) {
  or_csc_apply(op->dim, op->col_ptr, op->row_idx, op->re, op->im, x, y);
  if (op->shift != 0.0)
    for (int64_t i = 0; i < 2 * op->dim; ++i) y[i] -= op->shift * x[i];
  if (op->scale != 1.0)
    for (int64_t i = 0; i < 2 * op->dim; ++i) y[i] = op->scale * y[i];
}

static double vnorm(int64_t n, const double* v) {
  double s = 0.0;
  for (int64_t i = 0; i < 2 * n; ++i) s += v[i] * v[i];
  return sqrt(s);
}

static double cdot_re(int64_t n, const double* a, const double* b) { /* Re(sum conj(a) b) */
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s += a[2 * i] * b[2 * i] + a[2 * i + 1] * b[2 * i + 1];
  return s;
}

/* lanczos_pass_one (src/numerics/lanczos.h:130-175) with LanczosIteration
 * (:70-128) and lanczos_recurrence_step (:15-40).  Writes alphas[k],
 * betas[k-1]; returns steps taken, or -1 on zero norm.  If basis != NULL
 * and reorth != 0, stores the Lanczos vectors and applies full
 * re-orthogonalisation (classical Gram-Schmidt, twice) after each step --
 * an extension beyond the reference, which has none. */
int or_lanczos_pass_one(const or_op_ctx* op, const double* b, int k, double* alphas, double* betas,
                        double* b_norm_out, int reorth, double* basis) {
  const int64_t n = op->dim;
  const double tol = OR_TOL;
  double b_norm = vnorm(n, b);
  *b_norm_out = b_norm;
  if (b_norm <= tol) return -1;
  if (k == 0) return 0;
  double* v_prev = (double*)calloc((size_t)(2 * n), sizeof(double));
  double* v_curr = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* w = (double*)calloc((size_t)(2 * n), sizeof(double));
  for (int64_t i = 0; i < 2 * n; ++i) v_curr[i] = b[i] / b_norm;
  double beta_prev = 0.0;
  int steps = 0;
  for (int it = 0; it < k; ++it) {
    if (reorth && basis) memcpy(basis + (size_t)2 * n * it, v_curr, sizeof(double) * 2 * (size_t)n);
    op_apply(op, v_curr, w);
    if (beta_prev != 0.0)
      for (int64_t i = 0; i < 2 * n; ++i) w[i] -= beta_prev * v_prev[i];
    double alpha = cdot_re(n, v_curr, w);
    for (int64_t i = 0; i < 2 * n; ++i) w[i] -= alpha * v_curr[i];
    if (reorth && basis) {
      for (int pass = 0; pass < 2; ++pass) {
        for (int j = 0; j <= it; ++j) {
          const double* vj = basis + (size_t)2 * n * j;
          double cr = 0.0, ci = 0.0; /* c = <vj, w> */
          for (int64_t i = 0; i < n; ++i) {
            cr += vj[2 * i] * w[2 * i] + vj[2 * i + 1] * w[2 * i + 1];
            ci += vj[2 * i] * w[2 * i + 1] - vj[2 * i + 1] * w[2 * i];
          }
          for (int64_t i = 0; i < n; ++i) {
            w[2 * i] -= cr * vj[2 * i] - ci * vj[2 * i + 1];
            w[2 * i + 1] -= cr * vj[2 * i + 1] + ci * vj[2 * i];
          }
        }
      }
    }
    double beta = vnorm(n, w);
    alphas[steps] = alpha;
    steps += 1;
    if (beta <= tol) break;
    if (it + 1 < k) betas[steps - 1] = beta;
    for (int64_t i = 0; i < 2 * n; ++i) {
      double wi = w[i] / beta;
      v_prev[i] = v_curr[i];
      v_curr[i] = wi;
    }
    beta_prev = beta;
  }
  free(v_prev);
  free(v_curr);
  free(w);
  return steps;
}

/* lanczos_pass_two (src/numerics/lanczos.h:177-218) with
 * lanczos_reconstruction_step (:43-57): x = sum_j y_j v_j, complex y. */
int or_lanczos_pass_two(const or_op_ctx* op, const double* b, int steps, const double* alphas,
                        const double* betas, double b_norm, const double* y_re, const double* y_im,
                        double* x) {
  const int64_t n = op->dim;
  if (b_norm <= OR_TOL) return -1;
  memset(x, 0, sizeof(double) * 2 * (size_t)n);
  if (steps == 0) return 0;
  double* v_prev = (double*)calloc((size_t)(2 * n), sizeof(double));
  double* v_curr = (double*)malloc(sizeof(double) * 2 * (size_t)n);
  double* w = (double*)calloc((size_t)(2 * n), sizeof(double));
  for (int64_t i = 0; i < 2 * n; ++i) v_curr[i] = b[i] / b_norm;
  for (int64_t i = 0; i < n; ++i) {
    x[2 * i] = v_curr[2 * i] * y_re[0] - v_curr[2 * i + 1] * y_im[0];
    x[2 * i + 1] = v_curr[2 * i] * y_im[0] + v_curr[2 * i + 1] * y_re[0];
  }
  for (int j = 0; j + 1 < steps; ++j) {
    double alpha_j = alphas[j], beta_j = betas[j];
    double beta_prev = j == 0 ? 0.0 : betas[j - 1];
    op_apply(op, v_curr, w);
    if (beta_prev != 0.0)
      for (int64_t i = 0; i < 2 * n; ++i) w[i] -= beta_prev * v_prev[i];
    for (int64_t i = 0; i < 2 * n; ++i) w[i] -= alpha_j * v_curr[i];
    for (int64_t i = 0; i < 2 * n; ++i) w[i] /= beta_j;
    for (int64_t i = 0; i < n; ++i) {
      x[2 * i] += w[2 * i] * y_re[j + 1] - w[2 * i + 1] * y_im[j + 1];
      x[2 * i + 1] += w[2 * i] * y_im[j + 1] + w[2 * i + 1] * y_re[j + 1];
    }
    double* tmp = v_prev;
    v_prev = v_curr;
    v_curr = w;
    w = tmp;
  }
  free(v_prev);
  free(v_curr);
  free(w);
  return 0;
}

/* find_min_eigenpair (src/numerics/lanczos.h:283-290): Lanczos on Negated<Op>
 * (linear_operator.h:93-105), T -> eig_sym, largest Ritz pair of -H, pass two.
 * Seed is given (the reference's arma::randu seed is not reproducible).
 * Returns steps taken; *e0 the lowest Ritz value; vec (may be NULL). */
int or_find_min_eigenpair(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx,
                          const double* re, const double* im, const double* seed, int k,
                          int reorth, double* e0, double* vec, double* alphas_out,
                          double* betas_out) {
  or_op_ctx op = {dim, col_ptr, row_idx, re, im, -1.0, 0.0};
  double* alphas = (double*)calloc((size_t)(k > 0 ? k : 1), sizeof(double));
  double* betas = (double*)calloc((size_t)(k > 0 ? k : 1), sizeof(double));
  double* basis = reorth ? (double*)malloc(sizeof(double) * 2 * (size_t)dim * (size_t)k) : NULL;
  double b_norm = 0.0;
  int m = or_lanczos_pass_one(&op, seed, k, alphas, betas, &b_norm, reorth, basis);
  if (m < 0) {
    free(basis);
    free(alphas);
    free(betas);
    return -1;
  }
  if (m == 0) {
    *e0 = 0.0;
    if (vec) memset(vec, 0, sizeof(double) * 2 * (size_t)dim);
    free(basis);
    free(alphas);
    free(betas);
    return 0;
  }
  double* d = (double*)malloc(sizeof(double) * (size_t)m);
  double* z = (double*)malloc(sizeof(double) * (size_t)m * (size_t)m);
  memcpy(d, alphas, sizeof(double) * (size_t)m);
  if (or_tridiag_eig(m, d, betas, z) != 0) {
    free(d); free(z); free(alphas); free(betas); free(basis);
    return -2;
  }
  *e0 = -d[m - 1];
  if (alphas_out) memcpy(alphas_out, alphas, sizeof(double) * (size_t)m);
  if (betas_out && m > 1) memcpy(betas_out, betas, sizeof(double) * (size_t)(m - 1));
  if (vec) {
    double* yr = (double*)malloc(sizeof(double) * (size_t)m);
    double* yi = (double*)calloc((size_t)m, sizeof(double));
    for (int i = 0; i < m; ++i) yr[i] = z[i + (size_t)m * (m - 1)] * b_norm;
    if (basis) { /* re-orthogonalised run: x = sum_j y_j v_j from the stored basis */
      memset(vec, 0, sizeof(double) * 2 * (size_t)dim);
      for (int j = 0; j < m; ++j) {
        const double* vj = basis + (size_t)2 * dim * j;
        for (int64_t i = 0; i < 2 * dim; ++i) vec[i] += yr[j] * vj[i];
      }
    } else {
      or_lanczos_pass_two(&op, seed, m, alphas, betas, b_norm, yr, yi, vec);
    }
    free(yr);
    free(yi);
  }
  free(d);
  free(z);
  free(alphas);
  free(betas);
  free(basis);
  return m;
}

/* ------------------------------------------------------------------------ */
/* Krylov evolution (src/numerics/evolve_state.h).                          */
/* ------------------------------------------------------------------------ */

/* expm_tridiagonal_first_column_{unitary,imaginary} (evolve_state.h:22-106):
 * y = Q exp(f(lambda)) Q^T e1 with f = -i t lambda (unitary) or -t lambda. */
int or_expm_tridiag_first_column(int n, const double* alphas, const double* betas, double t,
                                 int imaginary, double* y_re, double* y_im) {
  if (n == 0) return 0;
  double* d = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n * (size_t)n);
  memcpy(d, alphas, sizeof(double) * (size_t)n);
  if (or_tridiag_eig(n, d, betas, z) != 0) {
    free(d);
    free(z);
    return -1;
  }
  for (int i = 0; i < n; ++i) {
    double sr = 0.0, si = 0.0;
    for (int j = 0; j < n; ++j) {
      double w = z[0 + (size_t)n * j]; /* Q^T e1 */
      double er, ei;
      if (imaginary) {
        er = exp(-t * d[j]);
        ei = 0.0;
      } else {
        er = cos(-t * d[j]);
        ei = sin(-t * d[j]);
      }
      sr += z[i + (size_t)n * j] * er * w;
      si += z[i + (size_t)n * j] * ei * w;
    }
    y_re[i] = sr;
    y_im[i] = si;
  }
  free(d);
  free(z);
  return 0;
}

/* evolve_state + time_evolve_state / imaginary_time_evolve_state
 * (evolve_state.h:120-195): solve() = pass one, small expm, scale by
 * ||psi||, pass two. */
int or_time_evolve(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx, const double* re,
                   const double* im, const double* psi0, double t, int krylov_steps, int imaginary,
                   double* out) {
  or_op_ctx op = {dim, col_ptr, row_idx, re, im, 1.0, 0.0};
  if (dim == 0) return 0;
  double psi_norm = vnorm(dim, psi0);
  if (psi_norm <= OR_TOL) {
    memcpy(out, psi0, sizeof(double) * 2 * (size_t)dim);
    return 0;
  }
  int k = krylov_steps;
  if (k == 0 || k > dim) k = (int)dim;
  double* alphas = (double*)calloc((size_t)k, sizeof(double));
  double* betas = (double*)calloc((size_t)k, sizeof(double));
  double b_norm = 0.0;
  int m = or_lanczos_pass_one(&op, psi0, k, alphas, betas, &b_norm, 0, NULL);
  if (m <= 0) {
    memset(out, 0, sizeof(double) * 2 * (size_t)dim);
    free(alphas);
    free(betas);
    return m;
  }
  double* yr = (double*)malloc(sizeof(double) * (size_t)m);
  double* yi = (double*)malloc(sizeof(double) * (size_t)m);
  if (or_expm_tridiag_first_column(m, alphas, betas, t, imaginary, yr, yi) != 0) {
    free(alphas); free(betas); free(yr); free(yi);
    return -2;
  }
  for (int i = 0; i < m; ++i) {
    yr[i] *= b_norm;
    yi[i] *= b_norm;
  }
  or_lanczos_pass_two(&op, psi0, m, alphas, betas, b_norm, yr, yi, out);
  free(alphas);
  free(betas);
  free(yr);
  free(yi);
  return m;
}

/* ------------------------------------------------------------------------ */
/* KPM (src/numerics/kpm.h, src/numerics/rescaling.h).                      */
/* ------------------------------------------------------------------------ */

/* jackson_kernel (kpm.h:19-30) */
void or_jackson_kernel(int N, double* g) {
  const double denom = (double)(N + 1);
  const double cot_val = 1.0 / tan(OR_PI / denom);
  for (int n = 0; n <= N; ++n) {
    const double nd = (double)n;
    const double arg = OR_PI * nd / denom;
    g[n] = ((denom - nd) * cos(arg) + sin(arg) * cot_val) / denom;
  }
}

/* lorentz_kernel (kpm.h:34-44) */
void or_lorentz_kernel(int N, double lambda, double* g) {
  const double sl = sinh(lambda);
  for (int n = 0; n <= N; ++n) g[n] = sinh(lambda * (1.0 - (double)n / (double)N)) / sl;
}

/* projector_moments (kpm.h:51-61) */
void or_projector_moments(int M, double eps, double* mu) {
  const double ac = acos(eps);
  mu[0] = 1.0 - ac / OR_PI;
  for (int m = 1; m <= M; ++m) mu[m] = -2.0 * sin((double)m * ac) / ((double)m * OR_PI);
}

/* rescaling::from_bounds (rescaling.h:33-38) */
void or_rescaling_from_bounds(double emin, double emax, double padding, double* a, double* b) {
  *a = (emax - emin) / 2.0 * (1.0 + padding);
  *b = (emax + emin) / 2.0;
}

/* DOS Chebyshev moments mu_n = <r|T_n(Ht)|r> of one probe r, Ht = (H-b)/a,
 * by the recurrence T_{n+1} = 2 Ht T_n - T_{n-1} (kpm.h:212-229) with the
 * doubling identities mu_{2n} = 2<T_n|T_n> - mu_0 and
 * mu_{2n+1} = 2<T_{n+1}|T_n> - mu_1 (real parts).  A restatement: the
 * reference implements only the Fermi projector.  M = number of moments. */
int or_kpm_dos_moments(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx,
                       const double* re, const double* im, const double* r, int M, double a,
                       double b, double* mu) {
  or_op_ctx op = {dim, col_ptr, row_idx, re, im, 1.0 / a, b};
  const int64_t n2 = 2 * dim;
  for (int i = 0; i < M; ++i) mu[i] = 0.0;
  if (M <= 0) return 0;
  double* t_prev = (double*)malloc(sizeof(double) * (size_t)n2);
  double* t_curr = (double*)malloc(sizeof(double) * (size_t)n2);
  double* t_next = (double*)malloc(sizeof(double) * (size_t)n2);
  memcpy(t_prev, r, sizeof(double) * (size_t)n2);
  double mu0 = cdot_re(dim, r, r);
  mu[0] = mu0;
  if (M == 1) goto done;
  op_apply(&op, r, t_curr);
  double mu1 = cdot_re(dim, r, t_curr);
  mu[1] = mu1;
  /* n = 1: mu_2 = 2<T1|T1> - mu0 */
  for (int nn = 1; 2 * nn < M; ++nn) {
    mu[2 * nn] = 2.0 * cdot_re(dim, t_curr, t_curr) - mu0;
    if (2 * nn + 1 < M) {
      op_apply(&op, t_curr, t_next);
      for (int64_t i = 0; i < n2; ++i) t_next[i] = 2.0 * t_next[i] - t_prev[i];
      mu[2 * nn + 1] = 2.0 * cdot_re(dim, t_next, t_curr) - mu1;
      double* tmp = t_prev;
      t_prev = t_curr;
      t_curr = t_next;
      t_next = tmp;
    }
  }
done:
  free(t_prev);
  free(t_curr);
  free(t_next);
  return 0;
}

/* SparseKPMProjector::apply (kpm.h:212-229) on a complex vector:
 * out = sum_m g_m mu_m T_m(Ht) v with projector moments at E_fermi. */
int or_kpm_projector_apply(int64_t dim, const int64_t* col_ptr, const int64_t* row_idx,
                           const double* re, const double* im, int M, double emin, double emax,
                           double efermi, double padding, const double* v, double* out) {
  double a, b;
  or_rescaling_from_bounds(emin, emax, padding, &a, &b);
  double eps = (efermi - b) / a;
  double* g = (double*)malloc(sizeof(double) * (size_t)(M + 1));
  double* mu = (double*)malloc(sizeof(double) * (size_t)(M + 1));
  or_jackson_kernel(M, g);
  or_projector_moments(M, eps, mu);
  or_op_ctx op = {dim, col_ptr, row_idx, re, im, 1.0 / a, b};
  const int64_t n2 = 2 * dim;
  double* tp = (double*)malloc(sizeof(double) * (size_t)n2);
  double* tc = (double*)malloc(sizeof(double) * (size_t)n2);
  double* tn = (double*)malloc(sizeof(double) * (size_t)n2);
  memcpy(tp, v, sizeof(double) * (size_t)n2);
  for (int64_t i = 0; i < n2; ++i) out[i] = g[0] * mu[0] * tp[i];
  if (M > 0) {
    op_apply(&op, v, tc);
    for (int64_t i = 0; i < n2; ++i) out[i] += g[1] * mu[1] * tc[i];
    for (int m = 2; m <= M; ++m) {
      op_apply(&op, tc, tn);
      for (int64_t i = 0; i < n2; ++i) tn[i] = 2.0 * tn[i] - tp[i];
      for (int64_t i = 0; i < n2; ++i) out[i] += g[m] * mu[m] * tn[i];
      double* tmp = tp;
      tp = tc;
      tc = tn;
      tn = tmp;
    }
  }
  free(g);
  free(mu);
  free(tp);
  free(tc);
  free(tn);
  return 0;
}
