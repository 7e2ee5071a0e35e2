// Runs the reference's own numerics drivers (numerics/lanczos.h and
// numerics/evolve_state.h, unchanged, from the reference's source tree) on the
// CPU, on the reference's own SparseComplexMatrixOperator, with the minimal
// Armadillo stand-in of oracle/arma_shim; the oracle's restatements are
// compared with its outputs (tests/test_oracle_numerics_pin.py).  Test
// infrastructure, built by oracle/build_ref.sh into oracle/_ref/.
//
// Input (binary, native endianness): int64 dim, int64 nnz, int64 k,
// double t, int64 col_ptr[dim + 1], int64 row_idx[nnz], complex128
// values[nnz], complex128 seed[dim], complex128 psi[dim].
// Output: int64 m, double e0, double alphas[m], double betas[m - 1],
// complex128 vec[dim] (find_min_eigenpair from `seed`), then complex128
// exp(-i t H) psi and exp(-t H) psi (30 Krylov steps).
#include <cstdio>
#include <vector>

#include "numerics/evolve_state.h"
#include "numerics/lanczos.h"

template <typename T>
static bool read_all(std::FILE* f, T* p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  int64_t dim = 0, nnz = 0, k = 0;
  double t = 0.0;
  if (!read_all(in, &dim, 1) || !read_all(in, &nnz, 1) || !read_all(in, &k, 1) ||
      !read_all(in, &t, 1))
    return 4;
  arma::sp_cx_mat H;
  H.n_rows = H.n_cols = (arma::uword)dim;
  H.n_nonzero = (arma::uword)nnz;
  std::vector<int64_t> cp((size_t)dim + 1), ri((size_t)nnz);
  H.values.resize((size_t)nnz);
  std::vector<arma::cx_double> seed((size_t)dim), psi((size_t)dim);
  if (!read_all(in, cp.data(), cp.size()) || !read_all(in, ri.data(), ri.size()) ||
      !read_all(in, H.values.data(), H.values.size()) || !read_all(in, seed.data(), seed.size()) ||
      !read_all(in, psi.data(), psi.size()))
    return 5;
  std::fclose(in);
  H.col_ptrs.assign(cp.begin(), cp.end());
  H.row_indices.assign(ri.begin(), ri.end());

  SparseComplexMatrixOperator op(H);
  // find_min_eigenpair (lanczos.h:283-290) from `seed`: make_seed_vector's
  // fill::randu column takes it
  arma::detail::randu_source() = &seed;
  auto ev = find_min_eigenpair(op, (size_t)k);
  arma::detail::randu_source() = nullptr;
  // pass one of Negated<op> from the same seed: alpha, beta
  arma::cx_vec b((arma::uword)dim);
  for (int64_t i = 0; i < dim; ++i) b(i) = seed[(size_t)i];
  Negated<SparseComplexMatrixOperator> neg(op);
  auto decomp = lanczos_pass_one(neg, b, (size_t)k);

  arma::cx_vec p0((arma::uword)dim);
  for (int64_t i = 0; i < dim; ++i) p0(i) = psi[(size_t)i];
  EvolutionOptions opts{};
  opts.krylov_steps = 30;
  arma::cx_vec real_t = time_evolve_state(op, p0, t, opts);
  arma::cx_vec imag_t = imaginary_time_evolve_state(op, p0, t, opts);

  std::FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 6;
  const int64_t m = (int64_t)decomp.steps_taken;
  std::fwrite(&m, sizeof m, 1, out);
  std::fwrite(&ev.value, sizeof(double), 1, out);
  std::fwrite(decomp.alphas.data(), sizeof(double), (size_t)m, out);
  std::fwrite(decomp.betas.data(), sizeof(double), (size_t)(m > 0 ? m - 1 : 0), out);
  std::fwrite(ev.vector.memptr(), sizeof(arma::cx_double), (size_t)dim, out);
  std::fwrite(real_t.memptr(), sizeof(arma::cx_double), (size_t)dim, out);
  std::fwrite(imag_t.memptr(), sizeof(arma::cx_double), (size_t)dim, out);
  std::fclose(out);
  return 0;
}
