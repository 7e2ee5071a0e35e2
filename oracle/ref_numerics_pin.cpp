// Runs the reference's own numerics drivers (numerics/lanczos.h,
// numerics/evolve_state.h and numerics/kpm.h, unchanged, from the reference's
// source tree) on the CPU, on the reference's own SparseComplexMatrixOperator, with the minimal
// Armadillo stand-in of oracle/arma_shim; the oracle's restatements are
// compared with its outputs (tests/test_oracle_numerics_pin.py).  Test
// infrastructure, built by oracle/build_ref.sh into oracle/_ref/.
//
// Input (binary, native endianness): int64 dim, int64 nnz, int64 k,
// double t, int64 M, double e_min, e_max, e_fermi, padding, int64
// col_ptr[dim + 1], int64 row_idx[nnz], complex128 values[nnz], complex128
// seed[dim], complex128 psi[dim].
// Output: int64 m, double e0, double alphas[m], double betas[m - 1],
// complex128 vec[dim] (find_min_eigenpair from `seed`), then complex128
// exp(-i t H) psi and exp(-t H) psi (30 Krylov steps), then double
// jackson_kernel(M)[M + 1], lorentz_kernel(M, 4)[M + 1],
// projector_moments(M, eps)[M + 1] (eps = e_fermi rescaled by from_bounds),
// and complex128 P psi for the SparseKPMProjector of H's real part (applied to
// Re psi and Im psi: its vectors are real).
#include <cstdio>
#include <vector>

#include "numerics/evolve_state.h"
#include "numerics/kpm.h"
#include "numerics/lanczos.h"

template <typename T>
static bool read_all(std::FILE* f, T* p, size_t n) {
  return std::fread(p, sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  std::FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 3;
  int64_t dim = 0, nnz = 0, k = 0, M = 0;
  double t = 0.0, kb[4] = {0.0, 0.0, 0.0, 0.0};  // e_min, e_max, e_fermi, padding
  if (!read_all(in, &dim, 1) || !read_all(in, &nnz, 1) || !read_all(in, &k, 1) ||
      !read_all(in, &t, 1) || !read_all(in, &M, 1) || !read_all(in, kb, 4))
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

  // KPM (kpm.h): kernels, projector moments, the sparse projector
  const std::vector<double> jk = kpm::jackson_kernel((size_t)M);
  const std::vector<double> lk = kpm::lorentz_kernel((size_t)M, 4.0);
  const double eps = rescaling::from_bounds(kb[0], kb[1], kb[3]).rescale(kb[2]);
  const std::vector<double> pm = kpm::projector_moments((size_t)M, eps);
  arma::sp_mat Hr;
  Hr.n_rows = Hr.n_cols = (arma::uword)dim;
  Hr.n_nonzero = (arma::uword)nnz;
  Hr.col_ptrs = H.col_ptrs;
  Hr.row_indices = H.row_indices;
  for (const auto& v : H.values) Hr.values.push_back(v.real());
  kpm::SparseKPMProjector P(Hr, (size_t)M, kb[0], kb[1], kb[2], kb[3]);
  arma::vec pr((arma::uword)dim), pi((arma::uword)dim);
  for (int64_t i = 0; i < dim; ++i) {
    pr(i) = psi[(size_t)i].real();
    pi(i) = psi[(size_t)i].imag();
  }
  const arma::vec Pr = P.apply(pr), Pi = P.apply(pi);
  std::vector<arma::cx_double> Pc((size_t)dim);
  for (int64_t i = 0; i < dim; ++i) Pc[(size_t)i] = {Pr(i), Pi(i)};

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
  std::fwrite(jk.data(), sizeof(double), jk.size(), out);
  std::fwrite(lk.data(), sizeof(double), lk.size(), out);
  std::fwrite(pm.data(), sizeof(double), pm.size(), out);
  std::fwrite(Pc.data(), sizeof(arma::cx_double), Pc.size(), out);
  std::fclose(out);
  return 0;
}
