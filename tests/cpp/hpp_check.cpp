// Compiles the C++ layer (include/manybody_gb300.hpp) against the C ABI and
// exercises it the way the reference's code uses FermionBasis / HubbardModel
// / LinearOperator.  Exit 0 = all checks passed; prints one line per check.
//   hpp_check host   -- host-only checks (no GPU needed)
//   hpp_check gpu    -- also the operator apply and the device Lanczos
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>

#include "manybody_gb300.hpp"

// Minimal stand-in for arma::cx_vec: the members GpuHubbardOperator uses.
struct CxVec {
  explicit CxVec(size_t n) : n_elem(n), data(n) {}
  std::complex<double>* memptr() { return data.data(); }
  const std::complex<double>* memptr() const { return data.data(); }
  size_t n_elem;
  std::vector<std::complex<double>> data;
};

// Generic code written against the reference's LinearOperator concept
// (linear_operator.h:34-43): Rayleigh quotient <v, H v> / <v, v>.
template <typename Op>
double rayleigh(const Op& op, const typename Op::VectorType& v) {
  typename Op::VectorType w = op.apply(v);
  typename Op::ScalarType num = 0, den = 0;
  for (size_t i = 0; i < op.dimension(); ++i) {
    num += std::conj(v.data[i]) * w.data[i];
    den += std::conj(v.data[i]) * v.data[i];
  }
  return (num / den).real();
}

// The call shape of the reference's find_min_eigenpair (lanczos.h:283-290):
// the largest eigenvalue of Negated<Op> (linear_operator.h:93-105) by the
// Lanczos recurrence (lanczos.h:15-40) -- w = A v - beta v_prev, alpha =
// Re<v, w>, w -= alpha v, beta = ||w||, stop at beta <= 1000 eps -- through
// nothing but Op::apply and Op::dimension on the operator's own VectorType,
// then the tridiagonal's largest eigenvalue by Sturm bisection.
template <typename Op>
struct Negated {
  using VectorType = typename Op::VectorType;
  using ScalarType = typename Op::ScalarType;
  Op op;  // by value, as linear_operator.h:93-105 holds it
  VectorType apply(const VectorType& v) const {
    VectorType w = op.apply(v);
    for (auto& x : w.data) x = -x;
    return w;
  }
  size_t dimension() const { return op.dimension(); }
};

inline double tridiag_largest(const std::vector<double>& a, const std::vector<double>& b) {
  const size_t m = a.size();
  double lo = a[0], hi = a[0];
  for (size_t i = 0; i < m; ++i) {
    const double r = (i ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::fmin(lo, a[i] - r);
    hi = std::fmax(hi, a[i] + r);
  }
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    size_t below = 0;
    double q = 1.0;
    for (size_t i = 0; i < m; ++i) {
      q = a[i] - mid - (i ? b[i - 1] * b[i - 1] / q : 0.0);
      if (q == 0.0) q = -1e-300;
      if (q < 0.0) ++below;
    }
    if (below == m) hi = mid;
    else lo = mid;
  }
  return hi;
}

template <typename Op>
double lanczos_largest(const Op& op, const typename Op::VectorType& b, size_t k) {
  using V = typename Op::VectorType;
  const size_t n = op.dimension();
  V v(n), vp(n);
  double nb = 0.0;
  for (size_t i = 0; i < n; ++i) nb += std::norm(b.data[i]);
  nb = std::sqrt(nb);
  for (size_t i = 0; i < n; ++i) v.data[i] = b.data[i] / nb;
  std::vector<double> alpha, beta;
  double bprev = 0.0;
  for (size_t j = 0; j < k; ++j) {
    V w = op.apply(v);
    double al = 0.0;
    for (size_t i = 0; i < n; ++i) {
      w.data[i] -= bprev * vp.data[i];
      al += (std::conj(v.data[i]) * w.data[i]).real();
    }
    double nw = 0.0;
    for (size_t i = 0; i < n; ++i) {
      w.data[i] -= al * v.data[i];
      nw += std::norm(w.data[i]);
    }
    alpha.push_back(al);
    bprev = std::sqrt(nw);
    if (bprev <= 1000.0 * 2.220446049250313e-16) break;
    beta.push_back(bprev);
    vp = v;
    for (size_t i = 0; i < n; ++i) v.data[i] = w.data[i] / bprev;
  }
  return tridiag_largest(alpha, beta);
}

#define CHECK(cond)                                         \
  do {                                                      \
    if (!(cond)) {                                          \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); \
      return 1;                                             \
    }                                                       \
    std::printf("ok   %s\n", #cond);                        \
  } while (0)

int main(int argc, char** argv) {
  const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
  auto basis = mbgpu::FermionBasis::with_fixed_particle_number_and_spin(8, 8, 0);
  CHECK(basis.size() == 4900);
  auto keys = basis.keys();
  CHECK(keys.first[0] == 0b1111 && keys.second[0] == 0b1111000);  // reference index 0
  CHECK(basis.index_of(keys.first[123], keys.second[123]) == 123);
  CHECK(!basis.contains(0b1, 0b1));
  mbgpu::HubbardModel chain(1.0, 4.0, 8);
  CHECK(mbgpu::HubbardModel(1.0, 2.0, 2).term_count() == 6);
  CHECK(mbgpu::HubbardModel2D(1.0, 2.0, 2, 2).term_count() == 20);
  CHECK(mbgpu::HubbardModel3D(1.0, 2.0, 2, 2, 2).term_count() == 56);
  CHECK(chain.kinetic().term_count() + chain.interaction().term_count() == chain.term_count());
  CHECK(chain.kinetic().u == 0.0 && chain.interaction().t == 0.0);
  auto all = mbgpu::FermionBasis::with_fixed_particle_number(8, 8);
  CHECK(all.size() == 12870);  // C(16, 8): every spin projection
  auto ksec = mbgpu::FermionBasis::with_fixed_particle_number_spin_momentum(8, 4, 0, {8}, {0});
  CHECK(ksec.size() == 100);
  CHECK(mbgpu::HubbardModelMomentum(1.0, 4.0, {8}).term_count() == 524);
  bool threw = false;
  try {
    mbgpu::FermionBasis::with_fixed_particle_number_and_spin(4, 3, 0);
  } catch (const mbgpu::Error& e) {
    threw = e.status == MB_ERR_INVALID_ARG;
  }
  CHECK(threw);
  if (!gpu) {
    int n = 0;
    mb_device_count(&n);
    if (n == 0) {
      threw = false;
      try {
        mbgpu::GpuHubbardOperator<CxVec> op(basis, chain);
      } catch (const mbgpu::Error& e) {
        threw = e.status == MB_ERR_NO_DEVICE;
      }
      CHECK(threw);
    }
    return 0;
  }
  mbgpu::GpuHubbardOperator<CxVec> op(basis, chain);
  CHECK(op.dimension() == 4900);
  auto H = mbgpu::compute_matrix_elements(basis, chain);
  CHECK(H.row_ptr.back() == 49630);
  CxVec v(4900);
  for (size_t i = 0; i < v.n_elem; ++i) v.data[i] = {std::sin(0.1 * i), std::cos(0.37 * i)};
  CxVec w = op.apply(v);
  double err = 0, nrm = 0;
  for (size_t i = 0; i < H.n; ++i) {
    std::complex<double> s = 0;
    for (int64_t p = H.row_ptr[i]; p < H.row_ptr[i + 1]; ++p) s += H.values[p] * v.data[H.col_idx[p]];
    err += std::norm(s - w.data[i]);
    nrm += std::norm(s);
  }
  CHECK(std::sqrt(err / nrm) < 1e-13);
  const double rq = rayleigh(op, v);
  CHECK(std::isfinite(rq));
  // the tuned shape applies the same H (FP64: within rounding of the default)
  CHECK(op.autotune() > 0.0);
  CHECK(op.apply_shape().passes == 1);
  CxVec w2 = op.apply(v);
  double d2 = 0;
  for (size_t i = 0; i < H.n; ++i) d2 += std::norm(w2.data[i] - w.data[i]);
  CHECK(std::sqrt(d2 / nrm) < 1e-13);
  // a copy shares the device operator (the reference's Negated<Op> and
  // Scaled<Op> hold their operator by value)
  const mbgpu::GpuHubbardOperator<CxVec> copy = op;
  CHECK(copy.handle() == op.handle() && copy.dimension() == op.dimension());
  CxVec w3 = copy.apply(v);
  bool same = true;
  for (size_t i = 0; i < H.n; ++i) same = same && w3.data[i] == w2.data[i];
  CHECK(same);
  void* seed = nullptr;
  mbgpu::check(mb_alloc(&seed, sizeof(std::complex<double>) * 4900));
  mbgpu::check(mb_fill_uniform(op.handle(), 0, 0, seed, MB_ORDER_REFERENCE, nullptr));
  const double e0 = mbgpu::find_min_eigenpair(op, 200, seed);
  std::printf("E0 = %.12f\n", e0);
  CHECK(std::fabs(e0 - (-4.603526299989141)) < 1e-9);
  // the same seed driven from the host through GpuHubbardOperator::apply
  CxVec hseed(4900);
  mbgpu::check(mb_memcpy(hseed.memptr(), seed, sizeof(std::complex<double>) * 4900, 1));
  const double e0_host = -lanczos_largest(Negated<mbgpu::GpuHubbardOperator<CxVec>>{op}, hseed, 200);
  std::printf("E0 (host-driven Lanczos) = %.12f\n", e0_host);
  CHECK(std::fabs(e0_host - e0) < 1e-9);
  // HubbardMomentumFactorized, constructed as the reference's (basis, sizes,
  // t, U): the real-space ground state, reached in another orbital basis
  mbgpu::HubbardMomentumFactorized<CxVec> fact(basis, {8}, 1.0, 4.0);
  CHECK(fact.dimension() == 4900);
  mbgpu::check(mb_fill_uniform(fact.handle(), 0, 0, seed, MB_ORDER_REFERENCE, nullptr));
  const double e0k = mbgpu::find_min_eigenpair(fact, 200, seed);
  std::printf("E0 (momentum space) = %.12f\n", e0k);
  CHECK(std::fabs(e0k - e0) < 1e-9);
  mb_free(seed);
  return 0;
}
