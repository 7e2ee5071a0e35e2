// manybody_gb300.hpp -- header-only C++ layer over the C ABI that keeps the
// reference library's calling surface (keyehzy/manybody):
//
//   reference                                        here
//   FermionBasis::with_fixed_particle_number_and_spin mbgpu::FermionBasis::with_fixed_particle_number_and_spin
//     (src/algebra/basis.cpp:91-126); also with_fixed_particle_number (:69-89)
//     and with_fixed_particle_number_spin_momentum (:128-185)
//   basis.set.size() / index_of / contains            size() / index_of() / contains()
//   HubbardModel / 2D / 3D (t, u, sizes...)           mbgpu::HubbardModel / 2D / 3D
//     (src/algebra/fermion/model/hubbard_model.h)
//   HubbardModelMomentum (t, u, sizes)                mbgpu::HubbardModelMomentum
//   HubbardMomentumFactorized (basis, sizes, t, U)    mbgpu::HubbardMomentumFactorized<V>
//     (src/numerics/hubbard_momentum_factorized.h:32-249)
//   compute_matrix_elements<sp_cx_mat>(basis, H)      mbgpu::compute_matrix_elements(basis, model)
//     (src/algebra/matrix_elements.h:74-105)
//   SparseComplexMatrixOperator (linear_operator.h:81-91)
//                                                     mbgpu::GpuHubbardOperator<VectorType>
//   find_min_eigenpair(op, k) (lanczos.h:283-290)     mbgpu::find_min_eigenpair(op, k, seed)
//
// GpuHubbardOperator<V> models the reference's LinearOperator concept
// (VectorType, ScalarType, apply(const V&) const -> V, dimension()), so the
// reference's own header-only drivers (lanczos.h, kpm.h, evolve_state.h)
// accept it unchanged with V = arma::cx_vec: apply() copies the host vector
// to the GPU, applies H there (reference order) and copies the result back.
// V needs only V(n), .memptr() and .n_elem (arma::cx_vec has them).  The
// device-resident drivers (find_min_eigenpair etc. below) keep the whole
// Krylov iteration on the GPU and are the fast path.
//
// Errors: every failing mb_* call throws mbgpu::Error (a std::runtime_error
// carrying the mb_status), matching the reference's use of exceptions.
#pragma once

#include <complex>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "manybody_gb300.h"

namespace mbgpu {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status) {
  if (status != MB_OK) throw Error(status, mb_last_error());
}

class FermionBasis {
 public:
  static FermionBasis with_fixed_particle_number_and_spin(size_t orbitals, size_t particles,
                                                          int spin_projection) {
    mb_basis_t h = nullptr;
    check(mb_basis_create_fixed_spin((int64_t)orbitals, (int64_t)particles, spin_projection, &h));
    return FermionBasis(h, orbitals, particles);
  }
  // with_fixed_particle_number (src/algebra/basis.cpp:69-89): all spin projections
  static FermionBasis with_fixed_particle_number(size_t orbitals, size_t particles) {
    mb_basis_t h = nullptr;
    check(mb_basis_create_fixed_number((int64_t)orbitals, (int64_t)particles, &h));
    return FermionBasis(h, orbitals, particles);
  }
  // with_fixed_particle_number_spin_momentum (src/algebra/basis.cpp:128-185); the
  // reference passes an Index of the lattice sizes
  static FermionBasis with_fixed_particle_number_spin_momentum(
      size_t orbitals, size_t particles, int spin_projection, const std::vector<size_t>& sizes,
      const std::vector<size_t>& momentum) {
    std::vector<int64_t> d(sizes.begin(), sizes.end()), k(momentum.begin(), momentum.end());
    mb_basis_t h = nullptr;
    check(mb_basis_create_momentum(d.data(), (int)d.size(), (int64_t)particles, spin_projection,
                                   k.data(), &h));
    (void)orbitals;
    return FermionBasis(h, orbitals, particles);
  }
  FermionBasis(FermionBasis&& o) noexcept : h_(std::exchange(o.h_, nullptr)),
                                            orbitals(o.orbitals), particles(o.particles) {}
  FermionBasis& operator=(FermionBasis&& o) noexcept {
    std::swap(h_, o.h_);
    orbitals = o.orbitals;
    particles = o.particles;
    return *this;
  }
  FermionBasis(const FermionBasis&) = delete;
  FermionBasis& operator=(const FermionBasis&) = delete;
  ~FermionBasis() { mb_basis_destroy(h_); }

  size_t size() const {
    int64_t n = 0;
    check(mb_basis_size(h_, &n));
    return (size_t)n;
  }
  size_t index_of(uint64_t up_mask, uint64_t down_mask) const {
    int64_t i = 0;
    check(mb_basis_index_of(h_, up_mask, down_mask, &i));
    return (size_t)i;
  }
  bool contains(uint64_t up_mask, uint64_t down_mask) const {
    int64_t i = 0;
    return mb_basis_index_of(h_, up_mask, down_mask, &i) == MB_OK;
  }
  // Keys in reference index order as (up mask, down mask).
  std::pair<std::vector<uint64_t>, std::vector<uint64_t>> keys() const {
    std::vector<uint64_t> up(size()), down(size());
    check(mb_basis_export_reference_order(h_, up.data(), down.data()));
    return {std::move(up), std::move(down)};
  }
  mb_basis_t handle() const { return h_; }

 private:
  FermionBasis(mb_basis_t h, size_t o, size_t p) : h_(h), orbitals(o), particles(p) {}
  mb_basis_t h_ = nullptr;

 public:
  size_t orbitals = 0;
  size_t particles = 0;
};

class HubbardModelBase {
 public:
  HubbardModelBase(double t, double u, std::vector<int64_t> dims, bool momentum = false)
      : t(t), u(u), dims_(dims), momentum_(momentum) {
    if (momentum) check(mb_hubbard_momentum_create(dims.data(), (int)dims.size(), t, u, &h_));
    else check(mb_hubbard_create(dims.data(), (int)dims.size(), t, u, &h_));
  }
  // kinetic() / interaction() (hubbard_model.h:13-32): the hopping terms
  // alone (U = 0) or the U n_up n_down terms alone (t = 0), as models
  HubbardModelBase kinetic() const { return HubbardModelBase(t, 0.0, dims_, momentum_); }
  HubbardModelBase interaction() const { return HubbardModelBase(0.0, u, dims_, momentum_); }
  HubbardModelBase(HubbardModelBase&& o) noexcept
      : t(o.t), u(o.u), dims_(std::move(o.dims_)), momentum_(o.momentum_),
        h_(std::exchange(o.h_, nullptr)) {}
  HubbardModelBase(const HubbardModelBase&) = delete;
  HubbardModelBase& operator=(const HubbardModelBase&) = delete;
  ~HubbardModelBase() { mb_model_destroy(h_); }
  // FermionExpression::size() of hamiltonian()
  size_t term_count() const {
    int64_t n = 0;
    check(mb_model_term_count(h_, &n));
    return (size_t)n;
  }
  mb_model_t handle() const { return h_; }
  double t, u;

 private:
  std::vector<int64_t> dims_;
  bool momentum_ = false;
  mb_model_t h_ = nullptr;
};

struct HubbardModel : HubbardModelBase {
  HubbardModel(double t, double u, size_t size) : HubbardModelBase(t, u, {(int64_t)size}) {}
};
struct HubbardModel2D : HubbardModelBase {
  HubbardModel2D(double t, double u, size_t sx, size_t sy)
      : HubbardModelBase(t, u, {(int64_t)sx, (int64_t)sy}) {}
};
struct HubbardModel3D : HubbardModelBase {
  HubbardModel3D(double t, double u, size_t sx, size_t sy, size_t sz)
      : HubbardModelBase(t, u, {(int64_t)sx, (int64_t)sy, (int64_t)sz}) {}
};
// HubbardModelMomentum (src/algebra/fermion/model/hubbard_model_momentum.h:19-180)
struct HubbardModelMomentum : HubbardModelBase {
  HubbardModelMomentum(double t, double u, const std::vector<size_t>& size)
      : HubbardModelBase(t, u, std::vector<int64_t>(size.begin(), size.end()), true) {}
};

// Reference-order CSR of H, values complex<double>.
struct CsrMatrix {
  size_t n = 0;
  std::vector<int64_t> row_ptr, col_idx;
  std::vector<std::complex<double>> values;
};

inline CsrMatrix compute_matrix_elements(const FermionBasis& basis, const HubbardModelBase& model) {
  CsrMatrix m;
  m.n = basis.size();
  int64_t nnz = 0;
  m.row_ptr.resize(m.n + 1);
  check(mb_compute_matrix_elements_csr(basis.handle(), model.handle(), &nnz, m.row_ptr.data(),
                                       nullptr, nullptr));
  m.col_idx.resize((size_t)nnz);
  m.values.resize((size_t)nnz);
  check(mb_compute_matrix_elements_csr(basis.handle(), model.handle(), &nnz, m.row_ptr.data(),
                                       m.col_idx.data(),
                                       reinterpret_cast<double*>(m.values.data())));
  return m;
}

// The matrix-free GPU operator, shaped like the reference's LinearOperator.
// Copies share one device operator (its apply is const and safe from several
// threads), as the reference's drivers copy the operators they wrap:
// find_min_eigenpair builds Negated<Op>(op) by value (lanczos.h:283-290,
// linear_operator.h:93-105).
template <typename Vector>
class GpuHubbardOperator {
 public:
  using VectorType = Vector;
  using ScalarType = std::complex<double>;

  GpuHubbardOperator(const FermionBasis& basis, const HubbardModelBase& model,
                     int precision = MB_PREC_F64) {
    mb_op_t h = nullptr;
    check(mb_op_create(basis.handle(), model.handle(), precision, &h));
    h_ = std::shared_ptr<std::remove_pointer_t<mb_op_t>>(h, [](mb_op_t p) { mb_op_destroy(p); });
    check(mb_op_dimension(h, &dim_));
  }

  // LinearOperator::apply (linear_operator.h:41): a fresh vector H v.
  VectorType apply(const VectorType& v) const {
    if ((int64_t)v.n_elem != dim_) throw Error(MB_ERR_DIM_MISMATCH, "vector dimension mismatch");
    VectorType out((size_t)dim_);
    check(mb_op_apply_host(h_.get(), v.memptr(), out.memptr(), MB_ORDER_REFERENCE));
    return out;
  }
  size_t dimension() const { return (size_t)dim_; }
  mb_op_t handle() const { return h_.get(); }
  // Times the apply's kernel shapes on the GPU and keeps the fastest
  // (mb_op_autotune; cached per sector); returns ms per apply.
  double autotune() {
    mb_apply_shape s{};
    double ms = 0.0;
    check(mb_op_autotune(h_.get(), nullptr, &s, &ms));
    return ms;
  }
  mb_apply_shape apply_shape() const {
    mb_apply_shape s{};
    check(mb_op_get_apply_shape(h_.get(), &s));
    return s;
  }

 private:
  std::shared_ptr<std::remove_pointer_t<mb_op_t>> h_;
  int64_t dim_ = 0;
};

// HubbardMomentumFactorized (src/numerics/hubbard_momentum_factorized.h:32-249):
// the momentum-space Hubbard operator on a whole (N_up, N_down) basis,
// constructed as the reference's (basis, lattice_size, t, U); on the GPU it
// is block diagonal over the total momentum (one sector operator per K).
template <class Vector>
class HubbardMomentumFactorized : public GpuHubbardOperator<Vector> {
 public:
  HubbardMomentumFactorized(const FermionBasis& basis, const std::vector<size_t>& lattice_size,
                            double t, double U, int precision = MB_PREC_F64)
      : GpuHubbardOperator<Vector>(basis, HubbardModelMomentum(t, U, lattice_size), precision) {}
};

// Device-resident find_min_eigenpair (lanczos.h:283-290) from a device seed
// vector in reference order.  Returns E0; writes the Ritz vector if vec_dev.
template <typename Op>
double find_min_eigenpair(const Op& op, size_t k, const void* seed_dev, void* vec_dev = nullptr,
                          const mb_lanczos_opts* opts = nullptr) {
  double e0 = 0.0;
  int64_t steps = 0;
  check(mb_find_min_eigenpair(op.handle(), (int64_t)k, seed_dev, MB_ORDER_REFERENCE, opts, &e0,
                              vec_dev, &steps));
  return e0;
}

}  // namespace mbgpu
