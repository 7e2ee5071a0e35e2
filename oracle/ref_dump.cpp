// Dumps the reference library's fixed-(N, Sz) fermion basis and the Hubbard
// Hamiltonian as that library builds it, for golden fixtures.
//
//   ref_dump <dims> <t> <U> <particles> <spin_projection> <out.bin>
//     dims: "8" (1D chain), "4x4" (2D), "2x2x2" (3D), all periodic.
//   ref_dump --current <dims> <t> <particles> <spin_projection> <K> <Q> <direction> <out.bin>
//     the current operator J_d(Q) (hubbard_model_momentum.h:52-90) from sector K
//     to sector K+Q through compute_rectangular_matrix_elements
//     (src/algebra/matrix_elements.h:107-167); output "MBREF002", u64 n_terms,
//     u64 rows, u64 cols, the row basis masks (up, down), the column basis
//     masks, u64 nnz, records as below.
//   ref_dump --all <dims> <t> <U> <particles> <out.bin>
//     all spin projections: FermionBasis::with_fixed_particle_number
//     (src/algebra/basis.cpp:69-89,248-266) with the real-space model.
//   ref_dump --momentum <dims> <t> <U> <particles> <spin_projection> <K> <out.bin>
//     the momentum-space model on one total-momentum sector K ("1", "1x0"):
//     FermionBasis::with_fixed_particle_number_spin_momentum
//     (src/algebra/basis.cpp:128-185,304-356) and HubbardModelMomentum
//     (src/algebra/fermion/model/hubbard_model_momentum.h:19-180).
//   ref_dump --momentum-full <dims> <t> <U> <particles> <spin_projection> <out.bin>
//     the momentum-space model on the whole (N_up, N_down) basis
//     (with_fixed_particle_number_and_spin, every total momentum): the matrix
//     the reference's HubbardMomentumFactorized applies
//     (src/numerics/hubbard_momentum_factorized.h:32-249), as its own test
//     builds it (tests/numerics/test_hubbard_momentum_factorized.cpp:54-130).
//
// Calls, unchanged, the reference's
//   FermionBasis::with_fixed_particle_number_and_spin   (src/algebra/basis.cpp:91-126)
//   HubbardModel / HubbardModel2D / HubbardModel3D       (src/algebra/fermion/model/hubbard_model.h)
//   compute_matrix_elements<MatrixType>                  (src/algebra/matrix_elements.h:74-105)
// with a coordinate-list MatrixType standing in for arma::sp_cx_mat.
//
// Output (little endian): "MBREF001", u64 n_terms, u64 dim, u64 up[dim],
// u64 down[dim] (occupation bit masks in reference index order), u64 nnz,
// then nnz records {i64 row, i64 col, f64 re, f64 im} sorted by (row, col).
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "algebra/fermion/basis.h"
#include "algebra/fermion/expression.h"
#include "algebra/fermion/model/hubbard_model.h"
#include "algebra/fermion/model/hubbard_model_momentum.h"
#include "utils/index.h"
#include "algebra/matrix_elements.h"

namespace {

struct CooMatrix {
  using value_type = std::complex<double>;
  CooMatrix(size_t r, size_t c) : rows(r), cols(c) {}
  void zeros() { entries.clear(); }
  value_type& operator()(size_t i, size_t j) { return entries[{i, j}]; }
  size_t rows, cols;
  std::map<std::pair<size_t, size_t>, value_type> entries;
};

std::vector<size_t> parse_dims(const std::string& s) {
  std::vector<size_t> dims;
  size_t start = 0;
  while (start <= s.size()) {
    size_t x = s.find('x', start);
    if (x == std::string::npos) x = s.size();
    dims.push_back(std::stoul(s.substr(start, x - start)));
    start = x + 1;
  }
  return dims;
}

}  // namespace

void put_masks(FILE* f, const FermionBasis& basis) {
  const size_t dim = basis.set.size();
  std::vector<uint64_t> up(dim, 0), down(dim, 0);
  for (size_t i = 0; i < dim; ++i) {
    for (const auto& op : basis.set[i]) {
      if (op.spin() == FermionOperator::Spin::Up)
        up[i] |= uint64_t{1} << op.value();
      else
        down[i] |= uint64_t{1} << op.value();
    }
  }
  std::fwrite(up.data(), 8, dim, f);
  std::fwrite(down.data(), 8, dim, f);
}

int dump_current(char** argv) {
  const std::vector<size_t> dims = parse_dims(argv[2]);
  const double t = std::atof(argv[3]);
  const size_t particles = std::stoul(argv[4]);
  const int sz = std::atoi(argv[5]);
  const std::vector<size_t> k = parse_dims(argv[6]), q = parse_dims(argv[7]);
  const size_t direction = std::stoul(argv[8]);
  size_t orbitals = 1;
  for (size_t d : dims) orbitals *= d;
  std::vector<size_t> kq(dims.size());
  for (size_t d = 0; d < dims.size(); ++d) kq[d] = (k[d] + q[d]) % dims[d];
  const FermionExpression j = HubbardModelMomentum(t, 0.0, dims).current(q, direction);
  FermionBasis col = FermionBasis::with_fixed_particle_number_spin_momentum(orbitals, particles, sz,
                                                                           Index(dims), k);
  FermionBasis row = FermionBasis::with_fixed_particle_number_spin_momentum(orbitals, particles, sz,
                                                                           Index(dims), kq);
  CooMatrix m = compute_rectangular_matrix_elements<CooMatrix>(row, col, j);
  FILE* f = std::fopen(argv[9], "wb");
  if (!f) return 3;
  std::fwrite("MBREF002", 1, 8, f);
  const uint64_t head[3] = {j.size(), row.set.size(), col.set.size()};
  std::fwrite(head, 8, 3, f);
  put_masks(f, row);
  put_masks(f, col);
  const uint64_t nnz = m.entries.size();
  std::fwrite(&nnz, 8, 1, f);
  for (const auto& [ij, v] : m.entries) {
    const int64_t rc[2] = {static_cast<int64_t>(ij.first), static_cast<int64_t>(ij.second)};
    const double re_im[2] = {v.real(), v.imag()};
    std::fwrite(rc, 8, 2, f);
    std::fwrite(re_im, 8, 2, f);
  }
  std::fclose(f);
  return 0;
}

int main(int argc, char** argv) {
  if (argc == 10 && std::string(argv[1]) == "--current") return dump_current(argv);
  const bool all_sz = argc == 7 && std::string(argv[1]) == "--all";
  if (all_sz) {  // same layout as the fixed-spin dump below, spin projection unused
    static char zero[] = "0";
    static char* shifted[8];
    shifted[0] = argv[0];
    shifted[1] = argv[2];
    shifted[2] = argv[3];
    shifted[3] = argv[4];
    shifted[4] = argv[5];
    shifted[5] = zero;
    shifted[6] = argv[6];
    argv = shifted;
  }
  const bool momentum_full = argc == 8 && std::string(argv[1]) == "--momentum-full";
  if (momentum_full) {  // the fixed-spin layout below, momentum-space model
    static char* shifted[8];
    for (int i = 0; i < 7; ++i) shifted[i] = argv[i + (i ? 1 : 0)];
    argv = shifted;
    argc = 7;
  }
  const bool momentum = argc == 9 && std::string(argv[1]) == "--momentum";
  if (argc != 7 && !momentum) {
    std::fprintf(stderr,
                 "usage: ref_dump <dims> <t> <U> <particles> <spin_projection> <out>\n"
                 "       ref_dump --momentum <dims> <t> <U> <particles> <spin_projection> <K> <out>\n");
    return 2;
  }
  char** a = momentum ? argv + 1 : argv;
  const std::vector<size_t> dims = parse_dims(a[1]);
  const double t = std::atof(a[2]);
  const double u = std::atof(a[3]);
  const size_t particles = std::stoul(a[4]);
  const int sz = std::atoi(a[5]);
  const char* out_path = momentum ? argv[8] : argv[6];

  size_t orbitals = 1;
  for (size_t d : dims) orbitals *= d;

  FermionExpression h;
  FermionBasis basis;
  if (momentum) {
    const std::vector<size_t> k = parse_dims(argv[7]);
    h = HubbardModelMomentum(t, u, dims).hamiltonian();
    basis = FermionBasis::with_fixed_particle_number_spin_momentum(orbitals, particles, sz,
                                                                   Index(dims), k);
  } else if (momentum_full) {
    h = HubbardModelMomentum(t, u, dims).hamiltonian();
    basis = FermionBasis::with_fixed_particle_number_and_spin(orbitals, particles, sz);
  } else {
    if (dims.size() == 1) {
      h = HubbardModel(t, u, dims[0]).hamiltonian();
    } else if (dims.size() == 2) {
      h = HubbardModel2D(t, u, dims[0], dims[1]).hamiltonian();
    } else if (dims.size() == 3) {
      h = HubbardModel3D(t, u, dims[0], dims[1], dims[2]).hamiltonian();
    } else {
      std::fprintf(stderr, "ref_dump: 1 to 3 dimensions\n");
      return 2;
    }
    basis = all_sz ? FermionBasis::with_fixed_particle_number(orbitals, particles)
                   : FermionBasis::with_fixed_particle_number_and_spin(orbitals, particles, sz);
  }
  CooMatrix m = compute_matrix_elements<CooMatrix>(basis, h);

  FILE* f = std::fopen(out_path, "wb");
  if (!f) return 3;
  std::fwrite("MBREF001", 1, 8, f);
  const uint64_t n_terms = h.size();
  const uint64_t dim = basis.set.size();
  std::fwrite(&n_terms, 8, 1, f);
  std::fwrite(&dim, 8, 1, f);
  std::vector<uint64_t> up(dim, 0), down(dim, 0);
  for (size_t i = 0; i < dim; ++i) {
    for (const auto& op : basis.set[i]) {
      if (op.type() != FermionOperator::Type::Creation) return 4;
      if (op.spin() == FermionOperator::Spin::Up)
        up[i] |= uint64_t{1} << op.value();
      else
        down[i] |= uint64_t{1} << op.value();
    }
  }
  std::fwrite(up.data(), 8, dim, f);
  std::fwrite(down.data(), 8, dim, f);
  const uint64_t nnz = m.entries.size();
  std::fwrite(&nnz, 8, 1, f);
  for (const auto& [ij, v] : m.entries) {
    const int64_t rc[2] = {static_cast<int64_t>(ij.first), static_cast<int64_t>(ij.second)};
    const double re_im[2] = {v.real(), v.imag()};
    std::fwrite(rc, 8, 2, f);
    std::fwrite(re_im, 8, 2, f);
  }
  std::fclose(f);
  return 0;
}
