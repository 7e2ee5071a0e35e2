// Test infrastructure: writes a sparse complex matrix as a cereal binary
// archive through the cereal library the reference vendors
// (third-party/cereal), with the field sequence of the reference's
// arma::SpMat save (src/utils/arma_cereal.h:9-17): a versioned non-member
// save of (n_rows, n_cols, n_nonzero), then (row, col, value) per non-zero
// in the matrix iterator's column-major order.  arma::uword is 64-bit on
// 64-bit hosts.  It pins the byte layout that the engine's own
// mb_cereal_write_csr / mb_cereal_read_csr produce and parse.
//
// stdin: "n_rows n_cols nnz" then nnz lines "row col re im" (column-major
// order); argv[1]: output path.
#include <cereal/archives/binary.hpp>
#include <cereal/cereal.hpp>
#include <cereal/types/complex.hpp>

#include <complex>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <vector>

struct SparseEntries {
  uint64_t n_rows = 0, n_cols = 0, n_nonzero = 0;
  std::vector<uint64_t> row, col;
  std::vector<std::complex<double>> val;
};

template <class Archive>
void save(Archive& ar, const SparseEntries& m, unsigned int /* version */) {
  ar(m.n_rows, m.n_cols, m.n_nonzero);
  for (uint64_t i = 0; i < m.n_nonzero; ++i) ar(m.row[i], m.col[i], m.val[i]);
}

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: cereal_pin OUT < entries.txt\n");
    return 2;
  }
  SparseEntries m;
  unsigned long long r, c, n;
  if (std::scanf("%llu %llu %llu", &r, &c, &n) != 3) return 3;
  m.n_rows = r;
  m.n_cols = c;
  m.n_nonzero = n;
  for (unsigned long long i = 0; i < n; ++i) {
    unsigned long long ri, ci;
    double re, im;
    if (std::scanf("%llu %llu %lf %lf", &ri, &ci, &re, &im) != 4) return 4;
    m.row.push_back(ri);
    m.col.push_back(ci);
    m.val.emplace_back(re, im);
  }
  std::ofstream ofs(argv[1], std::ios::binary);
  cereal::BinaryOutputArchive archive(ofs);
  archive(m);
  return 0;
}
