// Sparse matrices in the reference's Hamiltonian cache format.
//
// The reference caches sparse Hamiltonians (examples/
// hubbard_momentum_optical_conductivity.cpp:185-203) as cereal binary
// archives of arma::SpMat<std::complex<double>> (src/utils/arma_cereal.h:9-30):
//   uint32  class version (0; cereal writes it once for a versioned save)
//   uint64  n_rows, n_cols, n_nonzero            (arma::uword, 64-bit hosts)
//   n_nonzero x { uint64 row, uint64 col, float64 re, float64 im }
// in the matrix iterator's column-major order, little-endian.  Loading
// assigns t(row, col) = value per entry, so a later duplicate wins and an
// explicit zero stores nothing.  These host functions write and read that
// layout from and to CSR (the engine's sparse-matrix operators,
// mb_op_create_csr, take CSR).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "mb_internal.h"

namespace mb {
namespace {

struct File {
  std::FILE* f = nullptr;
  File(const char* path, const char* mode) : f(std::fopen(path, mode)) {}
  ~File() {
    if (f) std::fclose(f);
  }
};

template <typename T>
void put(std::FILE* f, T v) {
  MB_REQUIRE(std::fwrite(&v, sizeof(T), 1, f) == 1, MB_ERR_INVALID_ARG, "write failed");
}

template <typename T>
T get(std::FILE* f) {
  T v{};
  MB_REQUIRE(std::fread(&v, sizeof(T), 1, f) == 1, MB_ERR_INVALID_ARG,
             "truncated sparse-matrix archive");
  return v;
}

struct Entry {
  int64_t row, col;
  double re, im;
};

// Parses the archive into entries in file order.
void read_entries(const char* path, int64_t& n_rows, int64_t& n_cols, std::vector<Entry>& out) {
  File in(path, "rb");
  MB_REQUIRE(in.f, MB_ERR_INVALID_ARG, std::string("cannot open ") + path);
  const uint32_t version = get<uint32_t>(in.f);
  MB_REQUIRE(version == 0, MB_ERR_INVALID_ARG, "unknown sparse-matrix archive version");
  const uint64_t r = get<uint64_t>(in.f), c = get<uint64_t>(in.f), nz = get<uint64_t>(in.f);
  MB_REQUIRE(r < (uint64_t(1) << 62) && c < (uint64_t(1) << 62), MB_ERR_INVALID_ARG,
             "implausible matrix size in archive");
  MB_REQUIRE((r == 0 || c == 0) ? nz == 0 : nz / r <= c, MB_ERR_INVALID_ARG,
             "more non-zeros than matrix elements");
  n_rows = (int64_t)r;
  n_cols = (int64_t)c;
  out.clear();
  out.reserve((size_t)nz);
  for (uint64_t i = 0; i < nz; ++i) {
    Entry e;
    const uint64_t row = get<uint64_t>(in.f), col = get<uint64_t>(in.f);
    e.re = get<double>(in.f);
    e.im = get<double>(in.f);
    MB_REQUIRE(row < r && col < c, MB_ERR_INVALID_ARG, "entry outside the matrix");
    e.row = (int64_t)row;
    e.col = (int64_t)col;
    out.push_back(e);
  }
}

}  // namespace
}  // namespace mb

using namespace mb;

extern "C" {

int mb_cereal_write_csr(const char* path, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr,
                        const int64_t* col_idx, const double* values) {
  return guard([&] {
    MB_REQUIRE(path && row_ptr && n_rows >= 0 && n_cols >= 0, MB_ERR_INVALID_ARG,
               "NULL argument or negative size");
    const int64_t nnz = row_ptr[n_rows];
    MB_REQUIRE(nnz == 0 || (col_idx && values), MB_ERR_INVALID_ARG, "NULL col_idx or values");
    // column-major order: counting sort of the entries by column (rows stay
    // ascending inside a column because CSR rows are visited in order)
    std::vector<int64_t> start((size_t)n_cols + 1, 0);
    for (int64_t k = 0; k < nnz; ++k) {
      MB_REQUIRE(col_idx[k] >= 0 && col_idx[k] < n_cols, MB_ERR_INVALID_ARG,
                 "column index out of range");
      ++start[(size_t)col_idx[k] + 1];
    }
    std::partial_sum(start.begin(), start.end(), start.begin());
    std::vector<int64_t> order((size_t)nnz), rows((size_t)nnz);
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < n_rows; ++i) {
      MB_REQUIRE(row_ptr[i + 1] >= row_ptr[i], MB_ERR_INVALID_ARG, "row_ptr must not decrease");
      for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        const int64_t slot = fill[(size_t)col_idx[k]]++;
        order[(size_t)slot] = k;
        rows[(size_t)slot] = i;
      }
    }
    File out(path, "wb");
    MB_REQUIRE(out.f, MB_ERR_INVALID_ARG, std::string("cannot open ") + path);
    put<uint32_t>(out.f, 0u);
    put<uint64_t>(out.f, (uint64_t)n_rows);
    put<uint64_t>(out.f, (uint64_t)n_cols);
    put<uint64_t>(out.f, (uint64_t)nnz);
    for (int64_t s = 0; s < nnz; ++s) {
      const int64_t k = order[(size_t)s];
      put<uint64_t>(out.f, (uint64_t)rows[(size_t)s]);
      put<uint64_t>(out.f, (uint64_t)col_idx[k]);
      put<double>(out.f, values[2 * k]);
      put<double>(out.f, values[2 * k + 1]);
    }
    MB_REQUIRE(std::fflush(out.f) == 0, MB_ERR_INVALID_ARG, "write failed");
  });
}

int mb_cereal_read_csr(const char* path, int64_t* n_rows, int64_t* n_cols, int64_t* nnz,
                       int64_t* row_ptr, int64_t* col_idx, double* values) {
  return guard([&] {
    MB_REQUIRE(path && n_rows && n_cols && nnz, MB_ERR_INVALID_ARG, "NULL argument");
    int64_t r = 0, c = 0;
    std::vector<Entry> e;
    read_entries(path, r, c, e);
    // t(row, col) = value in file order: the last duplicate wins, zeros drop
    std::vector<size_t> idx(e.size());
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](size_t a, size_t b) {
      return e[a].row != e[b].row ? e[a].row < e[b].row : e[a].col < e[b].col;
    });
    std::vector<size_t> keep;
    keep.reserve(idx.size());
    for (size_t i = 0; i < idx.size(); ++i) {
      const bool last = i + 1 == idx.size() || e[idx[i + 1]].row != e[idx[i]].row ||
                        e[idx[i + 1]].col != e[idx[i]].col;
      if (last && (e[idx[i]].re != 0.0 || e[idx[i]].im != 0.0)) keep.push_back(idx[i]);
    }
    *n_rows = r;
    *n_cols = c;
    *nnz = (int64_t)keep.size();
    if (!row_ptr) return;
    MB_REQUIRE(keep.empty() || (col_idx && values), MB_ERR_INVALID_ARG, "NULL col_idx or values");
    std::fill(row_ptr, row_ptr + r + 1, 0);
    for (size_t i = 0; i < keep.size(); ++i) {
      const Entry& x = e[keep[i]];
      ++row_ptr[x.row + 1];
      col_idx[i] = x.col;
      values[2 * i] = x.re;
      values[2 * i + 1] = x.im;
    }
    for (int64_t i = 0; i < r; ++i) row_ptr[i + 1] += row_ptr[i];
  });
}

}  // extern "C"
