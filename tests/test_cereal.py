"""The reference's sparse-matrix cache format (cereal binary archive of
arma::sp_cx_mat, src/utils/arma_cereal.h:9-30), through the C ABI on the host.

Pinned against archives written by the cereal library the reference vendors
(tests/golden/make_cereal_golden.py): bytes must be identical on write, and
entries identical on read.
"""
import os
import struct

import numpy as np
import pytest

from conftest import load_golden

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden_csr(mb, name):
    g = load_golden(name)
    import scipy.sparse as sp
    n = len(g["up"])
    m = sp.csr_matrix((g["val"].astype(np.complex128), (g["row"], g["col"])), shape=(n, n))
    m.sort_indices()
    return mb.CsrMatrix(n, m.indptr.astype(np.int64), m.indices.astype(np.int64), m.data)


def test_write_matches_vendored_cereal_bytes(mb, tmp_path):
    m = golden_csr(mb, "chain4_n4")
    out = tmp_path / "h.bin"
    mb.write_cereal(str(out), m)
    assert out.read_bytes() == open(os.path.join(GOLDEN, "cereal_chain4_n4.bin"), "rb").read()


def test_read_golden_archive(mb):
    m = mb.read_cereal(os.path.join(GOLDEN, "cereal_chain4_n4.bin"))
    ref = golden_csr(mb, "chain4_n4")
    assert m.dim == ref.dim and m.cols == ref.dim
    assert np.array_equal(m.row_ptr, ref.row_ptr)
    assert np.array_equal(m.col_idx, ref.col_idx)
    assert np.array_equal(m.values, ref.values)


def test_complex_rectangular_round_trip(mb, tmp_path):
    f = np.load(os.path.join(GOLDEN, "cereal_complex_5x7.npz"))
    m = mb.read_cereal(os.path.join(GOLDEN, "cereal_complex_5x7.bin"))
    assert (m.dim, m.cols, m.nnz) == (5, 7, len(f["rows"]))
    dense = m.to_scipy().toarray()
    ref = np.zeros((5, 7), np.complex128)
    ref[f["rows"], f["cols"]] = f["vals"]
    assert np.array_equal(dense, ref)
    out = tmp_path / "m.bin"
    mb.write_cereal(str(out), m)
    assert out.read_bytes() == open(os.path.join(GOLDEN, "cereal_complex_5x7.bin"), "rb").read()


def raw_archive(path, n_rows, n_cols, entries, version=0):
    with open(path, "wb") as fh:
        fh.write(struct.pack("<IQQQ", version, n_rows, n_cols, len(entries)))
        for r, c, v in entries:
            fh.write(struct.pack("<QQdd", r, c, v.real, v.imag))


def test_load_semantics_last_duplicate_wins_and_zero_drops(mb, tmp_path):
    p = str(tmp_path / "d.bin")
    raw_archive(p, 3, 3, [(0, 0, 1.0), (2, 1, 2.0 + 1j), (0, 0, 5.0), (1, 1, 3.0), (1, 1, 0.0),
                          (2, 2, 0.0)])
    m = mb.read_cereal(p)
    dense = m.to_scipy().toarray()
    ref = np.zeros((3, 3), np.complex128)
    ref[0, 0] = 5.0
    ref[2, 1] = 2.0 + 1j
    assert np.array_equal(dense, ref)
    assert m.nnz == 2


def test_bad_archives_are_rejected(mb, tmp_path):
    p = str(tmp_path / "bad.bin")
    raw_archive(p, 2, 2, [(0, 0, 1.0)], version=1)
    with pytest.raises(mb.MbError):
        mb.read_cereal(p)
    raw_archive(p, 2, 2, [(2, 0, 1.0)])
    with pytest.raises(mb.MbError):
        mb.read_cereal(p)
    raw_archive(p, 2, 2, [(0, 0, 1.0), (1, 1, 1.0)])
    with open(p, "r+b") as fh:
        fh.truncate(os.path.getsize(p) - 8)
    with pytest.raises(mb.MbError):
        mb.read_cereal(p)
    with pytest.raises(mb.MbError):
        mb.read_cereal(str(tmp_path / "missing.bin"))
