"""Regenerates the sparse-matrix cache-format fixtures in tests/golden/.

oracle/_ref/cereal_pin (oracle/cereal_pin.cpp, built by oracle/build_ref.sh
against the cereal library the reference vendors) writes a matrix as a cereal
binary archive with the field sequence of the reference's arma::SpMat save
(src/utils/arma_cereal.h:9-17).  Two fixtures:

  cereal_chain4_n4.bin      the reference's H for 1D L=4, 2+2, U=4 (from the
                            golden COO in chain4_n4.npz), column-major order;
  cereal_complex_5x7.bin    a rectangular complex matrix (entries in
                            cereal_complex_5x7.npz), for the value layout.

    python tests/golden/make_cereal_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
PIN = os.path.join(ROOT, "oracle", "_ref", "cereal_pin")


def write(path, n_rows, n_cols, rows, cols, vals):
    text = f"{n_rows} {n_cols} {len(rows)}\n" + "".join(
        f"{int(r)} {int(c)} {float(v.real)!r} {float(v.imag)!r}\n" for r, c, v in zip(rows, cols, vals))
    subprocess.run([PIN, path], input=text.encode(), check=True)


def column_major(rows, cols, vals):
    order = np.lexsort((rows, cols))
    return rows[order], cols[order], vals[order]


def main():
    if not os.path.exists(PIN):
        sys.exit("build oracle/_ref/cereal_pin first: oracle/build_ref.sh")
    g = np.load(os.path.join(HERE, "chain4_n4.npz"))
    n = len(g["up"])
    r, c, v = column_major(g["row"].astype(np.int64), g["col"].astype(np.int64),
                           g["val"].astype(np.complex128))
    write(os.path.join(HERE, "cereal_chain4_n4.bin"), n, n, r, c, v)
    rows = np.array([0, 3, 4, 1, 0, 2, 4], np.int64)
    cols = np.array([0, 0, 2, 3, 5, 6, 6], np.int64)
    vals = np.array([1.5, -2.25 + 0.5j, 1e-300, -0.0 + 3j, 7.0 - 7.0j, 0.125, -1e300j],
                    np.complex128)
    write(os.path.join(HERE, "cereal_complex_5x7.bin"), 5, 7, rows, cols, vals)
    np.savez_compressed(os.path.join(HERE, "cereal_complex_5x7.npz"), rows=rows, cols=cols,
                        vals=vals)
    print("wrote cereal_chain4_n4.bin, cereal_complex_5x7.bin")


if __name__ == "__main__":
    main()
