"""Regenerates the golden Hubbard fixtures in tests/golden/ from the reference.

The real-space sectors (CASES); as mom_*.npz, the momentum-space model on
total-momentum sectors (MOMENTUM_CASES; their npz adds the K vector); as
cur_*.npz, the current operator between two sectors (CURRENT_CASES); as
all_*.npz, all spin projections (ALL_SZ_CASES); as mfull_*.npz, the
momentum-space model on a whole (N_up, N_down) basis (MOMENTUM_FULL_CASES).

Runs oracle/_ref/ref_dump (built by oracle/build_ref.sh from the reference
sources: its basis enumeration, HubbardModel{,2D,3D} and
compute_matrix_elements) for each case below and stores, per case, the
reference-order basis masks, the sparse H as COO (row, col, value) and the
Hamiltonian term count, in one compressed .npz per case.  Values are real for
the real-space Hubbard model; the script checks that every imaginary part is
exactly zero.

Needs the reference sources, so it runs only where they are present; the
fixtures it writes are committed and travel with the tests.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_DUMP = os.path.join(ROOT, "oracle", "_ref", "ref_dump")

# (name, dims, t, U, particles, spin_projection)
CASES = [
    ("chain2_n1_sz1", "2", 1.0, 2.0, 1, 1),
    ("chain2_n2", "2", 1.0, 2.0, 2, 0),
    ("chain4_n4", "4", 1.0, 4.0, 4, 0),
    ("chain4_n4_u0", "4", 1.0, 0.0, 4, 0),
    ("chain5_n5_sz1", "5", 0.7, 3.0, 5, 1),
    ("chain6_n6", "6", 1.0, 4.0, 6, 0),
    ("chain6_n4_sz2", "6", 1.3, 2.5, 4, 2),
    ("chain8_n8", "8", 1.0, 4.0, 8, 0),       # the 1D L=8, 4+4 CPU configuration
    ("chain3_n0", "3", 1.0, 4.0, 0, 0),       # empty occupation: vacuum only
    ("chain4_full", "4", 1.0, 4.0, 8, 0),     # completely filled
    ("chain1_n2", "1", 1.0, 4.0, 2, 0),       # single site: self bond, diagonal cancels to 0
    ("chain1_n2_u3", "1", 1.0, 3.0, 2, 0),    # single site: self bond + U
    ("sq2x2_n2", "2x2", 1.0, 2.0, 2, 0),
    ("sq2x2_n4", "2x2", 1.0, 2.0, 4, 0),
    ("sq3x3_n4", "3x3", 1.0, 8.0, 4, 0),
    ("sq3x3_n5_sz1", "3x3", 1.0, 8.0, 5, 1),
    ("rect2x4_n4", "2x4", 1.0, 3.0, 4, 0),
    ("rect2x3_n4", "2x3", 0.5, 6.0, 4, 0),
    ("rect3x4_n4", "3x4", 1.0, 5.0, 4, 0),
    ("cube2x2x2_n4", "2x2x2", 1.0, 2.0, 4, 0),
]

TERM_COUNT_CASES = [("1", 2), ("2x2", 2), ("2x2x2", 3)]

# Momentum-space model on one total-momentum sector (ref_dump --momentum):
# (name, dims, t, U, particles, spin_projection, K)
MOMENTUM_CASES = [
    ("mom_chain4_n2_k0", "4", 1.0, 2.0, 2, 0, "0"),
    ("mom_chain4_n4_k1", "4", 1.0, 4.0, 4, 0, "1"),
    ("mom_chain4_n4_u0_k2", "4", 1.0, 0.0, 4, 0, "2"),    # U = 0: diagonal only
    ("mom_chain6_n4_k2", "6", 1.0, 4.0, 4, 0, "2"),
    ("mom_chain6_n4_t0_k0", "6", 0.0, 4.0, 4, 0, "0"),    # t = 0: no kinetic terms
    ("mom_chain6_n3_sz1_k3", "6", 0.7, 3.0, 3, 1, "3"),
    ("mom_chain8_n4_k0", "8", 1.0, 4.0, 4, 0, "0"),
    ("mom_sq2x2_n4_k10", "2x2", 1.0, 2.0, 4, 0, "1x0"),
    ("mom_sq3x3_n4_k11", "3x3", 1.0, 8.0, 4, 0, "1x1"),
    ("mom_rect2x3_n4_k01", "2x3", 0.5, 6.0, 4, 0, "0x1"),
    ("mom_cube2x2x2_n4_k101", "2x2x2", 1.0, 2.0, 4, 0, "1x0x1"),
]

# Momentum-space model on the whole (N_up, N_down) basis, every total momentum
# (ref_dump --momentum-full): the matrix HubbardMomentumFactorized applies.
# (name, dims, t, U, particles, spin_projection)
MOMENTUM_FULL_CASES = [
    ("mfull_chain2_n2_t0", "2", 0.0, 3.0, 2, 0),      # interaction only
    ("mfull_chain4_n2", "4", 1.0, 4.0, 2, 0),
    ("mfull_chain6_n4_u0", "6", 1.5, 0.0, 4, 0),      # kinetic only
    ("mfull_chain6_n3_sz1", "6", 1.0, -2.0, 3, 1),    # attractive U, 2 up + 1 down
    ("mfull_sq2x2_n3_sz1", "2x2", 1.0, 2.0, 3, 1),
    ("mfull_rect2x3_n4", "2x3", 1.0, 4.0, 4, 0),
    ("mfull_sq3x3_n3_sz1", "3x3", 1.0, 8.0, 3, 1),
]

# All spin projections, real-space model (ref_dump --all): (name, dims, t, U, particles)
ALL_SZ_CASES = [
    ("all_chain1_n1", "1", 1.0, 3.0, 1),
    ("all_chain4_n2", "4", 1.0, 4.0, 2),
    ("all_chain4_n4", "4", 1.0, 4.0, 4),
    ("all_chain5_n5", "5", 0.7, 3.0, 5),
    ("all_chain6_n3", "6", 1.0, 2.0, 3),
    ("all_sq2x2_n3", "2x2", 1.0, 2.0, 3),
    ("all_rect2x3_n4", "2x3", 1.0, 6.0, 4),
]

# Current operator J_d(Q) from sector K to K+Q (ref_dump --current):
# (name, dims, t, particles, spin_projection, K, Q, direction)
CURRENT_CASES = [
    ("cur_chain4_n2_k0_q1", "4", 1.0, 2, 0, "0", "1", 0),
    ("cur_chain6_n4_k2_q1", "6", 1.0, 4, 0, "2", "1", 0),
    ("cur_chain6_n4_k2_q0", "6", 1.0, 4, 0, "2", "0", 0),
    ("cur_chain6_n3_sz1_k1_q3", "6", 0.7, 3, 1, "1", "3", 0),
    ("cur_chain8_n4_k0_q2", "8", 1.0, 4, 0, "0", "2", 0),
    ("cur_sq3x3_n4_k11_q10_d0", "3x3", 1.0, 4, 0, "1x1", "1x0", 0),
    ("cur_sq3x3_n4_k11_q10_d1", "3x3", 1.0, 4, 0, "1x1", "1x0", 1),
    ("cur_rect2x4_n4_k00_q01_d1", "2x4", 1.0, 4, 0, "0x0", "0x1", 1),
]


def dump_current(dims, t, n, sz, k, q, d):
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        path = f.name
    try:
        subprocess.run([REF_DUMP, "--current", dims, repr(t), str(n), str(sz), k, q, str(d), path],
                       check=True)
        b = open(path, "rb").read()
    finally:
        os.unlink(path)
    assert b[:8] == b"MBREF002"
    n_terms, nr, nc = (int(v) for v in np.frombuffer(b[8:32], "<u8"))
    o = 32
    parts = []
    for n_ in (nr, nr, nc, nc):
        parts.append(np.frombuffer(b[o:o + 8 * n_], "<u8").copy())
        o += 8 * n_
    nnz = int(np.frombuffer(b[o:o + 8], "<u8")[0])
    rec = np.frombuffer(b[o + 8:], np.dtype([("r", "<i8"), ("c", "<i8"), ("re", "<f8"),
                                             ("im", "<f8")]))
    assert len(rec) == nnz
    assert np.all(rec["im"] == 0.0)
    return n_terms, parts, rec


def dump(dims, t, U, n, sz, momentum=None, all_sz=False, momentum_full=False):
    with tempfile.NamedTemporaryFile(suffix=".bin", delete=False) as f:
        path = f.name
    try:
        args = [dims, repr(t), repr(U), str(n), str(sz)]
        if momentum is not None:
            args = ["--momentum", *args, momentum]
        if momentum_full:
            args = ["--momentum-full", *args]
        if all_sz:
            args = ["--all", dims, repr(t), repr(U), str(n)]
        subprocess.run([REF_DUMP, *args, path], check=True)
        b = open(path, "rb").read()
    finally:
        os.unlink(path)
    assert b[:8] == b"MBREF001"
    n_terms, dim = (int(v) for v in np.frombuffer(b[8:24], "<u8"))
    up = np.frombuffer(b[24:24 + 8 * dim], "<u8").copy()
    dn = np.frombuffer(b[24 + 8 * dim:24 + 16 * dim], "<u8").copy()
    o = 24 + 16 * dim
    nnz = int(np.frombuffer(b[o:o + 8], "<u8")[0])
    rec = np.frombuffer(b[o + 8:], np.dtype([("r", "<i8"), ("c", "<i8"), ("re", "<f8"),
                                             ("im", "<f8")]))
    assert len(rec) == nnz
    assert np.all(rec["im"] == 0.0)
    return n_terms, up, dn, rec


def main():
    if not os.path.exists(REF_DUMP):
        sys.exit("build oracle/_ref/ref_dump first: oracle/build_ref.sh")
    for name, dims, t, U, n, sz in CASES:
        n_terms, up, dn, rec = dump(dims, t, U, n, sz)
        dvec = [int(x) for x in dims.split("x")]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), dims=np.array(dvec, np.int32),
                            t=t, U=U, particles=n, spin_projection=sz, n_terms=n_terms,
                            up=up, down=dn, row=rec["r"].astype(np.int32),
                            col=rec["c"].astype(np.int32), val=rec["re"].copy())
        print(f"{name}: dim={len(up)} nnz={len(rec)} terms={n_terms}")
    for name, dims, t, U, n, sz, k in MOMENTUM_CASES:
        n_terms, up, dn, rec = dump(dims, t, U, n, sz, k)
        dvec = [int(x) for x in dims.split("x")]
        kvec = [int(x) for x in k.split("x")]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), dims=np.array(dvec, np.int32),
                            t=t, U=U, particles=n, spin_projection=sz,
                            momentum=np.array(kvec, np.int32), n_terms=n_terms, up=up, down=dn,
                            row=rec["r"].astype(np.int32), col=rec["c"].astype(np.int32),
                            val=rec["re"].copy())
        print(f"{name}: dim={len(up)} nnz={len(rec)} terms={n_terms}")
    for name, dims, t, U, n, sz in MOMENTUM_FULL_CASES:
        n_terms, up, dn, rec = dump(dims, t, U, n, sz, momentum_full=True)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                            dims=np.array([int(x) for x in dims.split("x")], np.int32), t=t, U=U,
                            particles=n, spin_projection=sz, n_terms=n_terms, up=up, down=dn,
                            row=rec["r"].astype(np.int32), col=rec["c"].astype(np.int32),
                            val=rec["re"].copy())
        print(f"{name}: dim={len(up)} nnz={len(rec)} terms={n_terms}")
    for name, dims, t, U, n in ALL_SZ_CASES:
        n_terms, up, dn, rec = dump(dims, t, U, n, 0, all_sz=True)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                            dims=np.array([int(x) for x in dims.split("x")], np.int32), t=t, U=U,
                            particles=n, n_terms=n_terms, up=up, down=dn,
                            row=rec["r"].astype(np.int32), col=rec["c"].astype(np.int32),
                            val=rec["re"].copy())
        print(f"{name}: dim={len(up)} nnz={len(rec)} terms={n_terms}")
    for name, dims, t, n, sz, k, q, d in CURRENT_CASES:
        n_terms, (ru, rd, cu, cd), rec = dump_current(dims, t, n, sz, k, q, d)
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"),
                            dims=np.array([int(x) for x in dims.split("x")], np.int32), t=t,
                            particles=n, spin_projection=sz,
                            momentum=np.array([int(x) for x in k.split("x")], np.int32),
                            transfer=np.array([int(x) for x in q.split("x")], np.int32),
                            direction=d, n_terms=n_terms, row_up=ru, row_down=rd, col_up=cu,
                            col_down=cd, row=rec["r"].astype(np.int32),
                            col=rec["c"].astype(np.int32), val=rec["re"].copy())
        print(f"{name}: {len(ru)}x{len(cu)} nnz={len(rec)} terms={n_terms}")


if __name__ == "__main__":
    main()
