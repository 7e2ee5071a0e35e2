"""The oracle's restatements of the reference's Lanczos, Krylov-evolution and
KPM code, pinned against the reference's own code: numerics/lanczos.h,
numerics/evolve_state.h and numerics/kpm.h, unchanged, run on the CPU on the
reference's SparseComplexMatrixOperator (and SparseKPMProjector), with a minimal Armadillo stand-in for the library
the reference links (oracle/ref_numerics_pin.cpp, built into oracle/_ref/ by
oracle/build_ref.sh where the reference sources are present).  Same matrix, same start vectors:
find_min_eigenpair (its seed handed to make_seed_vector), pass one's alpha and
beta, exp(-i t H) psi, exp(-t H) psi, the Jackson and Lorentz kernels, the
projector moments and the sparse KPM projector applied to psi.  Skipped where
the reference sources are absent.

Tolerances: E0 1e-10 relative; the first 20 alpha, beta 1e-12 absolute, up to
an invariant subspace's end (beta below 1e-8: the rest is rounding noise), since
later steps amplify rounding differences once Ritz values converge (measured:
alpha agrees to 1e-12 for the first 33 to 70 steps); the Ritz vectors' overlap
>= 1 - 1e-3 (after convergence the two recurrences part at the rounding level,
and a degenerate ground state's vector follows them); the evolved states 1e-10
relative (measured: 1e-14); the kernels and moments 1e-14; the projector
1e-12 relative.
"""
import os
import struct
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT

PIN = os.path.join(ROOT, "oracle", "_ref", "ref_numerics_pin")

# (dims, t, U, N_up, N_down, Lanczos steps, evolution time)
CASES = [
    ([8], 1.0, 4.0, 4, 4, 200, 0.25),
    ([2, 3], 1.0, 3.0, 2, 2, 60, 0.5),
    ([3, 3], 1.0, 8.0, 3, 2, 200, 0.3),
    ([6], 1.0, 0.0, 3, 3, 100, 0.7),
    ([2, 2], 1.0, -2.0, 2, 1, 16, 1.0),
]


@pytest.fixture(scope="module")
def pin_binary():
    if not os.path.exists(PIN):
        pytest.skip("oracle/_ref/ref_numerics_pin is built only where the reference sources are")
    return PIN


def run_reference(binary, tmp_path, H, k, t, seed, psi, M, kb):
    n = H.dim
    vals = (H.re + 1j * H.im).astype(np.complex128)
    blob = struct.pack("<qqqdq4d", n, H.nnz, k, t, M, *kb)
    blob += np.asarray(H.col_ptr, np.int64).tobytes() + np.asarray(H.row_idx, np.int64).tobytes()
    blob += vals.tobytes() + seed.astype(np.complex128).tobytes() + psi.astype(np.complex128).tobytes()
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    fin.write_bytes(blob)
    r = subprocess.run([binary, str(fin), str(fout)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = fout.read_bytes()
    m = struct.unpack_from("<q", raw, 0)[0]
    off = 8
    e0 = struct.unpack_from("<d", raw, off)[0]
    off += 8
    al = np.frombuffer(raw, np.float64, m, off)
    off += 8 * m
    be = np.frombuffer(raw, np.float64, max(m - 1, 0), off)
    off += 8 * max(m - 1, 0)
    vec, real_t, imag_t = (np.frombuffer(raw, np.complex128, n, off + 16 * n * i) for i in range(3))
    off += 48 * n
    jk, lk, pm = (np.frombuffer(raw, np.float64, M + 1, off + 8 * (M + 1) * i) for i in range(3))
    off += 24 * (M + 1)
    proj = np.frombuffer(raw, np.complex128, n, off)
    return m, e0, al, be, vec, real_t, imag_t, (jk, lk, pm, proj)


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference_drivers(pin_binary, tmp_path, case):
    dims, t, u, nu, nd, k, tev = case
    H = oracle.hubbard_csc(dims, t, u, nu, nd)
    n = H.dim
    k = min(k, n)
    rng = np.random.default_rng(5)
    seed = rng.uniform(0, 1, n) + 1j * rng.uniform(0, 1, n)  # randu, as make_seed_vector draws
    psi = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    psi /= np.linalg.norm(psi)
    E = np.linalg.eigvalsh(H.to_dense())
    assert not np.any(H.im)  # the Hubbard H is real: the sparse projector's vectors are real
    M = 48
    kb = (float(E[0]), float(E[-1]), float((E[0] + E[-1]) / 2 - 0.1 * (E[-1] - E[0])), 0.01)
    m, e0, al, be, vec, real_t, imag_t, kpm_out = run_reference(pin_binary, tmp_path, H, k, tev,
                                                                seed, psi, M, kb)

    e_or, vec_or, m_or, al_or, be_or = H.find_min_eigenpair(seed, k)
    assert m == m_or
    assert abs(e0 - e_or) <= 1e-10 * max(abs(e_or), 1.0)
    small = np.nonzero(be_or < 1e-8)[0]
    q = min(20, m, int(small[0]) + 1 if len(small) else m)
    assert q >= 10
    assert np.allclose(al[:q], al_or[:q], rtol=0, atol=1e-12)
    assert np.allclose(be[:q - 1], be_or[:q - 1], rtol=0, atol=1e-12)
    ov = abs(np.vdot(vec, vec_or)) / (np.linalg.norm(vec) * np.linalg.norm(vec_or))
    assert ov >= 1 - 1e-3
    for imaginary, got in ((False, real_t), (True, imag_t)):
        ref = H.time_evolve(psi, tev, 30, imaginary)
        assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref), imaginary
    # and both are right: E0 against a dense solve
    assert abs(e0 - E[0]) <= 1e-8 * max(abs(E[0]), 1.0)
    # KPM (kpm.h:19-61, 184-229)
    jk, lk, pm, proj = kpm_out
    a = (kb[1] - kb[0]) / 2 * (1 + kb[3])
    eps = (kb[2] - (kb[1] + kb[0]) / 2) / a
    assert np.allclose(jk, oracle.jackson_kernel(M), rtol=0, atol=1e-14)
    assert np.allclose(lk, oracle.lorentz_kernel(M, 4.0), rtol=0, atol=1e-14)
    assert np.allclose(pm, oracle.projector_moments(M, eps), rtol=0, atol=1e-14)
    ref_p = H.kpm_projector_apply(psi, M, kb[0], kb[1], kb[2], kb[3])
    assert np.linalg.norm(proj - ref_p) <= 1e-12 * np.linalg.norm(ref_p)
