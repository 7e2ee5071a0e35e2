"""The CPU oracle against the reference's own outputs (golden fixtures) and
against the reference's numerics test expectations."""
import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_golden


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_basis_and_matrix_bit_exact(name):
    g = load_golden(name)
    up, dn = oracle.basis(g["L"], g["n_up"], g["n_down"])
    assert np.array_equal(up, g["up"]) and np.array_equal(dn, g["down"])
    H = oracle.hubbard_csc(list(g["dims"]), float(g["t"]), float(g["U"]), g["n_up"], g["n_down"])
    cols = np.repeat(np.arange(H.dim), np.diff(H.col_ptr))
    order = np.lexsort((cols, H.row_idx))
    assert np.array_equal(H.row_idx[order], g["row"])
    assert np.array_equal(cols[order], g["col"])
    assert np.array_equal(H.re[order], g["val"])          # bit-exact values
    assert not H.im.any()
    assert oracle.term_count(list(g["dims"]), float(g["t"]), float(g["U"])) == int(g["n_terms"])


def test_term_counts_match_reference_tests():
    # tests/algebra/test_model.cpp:58-74
    assert oracle.term_count([2], 1.0, 2.0) == 6
    assert oracle.term_count([2, 2], 1.0, 2.0) == 20
    assert oracle.term_count([2, 2, 2], 1.0, 2.0) == 56


def test_basis_sizes_match_reference_tests():
    # tests/algebra/test_basis.cpp:22-41: (orbitals 2, particles 2, Sz 0) has 4 states
    up, dn = oracle.basis(2, 1, 1)
    assert len(up) == 4
    assert {(int(u), int(d)) for u, d in zip(up, dn)} == {(1, 1), (1, 2), (2, 1), (2, 2)}
    up, dn = oracle.basis(1, 1, 0)
    assert len(up) == 1


def test_jackson_and_lorentz_kernels():
    # tests/numerics/test_kpm.cpp:11-58: g_0 = 1, decreasing, positive.
    g = oracle.jackson_kernel(64)
    assert abs(g[0] - 1.0) < 1e-12
    assert np.all(np.diff(g) <= 1e-15) and np.all(g > -1e-12)
    l = oracle.lorentz_kernel(64, 4.0)
    assert abs(l[0] - 1.0) < 1e-12 and abs(l[-1]) < 1e-12


def test_projector_moments_sum_rule():
    # mu_0 = 1 - acos(eps)/pi  (kpm.h:51-61)
    mu = oracle.projector_moments(16, 0.3)
    assert abs(mu[0] - (1 - np.arccos(0.3) / np.pi)) < 1e-15


def test_tridiag_eig_matches_numpy():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 40, 200):
        a = rng.normal(size=n)
        b = rng.normal(size=n - 1)
        d, z = oracle.tridiag_eig(a, b)
        T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
        assert np.allclose(d, np.linalg.eigvalsh(T), atol=1e-12 * max(1, np.abs(d).max()))
        assert np.allclose(T @ z, z * d, atol=1e-10)


def test_lanczos_ground_state_chain8():
    # 1D L=8, 4+4, t=1, U=4: oracle Lanczos vs dense eigvalsh of the reference H.
    H = oracle.hubbard_csc([8], 1.0, 4.0, 4, 4)
    E = np.linalg.eigvalsh(H.to_dense())
    seed = oracle.philox_uniform(0, H.dim)
    e0, vec, m, _, _ = H.find_min_eigenpair(seed, 200, reorth=True)
    assert abs(e0 - E[0]) < 1e-10 * abs(E[0])
    hv = H.apply(vec)
    lam = np.vdot(vec, hv).real / np.vdot(vec, vec).real
    assert abs(lam - E[0]) < 1e-9


def test_evolution_matches_dense_expm():
    # test_evolve_state.cpp pattern: Krylov evolution vs exact exp(-iHt).
    import scipy.linalg as sla
    H = oracle.hubbard_csc([4], 1.0, 4.0, 2, 2)
    Hd = H.to_dense()
    psi = oracle.philox_uniform(5, H.dim)
    out = H.time_evolve(psi, 0.3, krylov_steps=30)
    ref = sla.expm(-1j * 0.3 * Hd) @ psi
    assert np.linalg.norm(out - ref) < 1e-8 * np.linalg.norm(ref)
    out_i = H.time_evolve(psi, 0.2, krylov_steps=30, imaginary=True)
    ref_i = sla.expm(-0.2 * Hd) @ psi
    assert np.linalg.norm(out_i - ref_i) < 1e-8 * np.linalg.norm(ref_i)


def test_kpm_dos_moments_match_dense_chebyshev():
    H = oracle.hubbard_csc([4], 1.0, 2.0, 2, 2)
    Hd = H.to_dense()
    E = np.linalg.eigvalsh(Hd)
    a = (E[-1] - E[0]) / 2 * 1.01
    b = (E[-1] + E[0]) / 2
    r = oracle.philox_phase(1, H.dim, 1)
    mu = H.kpm_dos_moments(r, 12, a, b)
    Ht = (Hd - b * np.eye(H.dim)) / a
    T0, T1 = r.copy(), Ht @ r
    ref = [np.vdot(r, T0).real, np.vdot(r, T1).real]
    for _ in range(10):
        T0, T1 = T1, 2 * Ht @ T1 - T0
        ref.append(np.vdot(r, T1).real)
    assert np.allclose(mu, ref, atol=1e-10 * H.dim)


def test_parallel_hermitian_apply_matches_serial_scatter():
    """The multi-core CPU figure's row gather equals the reference-style serial
    column scatter on a Hubbard sector and on a random complex Hermitian matrix."""
    import scipy.sparse as sp
    rng = np.random.default_rng(5)
    H = oracle.hubbard_csc([3, 3], 1.0, 8.0, 3, 3)
    x = rng.uniform(-1, 1, H.dim) + 1j * rng.uniform(-1, 1, H.dim)
    np.testing.assert_allclose(H.apply_parallel(x), H.apply(x), rtol=0, atol=1e-12)
    n = 500
    A = sp.random(n, n, density=0.02, random_state=7, dtype=np.complex128)
    A = (A + A.conj().T).tocsc()
    A.sort_indices()
    M = oracle.CscMatrix(n, A.indptr.astype(np.int64), A.indices.astype(np.int64),
                         np.ascontiguousarray(A.data.real), np.ascontiguousarray(A.data.imag))
    v = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    np.testing.assert_allclose(M.apply_parallel(v), A @ v, rtol=0, atol=1e-12)
    np.testing.assert_allclose(M.apply(v), A @ v, rtol=0, atol=1e-12)
