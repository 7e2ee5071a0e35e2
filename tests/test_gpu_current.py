"""The current operator J_d(Q) between momentum sectors and the stochastic
current-current correlator (the reference's optical-conductivity driver,
examples/hubbard_momentum_optical_conductivity.cpp:340-410) on the GPU.

Tolerances: J's structure and values bit-exact against the reference's
compute_rectangular_matrix_elements (tests/golden/cur_*.npz); J and J+
applies <= 1e-13 ||y||; the correlator <= 1e-9 against a dense restatement
with exact exponentials and the same probes.
"""
import numpy as np
import pytest

import oracle
from conftest import current_cases, load_golden

pytestmark = pytest.mark.gpu


def sectors(mb, g):
    dims = [int(d) for d in g["dims"]]
    L = int(np.prod(dims))
    k = [int(x) for x in g["momentum"]]
    q = [int(x) for x in g["transfer"]]
    kq = [(a + b) % d for a, b, d in zip(k, q, dims)]
    n, sz = int(g["particles"]), int(g["spin_projection"])
    col = mb.FermionBasis.with_fixed_particle_number_spin_momentum(L, n, sz, dims, k)
    row = mb.FermionBasis.with_fixed_particle_number_spin_momentum(L, n, sz, dims, kq)
    j = mb.CurrentOperator(float(g["t"]), dims, q, int(g["direction"]))
    return row, col, j


@pytest.mark.parametrize("name", current_cases())
def test_current_matrix_elements_match_reference(mb, cuda, name):
    g = load_golden(name)
    row, col, j = sectors(mb, g)
    ru, rd = row.keys()
    cu, cd = col.keys()
    assert np.array_equal(ru, g["row_up"].astype(np.uint64)) and np.array_equal(rd, g["row_down"].astype(np.uint64))
    assert np.array_equal(cu, g["col_up"].astype(np.uint64)) and np.array_equal(cd, g["col_down"].astype(np.uint64))
    m = mb.compute_rectangular_matrix_elements(row, col, j)
    rows = np.repeat(np.arange(m.dim), np.diff(m.row_ptr))
    assert m.nnz == len(g["row"])
    assert np.array_equal(rows, g["row"]) and np.array_equal(m.col_idx, g["col"])
    if any(int(x) for x in g["transfer"]):   # one v(k) per entry: bit-exact
        assert np.array_equal(m.values.real, g["val"])
    else:                                     # Q = 0: merged sums, another order
        assert np.max(np.abs(m.values.real - g["val"])) <= 1e-14 * np.abs(g["val"]).max()
    assert not m.values.imag.any()


@pytest.mark.parametrize("name", current_cases())
def test_current_apply_and_adjoint(mb, cuda, name):
    torch = cuda
    import scipy.sparse as sp
    g = load_golden(name)
    row, col, j = sectors(mb, g)
    J = sp.csr_matrix((g["val"], (g["row"], g["col"])), shape=(row.size(), col.size()))
    op = mb.GpuCurrentOperator(row, col, j)
    rng = np.random.default_rng(5)
    x = rng.normal(size=col.size()) + 1j * rng.normal(size=col.size())
    y = op.apply(torch.tensor(x, device="cuda")).cpu().numpy()
    ref = J @ x
    assert np.linalg.norm(y - ref) <= 1e-13 * max(np.linalg.norm(ref), 1e-300)
    w = rng.normal(size=row.size()) + 1j * rng.normal(size=row.size())
    yt = op.apply(torch.tensor(w, device="cuda"), adjoint=True).cpu().numpy()
    ref_t = J.conj().T @ w
    assert np.linalg.norm(yt - ref_t) <= 1e-13 * max(np.linalg.norm(ref_t), 1e-300)


def test_current_correlator_matches_dense_restatement(mb, cuda):
    from scipy.linalg import expm
    dims, n, beta, dt, steps, samples, seed = [6], 4, 2.0, 0.1, 12, 3, 17
    k, q = [1], [2]
    kq = [(k[0] + q[0]) % 6]
    model = mb.HubbardModelMomentum(1.0, 4.0, dims)
    bk = mb.FermionBasis.with_fixed_particle_number_spin_momentum(6, n, 0, dims, k)
    bkq = mb.FermionBasis.with_fixed_particle_number_spin_momentum(6, n, 0, dims, kq)
    jm = mb.CurrentOperator(1.0, dims, q, 0)
    Hk = mb.compute_matrix_elements(bk, model).to_scipy().toarray()
    Hkq = mb.compute_matrix_elements(bkq, model).to_scipy().toarray()
    J = mb.compute_rectangular_matrix_elements(bkq, bk, jm).to_scipy().toarray()
    c = mb.current_correlator(mb.GpuHubbardOperator(bk, model), mb.GpuHubbardOperator(bkq, model),
                              mb.GpuCurrentOperator(bkq, bk, jm), samples, seed, beta, dt, steps,
                              krylov_steps=30)
    ref = np.zeros(steps, np.complex128)
    Uk, Ukq = expm(-1j * dt * Hk), expm(-1j * dt * Hkq)
    for s in range(samples):
        v = oracle.philox_phase(seed, bk.size(), 1 + s)
        vb = expm(-0.5 * beta * Hk) @ v
        z = np.vdot(vb, vb).real
        p1, p2 = vb, J @ vb
        for i in range(steps):
            ref[i] += np.vdot(p1, J.conj().T @ p2) / z
            p1, p2 = Uk @ p1, Ukq @ p2
    ref /= samples
    assert np.max(np.abs(c - ref)) <= 1e-9 * max(np.abs(ref).max(), 1.0)
