"""Sparse-matrix operators (SparseComplexMatrixOperator,
src/numerics/linear_operator.h:81-91, on the GPU): any square complex CSR,
e.g. a Hamiltonian read from the reference's cache format, through the same
drivers as the lattice operators.

Tolerances: apply <= 1e-13 ||y|| (FP64), <= 2e-6 ||y|| (FP32); E0 <= 1e-10
|E0|; evolution <= 1e-10 relative; DOS moments <= 1e-10 absolute.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import load_golden

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def csr_of(mb, a):
    import scipy.sparse as sp
    m = sp.csr_matrix(a)
    m.sort_indices()
    return mb.CsrMatrix(m.shape[0], m.indptr.astype(np.int64), m.indices.astype(np.int64),
                        m.data.astype(np.complex128))


def random_hermitian(n, density, seed):
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    a = sp.random(n, n, density=density, random_state=rng, dtype=np.complex128,
                  data_rvs=lambda k: rng.normal(size=k) + 1j * rng.normal(size=k))
    assert np.abs(a.data.imag).max() > 0
    return (a + a.conj().T).tocsr() + sp.diags(rng.normal(size=n))


@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-6)])
def test_sparse_apply_matches_scipy(mb, cuda, prec, tol):
    torch = cuda
    a = random_hermitian(3000, 0.004, 1)
    op = mb.GpuSparseOperator(csr_of(mb, a), prec)
    x = np.random.default_rng(2).normal(size=3000) + 1j * np.random.default_rng(3).normal(size=3000)
    dt = torch.complex64 if prec else torch.complex128
    y = op.apply(torch.tensor(x, dtype=dt, device="cuda")).cpu().numpy()
    ref = a @ x
    assert np.linalg.norm(y - ref) <= tol * np.linalg.norm(ref)
    # affine form and order independence (the matrix's own order)
    z = np.random.default_rng(4).normal(size=3000) + 0j
    ya = op.apply_affine(torch.tensor(x, dtype=dt, device="cuda"), scale=0.5, shift=1.25, beta=-2.0,
                         z=torch.tensor(z, dtype=dt, device="cuda"), order=mb.ORDER_TENSOR)
    ref_a = 0.5 * (ref - 1.25 * x) - 2.0 * z
    assert np.linalg.norm(ya.cpu().numpy() - ref_a) <= tol * np.linalg.norm(ref_a)


def test_cached_hamiltonian_ground_state(mb, cuda):
    """H from the cache-format fixture (written by the vendored cereal):
    Lanczos on the GPU meets the dense spectrum."""
    m = mb.read_cereal(os.path.join(GOLDEN, "cereal_chain4_n4.bin"))
    E = np.linalg.eigvalsh(m.to_scipy().toarray())
    op = mb.GpuSparseOperator(m)
    res = mb.find_min_eigenpair(op, m.dim, reorth=True)
    assert abs(res.value - E[0]) <= 1e-10 * abs(E[0])
    res = mb.find_max_eigenpair(op, m.dim, reorth=True)
    assert abs(res.value - E[-1]) <= 1e-10 * abs(E[-1])


def test_lattice_hamiltonian_through_the_cache(mb, cuda, tmp_path):
    """compute_matrix_elements -> cache file -> sparse operator: the same
    operator as the matrix-free one, in reference order."""
    torch = cuda
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(9, 5, 1)
    model = mb.HubbardModel2D(1.0, 8.0, 3, 3)
    path = str(tmp_path / "h.bin")
    mb.write_cereal(path, mb.compute_matrix_elements(basis, model))
    sop = mb.GpuSparseOperator(mb.read_cereal(path))
    lop = mb.GpuHubbardOperator(basis, model)
    x = lop.seed_vector(5)
    ys = sop.apply(x)
    yl = lop.apply(x)
    assert float(torch.linalg.norm(ys - yl)) <= 1e-13 * float(torch.linalg.norm(yl))


def test_complex_sparse_evolution_and_dos(mb, cuda):
    torch = cuda
    a = random_hermitian(400, 0.02, 7)
    dense = a.toarray()
    E, V = np.linalg.eigh(dense)
    op = mb.GpuSparseOperator(csr_of(mb, a))
    psi = op.seed_vector(3)
    out = mb.time_evolve_state(op, psi, 0.3, krylov_steps=40).cpu().numpy()
    p = psi.cpu().numpy()
    ref = V @ (np.exp(-1j * 0.3 * E) * (V.conj().T @ p))
    assert np.linalg.norm(out - ref) <= 1e-10 * np.linalg.norm(ref)
    M, R = 32, 2
    mu = mb.kpm_dos_moments(op, M, R, 9, E[0], E[-1], 0.01)
    a_ = (E[-1] - E[0]) / 2 * 1.01
    b_ = (E[-1] + E[0]) / 2
    ref_mu = np.zeros(M)
    Ht = (dense - b_ * np.eye(400)) / a_
    for q in range(R):
        r = oracle.philox_phase(9, 400, 1 + q)
        t0, t1 = r, Ht @ r
        ts = [t0, t1]
        for _ in range(2, M):
            ts.append(2 * Ht @ ts[-1] - ts[-2])
        ref_mu += np.array([np.vdot(r, t).real for t in ts])
    ref_mu /= R * 400
    assert np.max(np.abs(mu - ref_mu)) <= 1e-10


def test_sparse_operator_argument_checks(mb, cuda):
    with pytest.raises(mb.MbError):
        mb.GpuSparseOperator(csr_of(mb, random_hermitian(10, 0.3, 1)), mb.PREC_Q64)
    bad = csr_of(mb, random_hermitian(10, 0.3, 1))
    bad.col_idx = bad.col_idx.copy()
    bad.col_idx[0] = 10
    with pytest.raises(mb.MbError):
        mb.GpuSparseOperator(bad)
    op = mb.GpuSparseOperator(csr_of(mb, random_hermitian(10, 0.3, 1)))
    x = op.seed_vector(0)
    with pytest.raises(mb.MbError):
        op.apply_noalloc(x)
