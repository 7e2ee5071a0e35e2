"""All spin projections (with_fixed_particle_number) on the GPU: the
block-diagonal operator (one matrix-free block per (N_up, N_down)) against the
reference's own matrices (tests/golden/all_*.npz).

Tolerances: H structure, signs and values bit-exact; apply <= 1e-13 ||y||
(FP64), <= 2e-6 ||y|| (FP32); E0 <= 1e-10 |E0|.
"""
import numpy as np
import pytest

import oracle
from conftest import all_sz_cases, load_golden

pytestmark = pytest.mark.gpu


def make(mb, g, prec=0):
    dims = [int(d) for d in g["dims"]]
    L = int(np.prod(dims))
    b = mb.FermionBasis.with_fixed_particle_number(L, int(g["particles"]))
    return b, mb._Hubbard(float(g["t"]), float(g["U"]), dims)


def ref_csr(g):
    import scipy.sparse as sp
    n = len(g["up"])
    return sp.csr_matrix((g["val"], (g["row"], g["col"])), shape=(n, n))


@pytest.mark.parametrize("name", all_sz_cases())
def test_all_sz_matrix_elements_bit_exact(mb, cuda, name):
    g = load_golden(name)
    b, model = make(mb, g)
    H = mb.compute_matrix_elements(b, model)
    rows = np.repeat(np.arange(H.dim), np.diff(H.row_ptr))
    assert H.nnz == len(g["row"])
    assert np.array_equal(rows, g["row"]) and np.array_equal(H.col_idx, g["col"])
    assert np.array_equal(H.values.real, g["val"]) and not H.values.imag.any()


@pytest.mark.parametrize("name", all_sz_cases())
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-6)])
def test_all_sz_apply(mb, cuda, name, prec, tol):
    torch = cuda
    g = load_golden(name)
    b, model = make(mb, g)
    op = mb.GpuHubbardOperator(b, model, prec)
    n = op.dimension()
    x = np.random.default_rng(9).normal(size=n) + 1j * np.random.default_rng(10).normal(size=n)
    dt = torch.complex64 if prec else torch.complex128
    y = op.apply(torch.tensor(x, dtype=dt, device="cuda")).cpu().numpy()
    ref = ref_csr(g) @ x
    assert np.linalg.norm(y - ref) <= tol * max(np.linalg.norm(ref), 1e-300)


def test_all_sz_ground_state(mb, cuda):
    """The reference's hubbard_exact_diagonalization example: 1D L=8 with 8
    particles over all spin projections; E0 = the lowest of the fixed-Sz E0s."""
    b = mb.FermionBasis.with_fixed_particle_number(8, 8)
    op = mb.GpuHubbardOperator(b, mb.HubbardModel(1.0, 4.0, 8))
    assert op.dimension() == 12870
    res = mb.find_min_eigenpair(op, 300, reorth=True)
    e_sz = [np.linalg.eigvalsh(oracle.hubbard_csc([8], 1.0, 4.0, nu, 8 - nu).to_dense())[0]
            for nu in range(0, 9)]
    assert abs(res.value - min(e_sz)) <= 1e-10 * abs(min(e_sz))
    # the vector is an eigenvector of the full operator
    hv = op.apply(res.vector)
    lam = op.dot_re(res.vector, hv) / op.dot_re(res.vector, res.vector)
    assert abs(lam - res.value) <= 1e-9 * abs(res.value)


@pytest.mark.parametrize("kind", ["all_sz", "momentum_factorized"])
@pytest.mark.parametrize("pinned", [True, False])
def test_block_diagonal_host_apply_bit_identical(mb, cuda, kind, pinned):
    """Block-diagonal operators (one block per (N_up, N_down), or per total
    momentum) through the host-buffer call equal the device-buffer call bit for
    bit, with page-locked and pageable buffers."""
    torch = cuda
    if kind == "all_sz":
        op = mb.GpuHubbardOperator(mb.FermionBasis.with_fixed_particle_number(8, 8),
                                   mb.HubbardModel(1.0, 4.0, 8))
    else:
        op = mb.HubbardMomentumFactorized(mb.FermionBasis.with_fixed_particle_number_and_spin(8, 8, 0),
                                          [8], 1.0, 4.0)
    x = op.seed_vector(3)
    y = op.apply(x).cpu()
    xh = x.cpu()
    yh = torch.full_like(xh, float("nan"))
    if pinned:
        xh, yh = xh.pin_memory(), yh.pin_memory()
    op.apply_host(xh, yh)
    assert torch.equal(yh, y)
