"""Momentum-space Hubbard sectors on the GPU: the sector's H built on the
device (compute_matrix_elements of HubbardModelMomentum on
with_fixed_particle_number_spin_momentum) against the reference's own
matrices (tests/golden/mom_*.npz), and the sector operators through the
Krylov drivers.

Tolerances: structure and off-diagonal values (+-U/N) bit-exact; diagonal
values <= 1e-14 |H|max (the reference sums the same terms in its own order);
apply <= 1e-13 ||y|| (FP64 and the block-floating-point Q64), <= 2e-6 ||y||
(FP32); E0 <= 1e-10 |E0| (Q64 against FP64: 1e-12); DOS moments Q64 against
FP64 <= 1e-10.
"""
import numpy as np
import pytest

import oracle
from conftest import load_golden, momentum_cases, momentum_full_cases

pytestmark = pytest.mark.gpu


def make(mb, g, prec=0):
    dims = [int(d) for d in g["dims"]]
    basis = mb.FermionBasis.with_fixed_particle_number_spin_momentum(
        int(np.prod(dims)), int(g["particles"]), int(g["spin_projection"]), dims,
        [int(k) for k in g["momentum"]])
    model = mb.HubbardModelMomentum(float(g["t"]), float(g["U"]), dims)
    return basis, model


def ref_csr(g):
    import scipy.sparse as sp
    n = len(g["up"])
    return sp.csr_matrix((g["val"], (g["row"], g["col"])), shape=(n, n))


@pytest.mark.parametrize("name", momentum_cases())
def test_momentum_matrix_elements_match_reference(mb, cuda, name):
    g = load_golden(name)
    basis, model = make(mb, g)
    H = mb.compute_matrix_elements(basis, model)
    rows = np.repeat(np.arange(H.dim), np.diff(H.row_ptr))
    assert H.nnz == len(g["row"])
    assert np.array_equal(rows, g["row"]) and np.array_equal(H.col_idx, g["col"])
    off = rows != H.col_idx
    assert np.array_equal(H.values.real[off], g["val"][off])
    scale = max(np.abs(g["val"]).max(), 1.0)
    assert np.max(np.abs(H.values.real[~off] - g["val"][~off]), initial=0.0) <= 1e-14 * scale
    assert not H.values.imag.any()


@pytest.mark.parametrize("name", momentum_cases())
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-6), (2, 1e-13)])
def test_momentum_operator_apply(mb, cuda, name, prec, tol):
    torch = cuda
    g = load_golden(name)
    basis, model = make(mb, g)
    op = mb.GpuHubbardOperator(basis, model, prec)
    n = op.dimension()
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    dt = torch.complex64 if prec == 1 else torch.complex128
    y = op.apply(torch.tensor(x, dtype=dt, device="cuda")).cpu().numpy()
    ref = ref_csr(g) @ x
    assert np.linalg.norm(y - ref) <= tol * max(np.linalg.norm(ref), 1e-300)


def test_momentum_sectors_reproduce_the_real_space_spectrum(mb, cuda):
    """1D L=6, 2+2: the union over K of the sector spectra is the spectrum
    of the real-space Hamiltonian (the Fourier transform is unitary)."""
    dims, n = [6], 4
    E_real = np.linalg.eigvalsh(oracle.hubbard_csc(dims, 1.0, 3.0, 2, 2).to_dense())
    model = mb.HubbardModelMomentum(1.0, 3.0, dims)
    parts = []
    for k in range(6):
        b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(6, n, 0, dims, [k])
        parts.append(np.linalg.eigvalsh(mb.compute_matrix_elements(b, model).to_scipy().toarray()))
    E_mom = np.sort(np.concatenate(parts))
    assert len(E_mom) == len(E_real)
    assert np.max(np.abs(E_mom - E_real)) <= 1e-10 * np.abs(E_real).max()


def test_momentum_ground_state_matches_real_space(mb, cuda):
    """3x3, 3+3 (dim 7056 real space): the lowest sector ground state over
    all nine momenta equals the real-space ground state (Lanczos on both)."""
    dims = [3, 3]
    real = mb.GpuHubbardOperator(mb.FermionBasis.with_fixed_particle_number_and_spin(9, 6, 0),
                                 mb.HubbardModel2D(1.0, 4.0, 3, 3))
    e_real = mb.find_min_eigenpair(real, 200, reorth=True, want_vector=False).value
    model = mb.HubbardModelMomentum(1.0, 4.0, dims)
    best = None
    for kx in range(3):
        for ky in range(3):
            b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(9, 6, 0, dims, (kx, ky))
            op = mb.GpuHubbardOperator(b, model)
            e = mb.find_min_eigenpair(op, min(200, op.dimension()), reorth=True,
                                      want_vector=False).value
            best = e if best is None else min(best, e)
    assert abs(best - e_real) <= 1e-10 * abs(e_real)


def test_q64_momentum_sector_matches_fp64(mb, cuda):
    """4x4, N_up = N_down = 4, K = (0, 0) (207,184 states): the block-floating-
    point sector operator (exact integer sums of the +-U/N entries, the
    diagonal as a per-row fixed-point coefficient) gives the FP64 operator's
    apply, ground state and DOS moments."""
    torch = cuda
    dims = [4, 4]
    b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(16, 8, 0, dims, (0, 0))
    model = mb.HubbardModelMomentum(1.0, 8.0, dims)
    f64 = mb.GpuHubbardOperator(b, model, mb.PREC_F64)
    q64 = mb.GpuHubbardOperator(b, model, mb.PREC_Q64)
    x = f64.seed_vector(5)
    y64, yq = f64.apply(x), q64.apply(x)
    assert float(torch.linalg.norm(yq - y64)) <= 1e-13 * float(torch.linalg.norm(y64))
    # affine form: 0.5 (H - 1.5) x + 0.25 z through both
    z = f64.seed_vector(6)
    a64 = f64.apply_affine(x, 0.5, 1.5, 0.25, z)
    aq = q64.apply_affine(x, 0.5, 1.5, 0.25, z)
    assert float(torch.linalg.norm(aq - a64)) <= 1e-13 * float(torch.linalg.norm(a64))
    e64 = mb.find_min_eigenpair(f64, 300, x, conv_tol=1e-13, want_vector=False).value
    eq = mb.find_min_eigenpair(q64, 300, x, conv_tol=1e-13, want_vector=False).value
    assert abs(eq - e64) <= 1e-12 * abs(e64)
    lo, hi = e64 - 0.5, 60.0
    m64 = mb.kpm_dos_moments(f64, 64, 2, 7, lo, hi, 0.01)
    mq = mb.kpm_dos_moments(q64, 64, 2, 7, lo, hi, 0.01)
    assert np.max(np.abs(np.asarray(mq) - np.asarray(m64))) <= 1e-10


def test_momentum_operator_rejects_mixed_models(mb, cuda):
    b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(4, 2, 0, [4], [0])
    with pytest.raises(mb.MbError):
        mb.GpuHubbardOperator(b, mb.HubbardModel(1.0, 2.0, 4))
    with pytest.raises(mb.MbError):  # a whole basis as well: no Q64 for momentum space
        mb.HubbardMomentumFactorized(mb.FermionBasis.with_fixed_particle_number_and_spin(4, 2, 0),
                                     [4], 1.0, 2.0, mb.PREC_Q64)
    with pytest.raises(mb.MbError):  # lattice of 4 sites, basis of 6 orbitals
        mb.HubbardMomentumFactorized(mb.FermionBasis.with_fixed_particle_number_and_spin(6, 2, 0),
                                     [4], 1.0, 2.0)


def make_full(mb, g):
    dims = [int(d) for d in g["dims"]]
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(
        int(np.prod(dims)), int(g["particles"]), int(g["spin_projection"]))
    return basis, dims


@pytest.mark.parametrize("name", momentum_full_cases())
def test_whole_basis_momentum_matrix_matches_reference(mb, cuda, name):
    """compute_matrix_elements of HubbardModelMomentum on a whole (N_up, N_down)
    basis (the matrix of HubbardMomentumFactorized), union of the K sectors."""
    g = load_golden(name)
    basis, dims = make_full(mb, g)
    H = mb.compute_matrix_elements(basis, mb.HubbardModelMomentum(float(g["t"]), float(g["U"]), dims))
    rows = np.repeat(np.arange(H.dim), np.diff(H.row_ptr))
    assert H.nnz == len(g["row"])
    assert np.array_equal(rows, g["row"]) and np.array_equal(H.col_idx, g["col"])
    off = rows != H.col_idx
    assert np.array_equal(H.values.real[off], g["val"][off])
    scale = max(np.abs(g["val"]).max(), 1.0)
    assert np.max(np.abs(H.values.real[~off] - g["val"][~off]), initial=0.0) <= 1e-14 * scale
    assert not H.values.imag.any()


@pytest.mark.parametrize("name", momentum_full_cases())
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-6)])
def test_factorized_operator_apply(mb, cuda, name, prec, tol):
    """HubbardMomentumFactorized(basis, lattice_size, t, U).apply against the
    reference's matrix, on device and host buffers (reference order)."""
    torch = cuda
    g = load_golden(name)
    basis, dims = make_full(mb, g)
    op = mb.HubbardMomentumFactorized(basis, dims, float(g["t"]), float(g["U"]), prec)
    n = op.dimension()
    rng = np.random.default_rng(5)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    dt = torch.complex64 if prec else torch.complex128
    ref = ref_csr(g) @ x
    scale = max(np.linalg.norm(ref), 1e-300)
    y = op.apply(torch.tensor(x, dtype=dt, device="cuda")).cpu().numpy()
    assert np.linalg.norm(y - ref) <= tol * scale
    yh = np.zeros(n, np.complex64 if prec else np.complex128)
    op.apply_host(x.astype(yh.dtype), yh)
    assert np.linalg.norm(yh - ref) <= tol * scale


def test_factorized_operator_spectrum_and_ground_state(mb, cuda):
    """The factorized momentum-space operator is the real-space Hamiltonian in
    another single-particle basis: 1D L=6, 2+2 spectra agree (dense), and at
    3x3, 3+3 (7056 states) Lanczos on it gives the real-space ground state."""
    dims = [6]
    E_real = np.linalg.eigvalsh(oracle.hubbard_csc(dims, 1.0, 3.0, 2, 2).to_dense())
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(6, 4, 0)
    H = mb.compute_matrix_elements(basis, mb.HubbardModelMomentum(1.0, 3.0, dims))
    E_mom = np.linalg.eigvalsh(H.to_scipy().toarray())
    assert np.max(np.abs(E_mom - E_real)) <= 1e-10 * np.abs(E_real).max()
    real = mb.GpuHubbardOperator(mb.FermionBasis.with_fixed_particle_number_and_spin(9, 6, 0),
                                 mb.HubbardModel2D(1.0, 4.0, 3, 3))
    e_real = mb.find_min_eigenpair(real, 200, reorth=True, want_vector=False).value
    fact = mb.HubbardMomentumFactorized(mb.FermionBasis.with_fixed_particle_number_and_spin(9, 6, 0),
                                        [3, 3], 1.0, 4.0)
    assert fact.dimension() == 7056
    e_fact = mb.find_min_eigenpair(fact, 200, reorth=True, want_vector=False).value
    assert abs(e_fact - e_real) <= 1e-10 * abs(e_real)
