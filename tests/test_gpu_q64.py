"""Block-floating-point (MB_PREC_Q64) operators: FP64-class results computed
with integer arithmetic on GB300.

Tolerances: the apply is compared with the reference CSR at the FP64 bar,
||y - y_ref|| <= 1e-13 ||y_ref|| (mantissas keep >= 56 bits relative to the
largest element); ground-state energies |dE0| <= 1e-10 |E0|; Krylov
evolution <= 1e-10 relative; DOS moments <= 1e-10 absolute.
"""
import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


def make(mb, dims, t, u, n_up, n_down, prec=2):
    L = int(np.prod(dims))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, n_up + n_down, n_up - n_down)
    model = mb._Hubbard(t, u, dims)
    return basis, model, mb.GpuHubbardOperator(basis, model, prec)


def ref_csr(g):
    import scipy.sparse as sp
    n = len(g["up"])
    return sp.csr_matrix((g["val"], (g["row"], g["col"])), shape=(n, n))


@pytest.mark.parametrize("name", golden_cases())
def test_q64_apply_matches_reference_csr(mb, cuda, name):
    torch = cuda
    g = load_golden(name)
    dims = [int(d) for d in g["dims"]]
    if 1 in dims:  # a size-1 dimension makes self bonds: Q64 refuses those
        with pytest.raises(mb.MbError) as e:
            make(mb, dims, float(g["t"]), float(g["U"]), g["n_up"], g["n_down"])
        assert e.value.status == mb.MB_ERR_INVALID_ARG
        return
    _, _, op = make(mb, dims, float(g["t"]), float(g["U"]), g["n_up"], g["n_down"])
    n = op.dimension()
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    y_ref = ref_csr(g) @ x
    y = op.apply(torch.tensor(x, device="cuda")).cpu().numpy()
    scale = np.linalg.norm(y_ref)
    assert np.linalg.norm(y - y_ref) <= 1e-13 * scale + 1e-300
    perm = op.basis.permutation()
    yt = op.apply(torch.tensor(x[perm], device="cuda"), order=mb.ORDER_TENSOR).cpu().numpy()
    assert np.linalg.norm(yt - y_ref[perm]) <= 1e-13 * scale + 1e-300
    # host buffers (pipelined: chunked upload, split row schedule): the same
    # arithmetic as the device call, so bit-identical; pageable and page-locked
    yh = np.zeros(n, np.complex128)
    op.apply_host(x, yh)
    assert np.array_equal(yh, y)
    xp = torch.tensor(x).pin_memory()
    yp = torch.zeros(n, dtype=torch.complex128).pin_memory()
    op.apply_host(xp, yp)
    assert np.array_equal(yp.numpy(), y)


def test_q64_roundtrip_and_native_apply(mb, cuda):
    torch = cuda
    g = load_golden("sq3x3_n5_sz1")
    _, _, op = make(mb, [3, 3], 1.0, 8.0, g["n_up"], g["n_down"])
    bits = op.q64_mantissa_bits()
    assert 50 <= bits <= 62
    x = op.seed_vector(3)
    q, e = op.q64_from_f64(x)
    assert int(q.abs().max()) < 2 ** bits
    back = op.q64_to_f64(q, e)
    # f64 -> Q64 -> f64 loses nothing above the quantum 2^e
    assert float((back - x).abs().max()) <= 2.0 ** e
    yq, ey = op.apply_q64(q, e)
    y = op.q64_to_f64(yq, ey).cpu().numpy()
    ref = ref_csr(g) @ x.cpu().numpy()
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
    assert int(yq.abs().max()) < 2 ** bits


def test_q64_conversion_edge_values(mb, cuda):
    """Exact round trip of values that are whole multiples of the quantum,
    signs, zeros, and a vector with a huge dynamic range."""
    torch = cuda
    _, _, op = make(mb, [4], 1.0, 4.0, 2, 2)
    n = op.dimension()
    vals = np.zeros(n, np.complex128)
    vals[0] = 1.0 - 0.5j
    vals[1] = -3.0 + 0.0j
    vals[2] = 1e-300
    vals[3] = -2.0 ** -40 + 1j * 2.0 ** -30
    vals[5] = 0.75
    x = torch.tensor(vals, device="cuda")
    q, e = op.q64_from_f64(x)
    back = op.q64_to_f64(q, e).cpu().numpy()
    assert back[0] == vals[0] and back[1] == vals[1] and back[5] == vals[5]
    assert back[3] == vals[3]
    assert back[2] == 0.0          # far below the quantum: flushed
    assert np.all(back[6:] == 0.0)


def test_q64_ground_state_chain8(mb, cuda):
    _, _, op = make(mb, [8], 1.0, 4.0, 4, 4)
    E = np.linalg.eigvalsh(oracle.hubbard_csc([8], 1.0, 4.0, 4, 4).to_dense())
    res = mb.find_min_eigenpair(op, 200, op.seed_vector(0))
    assert res.steps == 200
    assert abs(res.value - E[0]) <= 1e-10 * abs(E[0])
    v = res.vector
    op64 = mb.GpuHubbardOperator(op.basis, op.model, mb.PREC_F64)
    hv = op64.apply(v)
    lam = op64.dot_re(v, hv) / op64.dot_re(v, v)
    assert abs(lam - E[0]) <= 1e-9 * abs(E[0])


def test_q64_ground_state_reorth_2x4(mb, cuda):
    """2x4 lattice (doubled bonds), full re-orthogonalisation, early stop."""
    _, _, op = make(mb, [2, 4], 1.0, 3.0, 2, 2)
    E = np.linalg.eigvalsh(oracle.hubbard_csc([2, 4], 1.0, 3.0, 2, 2).to_dense())
    res = mb.find_min_eigenpair(op, 150, reorth=True, conv_tol=1e-14, check_every=5)
    assert abs(res.value - E[0]) <= 1e-10 * abs(E[0])
    res = mb.find_max_eigenpair(op, 150, reorth=True)
    assert abs(res.value - E[-1]) <= 1e-10 * abs(E[-1])


@pytest.mark.parametrize("imaginary", [False, True])
def test_q64_time_evolution(mb, cuda, imaginary):
    _, _, op = make(mb, [6], 1.0, 4.0, 3, 3)
    H = oracle.hubbard_csc([6], 1.0, 4.0, 3, 3)
    psi = op.seed_vector(9)
    fn = mb.imaginary_time_evolve_state if imaginary else mb.time_evolve_state
    out = fn(op, psi, 0.25).cpu().numpy()
    ref = H.time_evolve(psi.cpu().numpy(), 0.25, 30, imaginary)
    assert np.linalg.norm(out - ref) <= 1e-10 * np.linalg.norm(ref)


@pytest.mark.parametrize("dims,nu,nd", [([6], 3, 3), ([2, 4], 2, 2)])
def test_q64_kpm_dos_moments_match_oracle(mb, cuda, dims, nu, nd):
    """DOS Chebyshev moments on Q64 vectors (exact integer dot products)
    against the oracle's FP64 recurrence with the same probes: <= 1e-10."""
    _, _, op = make(mb, dims, 1.0, 4.0, nu, nd)
    H = oracle.hubbard_csc(dims, 1.0, 4.0, nu, nd)
    E = np.linalg.eigvalsh(H.to_dense())
    M, R = 64, 3
    mu = mb.kpm_dos_moments(op, M, R, 11, E[0], E[-1], 0.01)
    a = (E[-1] - E[0]) / 2 * 1.01
    b = (E[-1] + E[0]) / 2
    perm = op.basis.permutation()
    ref = np.zeros(M)
    for p in range(R):
        rt = oracle.philox_phase(11, op.dimension(), 1 + p)
        r = np.empty_like(rt)
        r[perm] = rt
        ref += H.kpm_dos_moments(r, M, a, b)
    ref /= R * op.dimension()
    assert abs(mu[0] - 1.0) < 1e-12
    assert np.max(np.abs(mu - ref)) <= 1e-10


def test_q64_full_size_4x4_matches_f64(mb, cuda):
    """4x4, 6+6 at full size: the Q64 apply agrees with the FP64 apply."""
    torch = cuda
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 12, 0)
    model = mb.HubbardModel2D(1.0, 8.0, 4, 4)
    opq = mb.GpuHubbardOperator(basis, model, mb.PREC_Q64)
    op64 = mb.GpuHubbardOperator(basis, model, mb.PREC_F64)
    x = op64.seed_vector(1, order=mb.ORDER_TENSOR)
    y64 = op64.apply(x, order=mb.ORDER_TENSOR)
    q, e = opq.q64_from_f64(x, order=mb.ORDER_TENSOR)
    del opq  # the native path below needs only the operator tables
    opq = mb.GpuHubbardOperator(basis, model, mb.PREC_Q64)
    yq, ey = opq.apply_q64(q, e)
    y = opq.q64_to_f64(yq, ey, order=mb.ORDER_TENSOR)
    rel = float(torch.linalg.norm(y - y64)) / float(torch.linalg.norm(y64))
    assert rel <= 1e-13


@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("dims,n_up,n_down", [
    ((4, 4), 5, 5),  # eight row groups
    ((14,), 4, 3),   # 1,001 rows: seven groups, the last wave partial
    ((12,), 3, 3),   # 220 rows: two groups
    ((8,), 0, 3),    # a single row group
    ((3, 2), 2, 3),
])
def test_q64_host_apply_groups_bit_identical(mb, cuda, pinned, dims, n_up, n_down):
    """The pipelined host-buffer apply of a Q64 operator (rows in groups, each
    finished reference prefix downloaded while later groups run) equals the
    device-buffer apply bit for bit, page-locked and pageable."""
    torch = cuda
    L = int(np.prod(dims))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, n_up + n_down, n_up - n_down)
    op = mb.GpuHubbardOperator(basis, mb._Hubbard(1.0, 8.0, list(dims)), mb.PREC_Q64)
    x = op.seed_vector(11)
    y = op.apply(x).cpu()
    xh = x.cpu()
    yh = torch.full_like(xh, float("nan"))
    if pinned:
        xh, yh = xh.pin_memory(), yh.pin_memory()
    op.apply_host(xh, yh)
    assert torch.equal(yh, y)


def test_q64_host_apply_full_size_bit_identical(mb, cuda):
    """4x4, 6+6: the pipelined host-buffer apply (page-locked buffers) equals
    the device-buffer apply in reference order bit for bit."""
    torch = cuda
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 12, 0)
    model = mb.HubbardModel2D(1.0, 8.0, 4, 4)
    op = mb.GpuHubbardOperator(basis, model, mb.PREC_Q64)
    x = op.seed_vector(3)
    y = op.apply(x).cpu()
    xh = x.cpu().pin_memory()
    yh = torch.empty_like(xh).pin_memory()
    op.apply_host(xh, yh)
    assert torch.equal(yh, y)
    del x, y
    torch.cuda.empty_cache()


def test_q64_on_a_large_dynamic_range_vector(mb, cuda):
    """Block floating point keeps one exponent per vector, so an element far
    below the largest keeps fewer significant bits (~56 - log2(max/|x_i|)).
    On the converged 3x3, U = 8 ground state (components spread over many
    decades) the Q64 apply, a Lanczos run started from it and a KPM projector
    applied to it agree with FP64 to the FP64 bars: the error of every element
    stays below 2^-50 of the vector's largest, and the norm-wise and energy
    errors below 1e-13 and 1e-12."""
    torch = cuda
    dims, nu, nd, u = (3, 3), 4, 4, 8.0
    _, _, op64 = make(mb, dims, 1.0, u, nu, nd, prec=0)
    _, _, opq = make(mb, dims, 1.0, u, nu, nd, prec=2)
    gs = mb.find_min_eigenpair(op64, 300, op64.seed_vector(0), reorth=True, conv_tol=1e-14)
    x = gs.vector
    a = torch.abs(x)
    nz = a[a > 0]
    spread = float(nz.max() / nz.min())
    assert spread > 1e6, spread                       # a large dynamic range
    y64 = op64.apply(x)
    yq = opq.apply(x)
    err = torch.abs(yq - y64)
    assert float(err.max()) <= 2.0 ** -50 * float(torch.abs(y64).max())
    assert float(torch.linalg.norm(yq - y64)) <= 1e-13 * float(torch.linalg.norm(y64))
    # Lanczos from the ground state (a start vector of large dynamic range)
    e64 = mb.find_min_eigenpair(op64, 20, x, want_vector=False).value
    eq = mb.find_min_eigenpair(opq, 20, x, want_vector=False).value
    assert abs(eq - e64) <= 1e-12 * abs(e64)
    assert abs(e64 - gs.value) <= 1e-10 * abs(gs.value)
    # the KPM Fermi projector (a 256-term Chebyshev sum) applied to it
    lo, hi = gs.value, mb.find_max_eigenpair(op64, 200, op64.seed_vector(1), conv_tol=1e-12,
                                             want_vector=False).value
    p64 = mb.SparseKPMProjector(op64, 256, lo, hi, 0.5 * (lo + hi)).apply(x)
    pq = mb.SparseKPMProjector(opq, 256, lo, hi, 0.5 * (lo + hi)).apply(x)
    assert float(torch.linalg.norm(pq - p64)) <= 1e-12 * float(torch.linalg.norm(p64))
