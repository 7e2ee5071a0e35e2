"""GPU parity: the CUDA path against the reference's own outputs (golden
fixtures) and the CPU oracle, through the C ABI.

Tolerances (stated here, used below):
  * sparse structure, signs and values of H: bit-exact;
  * FP64 apply vs the reference CSR: ||y - y_ref|| <= 1e-13 ||y_ref||;
  * FP32 apply vs the reference CSR: ||y - y_ref|| <= 2e-6 ||y_ref||;
  * FP64 ground-state energy vs the oracle's Lanczos and vs dense eigvalsh:
    |dE0| <= 1e-10 |E0|;
  * Krylov evolution vs the oracle: <= 1e-10 relative;
  * KPM DOS moments vs the oracle: <= 1e-10 absolute (moments are O(1)).
"""
import numpy as np
import pytest

import oracle
from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu


def make(mb, dims, t, u, n_up, n_down, prec=0):
    L = int(np.prod(dims))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, n_up + n_down, n_up - n_down)
    model = mb._Hubbard(t, u, dims)
    op = mb.GpuHubbardOperator(basis, model, prec)
    return basis, model, op


def ref_csr(g):
    import scipy.sparse as sp
    n = len(g["up"])
    return sp.csr_matrix((g["val"], (g["row"], g["col"])), shape=(n, n))


@pytest.mark.parametrize("name", golden_cases())
def test_gpu_matrix_elements_bit_exact(mb, cuda, name):
    g = load_golden(name)
    basis, model, _ = make(mb, [int(d) for d in g["dims"]], float(g["t"]), float(g["U"]),
                           g["n_up"], g["n_down"])
    H = mb.compute_matrix_elements(basis, model)
    rows = np.repeat(np.arange(H.dim), np.diff(H.row_ptr))
    assert H.nnz == len(g["row"])
    assert np.array_equal(rows, g["row"])
    assert np.array_equal(H.col_idx, g["col"])
    assert np.array_equal(H.values.real, g["val"])
    assert not H.values.imag.any()


@pytest.mark.parametrize("name", golden_cases())
@pytest.mark.parametrize("prec", [0, 1])
def test_gpu_apply_matches_reference_csr(mb, cuda, name, prec):
    torch = cuda
    g = load_golden(name)
    _, _, op = make(mb, [int(d) for d in g["dims"]], float(g["t"]), float(g["U"]), g["n_up"],
                    g["n_down"], prec)
    n = op.dimension()
    rng = np.random.default_rng(7)
    x = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    y_ref = ref_csr(g) @ x
    dt = torch.complex64 if prec else torch.complex128
    xd = torch.tensor(x, dtype=dt, device="cuda")
    y = op.apply(xd).cpu().numpy()
    tol = 2e-6 if prec else 1e-13
    scale = max(np.linalg.norm(y_ref), 1e-300)
    assert np.linalg.norm(y - y_ref) <= tol * scale + (0 if np.linalg.norm(y_ref) else 1e-300)
    # tensor order is the same operator under the basis permutation
    perm = op.basis.permutation()
    xt = torch.tensor(x[perm], dtype=dt, device="cuda")
    yt = op.apply(xt, order=mb.ORDER_TENSOR).cpu().numpy()
    assert np.linalg.norm(yt - y_ref[perm]) <= tol * scale
    # host-buffer apply
    yh = np.zeros(n, np.complex64 if prec else np.complex128)
    op.apply_host(x.astype(yh.dtype), yh)
    assert np.linalg.norm(yh - y_ref) <= tol * scale


def test_gpu_apply_affine(mb, cuda):
    torch = cuda
    g = load_golden("sq3x3_n5_sz1")
    _, _, op = make(mb, [3, 3], 1.0, 8.0, g["n_up"], g["n_down"])
    n = op.dimension()
    rng = np.random.default_rng(1)
    x = rng.normal(size=n) + 1j * rng.normal(size=n)
    z = rng.normal(size=n) + 1j * rng.normal(size=n)
    H = ref_csr(g)
    ref = 0.37 * (H @ x - 1.5 * x) - 0.8 * z
    xd = torch.tensor(x, device="cuda")
    zd = torch.tensor(z, device="cuda")
    y = op.apply_affine(xd, scale=0.37, shift=1.5, beta=-0.8, z=zd).cpu().numpy()
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)
    # in place on z (Chebyshev step form), tensor order
    perm = op.basis.permutation()
    xt = torch.tensor(x[perm], device="cuda")
    zt = torch.tensor(z[perm], device="cuda")
    op.apply_affine(xt, scale=0.37, shift=1.5, beta=-0.8, z=zt, out=zt, order=mb.ORDER_TENSOR)
    assert np.linalg.norm(zt.cpu().numpy() - ref[perm]) <= 1e-13 * np.linalg.norm(ref)


def test_seed_vectors_match_oracle_bits(mb, cuda):
    _, _, op = make(mb, [8], 1.0, 4.0, 4, 4)
    perm = op.basis.permutation()
    v_t = op.seed_vector(0, order=mb.ORDER_TENSOR).cpu().numpy()
    ref = oracle.philox_uniform(0, op.dimension())
    assert np.array_equal(v_t, ref)                       # bit-identical, tensor order
    v_r = op.seed_vector(0).cpu().numpy()
    assert np.array_equal(v_r[perm], ref)                 # same values in reference order
    ph = op.phase_vector(3, 2, order=mb.ORDER_TENSOR).cpu().numpy()
    ph_ref = oracle.philox_phase(3, op.dimension(), 2)
    assert np.max(np.abs(ph - ph_ref)) < 1e-15


def oracle_chain8():
    H = oracle.hubbard_csc([8], 1.0, 4.0, 4, 4)
    return H


def test_ground_state_chain8_plain_lanczos(mb, cuda):
    """1D L=8 4+4, U=4, 200 plain Lanczos steps from the seed-0 vector."""
    _, _, op = make(mb, [8], 1.0, 4.0, 4, 4)
    H = oracle_chain8()
    E = np.linalg.eigvalsh(H.to_dense())
    perm = op.basis.permutation()
    seed_t = oracle.philox_uniform(0, op.dimension())
    seed_ref = np.empty_like(seed_t)
    seed_ref[perm] = seed_t
    e_or, vec_or, m_or, al_or, be_or = H.find_min_eigenpair(seed_ref, 200)
    res = mb.find_min_eigenpair(op, 200, op.seed_vector(0))
    assert abs(res.value - e_or) <= 1e-10 * abs(e_or)
    assert abs(res.value - E[0]) <= 1e-10 * abs(E[0])
    assert res.steps == m_or
    v = res.vector.cpu().numpy()
    ov = abs(np.vdot(v, vec_or)) / (np.linalg.norm(v) * np.linalg.norm(vec_or))
    assert ov > 1 - 1e-6


def test_ground_state_reorth_and_early_stop(mb, cuda):
    import torch
    _, _, op = make(mb, [8], 1.0, 4.0, 4, 4)
    E = np.linalg.eigvalsh(oracle_chain8().to_dense())
    res = mb.find_min_eigenpair(op, 200, reorth=True)
    assert abs(res.value - E[0]) <= 1e-10 * abs(E[0])
    v = res.vector
    hv = op.apply(v)
    lam = op.dot_re(v, hv) / op.dot_re(v, v)
    r = hv - lam * v
    assert float(torch.linalg.norm(r)) <= 1e-7 * float(torch.linalg.norm(v))
    res2 = mb.find_min_eigenpair(op, 200, reorth=True, conv_tol=1e-13, check_every=5)
    assert res2.steps < 200
    assert abs(res2.value - E[0]) <= 1e-10 * abs(E[0])
    res3 = mb.find_min_eigenpair(op, 120, reorth=True, basis_precision=1)
    assert abs(res3.value - E[0]) <= 1e-9 * abs(E[0])


def test_find_max_eigenpair(mb, cuda):
    _, _, op = make(mb, [3, 3], 1.0, 8.0, 2, 2)
    H = oracle.hubbard_csc([3, 3], 1.0, 8.0, 2, 2)
    E = np.linalg.eigvalsh(H.to_dense())
    res = mb.find_max_eigenpair(op, 150, reorth=True)
    assert abs(res.value - E[-1]) <= 1e-10 * abs(E[-1])


def test_lanczos_pass_one_two_roundtrip(mb, cuda):
    """solve() = pass one, small solve, pass two (lanczos.h:220-237) vs the oracle."""
    _, _, op = make(mb, [6], 1.0, 4.0, 3, 3)
    H = oracle.hubbard_csc([6], 1.0, 4.0, 3, 3)
    n = op.dimension()
    b = op.seed_vector(5)
    dec = mb.lanczos_pass_one(op, b, 40)
    bh = b.cpu().numpy()
    assert dec.steps_taken == 40
    assert abs(dec.b_norm - np.linalg.norm(bh)) <= 1e-13 * dec.b_norm
    # alpha_0 = <v0, H v0>
    v0 = bh / np.linalg.norm(bh)
    assert abs(dec.alphas[0] - np.vdot(v0, H.apply(v0)).real) <= 1e-12
    # pass two with y = ||b|| e1 rebuilds b; with y = ||b|| (alpha0, beta0, 0, ...)
    # it rebuilds H b = ||b|| (alpha0 v0 + beta0 v1).
    y = np.zeros(40, np.complex128)
    y[0] = dec.b_norm
    x = mb.lanczos_pass_two(op, b, dec, y).cpu().numpy()
    assert np.linalg.norm(x - bh) <= 1e-13 * np.linalg.norm(bh)
    y[0] = dec.b_norm * dec.alphas[0]
    y[1] = dec.b_norm * dec.betas[0]
    x = mb.lanczos_pass_two(op, b, dec, y).cpu().numpy()
    hb = H.apply(bh)
    assert np.linalg.norm(x - hb) <= 1e-12 * np.linalg.norm(hb)
    # tridiagonal entries agree with the oracle's pass one (find_max on H)
    e_or, _, m_or, al_or, be_or = H.find_min_eigenpair(bh, 40, want_vec=False)
    # the oracle ran on -H: alphas flip sign, betas agree
    # (first 20 steps: later ones amplify rounding differences once Ritz values converge)
    assert np.allclose(-al_or[:20], dec.alphas[:20], atol=1e-9)
    assert np.allclose(be_or[:20], dec.betas[:20], atol=1e-9)


@pytest.mark.parametrize("imaginary", [False, True])
def test_time_evolution_matches_oracle(mb, cuda, imaginary):
    _, _, op = make(mb, [6], 1.0, 4.0, 3, 3)
    H = oracle.hubbard_csc([6], 1.0, 4.0, 3, 3)
    psi = op.seed_vector(9)
    ph = psi.cpu().numpy()
    t = 0.25
    if imaginary:
        out = mb.imaginary_time_evolve_state(op, psi, t).cpu().numpy()
    else:
        out = mb.time_evolve_state(op, psi, t).cpu().numpy()
    ref = H.time_evolve(ph, t, 30, imaginary)
    assert np.linalg.norm(out - ref) <= 1e-10 * np.linalg.norm(ref)


def test_time_evolve_steps_unitary(mb, cuda):
    import scipy.linalg as sla
    _, _, op = make(mb, [4], 1.0, 2.0, 2, 2)
    H = oracle.hubbard_csc([4], 1.0, 2.0, 2, 2).to_dense()
    psi = op.seed_vector(2)
    p0 = psi.cpu().numpy()
    mb.time_evolve_state_steps(op, psi, 0.0, 1.0, 0.1)
    ref = sla.expm(-1j * 1.0 * H) @ p0
    assert np.linalg.norm(psi.cpu().numpy() - ref) <= 1e-8 * np.linalg.norm(ref)


def test_kpm_dos_moments_match_oracle(mb, cuda):
    _, _, op = make(mb, [6], 1.0, 4.0, 3, 3)
    H = oracle.hubbard_csc([6], 1.0, 4.0, 3, 3)
    E = np.linalg.eigvalsh(H.to_dense())
    emin, emax = E[0], E[-1]
    M, R = 64, 3
    mu = mb.kpm_dos_moments(op, M, R, 11, emin, emax, 0.01)
    a = (emax - emin) / 2 * 1.01
    b = (emax + emin) / 2
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
    # the exact trace moments, (1/D) Tr T_n(Ht), are close to the stochastic ones
    x = (E - b) / a
    exact = np.array([np.mean(np.cos(n * np.arccos(x))) for n in range(M)])
    assert np.max(np.abs(mu - exact)) < 0.2


def test_kpm_projector_apply_matches_oracle(mb, cuda):
    _, _, op = make(mb, [4], 1.0, 2.0, 2, 2)
    H = oracle.hubbard_csc([4], 1.0, 2.0, 2, 2)
    E = np.linalg.eigvalsh(H.to_dense())
    v = op.seed_vector(4)
    P = mb.SparseKPMProjector(op, 40, E[0], E[-1], 0.5, 0.01)
    out = P.apply(v).cpu().numpy()
    ref = H.kpm_projector_apply(v.cpu().numpy(), 40, E[0], E[-1], 0.5, 0.01)
    assert np.linalg.norm(out - ref) <= 1e-11 * np.linalg.norm(ref)


def test_estimate_bounds_brackets_spectrum(mb, cuda):
    _, _, op = make(mb, [6], 1.0, 4.0, 3, 3)
    E = np.linalg.eigvalsh(oracle.hubbard_csc([6], 1.0, 4.0, 3, 3).to_dense())
    lo, hi = mb.estimate_bounds(op, 400, 0.01)
    assert lo <= hi
    assert abs(lo - E[0]) < 0.5 and abs(hi - E[-1]) < 0.5


def test_error_paths(mb, cuda):
    torch = cuda
    _, _, op = make(mb, [4], 1.0, 2.0, 2, 2)
    z = torch.zeros(op.dimension(), dtype=torch.complex128, device="cuda")
    with pytest.raises(mb.MbError) as e:
        mb.find_min_eigenpair(op, 10, z)
    assert e.value.status == mb.MB_ERR_ZERO_NORM
    x = op.seed_vector(1)
    with pytest.raises(mb.MbError):
        op.apply(x, out=x)          # overlapping in/out
    rc = mb.lib().mb_op_apply(op.handle, x.data_ptr(), op.empty().data_ptr(), 7, None)
    assert rc == mb.MB_ERR_INVALID_ARG                                            # bad order


def test_concurrent_apply_on_streams(mb, cuda):
    """apply() on one operator from several streams (the reference's OpenMP
    sample loops call apply concurrently on a shared operator)."""
    torch = cuda
    g = load_golden("chain8_n8")
    _, _, op = make(mb, [8], 1.0, 4.0, 4, 4)
    H = ref_csr(g)
    xs = [op.seed_vector(s) for s in range(4)]
    streams = [torch.cuda.Stream() for _ in range(4)]
    ys = []
    for x, s in zip(xs, streams):
        with torch.cuda.stream(s):
            ys.append(op.apply(x, stream=s.cuda_stream))
    torch.cuda.synchronize()
    for x, y in zip(xs, ys):
        ref = H @ x.cpu().numpy()
        assert np.linalg.norm(y.cpu().numpy() - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("pinned", [True, False])
@pytest.mark.parametrize("dims,n_up,n_down", [
    ((4, 4), 5, 5),  # 19,079,424 states: eight row groups, eight landing chunks
    ((14,), 4, 3),   # 1,001 rows: seven (FP64) or four (FP32) groups, the last wave partial
    ((12,), 3, 3),   # 220 rows: two groups (FP64), one (FP32)
    ((8,), 0, 3),    # one up configuration: a single row group
    ((6,), 6, 2),    # a full up band: a single row group
    ((3, 2), 2, 3),
])
def test_host_apply_bit_identical(mb, cuda, prec, pinned, dims, n_up, n_down):
    """The pipelined host-buffer apply of a complex128 / complex64 operator in
    reference order (rows applied in groups, each finished reference prefix
    downloaded while later groups run) equals the device-buffer apply bit for
    bit, with page-locked and with pageable host buffers."""
    torch = cuda
    _, _, op = make(mb, dims, 1.0, 8.0, n_up, n_down, prec)
    x = op.seed_vector(5)
    y = op.apply(x).cpu()
    xh = x.cpu()
    yh = torch.full_like(xh, float("nan"))
    if pinned:
        xh, yh = xh.pin_memory(), yh.pin_memory()
    op.apply_host(xh, yh)
    assert torch.equal(yh, y)
    del x, y
    torch.cuda.empty_cache()


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_concurrent_apply_from_host_threads(mb, cuda, prec):
    """Several host threads share one operator: each applies on its own stream
    in reference order (per-stream scratch) and through host buffers (calls
    serialised on the operator)."""
    import threading
    torch = cuda
    g = load_golden("sq3x3_n5_sz1")
    _, _, op = make(mb, [3, 3], 1.0, 8.0, g["n_up"], g["n_down"], prec)
    H = ref_csr(g)
    tol = 2e-6 if prec == 1 else 1e-13
    n = op.dimension()
    errors = []

    def work(k):
        try:
            s = torch.cuda.Stream()
            with torch.cuda.stream(s):
                x = op.seed_vector(10 + k)
                for _ in range(20):
                    y = op.apply(x, stream=s.cuda_stream)
            s.synchronize()
            ref = H @ x.cpu().numpy()
            errors.append(np.linalg.norm(y.cpu().numpy() - ref) / np.linalg.norm(ref))
            xh = x.cpu().numpy()
            yh = np.zeros_like(xh)
            op.apply_host(xh, yh)
            errors.append(np.linalg.norm(yh - ref) / np.linalg.norm(ref))
        except Exception as exc:  # reported to the main thread
            errors.append(exc)

    threads = [threading.Thread(target=work, args=(k,)) for k in range(6)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert len(errors) == 12
    for e in errors:
        assert not isinstance(e, Exception), e
        assert e <= tol


@pytest.mark.parametrize("dims,n", [((4, 4), 6), ((16,), 8)])
def test_full_size_operator_properties(mb, cuda, dims, n):
    """The 4x4 6+6 and 1D L=16 8+8 sectors at full size (64.1M / 165.6M
    states): Hermiticity <x,Hy> = <Hx,y>, linearity, FP32 vs FP64 agreement,
    and the diagonal expectation <e_i|H|e_i> = U*n_double."""
    torch = cuda
    L = int(np.prod(dims))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, 2 * n, 0)
    model = mb._Hubbard(1.0, 8.0, dims)
    op = mb.GpuHubbardOperator(basis, model, 0)
    x = op.seed_vector(1, order=mb.ORDER_TENSOR)
    y = op.seed_vector(2, order=mb.ORDER_TENSOR)
    hx = op.apply(x, order=mb.ORDER_TENSOR)
    hy = op.apply(y, order=mb.ORDER_TENSOR)
    a = op.dot_re(x, hy)
    b = op.dot_re(hx, y)
    assert abs(a - b) <= 1e-11 * op.norm(x) * op.norm(hy)
    # linearity: H(x + 2y) = Hx + 2Hy
    z = x + 2 * y
    hz = op.apply(z, order=mb.ORDER_TENSOR)
    d = hz - (hx + 2 * hy)
    assert float(torch.linalg.norm(d)) <= 1e-13 * float(torch.linalg.norm(hz))
    del z, hz, d
    # FP32 operator agrees to single precision
    op32 = mb.GpuHubbardOperator(basis, model, 1)
    x32 = x.to(torch.complex64)
    hx32 = op32.apply(x32, order=mb.ORDER_TENSOR)
    rel = float(torch.linalg.norm(hx32.to(torch.complex128) - hx)) / float(torch.linalg.norm(hx))
    assert rel < 2e-6


def test_fp32_lanczos_with_fp64_refinement(mb, cuda):
    """Precision path: complex64 vectors, FP64 alpha/beta and re-orthogonalisation
    coefficients, one FP64 Rayleigh-quotient sweep: |dE0| <= 1e-8 |E0|."""
    _, _, op = make(mb, [3, 3], 1.0, 8.0, 3, 2, prec=1)
    E = np.linalg.eigvalsh(oracle.hubbard_csc([3, 3], 1.0, 8.0, 3, 2).to_dense())
    raw = mb.find_min_eigenpair(op, 150, reorth=True, want_vector=False)
    ref = mb.find_min_eigenpair(op, 150, reorth=True, want_vector=False, refine=True)
    assert abs(raw.value - E[0]) <= 1e-5 * abs(E[0])
    assert abs(ref.value - E[0]) <= 1e-8 * abs(E[0])


def test_fp32_refinement_past_convergence(mb, cuda):
    """Plain (not re-orthogonalised) FP32 Lanczos run well past convergence:
    a ghost copy of E0 enters T_k, and a Ritz vector taken from T_k can be a
    near-cancelling mix of the two copies.  The refined energy takes its Ritz
    vector from the first converged checkpoint: |dE0| <= 1e-8 |E0| (the
    unrefined Ritz value only to FP32-level 1e-6)."""
    u = 5.2292243302455415
    _, _, op = make(mb, [8], 1.0, u, 4, 4, prec=1)
    H = oracle.hubbard_csc([8], 1.0, u, 4, 4)
    e_ref = H.find_min_eigenpair(oracle.philox_uniform(1, H.dim), 200, reorth=True,
                                 want_vec=False)[0]
    seed = op.seed_vector(0, order=mb.ORDER_TENSOR)
    raw = mb.find_min_eigenpair(op, 150, seed, order=mb.ORDER_TENSOR, want_vector=False)
    ref = mb.find_min_eigenpair(op, 150, seed, order=mb.ORDER_TENSOR, want_vector=False,
                                refine=True)
    assert raw.steps == 150
    assert abs(raw.value - e_ref) <= 1e-6 * abs(e_ref)
    assert abs(ref.value - e_ref) <= 1e-8 * abs(e_ref)


def test_refinement_far_from_zero(mb, cuda):
    """1D L=14, N_up = N_down = 13 at U = 9.24 (196 states, spectrum 107..121):
    the FP32 Ritz vector is close to an eigenvector (beta_0 ~ 1e-5) of an
    operator far from zero, where the refinement's Gram-Schmidt needs its
    second pass (with one, orthogonality decays by ~|theta|/beta a step and
    the lowest Ritz value falls below E0).  Refined E0 within 1e-8."""
    u = 9.240847688353895
    _, _, op = make(mb, [14], 1.0, u, 13, 13, prec=1)
    E = np.linalg.eigvalsh(oracle.hubbard_csc([14], 1.0, u, 13, 13).to_dense())
    for seed in range(4):
        s = op.seed_vector(seed, order=mb.ORDER_TENSOR)
        r = mb.find_min_eigenpair(op, 400, s, order=mb.ORDER_TENSOR, conv_tol=1e-10,
                                  want_vector=False, refine=True)
        assert abs(r.value - E[0]) <= 1e-8 * abs(E[0])


@pytest.mark.parametrize("prec", [1, 2])
def test_replayed_ritz_vector_is_the_ground_state(mb, cuda, prec):
    """1D L=7, N_up = N_down = 6, U = 0.001 (49 states, E1 - E0 = 1.4e-4): plain
    Lanczos over all 49 steps loses orthogonality once its Ritz pair converges,
    and pass two has to rebuild pass one's vectors exactly for the Ritz vector
    to be the ground state (a replay in other arithmetic gave an FP32 vector
    6 % off it, overlap 1 - 1.9e-3, and a refined energy 1.5e-7 off).  The
    refined FP32 energy within 1e-8; overlap with the exact ground state
    >= 1 - 5e-4 in FP32 (the vector of a Ritz value stable to 1e-9 against a
    gap of 3.5e-5 |H|), >= 1 - 1e-5 in Q64."""
    u = 0.001
    _, _, op = make(mb, [7], 1.0, u, 6, 6, prec=prec)
    E, V = np.linalg.eigh(oracle.hubbard_csc([7], 1.0, u, 6, 6).to_dense())
    for seed in (158, 0, 1, 2, 3):
        s = op.seed_vector(seed)
        r = mb.find_min_eigenpair(op, 49, s, conv_tol=1e-10, refine=prec == 1)
        v = r.vector.cpu().numpy()
        ov = abs(np.vdot(V[:, 0], v)) / np.linalg.norm(v)
        if prec == 1:
            assert abs(r.value - E[0]) <= 1e-8 * abs(E[0]), (seed, r.value - E[0])
        assert ov >= 1 - (5e-4 if prec == 1 else 1e-5), (seed, ov)


def test_solve_linear_system(mb, cuda):
    """solve(op, b, k, solver) (lanczos.h:220-237) with a tridiagonal solver
    T y = e1: over the full Krylov space x = H^-1 b."""
    torch = cuda
    g = load_golden("rect2x3_n4")  # nonsingular: |eigenvalues| >= 0.089
    _, _, op = make(mb, [2, 3], float(g["t"]), float(g["U"]), g["n_up"], g["n_down"])
    n = op.dimension()
    H = ref_csr(g).toarray()
    rng = np.random.default_rng(4)
    b = rng.normal(size=n) + 1j * rng.normal(size=n)

    def tridiag_solve(a, be):
        T = np.diag(a) + np.diag(be, 1) + np.diag(be, -1)
        e1 = np.zeros(len(a))
        e1[0] = 1.0
        return np.linalg.solve(T, e1)

    x = mb.solve(op, torch.tensor(b, device="cuda"), n, tridiag_solve).cpu().numpy()
    assert np.linalg.norm(H @ x - b) <= 1e-7 * np.linalg.norm(b)
    # a zero right-hand side is an error, as in lanczos_pass_one (lanczos.h:144)
    with pytest.raises(mb.MbError) as e:
        mb.solve(op, torch.zeros(n, dtype=torch.complex128, device="cuda"), n, tridiag_solve)
    assert e.value.status == mb.MB_ERR_ZERO_NORM


@pytest.mark.parametrize("prec", [0, 2])
def test_reorth_lanczos_through_breakdown(mb, cuda, prec):
    """More Lanczos steps than the sector has states, with full
    re-orthogonalisation: the Krylov space fills the sector, w becomes
    (numerically) dependent on the stored vectors, so the Gram-Schmidt pass
    cancels most of it and the second pass runs (the DGKS test).  The
    recurrence must stop at the breakdown (beta <= 1000 eps, lanczos.h:106-110)
    within dim steps, with E0 exact to 1e-12."""
    _, _, op = make(mb, [4], 1.0, 4.0, 2, 1, prec)
    n = op.dimension()
    assert n == 24
    H = oracle.hubbard_csc([4], 1.0, 4.0, 2, 1)
    E = np.linalg.eigvalsh(H.to_dense())
    res = mb.find_min_eigenpair(op, 3 * n, reorth=True)
    assert res.steps <= n
    assert abs(res.value - E[0]) <= 1e-12 * abs(E[0])
