"""A seeded sweep over many small sectors: every refined ground-state energy
(the serving engine's path and the single-operator FP32 path) against an
independent FP64 eigensolver (ARPACK through scipy on the oracle's matrix, dense
for the smallest); Krylov time evolution and DOS Chebyshev moments in the three
precisions against the oracle.

Sectors: 1D L = 4..10 and 2x2, 2x3, 3x3, 2x4 periodic; every filling
1 <= N_up, N_down <= L-1 (N_up != N_down too); U from -4 to 20, including 0,
1e-3 and the values where a refinement needs both Gram-Schmidt passes or an
exact replay.  Bar: |dE0| <= 1e-8 max(|E0|, 1) (the batch and serving bar,
absolute where E0 is near zero).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

LATTICES = [(4,), (5,), (6,), (7,), (8,), (9,), (10,), (2, 2), (2, 3), (3, 3), (2, 4)]
US = [0.0, 1e-3, 0.5, 2.0, 4.0, 9.24, 15.0, 20.0, -3.0]


def sweep_cases(n=80, seed=2024):
    rng = np.random.default_rng(seed)
    cases = []
    for i in range(n):
        dims = LATTICES[int(rng.integers(len(LATTICES)))]
        L = int(np.prod(dims))
        nu = int(rng.integers(1, L))
        nd = nu if rng.uniform() < 0.7 else int(rng.integers(1, L))
        u = US[int(rng.integers(len(US)))] if rng.uniform() < 0.6 else float(rng.uniform(-4, 20))
        cases.append((dims, nu, nd, u, i))
    return cases


def exact_e0(dims, nu, nd, u):
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla
    H = oracle.hubbard_csc(list(dims), 1.0, u, nu, nd)
    if H.dim <= 400:
        return float(np.linalg.eigvalsh(H.to_dense())[0])
    A = sp.csc_matrix((H.re + 1j * H.im, H.row_idx, H.col_ptr), shape=(H.dim, H.dim))
    rng = np.random.default_rng(7)  # a random start: a symmetric one can miss the ground state
    v0 = rng.uniform(-1, 1, H.dim) + 1j * rng.uniform(-1, 1, H.dim)
    return float(sla.eigsh(A, k=1, which="SA", tol=1e-14, v0=v0)[0][0])


@pytest.fixture(scope="module")
def cases():
    cs = sweep_cases()
    return [(c, exact_e0(*c[:4])) for c in cs]


def test_sweep_engine_serving_path(mb, cuda, cases):
    """All sectors submitted to one engine as ground-state requests (Ritz
    stability 1e-10, refinement), stepped until every one completes."""
    eng = mb.Engine()
    live, got = {}, {}
    pending = [c for c, _ in cases]
    for _ in range(100000):
        if not pending and not live:
            break
        while pending:
            dims, nu, nd, u, i = pending[0]
            rid = eng.try_submit(mb.sector(dims, nu, nd, 1.0, u), seed=i, kmax=400,
                                 rel_tol=1e-10, refine=True)
            if rid is None:
                break
            live[rid] = pending.pop(0)
        eng.step(1)
        for rid in eng.completed():
            got[live.pop(rid)[4]] = eng.poll(rid).e0
    for (dims, nu, nd, u, i), e in cases:
        assert abs(got[i] - e) <= 1e-8 * max(abs(e), 1.0), (dims, nu, nd, u, got[i], e)


def test_sweep_single_operator_fp32(mb, cuda, cases):
    """The same sectors through find_min_eigenpair on FP32 operators: plain
    Lanczos to Ritz stability 1e-10 (at most 400 steps or the dimension),
    replayed Ritz vector, FP64 refinement."""
    for (dims, nu, nd, u, i), e in cases:
        L = int(np.prod(dims))
        b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
        op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), mb.PREC_F32)
        s = op.seed_vector(i, order=mb.ORDER_TENSOR)
        r = mb.find_min_eigenpair(op, min(400, op.dimension()), s, order=mb.ORDER_TENSOR,
                                  conv_tol=1e-10, want_vector=False, refine=True)
        assert abs(r.value - e) <= 1e-8 * max(abs(e), 1.0), (dims, nu, nd, u, r.value, e)


@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 1e-4), (2, 1e-10)])
@pytest.mark.parametrize("imaginary", [False, True])
def test_sweep_time_evolution(mb, cuda, prec, tol, imaginary):
    """Krylov evolution (30 steps, t = 0.1; the result summed from the kept
    Lanczos vectors) on 16 of the sweep's sectors with at most 5,000 states and
    |U| <= 10 (|H| t below ~7, where 30 steps converge and the late Lanczos
    vectors carry no weight), against the oracle's restatement of
    evolve_state.h on the same start vector: ||dpsi|| <= tol ||psi|| (FP64 and
    Q64 1e-10, FP32 1e-4)."""
    n = 0
    for dims, nu, nd, u, i in sweep_cases():
        if n == 16:
            break
        L = int(np.prod(dims))
        if abs(u) > 10.0:
            continue
        H = oracle.hubbard_csc(list(dims), 1.0, u, nu, nd)
        if H.dim > 5000:
            continue
        n += 1
        b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
        op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), prec)
        psi = op.seed_vector(i)
        ph = psi.cpu().numpy().astype(np.complex128)
        fn = mb.imaginary_time_evolve_state if imaginary else mb.time_evolve_state
        out = fn(op, psi, 0.1).cpu().numpy().astype(np.complex128)
        ref = H.time_evolve(ph, 0.1, 30, imaginary)
        assert np.linalg.norm(out - ref) <= tol * np.linalg.norm(ref), (dims, nu, nd, u)


# FP32: the Chebyshev recurrence's rounding model, 8 k^2 u32 with k = M/2 + 1
# steps behind the last moment (each step adds up to ~8 u32, and an error made
# at step j reaches step k through U_(k-j), norm <= k - j + 1 on [-1, 1])
@pytest.mark.parametrize("prec,tol", [(0, 1e-10), (1, 8 * 65 ** 2 * 2.0 ** -24), (2, 1e-10)])
def test_sweep_kpm_moments(mb, cuda, prec, tol):
    """DOS Chebyshev moments (128 moments, 2 random-phase probes, exact spectral
    bounds padded by 1 %) on 12 of the sweep's sectors with at most 5,000
    states, against the oracle's restatement of kpm.h on the same probes:
    max |dmu_n| <= tol (FP64 and Q64 1e-10, FP32 the rounding model)."""
    M, R, key = 128, 2, 11
    n = 0
    for dims, nu, nd, u, i in sweep_cases():
        if n == 12:
            break
        L = int(np.prod(dims))
        H = oracle.hubbard_csc(list(dims), 1.0, u, nu, nd)
        if H.dim > 5000:
            continue
        n += 1
        E = np.linalg.eigvalsh(H.to_dense())
        emin, emax = float(E[0]), float(E[-1])
        if emax - emin < 1e-9:
            continue
        b = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
        op = mb.GpuHubbardOperator(b, mb._Hubbard(1.0, u, dims), prec)
        mu = mb.kpm_dos_moments(op, M, R, key, emin, emax, 0.01)
        a = (emax - emin) / 2 * 1.01
        c = (emax + emin) / 2
        perm = op.basis.permutation()
        ref = np.zeros(M)
        for p in range(R):
            rt = oracle.philox_phase(key, op.dimension(), 1 + p)
            r = np.empty_like(rt)
            r[perm] = rt
            ref += H.kpm_dos_moments(r, M, a, c)
        ref /= R * op.dimension()
        assert np.max(np.abs(mu - ref)) <= tol, (dims, nu, nd, u, float(np.max(np.abs(mu - ref))))
