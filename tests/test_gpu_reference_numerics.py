"""The reference's generic numerics checks (tests/numerics/test_lanczos.cpp,
test_kpm.cpp, test_linear_operator.cpp) restated on the GPU drivers, with the
small matrices given to GpuSparseOperator (SparseComplexMatrixOperator on the
device).  Same matrices, the same properties and the same tolerances as the
reference's own tests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def csr(mb, A):
    import scipy.sparse as sp
    M = sp.csr_matrix(np.asarray(A, np.complex128))
    M.sort_indices()
    return mb.CsrMatrix(M.shape[0], M.indptr.astype(np.int64), M.indices.astype(np.int64),
                        M.data.astype(np.complex128))


def op_of(mb, A):
    return mb.GpuSparseOperator(csr(mb, A))


def tridiag_solve(a, b):
    T = np.diag(a) + np.diag(b, 1) + np.diag(b, -1)
    e1 = np.zeros(len(a))
    e1[0] = 1.0
    return np.linalg.solve(T, e1)


def test_extreme_eigenpairs_of_a_diagonal(mb, cuda):
    """lanczos_max/min_eigenpair_matches_diagonal (test_lanczos.cpp:54-71)."""
    torch = cuda
    op = op_of(mb, np.diag([1.0, 3.0, -2.0]))
    seed = torch.tensor([0.3 + 0.1j, 0.5 - 0.2j, 0.7 + 0.4j], dtype=torch.complex128, device="cuda")
    top = mb.find_max_eigenpair(op, 3, seed)
    assert abs(top.value - 3.0) < 1e-6
    v = top.vector
    hv = op.apply(v)
    rq = (torch.vdot(v, hv) / torch.vdot(v, v)).real.item()
    assert abs(rq - top.value) < 1e-6
    assert abs(mb.find_min_eigenpair(op, 3, seed).value + 2.0) < 1e-6


def test_decomposition_tracks_steps_and_norm(mb, cuda):
    """lanczos_decomposition_tracks_steps_and_norm (test_lanczos.cpp:166-185)."""
    torch = cuda
    A = np.diag(np.full(6, 4.0)) + np.diag(np.ones(5), 1) + np.diag(np.ones(5), -1)
    op = op_of(mb, A)
    b = torch.ones(6, dtype=torch.complex128, device="cuda")
    d = mb.lanczos_pass_one(op, b, 5)
    assert 0 < d.steps_taken <= 5
    assert len(d.alphas) == d.steps_taken and len(d.betas) + 1 == d.steps_taken
    assert abs(d.b_norm - np.sqrt(6.0)) < 1e-12
    assert all(beta > 0.0 for beta in d.betas)


def test_inverse_approximation_improves_with_k(mb, cuda):
    """lanczos_inverse_approximation_improves_with_k (test_lanczos.cpp:136-164):
    solve(op, b, k, tridiagonal solver) approaches A^-1 b as k grows."""
    torch = cuda
    A = np.diag([10.0, 8.0, 6.0, 5.0]) + np.diag([1.0, 1.0, 1.0], 1) + np.diag([1.0, 1.0, 1.0], -1)
    b = np.ones(4)
    exact = np.linalg.solve(A, b)
    op = op_of(mb, A)
    errs = []
    for k in (2, 3, 4):
        x = mb.solve(op, torch.tensor(b + 0j, device="cuda"), k, tridiag_solve).cpu().numpy()
        errs.append(np.linalg.norm(x - exact) / np.linalg.norm(exact))
    assert errs[1] <= errs[0] and errs[2] <= errs[1] and errs[2] < 1e-10


def test_max_eigenpair_of_a_nearest_neighbour_chain(mb, cuda):
    """lanczos_max_eigenpair_matches_nearest_neighbor_chain (test_lanczos.cpp:221-236):
    n = 80, diagonal 2, hopping -1, 50 steps, within 2e-2 of the exact top."""
    n, diag, hop = 80, 2.0, -1.0
    A = np.diag(np.full(n, diag)) + np.diag(np.full(n - 1, hop), 1) + np.diag(np.full(n - 1, hop), -1)
    op = op_of(mb, A)
    top = mb.find_max_eigenpair(op, 50, want_vector=False).value
    exact = diag + 2.0 * hop * np.cos(n * np.pi / (n + 1.0))
    assert abs(top - exact) < 2e-2


def projector_matrix(mb, torch, A, order, e_fermi):
    """The KPM projector's matrix, column by column from unit vectors."""
    op = op_of(mb, A)
    E = np.linalg.eigvalsh(A)
    P = mb.SparseKPMProjector(op, order, float(E[0]), float(E[-1]), e_fermi)
    n = A.shape[0]
    cols = []
    for i in range(n):
        e = torch.zeros(n, dtype=torch.complex128, device="cuda")
        e[i] = 1.0
        cols.append(P.apply(e).cpu().numpy())
    return np.array(cols).T


def test_kpm_projector_reproduces_the_exact_projector(mb, cuda):
    """kpm_projector_reproduces_exact_projector (test_kpm.cpp:74-101)."""
    A = np.diag([-2.0, -0.5, 0.5, 2.0])
    A[0, 1] = A[1, 0] = A[2, 3] = A[3, 2] = 0.1
    E, V = np.linalg.eigh(A)
    P_exact = sum(np.outer(V[:, i], V[:, i]) for i in range(4) if E[i] < 0.0)
    P = projector_matrix(mb, cuda, A, 200, 0.0)
    assert np.linalg.norm(P - P_exact) < 1e-2


def test_kpm_projector_is_idempotent_and_counts_states(mb, cuda):
    """kpm_projector_idempotent and kpm_projector_trace_counts_states
    (test_kpm.cpp:123-146)."""
    P = projector_matrix(mb, cuda, np.diag([-1.5, -0.5, 0.5, 1.5]), 200, 0.0)
    assert np.linalg.norm(P @ P - P) < 0.1
    P6 = projector_matrix(mb, cuda, np.diag([-2.0, -1.0, -0.5, 0.5, 1.0, 2.0]), 200, 0.0)
    assert abs(np.trace(P6).real - 3.0) < 0.1


def test_estimate_bounds_of_a_diagonal_spectrum(mb, cuda):
    """linear_operator_estimate_bounds_matches_diagonal_spectrum
    (test_linear_operator.cpp:137-144): 40 power iterations, padding 0.2."""
    lo, hi = mb.estimate_bounds(op_of(mb, np.diag([-2.0, 0.5, 4.0])), 40, 0.2)
    assert abs(lo + 2.0) < 1e-3 and abs(hi - 4.0) < 1e-3


def test_vectors_of_the_wrong_type_or_size_are_refused(mb, cuda):
    """A complex64 or short vector given to a complex128 operator is an error
    in the Python layer, before the library touches it."""
    torch = cuda
    op = op_of(mb, np.diag([1.0, 3.0, -2.0]))
    bad = [torch.ones(3, dtype=torch.complex64, device="cuda"),
           torch.ones(2, dtype=torch.complex128, device="cuda"),
           torch.ones(3, dtype=torch.complex128)]
    for v in bad:
        with pytest.raises(mb.MbError) as e:
            op.apply(v)
        assert e.value.status == mb.MB_ERR_INVALID_ARG
        with pytest.raises(mb.MbError):
            mb.find_min_eigenpair(op, 3, v)


def exact_evolution(A, psi, t, imaginary=False):
    E, V = np.linalg.eigh(A)
    f = np.exp(-t * E) if imaginary else np.exp(-1j * t * E)
    return V @ (f * (V.conj().T @ psi))


def test_stepped_evolution_with_callback_matches_exact(mb, cuda):
    """time_evolve_state_steps_calls_callback_and_matches_exact_expm
    (test_evolve_state.cpp:67-98): 2x2 diagonal, 2 Krylov steps, t 0 -> 0.3 by
    0.1: four callbacks from t0 to t1, state within 1e-8 of exp(-i t H)."""
    torch = cuda
    A = np.diag([0.5, 1.5])
    op = op_of(mb, A)
    psi0 = np.array([0.3 - 0.4j, 0.2 + 0.1j])
    psi = torch.tensor(psi0, dtype=torch.complex128, device="cuda")
    times = []
    mb.time_evolve_state_steps(op, psi, 0.0, 0.3, 0.1, krylov_steps=2,
                               callback=lambda t, v: times.append(t))
    assert len(times) == 4 and abs(times[0]) < 1e-12 and abs(times[-1] - 0.3) < 1e-12
    ref = exact_evolution(A, psi0, 0.3)
    assert np.linalg.norm(psi.cpu().numpy() - ref) / np.linalg.norm(ref) < 1e-8
    # the library's own loop, no callback (time_evolve_state_steps_matches_exact_expm)
    A2 = np.diag([1.0, 2.0])
    p2 = torch.tensor([1.0, 1j], dtype=torch.complex128, device="cuda")
    mb.time_evolve_state_steps(op_of(mb, A2), p2, 0.0, 0.3, 0.1, krylov_steps=2)
    ref2 = exact_evolution(A2, np.array([1.0, 1j]), 0.3)
    assert np.linalg.norm(p2.cpu().numpy() - ref2) / np.linalg.norm(ref2) < 1e-8


def test_imaginary_time_evolution_matches_exact(mb, cuda):
    """imaginary_time_evolve_state_matches_exact_expm (test_evolve_state.cpp:100-121)."""
    torch = cuda
    A = np.diag([0.2, 1.1])
    psi0 = np.array([0.6 + 0.1j, -0.3 + 0.2j])
    y = mb.imaginary_time_evolve_state(op_of(mb, A), torch.tensor(psi0, device="cuda"), 0.7,
                                       krylov_steps=2).cpu().numpy()
    ref = exact_evolution(A, psi0, 0.7, imaginary=True)
    assert np.linalg.norm(y - ref) / np.linalg.norm(ref) < 1e-8


def test_lanczos_exp_solver_matches_direct_expm(mb, cuda):
    """lanczos_exp_solver_matches_direct_expm (test_lanczos.cpp:104-134): solve()
    with y = exp(T) e1 over the full Krylov space is exp(A) b."""
    torch = cuda
    rng = np.random.default_rng(2)
    M = rng.normal(size=(5, 5))
    A = (M + M.T) / 4.0
    b = rng.normal(size=5)

    def exp_solver(a, be):
        T = np.diag(a) + np.diag(be, 1) + np.diag(be, -1)
        E, V = np.linalg.eigh(T)
        return V @ (np.exp(E) * V[0])

    x = mb.solve(op_of(mb, A), torch.tensor(b + 0j, device="cuda"), 5, exp_solver).cpu().numpy()
    E, V = np.linalg.eigh(A)
    ref = V @ (np.exp(E) * (V.T @ b))
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-8


def test_kpm_projector_apply_matches_its_matrix(mb, cuda):
    """kpm_projector_apply_matches_matrix (test_kpm.cpp:103-121): a 6-site chain."""
    torch = cuda
    A = -(np.diag(np.ones(5), 1) + np.diag(np.ones(5), -1))
    P = projector_matrix(mb, torch, A, 100, 0.0)
    v = np.random.default_rng(6).normal(size=6)
    E = np.linalg.eigvalsh(A)
    proj = mb.SparseKPMProjector(op_of(mb, A), 100, float(E[0]), float(E[-1]), 0.0)
    pv = proj.apply(torch.tensor(v + 0j, device="cuda")).cpu().numpy()
    assert np.linalg.norm(P @ v - pv) < 1e-10

