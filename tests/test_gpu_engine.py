"""Batched / served ground states (mb_engine_*): many sectors of uneven size
advanced together, complex64 vectors with FP64 alpha/beta, replay + FP64
Rayleigh-quotient refinement.

Tolerances: refined energies |dE0| <= 1e-8 |E0| (the batch and serving accuracy bar);
unrefined Ritz values <= 1e-5 |E0|; a request gives bit-identical results
alone and in any mix (per-request fixed-order reductions).
"""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SECTORS = [  # (dims, n_up, n_down, U)
    ((6,), 3, 3, 4.0),
    ((6,), 2, 2, 1.5),
    ((8,), 4, 4, 4.0),
    ((8,), 3, 3, 7.0),
    ((2, 3), 2, 2, 3.0),
    ((3, 3), 2, 2, 8.0),
    ((4,), 2, 2, 0.5),
    ((2, 4), 2, 1, 2.0),
]


def exact_e0(dims, nu, nd, u):
    H = oracle.hubbard_csc(list(dims), 1.0, u, nu, nd)
    return np.linalg.eigvalsh(H.to_dense())[0]


@pytest.fixture(scope="module")
def exact():
    return [exact_e0(*s) for s in SECTORS]


def descs(mb):
    return [mb.sector(d, nu, nd, 1.0, u) for d, nu, nd, u in SECTORS]


def test_batch_matches_exact(mb, cuda, exact):
    res = mb.batch_ground_states(descs(mb), seeds=list(range(len(SECTORS))), kmax=150)
    for r, e in zip(res, exact):
        assert r is not None
        assert abs(r.e0 - e) <= 1e-8 * abs(e), (r.e0, e)
        assert abs(r.e0_raw - e) <= 1e-5 * abs(e), (r.e0_raw, e)


def test_same_result_alone_and_in_mix(mb, cuda):
    d = descs(mb)
    mixed = mb.batch_ground_states(d, seeds=[7] * len(d), kmax=120, autotune=False)
    for i in (0, 2, 5):
        alone = mb.batch_ground_states([d[i]], seeds=[7], kmax=120, autotune=False)[0]
        assert alone.e0 == mixed[i].e0 and alone.e0_raw == mixed[i].e0_raw
        assert alone.steps == mixed[i].steps


def test_graph_and_eager_agree(mb, cuda):
    d = descs(mb)[:4]
    a = mb.batch_ground_states(d, kmax=100, use_graph=True, autotune=False)
    b = mb.batch_ground_states(d, kmax=100, use_graph=False, autotune=False)
    assert [x.e0 for x in a] == [x.e0 for x in b]


def test_continuous_admission_and_convergence(mb, cuda, exact):
    """Budget for ~2 requests: later ones are admitted as earlier ones retire;
    each stops on its own convergence test."""
    d = descs(mb)
    foot = max(mb.Engine.footprint(x) for x in d)
    eng = mb.Engine(device_bytes_budget=2 * foot + 1)
    pending = list(range(len(d)))
    ids = {}
    rounds = 0
    while pending or any(eng.poll(r) is None for r in ids.values()):
        while pending:
            rid = eng.try_submit(d[pending[0]], seed=3, kmax=300, rel_tol=1e-12)
            if rid is None:
                break
            ids[pending.pop(0)] = rid
        eng.step(5)
        rounds += 1
        assert rounds < 2000
    for i, rid in ids.items():
        r = eng.poll(rid)
        assert abs(r.e0 - exact[i]) <= 1e-8 * abs(exact[i])
        assert r.latency_s > 0
    assert len(ids) == len(d)


def test_autotune_picks_a_valid_shape(mb, cuda):
    eng = mb.Engine()
    for x in descs(mb):
        assert eng.try_submit(x, 1, 50) is not None
    w, ms = eng.autotune()
    assert w in (2, 4, 8, 16) and ms > 0
    eng.set_warps(4)
    with pytest.raises(mb.MbError):
        eng.set_warps(3)


def test_engine_rejects_bad_requests(mb, cuda):
    eng = mb.Engine()
    with pytest.raises(mb.MbError):
        eng.try_submit(mb.sector((6,), 3, 3, 1.0, 1.0), 0, 10000)  # kmax > 512
    with pytest.raises(mb.MbError):
        eng.try_submit(mb.sector((6,), 3, 3, 0.0, 1.0), 0, 10)     # t = 0


# Lattices with a size-1 dimension: the reference's HubbardModel2D/3D call
# hopping(i, i) along it (src/algebra/fermion/model/hubbard_model.h:61-129),
# a self bond that puts -2t n on the diagonal per spin (term counts pinned by
# tests/algebra/test_model.cpp:58-62).
SELF_SECTORS = [
    ((1,), 1, 1, 4.0),        # the golden single-site sectors: the self bonds
    ((1,), 1, 1, 3.0),        # cancel U = 4, or leave U - 4 = -1
    ((1, 4), 2, 2, 4.0),      # 1x4: a self bond on every site, a ring of four
    ((1, 4), 2, 1, 2.0),
    ((1, 2, 3), 2, 1, 3.0),   # size-1, size-2 (doubled bonds) and size-3 sides
]


@pytest.mark.parametrize("fused", [1 << 62, 1])
def test_size1_dimensions_batch(mb, cuda, fused):
    """Ground states of self-bond lattices through the batch path (grouped and
    fused applies) against the exact spectrum of the oracle's matrix and the
    single-operator FP64 solve."""
    exact = [exact_e0(*x) for x in SELF_SECTORS]
    d = [mb.sector(dd, nu, nd, 1.0, u) for dd, nu, nd, u in SELF_SECTORS]
    res = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=100, autotune=False,
                                 fused_threshold=fused)
    for (dd, nu, nd, u), r, e in zip(SELF_SECTORS, res, exact):
        assert abs(r.e0 - e) <= max(1e-8 * abs(e), 1e-12), (dd, r.e0, e)
        L = int(np.prod(dd))
        basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
        op = mb.GpuHubbardOperator(basis, mb._Hubbard(1.0, u, dd), mb.PREC_F64)
        single = mb.find_min_eigenpair(op, min(100, basis.size()), op.seed_vector(0),
                                       want_vector=False)
        assert abs(single.value - r.e0) <= max(1e-8 * abs(e), 1e-12), (dd, single.value, r.e0)


def test_size1_dimensions_serve_dos(mb, cuda):
    """A DOS request and a ground-state request on a 1x4 lattice served
    together: moments within 1e-4 of the oracle's FP64 moments with the same
    bounds and probes, the ground state within 1e-8."""
    eng = mb.Engine()
    dims, nu, nd, u = (1, 4), 2, 2, 4.0
    M, R = 64, 2
    rid = eng.try_submit_dos(mb.sector(dims, nu, nd, 1.0, u), n_moments=M, n_probes=R, seed=5)
    gid = eng.try_submit(mb.sector((1, 2, 3), 2, 1, 1.0, 3.0), seed=1, kmax=200, rel_tol=1e-12)
    while eng.step(4):
        pass
    mu, lo, hi, _ = eng.poll_dos(rid)
    H = oracle.hubbard_csc(list(dims), 1.0, u, nu, nd)
    E = np.linalg.eigvalsh(H.to_dense())
    assert lo <= E[0] + 1e-9 and hi >= E[-1] - 1e-9
    a = (hi - lo) / 2 * 1.01
    b = (hi + lo) / 2
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(4, nu + nd, nu - nd)
    perm = basis.permutation()
    ref = np.zeros(M)
    for p in range(R):
        rt = oracle.philox_phase(5, H.dim, 1 + p)
        r = np.empty_like(rt)
        r[perm] = rt
        ref += H.kpm_dos_moments(r, M, a, b)
    ref /= R * H.dim
    assert np.max(np.abs(mu - ref)) <= 1e-4
    e_exact = exact_e0((1, 2, 3), 2, 1, 3.0)
    assert abs(eng.poll(gid).e0 - e_exact) <= 1e-8 * abs(e_exact)


def test_dos_requests_match_oracle_and_mix_with_ground_states(mb, cuda):
    """KPM DOS requests (complex64 Chebyshev, FP64 moment sums) next to ground-
    state requests in one engine: moments within 1e-4 of the oracle's FP64
    moments with the same bounds and probes; spectrum inside the bounds."""
    eng = mb.Engine()
    d_dos = mb.sector((6,), 3, 3, 1.0, 4.0)
    d_gs = mb.sector((8,), 4, 4, 1.0, 4.0)
    M, R = 64, 2
    rid = eng.try_submit_dos(d_dos, n_moments=M, n_probes=R, seed=5)
    gid = eng.try_submit(d_gs, seed=1, kmax=200, rel_tol=1e-12)
    while eng.step(4):
        pass
    mu, lo, hi, lat = eng.poll_dos(rid)
    H = oracle.hubbard_csc([6], 1.0, 4.0, 3, 3)
    E = np.linalg.eigvalsh(H.to_dense())
    assert lo <= E[0] + 1e-9 and hi >= E[-1] - 1e-9          # bounds enclose the spectrum
    a = (hi - lo) / 2 * 1.01
    b = (hi + lo) / 2
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(6, 6, 0)
    perm = basis.permutation()
    ref = np.zeros(M)
    for p in range(R):
        rt = oracle.philox_phase(5, H.dim, 1 + p)
        r = np.empty_like(rt)
        r[perm] = rt
        ref += H.kpm_dos_moments(r, M, a, b)
    ref /= R * H.dim
    assert abs(mu[0] - 1.0) < 1e-6
    assert np.max(np.abs(mu - ref)) <= 1e-4
    g = eng.poll(gid)
    e_exact = exact_e0((8,), 4, 4, 4.0)
    assert abs(g.e0 - e_exact) <= 1e-8 * abs(e_exact)


@pytest.mark.parametrize("use_graph", [True, False])
def test_fused_apply_path_matches_grouped(mb, cuda, exact, use_graph):
    """Every request through the fused complex64 apply (threshold 1) against
    none (threshold above every sector): the same refined energies, and the
    fused path alone equals it in the mix bit for bit."""
    d = descs(mb)
    big = 1 << 62
    grouped = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=150, autotune=False,
                                     use_graph=use_graph, fused_threshold=big)
    fused = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=150, autotune=False,
                                   use_graph=use_graph, fused_threshold=1)
    for g, f, e in zip(grouped, fused, exact):
        assert abs(f.e0 - e) <= 1e-8 * abs(e), (f.e0, e)
        assert abs(f.e0 - g.e0) <= 1e-9 * abs(e)
        assert abs(f.e0_raw - e) <= 1e-5 * abs(e)
    alone = mb.batch_ground_states([d[3]], seeds=[3], kmax=150, autotune=False,
                                   use_graph=use_graph, fused_threshold=1)[0]
    assert alone.e0 == fused[3].e0 and alone.e0_raw == fused[3].e0_raw


def test_fused_dos_and_mid_run_switch(mb, cuda):
    """DOS moments through the fused apply match the grouped path's; switching
    the threshold while requests run keeps their progress."""
    res = []
    for thr in (1 << 62, 1):
        eng = mb.Engine()
        eng.set_fused_threshold(thr)
        rid = eng.try_submit_dos(mb.sector((8,), 4, 4, 1.0, 4.0), n_moments=64, n_probes=1, seed=9)
        while eng.step(4):
            pass
        res.append(eng.poll_dos(rid))
    (mu_g, lo_g, hi_g, _), (mu_f, lo_f, hi_f, _) = res
    assert abs(lo_f - lo_g) <= 1e-4 * abs(lo_g) and abs(hi_f - hi_g) <= 1e-4 * abs(hi_g)
    assert np.max(np.abs(mu_f - mu_g)) <= 1e-4
    eng = mb.Engine()
    gid = eng.try_submit(mb.sector((8,), 4, 4, 1.0, 4.0), seed=1, kmax=300, rel_tol=1e-12)
    eng.step(20)
    eng.set_fused_threshold(1)
    eng.step(20)
    eng.set_fused_threshold(1 << 62)
    while eng.step(10):
        pass
    e_exact = exact_e0((8,), 4, 4, 4.0)
    assert abs(eng.poll(gid).e0 - e_exact) <= 1e-8 * abs(e_exact)
    with pytest.raises(mb.MbError):
        eng.set_fused_threshold(0)


def test_completed_queue_and_stats(mb, cuda):
    """completed() hands back each finished request once, oldest first; the
    step statistics count the steps run."""
    eng = mb.Engine()
    ids = [eng.try_submit(x, seed=2, kmax=60) for x in descs(mb)[:4]]
    seen = []
    while eng.step(3):
        seen += eng.completed()
    seen += eng.completed()
    assert sorted(seen) == sorted(ids) and len(set(seen)) == len(seen)
    assert eng.completed() == []
    for rid in seen:
        assert eng.poll(rid) is not None
    steps, wall_ms, dev_ms = eng.stats()
    assert steps > 0 and wall_ms > 0 and 0 < dev_ms <= wall_ms


def test_persistent_step_matches_grouped_kernels(mb, cuda):
    """The persistent fused step (one cooperative launch per batch) and the
    grouped kernels give the same bits for every request applied warp per row
    or row-staged in both."""
    d = descs(mb)
    big = 1 << 62
    a = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=120, autotune=False,
                               fused_threshold=big, persistent=True)
    b = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=120, autotune=False,
                               fused_threshold=big, persistent=False)
    for x, y in zip(a, b):
        assert x.e0 == y.e0 and x.e0_raw == y.e0_raw and x.steps == y.steps


def test_persistent_launch_boundaries_keep_bits(mb, cuda):
    """Within a launch the persistent step defers each Lanczos step's
    normalisation to the next step, and a launch's last step normalises:
    a batch stepped in launches of 1, 7 and 3 steps, then the rest, gives the
    bits of the grouped kernels (every step its own launches), with and
    without kept bases."""
    d = descs(mb)
    kmax = 60
    for limit in (None, 0):
        ref = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=kmax, autotune=False,
                                     persistent=False, basis_limit=limit)
        eng = mb.Engine()
        if limit is not None:
            eng.set_basis_limit(limit)
        ids = [eng.try_submit(x, i, kmax, 0.0, True) for i, x in enumerate(d)]
        for n in (1, 7, 3):
            eng.step_fixed(n, n != 7)
        while eng.step_fixed(kmax, True):
            pass
        for rid, r in zip(ids, ref):
            got = eng.poll(rid)
            assert got.e0 == r.e0 and got.e0_raw == r.e0_raw and got.steps == r.steps


def test_same_result_alone_and_in_mix_large_request(mb, cuda):
    """A sector of more than a million states (1D L=13, 6+6: 2,944,656) through
    the persistent step's block-per-row path gets the same bits alone and in a
    mix with small requests, with and without graph capture."""
    big = mb.sector((13,), 6, 6, 1.0, 5.0)
    small = descs(mb)[:4]
    for use_graph in (True, False):
        mixed = mb.batch_ground_states(small + [big], seeds=[7] * 5, kmax=60, autotune=False,
                                       use_graph=use_graph)
        alone = mb.batch_ground_states([big], seeds=[7], kmax=60, autotune=False,
                                       use_graph=use_graph)[0]
        assert alone.e0 == mixed[4].e0 and alone.e0_raw == mixed[4].e0_raw
        assert alone.steps == mixed[4].steps


def test_persistent_barrier_timeout_returns_status(mb, cuda):
    """A grid-barrier wait of the persistent step that runs past its budget
    (a budget of 0 cycles: every block that waits gives up) ends the step with
    MB_ERR_TIMEOUT instead of hanging; the engine then refuses work, and a new
    engine on the same GPU solves normally."""
    eng = mb.Engine()
    for x in descs(mb)[:4]:
        assert eng.try_submit(x, seed=1, kmax=50) is not None
    eng.set_wait_budget(0)
    with pytest.raises(mb.MbError) as e:
        eng.step(3)
    assert e.value.status == mb.MB_ERR_TIMEOUT
    with pytest.raises(mb.MbError) as e:
        eng.step(1)
    assert e.value.status == mb.MB_ERR_TIMEOUT
    del eng
    d = descs(mb)[:2]
    res = mb.batch_ground_states(d, seeds=[0, 1], kmax=150, autotune=False)
    for r, (dims, nu, nd, u) in zip(res, SECTORS[:2]):
        ex = exact_e0(dims, nu, nd, u)
        assert abs(r.e0 - ex) <= 1e-8 * abs(ex)


def test_engine_autotune_persistent_shape(mb, cuda):
    eng = mb.Engine()
    for x in descs(mb):
        assert eng.try_submit(x, seed=2, kmax=80) is not None
    eng.autotune()
    sh = eng.shape()
    assert sh["persistent"] == 1 and sh["row_min_cols"] in (64, 128, 256)
    assert sh["ctas_per_sm"] in (0, 1, 2) and sh["grid"] >= 1
    while eng.step(10):
        pass


@pytest.mark.parametrize("persistent", [True, False])
def test_kept_basis_matches_replay(mb, cuda, persistent):
    """A request that keeps its pass-one Lanczos vectors sums its Ritz vector
    from them in the replay's order and arithmetic: the same bits as the
    replayed recurrence, on both step paths."""
    d = descs(mb)
    kept = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=120, autotune=False,
                                  persistent=persistent)
    replay = mb.batch_ground_states(d, seeds=list(range(len(d))), kmax=120, autotune=False,
                                    persistent=persistent, basis_limit=0)
    for a, b in zip(kept, replay):
        assert a.e0 == b.e0 and a.e0_raw == b.e0_raw and a.steps == b.steps


def test_refinement_far_from_zero_in_engine(mb, cuda):
    """A served request whose refinement needs the second Gram-Schmidt pass:
    1D L=14, N_up = N_down = 13, U = 9.24, seed 44 (E0 ~ 107, start vector
    close to an eigenvector).  Alone and beside the other sectors, every
    refined energy within 1e-8."""
    u = 9.240847688353895
    far = mb.sector((14,), 13, 13, 1.0, u)
    e_far = exact_e0((14,), 13, 13, u)
    eng = mb.Engine()  # as served: stop at Ritz stability 1e-10, then refine
    rid = eng.try_submit(far, seed=44, kmax=400, rel_tol=1e-10, refine=True)
    for _ in range(1000):
        eng.step(1)
        if rid in eng.completed():
            break
    served = eng.poll(rid)
    assert abs(served.e0 - e_far) <= 1e-8 * abs(e_far)
    alone = mb.batch_ground_states([far], seeds=[44], kmax=150, autotune=False)[0]
    assert abs(alone.e0 - e_far) <= 1e-8 * abs(e_far)
    mixed = mb.batch_ground_states([far] + descs(mb), seeds=[44] * 9, kmax=150, autotune=False)
    for r, e in zip(mixed, [e_far] + [exact_e0(*x) for x in SECTORS]):
        assert abs(r.e0 - e) <= 1e-8 * abs(e)


def test_engine_reused_across_batches(mb, cuda, exact):
    """A second batch on the same engine (its memory pool and sector tables
    warm from the first) gives the first batch's bits."""
    eng = mb.Engine()
    first = mb.batch_ground_states(descs(mb), seeds=list(range(8)), kmax=80, engine=eng)
    second = mb.batch_ground_states(descs(mb), seeds=list(range(8)), kmax=80, engine=eng)
    for a, b, e in zip(first, second, exact):
        assert a.e0 == b.e0 and a.e0_raw == b.e0_raw and a.steps == b.steps
        assert abs(a.e0 - e) <= 1e-8 * abs(e)
