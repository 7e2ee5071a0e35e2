"""Momentum-sector bases and the momentum-space model on the host
(BasisImpl::with_fixed_particle_number_spin_momentum, src/algebra/basis.cpp:
128-185,304-356; HubbardModelMomentum, src/algebra/fermion/model/
hubbard_model_momentum.h:19-180), against the reference's own outputs
(tests/golden/mom_*.npz from oracle/_ref/ref_dump --momentum): the keys in
reference order and the term count, bit-exact.
"""
import numpy as np
import pytest

import oracle
from conftest import load_golden, momentum_cases, momentum_full_cases


def make(mb, g):
    dims = [int(d) for d in g["dims"]]
    basis = mb.FermionBasis.with_fixed_particle_number_spin_momentum(
        int(np.prod(dims)), int(g["particles"]), int(g["spin_projection"]), dims,
        [int(k) for k in g["momentum"]])
    model = mb.HubbardModelMomentum(float(g["t"]), float(g["U"]), dims)
    return basis, model


@pytest.mark.parametrize("name", momentum_cases())
def test_momentum_basis_matches_reference(mb, name):
    g = load_golden(name)
    basis, model = make(mb, g)
    up, dn = basis.keys()
    assert basis.size() == len(g["up"])
    assert np.array_equal(up, g["up"].astype(np.uint64))
    assert np.array_equal(dn, g["down"].astype(np.uint64))
    for i in range(0, len(up), max(1, len(up) // 17)):
        assert basis.index_of(int(up[i]), int(dn[i])) == i
    assert np.array_equal(basis.permutation(), np.arange(len(up)))
    assert model.term_count() == int(g["n_terms"])


def test_momentum_sectors_partition_the_full_sector(mb):
    """The sectors K of one lattice are disjoint and cover the (N_up, N_down)
    sector, each in the full sector's relative order."""
    dims, n, sz = (3, 2), 4, 0
    full = mb.FermionBasis.with_fixed_particle_number_and_spin(6, n, sz)
    fu, fd = full.keys()
    seen = 0
    for kx in range(3):
        for ky in range(2):
            b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(6, n, sz, dims, (kx, ky))
            up, dn = b.keys()
            ranks = [full.index_of(int(u), int(d)) for u, d in zip(up, dn)]
            assert ranks == sorted(ranks)
            seen += len(ranks)
            with pytest.raises(mb.MbError):  # a state of another momentum is not in b
                other = next(i for i in range(len(fu)) if (fu[i], fd[i]) not in set(zip(up, dn)))
                b.index_of(int(fu[other]), int(fd[other]))
    assert seen == full.size()


def test_momentum_argument_checks(mb):
    with pytest.raises(mb.MbError):
        mb.FermionBasis.with_fixed_particle_number_spin_momentum(4, 2, 0, (4,), (4,))
    with pytest.raises(mb.MbError):
        mb.FermionBasis.with_fixed_particle_number_spin_momentum(4, 3, 0, (4,), (0,))
    with pytest.raises(ValueError):
        mb.FermionBasis.with_fixed_particle_number_spin_momentum(4, 2, 0, (2, 2), (0,))


@pytest.mark.parametrize("name", __import__("conftest").current_cases())
def test_current_operator_term_count(mb, name):
    g = load_golden(name)
    dims = [int(d) for d in g["dims"]]
    j = mb.CurrentOperator(float(g["t"]), dims, [int(q) for q in g["transfer"]], int(g["direction"]))
    assert j.term_count() == int(g["n_terms"])


@pytest.mark.parametrize("name", __import__("conftest").all_sz_cases())
def test_all_spin_projection_basis_matches_reference(mb, name):
    """with_fixed_particle_number (src/algebra/basis.cpp:69-89,248-266): keys in
    the reference's order, index_of, and the block permutation."""
    g = load_golden(name)
    L = int(np.prod([int(d) for d in g["dims"]]))
    b = mb.FermionBasis.with_fixed_particle_number(L, int(g["particles"]))
    up, dn = b.keys()
    assert b.size() == len(g["up"])
    assert np.array_equal(up, g["up"].astype(np.uint64))
    assert np.array_equal(dn, g["down"].astype(np.uint64))
    for i in range(0, len(up), max(1, len(up) // 13)):
        assert b.index_of(int(up[i]), int(dn[i])) == i
    perm = b.permutation()
    assert np.array_equal(np.sort(perm), np.arange(len(up)))


@pytest.mark.parametrize("name", momentum_full_cases())
def test_factorized_restatement_matches_reference_matrix(mb, name):
    """The oracle's restatement of HubbardMomentumFactorized (rho_q products
    with the (-1)^(op_idx + insert_pos) rule) equals the reference's
    compute_matrix_elements of HubbardModelMomentum on the whole basis (what
    the reference's own test asserts), and the basis is the real-space one."""
    g = load_golden(name)
    n = len(g["up"])
    H_ref = np.zeros((n, n))
    H_ref[g["row"], g["col"]] = g["val"]
    H = oracle.momentum_factorized_matrix(g["dims"], float(g["t"]), float(g["U"]), g["up"],
                                          g["down"])
    assert np.abs(H - H_ref).max() <= 1e-12 * max(1.0, np.abs(H_ref).max())
    L = int(np.prod(g["dims"]))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, int(g["particles"]),
                                                                int(g["spin_projection"]))
    up, dn = basis.keys()
    assert np.array_equal(up, g["up"].astype(np.uint64))
    assert np.array_equal(dn, g["down"].astype(np.uint64))
    model = mb.HubbardModelMomentum(float(g["t"]), float(g["U"]), [int(d) for d in g["dims"]])
    assert model.term_count() == int(g["n_terms"])
