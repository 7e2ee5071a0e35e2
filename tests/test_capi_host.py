"""Host-side logic of the C ABI (no GPU needed): library loads, exports every
symbol the header declares, basis order / index_of / permutation and model
term counts match the reference fixtures, invalid arguments are errors."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden_cases, load_golden


def header_symbols():
    src = open(os.path.join(ROOT, "include", "manybody_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mb_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(mb):
    names = header_symbols()
    assert len(names) >= 40
    L = C.CDLL(mb.LIB_PATH)
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(mb.SIGNATURES), set(names) ^ set(mb.SIGNATURES)


@pytest.mark.parametrize("name", golden_cases())
def test_basis_reference_order(mb, name):
    g = load_golden(name)
    n = int(g["particles"])
    sz = int(g["spin_projection"])
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(g["L"], n, sz)
    assert b.size() == len(g["up"])
    up, dn = b.keys()
    assert np.array_equal(up, g["up"]) and np.array_equal(dn, g["down"])
    # index_of(key_i) == i  (IndexedHashSet::index_of)
    for i in range(0, len(up), max(1, len(up) // 50)):
        assert b.index_of(int(up[i]), int(dn[i])) == i
    # permutation: tensor (colex up rank, colex down rank) -> reference index
    perm = b.permutation()
    assert np.array_equal(np.sort(perm), np.arange(len(perm)))
    sec = b.sector()
    assert sec["dim_up"] * sec["dim_down"] == b.size()


@pytest.mark.parametrize("name", golden_cases())
def test_model_term_count(mb, name):
    g = load_golden(name)
    m = mb._Hubbard(float(g["t"]), float(g["U"]), [int(d) for d in g["dims"]])
    assert m.term_count() == int(g["n_terms"])


def test_reference_term_counts(mb):
    # tests/algebra/test_model.cpp:58-74
    assert mb.HubbardModel(1.0, 2.0, 2).term_count() == 6
    assert mb.HubbardModel2D(1.0, 2.0, 2, 2).term_count() == 20
    assert mb.HubbardModel3D(1.0, 2.0, 2, 2, 2).term_count() == 56


def test_invalid_arguments_are_errors(mb):
    with pytest.raises(mb.MbError) as e:
        mb.FermionBasis.with_fixed_particle_number_and_spin(4, 3, 0)  # odd N + Sz
    assert e.value.status == mb.MB_ERR_INVALID_ARG
    with pytest.raises(mb.MbError):
        mb.FermionBasis.with_fixed_particle_number_and_spin(4, 10, 0)  # too many particles
    with pytest.raises(mb.MbError):
        mb.FermionBasis.with_fixed_particle_number_and_spin(4, 2, 4)   # |Sz| > N
    with pytest.raises(mb.MbError) as e:
        mb.FermionBasis.with_fixed_particle_number_and_spin(40, 2, 0)
    assert e.value.status == mb.MB_ERR_CAPACITY
    with pytest.raises(mb.MbError):
        mb.HubbardModel2D(1.0, 1.0, 0, 3)
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(4, 4, 0)
    with pytest.raises(mb.MbError):
        b.index_of(0b1, 0b11)  # wrong particle number: not in the basis
    assert not b.contains(0b111, 0b1)
    assert b.contains(0b11, 0b11)


def test_large_sector_sizes(mb):
    # 4x4, 6+6 and 1D L=16, 8+8 (the GPU workloads) are representable.
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 12, 0)
    assert b.size() == 8008 ** 2
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(16, 16, 0)
    assert b.size() == 12870 ** 2


def test_permutation_matches_closed_form_on_random_keys(mb):
    import oracle
    up, dn = oracle.basis(12, 5, 4)
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(12, 9, 1)
    rng = np.random.default_rng(0)
    for i in rng.integers(0, len(up), 200):
        assert b.index_of(int(up[i]), int(dn[i])) == i


def test_gpu_calls_fail_loudly_without_device(mb):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    b = mb.FermionBasis.with_fixed_particle_number_and_spin(4, 4, 0)
    m = mb.HubbardModel(1.0, 4.0, 4)
    with pytest.raises(mb.MbError) as e:
        mb.GpuHubbardOperator(b, m)
    assert e.value.status == mb.MB_ERR_NO_DEVICE


@pytest.mark.parametrize("L,nu,nd", [(12, 4, 4), (9, 3, 2), (8, 1, 4), (6, 0, 3), (5, 5, 2)])
def test_reference_order_leads_with_orbital_zero_up(mb, L, nu, nd):
    """The pipelined host-buffer apply returns the reference indices
    [0, C(L-1, N_up-1) * D_down) first: exactly the states whose up
    configuration holds orbital 0 (the operator (0, up) sorts first)."""
    from math import comb
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
    up, dn = basis.keys()
    n_a = (comb(L - 1, nu - 1) if nu > 0 else 0) * comb(L, nd)
    holds = (up & np.uint64(1)) != 0
    assert holds[:n_a].all() and not holds[n_a:].any()
    assert int(holds.sum()) == n_a


def test_model_parts_match_reference_term_counts(mb):
    """kinetic() / interaction() as models: their term counts add up to the
    hamiltonian's (the parts share no term) and the U = 0 / t = 0 golden
    sectors are their matrices' term counts."""
    for dims in ((8,), (2, 2), (3, 3), (2, 2, 2)):
        m = mb._Hubbard(1.0, 4.0, dims)
        assert m.kinetic().term_count() + m.interaction().term_count() == m.term_count()
        assert m.kinetic().u == 0.0 and m.interaction().t == 0.0
        assert type(m.kinetic()) is type(m) and m.hamiltonian() is m
    g = load_golden("chain4_n4_u0")
    assert mb.HubbardModel(float(g["t"]), 4.0, 4).kinetic().term_count() == int(g["n_terms"])
    mm = mb.HubbardModelMomentum(1.0, 3.0, [2])
    g = load_golden("mfull_chain2_n2_t0")
    assert mm.interaction().term_count() == int(g["n_terms"])


def test_rescaling_from_bounds(mb):
    """rescaling_from_bounds_* and rescale/inverse (test_rescaling.cpp:9-92), host side."""
    r = mb.rescaling_from_bounds(-3.0, 5.0, 0.0)
    assert r.a == 4.0 and r.b == 1.0
    assert r.rescale(-3.0) == -1.0 and r.rescale(5.0) == 1.0 and r.inverse(0.5) == 3.0
    for e in (-2.5, 0.0, 4.75):
        assert abs(r.inverse(r.rescale(e)) - e) < 1e-14
    rp = mb.rescaling_from_bounds(-3.0, 5.0, 0.1)
    assert abs(rp.a - 4.4) < 1e-14 and rp.b == 1.0
    assert -1.0 < rp.rescale(-3.0) < rp.rescale(5.0) < 1.0
