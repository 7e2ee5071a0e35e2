"""Kernel shapes of the lattice apply and the autotuner that picks them
(mb_op_set_apply_shape, mb_op_autotune).  Every shape of an MB_PREC_Q64
operator gives the same bits (its hop sums are exact integers in any order):
checked on the device apply, the reference-order host-buffer apply and a
Lanczos solve; the FP64/FP32 prefetch switch changes no arithmetic either."""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Q_SHAPES = [dict(passes=p, row_split=s, table_bits=t, prefetch=f, table_stage=0, csr_lanes=0)
            for p, s, t, f in itertools.product((1, 2), (1, 2, 4), (32, 16), (0, 1))]
Q_SHAPES += [dict(passes=1, row_split=s, table_bits=32, prefetch=f, table_stage=1, csr_lanes=0)
             for s, f in itertools.product((1, 2, 4), (0, 1))]


def make(mb, dims, nu, nd, u, prec):
    L = int(np.prod(dims))
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(L, nu + nd, nu - nd)
    return mb.GpuHubbardOperator(basis, mb._Hubbard(1.0, u, dims), prec)


@pytest.mark.parametrize("dims,nu,nd", [((4, 4), 4, 4), ((12,), 6, 5), ((2, 4), 3, 2)])
def test_q64_shapes_give_identical_bits(mb, cuda, dims, nu, nd):
    torch = cuda
    op = make(mb, dims, nu, nd, 6.0, mb.PREC_Q64)
    x = op.seed_vector(0)
    xq, ex = op.q64_from_f64(x, order=mb.ORDER_TENSOR)
    xh = x.cpu().numpy()
    ref_q = ref_y = ref_h = None
    for sh in Q_SHAPES:
        op.set_apply_shape(**sh)
        assert op.apply_shape() == sh
        yq, ey = op.apply_q64(xq, ex)
        y = op.apply(x)
        yh = np.empty_like(xh)
        op.apply_host(xh, yh)
        if ref_q is None:
            ref_q, ref_e, ref_y, ref_h = yq.clone(), ey, y.clone(), yh.copy()
            continue
        assert ey == ref_e and torch.equal(yq, ref_q), sh
        assert torch.equal(y, ref_y), sh
        assert np.array_equal(yh, ref_h), sh


def test_q64_lanczos_same_bits_in_every_pass_count(mb, cuda):
    op = make(mb, (3, 4), 4, 4, 8.0, mb.PREC_Q64)
    x = op.seed_vector(0)
    e = []
    for sh in (dict(passes=1), dict(passes=2), dict(table_stage=1)):
        op.set_apply_shape(**sh)
        e.append(mb.find_min_eigenpair(op, 120, x, want_vector=False).value)
    assert e[0] == e[1] == e[2]


@pytest.mark.parametrize("prec", [0, 1])
def test_prefetch_switch_keeps_fp_bits(mb, cuda, prec):
    torch = cuda
    op = make(mb, (4, 4), 4, 4, 4.0, prec)
    x = op.seed_vector(1)
    op.set_apply_shape(prefetch=0)
    a = op.apply(x)
    op.set_apply_shape(prefetch=1)
    b = op.apply(x)
    assert torch.equal(a, b)
    with pytest.raises(mb.MbError):
        op.set_apply_shape(passes=2)          # two passes: Q64 only
    with pytest.raises(mb.MbError):
        op.set_apply_shape(row_split=3)
    with pytest.raises(mb.MbError):
        op.set_apply_shape(csr_lanes=8)       # lanes a row: sparse-matrix operators only


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_autotune_picks_a_valid_shape_and_caches_it(mb, cuda, prec):
    torch = cuda
    op = make(mb, (4, 4), 5, 4, 8.0, prec)
    x = op.seed_vector(2)
    op.set_apply_shape()
    y0 = op.apply(x)
    shape, ms = op.autotune()
    assert ms > 0 and shape == op.apply_shape()
    y1 = op.apply(x)
    if prec == 2:
        assert torch.equal(y0, y1)
    else:
        assert float(torch.linalg.norm((y1 - y0).to(torch.complex128))) <= (
            2e-6 if prec == 1 else 1e-13) * float(torch.linalg.norm(y0.to(torch.complex128)))
    # a second operator of the same sector takes the cached choice
    op2 = make(mb, (4, 4), 5, 4, 3.0, prec)
    shape2, ms2 = op2.autotune()
    assert shape2 == shape and ms2 == ms


def momentum_op(mb, prec):
    dims = [4, 4]
    b = mb.FermionBasis.with_fixed_particle_number_spin_momentum(16, 6, 0, dims, (1, 0))
    return mb.GpuHubbardOperator(b, mb.HubbardModelMomentum(1.0, 6.0, dims), prec)


@pytest.mark.parametrize("prec,tol", [(0, 1e-14), (1, 1e-6), (2, 0.0)])
def test_csr_lanes_shapes(mb, cuda, prec, tol):
    """A momentum sector (4x4, 3+3, K = (1,0)) applied with 4, 8, 16 and 32
    lanes a row: the Q64 operator's integer row sums give the same bits at
    every width; the floating-point ones differ only in the order of the
    lanes' final additions.  The autotuner picks one of them and caches it
    per sector."""
    torch = cuda
    op = momentum_op(mb, prec)
    x = op.seed_vector(3)
    ref = None
    for lanes in (4, 8, 16, 32):
        op.set_apply_shape(csr_lanes=lanes)
        assert op.apply_shape()["csr_lanes"] == lanes
        y = op.apply(x)
        if ref is None:
            ref = y.clone()
        elif tol == 0.0:
            assert torch.equal(y, ref), lanes
        else:
            d = float(torch.linalg.norm((y - ref).to(torch.complex128)))
            assert d <= tol * float(torch.linalg.norm(ref.to(torch.complex128))), lanes
    with pytest.raises(mb.MbError):
        op.set_apply_shape(csr_lanes=12)
    op.set_apply_shape()
    shape, ms = op.autotune()
    assert ms > 0 and shape["csr_lanes"] in (4, 8, 16, 32) and shape == op.apply_shape()
    shape2, ms2 = momentum_op(mb, prec).autotune()
    assert shape2 == shape and ms2 == ms
