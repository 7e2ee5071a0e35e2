"""mb_op_apply_noalloc, the entry point for callers that cannot let the
library allocate device memory (their framework owns all device memory, or
their loop cannot afford cudaMalloc's implicit synchronisation): it must give
the same result as mb_op_apply, call after call, from its fixed in-library
scratch array, and a call after the first must leave the device's free memory
unchanged.  Collected last so that a failure here leaves every other test
already run."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(mb, torch, op, x, y):
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = mb.lib().mb_op_apply_noalloc(op.handle, x.data_ptr(), y.data_ptr(), st)
    assert rc == mb.MB_OK, mb.lib().mb_last_error()
    torch.cuda.synchronize()


# FP64 and FP32 to their tolerances; Q64 takes the same steps as mb_op_apply
# on a Q64 operator, so the bits must agree (tolerance 0).
@pytest.mark.parametrize("prec,tol", [(0, 1e-13), (1, 2e-6), (2, 0.0)])
def test_noalloc_apply_matches_apply_twice(mb, cuda, prec, tol):
    torch = cuda
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(10, 10, 0)   # 63,504 states
    model = mb.HubbardModel(1.0, 4.0, 10)
    op = mb.GpuHubbardOperator(basis, model, prec)
    xs = [op.seed_vector(seed) for seed in (3, 4)]     # two calls in a row, different inputs
    refs = [op.apply(x) for x in xs]
    ys = [op.empty() for _ in xs]
    torch.cuda.synchronize()
    _noalloc(mb, torch, op, xs[0], ys[0])               # the first call sets up
    free0 = torch.cuda.mem_get_info()[0]
    _noalloc(mb, torch, op, xs[1], ys[1])
    assert torch.cuda.mem_get_info()[0] == free0, "a call after the first allocated device memory"
    for y, ref in zip(ys, refs):
        if tol == 0.0:
            assert torch.equal(y, ref)
        else:
            d = float(torch.linalg.norm((y - ref).to(torch.complex128)))
            assert d <= tol * float(torch.linalg.norm(ref.to(torch.complex128)))


def test_noalloc_rejects_oversized_sector(mb, cuda):
    basis = mb.FermionBasis.with_fixed_particle_number_and_spin(12, 12, 0)   # 853,776: fits
    op = mb.GpuHubbardOperator(basis, mb.HubbardModel(1.0, 4.0, 12))
    x = op.seed_vector(1)
    y = op.apply_noalloc(x)
    ref = op.apply(x)
    assert float(abs(y - ref).max()) <= 1e-13 * float(abs(ref).max())
    big = mb.FermionBasis.with_fixed_particle_number_and_spin(14, 12, 0)     # 9,018,009
    opb = mb.GpuHubbardOperator(big, mb.HubbardModel(1.0, 4.0, 14))
    xb = opb.seed_vector(1)
    with pytest.raises(mb.MbError) as e:
        opb.apply_noalloc(xb)
    assert e.value.status == mb.MB_ERR_CAPACITY
