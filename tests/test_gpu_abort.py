"""The GEMMs' bounded waits: a wait that runs out aborts the launch cleanly
and the call returns TAGPU_ERR_TIMEOUT.

Made on purpose by a 1 ns bound (tagpu_set_wait_limit) on a contraction
large enough that its pipeline waits (loads, drains) take microseconds: a
wait gives up, the roles abort, copies and MMAs in flight finish, tensor
memory is released.  The same context then runs a normal contraction,
whose result must still be right.  No fault is involved: every wait is one
that would have completed.
"""
import numpy as np
import pytest

from helpers import gpu_operand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


def test_wait_limit_abort_then_recover(ta, world):
    h = [0] + [128 * (i + 1) for i in range(32)]          # 4096, tiles of 128
    A, _ = gpu_operand(ta, world, [h, h], 3, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 3, 1, kind=0)
    world.set_wait_limit(1e-9)
    try:
        with pytest.raises(ta.TAGPUError) as ei:
            ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
        assert ei.value.status == 5        # TAGPU_ERR_TIMEOUT
        assert "bounded wait" in str(ei.value)
    finally:
        world.set_wait_limit(4.0)
    C, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    Cp, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    x, y = C.to_dense(C.trange), Cp.to_dense(Cp.trange)
    assert np.linalg.norm(x - y) / np.linalg.norm(y) <= 1e-12


def test_wait_limit_abort_plain_then_recover(ta, world):
    """The plain FP64 GEMM's stage waits (bulk copies completing on an
    mbarrier) are bounded by the same limit: a 1 ns bound aborts the launch,
    the call returns TAGPU_ERR_TIMEOUT, and the context runs on."""
    h = [0] + [128 * (i + 1) for i in range(16)]          # 2048, tiles of 128
    A, _ = gpu_operand(ta, world, [h, h], 5, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 5, 1, kind=0)
    world.set_wait_limit(1e-9)
    try:
        with pytest.raises(ta.TAGPUError) as ei:
            ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_FP64)
        assert ei.value.status == 5
        assert "bounded" in str(ei.value)
    finally:
        world.set_wait_limit(4.0)
    C, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_FP64)
    x = C.to_dense(C.trange)
    a, b = A.to_dense(A.trange), B.to_dense(B.trange)
    ref = a @ b
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) <= 1e-13


def test_wait_limit_rejects_bad_values(ta, world):
    for bad in (0.0, -1.0, 1e9):
        with pytest.raises(ta.TAGPUError):
            world.set_wait_limit(bad)
