"""The k-phase schedule (TAGPU_KPHASE=1): every unit's k list starts at the
k block its start time points to in the default schedule, so the clusters of
a wave walk the same k blocks together.

The exact levels (2..5) are integer sums and do not depend on the order of
the k blocks; the two lowest-weight levels sum in fp32 over the whole output
block, so their rounding (below 2^-41 of sum_k |a b| per element) follows the
order.  Results therefore match the default schedule to well below the FP64
error of either, and both match the oracle within 1e-12.
"""
import numpy as np
import pytest

from helpers import gpu_operand, oracle_operand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


def uneven(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    h = [0]
    while h[-1] < n:
        h.append(min(n, h[-1] + int(rng.integers(lo, hi + 1))))
    return h


def _contract(ta, world, monkeypatch, kphase, *args):
    monkeypatch.setenv("TAGPU_KPHASE", "1" if kphase else "0")
    C, st = ta.contract(world, *args, precision=ta.PRECISION_OZAKI)
    return C


def test_kphase_blocksparse(oracle, ta, world, monkeypatch):
    h = uneven(3000, 48, 256, 21)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / 4.0)
    A, _ = gpu_operand(ta, world, [h, h], 21, 0, kind=0, tile_scale=scale)
    B, _ = gpu_operand(ta, world, [h, h], 21, 1, kind=0, tile_scale=scale)
    x = _contract(ta, world, monkeypatch, False, "i,j", 1.0, A, "i,k", B, "k,j")
    y = _contract(ta, world, monkeypatch, True, "i,j", 1.0, A, "i,k", B, "k,j")
    gx, gy = x.to_dense(x.trange), y.to_dense(y.trange)
    Ao = oracle_operand(oracle, [h, h], 21, 0, kind=0, tile_scale=scale)
    Bo = oracle_operand(oracle, [h, h], 21, 1, kind=0, tile_scale=scale)
    ref = oracle.contract("i,j", Ao, "i,k", Bo, "k,j").to_dense()
    rn = np.linalg.norm(ref)
    assert np.linalg.norm(gx - gy) / rn <= 1e-15
    assert np.linalg.norm(gy - ref) / rn <= 1e-12
    assert np.array_equal(x.norms(), y.norms())


def test_kphase_general_product(oracle, ta, world, monkeypatch):
    # c("b,i,k") = a("b,i,j") * b("b,j,k"): one GEMM plan per fused element
    hb = [0, 2, 5]
    hi = uneven(300, 40, 90, 5)
    hj = uneven(400, 40, 90, 6)
    hk = uneven(350, 40, 90, 7)
    A, _ = gpu_operand(ta, world, [hb, hi, hj], 8, 0, kind=0)
    B, _ = gpu_operand(ta, world, [hb, hj, hk], 8, 1, kind=0)
    x = _contract(ta, world, monkeypatch, False, "b,i,k", 1.0, A, "b,i,j", B, "b,j,k")
    y = _contract(ta, world, monkeypatch, True, "b,i,k", 1.0, A, "b,i,j", B, "b,j,k")
    gx, gy = x.to_dense(x.trange), y.to_dense(y.trange)
    Ao = oracle_operand(oracle, [hb, hi, hj], 8, 0, kind=0)
    Bo = oracle_operand(oracle, [hb, hj, hk], 8, 1, kind=0)
    ref = oracle.general_contract("b,i,k", Ao, "b,i,j", Bo, "b,j,k").to_dense()
    rn = np.linalg.norm(ref)
    assert np.linalg.norm(gx - gy) / rn <= 1e-15
    assert np.linalg.norm(gy - ref) / rn <= 1e-12
