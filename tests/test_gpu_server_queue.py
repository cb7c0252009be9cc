"""Continuous batching through the served GEMM's work queue.

A large emulated contraction is submitted, and a small one a moment later,
while the large one's units are on the GPU.  The small request's units go to
the lane the GEMM's clusters take first, so it must finish before the large
one; both results must equal the same contractions run alone, bit for bit
(every output block's sums follow a fixed order whichever cluster runs it).
"""
import time

import numpy as np
import pytest

from helpers import gpu_operand

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


def test_small_request_overtakes_large(ta, world):
    hl = uneven(8192, 96, 256, 41)      # ~0.5 TFLOP: tens of ms on the GPU
    hs = uneven(600, 40, 120, 42)
    Al, _ = gpu_operand(ta, world, [hl, hl], 41, 0, kind=0)
    Bl, _ = gpu_operand(ta, world, [hl, hl], 41, 1, kind=0)
    As, _ = gpu_operand(ta, world, [hs, hs], 42, 0, kind=0)
    Bs, _ = gpu_operand(ta, world, [hs, hs], 42, 1, kind=0)
    ref_l, _ = ta.contract(world, "i,j", 1.0, Al, "i,k", Bl, "k,j", precision=ta.PRECISION_OZAKI)
    ref_s, _ = ta.contract(world, "i,j", 1.0, As, "i,k", Bs, "k,j", precision=ta.PRECISION_OZAKI)
    srv = ta.Server(world, hbm_budget_bytes=32 << 30, precision=ta.PRECISION_OZAKI)
    try:
        # warm-up pair: the first request also creates the work queue
        w_id = srv.submit("i,j", 1.0, As, "i,k", Bs, "k,j")
        srv.wait(w_id, 60000)
        big = srv.submit("i,j", 1.0, Al, "i,k", Bl, "k,j")
        time.sleep(0.005)
        small = srv.submit("i,j", 1.0, As, "i,k", Bs, "k,j")
        Cs, rs = srv.wait(small, 60000)
        polled = srv.poll(big)            # the large one, if it is done already
        big_done_first = polled is not None
        Cl, rl = polled if polled is not None else srv.wait(big, 60000)
        assert rs["status"] == 0 and rl["status"] == 0
        assert not big_done_first, "the small request waited for the large one"
        assert rs["latency_ms"] < rl["latency_ms"]
        assert np.array_equal(Cs.download(), ref_s.download())
        assert np.array_equal(Cl.download(), ref_l.download())
        print(f"small {rs['latency_ms']:.2f} ms, large {rl['latency_ms']:.2f} ms, "
              f"in flight together {rs['batch_size']}")
    finally:
        srv.stop()
