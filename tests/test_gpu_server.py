"""Serving: continuous batching gives every request the same result it gets
alone, admission rejects requests whose footprint bound exceeds the budget,
and several host threads may submit at once."""
import threading

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


def make_requests(ta, world, count, seed=0):
    """Mixed sizes and forms (matrix products of several sizes, a 4-index
    contraction), both precisions."""
    rng = np.random.default_rng(seed)
    reqs = []
    for x in range(count):
        kind = x % 3
        if kind < 2:
            n = int(rng.integers(150, 700))
            h = uneven(n, 32, 128, 100 + x)
            A, _ = gpu_operand(ta, world, [h, h], 31, 2 * x, kind=0)
            B, _ = gpu_operand(ta, world, [h, h], 31, 2 * x + 1, kind=0)
            reqs.append(("i,j", 1.0, A, "i,k", B, "k,j",
                         ta.PRECISION_OZAKI if kind == 0 else ta.PRECISION_FP64))
        else:
            h1, h2 = uneven(40, 8, 24, x), uneven(30, 6, 16, x + 1)
            A, _ = gpu_operand(ta, world, [h1, h1, h2, h2], 31, 2 * x, kind=0)
            B, _ = gpu_operand(ta, world, [h2, h2, h1, h1], 31, 2 * x + 1, kind=0)
            reqs.append(("a,b,i,j", 0.5, A, "a,b,c,d", B, "c,d,i,j", ta.PRECISION_OZAKI))
    return reqs


def test_server_results_match_alone(ta, world):
    reqs = make_requests(ta, world, 12)
    alone = []
    for c, al, A, a, B, b, prec in reqs:
        C, _ = ta.contract(world, c, al, A, a, B, b, precision=prec)
        alone.append(C.download())
    srv = ta.Server(world, hbm_budget_bytes=8 << 30, max_batch=8)
    ids = [srv.submit(c, al, A, a, B, b, precision=prec) for c, al, A, a, B, b, prec in reqs]
    sizes = set()
    for rid, ref in zip(ids, alone):
        C, res = srv.wait(rid, 60000)
        assert res["status"] == 0
        sizes.add(res["batch_size"])
        assert np.array_equal(C.download(), ref)   # bit-identical: fixed per-tile order
    st = srv.stats()
    srv.stop()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    assert max(sizes) > 1, "requests were never batched together"


def test_server_rejects_by_footprint(ta, world):
    h = uneven(2000, 100, 256, 5)
    A, _ = gpu_operand(ta, world, [h, h], 1, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 1, 1, kind=0)
    srv = ta.Server(world, hbm_budget_bytes=1 << 20)
    with pytest.raises(ta.TAGPUError) as e:
        srv.submit("i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    assert e.value.status == 6
    st = srv.stats()
    srv.stop()
    assert st["rejected"] == 1 and st["submitted"] == 1


def test_unwritten_array_holds_no_storage(ta, world):
    """An array is only given device memory when written or read: a 4-index
    operand of 400^4 elements (205 GB stored, 358 GB of digit bricks) is
    created without allocating, refused by admission, and a small unwritten
    array reads as zero tiles."""
    hv, ho = list(range(0, 401, 50)), [0, 16, 32]
    V = ta.DistArray(world, ta.TiledRange([hv, hv, hv, hv]))
    T = ta.DistArray(world, ta.TiledRange([hv, hv, ho, ho]))
    srv = ta.Server(world, hbm_budget_bytes=150 << 30)
    with pytest.raises(ta.TAGPUError) as e:
        srv.submit("a,b,i,j", 1.0, V, "a,b,c,d", T, "c,d,i,j", precision=ta.PRECISION_OZAKI)
    assert e.value.status == 6
    srv.stop()
    small = ta.DistArray(world, ta.TiledRange([[0, 30, 70], [0, 50]]))
    assert np.array_equal(small.download(), np.zeros(70 * 50))


def test_server_concurrent_submitters(ta, world):
    reqs = make_requests(ta, world, 9, seed=3)
    alone = [ta.contract(world, c, al, A, a, B, b, precision=p)[0].download()
             for c, al, A, a, B, b, p in reqs]
    srv = ta.Server(world, hbm_budget_bytes=4 << 30, max_batch=4)
    ids = [None] * len(reqs)

    def worker(k):
        for x in range(k, len(reqs), 3):
            c, al, A, a, B, b, p = reqs[x]
            ids[x] = srv.submit(c, al, A, a, B, b, precision=p)

    th = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for rid, ref in zip(ids, alone):
        C, res = srv.wait(rid, 60000)
        assert res["status"] == 0
        assert np.array_equal(C.download(), ref)
    srv.stop()


def test_server_results_held_count_against_budget(ta, world):
    """A finished result stays in HBM until its client takes it, so it keeps
    its bytes of the admission budget until then (requests wait in the queue
    rather than fail for memory while results pile up): with nothing taken,
    the server's bytes in use after all requests finished are exactly the
    results' bytes, and zero once the client has taken them."""
    import time
    h = uneven(1200, 64, 200, 9)
    A, _ = gpu_operand(ta, world, [h, h], 5, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 5, 1, kind=0)
    ref, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    res_bytes = ref.info().elements * 8
    ref = ref.download()
    srv = ta.Server(world, hbm_budget_bytes=1 << 30, max_batch=2)
    ids = [srv.submit("i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
           for _ in range(6)]
    st = srv.stats()
    for _ in range(6000):
        st = srv.stats()
        if st["completed"] + st["failed"] == 6:
            break
        time.sleep(0.01)
    assert st["completed"] == 6 and st["failed"] == 0
    assert st["bytes_in_use"] == 6 * res_bytes
    for rid in ids:
        C, res = srv.wait(rid, 60000)
        assert res["status"] == 0
        assert np.array_equal(C.download(), ref)
        del C
    st = srv.stats()
    srv.stop()
    assert st["bytes_in_use"] == 0
