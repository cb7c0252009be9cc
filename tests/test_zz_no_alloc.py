"""The allocation-free pair-list entry point, called through the C ABI.

tagpu_pair_list_noalloc exists for callers that cannot allocate device
memory (their device memory is owned by another framework's pool, or they run
a loop that must not allocate).  They pass device buffers for every input and
output; the library keeps its only scratch in a fixed array.  This test is the
caller: it owns the device buffers (torch tensors) and checks the result of
two calls in a row against the ordinary entry point, tagpu_pair_list, which
takes host buffers.  The results are integer lists, so they must be equal.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(seed, M, N, K):
    rng = np.random.default_rng(seed)
    C = rng.random((M, N), dtype=np.float32)
    L = rng.random((M, K), dtype=np.float32)
    R = rng.random((K, N), dtype=np.float32)
    C[rng.random((M, N)) < 0.2] = 0
    L[rng.random((M, K)) < 0.3] = 0
    R[rng.random((K, N)) < 0.3] = 0
    return C, L, R, np.float32(0.2), np.float32(0.15), np.float32(0.1)


def _noalloc(world, torch, C, L, R, ct, lt, rt):
    M, N = C.shape
    K = L.shape[1]
    dev = torch.device("cuda", 0)
    dC, dL, dR = (torch.from_numpy(x).to(dev) for x in (C, L, R))
    offs = torch.empty(M * N + 1, dtype=torch.int64, device=dev)
    n = ctypes.c_int64(0)
    torch.cuda.synchronize()
    args = (world.h, M, N, K, ctypes.c_void_p(dC.data_ptr()), ct, ctypes.c_void_p(dL.data_ptr()),
            lt, ctypes.c_void_p(dR.data_ptr()), rt, ctypes.c_void_p(offs.data_ptr()))
    world.check(world.L.tagpu_pair_list_noalloc(*args, None, 0, ctypes.byref(n), None))
    kidx = torch.empty(max(1, n.value), dtype=torch.int32, device=dev)
    world.check(world.L.tagpu_pair_list_noalloc(*args, ctypes.c_void_p(kidx.data_ptr()),
                                                kidx.numel(), ctypes.byref(n), None))
    torch.cuda.synchronize()
    return offs.cpu().numpy(), kidx.cpu().numpy()[:n.value]


def test_noalloc_pair_list_matches_entry_point(world):
    torch = pytest.importorskip("torch")
    for seed, (M, N, K) in enumerate([(60, 70, 80), (106, 106, 106)]):  # two calls in a row
        C, L, R, ct, lt, rt = _case(seed, M, N, K)
        ref_offs, ref_kidx = world.pair_list(C, ct, L, lt, R, rt)
        offs, kidx = _noalloc(world, torch, C, L, R, ct, lt, rt)
        assert np.array_equal(offs, ref_offs)
        assert np.array_equal(kidx, ref_kidx)


def test_noalloc_rejects_oversize(world):
    import tiledarray_gb300 as ta
    n = ctypes.c_int64(0)
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    st = world.L.tagpu_pair_list_noalloc(world.h, 2048, 1024, 1, dummy, 0.1, dummy, 0.1, dummy,
                                         0.1, dummy, None, 0, ctypes.byref(n), None)
    assert st == 1
    assert b"1048576" in world.L.tagpu_last_error(world.h)
    assert ta.STATUS[st] == "invalid argument"
    # M * N = 2^80 wraps to 0 in int64: the bound is checked per factor first
    big = 1 << 40
    st = world.L.tagpu_pair_list_noalloc(world.h, big, big, 1, dummy, 0.1, dummy, 0.1, dummy,
                                         0.1, dummy, None, 0, ctypes.byref(n), None)
    assert st == 1
    assert b"1048576" in world.L.tagpu_last_error(world.h)
