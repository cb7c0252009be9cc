"""Parity on the benchmark configurations themselves, against the FP64
oracle (per-pair dgemm in k-ascending order, the reference's
Tensor::gemm -> math/blas.h:171-177 path), for both GEMM forms.

  dense     C(i,j) = A(i,k) B(k,j), N = M = K = 2048, tiles of 128 (full size)
  ccsd      R(a,b,i,j) = V(a,b,c,d) T(c,d,i,j), o = 48 (tiles 16), v = 128
            (tiles U[32,96]) with the configuration's block decay and
            threshold 1e-8, in the identity form, the transposed form of the
            reference's abcd example (T stored as (i,j,c,d),
            examples/gemm/ta_cc_abcd.cpp:240) and a general form (V read as
            (a,c,b,d): an explicit tile permutation into GEMM order)
  batched   the first 64 of the 512 independent C(i,j,l) = A(i,j,k) B(k,l)
            contractions (extents log-uniform [32,512], tiles U[32,128], 30%
            block dropout) as one batch: planned, captured, replayed

Every nonzero result tile is held to 1e-12 relative Frobenius error
(emulated) and 1e-14 (plain), the whole result to 1e-12.
"""
import ctypes

import numpy as np
import pytest

from helpers import gpu_operand, oracle_operand

pytestmark = pytest.mark.gpu

TOL = 1e-12
TOL_PLAIN = 1e-14


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


def per_tile(C, Co):
    """(global, worst tile) relative errors of GPU array C against oracle array Co."""
    off = C.tile_offsets()
    data = C.download()
    num = den = worst = 0.0
    for o, ref in Co.tiles.items():
        got = data[off[o]:off[o] + ref.size] if off[o] >= 0 else np.zeros(ref.size)
        d = float(np.sum((got - ref.ravel()) ** 2))
        r = float(np.sum(ref ** 2))
        num += d
        den += r
        if r > 0:
            worst = max(worst, (d / r) ** 0.5)
    assert all(off[o] < 0 for o in range(len(off)) if o not in Co.tiles), \
        "GPU result has tiles the oracle's shape screens out"
    return (num / den) ** 0.5, worst


def both_forms(ta, world, c, A, a, B, b, Co):
    out = {}
    for name, prec, tol_tile in (("emulated", ta.PRECISION_OZAKI, TOL),
                                 ("plain", ta.PRECISION_FP64, TOL_PLAIN)):
        C, st = ta.contract(world, c, 1.0, A, a, B, b, precision=prec)
        if not C.info().dense:
            assert np.array_equal(C.norms(), Co.norms.ravel().astype(np.float32))
        g, t = per_tile(C, Co)
        out[name] = (g, t)
        assert g <= TOL, (name, g)
        assert t <= tol_tile, (name, t)
    print(" ".join(f"{k}: global {g:.2e} max tile {t:.2e}" for k, (g, t) in out.items()))


def test_config_dense_2048(oracle, ta, world):
    # TArrayD: DensePolicy operands, as the benchmark's dense configuration
    h = list(range(0, 2049, 128))
    tr = ta.TiledRange([h, h])
    A, B = ta.DistArray(world, tr), ta.DistArray(world, tr)
    A.generate(0, 0, 0, None, False)
    B.generate(0, 1, 0, None, False)
    assert A.info().dense and B.info().dense
    Ao = oracle_operand(oracle, [h, h], 0, 0, kind=0)
    Bo = oracle_operand(oracle, [h, h], 0, 1, kind=0)
    Co = oracle.contract("i,j", Ao, "i,k", Bo, "k,j", use_blas=oracle.openblas_dgemm())
    both_forms(ta, world, "i,j", A, "i,k", B, "k,j", Co)


@pytest.mark.parametrize("form", ["identity", "transpose", "general"])
def test_config_ccsd_v128(oracle, ta, world, form):
    from tiledarray_gb300 import workloads as wl
    hv, ho, vs, ts = wl.ccsd(v=128, seed=0)
    thr = 1e-8
    world.threshold = thr
    try:
        V, _ = gpu_operand(ta, world, [hv] * 4, 0, 0, kind=0, tile_scale=vs, threshold=thr)
        Vo = oracle_operand(oracle, [hv] * 4, 0, 0, kind=0, tile_scale=vs, threshold=thr)
        if form == "transpose":
            tst = np.ascontiguousarray(ts.transpose(2, 3, 0, 1))
            dims, b_idx = [ho, ho, hv, hv], "i,j,c,d"
        else:
            tst, dims, b_idx = ts, [hv, hv, ho, ho], "c,d,i,j"
        T, _ = gpu_operand(ta, world, dims, 0, 1, kind=0, tile_scale=tst, threshold=thr)
        To = oracle_operand(oracle, dims, 0, 1, kind=0, tile_scale=tst, threshold=thr)
        a_idx = "a,c,b,d" if form == "general" else "a,b,c,d"
        Ro = oracle.contract("a,b,i,j", Vo, a_idx, To, b_idx, threshold=thr,
                             use_blas=oracle.openblas_dgemm())
        both_forms(ta, world, "a,b,i,j", V, a_idx, T, b_idx, Ro)
    finally:
        world.threshold = ta.FLT_EPSILON


def test_config_batched_slice(oracle, ta, world):
    from tiledarray_gb300 import workloads as wl
    cases = wl.batched(64, 0)
    L = world.L
    ops = []
    for x, (tsl, ka, kb) in enumerate(cases):
        A, _ = gpu_operand(ta, world, [tsl[0], tsl[1], tsl[2]], 0, 2 * x, kind=0, tile_scale=ka)
        B, _ = gpu_operand(ta, world, [tsl[2], tsl[3]], 0, 2 * x + 1, kind=0, tile_scale=kb)
        ops.append((A, B))
    for prec, tol_tile in ((ta.PRECISION_OZAKI, TOL), (ta.PRECISION_FP64, TOL_PLAIN)):
        bh = ctypes.c_void_p()
        world.check(L.tagpu_batch_create(world.h, ctypes.byref(bh)))
        outs = []
        opts = ta.ContractOpts(prec, 6, -1.0)
        for A, B in ops:
            ch = ctypes.c_void_p()
            world.check(L.tagpu_batch_add(bh, b"i,j,l", 1.0, A.h, b"i,j,k", B.h, b"k,l",
                                          ctypes.byref(opts), ctypes.byref(ch)))
            outs.append(ta.DistArray(world, _handle=ch))
        world.check(L.tagpu_batch_run(bh))   # plan, capture, first run
        world.check(L.tagpu_batch_run(bh))   # graph replay
        worst_g = worst_t = 0.0
        for x, (tsl, ka, kb) in enumerate(cases):
            Ao = oracle_operand(oracle, [tsl[0], tsl[1], tsl[2]], 0, 2 * x, kind=0, tile_scale=ka)
            Bo = oracle_operand(oracle, [tsl[2], tsl[3]], 0, 2 * x + 1, kind=0, tile_scale=kb)
            Co = oracle.contract("i,j,l", Ao, "i,j,k", Bo, "k,l")
            if not Co.tiles:
                continue
            g, t = per_tile(outs[x], Co)
            worst_g, worst_t = max(worst_g, g), max(worst_t, t)
        world.check(L.tagpu_batch_destroy(bh))
        print(f"precision {prec}: worst contraction {worst_g:.2e}, worst tile {worst_t:.2e}")
        assert worst_g <= TOL
        assert worst_t <= tol_tile
