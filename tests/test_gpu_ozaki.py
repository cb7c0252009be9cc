"""GPU parity of the emulated-FP64 form (bf16 digit slices on tcgen05).

Integer-valued data are represented exactly by the digits and every level
sum is exact integer arithmetic, so those results must equal the golden
values bit for bit; uniform[-1,1) data must stay within 1e-12 relative
Frobenius error of the FP64 oracle.
"""
import numpy as np
import pytest

from helpers import contraction_cases, golden, gpu_operand, oracle_operand, rel_fro

pytestmark = pytest.mark.gpu

TOL = 1e-12


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


@pytest.mark.parametrize("case", contraction_cases(), ids=lambda c: c["tag"])
def test_ozaki_golden_exact(ta, world, case):
    A, _ = gpu_operand(ta, world, case["trange_a"], *case["seed_a"], kind=1, keep=case["keep_a"])
    B, _ = gpu_operand(ta, world, case["trange_b"], *case["seed_b"], kind=1, keep=case["keep_b"])
    C, st = ta.contract(world, case["c"], case["alpha"], A, case["a"], B, case["b"],
                        precision=ta.PRECISION_OZAKI)
    exp = golden(f"contract_{case['tag']}.npz")["expected"]
    assert np.array_equal(C.to_dense(C.trange), exp)


@pytest.mark.parametrize("n,lo,hi,seed,decay", [(600, 48, 256, 1, 2.0), (1500, 48, 256, 2, 4.0),
                                                (700, 1, 90, 3, 3.0), (2100, 200, 256, 4, 8.0)])
def test_ozaki_uniform_vs_oracle(oracle, ta, world, n, lo, hi, seed, decay):
    h = uneven(n, lo, hi, seed)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / decay)
    scale[scale < 1e-10] = 0
    thr = 1e-8
    A, _ = gpu_operand(ta, world, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    B, _ = gpu_operand(ta, world, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    world.threshold = thr
    try:
        C, st = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
        Cp, stp = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    finally:
        world.threshold = ta.FLT_EPSILON
    Ao = oracle_operand(oracle, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    Bo = oracle_operand(oracle, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    ref = oracle.contract("i,j", Ao, "i,k", Bo, "k,j", threshold=thr).to_dense()
    got = C.to_dense(C.trange)
    err = rel_fro(got, ref)
    print(f"ozaki rel err {err:.3e}, plain {rel_fro(Cp.to_dense(Cp.trange), ref):.3e}")
    assert err <= TOL
    assert np.array_equal(C.norms(), Cp.norms())
    assert st["pairs"] == stp["pairs"]


@pytest.mark.parametrize("slices,bound", [(3, 1e-5), (4, 1e-7), (5, 1e-9), (6, 1e-12),
                                          (7, 1e-14)])
def test_ozaki_slices(oracle, ta, world, slices, bound):
    h = uneven(400, 40, 120, 9)
    A, _ = gpu_operand(ta, world, [h, h], 5, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 5, 1, kind=0)
    C, st = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                        slices=slices)
    Ao = oracle_operand(oracle, [h, h], 5, 0, kind=0)
    Bo = oracle_operand(oracle, [h, h], 5, 1, kind=0)
    ref = oracle.contract("i,j", Ao, "i,k", Bo, "k,j").to_dense()
    err = rel_fro(C.to_dense(C.trange), ref)
    print(f"slices={slices} rel err {err:.3e}")
    assert err <= bound


def test_ozaki_long_k_exact(ta, world):
    """All-positive integer data over a long k: every level grows at the
    worst-case rate within a chunk and the int64 drains must keep the whole
    sum exact."""
    hk = uneven(6000, 100, 256, 11)
    hm = [0, 130, 257]
    A, _ = gpu_operand(ta, world, [hm, hk], 1, 0, kind=1)
    B, _ = gpu_operand(ta, world, [hk, hm], 1, 1, kind=1)
    C, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    Cp, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    assert np.array_equal(C.download(), Cp.download())


@pytest.mark.parametrize("c,a,b", [("i,j", "i,k", "k,j"), ("i,j", "k,i", "j,k")])
def test_ozaki_tiny_tiles_exact(ta, world, c, a, b):
    """One-element tiles along rows and k: a 128 x 32 brick overlaps 4096
    tiles, more than the split stages, so tile offsets are looked up per
    element; both storage orders of A and B."""
    ones = list(range(0, 161))
    hn = [0, 50, 97]
    tra = [ones, ones]
    trb = [ones, hn] if b == "k,j" else [hn, ones]
    keep_a = (np.arange(160 * 160).reshape(160, 160) % 7 != 3).astype(float)
    A, _ = gpu_operand(ta, world, tra, 3, 0, kind=1, keep=keep_a)
    B, _ = gpu_operand(ta, world, trb, 3, 1, kind=1)
    C, _ = ta.contract(world, c, 1.0, A, a, B, b, precision=ta.PRECISION_OZAKI)
    Cp, _ = ta.contract(world, c, 1.0, A, a, B, b)
    assert np.array_equal(C.to_dense(C.trange), Cp.to_dense(Cp.trange))


def test_ozaki_transposed_and_4index(oracle, ta, world):
    h1, h2 = [0, 40, 96], [0, 32, 70, 96]
    for c, a, b, tra, trb in [("i,j", "k,i", "j,k", [h2, h1], [h1, h2]),
                              ("a,b,i,j", "a,b,c,d", "c,d,i,j", [h1, h2, h1, h2],
                               [h1, h2, h1, h2]),
                              ("i,j,a,b", "a,c,b,d", "c,d,i,j", [h1, h1, h2, h2],
                               [h1, h2, h1, h2])]:
        A, _ = gpu_operand(ta, world, tra, 2, 0, kind=0)
        B, _ = gpu_operand(ta, world, trb, 2, 1, kind=0)
        C, _ = ta.contract(world, c, 0.5, A, a, B, b, precision=ta.PRECISION_OZAKI)
        Ao = oracle_operand(oracle, tra, 2, 0, kind=0)
        Bo = oracle_operand(oracle, trb, 2, 1, kind=0)
        ref = oracle.contract(c, Ao, a, Bo, b, 0.5).to_dense()
        assert rel_fro(C.to_dense(C.trange), ref) <= TOL


def test_ozaki_batch_graph(ta, world):
    import ctypes
    L = world.L
    h = uneven(500, 48, 200, 13)
    pairs = []
    for x in range(3):
        A, _ = gpu_operand(ta, world, [h, h], 7, 2 * x, kind=0)
        B, _ = gpu_operand(ta, world, [h, h], 7, 2 * x + 1, kind=0)
        pairs.append((A, B))
    bh = ctypes.c_void_p()
    world.check(L.tagpu_batch_create(world.h, ctypes.byref(bh)))
    outs = []
    for A, B in pairs:
        ch = ctypes.c_void_p()
        opts = ta.ContractOpts(ta.PRECISION_OZAKI, 6, -1.0)
        world.check(L.tagpu_batch_add(bh, b"i,j", 1.0, A.h, b"i,k", B.h, b"k,j",
                                      ctypes.byref(opts), ctypes.byref(ch)))
        outs.append(ta.DistArray(world, _handle=ch))
    world.check(L.tagpu_batch_run(bh))
    first = [o.download().copy() for o in outs]
    for (A, B), f in zip(pairs, first):
        ref, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                             slices=6)
        assert np.array_equal(ref.download(), f)
    world.check(L.tagpu_batch_run(bh))
    for o, f in zip(outs, first):
        assert np.array_equal(o.download(), f)
    world.check(L.tagpu_batch_destroy(bh))


def test_ozaki_accumulator_edge_exact(ta, world):
    """x = 1 - 2^-8 splits into the extreme leading digits d1 = 128,
    d2 = -128, so level 2 (d1 e1) and level 3 (d1 e2 + d2 e1) grow by
    2^14 and 2^15 per k: within their restart periods (32 and 16 stages of
    32 k) they reach exactly +-2^24, the edge of exact fp32 integer sums.
    Every digit product is kept, so the result is exact."""
    x = 1.0 - 2.0 ** -8
    hm, hk, hn = [0, 128, 200], list(range(0, 4097, 256)), [0, 64, 130]
    A = ta.DistArray(world, ta.TiledRange([hm, hk]))
    B = ta.DistArray(world, ta.TiledRange([hk, hn]))
    nk = len(hk) - 1
    A.set_tiles({o: np.full((hm[o // nk + 1] - hm[o // nk]) * 256, x) for o in range(2 * nk)})
    B.set_tiles({o: np.full(256 * (hn[o % 2 + 1] - hn[o % 2]), x if o % 2 == 0 else -x)
                 for o in range(2 * nk)})
    C, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    exp = np.empty((200, 130))
    exp[:, :64], exp[:, 64:] = 4096 * x * x, -4096 * x * x   # exact in FP64
    assert np.array_equal(C.to_dense(C.trange), exp)


def test_ozaki_row_chunking_identical(ta, world, monkeypatch):
    """A digit bricks built and consumed one range of row blocks at a time
    (forced by a tiny budget) give bit-identical results."""
    h = uneven(1100, 48, 256, 21)
    A, _ = gpu_operand(ta, world, [h, h], 4, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 4, 1, kind=0)
    ref, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    monkeypatch.setenv("TAGPU_OZAKI_A_BYTES", str(3 * 6 * 8192 * 40))
    got, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    assert np.array_equal(got.download(), ref.download())


@pytest.mark.parametrize("n,kind", [(1100, 0), (6000, 1)])
def test_ozaki_epilogue_widths_identical(ta, world, monkeypatch, n, kind):
    """The eight-warp and sixteen-warp epilogues (chosen by the units'
    average stage count, forced here) fold the same levels into the same
    integers: results are bit-identical, on short and long k."""
    hk = uneven(n, 48, 256, 23)
    hm = uneven(700, 48, 256, 24)
    A, _ = gpu_operand(ta, world, [hm, hk], 5, 0, kind=kind)
    B, _ = gpu_operand(ta, world, [hk, hm], 5, 1, kind=kind)
    alpha = 0.75 if kind == 0 else 1.0
    out = {}
    for w in ("8", "16"):
        monkeypatch.setenv("TAGPU_EPILOGUE_WARPS", w)
        C, _ = ta.contract(world, "i,j", alpha, A, "i,k", B, "k,j",
                           precision=ta.PRECISION_OZAKI)
        out[w] = C.download()
    assert np.array_equal(out["8"], out["16"])
    if kind == 1:   # integer data: exact, equal to the plain form
        Cp, _ = ta.contract(world, "i,j", alpha, A, "i,k", B, "k,j")
        assert np.array_equal(out["8"], Cp.download())


def test_ozaki_autotune_identical_and_cached(ta, world, tmp_path, monkeypatch):
    """The autotuner only changes the schedule (block order and epilogue
    width): results are bit-identical; the chosen schedule is cached per
    shape bucket, and a cache line without the width still reads."""
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("TAGPU_TUNE_CACHE", str(cache))
    h = uneven(900, 48, 200, 31)
    A, _ = gpu_operand(ta, world, [h, h], 8, 0, kind=0)
    B, _ = gpu_operand(ta, world, [h, h], 8, 1, kind=0)
    ref, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI)
    got, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                         autotune=True)
    assert np.array_equal(got.download(), ref.download())
    lines = cache.read_text().split("\n")
    fields = lines[0].split()
    assert lines[0].startswith("S7_") and len(fields) == 5 and fields[4] in ("8", "16")
    again, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                           autotune=True)
    assert np.array_equal(again.download(), ref.download())
    assert len([x for x in cache.read_text().split("\n") if x]) == 1
    # a cache written before the width was tuned: four fields
    old = tmp_path / "tune_old.txt"
    old.write_text(" ".join(fields[:4]) + "\n")
    monkeypatch.setenv("TAGPU_TUNE_CACHE", str(old))
    legacy, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                            autotune=True)
    assert np.array_equal(legacy.download(), ref.download())
    assert len([x for x in old.read_text().split("\n") if x]) == 1
