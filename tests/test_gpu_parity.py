"""GPU parity: every kernel on the path against the CPU oracle, through the C ABI.

Bit-exact for the screened shapes, pair lists, permutations and integer-valued
contractions; relative Frobenius error <= 1e-12 for uniform[-1,1) data.
"""
import numpy as np
import pytest

from helpers import contraction_cases, golden, gpu_operand, oracle_operand, rel_fro

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative Frobenius error bound for floating-point data


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


def uneven_hashmarks(n_total, lo, hi, seed):
    rng = np.random.default_rng(seed)
    h = [0]
    while h[-1] < n_total:
        h.append(min(n_total, h[-1] + int(rng.integers(lo, hi + 1))))
    return h


@pytest.mark.parametrize("tr_dims,kind", [
    ([[0, 2, 5, 10, 17, 28]] * 3, 1),
    ([[0, 13, 40, 64], [0, 7, 31, 50]], 0),
    ([uneven_hashmarks(700, 32, 256, 1), uneven_hashmarks(500, 32, 256, 2)], 0),
    ([[0, 3, 7, 8], [0, 2, 6], [0, 3, 7, 8], [0, 2, 6]], 0),
])
def test_generate_and_shape_bitexact(oracle, ta, world, tr_dims, kind):
    n = int(np.prod([len(h) - 1 for h in tr_dims]))
    keep = (np.arange(n) % 3) != 1
    Ao = oracle_operand(oracle, tr_dims, 9, 4, kind=kind, keep=keep)
    Ag, tr = gpu_operand(ta, world, tr_dims, 9, 4, kind=kind, keep=keep)
    assert np.array_equal(Ag.norms(), Ao.norms.ravel())
    got = Ag.tiles(tr)
    assert set(got) == set(Ao.tiles)
    for o, t in Ao.tiles.items():
        assert np.array_equal(got[o], t)


def test_shape_gemm_kernel_matches_golden(oracle, ta, world):
    g = golden("shape_gemm.npz")
    tr = [list(h) for h in g["hashmarks"]]
    sizes = [np.asarray([h[i + 1] - h[i] for i in range(len(h) - 1)], np.float32) for h in tr]
    ks = oracle.outer_sizes([5, 5], np.concatenate(sizes[1:]), False)
    L, R = g["left"].reshape(5, 25), g["right"].reshape(25, 5)
    r_o, z_o = oracle.shape_gemm(L, R, ks, float(g["factor"]), float(g["threshold"]))
    r_g, z_g = world.shape_gemm(L, R, ks, float(g["factor"]), float(g["threshold"]))
    assert np.array_equal(r_g, r_o) and z_g == z_o


@pytest.mark.parametrize("M,N,K,seed", [(1, 1, 1, 0), (106, 106, 106, 1), (36, 9, 36, 2),
                                        (300, 7, 1000, 3), (5, 333, 0, 4)])
def test_shape_gemm_kernel_bitexact(oracle, ta, world, M, N, K, seed):
    rng = np.random.default_rng(seed)
    L = (rng.random((M, max(K, 1))) ** 4).astype(np.float32) * 1e-3
    R = (rng.random((max(K, 1), N)) ** 4).astype(np.float32) * 1e-3
    L[rng.random(L.shape) < 0.3] = 0
    ks = rng.integers(16, 9216, K).astype(np.float32) if K else None
    thr = np.float32(1e-8)
    r_o, z_o = oracle.shape_gemm(L, R, ks, -2.5, thr)
    r_g, z_g = world.shape_gemm(L, R, ks, -2.5, thr)
    assert np.array_equal(r_g, r_o) and z_g == z_o


def test_pair_list_kernel_matches_golden(ta, world):
    g = golden("pairs.npz")
    for c in range(int(g["ncases"])):
        thr = g[f"c{c}_thr"]
        offs, kidx = world.pair_list(g[f"c{c}_C"], thr[0], g[f"c{c}_L"], thr[1], g[f"c{c}_R"],
                                     thr[2])
        assert np.array_equal(offs, g[f"c{c}_offsets"])
        assert np.array_equal(kidx, g[f"c{c}_kidx"])


def test_pair_list_kernel_large(oracle, ta, world):
    rng = np.random.default_rng(7)
    M, N, K = 120, 110, 130
    C, L, R = (rng.random((M, N), np.float32), rng.random((M, K), np.float32),
               rng.random((K, N), np.float32))
    o1, k1 = oracle.pairs(C, 0.3, L, 0.5, R, 0.2)
    o2, k2 = world.pair_list(C, 0.3, L, 0.5, R, 0.2)
    assert np.array_equal(o1, o2) and np.array_equal(k1, k2)


def test_permute_kernel_matches_golden(ta, world):
    g = golden("permute.npz")
    for c in range(int(g["ncases"])):
        y = world.permute(g[f"c{c}_x"], list(g[f"c{c}_perm"]))
        assert np.array_equal(y, g[f"c{c}_y"])


@pytest.mark.parametrize("shape,perm", [((96, 80, 64, 32), (3, 1, 2, 0)),
                                        ((256, 255), (1, 0)), ((33, 17, 65), (0, 2, 1)),
                                        ((9, 96, 96), (1, 2, 0))])
def test_permute_kernel_large(oracle, ta, world, shape, perm):
    x = np.random.default_rng(1).random(shape)
    assert np.array_equal(world.permute(x, perm), oracle.permute(x, perm))


@pytest.mark.parametrize("case", contraction_cases(), ids=lambda c: c["tag"])
def test_contraction_dmma_golden(oracle, ta, world, case):
    """Reference test forms on integer data: exact equality with the golden
    dense result, result shape bit-exact with the oracle."""
    A, tra = gpu_operand(ta, world, case["trange_a"], *case["seed_a"], kind=1,
                         keep=case["keep_a"])
    B, trb = gpu_operand(ta, world, case["trange_b"], *case["seed_b"], kind=1,
                         keep=case["keep_b"])
    C, st = ta.contract(world, case["c"], case["alpha"], A, case["a"], B, case["b"])
    exp = golden(f"contract_{case['tag']}.npz")["expected"]
    got = C.to_dense(C.trange)
    assert np.array_equal(got, exp)
    Ao = oracle_operand(oracle, case["trange_a"], *case["seed_a"], kind=1, keep=case["keep_a"])
    Bo = oracle_operand(oracle, case["trange_b"], *case["seed_b"], kind=1, keep=case["keep_b"])
    Co, info = oracle.contract(case["c"], Ao, case["a"], Bo, case["b"], case["alpha"],
                               return_pairs=True)
    assert np.array_equal(C.norms(), Co.norms.ravel())
    assert st["pairs"] == len(info["kidx"])
    assert st["left_permtype"] == info["left_permtype"]
    assert st["right_permtype"] == info["right_permtype"]


def block_sparse_case(n, lo, hi, seed, decay=4.0, cut=1e-10):
    h = uneven_hashmarks(n, lo, hi, seed)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / decay)
    scale[scale < cut] = 0.0
    return h, scale


@pytest.mark.parametrize("n,lo,hi,seed", [(600, 48, 256, 1), (1000, 32, 128, 2),
                                          (257, 1, 64, 3)])
def test_contraction_dmma_uniform(oracle, ta, world, n, lo, hi, seed):
    h, scale = block_sparse_case(n, lo, hi, seed, decay=2.0)
    thr = 1e-8
    A, tr = gpu_operand(ta, world, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    B, _ = gpu_operand(ta, world, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    world.threshold = thr
    try:
        C, st = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    finally:
        world.threshold = ta.FLT_EPSILON
    Ao = oracle_operand(oracle, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    Bo = oracle_operand(oracle, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    Co, info = oracle.contract("i,j", Ao, "i,k", Bo, "k,j", threshold=thr, return_pairs=True)
    assert np.array_equal(C.norms(), Co.norms.ravel())
    assert st["pairs"] == len(info["kidx"])
    ref = Co.to_dense()
    got = C.to_dense(C.trange)
    assert rel_fro(got, ref) <= TOL


def test_batch_graph_replay(oracle, ta, world):
    import ctypes
    L = world.L
    forms = [("i,j", "i,k", "k,j"), ("i,j", "k,i", "k,j"), ("j,i", "i,k", "j,k")]
    h1 = uneven_hashmarks(300, 20, 90, 5)
    h2 = uneven_hashmarks(260, 20, 90, 6)
    ops = []
    for x, (c, a, b) in enumerate(forms):
        tra = [h1, h2] if a == "i,k" else [h2, h1]
        trb = [h2, h1] if b == "k,j" else [h1, h2]
        A, _ = gpu_operand(ta, world, tra, 3, 2 * x, kind=0)
        B, _ = gpu_operand(ta, world, trb, 3, 2 * x + 1, kind=0)
        ops.append((c, a, b, A, B))
    bh = ctypes.c_void_p()
    world.check(L.tagpu_batch_create(world.h, ctypes.byref(bh)))
    outs = []
    for c, a, b, A, B in ops:
        ch = ctypes.c_void_p()
        opts = ta.ContractOpts(ta.PRECISION_FP64, 0, -1.0)
        world.check(L.tagpu_batch_add(bh, c.encode(), 1.0, A.h, a.encode(), B.h, b.encode(),
                                      ctypes.byref(opts), ctypes.byref(ch)))
        outs.append(ta.DistArray(world, _handle=ch))
    world.check(L.tagpu_batch_run(bh))
    first = [o.download().copy() for o in outs]
    for c, a, b, A, B in ops:
        ref, _ = ta.contract(world, c, 1.0, A, a, B, b)
        assert np.array_equal(ref.download(), first[ops.index((c, a, b, A, B))])
    world.check(L.tagpu_batch_run(bh))  # graph replay
    for o, f in zip(outs, first):
        assert np.array_equal(o.download(), f)
    world.check(L.tagpu_batch_destroy(bh))


def test_invalid_and_unsupported_forms(ta, world):
    A, _ = gpu_operand(ta, world, [[0, 4, 8], [0, 3, 6]], 1, 0, kind=0)
    B, _ = gpu_operand(ta, world, [[0, 3, 6], [0, 5]], 1, 1, kind=0)
    with pytest.raises(ta.TAGPUError) as e:
        ta.contract(world, "i,j", 1.0, A, "i,j", B, "i,j")  # Hadamard, tilings differ
    assert e.value.status == 1
    with pytest.raises(ta.TAGPUError) as e:
        ta.contract(world, "i,j", 1.0, A, "i,k", B, "j,k")  # k tilings not congruent
    assert e.value.status == 1
    with pytest.raises(ta.TAGPUError) as e:
        ta.contract(world, "i,j", 1.0, A, "i,,k", B, "k,j")
    assert e.value.status == 1


def test_all_screened_result(ta, world):
    h = [0, 10, 20]
    A, _ = gpu_operand(ta, world, [h, h], 1, 0, kind=0, tile_scale=np.full(4, 1e-6))
    B, _ = gpu_operand(ta, world, [h, h], 1, 1, kind=0, tile_scale=np.full(4, 1e-6))
    C, st = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    assert st["nonzero_result_tiles"] == 0 and st["pairs"] == 0
    assert C.info().elements == 0


def test_fp64_rates_measured(ta, world):
    dmma, dfma = world.fp64_rates()
    assert 0.05 < dmma < 200 and 0.05 < dfma < 200


def test_get_tile_matches_download(ta, world):
    h = uneven_hashmarks(300, 20, 90, 8)
    keep = (np.arange((len(h) - 1) ** 2) % 4) != 1
    A, tr = gpu_operand(ta, world, [h, h], 4, 0, kind=0, keep=keep)
    full, offs = A.download(), A.tile_offsets()
    for o in np.flatnonzero(offs >= 0):
        t = A.tile(int(o))
        assert np.array_equal(t.ravel(), full[offs[o]:offs[o] + t.size])
    zero = int(np.flatnonzero(offs < 0)[0])
    with pytest.raises(ta.TAGPUError):
        A.tile(zero)


def test_truncate_matches_make_array(oracle, ta, world):
    """truncate with a larger threshold equals building the array with that
    threshold from the start (make_array semantics): same scaled norms, same
    surviving tiles, zero tiles stay zero."""
    h = uneven_hashmarks(600, 40, 120, 12)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) * 3.0)
    keep = (np.arange(nt * nt) % 5) != 2
    A, tr = gpu_operand(ta, world, [h, h], 6, 0, kind=0, keep=keep, tile_scale=scale,
                        threshold=1e-14)
    A.truncate(1e-6)
    Ao = oracle_operand(oracle, [h, h], 6, 0, kind=0, keep=keep, tile_scale=scale,
                        threshold=1e-6)
    assert np.array_equal(A.norms(), Ao.norms.ravel())
    got = A.tiles(tr)
    assert set(got) == set(Ao.tiles) and len(got) < int(keep.sum())
    for o, t in Ao.tiles.items():
        assert np.array_equal(got[o], t)
    info = A.info()
    assert info.zero_tiles == nt * nt - len(got)


def test_tile_norms_at_float_ties(oracle, ta, world):
    """Device tile norms equal the sequential-order norms bit for bit, also for
    tiles whose sum of squares sits at a float rounding boundary of the norm
    (where the kernel's error bound cannot decide and it sums in order), and
    for large tiles."""
    rng = np.random.default_rng(3)
    f = rng.uniform(1.0, 2.0, 48).astype(np.float32)
    f_next = np.nextafter(f, np.float32(np.inf))
    mids = (f.astype(np.float64) + f_next.astype(np.float64)) / 2   # halfway between floats
    tiles = []
    for x, m in enumerate(mids):
        kind = x % 4
        if kind == 0:
            t = np.array([m])                          # one element, at the tie
        elif kind == 1:
            t = np.full(100, m / 10.0)                 # equal elements, squares summing near m^2
        elif kind == 2:
            t = rng.uniform(-1.0, 1.0, 5000)
            t *= m / np.sqrt(np.sum(t * t))            # sum of squares near m^2
        else:
            t = rng.uniform(-1.0, 1.0, int(rng.integers(1, 70000)))
        tiles.append(t)
    h = [0] + np.cumsum([len(t) for t in tiles]).tolist()
    n = len(tiles)
    A = ta.DistArray(world, ta.TiledRange([h]), norms=np.ones(n, np.float32), do_not_scale=True,
                     threshold=0.0)
    A.upload(np.concatenate(tiles))
    A.truncate(0.0)   # the norms again, from the device data
    raw = np.asarray([oracle.tile_norm(t) for t in tiles], np.float32)
    want, _ = oracle.scale_norms(oracle.TiledRange([h]), raw, 0.0)
    assert np.array_equal(A.norms(), want.ravel())


@pytest.mark.parametrize("precision", [0, 1])
def test_contract_accumulate(ta, world, precision):
    """C("i,j") += alpha * A2("i,k") * B2("k,j"): the shape is the float sum of
    the two scaled norms, zero below the threshold (SparseShape::add); tiles in
    both are summed with one rounding, tiles in one are copied."""
    h = uneven_hashmarks(700, 40, 140, 14)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    band = lambda w0: np.where(np.abs(I - J) <= w0, 1.0, 0.0)
    thr = 1e-8
    world.threshold = thr
    try:
        A, _ = gpu_operand(ta, world, [h, h], 21, 0, kind=0, tile_scale=band(1), threshold=thr)
        B, _ = gpu_operand(ta, world, [h, h], 21, 1, kind=0, tile_scale=band(1), threshold=thr)
        A2, _ = gpu_operand(ta, world, [h, h], 22, 0, kind=0, tile_scale=band(2) * (I >= J),
                            threshold=thr)
        B2, _ = gpu_operand(ta, world, [h, h], 22, 1, kind=0, tile_scale=band(2), threshold=thr)
        C, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=precision)
        P, _ = ta.contract(world, "i,j", -0.75, A2, "i,k", B2, "k,j", precision=precision)
        c_n, c_off, c_d = C.norms(), C.tile_offsets(), C.download()
        p_n, p_off, p_d = P.norms(), P.tile_offsets(), P.download()
        ta.contract_accumulate(world, C, "i,j", -0.75, A2, "i,k", B2, "k,j", precision=precision)
    finally:
        world.threshold = ta.FLT_EPSILON
    exp_n = (c_n + p_n).astype(np.float32)
    exp_n[exp_n < np.float32(thr)] = 0
    assert np.array_equal(C.norms(), exp_n)
    assert (p_off >= 0).sum() > 0 and ((c_off < 0) & (p_off >= 0)).sum() > 0
    r_off, r_d = C.tile_offsets(), C.download()
    tr = C.trange
    for t in np.flatnonzero(r_off >= 0):
        i, j = divmod(int(t), nt)
        vol = (h[i + 1] - h[i]) * (h[j + 1] - h[j])
        c = c_d[c_off[t]:c_off[t] + vol] if c_off[t] >= 0 else None
        p = p_d[p_off[t]:p_off[t] + vol] if p_off[t] >= 0 else None
        want = c + p if (c is not None and p is not None) else (c if c is not None else p)
        assert np.array_equal(r_d[r_off[t]:r_off[t] + vol], want)
    assert set(np.flatnonzero(r_off >= 0)) == set(np.flatnonzero(exp_n > 0))


@pytest.mark.parametrize("sparse", [True, False])
def test_archive_roundtrip(ta, world, tmp_path, sparse):
    """save then load gives the same tiling, shape, offsets and tile data bit
    for bit; a file that is not an archive, or a truncated one, is rejected."""
    h1, h2 = uneven_hashmarks(500, 30, 140, 15), uneven_hashmarks(300, 20, 90, 16)
    if sparse:
        keep = (np.arange((len(h1) - 1) * (len(h2) - 1)) % 3) != 0
        A, tr = gpu_operand(ta, world, [h1, h2], 17, 0, kind=0, keep=keep)
    else:
        A = ta.DistArray(world, ta.TiledRange([h1, h2]))
        A.generate(17, 0, 0, None, False)
    path = tmp_path / "a.tagpu"
    A.save(path)
    B = ta.DistArray.load(world, path)
    ia, ib = A.info(), B.info()
    assert (ia.dense, ia.elements, ia.zero_tiles) == (ib.dense, ib.elements, ib.zero_tiles)
    assert B.trange.dims == A.trange.dims
    assert np.array_equal(A.tile_offsets(), B.tile_offsets())
    assert np.array_equal(A.norms(), B.norms())
    assert np.array_equal(A.download(), B.download())
    bad = tmp_path / "bad.tagpu"
    bad.write_bytes(b"not an archive at all")
    with pytest.raises(ta.TAGPUError) as e:
        ta.DistArray.load(world, bad)
    assert e.value.status == 1
    cut = tmp_path / "cut.tagpu"
    cut.write_bytes(path.read_bytes()[:-100])
    with pytest.raises(ta.TAGPUError):
        ta.DistArray.load(world, cut)


def test_host_buffers_roundtrip(ta, world):
    """Library-owned pinned host buffers carry an array's tiles both ways."""
    A, _ = gpu_operand(ta, world, [[0, 40, 100], [0, 64, 90]], 3, 0, kind=0)
    n = A.info().elements
    buf = world.host_array(n)
    buf[:] = A.download()
    B = ta.DistArray(world, A.trange)
    B.set_shape(A.norms(), do_not_scale=True, threshold=A.info().threshold)
    B.upload(buf)
    out = world.host_array(n)
    world.check(world.L.tagpu_array_download(B.h, out.ctypes.data_as(ta._f64p), n))
    assert np.array_equal(out, A.download())


@pytest.mark.parametrize("shift", [0, 1, 3])
def test_host_buffers_unaligned(ta, world, shift):
    """Registered host memory at offsets of 0, 1 and 3 doubles: the
    kernel-driven copies take their 16-byte and 8-byte paths, move every
    element both ways and write nothing outside the buffer."""
    A, _ = gpu_operand(ta, world, [[0, 40, 101], [0, 64, 93]], 4, 0, kind=0)
    n = A.info().elements
    base = world.host_array(n + 4)
    view = base[shift:shift + n]
    view[:] = A.download()
    B = ta.DistArray(world, A.trange)
    B.set_shape(A.norms(), do_not_scale=True, threshold=A.info().threshold)
    world.check(world.L.tagpu_array_upload(B.h, view.ctypes.data_as(ta._f64p), n))
    assert np.array_equal(B.download(), A.download())
    back = world.host_array(n + 4)
    back[:] = -1.0
    world.check(world.L.tagpu_array_download(B.h, back[shift:].ctypes.data_as(ta._f64p), n))
    assert np.array_equal(back[shift:shift + n], A.download())
    assert np.all(back[:shift] == -1.0) and np.all(back[shift + n:] == -1.0)
