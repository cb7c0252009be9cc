"""Generate the golden fixtures under tests/golden/ (run: python make_golden.py).

The reference's own tests (TiledArray tests/) hold no stored vectors: each
test recomputes its expectation with Eigen from MADNESS rand() data.  These
fixtures restate those scenarios with this project's seeded generator and
compute every expectation independently of the oracle's C code, in numpy:

  rng.npz            the counter-based generator itself (pure numpy splitmix64)
  scale_norms.npz    SparseShape(norms, trange) scaling, sparse_shape.h:150-215,
                     on the TiledRangeFixture tiling (primes 2,3,5,7,11:
                     tests/range_fixture.h:81-87, tests/ta_test.cpp:89-91)
  shape_gemm.npz     tests/sparse_shape.cpp:1478-1541 (alpha = -7.2, default
                     threshold 0.001 tweaked x10, fixture fills 0.1 seeds 23/82:
                     tests/sparse_shape_fixture.h:35-117)
  pairs.npz          Summa pair set (dist_eval/contraction_eval.h:630-650,
                     1093-1161, 1348-1384), brute force
  permute.npz        Tensor permute semantics (permutation.h:60-78) via numpy
  contract_*.npz     the expression tests' contraction forms
                     (tests/expressions_impl.h:1808-2675, 2792-2812) on
                     integer data (rand() % 101), dense and half-sparse
                     (tests/expressions_fixture.h:148-230), expected values by
                     dense numpy einsum (exact: integer data).
"""
from __future__ import annotations

import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
U64 = np.uint64


def splitmix64(x):
    x = (x + U64(0x9E3779B97F4A7C15))
    x = (x ^ (x >> U64(30))) * U64(0xBF58476D1CE4E5B9)
    x = (x ^ (x >> U64(27))) * U64(0x94D049BB133111EB)
    return x ^ (x >> U64(31))


def hash_(seed, stream, ordinal):
    with np.errstate(over="ignore"):
        key = splitmix64(np.asarray([seed], dtype=U64) * U64(0x9E3779B97F4A7C15) +
                         np.asarray([stream], dtype=U64))
        return splitmix64(key ^ np.asarray(ordinal, dtype=U64))


def values(seed, stream, ordinal, kind):
    h = hash_(seed, stream, ordinal)
    if kind == 1:
        return (h % U64(101)).astype(np.float64)
    return ((h >> U64(11)).astype(np.float64) * 2.0 ** -53) * 2.0 - 1.0


def dense_operand(extents, seed, stream, kind=1):
    n = int(np.prod(extents))
    with np.errstate(over="ignore"):
        return values(seed, stream, np.arange(n, dtype=np.uint64), kind).reshape(extents)


def hashmarks_primes(n=5):
    primes = [2, 3, 5, 7, 11, 13, 17]
    h = [0]
    for i in range(n):
        h.append(h[-1] + primes[i])
    return h


def tile_sizes(h):
    return [h[i + 1] - h[i] for i in range(len(h) - 1)]


def outer_inv(svs):
    """recursive_outer_product of inverse size vectors, float32 step by step."""
    if len(svs) == 1:
        return (np.float32(1) / np.asarray(svs[0], np.float32)).astype(np.float32)
    mid = (len(svs) >> 1) + (len(svs) & 1)
    l = outer_inv(svs[:mid])
    r = outer_inv(svs[mid:])
    return (l[:, None] * r[None, :]).astype(np.float32).ravel()


def scale(norms, tr, thr):
    svs = [tile_sizes(h) for h in tr]
    n = norms.astype(np.float32).ravel().copy()
    if len(tr) == 1:
        n = (n / np.asarray(svs[0], np.float32)).astype(np.float32)
    else:
        mid = (len(tr) >> 1) + (len(tr) & 1)
        l = outer_inv(svs[:mid])
        r = outer_inv(svs[mid:])
        xy = (l[:, None] * r[None, :]).astype(np.float32).ravel()
        n = (n * xy).astype(np.float32)
    z = int(np.sum(n < np.float32(thr)))
    n[n < np.float32(thr)] = 0
    return n.reshape([len(h) - 1 for h in tr]), z


def tile_volumes(tr):
    out = np.ones([len(h) - 1 for h in tr], np.float64)
    for d, h in enumerate(tr):
        s = np.asarray(tile_sizes(h), np.float64)
        shp = [1] * len(tr)
        shp[d] = len(s)
        out = out * s.reshape(shp)
    return out


def make_norm_tensor(tr, fill, seed, thr):
    """sparse_shape_fixture.h make_norm_tensor with this project's generator:
    norm = sqrt(r^2 * volume), r = hash % 101; then (1-fill)*n random tiles set
    to threshold*0.1."""
    vol = tile_volumes(tr).ravel()
    n = vol.size
    r = (hash_(seed, 0, np.arange(n, dtype=np.uint64)) % U64(101)).astype(np.float32)
    norms = np.sqrt(r * r * vol.astype(np.float32)).astype(np.float32)
    nz = int(float(n) * (1.0 - fill))
    picks = (hash_(seed, 1, np.arange(nz, dtype=np.uint64)) % U64(n)).astype(np.int64)
    for p in picks:
        norms[p] = np.float32(thr) * np.float32(0.1)
    return norms.reshape([len(h) - 1 for h in tr])


def gen_scale_norms():
    tr = [hashmarks_primes()] * 3
    thr = 0.001
    raw = make_norm_tensor(tr, 0.5, 42, thr)
    scaled, z = scale(raw, tr, thr)
    np.savez(os.path.join(HERE, "scale_norms.npz"), hashmarks=np.asarray(tr), raw=raw,
             scaled=scaled, zero_count=z, threshold=np.float32(thr))


def gen_shape_gemm():
    tr = [hashmarks_primes()] * 3
    thr = np.float32(0.001)
    left_raw = make_norm_tensor(tr, 0.1, 23, thr)
    right_raw = make_norm_tensor(tr, 0.1, 82, thr)
    left, _ = scale(left_raw, tr, thr)
    right, _ = scale(right_raw, tr, thr)
    vol = tile_volumes(tr)
    # the test's expectation (tests/sparse_shape.cpp:1503-1519), float64
    M, K, N = 5, 25, 5
    L = (left.astype(np.float64) * vol).reshape(M, K)
    R = (right.astype(np.float64) * vol).reshape(K, N)
    res = 7.2 * (L @ R)
    s = np.asarray(tile_sizes(tr[0]), np.float64)
    expected = res / (s[:, None] * s[None, :])
    rthr = 10 * thr
    expected[expected < rthr] = 0.0
    np.savez(os.path.join(HERE, "shape_gemm.npz"), hashmarks=np.asarray(tr), left=left,
             right=right, factor=-7.2, threshold=np.float32(rthr), expected=expected,
             tolerance_percent=0.0001)


def gen_pairs():
    out = {}
    for case, (M, N, K, seed) in enumerate([(7, 5, 9, 3), (16, 16, 16, 5), (1, 1, 40, 7),
                                             (33, 2, 65, 9)]):
        def mk(shape, st):
            h = hash_(seed, st, np.arange(int(np.prod(shape)), dtype=np.uint64))
            v = (h % U64(1000)).astype(np.float32) / np.float32(1000.0)
            v[(h >> U64(20)) % U64(3) == U64(0)] = 0.0
            return v.reshape(shape)
        C, L, R = mk((M, N), 0), mk((M, K), 1), mk((K, N), 2)
        cthr, lthr, rthr = np.float32(0.25), np.float32(0.1), np.float32(0.05)
        offs, kidx = [0], []
        for i in range(M):
            for j in range(N):
                if not (C[i, j] < cthr):
                    for k in range(K):
                        if not (L[i, k] < lthr) and not (R[k, j] < rthr):
                            kidx.append(k)
                offs.append(len(kidx))
        out[f"c{case}_C"], out[f"c{case}_L"], out[f"c{case}_R"] = C, L, R
        out[f"c{case}_thr"] = np.asarray([cthr, lthr, rthr], np.float32)
        out[f"c{case}_offsets"] = np.asarray(offs, np.int64)
        out[f"c{case}_kidx"] = np.asarray(kidx, np.int32)
    out["ncases"] = 4
    np.savez(os.path.join(HERE, "pairs.npz"), **out)


def gen_permute():
    out = {}
    cases = [((5, 7), (1, 0)), ((3, 4, 5), (1, 2, 0)), ((3, 4, 5), (0, 2, 1)),
             ((2, 3, 4, 5), (2, 3, 0, 1)), ((6, 5, 4, 3), (3, 2, 1, 0)),
             ((33, 65), (1, 0)), ((7, 1, 9), (2, 1, 0)), ((4, 4, 4, 4), (0, 1, 3, 2))]
    for c, (shape, perm) in enumerate(cases):
        x = dense_operand(shape, 11, c, kind=0)
        # result dim perm[d] = argument dim d  <=>  numpy axes order inv(perm)
        inv = [0] * len(perm)
        for d, p in enumerate(perm):
            inv[p] = d
        out[f"c{c}_x"] = x
        out[f"c{c}_perm"] = np.asarray(perm, np.int32)
        out[f"c{c}_y"] = np.ascontiguousarray(np.transpose(x, inv))
    out["ncases"] = len(cases)
    np.savez(os.path.join(HERE, "permute.npz"), **out)


def gen_rng():
    ords = np.asarray([0, 1, 2, 3, 1000, 123456789, 2 ** 40 + 7], np.uint64)
    np.savez(os.path.join(HERE, "rng.npz"), ordinals=ords,
             hash_s1_t2=hash_(1, 2, ords), uniform_s1_t2=values(1, 2, ords, 0),
             int101_s7_t0=values(7, 0, ords, 1))


def sparse_keep(tr, seed, stream):
    """make_random_sparseshape (expressions_fixture.h:216-230): each tile kept
    with probability 1/2."""
    n = int(np.prod([len(h) - 1 for h in tr]))
    h = hash_(seed, stream, np.arange(n, dtype=np.uint64))
    return (((h >> U64(33)) & U64(1)) == U64(0)).reshape([len(x) - 1 for x in tr])


CONTRACTIONS = [
    # name, c, a, b, alpha, trange of a (list of hashmarks per index), of b
    ("cont", "i,j", "i,b,c", "j,b,c", 1.0, "tr3", "tr3"),
    ("cont_permute", "i,j", "i,b,c", "j,c,b", 1.0, "tr3", "tr3"),
    ("cont_permute_permute", "i,j", "j,b,c", "i,c,b", 1.0, "tr3", "tr3"),
    ("scale_cont", "i,j", "i,b,c", "j,b,c", 30.0, "tr3", "tr3"),
    ("cont_non_uniform1", "x,y", "x,i,j,k", "y,i,j,k", 5.0, "nu1", "nu1"),
    ("cont_non_uniform2", "x,y", "x,i,j,k", "y,i,j,k", 5.0, "nu2", "nu2"),
    ("outer_product", "i,j", "i", "j", 1.0, "tr1", "tr1"),
    ("matmul", "i,j", "i,k", "k,j", 1.0, "tr2", "tr2"),
    ("matmul_tt", "i,j", "k,i", "j,k", 1.0, "tr2", "tr2"),
    ("abcd", "a,b,i,j", "a,b,c,d", "c,d,i,j", 1.0, "tr4", "tr4"),
    ("abcd_general", "a,b,i,j", "a,c,b,d", "c,d,i,j", 1.0, "tr4", "tr4"),
    ("abcd_result_perm", "i,j,a,b", "a,b,c,d", "c,d,i,j", 2.0, "tr4", "tr4"),
]

TRANGES = {
    "tr3": [hashmarks_primes()] * 3,
    "tr2": [[0, 2, 5, 10, 17, 28, 41], [0, 3, 6, 11, 18, 29, 42]],
    "tr1": [[0, 2, 5, 10, 17, 28, 41]],
    "nu1": [[0, 1, 2, 3, 4, 5], [0, 40], [0, 1, 2, 3, 4, 5], [0, 1, 2, 3, 4, 5]],
    "nu2": [[0, 1, 2, 3, 4, 5], [0, 1, 2, 3, 4, 5], [0, 40], [0, 40]],
    "tr4": [[0, 3, 7, 8], [0, 2, 6], [0, 3, 7, 8], [0, 2, 6]],
}


def gen_contractions():
    meta = []
    for sparse in (False, True):
        for (name, c, a, b, alpha, ta_, tb_) in CONTRACTIONS:
            ai, bi, ci = a.split(","), b.split(","), c.split(",")
            tra = TRANGES[ta_]
            trb = TRANGES[tb_]
            if name == "matmul_tt":
                tra = [TRANGES["tr2"][1], TRANGES["tr2"][0]]
                trb = [TRANGES["tr2"][0], TRANGES["tr2"][1]]
            if name == "matmul":
                trb = [TRANGES["tr2"][1], TRANGES["tr2"][0]]
            if name == "abcd_general":
                tra = [TRANGES["tr4"][0], TRANGES["tr4"][0], TRANGES["tr4"][1], TRANGES["tr4"][1]]
                trb = [TRANGES["tr4"][0], TRANGES["tr4"][1], TRANGES["tr4"][0], TRANGES["tr4"][1]]
            ext_a = [h[-1] - h[0] for h in tra]
            ext_b = [h[-1] - h[0] for h in trb]
            A = dense_operand(ext_a, 23, 0, kind=1)
            B = dense_operand(ext_b, 42, 1, kind=1)
            keep_a = keep_b = None
            if sparse:
                keep_a = sparse_keep(tra, 5, 0)
                keep_b = sparse_keep(trb, 5, 1)

                def mask(X, tr, keep):
                    X = X.copy()
                    for o in range(keep.size):
                        if keep.ravel()[o]:
                            continue
                        idx = np.unravel_index(o, keep.shape)
                        X[tuple(slice(tr[d][idx[d]], tr[d][idx[d] + 1])
                                for d in range(len(tr)))] = 0.0
                    return X
                A = mask(A, tra, keep_a)
                B = mask(B, trb, keep_b)
            letters = {}
            for v in ai + bi:
                if v not in letters:
                    letters[v] = chr(ord("a") + len(letters))
            es = "".join(letters[v] for v in ai) + "," + "".join(letters[v] for v in bi) + \
                "->" + "".join(letters[v] for v in ci)
            Cx = alpha * np.einsum(es, A, B)
            tag = ("sparse_" if sparse else "dense_") + name
            np.savez_compressed(os.path.join(HERE, f"contract_{tag}.npz"), expected=Cx)
            meta.append(dict(tag=tag, c=c, a=a, b=b, alpha=alpha, trange_a=tra, trange_b=trb,
                             seed_a=[23, 0], seed_b=[42, 1], kind=1, sparse=sparse,
                             keep_a=None if keep_a is None else keep_a.ravel().astype(int).tolist(),
                             keep_b=None if keep_b is None else keep_b.ravel().astype(int).tolist()))
    with open(os.path.join(HERE, "contractions.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    gen_rng()
    gen_scale_norms()
    gen_shape_gemm()
    gen_pairs()
    gen_permute()
    gen_contractions()
    print("golden fixtures written to", HERE)
