"""CPU oracle for the block-sparse contraction path (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package, and only as the checker.  The product library never calls
it.

It restates TiledArray's algorithm for ``C(c) = alpha * A(a) * B(b)`` on
block-sparse arrays, step by step, each step citing the reference file it
follows (paths relative to the TiledArray source tree):

* ``permopt``           expressions/permopt.h:258-396 (layout choice),
                        expressions/binary_engine.h:101-176 (permtypes)
* ``scale_norms``       sparse_shape.h:150-215, 407-422 (SparseShape ctor)
* ``shape_gemm``        sparse_shape.h:1589-1684
* ``pairs``             dist_eval/contraction_eval.h:630-650, 1093-1161, 1348-1384
* ``permute``           tensor/permute.h:124-210, permutation.h:60-78
* ``contract_tiles``    tile_op/contract_reduce.h:367-452, tensor/tensor.h:3132-3210
* ``tile_norm``         tensor/tensor.h:3768-3787, math/vector_op.h:561-577

The heavy loops live in ``liboracle.so`` (oracle.cpp, built by
``oracle/build.py``), compiled with -ffp-contract=off.
"""
from __future__ import annotations

import ctypes
import glob
import os
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)

DGEMM_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                            ctypes.c_double, _f64p, ctypes.c_int64, _f64p,
                            ctypes.c_int64, ctypes.c_double, _f64p,
                            ctypes.c_int64)

FLT_EPSILON = float(np.finfo(np.float32).eps)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build as _b
            _b.build()
        L = ctypes.CDLL(path)
        L.orc_hash.restype = ctypes.c_uint64
        L.orc_hash.argtypes = [ctypes.c_uint64] * 3
        L.orc_uniform.restype = ctypes.c_double
        L.orc_uniform.argtypes = [ctypes.c_uint64] * 3
        L.orc_fill_tile.argtypes = [ctypes.c_int, _i64p, _i64p, _i64p,
                                    ctypes.c_uint64, ctypes.c_uint64,
                                    ctypes.c_int, ctypes.c_double, _f64p]
        L.orc_tile_norm.restype = ctypes.c_float
        L.orc_tile_norm.argtypes = [ctypes.c_int64, _f64p]
        L.orc_scale_norms.restype = ctypes.c_int64
        L.orc_scale_norms.argtypes = [ctypes.c_int, _i64p, _f32p, ctypes.c_float, _f32p]
        L.orc_outer_sizes.argtypes = [ctypes.c_int, _i64p, _f32p, ctypes.c_int, _f32p]
        L.orc_shape_gemm.restype = ctypes.c_int64
        L.orc_shape_gemm.argtypes = [ctypes.c_int64] * 3 + [_f32p, _f32p, _f32p,
                                                            ctypes.c_double, ctypes.c_float, _f32p]
        L.orc_pairs.restype = ctypes.c_int64
        L.orc_pairs.argtypes = [ctypes.c_int64] * 3 + [_f32p, ctypes.c_float, _f32p,
                                                       ctypes.c_float, _f32p, ctypes.c_float,
                                                       _i64p, _i32p]
        L.orc_permute_f64.argtypes = [ctypes.c_int, _i64p, _i32p, _f64p, _f64p]
        L.orc_permute_f32.argtypes = [ctypes.c_int, _i64p, _i32p, _f32p, _f32p]
        cargs = [ctypes.c_int64] * 3 + [_i64p, _i64p, _i64p, _f64p, _i64p, ctypes.c_int,
                                        _f64p, _i64p, ctypes.c_int, _i64p, _i32p,
                                        ctypes.c_double, _f64p, _i64p]
        L.orc_contract.argtypes = cargs + [ctypes.c_int, ctypes.c_void_p]
        L.orc_contract_subset.argtypes = cargs + [_i64p, ctypes.c_int64, ctypes.c_int,
                                                  ctypes.c_void_p]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(t)


# ----------------------------------------------------------------------------
# generator
# ----------------------------------------------------------------------------

def uniform(seed: int, stream: int, ordinal: int) -> float:
    return lib().orc_uniform(seed, stream, ordinal)


def fill_tile(lo, hi, global_extent, seed, stream, kind=0, scale=1.0):
    rank = len(lo)
    lo_a = np.asarray(lo, dtype=np.int64)
    hi_a = np.asarray(hi, dtype=np.int64)
    ge = np.asarray(global_extent, dtype=np.int64)
    out = np.empty(int(np.prod(hi_a - lo_a)), dtype=np.float64)
    lib().orc_fill_tile(rank, _p(lo_a, _i64p), _p(hi_a, _i64p), _p(ge, _i64p),
                        seed, stream, kind, scale, _p(out, _f64p))
    return out.reshape(tuple(hi_a - lo_a))


def tile_norm(x: np.ndarray) -> np.float32:
    x = np.ascontiguousarray(x, dtype=np.float64).ravel()
    return np.float32(lib().orc_tile_norm(x.size, _p(x, _f64p)))


# ----------------------------------------------------------------------------
# tilings and shapes
# ----------------------------------------------------------------------------

@dataclass
class TiledRange:
    """Per-dimension tile boundaries (TiledRange1 hashmarks)."""
    dims: list

    @property
    def rank(self):
        return len(self.dims)

    def ntiles(self):
        return [len(h) - 1 for h in self.dims]

    def extents(self):
        return [h[-1] - h[0] for h in self.dims]

    def tile_sizes(self, d):
        h = self.dims[d]
        return [h[i + 1] - h[i] for i in range(len(h) - 1)]

    def tile_lo_hi(self, idx):
        lo = [self.dims[d][idx[d]] for d in range(self.rank)]
        hi = [self.dims[d][idx[d] + 1] for d in range(self.rank)]
        return lo, hi

    def tile_index(self, ordinal):
        idx = []
        for n in reversed(self.ntiles()):
            idx.append(ordinal % n)
            ordinal //= n
        return list(reversed(idx))

    def permuted(self, perm):
        out = [None] * self.rank
        for d in range(self.rank):
            out[perm[d]] = self.dims[d]
        return TiledRange(out)


def size_vectors(tr: TiledRange):
    return np.concatenate([np.asarray(tr.tile_sizes(d), dtype=np.float32)
                           for d in range(tr.rank)]) if tr.rank else np.zeros(0, np.float32)


def scale_norms(tr: TiledRange, norms: np.ndarray, threshold: float):
    """SparseShape(tile_norms, trange): scale by inverse volume, screen."""
    n = np.ascontiguousarray(norms, dtype=np.float32).copy()
    nt = np.asarray(tr.ntiles(), dtype=np.int64)
    sv = size_vectors(tr)
    z = lib().orc_scale_norms(tr.rank, _p(nt, _i64p), _p(sv, _f32p),
                              np.float32(threshold), _p(n, _f32p))
    return n.reshape(tr.ntiles()), int(z)


def outer_sizes(tr_dims_ntiles, sizes, inverse=False):
    nt = np.asarray(tr_dims_ntiles, dtype=np.int64)
    sv = np.ascontiguousarray(sizes, dtype=np.float32)
    out = np.empty(int(np.prod(nt)) if len(nt) else 1, dtype=np.float32)
    lib().orc_outer_sizes(len(nt), _p(nt, _i64p), _p(sv, _f32p), int(inverse),
                          _p(out, _f32p))
    return out


def shape_gemm(left, right, k_sizes, factor, threshold):
    """SparseShape::gemm on GEMM-order norm matrices (M x K, K x N)."""
    left = np.ascontiguousarray(left, dtype=np.float32)
    right = np.ascontiguousarray(right, dtype=np.float32)
    M = left.shape[0]
    N = right.shape[1] if right.ndim == 2 else right.shape[0]
    K = 0 if k_sizes is None else len(k_sizes)
    ks = np.ascontiguousarray(k_sizes if k_sizes is not None else np.zeros(1), dtype=np.float32)
    out = np.empty((M, N), dtype=np.float32)
    z = lib().orc_shape_gemm(M, N, K, _p(left, _f32p), _p(right, _f32p), _p(ks, _f32p),
                             float(factor), np.float32(threshold), _p(out, _f32p))
    return out, int(z)


def pairs(cnorm, c_thr, lnorm, l_thr, rnorm, r_thr):
    cnorm = np.ascontiguousarray(cnorm, dtype=np.float32)
    lnorm = np.ascontiguousarray(lnorm, dtype=np.float32)
    rnorm = np.ascontiguousarray(rnorm, dtype=np.float32)
    M, N = cnorm.shape
    K = lnorm.shape[1]
    offsets = np.empty(M * N + 1, dtype=np.int64)
    n = lib().orc_pairs(M, N, K, _p(cnorm, _f32p), np.float32(c_thr), _p(lnorm, _f32p),
                        np.float32(l_thr), _p(rnorm, _f32p), np.float32(r_thr),
                        _p(offsets, _i64p), None)
    kidx = np.empty(max(n, 1), dtype=np.int32)
    lib().orc_pairs(M, N, K, _p(cnorm, _f32p), np.float32(c_thr), _p(lnorm, _f32p),
                    np.float32(l_thr), _p(rnorm, _f32p), np.float32(r_thr),
                    _p(offsets, _i64p), _p(kidx, _i32p))
    return offsets, kidx[:n]


def permute(x: np.ndarray, perm):
    """result dim perm[d] = argument dim d."""
    x = np.ascontiguousarray(x)
    ext = np.asarray(x.shape, dtype=np.int64)
    p = np.asarray(perm, dtype=np.int32)
    rshape = [0] * x.ndim
    for d in range(x.ndim):
        rshape[perm[d]] = x.shape[d]
    out = np.empty(rshape, dtype=x.dtype)
    if x.size == 0:
        return out
    if x.dtype == np.float64:
        lib().orc_permute_f64(x.ndim, _p(ext, _i64p), _p(p, _i32p), _p(x, _f64p), _p(out, _f64p))
    elif x.dtype == np.float32:
        lib().orc_permute_f32(x.ndim, _p(ext, _i64p), _p(p, _i32p), _p(x, _f32p), _p(out, _f32p))
    else:
        raise TypeError(x.dtype)
    return out


# ----------------------------------------------------------------------------
# permutation optimizer (expressions/permopt.h:258-396)
# ----------------------------------------------------------------------------

IDENTITY, MATRIX_TRANSPOSE, GENERAL = 1, 2, 3


def parse_indices(s: str):
    return [t.strip() for t in s.split(",")] if s.strip() else []


def permopt(left, right, prefer_left=True):
    """Returns (left_target, right_target, result, left_permtype, right_permtype)."""
    lr, rr = len(left), len(right)
    res_left, res_right, result = [], [], []
    for v in left:
        if v not in right:
            res_left.append(v)
            result.append(v)
        else:
            res_right.append(v)
    inner = len(res_right)
    lo = len(res_left)
    ro = rr - inner
    if inner == 0:
        for v in right:
            res_right.append(v)
            result.append(v)
        return res_left, res_right, result, GENERAL, GENERAL
    ordered = lnt = lt = rnt = rt = True
    perm_left = lr < rr or (lr == rr and prefer_left)
    for i, idx in enumerate(right):
        j = left.index(idx) if idx in left else lr
        if j == lr:
            res_right.append(idx)
            result.append(idx)
            continue
        x = len(res_left) - lo
        ordered = ordered and res_right[x] == idx
        lnt = lnt and j >= lo
        lt = lt and j < inner
        rnt = rnt and i < inner
        rt = rt and i >= ro
        if ordered:
            res_left.append(idx)
        elif perm_left:
            res_left.append(idx)
            res_right[x] = idx
            lnt = lt = False
        else:
            res_left.append(res_right[x])
            rnt = rt = False

    def op(nt, t):
        return IDENTITY if nt else (MATRIX_TRANSPOSE if t else GENERAL)

    return res_left, res_right, result, op(lnt, lt), op(rnt, rt)


def perm_between(src, dst):
    """Permutation p with result dim p[d] = argument dim d mapping src -> dst."""
    return [dst.index(v) for v in src]


# ----------------------------------------------------------------------------
# block-sparse array and the full contraction pipeline
# ----------------------------------------------------------------------------

@dataclass
class Array:
    """Single-process block-sparse array: tiling, scaled norms, tiles."""
    tr: TiledRange
    norms: np.ndarray            # scaled per-element norms over the tile grid
    threshold: float             # the shape's own threshold (my_threshold_)
    tiles: dict = field(default_factory=dict)  # ordinal -> ndarray (tile shape)

    def is_zero(self, ordinal):
        return self.norms.ravel()[ordinal] < self.threshold

    def to_dense(self):
        out = np.zeros(self.tr.extents(), dtype=np.float64)
        for o, t in self.tiles.items():
            idx = self.tr.tile_index(o)
            lo, hi = self.tr.tile_lo_hi(idx)
            out[tuple(slice(lo[d] - self.tr.dims[d][0], hi[d] - self.tr.dims[d][0])
                      for d in range(self.tr.rank))] = t
        return out

    def permuted(self, perm):
        ntr = self.tr.permuted(perm)
        nn = permute(self.norms.astype(np.float32), perm)
        out = Array(ntr, nn, self.threshold)
        for o, t in self.tiles.items():
            idx = self.tr.tile_index(o)
            nidx = [0] * len(idx)
            for d in range(len(idx)):
                nidx[perm[d]] = idx[d]
            no = int(np.ravel_multi_index(nidx, ntr.ntiles()))
            out.tiles[no] = permute(t, perm)
        return out


def make_array(tr: TiledRange, seed: int, stream: int, kind=0, tile_scale=None,
               keep=None, threshold=FLT_EPSILON):
    """make_array semantics (conversions/make_array.h:151-199): fill each kept
    tile, take its norm, build the SparseShape from the norms."""
    nt = tr.ntiles()
    ntot = int(np.prod(nt)) if nt else 1
    norms = np.zeros(ntot, dtype=np.float32)
    tiles = {}
    ge = tr.extents()
    for o in range(ntot):
        idx = tr.tile_index(o)
        if keep is not None and not keep(idx):
            continue
        lo, hi = tr.tile_lo_hi(idx)
        sc = 1.0 if tile_scale is None else tile_scale(idx)
        t = fill_tile([l - tr.dims[d][0] for d, l in enumerate(lo)],
                      [h - tr.dims[d][0] for d, h in enumerate(hi)], ge, seed, stream, kind, sc)
        tiles[o] = t
        norms[o] = tile_norm(t)
    scaled, _ = scale_norms(tr, norms.reshape(nt), threshold)
    flat = scaled.ravel()
    kept = {o: t for o, t in tiles.items() if flat[o] >= threshold}
    return Array(tr, scaled, threshold, kept)


def contract(c_idx: str, A: Array, a_idx: str, B: Array, b_idx: str, alpha=1.0,
             threshold=FLT_EPSILON, use_blas=None, nthreads=0, return_pairs=False):
    """C(c_idx) = alpha * A(a_idx) * B(b_idx) as TiledArray evaluates it."""
    ai, bi, ci = parse_indices(a_idx), parse_indices(b_idx), parse_indices(c_idx)
    lt, rt, res, lop, rop = permopt(ai, bi, True)
    inner = (len(ai) + len(bi) - len(res)) // 2
    lorank = len(ai) - inner
    # shapes always go to GEMM order (leaf_engine.h:169, sparse_shape.h:1222)
    lperm = perm_between(ai, lt)
    rperm = perm_between(bi, rt)
    ln = permute(A.norms.astype(np.float32), lperm)
    rn = permute(B.norms.astype(np.float32), rperm)
    ltr = A.tr.permuted(lperm)
    rtr = B.tr.permuted(rperm)
    lnt = ltr.ntiles()
    rnt = rtr.ntiles()
    Mt = int(np.prod(lnt[:lorank])) if lorank else 1
    Kt = int(np.prod(lnt[lorank:])) if inner else 1
    Nt = int(np.prod(rnt[inner:])) if len(rt) > inner else 1
    # k sizes: recursive outer product of the contracted size vectors
    ksv = np.concatenate([np.asarray(ltr.tile_sizes(d), np.float32)
                          for d in range(lorank, ltr.rank)]) if inner else None
    ks = outer_sizes(lnt[lorank:], ksv, False) if inner else None
    cn, zc = shape_gemm(ln.reshape(Mt, Kt if inner else 1), rn.reshape(Kt if inner else 1, Nt),
                        ks, alpha, threshold)
    # pair set (Summa)
    offs, kidx = pairs(cn, threshold, ln.reshape(Mt, -1), A.threshold,
                       rn.reshape(-1, Nt), B.threshold)
    # tile data in GEMM order: general permtype -> explicit permute; identity /
    # matrix_transpose -> fused into the GEMM (binary_engine.h:159-175)
    if lop == GENERAL:
        Al = A.permuted(lperm)
        left_trans = 0
        lord = lambda m, k: m * Kt + k
        Ltr = ltr
    else:
        Al = A
        left_trans = 1 if lop == MATRIX_TRANSPOSE else 0
        lord = (lambda m, k: k * Mt + m) if left_trans else (lambda m, k: m * Kt + k)
    if rop == GENERAL:
        Br = B.permuted(rperm)
        right_trans = 0
        rord = lambda k, n: k * Nt + n
    else:
        Br = B
        right_trans = 1 if rop == MATRIX_TRANSPOSE else 0
        rord = (lambda k, n: n * Kt + k) if right_trans else (lambda k, n: k * Nt + n)
    # fused tile sizes
    def fused(tr, dims):
        sizes = [np.asarray(tr.tile_sizes(d), np.int64) for d in dims]
        if not sizes:
            return np.ones(1, np.int64)
        out = sizes[0]
        for s in sizes[1:]:
            out = np.outer(out, s).ravel()
        return out
    msz = fused(ltr, range(lorank))
    ksz = fused(ltr, range(lorank, ltr.rank)) if inner else np.ones(1, np.int64)
    nsz = fused(rtr, range(inner, rtr.rank))
    # pack tiles
    lbuf, loff = [], np.full(Mt * max(Kt, 1), -1, np.int64)
    pos = 0
    for m in range(Mt):
        for k in range(Kt):
            t = Al.tiles.get(lord(m, k))
            if t is not None:
                loff[m * Kt + k] = pos
                lbuf.append(t.ravel())
                pos += t.size
    rbuf, roff = [], np.full(max(Kt, 1) * Nt, -1, np.int64)
    pos = 0
    for k in range(Kt):
        for n in range(Nt):
            t = Br.tiles.get(rord(k, n))
            if t is not None:
                roff[k * Nt + n] = pos
                rbuf.append(t.ravel())
                pos += t.size
    lbuf = np.concatenate(lbuf) if lbuf else np.zeros(1)
    rbuf = np.concatenate(rbuf) if rbuf else np.zeros(1)
    res_off = np.full(Mt * Nt, -1, np.int64)
    pos = 0
    flat_cn = cn.ravel()
    for t in range(Mt * Nt):
        if flat_cn[t] >= threshold:
            res_off[t] = pos
            pos += int(msz[t // Nt] * nsz[t % Nt])
    cbuf = np.zeros(max(pos, 1), np.float64)
    fn = None
    if use_blas:
        fn = DGEMM_FN(use_blas) if not isinstance(use_blas, DGEMM_FN) else use_blas
    lib().orc_contract(Mt, Nt, Kt, _p(msz, _i64p), _p(nsz, _i64p), _p(ksz, _i64p),
                       _p(lbuf, _f64p), _p(loff, _i64p), left_trans, _p(rbuf, _f64p),
                       _p(roff, _i64p), right_trans, _p(offs, _i64p), _p(kidx, _i32p),
                       float(alpha), _p(cbuf, _f64p), _p(res_off, _i64p), nthreads,
                       ctypes.cast(fn, ctypes.c_void_p) if fn else None)
    # result array in "res" order, then post-permute to the target
    rtr_res = TiledRange([ltr.dims[d] for d in range(lorank)] +
                         [rtr.dims[d] for d in range(inner, rtr.rank)])
    C = Array(rtr_res, cn.reshape(rtr_res.ntiles()) if rtr_res.rank else cn, threshold)
    for t in range(Mt * Nt):
        if res_off[t] >= 0:
            idx = rtr_res.tile_index(t)
            lo, hi = rtr_res.tile_lo_hi(idx)
            shp = [hi[d] - lo[d] for d in range(rtr_res.rank)]
            C.tiles[t] = cbuf[res_off[t]:res_off[t] + int(np.prod(shp))].reshape(shp).copy()
    if res != ci:
        C = C.permuted(perm_between(res, ci))
    if return_pairs:
        return C, dict(Mt=Mt, Nt=Nt, Kt=Kt, offsets=offs, kidx=kidx, cnorm=cn,
                       zero_count=zc, left_permtype=lop, right_permtype=rop,
                       left_target=lt, right_target=rt, result=res)
    return C


def general_contract(c_idx: str, A: Array, a_idx: str, B: Array, b_idx: str, alpha=1.0,
                     threshold=FLT_EPSILON, return_pairs=False):
    """General (fused-index) product as TiledArray evaluates it
    (ContEngine::init_struct_general; SparseShape::gemm_batched,
    sparse_shape.h:1707-1885): indices in both arguments and the target are
    fused, in both arguments only contracted, in one argument and the target
    free.  Arguments are permuted to (fused, left free, contracted) and
    (fused, contracted, right free); every fused-tile slab is screened and
    contracted as gemm does (same k sizes, no fused-size scaling; outer
    product norms left*right*|alpha| without contracted modes); each fused
    element of a slab's tiles is its own matrix product."""
    ai, bi, ci = parse_indices(a_idx), parse_indices(b_idx), parse_indices(c_idx)
    F = [x for x in ai if x in bi and x in ci]
    K = [x for x in ai if x in bi and x not in ci]
    L = [x for x in ai if x not in bi and x in ci]
    R = [x for x in bi if x not in ai and x in ci]
    lperm = perm_between(ai, F + L + K)
    rperm = perm_between(bi, F + K + R)
    Al, Br = A.permuted(lperm), B.permuted(rperm)
    ltr, rtr = Al.tr, Br.tr
    nf, nl, nk = len(F), len(L), len(K)
    lnt, rnt = ltr.ntiles(), rtr.ntiles()
    Ht = int(np.prod(lnt[:nf]))
    Mt = int(np.prod(lnt[nf:nf + nl])) if nl else 1
    Kt = int(np.prod(lnt[nf + nl:])) if nk else 1
    Nt = int(np.prod(rnt[nf + nk:])) if len(R) else 1
    ln = Al.norms.astype(np.float32).reshape(Ht, Mt, Kt)
    rn = Br.norms.astype(np.float32).reshape(Ht, Kt, Nt)
    ks = None
    if nk:
        ksv = np.concatenate([np.asarray(ltr.tile_sizes(d), np.float32)
                              for d in range(nf + nl, ltr.rank)])
        ks = outer_sizes(lnt[nf + nl:], ksv, False)
    cn = np.zeros((Ht, Mt, Nt), np.float32)
    zc = 0
    offs_all, kidx_all, base = [], [], 0
    for h in range(Ht):
        c_h, z_h = shape_gemm(ln[h], rn[h], ks, alpha, threshold)
        cn[h] = c_h
        zc += z_h
        o_h, k_h = pairs(c_h, threshold, ln[h], A.threshold, rn[h], B.threshold)
        offs_all.append(o_h[:-1] + base)
        kidx_all.append(k_h)
        base += int(o_h[-1])
    offs = np.concatenate(offs_all + [np.asarray([base], np.int64)]).astype(np.int64)
    kidx = np.concatenate(kidx_all).astype(np.int32) if kidx_all else np.zeros(0, np.int32)
    res_tr = TiledRange([ltr.dims[d] for d in range(nf + nl)] +
                        [rtr.dims[d] for d in range(nf + nk, rtr.rank)])
    C = Array(res_tr, cn.reshape(res_tr.ntiles()), threshold)
    for h in range(Ht):
        for t in range(Mt * Nt):
            if cn[h].ravel()[t] < threshold:
                continue
            i, j = divmod(t, Nt)
            o = (h * Mt + i) * Nt + j
            lo, hi = res_tr.tile_lo_hi(res_tr.tile_index(o))
            shp = [hi[d] - lo[d] for d in range(res_tr.rank)]
            he = int(np.prod(shp[:nf]))
            m = int(np.prod(shp[nf:nf + nl])) if nl else 1
            n = int(np.prod(shp[nf + nl:])) if len(R) else 1
            acc = np.zeros((he, m, n))
            for p in range(int(offs[o]), int(offs[o + 1])):
                k = int(kidx[p])
                ta = Al.tiles.get((h * Mt + i) * Kt + k)
                tb = Br.tiles.get((h * Kt + k) * Nt + j)
                if ta is None or tb is None:
                    continue
                acc += ta.reshape(he, m, -1) @ tb.reshape(he, -1, n)
            C.tiles[o] = (alpha * acc).reshape(shp)
    res = F + L + R
    if res != ci:
        C = C.permuted(perm_between(res, ci))
    if return_pairs:
        return C, dict(Ht=Ht, Mt=Mt, Nt=Nt, Kt=Kt, offsets=offs, kidx=kidx, cnorm=cn,
                       zero_count=zc)
    return C


def openblas_dgemm():
    """Address of numpy's bundled ILP64 cblas_dgemm, or None."""
    import numpy
    d = os.path.dirname(numpy.__file__)
    cands = glob.glob(os.path.join(d, "..", "numpy.libs", "libscipy_openblas64_*.so")) + \
        glob.glob(os.path.join(d, ".libs", "libscipy_openblas64_*.so"))
    for c in cands:
        try:
            L = ctypes.CDLL(c)
            fn = L.scipy_cblas_dgemm64_
            for setter in ("scipy_openblas_set_num_threads64_", "openblas_set_num_threads64_"):
                if hasattr(L, setter):
                    getattr(L, setter)(1)
                    break
            return ctypes.cast(fn, ctypes.c_void_p).value
        except (OSError, AttributeError):
            continue
    return None
