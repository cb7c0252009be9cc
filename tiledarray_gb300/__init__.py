"""tiledarray_gb300 — Python mirror of TiledArray's block-sparse contraction API
over the tagpu C ABI (libtagpu.so, built in-tree for sm_103a).

    import tiledarray_gb300 as ta
    world = ta.World()                               # TA::initialize
    tr = ta.TiledRange([[0, 2, 5, 10], [0, 3, 6]])   # TiledRange of TiledRange1
    A = ta.TSpArrayD(world, tr, norms)               # DistArray + SparseShape
    A.set_tiles(tiles)                               # DistArray::set
    C = ta.TSpArrayD(world)
    C["i,j"] = A["i,k"] * B["k,j"]                   # TsrExpr::operator=
    C["i,j"] = 5 * (A["i,k"] * B["k,j"])             # scaled contraction

The compute path is the CUDA library only: importing this package on a
machine without libtagpu.so raises, and every operation goes through
tagpu_* entry points.  Errors are raised as TAGPUError carrying the
library's status and message (TiledArray raises TiledArray::Exception).
"""
from __future__ import annotations

import ctypes
import os
import weakref

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtagpu.so")

PRECISION_FP64 = 0
PRECISION_OZAKI = 1
FLT_EPSILON = float(np.finfo(np.float32).eps)

_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p

STATUS = {0: "ok", 1: "invalid argument", 2: "unsupported", 3: "out of device memory",
          4: "CUDA error", 5: "timeout", 6: "rejected", 7: "not ready", 8: "bad state"}


class TAGPUError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"tagpu status {status} ({STATUS.get(status, '?')}): {msg}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("hbm_budget_bytes", ctypes.c_size_t)]


class ArrayInfo(ctypes.Structure):
    _fields_ = [("rank", ctypes.c_int), ("dense", ctypes.c_int),
                ("ntiles_total", ctypes.c_int64), ("nonzero_tiles", ctypes.c_int64),
                ("zero_tiles", ctypes.c_int64), ("elements", ctypes.c_int64),
                ("threshold", ctypes.c_float), ("device_bytes", ctypes.c_size_t),
                ("ntiles", ctypes.c_int64 * 8)]


class ContractOpts(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int), ("slices", ctypes.c_int),
                ("threshold", ctypes.c_float), ("autotune", ctypes.c_int)]


class ContractStats(ctypes.Structure):
    _fields_ = [("result_tiles", ctypes.c_int64), ("nonzero_result_tiles", ctypes.c_int64),
                ("zero_tiles", ctypes.c_int64), ("pairs", ctypes.c_int64),
                ("flops", ctypes.c_double), ("ms_shape", ctypes.c_double),
                ("ms_pairs", ctypes.c_double), ("ms_permute", ctypes.c_double),
                ("ms_split", ctypes.c_double), ("ms_gemm", ctypes.c_double),
                ("ms_total", ctypes.c_double), ("left_permtype", ctypes.c_int),
                ("right_permtype", ctypes.c_int), ("precision", ctypes.c_int),
                ("slices", ctypes.c_int), ("gemm_blocks", ctypes.c_int64),
                ("gemm_launches", ctypes.c_int64), ("kernel_launches", ctypes.c_int64),
                ("mma_flops", ctypes.c_double)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_size_t), ("max_batch", ctypes.c_int),
                ("precision", ctypes.c_int), ("slices", ctypes.c_int)]


class Request(ctypes.Structure):
    _fields_ = [("c_idx", ctypes.c_char_p), ("alpha", ctypes.c_double), ("A", _vp),
                ("a_idx", ctypes.c_char_p), ("B", _vp), ("b_idx", ctypes.c_char_p),
                ("precision", ctypes.c_int), ("slices", ctypes.c_int)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("latency_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("flops", ctypes.c_double),
                ("pairs", ctypes.c_int64), ("batch_size", ctypes.c_int),
                ("batch_id", ctypes.c_uint64)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_int64), ("completed", ctypes.c_int64),
                ("rejected", ctypes.c_int64), ("failed", ctypes.c_int64),
                ("batches", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("mean_ms", ctypes.c_double),
                ("flops", ctypes.c_double), ("wall_ms", ctypes.c_double),
                ("bytes_in_use", ctypes.c_size_t), ("peak_bytes", ctypes.c_size_t)]

    def as_dict(self):
        return {f: getattr(self, f) for f, _ in self._fields_}


_L = None

# name -> (restype, argtypes); every symbol include/tagpu.h declares
SIGNATURES = {
    "tagpu_init": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_vp)]),
    "tagpu_shutdown": (ctypes.c_int, [_vp]),
    "tagpu_last_error": (ctypes.c_char_p, [_vp]),
    "tagpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "tagpu_sync": (ctypes.c_int, [_vp]),
    "tagpu_timer_start": (ctypes.c_int, [_vp]),
    "tagpu_device_fp64_rates": (ctypes.c_int, [_vp, _f64p, _f64p]),
    "tagpu_device_mma_sync_rates": (ctypes.c_int, [_vp, _f64p, _f64p]),
    "tagpu_timer_stop": (ctypes.c_int, [_vp, _f64p]),
    "tagpu_threshold_get": (ctypes.c_float, [_vp]),
    "tagpu_threshold_set": (None, [_vp, ctypes.c_float]),
    "tagpu_set_wait_limit": (ctypes.c_int, [_vp, ctypes.c_double]),
    "tagpu_array_create": (ctypes.c_int, [_vp, ctypes.c_int, _i64p,
                                          ctypes.POINTER(_i64p), ctypes.POINTER(_vp)]),
    "tagpu_array_destroy": (ctypes.c_int, [_vp]),
    "tagpu_array_set_shape": (ctypes.c_int, [_vp, _f32p, ctypes.c_int, ctypes.c_float]),
    "tagpu_array_upload": (ctypes.c_int, [_vp, _f64p, ctypes.c_int64]),
    "tagpu_array_download": (ctypes.c_int, [_vp, _f64p, ctypes.c_int64]),
    "tagpu_array_generate": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int,
                                            _f64p, ctypes.c_int, ctypes.c_float]),
    "tagpu_array_get_info": (ctypes.c_int, [_vp, ctypes.POINTER(ArrayInfo)]),
    "tagpu_array_get_norms": (ctypes.c_int, [_vp, _f32p]),
    "tagpu_array_get_tile_offsets": (ctypes.c_int, [_vp, _i64p]),
    "tagpu_array_get_tile": (ctypes.c_int, [_vp, ctypes.c_int64, _f64p, ctypes.c_int64]),
    "tagpu_array_truncate": (ctypes.c_int, [_vp, ctypes.c_float]),
    "tagpu_array_save": (ctypes.c_int, [_vp, ctypes.c_char_p]),
    "tagpu_host_alloc": (ctypes.c_int, [_vp, ctypes.c_size_t, ctypes.POINTER(_vp)]),
    "tagpu_host_free": (ctypes.c_int, [_vp, _vp]),
    "tagpu_array_load": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.POINTER(_vp)]),
    "tagpu_array_serialize": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_uint64,
                                             ctypes.c_uint64]),
    "tagpu_array_deserialize": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int,
                                               ctypes.POINTER(_vp),
                                               ctypes.POINTER(ctypes.c_uint64),
                                               ctypes.POINTER(ctypes.c_uint64)]),
    "tagpu_contract_accumulate": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, _vp,
                                                 ctypes.c_char_p, _vp, ctypes.c_char_p, _vp,
                                                 _vp]),
    "tagpu_array_get_hashmarks": (ctypes.c_int, [_vp, ctypes.c_int, _i64p]),
    "tagpu_contract": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, _vp,
                                      ctypes.c_char_p, _vp, ctypes.c_char_p,
                                      ctypes.POINTER(ContractOpts), ctypes.POINTER(_vp)]),
    "tagpu_last_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ContractStats)]),
    "tagpu_shape_gemm": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                        _f32p, _f32p, _f32p, ctypes.c_double, ctypes.c_float,
                                        _f32p, _i64p]),
    "tagpu_pair_list": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                       _f32p, ctypes.c_float, _f32p, ctypes.c_float, _f32p,
                                       ctypes.c_float, _i64p, _i32p, ctypes.c_int64, _i64p]),
    "tagpu_permute": (ctypes.c_int, [_vp, ctypes.c_int, _i64p, _i32p, _f64p, _f64p]),
    "tagpu_pair_list_noalloc": (ctypes.c_int, [_vp, ctypes.c_int64, ctypes.c_int64,
                                               ctypes.c_int64, _vp, ctypes.c_float, _vp,
                                               ctypes.c_float, _vp, ctypes.c_float, _vp, _vp,
                                               ctypes.c_int64, _i64p, _vp]),
    "tagpu_batch_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "tagpu_batch_add": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_double, _vp,
                                       ctypes.c_char_p, _vp, ctypes.c_char_p,
                                       ctypes.POINTER(ContractOpts), ctypes.POINTER(_vp)]),
    "tagpu_batch_run": (ctypes.c_int, [_vp]),
    "tagpu_batch_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ContractStats)]),
    "tagpu_batch_destroy": (ctypes.c_int, [_vp]),
    "tagpu_server_start": (ctypes.c_int, [_vp, ctypes.POINTER(ServerConfig), ctypes.POINTER(_vp)]),
    "tagpu_server_submit": (ctypes.c_int, [_vp, ctypes.POINTER(Request),
                                           ctypes.POINTER(ctypes.c_uint64)]),
    "tagpu_server_poll": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.POINTER(_vp),
                                         ctypes.POINTER(RequestResult)]),
    "tagpu_server_wait": (ctypes.c_int, [_vp, ctypes.c_uint64, ctypes.c_double,
                                         ctypes.POINTER(_vp), ctypes.POINTER(RequestResult)]),
    "tagpu_server_get_stats": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "tagpu_server_stop": (ctypes.c_int, [_vp]),
}


def lib():
    """Load libtagpu.so; raises if it has not been built (no fallback)."""
    global _L
    if _L is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                              "(the CUDA library is the only compute path)")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _L = L
    return _L


def _p(a, t):
    return a.ctypes.data_as(t)


class World:
    """A tagpu context on one GPU (TA::initialize + default World)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0):
        L = lib()
        cfg = Config(device, hbm_budget_bytes)
        h = _vp()
        st = L.tagpu_init(ctypes.byref(cfg), ctypes.byref(h))
        if st:
            raise TAGPUError(st, "tagpu_init failed (no usable CUDA device?)")
        self.h = h
        self.L = L

    def check(self, st):
        if st:
            raise TAGPUError(st, self.L.tagpu_last_error(self.h).decode())

    @property
    def threshold(self):
        return self.L.tagpu_threshold_get(self.h)

    @threshold.setter
    def threshold(self, v):
        self.L.tagpu_threshold_set(self.h, float(v))

    def sync(self):
        self.check(self.L.tagpu_sync(self.h))

    def set_wait_limit(self, seconds):
        """Bound (seconds) of every pipeline wait in the emulated GEMM."""
        self.check(self.L.tagpu_set_wait_limit(self.h, float(seconds)))

    def mma_sync_rates(self):
        """Measured (INT8 TOP/s, bf16 TFLOP/s) of the warp-level mma.sync path."""
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        self.check(self.L.tagpu_device_mma_sync_rates(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def fp64_rates(self):
        """Measured (DMMA, DFMA) TFLOP/s of this GPU."""
        a, b = ctypes.c_double(0), ctypes.c_double(0)
        self.check(self.L.tagpu_device_fp64_rates(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def timer_start(self):
        self.check(self.L.tagpu_timer_start(self.h))

    def timer_stop(self):
        ms = ctypes.c_double(0)
        self.check(self.L.tagpu_timer_stop(self.h, ctypes.byref(ms)))
        return ms.value

    def host_array(self, n, dtype=np.float64):
        """A numpy array of n elements in pinned host memory owned by the
        library (tagpu_host_alloc), freed when the array is collected."""
        dt = np.dtype(dtype)
        p = _vp()
        self.check(self.L.tagpu_host_alloc(self.h, max(1, n) * dt.itemsize, ctypes.byref(p)))
        buf = (ctypes.c_char * (max(1, n) * dt.itemsize)).from_address(p.value)
        arr = np.frombuffer(buf, dtype=dt, count=n)
        # the buffer outlives every array and view made from it
        weakref.finalize(buf, self.L.tagpu_host_free, self.h, p)
        return arr

    def last_stats(self):
        s = ContractStats()
        self.check(self.L.tagpu_last_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if self.h:
            self.L.tagpu_shutdown(self.h)
            self.h = None

    # single steps on host buffers -------------------------------------------
    def shape_gemm(self, left, right, k_sizes, factor, threshold):
        left = np.ascontiguousarray(left, np.float32)
        right = np.ascontiguousarray(right, np.float32)
        M = left.shape[0]
        N = right.shape[-1]
        K = 0 if k_sizes is None else len(k_sizes)
        ks = None if k_sizes is None else np.ascontiguousarray(k_sizes, np.float32)
        out = np.empty((M, N), np.float32)
        z = ctypes.c_int64(0)
        self.check(self.L.tagpu_shape_gemm(self.h, M, N, K, _p(left, _f32p), _p(right, _f32p),
                                           None if ks is None else _p(ks, _f32p), float(factor),
                                           np.float32(threshold), _p(out, _f32p),
                                           ctypes.byref(z)))
        return out, z.value

    def pair_list(self, cnorm, c_thr, lnorm, l_thr, rnorm, r_thr):
        cnorm = np.ascontiguousarray(cnorm, np.float32)
        lnorm = np.ascontiguousarray(lnorm, np.float32)
        rnorm = np.ascontiguousarray(rnorm, np.float32)
        M, N = cnorm.shape
        K = lnorm.shape[1]
        offs = np.empty(M * N + 1, np.int64)
        n = ctypes.c_int64(0)
        args = (self.h, M, N, K, _p(cnorm, _f32p), np.float32(c_thr), _p(lnorm, _f32p),
                np.float32(l_thr), _p(rnorm, _f32p), np.float32(r_thr), _p(offs, _i64p))
        self.check(self.L.tagpu_pair_list(*args, None, 0, ctypes.byref(n)))
        kidx = np.empty(max(1, n.value), np.int32)
        self.check(self.L.tagpu_pair_list(*args, _p(kidx, _i32p), kidx.size, ctypes.byref(n)))
        return offs, kidx[:n.value]

    def permute(self, x, perm):
        x = np.ascontiguousarray(x, np.float64)
        ext = np.asarray(x.shape, np.int64)
        p = np.asarray(perm, np.int32)
        rshape = [0] * x.ndim
        for d in range(x.ndim):
            rshape[perm[d]] = x.shape[d]
        out = np.empty(rshape, np.float64)
        self.check(self.L.tagpu_permute(self.h, x.ndim, _p(ext, _i64p), _p(p, _i32p),
                                        _p(x, _f64p), _p(out, _f64p)))
        return out


class TiledRange:
    """TiledRange: one list of hashmarks (TiledRange1) per dimension."""

    def __init__(self, dims):
        self.dims = [list(map(int, h)) for h in dims]

    @property
    def rank(self):
        return len(self.dims)

    def ntiles(self):
        return [len(h) - 1 for h in self.dims]

    def extents(self):
        return [h[-1] - h[0] for h in self.dims]

    def tile_index(self, ordinal):
        idx = []
        for n in reversed(self.ntiles()):
            idx.append(ordinal % n)
            ordinal //= n
        return list(reversed(idx))

    def tile_lo_hi(self, idx):
        return ([self.dims[d][idx[d]] for d in range(self.rank)],
                [self.dims[d][idx[d] + 1] for d in range(self.rank)])

    def tile_shape(self, idx):
        lo, hi = self.tile_lo_hi(idx)
        return [h - l for l, h in zip(lo, hi)]

    def __eq__(self, other):
        return isinstance(other, TiledRange) and self.dims == other.dims

    def __repr__(self):
        return f"TiledRange({self.dims})"


class TsrExpr:
    def __init__(self, array, indices, factor=1.0):
        self.array, self.indices, self.factor = array, indices, factor

    def __iadd__(self, expr):
        """C("i,j") += A("i,k") * B("k,j") (TsrExpr::operator+=)."""
        if not isinstance(expr, MultExpr):
            raise TypeError("only contractions A(...) * B(...) are on this path")
        a = self.array
        opts = ContractOpts(a.precision, a.slices, -1.0, 0)
        W = a.world
        W.check(W.L.tagpu_contract_accumulate(
            W.h, self.indices.encode(), float(expr.factor), expr.left.array.h,
            expr.left.indices.encode(), expr.right.array.h, expr.right.indices.encode(),
            ctypes.byref(opts), a.h))
        return _Accumulated(self)

    def __mul__(self, other):
        if isinstance(other, TsrExpr):
            return MultExpr(self, other, self.factor * other.factor)
        return TsrExpr(self.array, self.indices, self.factor * float(other))

    def __rmul__(self, s):
        return TsrExpr(self.array, self.indices, self.factor * float(s))


class _Accumulated:
    """Result of `+=` on a TsrExpr: the target already holds the sum."""

    def __init__(self, target):
        self.target = target


class MultExpr:
    def __init__(self, left, right, factor):
        self.left, self.right, self.factor = left, right, factor

    def __rmul__(self, s):
        return MultExpr(self.left, self.right, self.factor * float(s))

    __mul__ = __rmul__


class DistArray:
    """Block-sparse (SparsePolicy) or dense (DensePolicy) array of FP64 tiles
    resident in device memory."""

    def __init__(self, world: World, trange: TiledRange | None = None, norms=None,
                 do_not_scale=False, threshold=-1.0, dense=False, _handle=None):
        self.world = world
        self.h = None
        self.precision = PRECISION_FP64
        self.slices = 0
        if _handle is not None:
            self.h = _handle
            return
        if trange is None:
            return
        hm = [np.asarray(h, np.int64) for h in trange.dims]
        nt = np.asarray([len(h) - 1 for h in hm], np.int64)
        arr = (_i64p * max(1, len(hm)))(*[_p(h, _i64p) for h in hm])
        h = _vp()
        world.check(world.L.tagpu_array_create(world.h, len(hm), _p(nt, _i64p), arr,
                                               ctypes.byref(h)))
        self.h = h
        if not dense and norms is not None:
            self.set_shape(norms, do_not_scale, threshold)

    def __del__(self):
        try:
            if self.h is not None and self.world.h is not None:
                self.world.L.tagpu_array_destroy(self.h)
        except Exception:
            pass
        self.h = None

    # shape and data -----------------------------------------------------------
    def set_shape(self, norms, do_not_scale=False, threshold=-1.0):
        n = np.ascontiguousarray(norms, np.float32).ravel()
        self.world.check(self.world.L.tagpu_array_set_shape(self.h, _p(n, _f32p),
                                                            int(do_not_scale),
                                                            np.float32(threshold)))

    def info(self):
        i = ArrayInfo()
        self.world.check(self.world.L.tagpu_array_get_info(self.h, ctypes.byref(i)))
        return i

    @property
    def trange(self):
        i = self.info()
        dims = []
        for d in range(i.rank):
            buf = np.empty(i.ntiles[d] + 1, np.int64)
            self.world.check(self.world.L.tagpu_array_get_hashmarks(self.h, d, _p(buf, _i64p)))
            dims.append(buf.tolist())
        return TiledRange(dims)

    def norms(self):
        i = self.info()
        out = np.empty(i.ntiles_total, np.float32)
        self.world.check(self.world.L.tagpu_array_get_norms(self.h, _p(out, _f32p)))
        return out

    def tile_offsets(self):
        i = self.info()
        out = np.empty(i.ntiles_total, np.int64)
        self.world.check(self.world.L.tagpu_array_get_tile_offsets(self.h, _p(out, _i64p)))
        return out

    def tile(self, ordinal: int, shape=None):
        """One nonzero tile (DistArray::find(i).get()), reshaped to `shape`."""
        tr = self.trange
        idx, o = [], int(ordinal)
        for d in reversed(range(len(tr.dims))):
            n = len(tr.dims[d]) - 1
            idx.append(o % n)
            o //= n
        idx.reverse()
        ext = tuple(tr.dims[d][x + 1] - tr.dims[d][x] for d, x in enumerate(idx))
        out = np.empty(max(1, int(np.prod(ext))), np.float64)
        self.world.check(self.world.L.tagpu_array_get_tile(self.h, int(ordinal), _p(out, _f64p),
                                                           int(np.prod(ext))))
        return out[:int(np.prod(ext))].reshape(shape if shape is not None else ext)

    def upload(self, packed):
        packed = np.ascontiguousarray(packed, np.float64)
        self.world.check(self.world.L.tagpu_array_upload(self.h, _p(packed, _f64p), packed.size))

    def download(self):
        n = self.info().elements
        out = np.empty(max(1, n), np.float64)
        self.world.check(self.world.L.tagpu_array_download(self.h, _p(out, _f64p), n))
        return out[:n]

    def set_tiles(self, tiles: dict):
        """tiles: ordinal -> ndarray for every nonzero tile of the shape."""
        offs = self.tile_offsets()
        n = self.info().elements
        buf = np.zeros(n, np.float64)
        for o, off in enumerate(offs):
            if off >= 0:
                t = tiles.get(o)
                if t is not None:
                    t = np.ascontiguousarray(t, np.float64).ravel()
                    buf[off:off + t.size] = t
        self.upload(buf)

    def generate(self, seed, stream, kind=0, tile_scale=None, compute_shape=True,
                 threshold=-1.0):
        ts = None
        if tile_scale is not None:
            ts = np.ascontiguousarray(tile_scale, np.float64).ravel()
        self.world.check(self.world.L.tagpu_array_generate(
            self.h, int(seed), int(stream), int(kind), None if ts is None else _p(ts, _f64p),
            int(compute_shape), np.float32(threshold)))

    def save(self, path):
        """The engine's own archive of the array (versioned, streamed)."""
        self.world.check(self.world.L.tagpu_array_save(self.h, os.fsencode(path)))

    def serialize(self, path, array_type_hash=0, pmap_type_hash=0):
        """The byte stream DistArray::serialize writes to a MADNESS binary
        archive on one rank (the hash codes are the reading build's)."""
        self.world.check(self.world.L.tagpu_array_serialize(
            self.h, os.fsencode(path), int(array_type_hash), int(pmap_type_hash)))

    @staticmethod
    def load(world, path):
        """An array read back from tagpu_array_save's archive."""
        h = _vp()
        world.check(world.L.tagpu_array_load(world.h, os.fsencode(path), ctypes.byref(h)))
        return DistArray(world, _handle=h)

    @staticmethod
    def deserialize(world, path, sparse=True):
        """An array read from a DistArray::serialize stream of one rank;
        returns (array, array type hash, pmap type hash)."""
        h = _vp()
        th, ph = ctypes.c_uint64(0), ctypes.c_uint64(0)
        world.check(world.L.tagpu_array_deserialize(world.h, os.fsencode(path), int(sparse),
                                                    ctypes.byref(h), ctypes.byref(th),
                                                    ctypes.byref(ph)))
        return DistArray(world, _handle=h), th.value, ph.value

    def truncate(self, threshold=-1.0):
        """TiledArray::truncate: shape from the stored tiles' norms, small tiles dropped."""
        self.world.check(self.world.L.tagpu_array_truncate(self.h, np.float32(threshold)))

    def tiles(self, trange: TiledRange):
        data = self.download()
        offs = self.tile_offsets()
        out = {}
        for o, off in enumerate(offs):
            if off >= 0:
                shp = trange.tile_shape(trange.tile_index(o))
                out[o] = data[off:off + int(np.prod(shp))].reshape(shp)
        return out

    def to_dense(self, trange: TiledRange):
        out = np.zeros(trange.extents(), np.float64)
        for o, t in self.tiles(trange).items():
            lo, hi = trange.tile_lo_hi(trange.tile_index(o))
            out[tuple(slice(l - trange.dims[d][0], h - trange.dims[d][0])
                      for d, (l, h) in enumerate(zip(lo, hi)))] = t
        return out

    # expressions ---------------------------------------------------------------
    def __call__(self, indices: str):
        return TsrExpr(self, indices)

    def __getitem__(self, indices: str):
        return TsrExpr(self, indices)

    def __setitem__(self, indices: str, expr):
        if isinstance(expr, _Accumulated) and expr.target.array is self:
            return
        if not isinstance(expr, MultExpr):
            raise TypeError("only contractions A(...) * B(...) are on this path")
        opts = ContractOpts(self.precision, self.slices, -1.0, 0)
        h = _vp()
        W = self.world
        W.check(W.L.tagpu_contract(W.h, indices.encode(), float(expr.factor), expr.left.array.h,
                                   expr.left.indices.encode(), expr.right.array.h,
                                   expr.right.indices.encode(), ctypes.byref(opts),
                                   ctypes.byref(h)))
        if self.h is not None:
            W.L.tagpu_array_destroy(self.h)
        self.h = h


def TSpArrayD(world, trange=None, norms=None, **kw):
    return DistArray(world, trange, norms, **kw)


def TArrayD(world, trange=None, **kw):
    return DistArray(world, trange, None, dense=True, **kw)


def contract(world, c_idx, alpha, A, a_idx, B, b_idx, precision=PRECISION_FP64, slices=0,
             threshold=-1.0, autotune=False):
    """Functional form of C(c_idx) = alpha * A(a_idx) * B(b_idx); returns
    (result DistArray, stats dict)."""
    opts = ContractOpts(precision, slices, threshold, int(autotune))
    h = _vp()
    world.check(world.L.tagpu_contract(world.h, c_idx.encode(), float(alpha), A.h,
                                       a_idx.encode(), B.h, b_idx.encode(), ctypes.byref(opts),
                                       ctypes.byref(h)))
    return DistArray(world, _handle=h), world.last_stats()


def contract_accumulate(world, C, c_idx, alpha, A, a_idx, B, b_idx, precision=PRECISION_FP64,
                        slices=0, threshold=-1.0):
    """C(c_idx) += alpha * A(a_idx) * B(b_idx) in place; returns the product's stats."""
    opts = ContractOpts(precision, slices, threshold, 0)
    world.check(world.L.tagpu_contract_accumulate(world.h, c_idx.encode(), float(alpha), A.h,
                                                  a_idx.encode(), B.h, b_idx.encode(),
                                                  ctypes.byref(opts), C.h))
    return world.last_stats()


class Server:
    """Request loop: HBM-footprint admission and continuous batching."""

    def __init__(self, world: World, hbm_budget_bytes=0, max_batch=64,
                 precision=PRECISION_FP64, slices=7):
        self.world = world
        cfg = ServerConfig(hbm_budget_bytes, max_batch, precision, slices)
        h = _vp()
        world.check(world.L.tagpu_server_start(world.h, ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self._keep = {}

    def submit(self, c_idx, alpha, A, a_idx, B, b_idx, precision=-1, slices=0):
        """Returns a request id; raises TAGPUError (status 6) on rejection."""
        req = Request(c_idx.encode(), float(alpha), A.h, a_idx.encode(), B.h, b_idx.encode(),
                      int(precision), int(slices))
        rid = ctypes.c_uint64(0)
        self.world.check(self.world.L.tagpu_server_submit(self.h, ctypes.byref(req),
                                                           ctypes.byref(rid)))
        self._keep[rid.value] = (A, B)
        return rid.value

    def wait(self, rid, timeout_ms=-1.0):
        c = _vp()
        res = RequestResult()
        self.world.check(self.world.L.tagpu_server_wait(self.h, rid, float(timeout_ms),
                                                         ctypes.byref(c), ctypes.byref(res)))
        self._keep.pop(rid, None)
        arr = DistArray(self.world, _handle=c) if c.value else None
        return arr, res.as_dict()

    def poll(self, rid):
        c = _vp()
        res = RequestResult()
        st = self.world.L.tagpu_server_poll(self.h, rid, ctypes.byref(c), ctypes.byref(res))
        if st == 7:
            return None
        self.world.check(st)
        self._keep.pop(rid, None)
        return (DistArray(self.world, _handle=c) if c.value else None), res.as_dict()

    def stats(self):
        s = ServerStats()
        self.world.check(self.world.L.tagpu_server_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def stop(self):
        if self.h is not None:
            self.world.check(self.world.L.tagpu_server_stop(self.h))
            self.h = None
