"""A restatement, in Python, of the byte stream DistArray::serialize hands a
MADNESS binary archive on one rank (dist_array.h:1583-1590), used to build
streams by hand and to parse what the engine writes.

Scalars are raw little-endian bytes; arrays written through archive::wrap
carry no length; vectors carry a size_t count first.
  Range (range.h:1143-1157): u32 rank, i64 lobound[r], upbound[r], extent[r],
    stride[r] (row-major), i64 offset = sum lobound*stride, u64 volume
  Range1 (range1.h:195-204): i64 first, i64 second
  TiledRange1 (tiled_range1.h:405): Range1 tiles, Range1 elements,
    vector<Range1> per-tile ranges
  TiledRange (tiled_range.h:392): Range tiles, Range elements,
    vector<TiledRange1>
  SparseShape<float> (sparse_shape.h:1918-1923): Tensor<float> norms, per
    mode ValArray<float> tile extents (u64 size + floats), u64 zero count
  Tensor<T> (tensor/tensor.h:1389-1416): u8 empty, then Range, u64 nbatch,
    data[volume * nbatch]
"""
import struct

import numpy as np


def _range(lo, up):
    r = len(lo)
    ext = [u - l for l, u in zip(lo, up)]
    stride = [0] * r
    vol, off = 1, 0
    for d in range(r - 1, -1, -1):
        stride[d] = vol
        off += lo[d] * stride[d]
        vol *= ext[d]
    return struct.pack(f"<I{4 * r}qqQ", r, *lo, *up, *ext, *stride, off, vol)


def write(hashmarks, tiles, norms=None, type_hash=0, pmap_hash=0, world=(1, 0)):
    """hashmarks per mode; tiles: {tile index tuple: ndarray}; norms: scaled
    norm tensor over the tile grid (None: DenseShape)."""
    nt = [len(h) - 1 for h in hashmarks]
    r = len(nt)
    out = [struct.pack("<Qii", type_hash, *world)]
    out.append(_range([0] * r, nt))
    out.append(_range([h[0] for h in hashmarks], [h[-1] for h in hashmarks]))
    out.append(struct.pack("<Q", r))
    for h in hashmarks:
        out.append(struct.pack("<qqqqQ", 0, len(h) - 1, h[0], h[-1], len(h) - 1))
        for i in range(len(h) - 1):
            out.append(struct.pack("<qq", h[i], h[i + 1]))
    if norms is not None:
        n = np.asarray(norms, np.float32)
        out.append(struct.pack("<B", 0))
        out.append(_range([0] * r, nt))
        out.append(struct.pack("<Q", 1))
        out.append(n.ravel().tobytes())
        for h in hashmarks:
            out.append(struct.pack("<Q", len(h) - 1))
            out.append(np.diff(np.asarray(h)).astype(np.float32).tobytes())
        out.append(struct.pack("<Q", int(np.sum(n == 0))))
    out.append(struct.pack("<Qq", pmap_hash, len(tiles)))
    for idx in sorted(tiles):
        lo = [hashmarks[d][idx[d]] for d in range(r)]
        up = [hashmarks[d][idx[d] + 1] for d in range(r)]
        out.append(struct.pack("<B", 0))
        out.append(_range(lo, up))
        out.append(struct.pack("<Q", 1))
        out.append(np.ascontiguousarray(tiles[idx], np.float64).tobytes())
    return b"".join(out)
