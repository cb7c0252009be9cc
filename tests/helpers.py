"""Shared test helpers: build the same operands for the oracle and the GPU."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def contraction_cases():
    with open(os.path.join(GOLDEN, "contractions.json")) as f:
        return json.load(f)


def oracle_operand(O, tr_dims, seed, stream, kind=1, keep=None, tile_scale=None,
                   threshold=None):
    tr = O.TiledRange(tr_dims)
    kp = None
    if keep is not None:
        flat = np.asarray(keep).ravel()
        kp = lambda idx: bool(flat[int(np.ravel_multi_index(idx, tr.ntiles()))])
    ts = None
    if tile_scale is not None:
        flat_s = np.asarray(tile_scale).ravel()
        ts = lambda idx: float(flat_s[int(np.ravel_multi_index(idx, tr.ntiles()))])
        kp0 = kp
        kp = lambda idx: (kp0 is None or kp0(idx)) and ts(idx) != 0.0
    return O.make_array(tr, seed, stream, kind, tile_scale=ts, keep=kp,
                        threshold=O.FLT_EPSILON if threshold is None else threshold)


def gpu_operand(ta, world, tr_dims, seed, stream, kind=1, keep=None, tile_scale=None,
                threshold=-1.0):
    tr = ta.TiledRange(tr_dims)
    A = ta.DistArray(world, tr)
    n = int(np.prod(tr.ntiles())) if tr.rank else 1
    sc = np.ones(n)
    if tile_scale is not None:
        sc = np.asarray(tile_scale, np.float64).ravel().copy()
    if keep is not None:
        sc = sc * np.asarray(keep, np.float64).ravel()
    A.generate(seed, stream, kind, sc, compute_shape=True, threshold=threshold)
    return A, tr


def rel_fro(x, ref):
    d = np.linalg.norm((x - ref).ravel())
    r = np.linalg.norm(ref.ravel())
    return d / r if r > 0 else d
