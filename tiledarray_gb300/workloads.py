"""Synthetic workloads of the benchmark configurations (seeded, generated on
the device through tagpu_array_generate).

  dense      TArrayD C(i,j) = A(i,k) * B(k,j), N = M = K = 2048, tiles of 128
  blocksparse TSpArrayD matrix product, N = 16384, tiles U[48,256],
             blocks scaled by exp(-|I-J|/4), absent below 1e-10, threshold 1e-8
  ccsd       R(a,b,i,j) = V(a,b,c,d) * T(c,d,i,j), o = 48 (tiles of 16),
             v = 384 (tiles U[32,96]); V blocks exp(-(|A-C|+|B-D|)/3),
             T blocks exp(-(|C-I|+|D-J|)/3), threshold 1e-8
  batched    512 independent C(i,j,l) = A(i,j,k) * B(k,l), extents
             log-uniform in [32,512], tiles U[32,128], 30% block dropout
"""
from __future__ import annotations

import numpy as np


def tiling(n, lo, hi, rng):
    """Seeded uneven tiling of [0, n): sizes U{lo..hi}, the last tile absorbs
    a remainder below lo."""
    h = [0]
    while h[-1] < n:
        rem = n - h[-1]
        s = int(rng.integers(lo, hi + 1))
        if rem - s < lo:
            s = rem
        h.append(h[-1] + s)
    return h


def blocksparse(n=16384, seed=0, lo=48, hi=256, decay=4.0, cut=1e-10):
    rng = np.random.default_rng(seed)
    h = tiling(n, lo, hi, rng)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / decay)
    scale[scale < cut] = 0.0
    return h, scale


def ccsd(o=48, v=384, seed=0, otile=16, vlo=32, vhi=96, decay=3.0):
    rng = np.random.default_rng(seed)
    ho = list(range(0, o + 1, otile))
    if ho[-1] != o:
        ho.append(o)
    hv = tiling(v, vlo, vhi, rng)
    nv, no = len(hv) - 1, len(ho) - 1
    A, B, C, D = np.meshgrid(*[np.arange(nv)] * 4, indexing="ij")
    vscale = np.exp(-(np.abs(A - C) + np.abs(B - D)) / decay)
    C2, D2, I2, J2 = np.meshgrid(np.arange(nv), np.arange(nv), np.arange(no), np.arange(no),
                                 indexing="ij")
    tscale = np.exp(-(np.abs(C2 - I2) + np.abs(D2 - J2)) / decay)
    return hv, ho, vscale, tscale


def batched(count=512, seed=0, lo=32, hi=512, tlo=32, thi=128, keep=0.7):
    """List of (tiling_i, tiling_j, tiling_k, tiling_l, keepA, keepB)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        ext = np.exp(rng.uniform(np.log(lo), np.log(hi), 4)).astype(int)
        ts = [tiling(int(e), tlo, thi, rng) for e in ext]
        nA = (len(ts[0]) - 1) * (len(ts[1]) - 1) * (len(ts[2]) - 1)
        nB = (len(ts[2]) - 1) * (len(ts[3]) - 1)
        out.append((ts, (rng.random(nA) < keep).astype(float), (rng.random(nB) < keep).astype(float)))
    return out
