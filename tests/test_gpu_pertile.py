"""Per-result-tile accuracy against the FP64 oracle on decaying operands.

The block-sparse product's rule: block (I, J) of both operands filled with
uniform[-1, 1) entries scaled by exp(-|I-J|/4), absent below 1e-10, shapes
screened at 1e-8.  A result tile far from the diagonal is many orders of
magnitude below the tiles near it, so one Frobenius norm over the whole
result says nothing about it: every nonzero result tile is held to its own
relative bound, as a per-tile FP64 dgemm (math/blas.h:171-177 in the
reference) would be.  Small tiles (32-96) make the band reach |i-j| > 90 at a
size the oracle finishes in seconds.
"""
import numpy as np
import pytest

from helpers import gpu_operand, oracle_operand

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta

TOL_GLOBAL = 1e-12
TOL_TILE = {6: 5e-12,     # emulated form, every nonzero result tile: 47-bit digits
            7: 1e-12}     # 55-bit digits
TOL_TILE_PLAIN = 1e-14    # plain FP64 (DMMA) form, every nonzero result tile


def uneven(n, lo, hi, seed):
    rng = np.random.default_rng(seed)
    h = [0]
    while h[-1] < n:
        rem = n - h[-1]
        s = int(rng.integers(lo, hi + 1))
        if rem - s < lo:
            s = rem
        h.append(h[-1] + s)
    return h


def tile_errors(got, ref, h):
    """Relative Frobenius error of every tile of ref with a nonzero norm."""
    nt = len(h) - 1
    err = np.full((nt, nt), np.nan)
    for i in range(nt):
        for j in range(nt):
            r = ref[h[i]:h[i + 1], h[j]:h[j + 1]]
            rn = np.linalg.norm(r)
            if rn > 0:
                err[i, j] = np.linalg.norm(got[h[i]:h[i + 1], h[j]:h[j + 1]] - r) / rn
    return err


@pytest.mark.parametrize("slices", [6, 7])
@pytest.mark.parametrize("n,lo,hi,seed", [(6000, 32, 96, 11), (12000, 48, 256, 12)])
def test_pertile_error_decaying_band(oracle, ta, world, n, lo, hi, seed, slices):
    h = uneven(n, lo, hi, seed)
    nt = len(h) - 1
    I, J = np.meshgrid(np.arange(nt), np.arange(nt), indexing="ij")
    scale = np.exp(-np.abs(I - J) / 4.0)
    scale[scale < 1e-10] = 0
    thr = 1e-8
    A, _ = gpu_operand(ta, world, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    B, _ = gpu_operand(ta, world, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    world.threshold = thr
    try:
        C, st = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j", precision=ta.PRECISION_OZAKI,
                            slices=slices)
        Cp, _ = ta.contract(world, "i,j", 1.0, A, "i,k", B, "k,j")
    finally:
        world.threshold = ta.FLT_EPSILON
    Ao = oracle_operand(oracle, [h, h], seed, 0, kind=0, tile_scale=scale, threshold=thr)
    Bo = oracle_operand(oracle, [h, h], seed, 1, kind=0, tile_scale=scale, threshold=thr)
    ref = oracle.contract("i,j", Ao, "i,k", Bo, "k,j", threshold=thr,
                          use_blas=oracle.openblas_dgemm()).to_dense()
    got = C.to_dense(C.trange)
    gp = Cp.to_dense(Cp.trange)
    e = tile_errors(got, ref, h)
    ep = tile_errors(gp, ref, h)
    d = np.abs(I - J)
    band = " ".join(f"{k}:{np.nanmax(np.where((d >= k) & (d < k + 10), e, np.nan)):.1e}"
                    for k in range(0, int(d[~np.isnan(e)].max()) + 1, 10))
    g = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    print(f"S={slices} nt={nt} global {g:.2e} max tile {np.nanmax(e):.2e} (plain {np.nanmax(ep):.2e}); "
          f"by |i-j|: {band}; mma/fp64 flops {st['mma_flops'] / st['flops']:.2f}")
    assert int(d[~np.isnan(e)].max()) >= 60
    assert g <= TOL_GLOBAL
    assert np.nanmax(e) <= TOL_TILE[slices]
    assert np.nanmax(ep) <= TOL_TILE_PLAIN
