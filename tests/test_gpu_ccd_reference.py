"""The reference's own CCD example (examples/cc: H2O in cc-pVDZ) run through
the GPU engine: every contraction of the CCD iteration restated in
tests/ccd_h2o.py is a `tagpu_contract` call on block-sparse arrays, and the
printed residual norms and energies of the reference program
(CCD_output.txt, 12 significant digits) must come out, in the plain FP64
form and in the emulated form.

Two tilings: spin blocks (2 tiles per mode) with the default SparseShape
threshold, as the oracle's check runs; and a tile per run of equal symmetry
and spin (tiles of 1 to 3 elements, 91 % of them zero) with the screening
threshold at 1e-30, so that only exactly zero tiles drop — with tiles that
small the default threshold screens out small nonzero tiles (of the
two-index intermediate F_ae above all: the oracle shows t(a,e,i,j) F(b,e)
changing by 9e-5 relative), which the reference's own, coarser spin-adapted
tiling does not."""
import numpy as np
import pytest

import ccd_h2o as C

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


@pytest.fixture(scope="module")
def h2o():
    return C.H2O()


@pytest.mark.parametrize("tiling", ["spin", "sym"])
@pytest.mark.parametrize("precision", ["fp64", "ozaki"])
def test_gpu_reproduces_reference_ccd_output(ta, world, h2o, precision, tiling):
    prec = ta.PRECISION_OZAKI if precision == "ozaki" else ta.PRECISION_FP64
    thr = -1.0 if tiling == "spin" else 1e-30
    pairs = []

    def contract(c, alpha, X, x, Y, y):
        arrays = []
        for dense, idx in ((X, x), (Y, y)):
            dims = h2o.tiling(idx, tiling)
            tiles, norms = C.tiles_of(dense, dims)
            A = ta.DistArray(world, ta.TiledRange(dims), norms=norms.astype(np.float32),
                             threshold=thr)
            A.set_tiles(tiles)
            arrays.append(A)
        R, st = ta.contract(world, c, alpha, arrays[0], x, arrays[1], y, precision=prec,
                            threshold=thr)
        pairs.append(st["pairs"])
        return R.to_dense(R.trange)

    res = h2o.iterate(contract, 4)
    for k, (err, energy) in enumerate(res):
        assert abs(err - h2o.ref_error[k]) <= 1e-11 * abs(h2o.ref_error[k]), (k, err)
        assert abs(energy - h2o.ref_energy[k]) <= 1e-12, (k, energy)
    assert min(pairs) > 0 and len(pairs) == 3 * 10
