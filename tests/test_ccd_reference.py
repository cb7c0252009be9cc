"""The reference's own CCD example (examples/cc: H2O in cc-pVDZ) as a known
answer: its printed residual norms and energies per iteration
(CCD_output.txt, 12 significant digits) must come out of the CCD iteration
restated in tests/ccd_h2o.py, first with numpy's einsum (which checks the
restatement and the fixture), then with every contraction done by the
oracle's block-sparse pipeline (which pins the oracle to outputs of the
reference itself).  The GPU engine runs the same check in
test_gpu_ccd_reference.py."""
import numpy as np
import pytest

import ccd_h2o as C


@pytest.fixture(scope="module")
def h2o():
    return C.H2O()


def check(h2o, res):
    for k, (err, energy) in enumerate(res):
        # printed with 12 significant digits
        assert abs(err - h2o.ref_error[k]) <= 1e-11 * abs(h2o.ref_error[k]), (k, err)
        assert abs(energy - h2o.ref_energy[k]) <= 1e-12, (k, energy)


def test_restatement_reproduces_reference_output(h2o):
    check(h2o, h2o.iterate(C.einsum_contract, 8))


def test_oracle_reproduces_reference_output(oracle, h2o):
    """Spin-block tiling (2 tiles per mode; the spin-forbidden blocks are
    zero tiles of the shapes), the reference's default threshold."""
    def contract(c, alpha, X, x, Y, y):
        arrays = []
        for dense, idx in ((X, x), (Y, y)):
            dims = h2o.tiling(idx, "spin")
            tr = oracle.TiledRange(dims)
            tiles, norms = C.tiles_of(dense, dims)
            scaled, _ = oracle.scale_norms(tr, norms.astype(np.float32), oracle.FLT_EPSILON)
            A = oracle.Array(tr, scaled, oracle.FLT_EPSILON)
            flat = scaled.ravel()
            for o, tile in tiles.items():
                if flat[o] >= oracle.FLT_EPSILON:
                    A.tiles[o] = tile
            arrays.append(A)
        return oracle.contract(c, arrays[0], x, arrays[1], y, alpha).to_dense()
    check(h2o, h2o.iterate(contract, 3))
