"""General (fused-index) products on the GPU against the oracle: screened
shapes bit for bit, integer data exactly (as the reference's tests compare
against einsum), uniform data within 1e-12 relative Frobenius error, in the
plain FP64 form and in the emulated form (one digit-slice GEMM per fused
element)."""
import numpy as np
import pytest

import general_forms as G
from helpers import gpu_operand, oracle_operand, rel_fro

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ta():
    import tiledarray_gb300 as ta
    return ta


PRECISIONS = [("fp64", 0), ("ozaki", 1)]


@pytest.mark.parametrize("prec", PRECISIONS, ids=lambda p: p[0])
@pytest.mark.parametrize("form", G.FORMS, ids=lambda f: f[0])
def test_general_product_integer(oracle, ta, world, form, prec):
    tag, c, a, b, tra, trb, sparse = form
    ka = G.keep_mask(tra, 1) if sparse else None
    kb = G.keep_mask(trb, 2) if sparse else None
    A, _ = gpu_operand(ta, world, tra, 3, 0, kind=1, keep=ka)
    B, _ = gpu_operand(ta, world, trb, 3, 1, kind=1, keep=kb)
    precision = ta.PRECISION_OZAKI if prec[1] else ta.PRECISION_FP64
    C, st = ta.contract(world, c, 1.0, A, a, B, b, precision=precision)
    Ao = oracle_operand(oracle, tra, 3, 0, kind=1, keep=ka)
    Bo = oracle_operand(oracle, trb, 3, 1, kind=1, keep=kb)
    Co, info = oracle.general_contract(c, Ao, a, Bo, b, return_pairs=True)
    assert np.array_equal(C.norms(), Co.norms.ravel())
    assert st["pairs"] == len(info["kidx"])
    assert np.array_equal(C.to_dense(C.trange), Co.to_dense())
    ref = np.einsum(G.einsum_spec(c, a, b), Ao.to_dense(), Bo.to_dense())
    assert np.array_equal(C.to_dense(C.trange), ref)


@pytest.mark.parametrize("prec", PRECISIONS, ids=lambda p: p[0])
def test_general_product_uniform_larger(oracle, ta, world, prec):
    """Uneven tiles, several fused tiles and elements, scaled factor and a
    non-canonical target order; uniform data."""
    rng = np.random.default_rng(5)

    def tiling(n, lo, hi):
        h = [0]
        while h[-1] < n:
            h.append(min(n, h[-1] + int(rng.integers(lo, hi + 1))))
        return h
    tb, ti, tj, tk = tiling(13, 2, 6), tiling(150, 20, 70), tiling(200, 30, 90), tiling(120, 20, 60)
    tra, trb = [tb, ti, tj], [tk, tj, tb]
    A, _ = gpu_operand(ta, world, tra, 11, 0, kind=0)
    B, _ = gpu_operand(ta, world, trb, 11, 1, kind=0)
    precision = ta.PRECISION_OZAKI if prec[1] else ta.PRECISION_FP64
    C, _ = ta.contract(world, "i,k,b", -0.5, A, "b,i,j", B, "k,j,b", precision=precision)
    Ao = oracle_operand(oracle, tra, 11, 0, kind=0)
    Bo = oracle_operand(oracle, trb, 11, 1, kind=0)
    Co = oracle.general_contract("i,k,b", Ao, "b,i,j", Bo, "k,j,b", alpha=-0.5)
    assert np.array_equal(C.norms(), Co.norms.ravel())
    assert rel_fro(C.to_dense(C.trange), Co.to_dense()) <= 1e-12


def test_general_product_rejections(ta, world):
    A, _ = gpu_operand(ta, world, [G.TB, G.TI, G.TJ], 3, 0, kind=0)
    B, _ = gpu_operand(ta, world, [[0, 1, 5], G.TJ, G.TK], 3, 1, kind=0)
    with pytest.raises(ta.TAGPUError) as e:   # fused b tiled differently
        ta.contract(world, "b,i,k", 1.0, A, "b,i,j", B, "b,j,k")
    assert e.value.status == 1
