"""The CPU oracle pinned against the golden fixtures (no GPU).

The fixtures restate the reference tests' scenarios with expectations computed
independently in numpy (tests/golden/make_golden.py).
"""
import numpy as np
import pytest

from helpers import contraction_cases, golden, oracle_operand


def test_generator_matches_golden(oracle):
    g = golden("rng.npz")
    for o, h, u in zip(g["ordinals"], g["hash_s1_t2"], g["uniform_s1_t2"]):
        assert oracle.lib().orc_hash(1, 2, int(o)) == int(h)
        assert oracle.uniform(1, 2, int(o)) == float(u)
    for o, v in zip(g["ordinals"], g["int101_s7_t0"]):
        t = oracle.fill_tile([int(o)], [int(o) + 1], [int(o) + 1], 7, 0, kind=1)
        assert t[0] == v


def test_scale_norms_matches_golden(oracle):
    g = golden("scale_norms.npz")
    tr = oracle.TiledRange([list(h) for h in g["hashmarks"]])
    scaled, z = oracle.scale_norms(tr, g["raw"], float(g["threshold"]))
    assert np.array_equal(scaled, g["scaled"])  # bit-exact float32
    assert z == int(g["zero_count"])


def test_scale_norms_rank1(oracle):
    tr = oracle.TiledRange([[0, 2, 5, 10, 17, 28, 41]])
    raw = np.asarray([1, 2, 3, 4, 5, 6], np.float32)
    scaled, z = oracle.scale_norms(tr, raw, 0.2)
    sizes = np.asarray([2, 3, 5, 7, 11, 13], np.float32)
    exp = (raw / sizes).astype(np.float32)
    exp[exp < np.float32(0.2)] = 0
    assert np.array_equal(scaled, exp)
    assert z == int(np.sum(exp == 0))


def test_shape_gemm_matches_reference_test(oracle):
    """tests/sparse_shape.cpp:1478-1541: result = |a| (L*vol) x (R*vol) / (m n),
    threshold, BOOST_CHECK_CLOSE tolerance 1e-4 percent."""
    g = golden("shape_gemm.npz")
    tr = [list(h) for h in g["hashmarks"]]
    left, right = g["left"], g["right"]
    sizes = [np.asarray([h[i + 1] - h[i] for i in range(len(h) - 1)], np.float32) for h in tr]
    ks = oracle.outer_sizes([5, 5], np.concatenate(sizes[1:]), False)
    res, z = oracle.shape_gemm(left.reshape(5, 25), right.reshape(25, 5), ks, float(g["factor"]),
                               float(g["threshold"]))
    exp = g["expected"]
    tol = float(g["tolerance_percent"]) / 100.0
    nz = exp != 0
    assert np.array_equal(res == 0, ~nz)
    assert np.all(np.abs(res[nz] - exp[nz]) <= tol * np.abs(exp[nz]) * 10)
    assert z == int(np.sum(~nz))


def test_shape_gemm_outer_and_empty(oracle):
    l = np.asarray([[0.5], [2.0]], np.float32)
    r = np.asarray([[3.0, 0.1]], np.float32)
    res, z = oracle.shape_gemm(l, r, None, 2.0, 0.5)
    exp = np.asarray([[3.0, 0.0], [12.0, 0.4]], np.float32)
    exp[exp < 0.5] = 0
    assert np.array_equal(res, exp) and z == 2


def test_pairs_match_golden(oracle):
    g = golden("pairs.npz")
    for c in range(int(g["ncases"])):
        thr = g[f"c{c}_thr"]
        offs, kidx = oracle.pairs(g[f"c{c}_C"], thr[0], g[f"c{c}_L"], thr[1], g[f"c{c}_R"], thr[2])
        assert np.array_equal(offs, g[f"c{c}_offsets"])
        assert np.array_equal(kidx, g[f"c{c}_kidx"])


def test_permute_matches_golden(oracle):
    g = golden("permute.npz")
    for c in range(int(g["ncases"])):
        y = oracle.permute(g[f"c{c}_x"], list(g[f"c{c}_perm"]))
        assert np.array_equal(y, g[f"c{c}_y"])


@pytest.mark.parametrize("form,expected", [
    # (left, right) -> (left target, right target, result, left permtype, right permtype)
    ((["i", "b", "c"], ["j", "b", "c"]), (["i", "b", "c"], ["b", "c", "j"], ["i", "j"], 1, 2)),
    ((["i", "b", "c"], ["j", "c", "b"]), (["i", "c", "b"], ["c", "b", "j"], ["i", "j"], 3, 2)),
    ((["j", "b", "c"], ["i", "c", "b"]), (["j", "c", "b"], ["c", "b", "i"], ["j", "i"], 3, 2)),
    ((["i", "k"], ["k", "j"]), (["i", "k"], ["k", "j"], ["i", "j"], 1, 1)),
    ((["k", "i"], ["j", "k"]), (["i", "k"], ["k", "j"], ["i", "j"], 2, 2)),
    ((["a", "b", "c", "d"], ["c", "d", "i", "j"]),
     (["a", "b", "c", "d"], ["c", "d", "i", "j"], ["a", "b", "i", "j"], 1, 1)),
    ((["i"], ["j"]), (["i"], ["j"], ["i", "j"], 3, 3)),
])
def test_permopt_known_answers(oracle, form, expected):
    """Layouts chosen by GEMMPermutationOptimizer (expressions/permopt.h:258-376)."""
    got = oracle.permopt(*form, True)
    assert (list(got[0]), list(got[1]), list(got[2]), got[3], got[4]) == expected


@pytest.mark.parametrize("case", contraction_cases(), ids=lambda c: c["tag"])
def test_contraction_matches_golden(oracle, case):
    """Full pipeline (shape gemm, pairs, permutes, per-tile reduction) on
    integer data equals the dense einsum exactly."""
    A = oracle_operand(oracle, case["trange_a"], *case["seed_a"], kind=case["kind"],
                       keep=case["keep_a"])
    B = oracle_operand(oracle, case["trange_b"], *case["seed_b"], kind=case["kind"],
                       keep=case["keep_b"])
    C = oracle.contract(case["c"], A, case["a"], B, case["b"], case["alpha"])
    exp = golden(f"contract_{case['tag']}.npz")["expected"]
    assert np.array_equal(C.to_dense(), exp)


def test_oracle_blas_path_matches_loop(oracle):
    fn = oracle.openblas_dgemm()
    if fn is None:
        pytest.skip("numpy's bundled OpenBLAS not found")
    tr = [[0, 13, 40, 64], [0, 7, 31, 50]]
    A = oracle_operand(oracle, tr, 3, 0, kind=0)
    B = oracle_operand(oracle, [tr[1], tr[0]], 3, 1, kind=0)
    C1 = oracle.contract("i,j", A, "i,k", B, "k,j").to_dense()
    C2 = oracle.contract("i,j", A, "i,k", B, "k,j", use_blas=fn).to_dense()
    assert np.max(np.abs(C1 - C2)) <= 1e-13 * np.max(np.abs(C1))


@pytest.mark.parametrize("form", __import__("general_forms").FORMS, ids=lambda f: f[0])
def test_oracle_general_product_matches_einsum(oracle, form):
    """The oracle's general product equals numpy.einsum on integer data (exact)."""
    import general_forms as G
    tag, c, a, b, tra, trb, sparse = form
    A = oracle_operand(oracle, tra, 3, 0, kind=1, keep=G.keep_mask(tra, 1) if sparse else None)
    B = oracle_operand(oracle, trb, 3, 1, kind=1, keep=G.keep_mask(trb, 2) if sparse else None)
    C = oracle.general_contract(c, A, a, B, b)
    ref = np.einsum(G.einsum_spec(c, a, b), A.to_dense(), B.to_dense())
    assert np.array_equal(C.to_dense(), ref)
