"""General (fused-index) product forms of the reference's tests
(tests/general_product.cpp: expression_general_product_dense,
_dense_permuted_args, _dense_batched_outer, _sparse, _sparse_batched_outer,
a pure Hadamard product, and a fused broadcast without right free indices),
with the tilings used there."""
import numpy as np

TB = [0, 2, 5]           # b
TI = [0, 3, 4]           # i
TJ = [0, 2, 6, 7]        # j (contracted)
TK = [0, 4, 5]           # k

FORMS = [
    # tag, c, a, b, tiling of a, tiling of b, sparse
    ("dense", "b,i,k", "b,i,j", "b,j,k", [TB, TI, TJ], [TB, TJ, TK], False),
    ("permuted_args", "b,i,k", "i,j,b", "k,j,b", [TI, TJ, TB], [TK, TJ, TB], False),
    ("batched_outer", "b,i,k", "b,i", "b,k", [TB, TI], [TB, TK], False),
    ("hadamard", "b,i,j", "b,i,j", "b,i,j", [TB, TI, TJ], [TB, TI, TJ], False),
    ("broadcast", "b,i", "b,i,j", "b,j", [TB, TI, TJ], [TB, TJ], False),
    ("sparse", "b,i,k", "b,i,j", "b,j,k", [TB, TI, TJ], [TB, TJ, TK], True),
    ("sparse_batched_outer", "b,i,k", "b,i", "b,k", [TB, TI], [TB, TK], True),
    ("target_permuted", "k,b,i", "b,i,j", "b,j,k", [TB, TI, TJ], [TB, TJ, TK], True),
]


def keep_mask(tiling, seed):
    n = int(np.prod([len(h) - 1 for h in tiling]))
    return (np.arange(n) * 7 + seed) % 3 != 0


def einsum_spec(c, a, b):
    m = {}
    for x in a.split(",") + b.split(",") + c.split(","):
        m.setdefault(x, "abcdefghijklmnopqrstuvwxyz"[len(m)])
    f = lambda s: "".join(m[x] for x in s.split(","))
    return f"{f(a)},{f(b)}->{f(c)}"
