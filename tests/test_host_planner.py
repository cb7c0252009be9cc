"""Host-side planning logic that needs no GPU: index parsing and layout
choice are checked through the Python oracle restatement; the C++ planner is
exercised on the GPU by the parity tests."""
import numpy as np
import pytest


@pytest.mark.parametrize("L,R", [
    ("i,b,c", "j,b,c"), ("i,b,c", "j,c,b"), ("j,b,c", "i,c,b"), ("a,b,c,d", "c,d,i,j"),
    ("a,c,b,d", "c,d,i,j"), ("k,i", "j,k"), ("x,i,j,k", "y,i,j,k"), ("i", "j"),
    ("c,d,a,b", "i,j,c,d"), ("i,j,c,d", "a,b,c,d"),
])
def test_permopt_invariants(oracle, L, R):
    lt, rt, res, lop, rop = oracle.permopt(L.split(","), R.split(","), True)
    inner = (len(lt) + len(rt) - len(res)) // 2
    assert sorted(lt) == sorted(L.split(","))
    assert sorted(rt) == sorted(R.split(","))
    if inner:
        # inner indices in the same order at the end of left, start of right
        assert lt[len(lt) - inner:] == rt[:inner]
        assert res == lt[:len(lt) - inner] + rt[inner:]
    for op, orig, tgt in ((lop, L.split(","), lt), (rop, R.split(","), rt)):
        if op == 1:
            assert orig == tgt
