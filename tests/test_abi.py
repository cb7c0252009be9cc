"""The C-ABI library builds, loads without a GPU, and exports every entry
point include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(tagpu_\w+)\s*\(", text, re.M):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["tagpu_init", "tagpu_contract", "tagpu_shape_gemm", "tagpu_pair_list",
              "tagpu_permute", "tagpu_array_generate", "tagpu_batch_run"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    from tiledarray_gb300 import build as tb
    path = tb.build()
    L = ctypes.CDLL(path)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_mirror_binds_every_symbol():
    import tiledarray_gb300 as ta
    assert set(declared_symbols()) <= set(ta.SIGNATURES), \
        set(declared_symbols()) - set(ta.SIGNATURES)


def test_library_has_no_oracle_dependency():
    """The product library neither links nor names the CPU oracle."""
    from tiledarray_gb300 import build as tb
    path = tb.build()
    data = open(path, "rb").read()
    assert b"liboracle" not in data and b"orc_" not in data


def test_no_gpu_init_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import tiledarray_gb300 as ta
    with pytest.raises(ta.TAGPUError):
        ta.World(0)
