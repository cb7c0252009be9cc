"""Fixture from the reference's own CCD example: H2O in cc-pVDZ
(examples/cc/input: orbital symmetries, the Fock diagonal, two-electron
integrals in chemists' notation) and the energies and residual norms the
reference program printed for it (examples/cc/CCD_output.txt).

Kept: the orbital symmetries (they define the TiledRange1 of every mode: a
tile per run of equal symmetry), the Fock diagonal, and every nonzero v_ab
element in physicists' notation <p1 p2 | p3 p4>; plus the printed error and
energy of every iteration.  Run once where the reference tree is present:

    python tests/golden/make_ccd_h2o.py /root/reference/examples/cc
"""
import os
import re
import sys

import numpy as np


def main(src):
    with open(os.path.join(src, "input")) as f:
        lines = f.read().split("\n")
    kv = {}
    i = 0
    for key in ("name", "nirreps", "nmo", "nocc_act_alpha", "nocc_act_beta",
                "nvir_act_alpha", "nvir_act_beta"):
        label, val = lines[i].split()
        assert label.rstrip(":") == key
        kv[key] = val
        i += 1
    nmo, nocc = int(kv["nmo"]), int(kv["nocc_act_alpha"])
    assert lines[i].startswith("obs_mosym_alpha")
    sym_a = [int(x) for x in lines[i + 1:i + 1 + nmo]]
    i += 1 + nmo
    assert lines[i].startswith("obs_mosym_beta")
    sym_b = [int(x) for x in lines[i + 1:i + 1 + nmo]]
    i += 1 + nmo
    assert sym_a == sym_b and int(kv["nocc_act_beta"]) == nocc
    # blank line, then f (p q value) until a blank line, then v (p q r s value)
    while lines[i].strip() == "":
        i += 1
    f = []
    while lines[i].strip():
        p, q, val = lines[i].split()
        f.append((int(p), int(q), float(val)))
        i += 1
    assert [(p, q) for p, q, _ in f] == [(k, k) for k in range(nmo)], "Fock not diagonal in order"
    fdiag = np.array([v for _, _, v in f])
    while lines[i].strip() == "":
        i += 1
    v = {}
    for line in lines[i:]:
        if not line.strip():
            break
        a, b, c, d, val = line.split()
        # chemists' (p1 p3 | p2 p4) -> physicists' <p1 p2 | p3 p4>
        p1, p3, p2, p4 = int(a), int(b), int(c), int(d)
        v[(p1, p2, p3, p4)] = float(val)   # a repeated element: the last one
    idx = np.array(sorted(v), dtype=np.int8)
    val = np.array([v[tuple(k)] for k in idx.tolist()])
    with open(os.path.join(src, "CCD_output.txt")) as fo:
        out = fo.read()
    errs = [float(x) for x in re.findall(r"error\s*=\s*([-0-9.eE+]+)", out)]
    ens = [float(x) for x in re.findall(r"energy\s*=\s*([-0-9.eE+]+)", out)]
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ccd_h2o.npz")
    np.savez_compressed(dst, nmo=nmo, nocc=nocc, sym=np.array(sym_a, np.int8), fdiag=fdiag,
                        v_idx=idx, v_val=val, ref_error=np.array(errs),
                        ref_energy=np.array(ens))
    print(dst, len(val), "elements;", len(ens), "printed iterations")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/examples/cc")
