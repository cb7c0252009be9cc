"""CCD on H2O / cc-pVDZ, the reference's own example (examples/cc/ccd.cpp with
examples/cc/input), restated in spin orbitals so that its printed residual
norms and energies (examples/cc/CCD_output.txt) check a contraction engine.

The fixture (tests/golden/ccd_h2o.npz, made by tests/golden/make_ccd_h2o.py)
holds the orbital symmetries, the Fock diagonal and the two-electron
integrals <pq|rs>.  Spin orbitals: occupied alpha, occupied beta, virtual
alpha, virtual beta; <PQ||RS> = <PQ|RS> - <PQ|SR> with spin selection.

The iteration is the reference's: amplitudes start at zero, the residual r
holds every term of the CCD equations (the Fock diagonal included), and
t <- t + D * r with D = 1 / (f_i + f_j - f_a - f_b); the program prints
||r_aa + r_ab + r_bb|| (its three spin blocks added elementwise) and
E = 1/4 sum <ab||ij> t_ij^ab.  The non-Fock terms are the standard
spin-orbital CCD equations with intermediates (the doubles part of the
CCSD equations of Stanton, Gauss, Watts and Bartlett, J. Chem. Phys. 94,
4334 (1991), with T1 = 0).  Every tensor contraction goes through `contract`,
so the same iteration runs on numpy, on the oracle and on the GPU engine.
"""
import os

import numpy as np

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ccd_h2o.npz")
OCC, VIR = "ijmn", "abef"


class H2O:
    def __init__(self):
        d = np.load(FIXTURE)
        self.nmo, self.nocc = int(d["nmo"]), int(d["nocc"])
        nmo, nocc = self.nmo, self.nocc
        nv = nmo - nocc
        self.ref_error, self.ref_energy = d["ref_error"], d["ref_energy"]
        v = np.zeros((nmo,) * 4)
        for (p, q, r, s), x in zip(d["v_idx"].astype(int), d["v_val"]):
            v[p, q, r, s] = x
        sym = d["sym"].astype(int)
        f = d["fdiag"]
        self.O, self.V = 2 * nocc, 2 * nv
        sp = np.array(list(range(nocc)) * 2 + list(range(nocc, nmo)) * 2)   # spatial orbital
        ss = np.array([0] * nocc + [1] * nocc + [0] * nv + [1] * nv)         # spin
        same = (ss[:, None] == ss[None, :]).astype(float)
        g = v[np.ix_(sp, sp, sp, sp)] * same[:, None, :, None] * same[None, :, None, :]
        g = g - g.transpose(0, 1, 3, 2)
        o, w = slice(0, self.O), slice(self.O, self.O + self.V)
        self.g_vvoo, self.g_oovv = g[w, w, o, o].copy(), g[o, o, w, w].copy()
        self.g_oooo, self.g_vvvv, self.g_ovvo = g[o, o, o, o].copy(), g[w, w, w, w].copy(), \
            g[o, w, w, o].copy()
        fs = f[sp]
        self.fo, self.fv = fs[o], fs[w]
        fo, fv = self.fo, self.fv
        self.fdiff = fv[:, None, None, None] + fv[None, :, None, None] - \
            fo[None, None, :, None] - fo[None, None, None, :]
        self.D = -1.0 / self.fdiff
        # tilings: a tile per run of equal (spin, symmetry), as the reference
        # tiles each mode by runs of equal symmetry within one spin
        key = ss * 16 + sym[sp]
        self.sym_tiling = {"o": _runs(key[:self.O]), "v": _runs(key[self.O:])}
        self.spin_tiling = {"o": [0, nocc, self.O], "v": [0, nv, self.V]}

    def tiling(self, idx, kind):
        t = self.sym_tiling if kind == "sym" else self.spin_tiling
        return [t["o"] if c in OCC else t["v"] for c in idx.split(",")]

    def iterate(self, contract, iterations):
        """Runs `iterations` CCD iterations; contract(c, alpha, X, x, Y, y)
        returns alpha * X(x) * Y(y) as a dense array in c's order.  Returns
        the (error, energy) of every iteration."""
        t = np.zeros((self.V, self.V, self.O, self.O))
        out = []
        for _ in range(iterations):
            r = self.residual(t, contract)
            t = t + self.D * r
            nv, no = self.V // 2, self.O // 2
            a, b, i, j = slice(0, nv), slice(nv, self.V), slice(0, no), slice(no, self.O)
            err = np.linalg.norm(r[a, a, i, i] + r[a, b, i, j] + r[b, b, j, j])
            out.append((float(err), float(0.25 * np.sum(self.g_vvoo * t))))
        return out

    def residual(self, t, contract):
        r = self.g_vvoo + self.fdiff * t
        if not np.any(t):
            return r
        go = self.g_oovv
        Fae = contract("a,e", -0.5, t, "a,f,m,n", go, "m,n,e,f")
        Fmi = contract("m,i", 0.5, go, "m,n,e,f", t, "e,f,i,n")
        Wmnij = self.g_oooo + contract("m,n,i,j", 0.25, go, "m,n,e,f", t, "e,f,i,j")
        Wabef = self.g_vvvv + contract("a,b,e,f", 0.25, t, "a,b,m,n", go, "m,n,e,f")
        Wmbej = self.g_ovvo + contract("m,b,e,j", -0.5, go, "m,n,e,f", t, "f,b,j,n")
        x = contract("a,b,i,j", 1.0, t, "a,e,i,j", Fae, "b,e")
        r = r + x - x.transpose(1, 0, 2, 3)
        x = contract("a,b,i,j", 1.0, t, "a,b,i,m", Fmi, "m,j")
        r = r - x + x.transpose(0, 1, 3, 2)
        r = r + contract("a,b,i,j", 0.5, t, "a,b,m,n", Wmnij, "m,n,i,j")
        r = r + contract("a,b,i,j", 0.5, Wabef, "a,b,e,f", t, "e,f,i,j")
        x = contract("a,b,i,j", 1.0, t, "a,e,i,m", Wmbej, "m,b,e,j")
        return r + x - x.transpose(0, 1, 3, 2) - x.transpose(1, 0, 2, 3) + x.transpose(1, 0, 3, 2)


def _runs(key):
    h = [0]
    for p in range(1, len(key)):
        if key[p] != key[p - 1]:
            h.append(p)
    h.append(len(key))
    return h


def einsum_contract(c, alpha, X, x, Y, y):
    letters = {}
    for ch in (x + "," + y + "," + c).split(","):
        letters.setdefault(ch, "abcdefghijklmnopqrstuvwxyz"[len(letters)])
    f = lambda s: "".join(letters[q] for q in s.split(","))
    return alpha * np.einsum(f"{f(x)},{f(y)}->{f(c)}", X, Y, optimize=True)


def tile_norms(dense, dims):
    """Frobenius norm of every tile (tile grid, row-major)."""
    sq = dense * dense
    for d, h in enumerate(dims):
        sq = np.add.reduceat(sq, np.asarray(h[:-1]) - h[0], axis=d)
    return np.sqrt(sq).ravel()


def tile_slices(dims, ordinal):
    nt = [len(h) - 1 for h in dims]
    idx = np.unravel_index(ordinal, nt)
    return tuple(slice(dims[d][idx[d]] - dims[d][0], dims[d][idx[d] + 1] - dims[d][0])
                 for d in range(len(dims)))


def tiles_of(dense, dims):
    """ordinal -> tile, and the tile norms, of a dense array."""
    norms = tile_norms(dense, dims)
    tiles = {int(o): np.ascontiguousarray(dense[tile_slices(dims, int(o))])
             for o in np.nonzero(norms)[0]}
    return tiles, norms
