"""Writes the golden fixtures of this directory. Run from the repository root:

    python tests/golden/make_golden.py

hydrogenic_slater.json
    Closed-form Slater integrals R^k(ab;cd) of nonrelativistic hydrogenic
    orbitals (n <= 2), in units of Z, as exact fractions. Computed here with
    sympy from P_nl(r) = r R_nl(r) (R_nl: the textbook hydrogen radial
    functions) by splitting the double integral at r1 = r2. The Dirac
    orbitals of the library approach these values as c -> infinity.

quad_kat.json
    The reference's only numeric unit test (test/lib9290_quad.f90:22-33):
    QUAD of exp(-2r) on the 590-point log grid (RNT = 2e-6, H = 0.05) is 0.5
    within 1e-12.

ne7_regression.npz
    Regression vectors of the oracle (the CPU restatement of the reference)
    for the Ne VII J=0 even block: the R^k table (INDTEIRK, VALTEIRK, KSTART
    of genintrk.f90), the one-body I(ab) table, the assembled EMT and EAV of
    SETHAM (EMT as assembled and with the average diagonal EAV taken off the
    diagonal, as rci's GENMAT does) and the lowest three MANEIG eigenpairs. The GPU tests compare the
    CUDA path with these stored arrays as well as with the live oracle.
"""
import json
import os
import sys
from fractions import Fraction

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def hydrogenic_slater():
    import sympy as sp
    r, r1, r2, Z = sp.symbols("r r1 r2 Z", positive=True)

    def P(n, l, x):  # r R_nl(r) for hydrogen-like Z, normalised
        R = sp.sqrt((2 * Z / n) ** 3 * sp.factorial(n - l - 1) / (2 * n * sp.factorial(n + l))) \
            * sp.exp(-Z * x / n) * (2 * Z * x / n) ** l * sp.assoc_laguerre(n - l - 1, 2 * l + 1, 2 * Z * x / n)
        return sp.simplify(x * R)

    def rk(a, b, c, d, k):
        f = sp.expand(P(*a, r1) * P(*c, r1))
        g = sp.expand(P(*b, r2) * P(*d, r2))
        inner_lo = sp.integrate(g * r2 ** k, (r2, 0, r1)) / r1 ** (k + 1)       # r2 < r1
        inner_hi = sp.integrate(g / r2 ** (k + 1), (r2, r1, sp.oo)) * r1 ** k    # r2 > r1
        val = sp.integrate(sp.expand(f * (inner_lo + inner_hi)), (r1, 0, sp.oo))
        return sp.nsimplify(sp.simplify(val / Z))

    # (n, l) pairs; kappa labels of the Dirac orbitals these limits belong to
    s1, s2, p2 = (1, 0), (2, 0), (2, 1)
    cases = [
        ("1s", "1s", "1s", "1s", 0, s1, s1, s1, s1),
        ("1s", "2s", "1s", "2s", 0, s1, s2, s1, s2),
        ("1s", "2s", "2s", "1s", 0, s1, s2, s2, s1),
        ("2s", "2s", "2s", "2s", 0, s2, s2, s2, s2),
        ("2p", "2p", "2p", "2p", 0, p2, p2, p2, p2),
        ("2p", "2p", "2p", "2p", 2, p2, p2, p2, p2),
        ("1s", "2p", "1s", "2p", 0, s1, p2, s1, p2),
        ("1s", "2p", "2p", "1s", 1, s1, p2, p2, s1),
        ("2s", "2p", "2s", "2p", 0, s2, p2, s2, p2),
        ("2s", "2p", "2p", "2s", 1, s2, p2, p2, s2),
    ]
    out = []
    for la, lb, lc, ld, k, a, b, c, d in cases:
        v = rk(a, b, c, d, k)
        fr = Fraction(int(sp.numer(v)), int(sp.denom(v)))
        out.append({"a": la, "b": lb, "c": lc, "d": ld, "k": k, "value_over_Z": f"{fr.numerator}/{fr.denominator}"})
        print(la, lb, lc, ld, k, fr)
    with open(os.path.join(HERE, "hydrogenic_slater.json"), "w") as fh:
        json.dump({"source": "tests/golden/make_golden.py (sympy, nonrelativistic hydrogenic)", "integrals": out},
                  fh, indent=1)


def quad_kat():
    with open(os.path.join(HERE, "quad_kat.json"), "w") as fh:
        json.dump({"source": "test/lib9290_quad.f90:22-33", "function": "exp(-2 r)", "rnt": 2e-6, "h": 0.05,
                   "n": 590, "value": 0.5, "tolerance": 1e-12}, fh, indent=1)


def ne7_regression():
    import oracle
    from common import hydrogenic_case, ne7_block, oracle_for
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    orbs, blk = ne7_block()
    o = oracle_for(case)
    ind, val, ks, j2 = o.genintrk()
    nw = case["orb"].nw
    iab = np.array([[o.rinti(a, b, 0) if case["orb"].nak[a - 1] == case["orb"].nak[b - 1] else 0.0
                     for b in range(1, nw + 1)] for a in range(1, nw + 1)])
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    emt_shift = emt.copy()
    eav = oracle.shift_eav(blk.ncf, blk.iendc, emt_shift)
    ev, vec, info = oracle.maneig(0, blk.ncf, 3, blk.iendc, blk.irow, emt_shift)
    n = ind.size
    np.savez_compressed(os.path.join(HERE, "ne7_regression.npz"), indteirk=ind, valteirk=val, kstart=ks,
                        j2max=np.int32(j2), iab=iab, iendc=blk.iendc, irow=blk.irow, emt=emt, emt_shifted=emt_shift, eav=np.float64(eav),
                        eval=ev, evec=vec)
    print("ne7: R^k", n, "ncf", blk.ncf, "nnz", blk.nnz, "E", ev)


if __name__ == "__main__":
    hydrogenic_slater()
    quad_kat()
    ne7_regression()
