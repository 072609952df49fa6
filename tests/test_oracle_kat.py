"""Pins the CPU oracle (the checker) against known answers.

- QUAD: the reference's own unit test, test/lib9290_quad.f90:22-33
  (integral of exp(-2r) on the 590-point grid = 0.5 within 1e-12).
- RINTI: for an exact Dirac-Coulomb eigenfunction (DCBSRW) and a point
  nucleus, I(aa) equals minus the binding energy DCBSRW returns.
- SLATER / YZK: hydrogenic Slater integrals in the nonrelativistic limit
  (speed of light scaled up) against their closed forms, e.g.
  F0(1s,1s) = 5Z/8 (Condon & Shortley; Bethe & Salpeter).
- R^k symmetries, TRIANGRK, GENINTRK ordering, RKINTC lookups, CLRX.
"""
from fractions import Fraction as F

import numpy as np
import pytest

from tests.common import CVAC, hydrogenic_case, oracle_for


def test_quad_kat(oracle_mod):
    o = oracle_mod.Oracle(n=590, rnt=2.0e-6, h=0.05, c=CVAC, z=1)
    r, rp, _ = o.grid()
    ta = np.exp(-2 * r) * rp
    res = o.quad(ta, 590)
    assert abs(res - 0.5) <= 1e-12


def test_grid_radgrd(oracle_mod):
    o = oracle_mod.Oracle(n=590, rnt=2.0e-6 / 26, h=0.05, c=CVAC, z=26)
    r, rp, rpor = o.grid()
    i = np.arange(600)
    assert r[0] == 0.0 and rp[0] == 2.0e-6 / 26
    np.testing.assert_allclose(r[1:], 2.0e-6 / 26 * np.expm1(0.05 * i[1:]), rtol=1e-13)
    np.testing.assert_allclose(rpor[1:], rp[1:] / r[1:], rtol=1e-13)


def test_setqic_constants(oracle_mod):
    o = oracle_mod.Oracle(n=590, rnt=2.0e-6, h=0.05, c=CVAC, z=1)
    c, cnc = o.qic()
    f = 0.05 / 720.0
    assert c[0] == f * 224 and c[1] == f * 1024 and c[2] == f * 384 and c[3] == 2 * c[0]
    # CNC5C(2:5, 2): the semi-open 5-point starter rows (setqic.f90 C5NUM)
    np.testing.assert_array_equal(cnc[0], f * np.array([646.0, -264.0, 106.0, -19.0]))


@pytest.mark.parametrize("z", [1.0, 10.0, 26.0])
def test_rinti_hydrogenic_energy(oracle_mod, z):
    case = hydrogenic_case(nmax=3, lmax=2, z=z, sigma=np.zeros(9))
    o = oracle_for(case)
    e = case["orb"].e
    for j in range(1, case["orb"].nw + 1):
        val = o.rinti(j, j, 0)
        assert abs(val + e[j - 1]) <= 2e-9 * abs(e[j - 1]), (j, val, -e[j - 1])


HYD = [  # (a, b, c, d, k, value / Z) for nonrelativistic hydrogenic orbitals
    ((1, -1), (1, -1), (1, -1), (1, -1), 0, F(5, 8)),
    ((1, -1), (2, -1), (1, -1), (2, -1), 0, F(17, 81)),
    ((1, -1), (2, -1), (2, -1), (1, -1), 0, F(16, 729)),
    ((2, -1), (2, -1), (2, -1), (2, -1), 0, F(77, 512)),
    ((2, -2), (2, -2), (2, -2), (2, -2), 0, F(93, 512)),
    ((2, -2), (2, -2), (2, -2), (2, -2), 2, F(45, 512)),
    ((1, -1), (2, -2), (1, -1), (2, -2), 0, F(59, 243)),
    ((1, -1), (2, -2), (2, -2), (1, -1), 1, F(112, 2187)),
    ((2, -1), (2, 1), (2, -1), (2, 1), 0, F(83, 512)),
    ((2, -1), (2, 1), (2, 1), (2, -1), 1, F(45, 512)),
]


def test_slater_hydrogenic_nonrel_limit(oracle_mod):
    z = 2.0
    case = hydrogenic_case(nmax=2, lmax=1, z=z, c=CVAC * 1.0e4, sigma=np.zeros(4))
    o = oracle_for(case)
    idx = {orb: j + 1 for j, orb in enumerate(case["orbs"])}
    for a, b, c, d, k, frac in HYD:
        v = o.slater(idx[a], idx[b], idx[c], idx[d], k)
        ref = float(frac) * z
        # DCBSRW cuts each orbital's tail at ACCY/10 = 1.6e-9 (dcbsrw.f90:218),
        # which bounds the agreement with the closed forms at ~1e-8
        assert abs(v - ref) <= 2e-8 * ref, (a, b, c, d, k, v, ref)


def test_slater_symmetries(oracle_mod):
    case = hydrogenic_case(nmax=3, lmax=2, z=10.0)
    o = oracle_for(case)
    rng = np.random.default_rng(0)
    from inputs.synth import lval
    L = [lval(k) for _, k in case["orbs"]]
    nw = len(L)
    checked = 0
    while checked < 40:
        a, b, c, d = rng.integers(1, nw + 1, size=4)
        for k in range(0, 5):
            if not (oracle_mod.triangrk(L[a - 1], k, L[c - 1]) and oracle_mod.triangrk(L[b - 1], k, L[d - 1])):
                continue
            v = o.slater(a, b, c, d, k)
            # a <-> c and b <-> d leave SLATER's arithmetic unchanged: bit-identical.
            # The pair swap (ac) <-> (bd) is not a symmetry of the reference's
            # numbers: it integrates rho_bd Y_ac instead of rho_ac Y_bd with the
            # MTP cut of slater.f90:56-60, and for k = 0 with b != d YZK forces
            # the asymptote of Z to 0 (yzk.f90:154-158) even when b and d differ
            # only in j. GENINTRK fixes the order (a <= b) and so does this library.
            assert o.slater(c, b, a, d, k) == v and o.slater(a, d, c, b, k) == v
            checked += 1


def test_triangrk():
    import oracle
    assert oracle.triangrk(1, 1, 0) and not oracle.triangrk(1, 0, 0) and oracle.triangrk(2, 2, 2)
    assert not oracle.triangrk(1, 3, 1) and oracle.triangrk(3, 6, 3) and not oracle.triangrk(0, 1, 0)


def test_genintrk_order_and_rkintc(oracle_mod):
    case = hydrogenic_case(nmax=3, lmax=2, z=10.0)
    o = oracle_for(case)
    ind, val, ks, j2 = o.genintrk()
    assert j2 == 5  # 3d has 2j = 5
    for k in range(j2 + 1):
        seg = ind[ks[k] - 1:ks[k + 1] - 1]
        assert np.all(np.diff(seg) > 0)  # ascending within each k (rkintc binary search)
    key = o.nw + 1
    rng = np.random.default_rng(1)
    for t in rng.integers(0, len(ind), size=50):
        k = int(np.searchsorted(ks, t + 1, side="right") - 1)
        p = int(ind[t])
        a, b, c, d = p // key ** 3, (p // key ** 2) % key, (p // key) % key, p % key
        # any symmetric permutation finds the same entry
        assert o.rkintc((ind, val, ks), c, d, a, b, k) == val[t]
        assert o.rkintc((ind, val, ks), a, b, c, d, k) == val[t]
        assert abs(val[t] - o.slater(a, b, c, d, k)) == 0.0
    with pytest.raises(KeyError):
        o.rkintc((ind, val, ks), 1, 1, 1, 3, 0)  # 1s-2p- with k = 0 violates parity


def test_clrx_values(oracle_mod):
    # CLRX(kappa, k, kappa') is the 3j symbol (j k j'; 1/2 0 -1/2)
    # |<1s|C^0|1s>| -> CLRX(-1,0,-1)^2 = 1/2 ; (1/2 1 1/2; 1/2 0 -1/2)^2 = 1/6
    assert abs(oracle_mod.clrx(-1, 0, -1) ** 2 - 0.5) < 1e-14
    assert abs(oracle_mod.clrx(-1, 1, 1) ** 2 - 1.0 / 6.0) < 1e-14
    assert oracle_mod.clrx(-1, 2, -1) == 0.0
