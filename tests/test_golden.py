"""Golden fixtures (tests/golden, written by tests/golden/make_golden.py):
closed-form hydrogenic Slater integrals, the reference's QUAD unit test, and
stored oracle vectors for the Ne VII block. CPU tests pin the oracle to them;
the GPU tests compare the CUDA path with the stored vectors.

Tolerances: index arrays bit-exact; R^k <= 1e-12 relative (1e-14 absolute
floor); I(ab) and EMT <= 1e-12 relative to the largest |value|; eigenvalues
<= 1e-9 Eh; eigenvectors <= 1e-7 after the dominant-component sign fix.
"""
import json
import os
from fractions import Fraction

import numpy as np
import pytest

from tests.common import CVAC, hydrogenic_case, ne7_block, oracle_for

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
KAPPA = {"1s": (1, -1), "2s": (2, -1), "2p": (2, 1)}  # 2p-: its nonrelativistic limit is the 2p closed form


def load_ne7():
    return dict(np.load(os.path.join(GOLD, "ne7_regression.npz")))


def test_quad_kat_fixture(oracle_mod):
    with open(os.path.join(GOLD, "quad_kat.json")) as fh:
        kat = json.load(fh)
    o = oracle_mod.Oracle(n=kat["n"], rnt=kat["rnt"], h=kat["h"], zz=np.ones(kat["n"]))
    r, rp, _ = o.grid()
    ta = rp * np.exp(-2.0 * r)
    assert abs(o.quad(ta, kat["n"]) - kat["value"]) <= kat["tolerance"]


def test_hydrogenic_slater_fixture(oracle_mod):
    with open(os.path.join(GOLD, "hydrogenic_slater.json")) as fh:
        gold = json.load(fh)["integrals"]
    z = 2.0
    case = hydrogenic_case(nmax=2, lmax=1, z=z, c=CVAC * 1.0e4, sigma=np.zeros(4))
    o = oracle_for(case)
    idx = {orb: j + 1 for j, orb in enumerate(case["orbs"])}
    for g in gold:
        ref = float(Fraction(g["value_over_Z"])) * z
        v = o.slater(idx[KAPPA[g["a"]]], idx[KAPPA[g["b"]]], idx[KAPPA[g["c"]]], idx[KAPPA[g["d"]]], g["k"])
        # DCBSRW's tail cut (dcbsrw.f90:218) bounds the agreement at ~1e-8
        assert abs(v - ref) <= 2e-8 * ref, (g, v, ref)


def test_ne7_oracle_regression(oracle_mod):
    g = load_ne7()
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    np.testing.assert_array_equal(blk.iendc, g["iendc"])
    np.testing.assert_array_equal(blk.irow, g["irow"])
    o = oracle_for(case)
    ind, val, ks, j2 = o.genintrk()
    np.testing.assert_array_equal(ind, g["indteirk"])
    np.testing.assert_array_equal(ks, g["kstart"])
    assert j2 == int(g["j2max"])
    np.testing.assert_allclose(val, g["valteirk"], rtol=1e-13, atol=1e-15)
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    np.testing.assert_allclose(emt, g["emt"], rtol=0, atol=1e-12 * np.abs(g["emt"]).max())


@pytest.mark.gpu
def test_ne7_gpu_against_golden(gpu_ready):
    from grasp_gb300 import Context, HMatrix
    g = load_ne7()
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    _, blk = ne7_block()
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ctx.genintrk()
    ind, val, ks = ctx.rk_table()
    np.testing.assert_array_equal(ind, g["indteirk"])
    np.testing.assert_array_equal(ks, g["kstart"])
    ref = g["valteirk"]
    big = np.abs(ref) > 1e-14
    assert np.all(np.abs(val[big] - ref[big]) <= 1e-12 * np.abs(ref[big]))
    assert np.all(np.abs(val[~big] - ref[~big]) <= 1e-14)
    iab = ctx.iabint_table()
    same = ob.nak[:, None] == ob.nak[None, :]  # I(ab) exists for kappa_a = kappa_b (NaN elsewhere)
    assert np.all(np.isnan(iab[~same]))
    np.testing.assert_allclose(iab[same], g["iab"][same], rtol=0, atol=1e-12 * np.abs(g["iab"]).max())
    H = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    eav = H.setham(blk.iq, blk.tlist, blk.vlists)
    assert abs(eav - float(g["eav"])) <= 1e-12 * abs(float(g["eav"]))
    np.testing.assert_allclose(H.emt(), g["emt_shifted"], rtol=0, atol=1e-12 * np.abs(g["emt"]).max())
    for precision in (0, 1):
        ev, vec, _ = H.maneig(3, flavour=0, precision=precision)
        assert np.abs(ev - g["eval"]).max() <= 1e-9
        assert np.abs(vec - g["evec"]).max() <= 1e-7
