"""The oracle's YPOT and XPOT (rmcdhf90/ypot.f90, xpot.f90) on GRASP's He
orbitals: the direct and exchange potentials of a SETCOF-style coefficient
list are the list's YZK functions combined in order (checked against the
oracle's own YZK, element by element), and bad labels are errors."""
import numpy as np
import pytest

from tests import grasp_examples as G

KEY = 215


def _lists(nw, n=30, seed=4):
    rng = np.random.default_rng(seed)
    k = rng.integers(0, 5, n)
    a = rng.integers(1, nw + 1, n)
    b = rng.integers(1, nw + 1, n)
    io = rng.integers(1, nw + 1, n)
    nya = ((b * KEY + a) * KEY + k).astype(np.int32)
    nxa = (((io * KEY + b) * KEY + a) * KEY + k).astype(np.int32)
    return k, a, b, io, nya, nxa, rng.normal(size=n)


def test_ypot_xpot_are_ordered_yzk_sums(oracle_mod):
    d = G.load("He", oracle_mod)
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    nw = len(d["nak"])
    k, a, b, io, nya, nxa, co = _lists(nw)
    yp0 = d["zz"][:d["n"]].copy()
    xp0 = np.zeros(d["n"]); xq0 = np.zeros(d["n"])
    for t in range(len(co)):
        tb, _ = o.yzk(int(k[t]), int(a[t]), int(b[t]))
        yp0 = yp0 - co[t] * tb
        ctb = (co[t] / d["c"]) * tb
        xp0 = xp0 + ctb * d["qf"][io[t] - 1, :d["n"]]
        xq0 = xq0 - ctb * d["pf"][io[t] - 1, :d["n"]]
    np.testing.assert_array_equal(o.ypot(nya, co), yp0)
    xp, xq = o.xpot(nxa, co)
    np.testing.assert_array_equal(xp, xp0)
    np.testing.assert_array_equal(xq, xq0)
    with pytest.raises(ValueError):
        o.ypot(np.array([(1 * KEY + (nw + 1)) * KEY], np.int32), np.ones(1))
