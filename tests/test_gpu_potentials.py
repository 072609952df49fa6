"""gg_ypot / gg_xpot (rmcdhf's YPOT and XPOT, rmcdhf90/ypot.f90:35-49,
xpot.f90:31-54) on GRASP's own orbitals (He: 220-point grid, 36 subshells;
Ge II: Fermi nucleus, 590 points) against the oracle's YPOT and XPOT for the
same coefficient lists: the device builds every YZK function of the list on
all N points and combines them in the list's order, so the potentials agree
to rounding (bar: 1e-14 of the largest |value|). Labels outside the orbital
set are errors."""
import numpy as np
import pytest

from tests import grasp_examples as G
from tests.test_potentials import KEY, _lists

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_potentials_match_oracle(gpu_ready, oracle_mod, run):
    from grasp_gb300 import Context, GGError
    d = G.load(run, oracle_mod)
    ctx = Context(0)
    ctx.set_grid(d["n"], d["rnt"], d["h"], d["c"], d["zz"])
    ctx.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    nw = len(d["nak"])
    for seed in (4, 5):
        k, a, b, io, nya, nxa, co = _lists(nw, n=60, seed=seed)
        yp, yp0 = ctx.ypot(nya, co), o.ypot(nya, co)
        assert np.abs(yp - yp0).max() <= 1e-14 * np.abs(yp0).max(), np.abs(yp - yp0).max()
        (xp, xq), (xp0, xq0) = ctx.xpot(nxa, co), o.xpot(nxa, co)
        assert np.abs(xp - xp0).max() <= 1e-14 * np.abs(xp0).max()
        assert np.abs(xq - xq0).max() <= 1e-14 * np.abs(xq0).max()
    # an empty list: YP = ZZ, XP = XQ = 0
    np.testing.assert_array_equal(ctx.ypot(np.zeros(0, np.int32), np.zeros(0)), d["zz"][:d["n"]])
    with pytest.raises(GGError):
        ctx.ypot(np.array([(1 * KEY + (nw + 1)) * KEY], np.int32), np.ones(1))
    with pytest.raises(GGError):
        ctx.xpot(np.array([((1 * KEY + 1) * KEY + 1) * KEY + 21], np.int32), np.ones(1))  # K above 20
