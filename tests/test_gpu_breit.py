"""Breit integrals on the device (gg_genintbreit, gg_brint, gg_brintf:
rci90/genintbreit1.f90, genintbreit2.f90, brint1.f90, brintf.f90) against
the oracle's restatement of BESSEL, ZKF, RKINT, SKINT and BRRA:

- the tables' index structure (INDTP, KSTARTBREIT) is the oracle's exactly;
- the values agree to 1e-13 of the table's largest value: the device runs
  the reference's operations in the same order (no FMA contraction), and
  only log (QUAD's head term), sin and cos (the Bessel functions' asymptotic
  form) may round differently;
- every BRINTF type, including the coinciding-index cases BRRA branches
  on, at zero and at full frequency (WFACT 0 and 1);
- on GRASP's He orbitals with their rwfn energies (36 subshells), a sample
  of both tables."""
import numpy as np
import pytest

from tests import grasp_examples as G
from tests.common import hydrogenic_case, oracle_for

pytestmark = pytest.mark.gpu


def _hyd():
    from grasp_gb300 import Context
    case = hydrogenic_case(nmax=3, lmax=2, z=10.0)
    o = oracle_for(case)
    ob = case["orb"]
    nw = len(ob.nak)
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    e = -np.linspace(50.0, 1.0, nw)
    return ctx, o, nw, e


@pytest.mark.parametrize("wfact", [1.0, 0.0])
@pytest.mark.parametrize("itype", [1, 2])
def test_tables_match_oracle(gpu_ready, oracle_mod, itype, wfact):
    ctx, o, nw, e = _hyd()
    ind, val, kst, j2 = ctx.genintbreit(itype, wfact, e)
    ind0, val0, kst0, j20 = o.genintbreit(itype, wfact, e, nthreads=8)
    assert j2 == j20
    np.testing.assert_array_equal(ind, ind0)
    np.testing.assert_array_equal(kst, kst0)
    scale = np.abs(val0).max()
    err = np.abs(val - val0).max() / scale
    assert err <= 1e-13, err


def test_brintf_every_type_and_branch(gpu_ready, oracle_mod):
    ctx, o, nw, e = _hyd()
    items = []
    for t in range(1, 7):
        for (a, b, c, d) in [(2, 5, 4, 6), (3, 3, 7, 8), (2, 3, 2, 3), (2, 3, 3, 2), (4, 4, 4, 4), (1, 6, 6, 2)]:
            for k in (0, 1, 2):
                items.append((t, a, b, c, d, k))
    items = np.array(items, np.int32)
    for wfact in (1.0, 0.0):
        v = ctx.brintf(items, wfact, e)
        v0 = np.array([o.brintf(*map(int, it), wfact, e) for it in items])
        scale = max(1e-300, np.abs(v0).max())
        assert np.all(np.isfinite(v))
        assert np.abs(v - v0).max() <= 1e-13 * scale, (wfact, np.abs(v - v0).max() / scale)


def test_brint_lookup(gpu_ready, oracle_mod):
    from grasp_gb300 import GGError
    ctx, o, nw, e = _hyd()
    key = nw + 1
    ind, val, kst, j2 = ctx.genintbreit(1, 1.0, e)
    for pos in (0, ind.size // 3, ind.size - 1):
        k = int(np.searchsorted(kst, pos + 1, side="right") - 1)
        x = int(ind[pos])
        d = x % key; x //= key
        c = x % key; x //= key
        b = x % key; a = x // key
        assert ctx.brint(1, a, b, c, d, k) == val[pos]
    with pytest.raises(GGError):
        ctx.brint(1, 1, 1, 1, 1, j2 + 1)
    with pytest.raises(GGError):
        ctx.brint(2, 1, 2, 3, 4, 0)  # no type-2 table yet


def test_grasp_he_tables_sampled(gpu_ready, oracle_mod):
    from grasp_gb300 import Context
    d = G.load("He", oracle_mod)
    ctx = Context(0)
    ctx.set_grid(d["n"], d["rnt"], d["h"], d["c"], d["zz"])
    ctx.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    nw = len(d["nak"])
    key = nw + 1
    for itype in (1, 2):
        ind, val, kst, j2 = ctx.genintbreit(itype, 1.0, d["e"])
        assert ind.size == kst[-1] - 1 and np.all(np.isfinite(val))
        rng = np.random.default_rng(itype)
        pos = rng.choice(ind.size, 200, replace=False)
        got, ref = [], []
        for p in pos:
            k = int(np.searchsorted(kst, p + 1, side="right") - 1)
            x = int(ind[p])
            dd = x % key; x //= key
            c = x % key; x //= key
            b = x % key; a = x // key
            got.append(val[p])
            ref.append(o.brintf(itype, a, b, c, dd, k, 1.0, d["e"]))
        got, ref = np.array(got), np.array(ref)
        assert np.abs(got - ref).max() <= 1e-13 * np.abs(val).max(), np.abs(got - ref).max() / np.abs(val).max()
