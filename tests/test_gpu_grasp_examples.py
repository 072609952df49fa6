"""The CUDA path on GRASP's own data (tests/golden/grasp_examples): the
orbitals rmcdhf wrote for He (220-point grid, 36 subshells up to 6h, point
nucleus) and Ge II (590-point grid, Fermi nucleus, 28-electron core), and
the T/V lists of their CSF lists from the angular engine.

- R^k tables (GENINTRK, FP64 and the tensor-core split) and I(ab) against
  the oracle on the same orbitals; SLATER spot values.
- SETHAM on the device against the oracle's.
- MANEIG on the device: the level energies rmcdhf printed, and for Ge II
  its mixing coefficients (.m), sign included.
"""
import numpy as np
import pytest

from grasp_gb300 import angular as A
from grasp_gb300 import formats as F
from tests import grasp_examples as G

pytestmark = pytest.mark.gpu


def _setup(run, oracle_mod):
    from grasp_gb300 import Context
    d = G.load(run, oracle_mod)
    ctx = Context(0)
    ctx.set_grid(d["n"], d["rnt"], d["h"], d["c"], d["zz"])
    ctx.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    o = oracle_mod.Oracle(n=d["n"], rnt=d["rnt"], h=d["h"], c=d["c"], zz=d["zz"])
    o.set_orbitals(d["nak"], d["mf"], d["pf"], d["qf"])
    return d, ctx, o


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_tables_on_grasp_orbitals(gpu_ready, oracle_mod, run):
    from grasp_gb300 import FP64, SPLIT
    d, ctx, o = _setup(run, oracle_mod)
    ind0, val0, ks0, j2 = o.genintrk()
    scale = np.maximum(np.abs(val0), 1e-2)
    for prec in (FP64, SPLIT):
        n, j2g = ctx.genintrk(precision=prec)
        assert (n, j2g) == (ind0.size, j2)
        ind, val, ks = ctx.rk_table()
        np.testing.assert_array_equal(ind, ind0)
        np.testing.assert_array_equal(ks, ks0)
        err = np.abs(val - val0) / scale
        assert err.max() <= 1e-12, (prec, err.max())
    iab = ctx.iabint_table()
    nw = len(d["nak"])
    for a in range(nw):
        for b in range(nw):
            if d["nak"][a] == d["nak"][b]:
                ref = o.rinti(a + 1, b + 1)
                assert abs(iab[a, b] - ref) <= 1e-12 * max(1.0, abs(ref)), (a, b, iab[a, b], ref)
            else:
                assert np.isnan(iab[a, b])
    rng = np.random.default_rng(3)
    for _ in range(12):
        a, b, c, e = (int(x) for x in rng.integers(1, nw + 1, size=4))
        for k in range(0, 4):
            ref = o.slater(a, b, c, e, k)
            got = ctx.slater(a, b, c, e, k)
            assert abs(got - ref) <= 1e-12 * max(abs(ref), 1e-2), (a, b, c, e, k, got, ref)


@pytest.mark.parametrize("run", ["He", "Ge"])
def test_setham_and_maneig_reproduce_rmcdhf(gpu_ready, oracle_mod, run):
    from grasp_gb300 import FP64, SPLIT, HMatrix
    d, ctx, o = _setup(run, oracle_mod)
    o.genintrk()
    csl = F.read_csl(f"{G.ROOT}/{G.RUNS[run]}.c")
    mix = F.read_mix(f"{G.ROOT}/{G.RUNS[run]}.m") if run == "Ge" else None
    for prec in (FP64, SPLIT):
        ctx.genintrk(precision=prec)
        ctx.iabint_table()
        for bi, blk in enumerate(csl.blocks):
            ab = A.block_lists(csl, bi)
            H = HMatrix(ctx, ab.ncf, ab.iendc, ab.irow)
            eav = H.setham(ab.iq, ab.tlist, ab.vlists)
            emt0 = o.setham(ab.ncf, ab.nnz, ab.iendc, ab.iq, ab.tlist, ab.vlists)
            eav0 = oracle_mod.shift_eav(ab.ncf, ab.iendc, emt0)
            assert abs(eav - eav0) <= 1e-12 * abs(eav0)
            emt = H.emt()
            assert np.abs(emt - emt0).max() <= 1e-12 * np.abs(emt0).max()
            levels = [lv for lv in d["levels"] if lv[1] == blk.two_j]
            nvec = max(lv[0] for lv in levels)
            for flavour in (0, 1):
                ev, vec, info = H.maneig(nvec, flavour=flavour, precision=prec)
                for lv in levels:
                    # printed with 13 significant digits
                    tol = 1e-12 if run == "He" else 1e-9
                    assert abs(eav + ev[lv[0] - 1] - lv[3]) <= tol, (run, prec, flavour, blk.two_j, lv, eav + ev)
                if mix is not None:
                    mb = mix.blocks[bi]
                    assert abs(eav - mb.eav) <= 1e-10
                    np.testing.assert_allclose(vec[:, 0], mb.evec[:, 0], atol=1e-7)
            H.close()
