"""The SpMV autotuner (gg_hmat_tune, gg_hmat_tune_force): every variant it
may pick computes SPICMV2 (lib9290/spicmv2.f90:2-60) like the oracle, and
the tuner reports a timing for each and picks the fastest."""
import numpy as np
import pytest

from tests.common import hydrogenic_case

pytestmark = pytest.mark.gpu


def _block():
    from grasp_gb300 import Context, HMatrix
    from inputs import synth as S
    orbs = S.orbital_set(6, 3)
    case = hydrogenic_case(nmax=6, lmax=3, z=10.0)
    occ = lambda d: S.occupation(orbs, d)  # noqa: E731
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, -2): 2})]
    blk = S.ci_block(orbs, refs, [0] * len(orbs), two_j=2, parity=0, density=0.05, seed=9)
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ctx.genintrk()
    ctx.iabint_table()
    H = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    H.setham(blk.iq, blk.tlist, blk.vlists)
    return ctx, H, blk


@pytest.mark.parametrize("kernel,m,nvar", [(0, 10, 9), (0, 3, 9), (1, 1, 6)])
def test_every_variant_matches_oracle_spicmv2(gpu_ready, oracle_mod, kernel, m, nvar):
    from grasp_gb300 import SPLIT
    ctx, H, blk = _block()
    emt = H.emt()
    b = np.random.default_rng(7).normal(size=(blk.ncf, m))
    c0 = oracle_mod.spicmv2(blk.ncf, blk.iendc, blk.irow, emt, b)
    scale = np.abs(c0).max()
    outs = []
    for v in range(nvar):
        H.tune_force(kernel, m, v)
        c = H.spicmv2(b, precision=SPLIT)
        assert np.abs(c - c0).max() <= 1e-11 * scale, (kernel, m, v, np.abs(c - c0).max() / scale)
        outs.append(c)
    H.tune_force(kernel, m, -1)
    # the variants differ only in the order of their partial sums
    for c in outs[1:]:
        assert np.abs(c - outs[0]).max() <= 1e-13 * scale
    t = H.tune(kernel, m)
    assert len(t["ms"]) == nvar and all(x > 0 for x in t["ms"].values())
    assert t["chosen"] == min(t["ms"], key=t["ms"].get)


def test_solve_with_tuned_kernels_matches_oracle(gpu_ready, oracle_mod):
    """MANEIG with block passes and with single-vector passes, after the
    tuner picked its variants, against the oracle's MANEIG."""
    ctx, H, blk = _block()
    emt = H.emt()
    ev0, vec0, _ = oracle_mod.maneig(0, blk.ncf, 4, blk.iendc, blk.irow, emt, robust=True)
    for mblock in (1, 4):
        ev, vec, info = H.maneig(4, flavour=0, precision=1, mblock=mblock, robust=True)
        assert np.abs(ev - ev0).max() <= 1e-9
        assert np.abs(vec - vec0).max() <= 1e-7
