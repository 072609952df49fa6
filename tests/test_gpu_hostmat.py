"""Blocks whose matrix is not on the device.

SPODMV (rci90/spodmv.f90:3, the product for a block too large to keep in
memory) -> gg_hmat_create_host + gg_spodmv: the full symmetric matrix in
pinned host memory, read over the host link by the same kernels as a
device-resident matrix. The products are bit for bit those of the same
matrix on the device (same entry order, same sums) and match the oracle's
SPODMV to the SPICMV2 tolerances (FP64 1e-13, split 1e-11 relative to the
largest |y|); MANEIG on it returns the device-resident solve's eigenpairs
bit for bit. DNICMV (rci90/dnicmv.f90:3, the dense packed triangle) ->
gg_hmat_create_packed + gg_spicmv2.
"""
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
    eav = H.setham(blk.iq, blk.tlist, blk.vlists)
    shifted = H.emt()
    # the rows as rci writes them to rci.res: the diagonal unshifted
    raw = shifted.copy()
    d = blk.iendc[1:] - 1
    raw[d] += eav
    return ctx, H, blk, raw, eav


def _pair(ctx, blk, raw, eav, precision):
    """The same matrix in host memory and on the device (diagonal EMT - EAV
    computed the same way for both)."""
    from grasp_gb300 import HMatrix
    hm = HMatrix.host(ctx, blk.ncf, blk.iendc, blk.irow, raw, eav, precision)
    dm = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    emt = raw.copy()
    d = blk.iendc[1:] - 1
    emt[d] = raw[d] - eav
    dm.set_emt(emt)
    # the single-vector split kernel's sums depend on its lanes per row:
    # both matrices launch the same variants
    if precision == 1:
        for x in (hm, dm):
            for m in range(1, 17):
                x.tune_force(0, m, 4)
            x.tune_force(1, 1, 1)
    return hm, dm


@pytest.mark.parametrize("precision", [0, 1])
def test_host_products_match_device_and_oracle(gpu_ready, oracle_mod, precision):
    ctx, H, blk, raw, eav = _block()
    hm, dm = _pair(ctx, blk, raw, eav, precision)
    assert hm.host_precision == precision and dm.host_precision is None
    rng = np.random.default_rng(5)
    for m in (1, 3, 10, 17):
        b = rng.standard_normal((blk.ncf, m))
        c = hm.spodmv(b)
        np.testing.assert_array_equal(c, dm.spicmv2(b, precision))
        np.testing.assert_array_equal(c, hm.spicmv2(b, precision))
        c0 = oracle_mod.spodmv(blk.ncf, blk.iendc, blk.irow, raw, eav, b)
        tol = 1e-13 if precision == 0 else 1e-11
        assert np.abs(c - c0).max() <= tol * np.abs(c0).max(), (m, np.abs(c - c0).max())


@pytest.mark.parametrize("precision", [0, 1])
def test_host_maneig_matches_device_and_oracle(gpu_ready, oracle_mod, precision):
    """MANEIG on a host-resident block (the leading-block stage from its kept
    leading rows, the full stage reading the matrix over the host link)."""
    ctx, H, blk, raw, eav = _block()
    hm, dm = _pair(ctx, blk, raw, eav, precision)
    assert blk.ncf > 2000
    emt = raw.copy()
    emt[blk.iendc[1:] - 1] -= eav
    # the robust first shift: the reference's sentinel shift can stop this
    # block's non-robust run early (gg_dvd_params.robust)
    ev0, vec0, _ = oracle_mod.maneig(0, blk.ncf, 4, blk.iendc, blk.irow, emt, nthreads=8, robust=True)
    for mblock in (1, 4):
        ev, vec, info = hm.maneig(4, flavour=0, precision=precision, mblock=mblock, robust=True)
        evd, vecd, infod = dm.maneig(4, flavour=0, precision=precision, mblock=mblock, robust=True)
        assert info["ierr"] == 0 and info["nloops"] == infod["nloops"]
        np.testing.assert_array_equal(ev, evd)
        np.testing.assert_array_equal(vec, vecd)
        assert np.abs(ev - ev0).max() <= 1e-9, (mblock, ev, ev0)
        assert np.abs(vec - vec0).max() <= 1e-7


def test_host_matrix_refusals(gpu_ready):
    from grasp_gb300 import FP64, SPLIT, GGError, HMatrix, maneig_batched
    ctx, H, blk, raw, eav = _block()
    hm = HMatrix.host(ctx, blk.ncf, blk.iendc, blk.irow, raw, eav, SPLIT)
    b = np.ones((blk.ncf, 1))
    with pytest.raises(GGError):
        hm.spicmv2(b, FP64)
    with pytest.raises(GGError):
        hm.maneig(2, precision=FP64)
    with pytest.raises(GGError):
        hm.emt()
    with pytest.raises(GGError):
        hm.set_emt(raw)
    with pytest.raises(GGError):
        hm.setham(blk.iq, blk.tlist, blk.vlists)
    with pytest.raises(GGError):
        HMatrix.view(hm)
    with pytest.raises(GGError):
        maneig_batched(ctx, [hm], [2], precision=SPLIT)
    with pytest.raises(GGError):
        H.spodmv(b)  # a matrix on the device
    bad = blk.irow.copy()
    bad[blk.iendc[5] - 1] = 1  # row 5 no longer ends with its diagonal
    with pytest.raises(GGError):
        HMatrix.host(ctx, blk.ncf, blk.iendc, bad, raw, eav, FP64)
    with pytest.raises(GGError):
        HMatrix.host(ctx, blk.ncf, blk.iendc, blk.irow, raw, eav, 7)
    # the matrix still works after the refusals
    c = hm.spodmv(b)
    assert np.isfinite(c).all()


def test_packed_dense_dnicmv(gpu_ready, oracle_mod):
    from grasp_gb300 import Context, HMatrix
    n = 300
    rng = np.random.default_rng(2)
    a = rng.standard_normal((n, n)) * 0.01
    a = a + a.T + np.diag(np.arange(n, dtype=float))
    ap = np.concatenate([a[i, :i + 1] for i in range(n)])
    ctx = Context(0)
    hm = HMatrix.packed(ctx, n, ap)
    b = rng.standard_normal((n, 4))
    c = hm.spicmv2(b)
    c0 = oracle_mod.dnicmv(n, ap, b)
    assert np.abs(c - c0).max() <= 1e-13 * np.abs(c0).max()
    assert np.abs(c - a @ b).max() <= 1e-12 * np.abs(c0).max()
    ev, vec, info = hm.maneig(3, flavour=0)
    assert info["ierr"] == 0
    assert np.abs(ev - np.linalg.eigvalsh(a)[:3]).max() <= 1e-9
