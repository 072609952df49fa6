"""Pins the oracle's DSPEVX restatement, SPICMV2, SETHAM and MANEIG/DVDSON
against numpy's LAPACK (eigh) and dense algebra on seeded matrices."""
import numpy as np
import pytest

from tests.common import hydrogenic_case, ne7_block, oracle_for


def _dense(ncf, iendc, irow, emt):
    A = np.zeros((ncf, ncf))
    for i in range(ncf):
        for p in range(iendc[i], iendc[i + 1]):
            j = irow[p] - 1
            A[i, j] = A[j, i] = emt[p]
    return A


@pytest.mark.parametrize("n,m", [(1, 1), (2, 2), (7, 3), (60, 10), (300, 5)])
def test_dspevx_vs_lapack(oracle_mod, n, m):
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    A = A + A.T + np.diag(np.arange(n) * 0.5)
    ap = np.concatenate([A[: j + 1, j] for j in range(n)])
    w, z = oracle_mod.dspevx(ap, n, 1, m)
    w0, z0 = np.linalg.eigh(A)
    np.testing.assert_allclose(w, w0[:m], rtol=0, atol=1e-12 * max(1.0, np.abs(w0).max()))
    for j in range(m):
        assert abs(abs(z[:, j] @ z0[:, j]) - 1.0) < 1e-10
        np.testing.assert_allclose(A @ z[:, j], w[j] * z[:, j], atol=1e-10 * max(1.0, np.abs(w0).max()))


def test_dspevx_degenerate(oracle_mod):
    n = 12
    A = np.diag([1.0, 1.0, 1.0, 2.0, 3.0, 3.0] + list(range(4, 10)))
    q, _ = np.linalg.qr(np.random.default_rng(2).standard_normal((n, n)))
    A = q @ A @ q.T
    ap = np.concatenate([A[: j + 1, j] for j in range(n)])
    w, z = oracle_mod.dspevx(ap, n, 1, 6)
    np.testing.assert_allclose(w, [1, 1, 1, 2, 3, 3], atol=1e-12)
    np.testing.assert_allclose(z.T @ z, np.eye(6), atol=1e-10)


def test_spicmv2_vs_dense(oracle_mod):
    orbs, blk = ne7_block()
    rng = np.random.default_rng(4)
    emt = rng.standard_normal(blk.nnz)
    A = _dense(blk.ncf, blk.iendc, blk.irow, emt)
    b = rng.standard_normal((blk.ncf, 2))
    c = oracle_mod.spicmv2(blk.ncf, blk.iendc, blk.irow, emt, b)
    np.testing.assert_allclose(c, A @ b, rtol=0, atol=1e-12 * np.abs(A @ b).max())


def test_setham_and_maneig_vs_lapack(oracle_mod):
    orbs, blk = ne7_block()
    case = hydrogenic_case(nmax=4, lmax=3, z=10.0)
    o = oracle_for(case)
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    eav = oracle_mod.shift_eav(blk.ncf, blk.iendc, emt)
    diag = emt[blk.iendc[1:] - 1]
    assert abs(np.mean(diag)) < 1e-9 * abs(eav)
    A = _dense(blk.ncf, blk.iendc, blk.irow, emt)
    w0, z0 = np.linalg.eigh(A)
    for flavour in (0, 1):
        ev, vec, info = oracle_mod.maneig(flavour, blk.ncf, 3, blk.iendc, blk.irow, emt)
        np.testing.assert_allclose(ev, w0[:3], atol=1e-10)
        for j in range(3):
            assert abs(abs(vec[:, j] @ z0[:, j]) - 1) < 1e-9
            # dominant component positive (maneig.f90:532-555)
            assert vec[np.argmax(np.abs(vec[:, j])), j] > 0


def test_gdvd_davidson_vs_lapack(oracle_mod):
    """The DVDSON restatement (rmcdhf flavour forces Davidson above 4000 only,
    so call with rci's flavour on a block above 2000 CSFs)."""
    from inputs import synth as S
    orbs = S.orbital_set(6, 3)
    occ = lambda d: S.occupation(orbs, d)  # noqa: E731
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, -2): 2})]
    blk = S.ci_block(orbs, refs, [0] * len(orbs), two_j=2, parity=0, density=0.05, seed=9)
    case = hydrogenic_case(nmax=6, lmax=3, z=10.0)
    o = oracle_for(case)
    ind, val, ks, _ = o.genintrk(nthreads=8)
    emt = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    oracle_mod.shift_eav(blk.ncf, blk.iendc, emt)
    A = _dense(blk.ncf, blk.iendc, blk.irow, emt)
    w0 = np.linalg.eigvalsh(A)
    # The reference exactly: INIEST2 on the leading 2000 block, then DVDSON.
    # Its first robust shift uses OLDVAL = 1e30 (dvdson.f90:703), the first
    # correction vector adds nothing and the coefficient test stops it after
    # two loops: eigenvalues are still good to ~1e-9 here, eigenvectors only
    # to the size of the residual.
    ev, vec, info = oracle_mod.maneig(0, blk.ncf, 4, blk.iendc, blk.irow, emt, nthreads=8)
    assert info["ierr"] == 0 and info["nloops"] == 2
    np.testing.assert_allclose(ev, w0[:4], atol=5e-9)
    # with a sane first shift DVDSON converges on the residual criterion
    ev, vec, info = oracle_mod.maneig(0, blk.ncf, 4, blk.iendc, blk.irow, emt, nthreads=8, robust=True)
    assert info["ierr"] == 0 and info["nloops"] > 2
    np.testing.assert_allclose(ev, w0[:4], atol=1e-9)
    r = A @ vec - vec * ev
    assert np.abs(r).max() < 1e-7
