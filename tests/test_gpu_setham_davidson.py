"""GPU parity: SETHAM (EMT from T/V lists), SPICMV2, MANEIG against the oracle.

- EMT: the GPU adds each element's contributions in the reference's order
  from the device R^k / I(ab) tables; the oracle calls SLATER/RINTI per
  label as rmcdhf's SETHAM does. They agree to 1e-12 relative (absolute floor
  1e-12 Eh on cancelled elements); the sparse structure is bit-exact.
- SPICMV2: FP64 to 1e-13 relative of the largest |y|, split to 1e-11.
- MANEIG: eigenvalues within 1e-9 Eh, eigenvectors within 1e-7 after the
  reference's sign fix (spec tolerances).
"""
import numpy as np
import pytest

from tests.common import hydrogenic_case, ne7_block, oracle_for

pytestmark = pytest.mark.gpu


def _setup(z=10.0, max_ncf=0, density=0.0, seed=3):
    import oracle
    from grasp_gb300 import Context, HMatrix
    orbs, blk = ne7_block(max_ncf=max_ncf, density=density, seed=seed)
    case = hydrogenic_case(nmax=4, lmax=3, z=z)
    assert case["orbs"] == orbs
    o = oracle_for(case)
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ctx.genintrk()
    ctx.iabint_table()
    H = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    return o, ctx, H, blk, oracle


def test_setham_parity(gpu_ready, oracle_mod):
    o, ctx, H, blk, oracle = _setup()
    eav = H.setham(blk.iq, blk.tlist, blk.vlists)
    emt = H.emt()
    ref = o.setham(blk.ncf, blk.nnz, blk.iendc, blk.iq, blk.tlist, blk.vlists)
    eav0 = oracle.shift_eav(blk.ncf, blk.iendc, ref)
    assert abs(eav - eav0) <= 1e-12 * abs(eav0)
    err = np.abs(emt - ref)
    assert np.all(err <= 1e-12 * np.abs(ref) + 1e-12), float(err.max())


def test_setham_bad_label_is_an_error(gpu_ready):
    from grasp_gb300 import GGError
    o, ctx, H, blk, oracle = _setup()
    t = dict(blk.tlist)
    t["lab"] = t["lab"].copy()
    t["lab"][0] = 215 * 1 + 3  # I(2p-, 1s): kappas differ
    with pytest.raises(GGError):
        H.setham(blk.iq, t, blk.vlists)
    t = dict(blk.tlist)
    t["loc"] = t["loc"].copy()
    t["loc"][0] = blk.nnz + 1  # LOC > NELMNT (setham.f90:264-268)
    with pytest.raises(GGError):
        H.setham(blk.iq, t, blk.vlists)


def test_hmat_bad_structure_is_an_error(gpu_ready):
    """IENDC / IROW outside the lower-triangle-by-rows mode of spicmv2.f90
    (checked on the device for IROW): the matrix is refused."""
    from grasp_gb300 import Context, GGError, HMatrix
    orbs, blk = ne7_block()
    ctx = Context(0)
    HMatrix(ctx, blk.ncf, blk.iendc, blk.irow).close()  # the real structure is accepted
    r = blk.iendc[5] - 1                                 # diagonal of row 5 (1-based)
    irow = blk.irow.copy()
    irow[r] = 3
    with pytest.raises(GGError, match="diagonal"):
        HMatrix(ctx, blk.ncf, blk.iendc, irow)
    irow = blk.irow.copy()
    row = int(np.argmax(np.diff(blk.iendc) > 1)) + 1     # a row with an off-diagonal entry
    irow[blk.iendc[row - 1]] = row + 1                   # above the diagonal
    with pytest.raises(GGError, match="lower triangle"):
        HMatrix(ctx, blk.ncf, blk.iendc, irow)
    iendc = blk.iendc.copy()
    iendc[3] = iendc[2]                                  # an empty row
    with pytest.raises(GGError):
        HMatrix(ctx, blk.ncf, iendc, blk.irow)


def test_spicmv2_parity(gpu_ready, oracle_mod):
    o, ctx, H, blk, oracle = _setup()
    H.setham(blk.iq, blk.tlist, blk.vlists)
    emt = H.emt()
    rng = np.random.default_rng(11)
    b = rng.standard_normal((blk.ncf, 3))
    c0 = oracle.spicmv2(blk.ncf, blk.iendc, blk.irow, emt, b)
    from grasp_gb300 import FP64, SPLIT
    c64 = H.spicmv2(b, FP64)
    cs = H.spicmv2(b, SPLIT)
    scale = np.abs(c0).max()
    assert np.abs(c64 - c0).max() <= 1e-13 * scale
    assert np.abs(cs - c0).max() <= 1e-11 * scale
    # deterministic: same bits on a second call
    np.testing.assert_array_equal(H.spicmv2(b, FP64), c64)


@pytest.mark.parametrize("precision", [0, 1])
def test_maneig_dense_range(gpu_ready, oracle_mod, precision):
    """ncf <= 2000: the reference (rci) uses DSPEVX; the GPU runs Davidson."""
    o, ctx, H, blk, oracle = _setup()
    H.setham(blk.iq, blk.tlist, blk.vlists)
    emt = H.emt()
    nvec = 3
    ev0, vec0, _ = oracle.maneig(0, blk.ncf, nvec, blk.iendc, blk.irow, emt)
    ev, vec, info = H.maneig(nvec, flavour=0, precision=precision)
    assert info["ierr"] == 0
    assert np.abs(ev - ev0).max() <= 1e-9, (ev, ev0)
    assert np.abs(vec - vec0).max() <= 1e-7
    # compare with LAPACK (numpy) on the dense matrix too
    A = np.zeros((blk.ncf, blk.ncf))
    for i in range(blk.ncf):
        for p in range(blk.iendc[i], blk.iendc[i + 1]):
            j = blk.irow[p] - 1
            A[i, j] = A[j, i] = emt[p]
    w = np.linalg.eigvalsh(A)[:nvec]
    assert np.abs(ev - w).max() <= 1e-9


def test_maneig_davidson_path(gpu_ready, oracle_mod):
    """ncf > 2000: INIEST2 on the leading 2000 block, then DVDSON (rci)."""
    import oracle
    from grasp_gb300 import Context, HMatrix
    from inputs import synth as S
    orbs = S.orbital_set(6, 3)
    case = hydrogenic_case(nmax=6, lmax=3, z=10.0)
    occ = lambda d: S.occupation(orbs, d)  # noqa: E731
    refs = [occ({(1, -1): 2, (2, -1): 2}), occ({(1, -1): 2, (2, 1): 2}), occ({(1, -1): 2, (2, -2): 2})]
    blk = S.ci_block(orbs, refs, [0] * len(orbs), two_j=2, parity=0, density=0.05, seed=9)
    assert blk.ncf > 2000
    ctx = Context(0)
    ctx.set_grid(case["n"], case["rnt"], case["h"], case["c"], case["zz"])
    ob = case["orb"]
    ctx.set_orbitals(ob.nak, ob.mf, ob.pf, ob.qf)
    ctx.genintrk()
    ctx.iabint_table()
    H = HMatrix(ctx, blk.ncf, blk.iendc, blk.irow)
    H.setham(blk.iq, blk.tlist, blk.vlists)
    emt = H.emt()
    nvec = 4
    for robust in (False, True):
        ev0, vec0, info0 = oracle.maneig(0, blk.ncf, nvec, blk.iendc, blk.irow, emt, nthreads=8, robust=robust)
        for precision in (0, 1):
            ev, vec, info = H.maneig(nvec, flavour=0, precision=precision, robust=robust)
            assert info0["ierr"] == 0 and info["ierr"] == 0
            assert np.abs(ev - ev0).max() <= 1e-9, (robust, precision, ev, ev0)
            assert np.abs(vec - vec0).max() <= 1e-7, (robust, precision, np.abs(vec - vec0).max())
    # block passes (DVDSON's MBLOCK = NVEC): fewer, wider passes converge to
    # the same eigenpairs as the reference's single-vector run
    for precision in (0, 1):
        ev, vec, info = H.maneig(nvec, flavour=0, precision=precision, mblock=nvec)
        assert info["ierr"] == 0
        assert np.abs(ev - ev0).max() <= 1e-9, (precision, ev, ev0)
        assert np.abs(vec - vec0).max() <= 1e-7, (precision, np.abs(vec - vec0).max())


def test_maneig_repeated_solves_bit_identical(gpu_ready):
    """Repeated solves of one matrix (the second one replays the CUDA graphs
    and workspaces kept with the matrix) give bit-identical eigenpairs and
    loop counts, for single-vector and block passes in both precisions: all
    reductions have a fixed order."""
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
    for precision in (0, 1):
        for mblock in (1, 4):
            ev0, vec0, info0 = H.maneig(4, flavour=0, precision=precision, mblock=mblock, robust=True)
            ev, vec, info = H.maneig(4, flavour=0, precision=precision, mblock=mblock, robust=True)
            assert info["nloops"] == info0["nloops"]
            assert np.array_equal(ev, ev0), (ev, ev0)
            assert np.array_equal(vec, vec0)


@pytest.mark.parametrize("flavour", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_maneig_tiny_blocks(gpu_ready, oracle_mod, flavour, precision):
    """Blocks of 1, 2 and 5 CSFs with NVEC = NCF: the trivial NCF = 1 case
    (rci90/maneig.f90:122-137) and Davidson in the full unit basis, for both
    MANEIG flavours and both matvec precisions, against the oracle's MANEIG."""
    import oracle
    from grasp_gb300 import Context
    from inputs import workloads as W
    ctx = Context(0)
    for c in (1, 2, 5):
        w = W.batch(zs=(10,), two_js=(0,), parities=(0,), max_ncf=c)
        (H,) = W.assemble_batch(w, ctx)
        b = w.blocks[0][2]
        assert b.ncf == c
        ev, vec, info = H.maneig(c, flavour=flavour, precision=precision)
        ev0, vec0, _ = oracle.maneig(flavour, b.ncf, c, b.iendc, b.irow, H.emt())
        assert info["ierr"] == 0
        assert np.abs(ev - ev0).max() <= 1e-9, (c, ev, ev0)
        assert np.abs(vec - vec0).max() <= 1e-7, c


def test_rmcdhf_warm_start(gpu_ready, oracle_mod):
    """rmcdhf's repeated MANEIG (rmcdhf90/maneig.f90:116-128): after the
    first solve of an SCF step, the next one starts from the previous
    eigenvectors instead of INIEST2. On the 43,493-CSF Fe XV block (above
    N1000 = 4000), flavour 1, both matvec precisions, cold and warm: all
    against the oracle's eigenpairs (its MANEIG with rci's settings, which
    converges to the same pairs with a 2000-row dense start instead of a
    4000-row one), and the warm solve of a slightly changed matrix (a
    perturbed diagonal, as after an orbital update) needs fewer loops than
    its cold solve. All solves use the robust first shift."""
    import os

    from grasp_gb300 import Context, HMatrix
    from inputs import workloads as W
    w = W.fe15()
    b = w.block
    ctx = Context(0)
    ctx.set_grid(w.n, w.rnt, w.h, w.c, w.zz)
    ctx.set_orbitals(w.orb.nak, w.orb.mf, w.orb.pf, w.orb.qf)
    ctx.genintrk()
    ctx.iabint_table()
    H = HMatrix(ctx, b.ncf, b.iendc, b.irow)
    H.setham(b.iq, b.tlist, b.vlists)
    emt = H.emt()
    ncf, nvec, nth = b.ncf, 3, os.cpu_count() or 1
    ev0, vec0, _ = oracle_mod.maneig(0, ncf, nvec, b.iendc, b.irow, emt, nthreads=nth, robust=True)
    # the next SCF step: the diagonal moves by up to 1e-4 Eh
    emt2 = emt.copy()
    emt2[b.iendc[1:] - 1] += 1e-4 * np.sin(np.arange(ncf))
    ev1, vec1, _ = oracle_mod.maneig(0, ncf, nvec, b.iendc, b.irow, emt2, nthreads=nth, robust=True)
    for precision in (0, 1):
        H.set_emt(emt)
        ev, vec, info = H.maneig(nvec, flavour=1, precision=precision, robust=True)
        assert np.abs(ev - ev0).max() <= 1e-9 and np.abs(vec - vec0).max() <= 1e-7
        evw, vecw, infow = H.maneig(nvec, flavour=1, precision=precision, start=vec, robust=True)
        assert np.abs(evw - ev0).max() <= 1e-9 and np.abs(vecw - vec0).max() <= 1e-7
        H.set_emt(emt2)
        evc, vecc, infoc = H.maneig(nvec, flavour=1, precision=precision, robust=True)
        evw, vecw, infow = H.maneig(nvec, flavour=1, precision=precision, start=vec, robust=True)
        for e, v in ((evc, vecc), (evw, vecw)):
            assert np.abs(e - ev1).max() <= 1e-9 and np.abs(v - vec1).max() <= 1e-7, precision
        assert infow["nloops"] < infoc["nloops"], (precision, infow, infoc)
