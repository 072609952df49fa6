"""GPU parity on blocks larger than 65,536 CSFs (32-bit matvec columns, the
large-scale workload's layout) with the seeded synthetic H of
workloads.synthetic_h, against the oracle's MANEIG (INIEST2 + DVDSON), and
split against FP64. Bar: eigenvalues within 1e-9 Eh, eigenvectors within
1e-7 after the sign convention."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_large_block_matches_oracle(gpu_ready, oracle_mod):
    import oracle
    from grasp_gb300 import FP64, SPLIT, Context, HMatrix
    from inputs import workloads as W
    ncf, nvec = 70000, 5
    iendc, irow, emt = W.synthetic_h(ncf, 3.0e6, seed=5)
    ctx = Context(0)
    H = HMatrix(ctx, ncf, iendc, irow)
    H.set_emt(emt)
    ev0, vec0, info0 = oracle.maneig(0, ncf, nvec, iendc, irow, emt, nthreads=8, robust=True)
    assert info0["ierr"] == 0
    for precision, mblock in ((FP64, 0), (SPLIT, 0), (SPLIT, nvec)):
        ev, vec, info = H.maneig(nvec, flavour=0, precision=precision, robust=True, mblock=mblock)
        assert info["ierr"] == 0
        assert np.abs(ev - ev0).max() <= 1e-9, (precision, mblock, ev, ev0)
        assert np.abs(vec - vec0).max() <= 1e-7, (precision, mblock, np.abs(vec - vec0).max())
    # the block matvec on this layout against the oracle's SPICMV2
    b = np.random.default_rng(3).normal(size=(ncf, 4))
    c0 = oracle.spicmv2(ncf, iendc, irow, emt, b)
    c1 = H.spicmv2(b, precision=SPLIT)
    assert np.abs(c1 - c0).max() <= 1e-11 * np.abs(c0).max()
