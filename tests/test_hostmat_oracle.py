"""The oracle's SPODMV (rci90/spodmv.f90:65-80) and DNICMV
(rci90/dnicmv.f90:52-64) restatements: SPODMV is SPICMV2's product with the
diagonal shifted by EAV as it is read (the same operations, so the same
bits as SPICMV2 on the shifted rows); DNICMV is SPICMV2's product on the
dense packed triangle (its dot product and its update loop touch each sum in
the same order as DMERGE's fused loop)."""
import numpy as np

import oracle


def _rows(n, seed):
    rng = np.random.default_rng(seed)
    iendc = [0]
    irow = []
    for r in range(1, n + 1):
        cols = sorted(rng.choice(np.arange(1, r), size=min(r - 1, rng.integers(0, 6)), replace=False)) if r > 1 else []
        irow += [int(c) for c in cols] + [r]
        iendc.append(len(irow))
    iendc = np.array(iendc, np.int64)
    irow = np.array(irow, np.int32)
    emt = rng.standard_normal(irow.size)
    return iendc, irow, emt


def test_spodmv_is_spicmv2_with_shifted_diagonal(oracle_mod):
    n, eav = 200, 3.25
    iendc, irow, raw = _rows(n, 1)
    b = np.random.default_rng(2).standard_normal((n, 3))
    c = oracle.spodmv(n, iendc, irow, raw, eav, b)
    emt = raw.copy()
    emt[iendc[1:] - 1] = raw[iendc[1:] - 1] - eav
    np.testing.assert_array_equal(c, oracle.spicmv2(n, iendc, irow, emt, b))
    a = np.zeros((n, n))
    for i in range(n):
        for p in range(iendc[i], iendc[i + 1]):
            a[i, irow[p] - 1] = a[irow[p] - 1, i] = emt[p]
    assert np.abs(c - a @ b).max() <= 1e-13 * np.abs(c).max()


def test_dnicmv_is_spicmv2_on_the_dense_triangle(oracle_mod):
    n = 120
    rng = np.random.default_rng(3)
    a = rng.standard_normal((n, n))
    a = a + a.T
    ap = np.concatenate([a[i, :i + 1] for i in range(n)])
    b = rng.standard_normal((n, 2))
    c = oracle.dnicmv(n, ap, b)
    iendc = np.concatenate([[0], np.cumsum(np.arange(1, n + 1))]).astype(np.int64)
    irow = np.concatenate([np.arange(1, i + 2) for i in range(n)]).astype(np.int32)
    np.testing.assert_array_equal(c, oracle.spicmv2(n, iendc, irow, ap, b))
    assert np.abs(c - a @ b).max() <= 1e-12 * np.abs(c).max()
