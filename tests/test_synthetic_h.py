"""The seeded synthetic Hamiltonian of the large-scale workload
(gs_synthetic_h via workloads.synthetic_h): GRASP's lower-triangle-by-rows
storage rules (IENDC(0) = 0, each row's columns ascending and below the row,
the diagonal last, 1-based IROW), the requested density, the value model,
and determinism (the same seed gives the same block; rows draw from their
own streams, so the thread count does not matter). No GPU."""
import numpy as np


def test_synthetic_h_structure_and_values():
    from inputs import workloads as W
    ncf, nnz = 5000, 400_000
    iendc, irow, emt = W.synthetic_h(ncf, nnz, seed=3)
    assert iendc[0] == 0 and iendc.size == ncf + 1 and np.all(np.diff(iendc) >= 1)
    assert irow.size == emt.size == iendc[-1]
    assert abs(iendc[-1] - nnz) < 0.01 * nnz
    rows = np.repeat(np.arange(ncf), np.diff(iendc))
    diag = iendc[1:] - 1
    assert np.array_equal(irow[diag], np.arange(1, ncf + 1))          # the diagonal last
    off = np.ones(irow.size, bool)
    off[diag] = False
    assert np.all(irow[off] >= 1) and np.all(irow[off] <= rows[off])  # below the diagonal (1-based)
    same = rows[1:] == rows[:-1]
    assert np.all(irow[1:][same] > irow[:-1][same])                  # ascending within a row
    d = emt[diag]
    assert np.all(np.abs(d - (-1000.0 + 30.0 * np.sqrt(np.arange(ncf) / ncf))) < 1e-2)
    o = emt[off]
    assert abs(o.mean()) < 1e-4 and abs(o.std() - 2e-3) < 1e-4


def test_synthetic_h_deterministic():
    from inputs import workloads as W
    a = W.synthetic_h(3000, 100_000, seed=11)
    b = W.synthetic_h(3000, 100_000, seed=11)
    c = W.synthetic_h(3000, 100_000, seed=12)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert not np.array_equal(a[1], c[1])
