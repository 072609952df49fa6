"""The host eigensolver of the Davidson iteration (DVDSON's DSPEVX call,
libdvd90/dvdson.f90:724) through the C ABI, against numpy's dense solver.
No GPU: it runs on the host by design.

Bar: eigenvalues within 1e-12 of the spectral norm; eigenvectors with
residual |S z - w z| within 1e-11 of the norm and orthonormal within 1e-12
(eigenvectors of (near-)degenerate eigenvalues are compared as a subspace)."""
import numpy as np
import pytest


def _lib_or_skip():
    from grasp_gb300 import _lib
    try:
        _lib.gpu()
    except (OSError, RuntimeError) as e:  # the library needs the CUDA runtime to load
        pytest.skip(f"libgraspgpu not loadable here: {e}")


def _davidson_like(n, seed):
    """A projected matrix of the shape the iteration sees after a restart:
    a diagonal leading block (Ritz values) bordered by the new columns."""
    rng = np.random.default_rng(seed)
    s = np.diag(-80.0 + np.sort(rng.uniform(0, 2.0, n)))
    r = n // 2
    b = rng.normal(scale=0.05, size=(n, n - r))
    s[:, r:] += b
    s[r:, :] += b.T
    return (s + s.T) / 2


@pytest.mark.parametrize("n,m,mvec,seed", [(1, 1, 1, 0), (2, 2, 1, 1), (11, 11, 10, 2), (40, 11, 10, 3),
                                           (80, 11, 10, 4), (80, 40, 40, 5), (200, 17, 16, 6)])
def test_projected_eig_matches_dense(n, m, mvec, seed):
    _lib_or_skip()
    from grasp_gb300.core import projected_eig
    s = _davidson_like(n, seed)
    w, z = projected_eig(s, m, mvec)
    w0, z0 = np.linalg.eigh(s)
    norm = np.abs(w0).max()
    assert np.abs(w - w0[:m]).max() <= 1e-12 * norm
    assert np.abs(s @ z - z * w[:mvec]).max() <= 1e-11 * norm
    assert np.abs(z.T @ z - np.eye(mvec)).max() <= 1e-12


def test_projected_eig_degenerate_cluster():
    """Exactly repeated eigenvalues (a rotated diagonal matrix with a triple
    eigenvalue): the vectors span the eigenspace and stay orthonormal."""
    _lib_or_skip()
    from grasp_gb300.core import projected_eig
    rng = np.random.default_rng(7)
    d = np.array([-3.0, -2.0, -2.0, -2.0, -1.0] + list(np.linspace(0, 5, 25)))
    q, _ = np.linalg.qr(rng.normal(size=(30, 30)))
    s = (q * d) @ q.T
    s = (s + s.T) / 2
    w, z = projected_eig(s, 6, 5)
    assert np.abs(w - np.sort(d)[:6]).max() <= 1e-12 * 5
    assert np.abs(z.T @ z - np.eye(5)).max() <= 1e-12
    assert np.abs(s @ z - z * w[:5]).max() <= 1e-11 * 5


def test_projected_eig_rejects_bad_sizes():
    _lib_or_skip()
    from grasp_gb300 import GGError
    from grasp_gb300.core import projected_eig
    with pytest.raises(GGError):
        projected_eig(np.eye(3), 4)
    with pytest.raises(GGError):
        projected_eig(np.eye(3), 2, 3)


@pytest.mark.parametrize("n,seed", [(12, 8), (41, 9)])
def test_projected_eig_trivial_reflectors(n, seed):
    """Columns that are already reduced (zero below the subdiagonal), so some
    Householder steps have nothing to do: a block-diagonal matrix with
    diagonal and tridiagonal blocks."""
    _lib_or_skip()
    from grasp_gb300.core import projected_eig
    rng = np.random.default_rng(seed)
    s = np.zeros((n, n))
    h = n // 3
    a = rng.normal(size=(h, h))
    s[:h, :h] = a + a.T
    s[h:2 * h, h:2 * h] = np.diag(rng.normal(size=h))
    t = 2 * h
    d = rng.normal(size=n - t)
    e = rng.normal(size=n - t - 1)
    s[t:, t:] = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    w, z = projected_eig(s, n // 2, n // 2 - 1)
    w0 = np.linalg.eigvalsh(s)
    norm = np.abs(w0).max()
    assert np.abs(w - w0[:n // 2]).max() <= 1e-12 * norm
    assert np.abs(s @ z - z * w[:n // 2 - 1]).max() <= 1e-11 * norm
    assert np.abs(z.T @ z - np.eye(n // 2 - 1)).max() <= 1e-12
