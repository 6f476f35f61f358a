"""Infinite-screen extrusion matrices (science/infScrn.py:549-746) on the host."""
import numpy as np

from dasp_gb300.infscreen import extrusion_matrices, new_column_host, phase_covariance


def test_covariance_structure():
    c = phase_covariance(16, 25.0, 0.05)
    assert c.shape == (48, 48)
    np.testing.assert_allclose(c, c.T)
    d = np.diag(c)
    assert np.allclose(d, d[0]) and d[0] > 0
    # covariance falls with distance: neighbours below the variance
    assert c[0, 1] < d[0] and c[0, 16] < d[0] and c[0, 1] > c[0, 2]
    np.linalg.cholesky(c[:32, :32])  # positive definite


def test_extrusion_matrices_reproduce_the_covariance():
    n = 12
    c = phase_covariance(n, 25.0, 0.05)
    a, b = extrusion_matrices(n, c)
    assert a.shape == (n, 2 * n) and b.shape == (n, n)
    zz, xz, xx = c[:2 * n, :2 * n], c[2 * n:, :2 * n], c[2 * n:, 2 * n:]
    # X = A Z + B n has <XZ^T> = A <ZZ^T> and <XX^T> = A<ZZ^T>A^T + B B^T
    np.testing.assert_allclose(a @ zz, xz, rtol=1e-6, atol=1e-9 * np.abs(xz).max())
    np.testing.assert_allclose(a @ zz @ a.T + b @ b.T, xx, rtol=1e-6, atol=1e-9 * np.abs(xx).max())


def test_new_column_host_orders_older_column_first():
    n = 4
    a = np.zeros((n, 2 * n))
    a[:, :n] = np.eye(n)  # copies the older column
    b = np.eye(n)
    cols = np.stack([np.arange(n), 10 + np.arange(n)], axis=1).astype(np.float32)
    out = new_column_host(cols, a, b, np.ones(n), 2.0, 0.5)
    np.testing.assert_allclose(out, np.arange(n) + 2.0 + 0.5)
