"""The device thin QR of a solve's n x k panels (dpca_qr_device) against LAPACK's QR.

The reference orthonormalizes each panel with dgeqrf + dorgqr (methods.cpp:947-961); the device
runs shifted CholeskyQR3, with the k x k factor and inverse in double-float arithmetic up to k = 48
and in FP64 above (48 and 49 are the boundary).  Q is defined up to the signs of its columns, so the
checks are: Q^T Q = I; A = Q R with R = Q^T A upper triangular (Q's first j columns span A's first
j); for well-conditioned panels, |Q_lapack^T Q| = I (the same columns up to sign); and one
cooperative launch and the separate kernels give the same bits.  Tolerances: 5e-12 for
orthonormality, the residual and R's lower triangle (relative to max |A|), 1e-9 for the
comparison with LAPACK.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(5, 1), (64, 8), (1000, 20), (2813, 10), (20000, 40), (4096, 47), (3000, 48), (3000, 49),
          (10000, 64), (2000, 128)]


def check_q(a, q, well_conditioned):
    k = a.shape[1]
    scale = np.abs(a).max()
    assert np.abs(q.T @ q - np.eye(k)).max() < 5e-12
    r = q.T @ a
    assert np.abs(np.tril(r, -1)).max() <= 5e-12 * scale
    assert np.abs(a - q @ np.triu(r)).max() <= 5e-12 * scale
    if well_conditioned:
        ql, _ = np.linalg.qr(a)
        c = ql.T @ q
        np.testing.assert_allclose(np.abs(c), np.eye(k), atol=1e-9)


@pytest.mark.parametrize("n,k", SHAPES)
def test_qr_matches_lapack(dpca, n, k):
    rng = np.random.default_rng(n + 7 * k)
    a = rng.standard_normal((n, k)) * 3.0 + 1.0
    q = dpca.qr_device(a)
    check_q(a, q, True)
    assert np.array_equal(q, dpca.qr_device(a, separate=True))


@pytest.mark.parametrize("n,k", [(1000, 20), (5000, 40), (3000, 48), (3000, 49)])
def test_qr_ill_conditioned(dpca, n, k):
    """Columns mixed across eight orders of magnitude (condition ~1e8): the shifted first step
    keeps the factorization defined and the two plain steps restore orthonormality."""
    rng = np.random.default_rng(k)
    u, _ = np.linalg.qr(rng.standard_normal((n, k)))
    v, _ = np.linalg.qr(rng.standard_normal((k, k)))
    a = (u * np.logspace(0, -8, k)) @ v.T
    q = dpca.qr_device(a)
    check_q(a, q, False)
    assert np.array_equal(q, dpca.qr_device(a, separate=True))


def test_qr_rank_deficient_panel(dpca):
    """A column that is an exact combination of earlier ones (a full-width block of a cohort with
    fewer directions than columns): the independent columns still come out orthonormal and exact,
    and the dependent one finite and orthogonal to them."""
    rng = np.random.default_rng(11)
    n, k = 2000, 24
    a = rng.standard_normal((n, k))
    a[:, 13] = a[:, 2] - 0.5 * a[:, 7]  # column 13 depends on columns 2 and 7
    q = dpca.qr_device(a)
    assert np.all(np.isfinite(q))
    good = [c for c in range(k) if c != 13]
    qg = q[:, good]
    assert np.abs(qg.T @ qg - np.eye(k - 1)).max() < 5e-12
    # the first 13 columns span exactly a's first 13
    ql, _ = np.linalg.qr(a[:, :13])
    np.testing.assert_allclose(np.abs(ql.T @ q[:, :13]), np.eye(13), atol=1e-9)
    assert np.abs(qg.T @ q[:, 13]).max() < 1e-6 * max(1.0, np.linalg.norm(q[:, 13]))
    assert np.array_equal(q, dpca.qr_device(a, separate=True))


def test_qr_scale_invariant(dpca):
    """The k x k factor runs on the Gram scaled by a power of two: panels of 1e-150 and 1e150 give
    Q as for the unit panel."""
    rng = np.random.default_rng(5)
    a = rng.standard_normal((3000, 24))
    q = dpca.qr_device(a)
    for s in (1e-150, 1e150):
        np.testing.assert_allclose(dpca.qr_device(a * s), q, atol=1e-12)


def test_qr_rejects_bad_arguments(dpca):
    assert dpca.lib().dpca_qr_device(0, 10, 0, None, 0) != 0  # k = 0
    assert dpca.lib().dpca_qr_device(0, 0, 4, None, 0) != 0  # n = 0, no array
