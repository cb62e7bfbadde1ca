"""The device k x k eigensolver of the Rayleigh-Ritz step (dpca_sym_eig_device) against LAPACK.

Every outer iteration of a solve diagonalizes the k x k matrix B = Q^T Z on the device (parallel
cyclic Jacobi, methods.cpp:981-1000 in the reference): in double-float arithmetic up to k = 48,
in FP64 above (k = 48 and 49 are the boundary).  The cases are those of the host
eigensolver's test: indefinite, positive semi-definite (like B), clustered and repeated
eigenvalues, already diagonal, zero, and a nearly diagonal matrix (B from the second iteration
on).  Tolerances as there: eigenvalues within 1e-12 of the largest, eigenvectors orthonormal and
A W = W diag(w) to 1e-12, eigenvalues in descending order.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def cases(k, rng):
    out = []
    g = rng.standard_normal((k, k))
    out.append(g + g.T)
    x = rng.standard_normal((3 * k + 5, k)) * np.logspace(0, -5, k)
    out.append(x.T @ x)
    q, _ = np.linalg.qr(rng.standard_normal((k, k)))
    lam = np.repeat(rng.standard_normal(k // 3 + 1), 3)[:k]
    out.append((q * lam) @ q.T)
    out.append(np.diag(rng.standard_normal(k)))
    out.append(np.zeros((k, k)))
    d = np.diag(np.sort(rng.uniform(1, 100, k))[::-1])
    e = 1e-7 * rng.standard_normal((k, k))
    out.append(d + e + e.T)
    return out


@pytest.mark.parametrize("k", [1, 2, 3, 8, 20, 40, 41, 47, 48, 49, 97, 112, 113, 128])
def test_device_eig_matches_lapack(dpca, k):
    rng = np.random.default_rng(100 + k)
    for a in cases(k, rng):
        upper = np.triu(a) + np.tril(rng.standard_normal((k, k)), -1) * 1e3  # the lower triangle is ignored
        w, W = dpca.sym_eig(upper, device=0)
        ref = np.linalg.eigvalsh(a)[::-1]
        scale = max(1.0, np.abs(ref).max())
        assert np.all(np.diff(w) <= 0)
        np.testing.assert_allclose(w, ref, atol=1e-12 * scale, rtol=0)
        np.testing.assert_allclose(W.T @ W, np.eye(k), atol=1e-12)
        assert np.abs(a @ W - W * w).max() <= 1e-12 * scale


def test_device_eig_is_deterministic(dpca):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((200, 40))
    b = x.T @ x
    w1, W1 = dpca.sym_eig(b, device=0)
    w2, W2 = dpca.sym_eig(b, device=0)
    assert np.array_equal(w1, w2) and np.array_equal(W1, W2)
