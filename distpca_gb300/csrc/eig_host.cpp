// The Rayleigh-Ritz eigenproblem on the host: the k x k symmetric matrix B = Q^T Z (k <= 128)
// -> eigenvalues in descending order and their eigenvectors, the result of the reference's
// LAPACKE_dsyev('V', 'U') followed by its column reversal (methods.cpp:981-1000).
//
// Why the host: the problem is tiny (k^3 ~ 1e5 flops) and sequential, and this GPU's FP64
// rate on the one SM such a solve can use is a few flops per cycle, so a device Jacobi solve of
// k = 40 took ~1.3 ms; a CPU core does it in tens of microseconds.  The matrix comes over with
// one stream synchronisation per outer iteration.
//
// Method (as dsyev): Householder reduction to tridiagonal form with the orthogonal factor
// accumulated, then the implicit symmetric QR algorithm with Wilkinson shifts (Golub & Van Loan,
// Matrix Computations, 4th ed., Algorithms 8.3.1 and 8.3.3), eigenvectors accumulated from the
// Givens rotations.  Backward stable; eigenvector signs are those the iteration produces (the
// solve's outputs are defined up to column sign, as the reference's are across LAPACK builds).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "dpca_internal.h"

namespace dpca {

dpca_status host_sym_eig_desc(int k, const double *B, double *w, double *W) {
    if (k <= 0 || !B || !w || !W) {
        set_error("sym_eig: bad arguments");
        return DPCA_ERR_INVALID;
    }
    const int n = k;
    std::vector<double> A((size_t)n * n), Q((size_t)n * n, 0.0), v(n), p(n), wv(n), d(n), e(std::max(n - 1, 1), 0.0);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) A[(size_t)i * n + j] = i <= j ? B[(size_t)i * n + j] : B[(size_t)j * n + i];
    for (int i = 0; i < n; ++i) Q[(size_t)i * n + i] = 1.0;

    // ---- Householder tridiagonalization: A <- H A H column by column, Q <- Q H
    for (int j = 0; j + 2 < n; ++j) {
        const int m = n - j - 1;  // length of x = A[j+1:, j]
        double xn2 = 0.0;
        for (int t = 0; t < m; ++t) xn2 += A[(size_t)(j + 1 + t) * n + j] * A[(size_t)(j + 1 + t) * n + j];
        const double x0 = A[(size_t)(j + 1) * n + j];
        const double tail2 = xn2 - x0 * x0;
        if (tail2 <= 0.0) continue;  // already tridiagonal in this column
        const double alpha = -std::copysign(std::sqrt(xn2), x0);
        for (int t = 0; t < m; ++t) v[t] = A[(size_t)(j + 1 + t) * n + j];
        v[0] -= alpha;
        double vn2 = 0.0;
        for (int t = 0; t < m; ++t) vn2 += v[t] * v[t];
        const double beta = 2.0 / vn2;
        // p = beta * A22 v, w = p - (beta/2)(p.v) v, A22 -= v w^T + w v^T
        double pv = 0.0;
        for (int r = 0; r < m; ++r) {
            double s = 0.0;
            for (int c = 0; c < m; ++c) s += A[(size_t)(j + 1 + r) * n + (j + 1 + c)] * v[c];
            p[r] = beta * s;
            pv += p[r] * v[r];
        }
        const double K = 0.5 * beta * pv;
        for (int r = 0; r < m; ++r) wv[r] = p[r] - K * v[r];
        for (int r = 0; r < m; ++r)
            for (int c = 0; c < m; ++c) A[(size_t)(j + 1 + r) * n + (j + 1 + c)] -= v[r] * wv[c] + wv[r] * v[c];
        A[(size_t)(j + 1) * n + j] = A[(size_t)j * n + (j + 1)] = alpha;
        for (int t = 1; t < m; ++t) A[(size_t)(j + 1 + t) * n + j] = A[(size_t)j * n + (j + 1 + t)] = 0.0;
        // Q[:, j+1:] -= beta (Q[:, j+1:] v) v^T
        for (int r = 0; r < n; ++r) {
            double s = 0.0;
            for (int c = 0; c < m; ++c) s += Q[(size_t)r * n + (j + 1 + c)] * v[c];
            s *= beta;
            for (int c = 0; c < m; ++c) Q[(size_t)r * n + (j + 1 + c)] -= s * v[c];
        }
    }
    for (int i = 0; i < n; ++i) d[i] = A[(size_t)i * n + i];
    for (int i = 0; i + 1 < n; ++i) e[i] = A[(size_t)i * n + i + 1];

    // ---- implicit symmetric QR steps with the Wilkinson shift on the unreduced blocks
    const double eps = std::ldexp(1.0, -52);
    int hi = n - 1, iters = 0;
    while (hi > 0) {
        // deflate negligible off-diagonals
        for (int i = 0; i < hi; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        if (e[hi - 1] == 0.0) {
            --hi;
            continue;
        }
        int lo = hi - 1;
        while (lo > 0 && e[lo - 1] != 0.0) --lo;
        if (++iters > 60 * n) {
            set_error("sym_eig: QR iteration did not converge");
            return DPCA_ERR_NUMERIC;
        }
        // Wilkinson shift: the eigenvalue of the trailing 2 x 2 closer to d[hi]
        const double a = d[hi - 1], b = e[hi - 1], c = d[hi];
        const double delta = 0.5 * (a - c);
        const double denom = delta + std::copysign(std::hypot(delta, b), delta == 0.0 ? 1.0 : delta);
        const double mu = c - b * b / denom;
        double x = d[lo] - mu, z = e[lo];
        for (int t = lo; t < hi; ++t) {
            // rotation G on (t, t+1) with G^T [x; z] = [r; 0]
            const double r = std::hypot(x, z);
            const double cs = r == 0.0 ? 1.0 : x / r, sn = r == 0.0 ? 0.0 : z / r;
            if (t > lo) e[t - 1] = r;
            const double dt = d[t], dt1 = d[t + 1], et = e[t];
            d[t] = cs * cs * dt + 2.0 * cs * sn * et + sn * sn * dt1;
            d[t + 1] = sn * sn * dt - 2.0 * cs * sn * et + cs * cs * dt1;
            e[t] = cs * sn * (dt1 - dt) + (cs * cs - sn * sn) * et;
            if (t + 1 < hi) {
                x = e[t];
                z = sn * e[t + 1];  // the bulge at (t, t+2)
                e[t + 1] *= cs;
            }
            for (int i = 0; i < n; ++i) {
                const double qt = Q[(size_t)i * n + t], qt1 = Q[(size_t)i * n + t + 1];
                Q[(size_t)i * n + t] = cs * qt + sn * qt1;
                Q[(size_t)i * n + t + 1] = -sn * qt + cs * qt1;
            }
        }
    }

    // ---- descending order (ties keep index order)
    std::vector<int> ord(n);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return d[a] > d[b]; });
    for (int c = 0; c < n; ++c) {
        w[c] = d[ord[c]];
        for (int i = 0; i < n; ++i) W[(size_t)i * n + c] = Q[(size_t)i * n + ord[c]];
    }
    return DPCA_OK;
}

// R^-1 of the Cholesky factor of G (+ shift I), both k x k row-major (upper triangle of R^-1,
// zeros below): one step of the shifted CholeskyQR3 (k_dense.cu launch_qr).  The shift
// 11 (n k + k (k + 1)) u trace(G) is applied when `shift` is set or when a plain factorization
// meets a non-positive pivot; a pivot that still fails is replaced by 1 (a zero or non-finite
// column stays unnormalised instead of dividing by zero).
void host_chol_inv(int k, int n, const double *G, bool shift, double *Rinv) {
    std::vector<double> R((size_t)k * k);
    double tr = 0.0;
    for (int i = 0; i < k; ++i) tr += G[(size_t)i * k + i];
    const double s = 11.0 * ((double)n * k + (double)k * (k + 1)) * std::ldexp(1.0, -53) * tr;
    for (int attempt = shift ? 1 : 0; attempt < 2; ++attempt) {
        bool broke = false;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) R[(size_t)i * k + j] = G[(size_t)i * k + j] + (attempt == 1 && i == j ? s : 0.0);
        for (int j = 0; j < k && !broke; ++j) {
            double d = R[(size_t)j * k + j];
            if (!(d > 0.0) || !std::isfinite(d)) {
                if (attempt == 0) {
                    broke = true;
                    break;
                }
                d = 1.0;
            }
            const double r = std::sqrt(d), inv = 1.0 / r;
            R[(size_t)j * k + j] = r;
            for (int c = j + 1; c < k; ++c) R[(size_t)j * k + c] *= inv;
            for (int a = j + 1; a < k; ++a) {
                const double rja = R[(size_t)j * k + a];
                for (int c = a; c < k; ++c) R[(size_t)a * k + c] -= rja * R[(size_t)j * k + c];
            }
        }
        if (!broke) break;
    }
    // R^-1 by back substitution, column by column
    for (int i = 0; i < k * k; ++i) Rinv[i] = 0.0;
    for (int c = 0; c < k; ++c) {
        Rinv[(size_t)c * k + c] = 1.0 / R[(size_t)c * k + c];
        for (int i = c - 1; i >= 0; --i) {
            double sum = 0.0;
            for (int l = i + 1; l <= c; ++l) sum += R[(size_t)i * k + l] * Rinv[(size_t)l * k + c];
            Rinv[(size_t)i * k + c] = -sum / R[(size_t)i * k + i];
        }
    }
}

}  // namespace dpca

extern "C" dpca_status dpca_sym_eig(int k, const double *b, double *w, double *W) {
    dpca::clear_error();
    return dpca::host_sym_eig_desc(k, b, w, W);
}
