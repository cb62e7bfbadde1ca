// The k x k symmetric eigenproblem on the host: B (k <= 128, upper triangle used) -> eigenvalues
// in descending order and their eigenvectors, the result of LAPACKE_dsyev('V', 'U') followed by
// the reference's column reversal (methods.cpp:981-1000).  This is dpca_sym_eig, a host-side
// utility of the C ABI (the solve itself runs its Rayleigh-Ritz step on the device, k_dense.cu).
//
// Method (as dsyev): Householder reduction to tridiagonal form with the orthogonal factor
// accumulated, then the implicit symmetric QR algorithm with Wilkinson shifts (Golub & Van Loan,
// Matrix Computations, 4th ed., Algorithms 8.3.1 and 8.3.3), eigenvectors accumulated from the
// Givens rotations.  Backward stable; eigenvector signs are those the iteration produces.
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

}  // namespace dpca

extern "C" dpca_status dpca_sym_eig(int k, const double *b, double *w, double *W) {
    dpca::clear_error();
    return dpca::host_sym_eig_desc(k, b, w, W);
}
