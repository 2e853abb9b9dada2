// Dense symmetric eigen-decomposition for the small projected matrices of
// the Lanczos solver (m up to a few hundred), in FP64 on the host:
// Householder reduction to tridiagonal form followed by the implicit
// symmetric QR iteration with Wilkinson shifts (Golub & Van Loan, "Matrix
// Computations", sections 8.3.1-8.3.3), eigenvectors accumulated.
// Stands in for the Hessenberg/Schur work ARPACK performs inside
// pdneupd_ (utilities/wrappers/arpack_wrapper.hpp:880).
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "ed_internal.h"

namespace edgb {

void sym_eigen(int m, const std::vector<double>& a_in, std::vector<double>& evals, std::vector<double>& evecs)
{
    ED_REQUIRE(m >= 1 && (int64_t)a_in.size() >= (int64_t)m * m, ED_ERR_ARG, "sym_eigen: bad size");
    std::vector<double> A(a_in.begin(), a_in.begin() + (size_t)m * m);
    std::vector<double> Q((size_t)m * m, 0.0);   // row-major, Q[i*m+j]
    for (int i = 0; i < m; ++i) Q[(size_t)i * m + i] = 1.0;
    std::vector<double> v(m), p(m), q(m);

    // ---- Householder tridiagonalisation: A <- H A H, Q <- Q H
    for (int k = 0; k + 2 < m; ++k) {
        const int len = m - k - 1;
        double nrm = 0.0;
        for (int i = 0; i < len; ++i) {
            const double x = A[(size_t)(k + 1 + i) * m + k];
            nrm += x * x;
        }
        nrm = std::sqrt(nrm);
        if (nrm == 0.0) continue;
        const double x0 = A[(size_t)(k + 1) * m + k];
        const double alpha = x0 > 0 ? -nrm : nrm;
        for (int i = 0; i < len; ++i) v[i] = A[(size_t)(k + 1 + i) * m + k];
        v[0] -= alpha;
        double vn2 = 0.0;
        for (int i = 0; i < len; ++i) vn2 += v[i] * v[i];
        if (vn2 == 0.0) continue;
        const double beta = 2.0 / vn2;
        // p = beta * A_sub v
        double vp = 0.0;
        for (int i = 0; i < len; ++i) {
            double s = 0.0;
            const double* row = &A[(size_t)(k + 1 + i) * m + (k + 1)];
            for (int j = 0; j < len; ++j) s += row[j] * v[j];
            p[i] = beta * s;
            vp += v[i] * p[i];
        }
        const double Kc = 0.5 * beta * vp;
        for (int i = 0; i < len; ++i) q[i] = p[i] - Kc * v[i];
        for (int i = 0; i < len; ++i) {
            double* row = &A[(size_t)(k + 1 + i) * m + (k + 1)];
            for (int j = 0; j < len; ++j) row[j] -= v[i] * q[j] + q[i] * v[j];
        }
        A[(size_t)(k + 1) * m + k] = alpha;
        A[(size_t)k * m + (k + 1)] = alpha;
        for (int i = 1; i < len; ++i) {
            A[(size_t)(k + 1 + i) * m + k] = 0.0;
            A[(size_t)k * m + (k + 1 + i)] = 0.0;
        }
        for (int r = 0; r < m; ++r) {
            double* row = &Q[(size_t)r * m + (k + 1)];
            double t = 0.0;
            for (int j = 0; j < len; ++j) t += row[j] * v[j];
            t *= beta;
            for (int j = 0; j < len; ++j) row[j] -= t * v[j];
        }
    }
    std::vector<double> d(m), e(m > 1 ? m - 1 : 1, 0.0);
    for (int i = 0; i < m; ++i) d[i] = A[(size_t)i * m + i];
    for (int i = 0; i + 1 < m; ++i) e[i] = A[(size_t)(i + 1) * m + i];

    // ---- implicit symmetric QR with Wilkinson shifts on (d, e)
    const double eps = 2.220446049250313e-16;
    int h = m - 1;
    int64_t guard = 0;
    const int64_t guard_max = 60LL * m + 100;
    while (h > 0) {
        for (int i = 0; i < h; ++i)
            if (std::fabs(e[i]) <= eps * (std::fabs(d[i]) + std::fabs(d[i + 1]))) e[i] = 0.0;
        if (e[h - 1] == 0.0) { --h; continue; }
        int l = h - 1;
        while (l > 0 && e[l - 1] != 0.0) --l;
        ED_REQUIRE(++guard <= guard_max, ED_ERR_INTERNAL, "sym_eigen: QR iteration did not converge");
        const double aa = d[h - 1], bb = e[h - 1], cc = d[h];
        const double delta = 0.5 * (aa - cc);
        const double sg = delta >= 0.0 ? 1.0 : -1.0;
        const double mu = cc - bb * bb / (delta + sg * std::hypot(delta, bb));
        double x = d[l] - mu, z = e[l];
        for (int k = l; k < h; ++k) {
            double r = std::hypot(x, z);
            double c = 1.0, s = 0.0;
            if (r != 0.0) { c = x / r; s = z / r; }
            if (k > l) e[k - 1] = r;
            const double a = d[k], b = e[k], dd = d[k + 1];
            d[k] = a * c * c + 2.0 * b * c * s + dd * s * s;
            d[k + 1] = a * s * s - 2.0 * b * c * s + dd * c * c;
            e[k] = (dd - a) * c * s + b * (c * c - s * s);
            if (k + 1 < h) {
                z = e[k + 1] * s;
                e[k + 1] = e[k + 1] * c;
                x = e[k];
            }
            for (int r2 = 0; r2 < m; ++r2) {
                double* row = &Q[(size_t)r2 * m];
                const double qk = row[k], qk1 = row[k + 1];
                row[k] = c * qk + s * qk1;
                row[k + 1] = -s * qk + c * qk1;
            }
        }
    }
    std::vector<int> order(m);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int i, int j) { return d[i] < d[j]; });
    evals.assign(m, 0.0);
    evecs.assign((size_t)m * m, 0.0);
    for (int j = 0; j < m; ++j) {
        evals[j] = d[order[j]];
        for (int i = 0; i < m; ++i) evecs[(size_t)i + (size_t)m * j] = Q[(size_t)i * m + order[j]];
    }
}

}  // namespace edgb
