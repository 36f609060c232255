// Global Newton-Raphson update: F/2, symmetrise, stable inversion and
// theta = 1/2 F_solver (d - b - t).  Follows core/quadratic_estimate.cpp:456-457,
// :261-288, :290-318 and mathtools/matrix_helper.cpp:220-358 (stableInvertSym).
// The reference decides damping from the singular values of F (dgesvd); F is
// symmetric, so they are the absolute eigenvalues, found here by Householder
// tridiagonalisation and implicit QL.  Inverses use Gauss-Jordan elimination
// with partial pivoting (the reference: LU, dgetrf + dgetri).  O(nkz^3) FP64.
#include "lqg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

struct lqg_ctx;

namespace {

using Mat = std::vector<double>;

// Eigenvalues of a symmetric n x n matrix (row-major), unordered.
bool sym_eigenvalues(Mat a, int n, std::vector<double> &d) {
    std::vector<double> e(n, 0.0);
    d.assign(n, 0.0);
    // Householder reduction to tridiagonal form, column by column
    for (int k = 0; k < n - 2; ++k) {
        double alpha = 0;
        for (int i = k + 1; i < n; ++i) alpha += a[(size_t) i * n + k] * a[(size_t) i * n + k];
        alpha = std::sqrt(alpha);
        if (alpha == 0) continue;
        double x0 = a[(size_t) (k + 1) * n + k];
        if (x0 > 0) alpha = -alpha;
        std::vector<double> u(n, 0.0);
        for (int i = k + 1; i < n; ++i) u[i] = a[(size_t) i * n + k];
        u[k + 1] -= alpha;
        double h = 0;
        for (int i = k + 1; i < n; ++i) h += u[i] * u[i];
        h /= 2;
        if (h == 0) continue;
        std::vector<double> p(n, 0.0);
        for (int i = k; i < n; ++i) {
            double s = 0;
            for (int j = k + 1; j < n; ++j) s += a[(size_t) i * n + j] * u[j];
            p[i] = s / h;
        }
        double kk = 0;
        for (int i = k + 1; i < n; ++i) kk += u[i] * p[i];
        kk /= (2 * h);
        std::vector<double> q(n, 0.0);
        for (int i = k; i < n; ++i) q[i] = p[i] - kk * u[i];
        for (int i = k; i < n; ++i)
            for (int j = k; j < n; ++j)
                a[(size_t) i * n + j] -= q[i] * u[j] + u[i] * q[j];
    }
    for (int i = 0; i < n; ++i) d[i] = a[(size_t) i * n + i];
    for (int i = 0; i + 1 < n; ++i) e[i] = a[(size_t) (i + 1) * n + i];
    e[n - 1] = 0;
    // implicit QL with Wilkinson-type shifts
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        while (true) {
            int m = l;
            for (; m < n - 1; ++m) {
                double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
                if (std::fabs(e[m]) + dd == dd) break;
            }
            if (m == l) break;
            if (++iter > 200) return false;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = std::hypot(g, 1.0);
            g = d[m] - d[l] + e[l] / (g + std::copysign(r, g));
            double s = 1, c = 1, p = 0;
            int i = m - 1;
            bool early = false;
            for (; i >= l; --i) {
                double f = s * e[i], b = c * e[i];
                r = std::hypot(f, g);
                e[i + 1] = r;
                if (r == 0) { d[i + 1] -= p; e[m] = 0; early = true; break; }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
            }
            if (early) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0;
        }
    }
    return true;
}

// Inverse by Gauss-Jordan elimination with partial pivoting; false if singular.
bool invert(Mat a, int n, Mat &inv) {
    inv.assign((size_t) n * n, 0.0);
    for (int i = 0; i < n; ++i) inv[(size_t) i * n + i] = 1.0;
    for (int col = 0; col < n; ++col) {
        int piv = col;
        double best = std::fabs(a[(size_t) col * n + col]);
        for (int r = col + 1; r < n; ++r) {
            double v = std::fabs(a[(size_t) r * n + col]);
            if (v > best) { best = v; piv = r; }
        }
        if (!(best > 0) || !std::isfinite(best)) return false;
        if (piv != col) {
            for (int j = 0; j < n; ++j) {
                std::swap(a[(size_t) piv * n + j], a[(size_t) col * n + j]);
                std::swap(inv[(size_t) piv * n + j], inv[(size_t) col * n + j]);
            }
        }
        double dinv = 1.0 / a[(size_t) col * n + col];
        for (int j = 0; j < n; ++j) { a[(size_t) col * n + j] *= dinv; inv[(size_t) col * n + j] *= dinv; }
        for (int r = 0; r < n; ++r) {
            if (r == col) continue;
            double f = a[(size_t) r * n + col];
            if (f == 0) continue;
            for (int j = 0; j < n; ++j) {
                a[(size_t) r * n + j] -= f * a[(size_t) col * n + j];
                inv[(size_t) r * n + j] -= f * inv[(size_t) col * n + j];
            }
        }
    }
    return true;
}

Mat matmul(const Mat &a, const Mat &b, int n) {
    Mat c((size_t) n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < n; ++k) {
            double aik = a[(size_t) i * n + k];
            if (aik == 0) continue;
            for (int j = 0; j < n; ++j) c[(size_t) i * n + j] += aik * b[(size_t) k * n + j];
        }
    return c;
}

}  // namespace

extern "C" int lqg_fisher_solve_n(int n, const double *fisher_sum, const double *dbt, double *fisher,
                                  double *solver, double *inverse, double *weighted, double *theta,
                                  int *damped, int *dof, double *damp_out) {
    if (n <= 0 || !fisher_sum || !dbt) return LQG_ERR_ARG;
    Mat F((size_t) n * n);
    for (size_t i = 0; i < F.size(); ++i) F[i] = 0.5 * fisher_sum[i];
    for (int i = 0; i < n; ++i)
        for (int j = i + 1; j < n; ++j) F[(size_t) j * n + i] = F[(size_t) i * n + j];
    if (fisher) std::copy(F.begin(), F.end(), fisher);
    Mat S = F;
    std::vector<int> empty;
    for (int i = 0; i < n; ++i)
        if (S[(size_t) i * n + i] == 0) { empty.push_back(i); S[(size_t) i * n + i] = 1.0; }
    std::vector<double> ev;
    if (!sym_eigenvalues(S, n, ev)) return LQG_ERR_SINGULAR;
    for (auto &v : ev) v = std::fabs(v);
    std::sort(ev.begin(), ev.end(), std::greater<double>());
    double damp = 0;
    for (int i = n - 1; i > 0; --i) {
        if (ev[i - 1] / ev[i] > 8.) damp = ev[i];
        else break;
    }
    Mat sol, inv;
    int warn = 0;
    if (damp != 0) {
        warn = 1;
        if (!invert(S, n, inv)) return LQG_ERR_SINGULAR;
        Mat A = matmul(S, S, n);
        for (int i = 0; i < n; ++i) A[(size_t) i * n + i] += damp;
        Mat Ai;
        if (!invert(A, n, Ai)) return LQG_ERR_SINGULAR;
        sol = matmul(Ai, S, n);
    } else {
        if (!invert(S, n, sol)) return LQG_ERR_SINGULAR;
        inv = sol;
    }
    for (int i : empty) { sol[(size_t) i * n + i] = 0; inv[(size_t) i * n + i] = 0; }
    std::vector<double> w(3 * (size_t) n, 0.0);
    for (int k = 0; k < 3; ++k)
        for (int i = 0; i < n; ++i) {
            double s = 0;
            for (int j = 0; j < n; ++j) s += sol[(size_t) i * n + j] * dbt[(size_t) k * n + j];
            w[(size_t) k * n + i] = 0.5 * s;
        }
    if (solver) std::copy(sol.begin(), sol.end(), solver);
    if (inverse) std::copy(inv.begin(), inv.end(), inverse);
    if (weighted) std::copy(w.begin(), w.end(), weighted);
    if (theta)
        for (int i = 0; i < n; ++i) theta[i] = w[i] - w[(size_t) n + i] - w[(size_t) 2 * n + i];
    if (damped) *damped = warn;
    if (dof) *dof = n - (int) empty.size();
    if (damp_out) *damp_out = damp;
    return LQG_OK;
}
