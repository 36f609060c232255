// Global Newton-Raphson update: F/2, symmetrise, stable inversion and
// theta = 1/2 F_solver (d - b - t).  Follows core/quadratic_estimate.cpp:456-457,
// :261-288, :290-318 and mathtools/matrix_helper.cpp:220-358 (stableInvertSym).
// The reference decides damping from the singular values of F (dgesvd); F is
// symmetric, so they are the absolute eigenvalues, found here by Householder
// tridiagonalisation and implicit QL, unless F is positive definite and a
// Lanczos estimate on its Cholesky factor shows its two smallest eigenvalues
// well within the damping threshold.  The undamped inverse of the positive
// definite F is taken from that factor, the columns solved on the host's
// cores; Gauss-Jordan elimination with partial pivoting where the factor
// fails and in the damped branch (the reference: LU, dgetrf + dgetri).
// O(nkz^3) FP64.
#include "lqg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <thread>
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

// Dot product of two contiguous rows with four independent partial sums, so
// that the inner loops of the factor and the substitutions are not one chain
// of dependent additions.
inline double dot(const double *a, const double *b, int len) {
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    int k = 0;
    for (; k + 4 <= len; k += 4) {
        s0 += a[k] * b[k];
        s1 += a[k + 1] * b[k + 1];
        s2 += a[k + 2] * b[k + 2];
        s3 += a[k + 3] * b[k + 3];
    }
    for (; k < len; ++k) s0 += a[k] * b[k];
    return (s0 + s1) + (s2 + s3);
}

// Cholesky factor of a symmetric positive definite matrix: a = L L^T by rows
// (left-looking, every inner product over contiguous rows); U = L^T row-major
// for the back substitutions.  False if a pivot is not positive.
bool spd_factor(const Mat &a, int n, Mat &L, Mat &U) {
    L.assign((size_t) n * n, 0.0);
    for (int j = 0; j < n; ++j) {
        const double *lj = &L[(size_t) j * n];
        double d = a[(size_t) j * n + j] - dot(lj, lj, j);
        if (!(d > 0) || !std::isfinite(d)) return false;
        d = std::sqrt(d);
        L[(size_t) j * n + j] = d;
        for (int i = j + 1; i < n; ++i)
            L[(size_t) i * n + j] = (a[(size_t) i * n + j] - dot(&L[(size_t) i * n], lj, j)) / d;
    }
    U.assign((size_t) n * n, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = 0; k <= i; ++k) U[(size_t) k * n + i] = L[(size_t) i * n + k];
    return true;
}

// x = (L L^T)^-1 b by forward and back substitution.
void spd_solve(const Mat &L, const Mat &U, int n, const double *b, double *y, double *x) {
    for (int i = 0; i < n; ++i) {
        const double *li = &L[(size_t) i * n];
        y[i] = (b[i] - dot(li, y, i)) / li[i];
    }
    for (int i = n - 1; i >= 0; --i) {
        const double *ui = &U[(size_t) i * n];
        x[i] = (y[i] - dot(ui + i + 1, x + i + 1, n - 1 - i)) / ui[i];
    }
}

// The inverse from the factor: column c from L y = e_c and L^T x = y, the
// columns split over up to 16 threads, created and joined here.
void spd_inverse(const Mat &L, const Mat &U, int n, Mat &inv) {
    inv.assign((size_t) n * n, 0.0);
    auto columns = [&](int first, int step) {
        std::vector<double> y(n), x(n);
        for (int c = first; c < n; c += step) {
            std::fill(y.begin(), y.begin() + c, 0.0);
            for (int i = c; i < n; ++i) {
                const double *li = &L[(size_t) i * n];
                y[i] = ((i == c ? 1.0 : 0.0) - dot(li + c, &y[c], i - c)) / li[i];
            }
            for (int i = n - 1; i >= 0; --i) {
                const double *ui = &U[(size_t) i * n];
                x[i] = (y[i] - dot(ui + i + 1, &x[i + 1], n - 1 - i)) / ui[i];
            }
            for (int i = 0; i < n; ++i) inv[(size_t) i * n + c] = x[i];
        }
    };
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = (int) std::max(1u, std::min(16u, hw ? hw : 1u));
    if (nt == 1 || n < 64) {
        columns(0, 1);
    } else {
        // columns t, t + nt, ... on thread t; a thread the system does not
        // grant runs its columns here instead
        std::vector<std::thread> pool;
        std::vector<int> inline_first;
        for (int t = 1; t < nt; ++t) {
            try {
                pool.emplace_back(columns, t, nt);
            } catch (...) {
                inline_first.push_back(t);
            }
        }
        columns(0, nt);
        for (int t : inline_first) columns(t, nt);
        for (auto &th : pool) th.join();
    }
}

// Whether the damping test of stableInvertSym could fire: it needs the two
// smallest eigenvalues of the positive definite F (its singular values) more
// than 8 apart.  They are the two largest of F^-1, estimated by 40 Lanczos
// steps with full reorthogonalisation (two triangular solves per step) from a
// fixed start vector: a component along the smallest eigenvector as small as
// rounding grows by the ratio (> 8) every step, so a separated smallest
// eigenvalue is not missed.  Returns false (no damping) only when the ratio of
// the estimates is below 4 and stable over the last 10 steps; true sends the
// caller to the full eigenvalue test.
bool damping_possible(const Mat &L, const Mat &U, int n) {
    const int K = 40;
    if (n < 64) return true;   // the full test costs little there
    std::vector<std::vector<double>> V(K + 1, std::vector<double>(n));
    for (int i = 0; i < n; ++i) V[0][i] = 1.0 + 0.25 * std::sin(1.0 + 0.7 * i);
    double nrm = 0;
    for (double v : V[0]) nrm += v * v;
    nrm = std::sqrt(nrm);
    for (double &v : V[0]) v /= nrm;
    std::vector<double> alpha(K), beta(K), w(n), y(n);
    double prev_ratio = -1, ratio = -1;
    for (int k = 0; k < K; ++k) {
        spd_solve(L, U, n, V[k].data(), y.data(), w.data());
        const double a = dot(w.data(), V[k].data(), n);
        alpha[k] = a;
        for (int pass = 0; pass < 2; ++pass)
            for (int j = 0; j <= k; ++j) {
                const double h = dot(w.data(), V[j].data(), n);
                for (int i = 0; i < n; ++i) w[i] -= h * V[j][i];
            }
        const double b = std::sqrt(dot(w.data(), w.data(), n));
        beta[k] = b;
        // the two largest Ritz values of the (k + 1) x (k + 1) tridiagonal
        const int m = k + 1;
        if (m >= 2) {
            Mat T((size_t) m * m, 0.0);
            for (int i = 0; i < m; ++i) {
                T[(size_t) i * m + i] = alpha[i];
                if (i + 1 < m) T[(size_t) i * m + i + 1] = T[(size_t) (i + 1) * m + i] = beta[i];
            }
            std::vector<double> ev;
            if (!sym_eigenvalues(T, m, ev)) return true;
            std::sort(ev.begin(), ev.end(), std::greater<double>());
            if (!(ev[1] > 0)) return true;
            if (k == K - 10) prev_ratio = ev[0] / ev[1];
            ratio = ev[0] / ev[1];   // lambda_2 / lambda_1 of F
        }
        // a Krylov space that closes early may have missed an eigenvector
        if (!(b > 1e-12 * std::fabs(a)) || !std::isfinite(b)) return true;
        for (int i = 0; i < n; ++i) V[k + 1][i] = w[i] / b;
    }
    if (!(ratio > 0) || !std::isfinite(ratio) || !(prev_ratio > 0)) return true;
    if (std::fabs(ratio - prev_ratio) > 1e-6 * ratio) return true;
    return !(ratio < 4.0);
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
    // F positive definite with its two smallest eigenvalues clearly within a
    // factor 8: no damping, and the inverse from the Cholesky factor, taken
    // while one more thread runs the Lanczos test (the damped branch, rare,
    // discards it)
    Mat L, U, spd_inv;
    const bool spd = spd_factor(S, n, L, U);
    bool possible = true;
    if (spd) {
        std::thread test;
        try {
            test = std::thread([&] { possible = damping_possible(L, U, n); });
        } catch (...) {
            possible = damping_possible(L, U, n);   // no thread granted: in turn
        }
        spd_inverse(L, U, n, spd_inv);
        if (test.joinable()) test.join();
    }
    double damp = 0;
    if (possible) {
        std::vector<double> ev;
        if (!sym_eigenvalues(S, n, ev)) return LQG_ERR_SINGULAR;
        for (auto &v : ev) v = std::fabs(v);
        std::sort(ev.begin(), ev.end(), std::greater<double>());
        for (int i = n - 1; i > 0; --i) {
            if (ev[i - 1] / ev[i] > 8.) damp = ev[i];
            else break;
        }
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
        if (spd) sol.swap(spd_inv);
        else if (!invert(S, n, sol)) return LQG_ERR_SINGULAR;
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
