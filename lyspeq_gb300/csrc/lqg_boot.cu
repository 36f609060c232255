// Poisson bootstrap over spectra, lyspeq's FastBootstrap
// (PoissonBootstrapper::_fastBootstrap and _meanBootstrap, core/bootstrapper.hpp,
// after OneQSOEstimate::collapseBootstrap, core/one_qso_estimate.cpp:200-238):
//
//   theta_q      = sum over the spectrum's chunks of d - b - t (placed at fisher_index_start)
//   x_b          = sum_q p_qb theta_q,   p_qb ~ Poisson(1)       (b < nboots realizations)
//   mean         = (sum_b x_b) / nboots
//   cov          = sum_b (x_b - mean)(x_b - mean)^T / (nboots - 1)
//   fisher_cov   = cov / 4,   covariance = F_solver^-1 fisher_cov F_solver^-T
//
// The coefficients are drawn on the host with the generator the reference uses
// (std::mt19937_64 seeded with the process index, std::poisson_distribution of
// mean 1, nboots draws per spectrum in queue order), so the realizations are
// the reference's.  The sums run on the GPU in FP64, every sum in the
// reference's order (spectra, then realizations, in sequence).
#include "lqg_internal.cuh"

#include <algorithm>
#include <random>
#include <string>
#include <vector>

namespace lqg {

namespace {

// theta[q][k] for spectrum q: its chunks' ((d - b) - t) added in batch order
__global__ void k_boot_theta(const ChunkDesc *meta, const double *results, const int *qoff, int nkz,
                             double *theta) {
    const int q = blockIdx.x;
    double *th = theta + (size_t) q * nkz;
    for (int k = threadIdx.x; k < nkz; k += blockDim.x) th[k] = 0.0;
    __syncthreads();
    for (int c = qoff[q]; c < qoff[q + 1]; ++c) {
        const ChunkDesc &ch = meta[c];
        const double *r = results + ch.res_off;
        for (int i = threadIdx.x; i < ch.nq; i += blockDim.x) {
            const double v = (r[i] - r[ch.nq + i]) - r[2 * ch.nq + i];
            th[ch.fis + i] += v;
        }
        __syncthreads();
    }
}

// x[b][k] = sum_q p[q][b] theta[q][k], q in order; 64 x 64 output tiles, 4 x 4 per thread
constexpr int BT = 64, BQ = 16;
__global__ void __launch_bounds__(256) k_boot_real(const unsigned char *p, const double *theta, int nq, int nb,
                                                   int nkz, double *x) {
    const int b0 = blockIdx.y * BT, k0 = blockIdx.x * BT;
    __shared__ double ps[BQ][BT + 1], ts[BQ][BT + 1];
    const int tb = (threadIdx.x / 16) * 4, tk = (threadIdx.x % 16) * 4;
    double acc[4][4] = {};
    for (int q0 = 0; q0 < nq; q0 += BQ) {
        for (int e = threadIdx.x; e < BQ * BT; e += blockDim.x) {
            const int qq = e / BT, cc = e % BT, q = q0 + qq;
            ps[qq][cc] = (q < nq && b0 + cc < nb) ? (double) p[(size_t) q * nb + b0 + cc] : 0.0;
            ts[qq][cc] = (q < nq && k0 + cc < nkz) ? theta[(size_t) q * nkz + k0 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int qq = 0; qq < BQ; ++qq) {
            double pv[4], tv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { pv[u] = ps[qq][tb + u]; tv[u] = ts[qq][tk + u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) acc[u][w] = fma(pv[u], tv[w], acc[u][w]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w)
            if (b0 + tb + u < nb && k0 + tk + w < nkz) x[(size_t) (b0 + tb + u) * nkz + k0 + tk + w] = acc[u][w];
}

// mean[k] = (sum_b x[b][k]) * (1 / nvalid), b over all nb slots
// (PoissonBootstrapper::_calcuateMean sums every slot and divides by the
// number of valid realizations)
__global__ void k_boot_mean(const double *x, int nb, int nkz, int nvalid, double *mean) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nkz) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += x[(size_t) b * nkz + k];
    mean[k] = s * (1. / nvalid);
}

// cov[i][j] = cov[j][i] = (sum_b (x_bi - m_i)(x_bj - m_j)) * (1 / (nvalid - 1)), i <= j,
// b over all nb slots (_calcuateCovariance)
__global__ void k_boot_cov(const double *x, const double *mean, int nb, int nkz, int nvalid, double *cov) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= nkz || j < i) return;
    const double mi = mean[i], mj = mean[j];
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s = fma(x[(size_t) b * nkz + i] - mi, x[(size_t) b * nkz + j] - mj, s);
    s *= 1. / (nvalid - 1);
    cov[(size_t) i * nkz + j] = s;
    cov[(size_t) j * nkz + i] = s;
}

// C = A B (transb = 0) or A B^T (transb = 1), n x n row-major FP64
__global__ void __launch_bounds__(256) k_boot_gemm(const double *A, const double *B, double *C, int n, int transb) {
    const int i0 = blockIdx.y * BT, j0 = blockIdx.x * BT;
    __shared__ double as[BQ][BT + 1], bs[BQ][BT + 1];
    const int ti = (threadIdx.x / 16) * 4, tj = (threadIdx.x % 16) * 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < n; k0 += BQ) {
        for (int e = threadIdx.x; e < BQ * BT; e += blockDim.x) {
            const int kk = e / BT, cc = e % BT, k = k0 + kk;
            as[kk][cc] = (k < n && i0 + cc < n) ? A[(size_t) (i0 + cc) * n + k] : 0.0;
            const int jj = j0 + cc;
            bs[kk][cc] = (k < n && jj < n) ? (transb ? B[(size_t) jj * n + k] : B[(size_t) k * n + jj]) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BQ; ++kk)
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) acc[u][w] = fma(as[kk][ti + u], bs[kk][tj + w], acc[u][w]);
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w)
            if (i0 + ti + u < n && j0 + tj + w < n) C[(size_t) (i0 + ti + u) * n + j0 + tj + w] = acc[u][w];
}

__global__ void k_scale(double *x, size_t n, double s) {
    for (size_t e = (size_t) blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (size_t) gridDim.x * blockDim.x)
        x[e] *= s;
}

// ---------------------------------------------------------------------------
// Complete bootstrap (FastBootstrap 0, PoissonBootstrapper::_oneBoot): every
// realization b sums the spectra's Fisher matrices with its coefficients and
// solves for its power spectrum,
//   F_b = sum_q p_bq F_q (upper),  r_b = sum_q p_bq theta_q,  x_b = F_b^-1 r_b,
// F_q the upper triangle of the spectrum's chunk Fisher matrices
// (OneQSOEstimate::collapseBootstrap, core/one_qso_estimate.cpp:225-235).  The
// solve is mxhelp::LAPACKE_safeSolveCho (mathtools/matrix_helper.cpp:385-396):
// zero diagonals are set to 1, F_b = U^T U by Cholesky, and the solution of
// those bins is set to 0; a realization whose F_b is not positive definite is
// dropped.

constexpr int kBootMaxKz = 1023;   // nkz + 1 augmented columns <= 1024
constexpr int kBootSub = 8;        // realizations per block of the Fisher build
constexpr int kBootNB = 16;        // Cholesky panel rows

// Block q: F_q (dim_q x dim_q, row-major at foff[q]), its chunks added in
// order at offset fisher_index_start - istart_q.
__global__ void k_bootc_collapse(const ChunkDesc *meta, const double *results, const int *qoff, const int *qstart,
                                 const int *qdim, const int64_t *foff, double *fq) {
    const int q = blockIdx.x, nd = qdim[q];
    double *F = fq + foff[q];
    for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) F[e] = 0.0;
    __syncthreads();
    for (int c = qoff[q]; c < qoff[q + 1]; ++c) {
        const ChunkDesc &ch = meta[c];
        const double *fc = results + ch.res_off + 3 * ch.nq;
        const int off = ch.fis - qstart[q];
        for (int e = threadIdx.x; e < ch.nq * ch.nq; e += blockDim.x) {
            const int i = e / ch.nq, j = e % ch.nq;
            if (j >= i) F[(size_t) (off + i) * nd + off + j] += fc[e];
        }
        __syncthreads();
    }
}

// Row i of the augmented [F_b | r_b] (ld = nkz + 1, upper triangle and the
// last column) for the kBootSub realizations b0 + kBootSub blockIdx.y + v:
// spectra in queue order, each product rounded before it is added
// (OneQSOEstimate::addBoot, core/one_qso_estimate.hpp:43-53).  Zero diagonals
// become 1 and are flagged in `empty`.
__global__ void __launch_bounds__(256) k_bootc_fisher(const unsigned char *p, int nboots, int n_qso,
                                                      const int *qstart, const int *qdim, const int64_t *foff,
                                                      const double *fq, const double *r, int nkz, int b0, int nbat,
                                                      double *A, unsigned char *empty) {
    const int i = blockIdx.x, bs = b0 + kBootSub * blockIdx.y;
    const size_t ld = (size_t) nkz + 1, mat = (size_t) nkz * ld;
    constexpr int CU = (kBootMaxKz + 1) / 256;
    double acc[CU][kBootSub];
#pragma unroll
    for (int u = 0; u < CU; ++u)
#pragma unroll
        for (int v = 0; v < kBootSub; ++v) acc[u][v] = 0.0;
    for (int q = 0; q < n_qso; ++q) {
        const int s0 = qstart[q], nd = qdim[q];
        if (i < s0 || i >= s0 + nd) continue;
        double pv[kBootSub];
#pragma unroll
        for (int v = 0; v < kBootSub; ++v) pv[v] = bs + v < nboots ? (double) p[(size_t) q * nboots + bs + v] : 0.0;
        const double *row = fq + foff[q] + (size_t) (i - s0) * nd - s0;   // row[j] = F_q(i - s0, j - s0)
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            const int j = i + threadIdx.x + 256 * u;
            if (j >= s0 + nd) continue;
            const double f = row[j];
#pragma unroll
            for (int v = 0; v < kBootSub; ++v) acc[u][v] = __dadd_rn(acc[u][v], __dmul_rn(pv[v], f));
        }
    }
#pragma unroll
    for (int v = 0; v < kBootSub; ++v) {
        const int b = bs + v;
        if (b >= b0 + nbat || b >= nboots) break;
        double *Ab = A + (size_t) (b - b0) * mat + (size_t) i * ld;
#pragma unroll
        for (int u = 0; u < CU; ++u) {
            const int j = i + threadIdx.x + 256 * u;
            if (j > nkz) continue;
            double val = j == nkz ? r[(size_t) b * nkz + i] : acc[u][v];
            if (j == i) {
                empty[(size_t) (b - b0) * nkz + i] = val == 0.0;
                if (val == 0.0) val = 1.0;
            }
            Ab[j] = val;
        }
    }
}

// Cholesky of [F_b | r_b] (upper rows, F_b = U^T U; the last column becomes
// y = U^-T r_b) and back substitution U x = y, one block per realization.
// Panels of kBootNB rows are factored in shared memory, the rows below
// updated in global memory one warp per row.  valid[b] = 0 when a pivot is
// not positive (LAPACK's dpotrf fails there).
__global__ void __launch_bounds__(256) k_bootc_solve(double *A, const unsigned char *empty, int nkz, int b0,
                                                     double *x, int *valid) {
    extern __shared__ double ps[];   // kBootNB x (nkz + 1 - kb) panel; later y
    const int b = b0 + blockIdx.x;
    const int ld = nkz + 1;
    double *M = A + (size_t) blockIdx.x * nkz * ld;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    bool bad = false;
    for (int kb = 0; kb < nkz && !bad; kb += kBootNB) {
        const int nb = min(kBootNB, nkz - kb), w = ld - kb;
        __syncthreads();
        for (int e = threadIdx.x; e < nb * w; e += blockDim.x) {
            const int rr = e / w, c = e % w;
            ps[rr * w + c] = c >= rr ? M[(size_t) (kb + rr) * ld + kb + c] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < nb; ++k) {
            const double d = ps[k * w + k];
            __syncthreads();
            if (!(d > 0.0)) { bad = true; break; }   // the same d in every thread
            const double u = sqrt(d);
            for (int c = k + threadIdx.x; c < w; c += blockDim.x) ps[k * w + c] = c == k ? u : ps[k * w + c] / u;
            __syncthreads();
            const int rows = nb - k - 1;
            for (int e = threadIdx.x; e < rows * w; e += blockDim.x) {
                const int rr = k + 1 + e / w, c = e % w;
                if (c >= rr) ps[rr * w + c] -= ps[k * w + rr] * ps[k * w + c];
            }
            __syncthreads();
        }
        if (bad) break;
        for (int e = threadIdx.x; e < nb * w; e += blockDim.x) {
            const int rr = e / w, c = e % w;
            if (c >= rr) M[(size_t) (kb + rr) * ld + kb + c] = ps[rr * w + c];
        }
        for (int i = kb + nb + warp; i < nkz; i += blockDim.x / 32) {
            const int ci = i - kb;
            for (int j = i + lane; j <= nkz; j += 32) {
                const int cj = j - kb;
                double a = 0.0;
#pragma unroll 4
                for (int rr = 0; rr < nb; ++rr) a = fma(ps[rr * w + ci], ps[rr * w + cj], a);
                M[(size_t) i * ld + j] -= a;
            }
        }
    }
    if (bad) {
        if (threadIdx.x == 0) valid[b] = 0;
        return;
    }
    __syncthreads();
    double *y = ps;
    for (int i = threadIdx.x; i < nkz; i += blockDim.x) y[i] = M[(size_t) i * ld + nkz];
    for (int j = nkz - 1; j >= 0; --j) {
        __syncthreads();
        const double xj = y[j] / M[(size_t) j * ld + j];
        __syncthreads();
        if (threadIdx.x == 0) y[j] = xj;
        for (int i = threadIdx.x; i < j; i += blockDim.x) y[i] -= M[(size_t) i * ld + j] * xj;
    }
    __syncthreads();
    const unsigned char *eb = empty + (size_t) blockIdx.x * nkz;
    for (int i = threadIdx.x; i < nkz; i += blockDim.x) x[(size_t) b * nkz + i] = eb[i] ? 0.0 : y[i];
    if (threadIdx.x == 0) valid[b] = 1;
}

// Slots of the realizations as the reference leaves them: the valid ones in
// order, then, if the last realization failed, its unsolved power (the slot
// it was written to before its solve failed), zeros after that.
__global__ void k_bootc_slots(const double *xs, const double *r, const int *src, int nboots, int nkz, double *out) {
    const int slot = blockIdx.x;
    const int b = src[slot];
    for (int k = threadIdx.x; k < nkz; k += blockDim.x) {
        double v = 0.0;
        if (b >= 0) v = xs[(size_t) b * nkz + k];
        else if (b == -2) v = r[(size_t) (nboots - 1) * nkz + k];
        out[(size_t) slot * nkz + k] = v;
    }
}


struct Buf {
    void *p = nullptr;
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 8)); }
    template <class T> T *as() { return static_cast<T *>(p); }
};

}  // namespace

// PoissonRNG(seed) (core/bootstrapper.hpp:20-37): std::mt19937_64 seeded with
// `seed`, std::poisson_distribution of mean 1.  FastBootstrap draws nboots
// coefficients per spectrum, spectra in queue order; the complete bootstrap
// draws one per spectrum per realization, realizations in order.  p is
// written spectrum-major, p[q * nboots + b], in either case.
int draw_coefficients(unsigned long long seed, int n_qso, int nboots, bool per_realization, unsigned char *p,
                      std::string &err) {
    std::mt19937_64 engine;
    engine.seed(seed);
    std::poisson_distribution<int> dist;
    const size_t n = (size_t) n_qso * nboots;
    for (size_t e = 0; e < n; ++e) {
        const int v = dist(engine);
        if (v > 255) {
            err = "lqg_bootstrap: Poisson coefficient above 255";
            return LQG_ERR_STATE;
        }
        const size_t q = per_realization ? e % n_qso : e / nboots, b = per_realization ? e / n_qso : e % nboots;
        p[q * nboots + b] = (unsigned char) v;
    }
    return LQG_OK;
}

namespace {

int check_offsets(int n_qso, const int *qso_offsets, int n_chunks, std::string &err) {
    if (qso_offsets[0] != 0 || qso_offsets[n_qso] != n_chunks) {
        err = "lqg_bootstrap: spectrum offsets must start at 0 and end at the batch size";
        return LQG_ERR_ARG;
    }
    for (int q = 0; q < n_qso; ++q)
        if (qso_offsets[q + 1] < qso_offsets[q]) {
            err = "lqg_bootstrap: spectrum offsets not increasing";
            return LQG_ERR_ARG;
        }
    return LQG_OK;
}

}  // namespace

int run_fast_bootstrap(cudaStream_t st, const ChunkDesc *d_meta, const double *d_results, int nkz, int n_chunks,
                       int n_qso, const int *qso_offsets, int nboots, unsigned long long seed,
                       const double *solver, double *mean, double *cov, double *fisher_cov, double *realizations,
                       std::string &err) {
    if (int rc = check_offsets(n_qso, qso_offsets, n_chunks, err)) return rc;
    std::vector<unsigned char> p((size_t) n_qso * nboots);
    if (int rc = draw_coefficients(seed, n_qso, nboots, false, p.data(), err)) return rc;
    Buf d_p, d_off, d_theta, d_x, d_mean, d_cov, d_solv, d_tmp;
    if (d_p.alloc(p.size()) || d_off.alloc((size_t) (n_qso + 1) * 4) || d_theta.alloc((size_t) n_qso * nkz * 8) ||
        d_x.alloc((size_t) nboots * nkz * 8) || d_mean.alloc((size_t) nkz * 8) || d_cov.alloc((size_t) nkz * nkz * 8) ||
        d_solv.alloc((size_t) nkz * nkz * 8) || d_tmp.alloc((size_t) nkz * nkz * 8)) {
        err = "lqg_bootstrap: device memory";
        return LQG_ERR_NOMEM;
    }
    cudaMemcpyAsync(d_p.p, p.data(), p.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_off.p, qso_offsets, (size_t) (n_qso + 1) * 4, cudaMemcpyHostToDevice, st);
    if (solver) cudaMemcpyAsync(d_solv.p, solver, (size_t) nkz * nkz * 8, cudaMemcpyHostToDevice, st);
    if (n_qso > 0)
        k_boot_theta<<<n_qso, 256, 0, st>>>(d_meta, d_results, d_off.as<int>(), nkz, d_theta.as<double>());
    k_boot_real<<<dim3((nkz + BT - 1) / BT, (nboots + BT - 1) / BT), 256, 0, st>>>(
        d_p.as<unsigned char>(), d_theta.as<double>(), n_qso, nboots, nkz, d_x.as<double>());
    k_boot_mean<<<(nkz + 127) / 128, 128, 0, st>>>(d_x.as<double>(), nboots, nkz, nboots, d_mean.as<double>());
    k_boot_cov<<<dim3((nkz + 127) / 128, nkz), 128, 0, st>>>(d_x.as<double>(), d_mean.as<double>(), nboots, nkz,
                                                            nboots, d_cov.as<double>());
    // FastBootstrap output (PoissonBootstrapper::_saveData): cov / 4, then F^-1 (cov / 4) F^-T
    k_scale<<<64, 256, 0, st>>>(d_cov.as<double>(), (size_t) nkz * nkz, 0.25);
    if (fisher_cov) cudaMemcpyAsync(fisher_cov, d_cov.p, (size_t) nkz * nkz * 8, cudaMemcpyDeviceToHost, st);
    if (cov) {
        if (!solver) {
            err = "lqg_bootstrap: the covariance needs the Fisher solver matrix";
            return LQG_ERR_ARG;
        }
        const dim3 g((nkz + BT - 1) / BT, (nkz + BT - 1) / BT);
        k_boot_gemm<<<g, 256, 0, st>>>(d_solv.as<double>(), d_cov.as<double>(), d_tmp.as<double>(), nkz, 0);
        k_boot_gemm<<<g, 256, 0, st>>>(d_tmp.as<double>(), d_solv.as<double>(), d_cov.as<double>(), nkz, 1);
        cudaMemcpyAsync(cov, d_cov.p, (size_t) nkz * nkz * 8, cudaMemcpyDeviceToHost, st);
    }
    if (mean) cudaMemcpyAsync(mean, d_mean.p, (size_t) nkz * 8, cudaMemcpyDeviceToHost, st);
    if (realizations)
        cudaMemcpyAsync(realizations, d_x.p, (size_t) nboots * nkz * 8, cudaMemcpyDeviceToHost, st);
    const cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        err = std::string("lqg_bootstrap: ") + cudaGetErrorString(e);
        return LQG_ERR_CUDA;
    }
    return LQG_OK;
}

int run_complete_bootstrap(cudaStream_t st, const ChunkDesc *d_meta, const double *d_results, int nkz,
                           int n_chunks, const int *chunk_fis, const int *chunk_nq, int n_qso,
                           const int *qso_offsets, int nboots, unsigned long long seed, double *mean, double *cov,
                           double *realizations, int *n_valid, std::string &err) {
    if (int rc = check_offsets(n_qso, qso_offsets, n_chunks, err)) return rc;
    if (nkz > kBootMaxKz) {
        err = "lqg_bootstrap_complete: more than 1023 (k, z) bins";
        return LQG_ERR_UNSUPPORTED;
    }
    std::vector<unsigned char> p((size_t) n_qso * nboots);
    if (int rc = draw_coefficients(seed, n_qso, nboots, true, p.data(), err)) return rc;
    // footprint of each spectrum: [istart, istart + ndim) over its chunks
    // (collapseBootstrap, core/one_qso_estimate.cpp:200-210); a spectrum
    // without chunks contributes nothing
    std::vector<int> qstart(n_qso), qdim(n_qso);
    std::vector<int64_t> foff(n_qso + 1, 0);
    for (int q = 0; q < n_qso; ++q) {
        int lo = nkz, hi = 0;
        for (int c = qso_offsets[q]; c < qso_offsets[q + 1]; ++c) {
            lo = std::min(lo, chunk_fis[c]);
            hi = std::max(hi, chunk_fis[c] + chunk_nq[c]);
        }
        qstart[q] = hi > lo ? lo : 0;
        qdim[q] = hi > lo ? hi - lo : 0;
        foff[q + 1] = foff[q] + (int64_t) qdim[q] * qdim[q];
    }
    const size_t ld = (size_t) nkz + 1, mat = (size_t) nkz * ld * 8;
    const int nbat = (int) std::max<size_t>(1, std::min<size_t>((size_t) nboots, (size_t) (1u << 30) / mat));
    Buf d_p, d_off, d_qs, d_qd, d_fo, d_fq, d_theta, d_r, d_xs, d_x, d_a, d_empty, d_valid, d_src, d_mean, d_cov;
    if (d_p.alloc(p.size()) || d_off.alloc((size_t) (n_qso + 1) * 4) || d_qs.alloc((size_t) n_qso * 4) ||
        d_qd.alloc((size_t) n_qso * 4) || d_fo.alloc((size_t) (n_qso + 1) * 8) || d_fq.alloc((size_t) foff[n_qso] * 8) ||
        d_theta.alloc((size_t) n_qso * nkz * 8) || d_r.alloc((size_t) nboots * nkz * 8) ||
        d_xs.alloc((size_t) nboots * nkz * 8) || d_x.alloc((size_t) nboots * nkz * 8) ||
        d_a.alloc((size_t) nbat * mat) || d_empty.alloc((size_t) nbat * nkz) || d_valid.alloc((size_t) nboots * 4) ||
        d_src.alloc((size_t) nboots * 4) || d_mean.alloc((size_t) nkz * 8) || d_cov.alloc((size_t) nkz * nkz * 8)) {
        err = "lqg_bootstrap_complete: device memory";
        return LQG_ERR_NOMEM;
    }
    cudaMemcpyAsync(d_p.p, p.data(), p.size(), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_off.p, qso_offsets, (size_t) (n_qso + 1) * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_qs.p, qstart.data(), (size_t) n_qso * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_qd.p, qdim.data(), (size_t) n_qso * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_fo.p, foff.data(), (size_t) (n_qso + 1) * 8, cudaMemcpyHostToDevice, st);
    if (n_qso > 0) {
        k_boot_theta<<<n_qso, 256, 0, st>>>(d_meta, d_results, d_off.as<int>(), nkz, d_theta.as<double>());
        k_bootc_collapse<<<n_qso, 256, 0, st>>>(d_meta, d_results, d_off.as<int>(), d_qs.as<int>(), d_qd.as<int>(),
                                               d_fo.as<int64_t>(), d_fq.as<double>());
    }
    k_boot_real<<<dim3((nkz + BT - 1) / BT, (nboots + BT - 1) / BT), 256, 0, st>>>(
        d_p.as<unsigned char>(), d_theta.as<double>(), n_qso, nboots, nkz, d_r.as<double>());
    const size_t smem = (size_t) kBootNB * ld * 8;
    cudaFuncSetAttribute(k_bootc_solve, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    for (int b0 = 0; b0 < nboots; b0 += nbat) {
        const int nb = std::min(nbat, nboots - b0);
        k_bootc_fisher<<<dim3(nkz, (nb + kBootSub - 1) / kBootSub), 256, 0, st>>>(
            d_p.as<unsigned char>(), nboots, n_qso, d_qs.as<int>(), d_qd.as<int>(), d_fo.as<int64_t>(),
            d_fq.as<double>(), d_r.as<double>(), nkz, b0, nb, d_a.as<double>(), d_empty.as<unsigned char>());
        k_bootc_solve<<<nb, 256, smem, st>>>(d_a.as<double>(), d_empty.as<unsigned char>(), nkz, b0, d_xs.as<double>(),
                                             d_valid.as<int>());
    }
    std::vector<int> valid(nboots);
    cudaMemcpyAsync(valid.data(), d_valid.p, (size_t) nboots * 4, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        err = std::string("lqg_bootstrap_complete: ") + cudaGetErrorString(e);
        return LQG_ERR_CUDA;
    }
    // slots as PoissonBootstrapper::run leaves allpowers (core/bootstrapper.hpp:126-135, 217-257)
    std::vector<int> src(nboots, -1);
    int nv = 0;
    for (int b = 0; b < nboots; ++b)
        if (valid[b]) src[nv++] = b;
    if (!valid[nboots - 1] && nv < nboots) src[nv] = -2;
    if (n_valid) *n_valid = nv;
    cudaMemcpyAsync(d_src.p, src.data(), (size_t) nboots * 4, cudaMemcpyHostToDevice, st);
    k_bootc_slots<<<nboots, 128, 0, st>>>(d_xs.as<double>(), d_r.as<double>(), d_src.as<int>(), nboots, nkz,
                                         d_x.as<double>());
    if (nv >= 2) {
        k_boot_mean<<<(nkz + 127) / 128, 128, 0, st>>>(d_x.as<double>(), nboots, nkz, nv, d_mean.as<double>());
        k_boot_cov<<<dim3((nkz + 127) / 128, nkz), 128, 0, st>>>(d_x.as<double>(), d_mean.as<double>(), nboots, nkz,
                                                                nv, d_cov.as<double>());
        if (mean) cudaMemcpyAsync(mean, d_mean.p, (size_t) nkz * 8, cudaMemcpyDeviceToHost, st);
        if (cov) cudaMemcpyAsync(cov, d_cov.p, (size_t) nkz * nkz * 8, cudaMemcpyDeviceToHost, st);
    }
    if (realizations)
        cudaMemcpyAsync(realizations, d_x.p, (size_t) nboots * nkz * 8, cudaMemcpyDeviceToHost, st);
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) {
        err = std::string("lqg_bootstrap_complete: ") + cudaGetErrorString(e);
        return LQG_ERR_CUDA;
    }
    if (nv < 2) {
        err = "lqg_bootstrap_complete: fewer than two realizations with a positive definite Fisher matrix";
        return LQG_ERR_STATE;
    }
    return LQG_OK;
}


}  // namespace lqg
