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

// mean[k] = (sum_b x[b][k]) * (1 / nb)
__global__ void k_boot_mean(const double *x, int nb, int nkz, double *mean) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nkz) return;
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += x[(size_t) b * nkz + k];
    mean[k] = s * (1. / nb);
}

// cov[i][j] = cov[j][i] = (sum_b (x_bi - m_i)(x_bj - m_j)) * (1 / (nb - 1)), i <= j
__global__ void k_boot_cov(const double *x, const double *mean, int nb, int nkz, double *cov) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y;
    if (j >= nkz || j < i) return;
    const double mi = mean[i], mj = mean[j];
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s = fma(x[(size_t) b * nkz + i] - mi, x[(size_t) b * nkz + j] - mj, s);
    s *= 1. / (nb - 1);
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

struct Buf {
    void *p = nullptr;
    ~Buf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 8)); }
    template <class T> T *as() { return static_cast<T *>(p); }
};

}  // namespace

int run_fast_bootstrap(cudaStream_t st, const ChunkDesc *d_meta, const double *d_results, int nkz, int n_chunks,
                       int n_qso, const int *qso_offsets, int nboots, unsigned long long seed,
                       const double *solver, double *mean, double *cov, double *fisher_cov, double *realizations,
                       std::string &err) {
    if (qso_offsets[0] != 0 || qso_offsets[n_qso] != n_chunks) {
        err = "lqg_bootstrap: spectrum offsets must start at 0 and end at the batch size";
        return LQG_ERR_ARG;
    }
    for (int q = 0; q < n_qso; ++q)
        if (qso_offsets[q + 1] < qso_offsets[q]) {
            err = "lqg_bootstrap: spectrum offsets not increasing";
            return LQG_ERR_ARG;
        }
    // PoissonRNG(seed): nboots draws per spectrum, spectra in queue order
    std::vector<unsigned char> p((size_t) n_qso * nboots);
    {
        std::mt19937_64 engine;
        engine.seed(seed);
        std::poisson_distribution<int> dist;
        for (size_t e = 0; e < p.size(); ++e) {
            const int v = dist(engine);
            if (v > 255) {
                err = "lqg_bootstrap: Poisson coefficient above 255";
                return LQG_ERR_STATE;
            }
            p[e] = (unsigned char) v;
        }
    }
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
    k_boot_mean<<<(nkz + 127) / 128, 128, 0, st>>>(d_x.as<double>(), nboots, nkz, d_mean.as<double>());
    k_boot_cov<<<dim3((nkz + 127) / 128, nkz), 128, 0, st>>>(d_x.as<double>(), d_mean.as<double>(), nboots, nkz,
                                                            d_cov.as<double>());
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

}  // namespace lqg
