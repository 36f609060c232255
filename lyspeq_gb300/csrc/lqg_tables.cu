// SQ lookup tables on the GPU: what SQLookupTable::computeTables
// (core/sq_table.cpp:201-323) writes to its FITS files, for a list of (R, dv)
// pairs, in the layout lqg_tables takes.
//
//   Q_k(v)   = (1/pi) int_{k1}^{k2} W^2(k) cos(k v) dk         (FourierIntegrator, GSL QAWO)
//   S(z, v)  = (1/L) c2r[ W^2(k_i) P_fid(k_i, z) ](RFT_M v / dv_table)   (RealField, FFTW)
//   W(k)     = sinc(k dv / 2) exp(-k^2 R^2 / 2),  R = c / R_fwhm / 2.35482
//   P_fid    = the Palanque-Delabrouille et al. 2013 fit (core/fiducial_cosmology.cpp:273-282)
//
// The derivative integrals use composite 8-point Gauss-Legendre quadrature on
// panels narrower than 3 / v_length (the cosine's period at the largest v is
// 2 pi / v_length), one FP64 thread per (table, band, v).  The signal is the
// reference's discretisation exactly: the real inverse FFT of W^2 P on the grid
// of RealField(nrft, dv_table / RFT_M) with nrft = 2^(ceil(log2(2 RFT_M nv)) + 1),
// sampled at every RFT_M-th point.  Only those samples are needed, so the
// spectrum is folded to nrft / 2 points and transformed by a radix-2 Stockham
// FFT in FP64 (one kernel per pass over all transforms of a group of tables).
#include "lqg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>

namespace lqg {

namespace {

constexpr int kRftM = 2;                 // RFT_M, core/sq_table.cpp:222
constexpr double kOneSigma2Fwhm = 2.35482004503;

struct Pd13 { double A, n, alpha, B, beta, lambda; };

// pd13::Palanque_Delabrouille_etal_2013_fit (core/fiducial_cosmology.cpp:273-282)
__device__ __forceinline__ double pd13_power(double k, double z, const Pd13 &p) {
    const double k0 = 0.009, z0 = 3.0;
    const double q0 = k / k0 + 1e-15, x0 = (1. + z) / (1. + z0);
    return (p.A * kPi / k0) * pow(q0, 2. + p.n + p.alpha * log(q0) + p.beta * log(x0)) * pow(x0, p.B) /
           (1. + p.lambda * k * k);
}

// W^2(k) of spectral_response_window_fn (core/fiducial_cosmology.cpp:305-313)
__device__ __forceinline__ double window2(double k, double dv, double r_kms) {
    const double x = k * dv / 2.;
    const double s = (x == 0.) ? 1. : sin(x) / x;
    const double kr = k * r_kms;
    const double w = s * exp(-kr * kr / 2.);
    return w * w;
}

// weights w_m W^2(k_m) / pi of every quadrature node for every table
__global__ void k_tab_weights(const double *nodes, const double *weights, int n_nodes, const double *tdv,
                              const double *trk, int n_tables, double *wt) {
    const int t = blockIdx.y;
    for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n_nodes; m += gridDim.x * blockDim.x)
        wt[(size_t) t * n_nodes + m] = weights[m] * window2(nodes[m], tdv[t], trk[t]) / kPi;
}

// deriv[t][kn][i] = sum over the band's nodes of wt * cos(k v_i)
__global__ void k_tab_deriv(const double *nodes, const double *wt, const int *band_off, int n_nodes, int nk,
                            int nv, double dv_grid, double *deriv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x, kn = blockIdx.y, t = blockIdx.z;
    if (i >= nv) return;
    const double v = dv_grid * i;
    const double *w = wt + (size_t) t * n_nodes;
    double acc = 0.0;
    for (int m = band_off[kn]; m < band_off[kn + 1]; ++m) acc += w[m] * cos(nodes[m] * v);
    deriv[((size_t) t * nk + kn) * nv + i] = acc;
}

// Folded spectrum of one (table, z): Z_j = Y_j + Y_{j + N} (j < N = nrft / 2)
// with Y the Hermitian extension of X_i = W^2(k_i) P(k_i, z), k_i = i 2 pi / L.
// Then x_{RFT_M m} = sum_j Z_j e^{+2 pi i j m / N}.
__global__ void k_tab_spectrum(int nrft, double length, const double *tdv, const double *trk, int t0,
                               const double *zs, int nzp, Pd13 fid, double2 *buf) {
    const int N = nrft / 2, tr = blockIdx.y;       // transform = (table in group, z)
    const int t = t0 + tr / nzp, iz = tr % nzp;
    const double kf = 2. * kPi / length;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < N; j += gridDim.x * blockDim.x) {
        // Y_j = X_j (j <= nrft/2);  Y_{j+N} = X_{nrft - (j+N)} = X_{N - j}
        const double kj = kf * j, kk = kf * (N - j);
        double z = window2(kj, tdv[t], trk[t]) * pd13_power(kj, zs[iz], fid);
        z += window2(kk, tdv[t], trk[t]) * pd13_power(kk, zs[iz], fid);
        buf[(size_t) tr * N + j] = make_double2(z, 0.0);
    }
}

// One radix-2 Stockham pass (e^{+} direction) over `batch` transforms of N points:
// v0 = a[j], v1 = a[j + N/2] w^(j mod ns) with w = e^{i pi / ns};
// b[(j / ns) 2 ns + j mod ns] = v0 + v1, b[... + ns] = v0 - v1.
__global__ void k_tab_fft_pass(const double2 *a, double2 *b, int N, int ns) {
    const int tr = blockIdx.y, half = N / 2;
    const double2 *x = a + (size_t) tr * N;
    double2 *y = b + (size_t) tr * N;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < half; j += gridDim.x * blockDim.x) {
        const int r = j % ns;
        double s, c;
        sincospi((double) r / ns, &s, &c);
        const double2 v0 = x[j], u = x[j + half];
        const double2 v1 = make_double2(u.x * c - u.y * s, u.x * s + u.y * c);
        const int o = (j / ns) * 2 * ns + r;
        y[o] = make_double2(v0.x + v1.x, v0.y + v1.y);
        y[o + ns] = make_double2(v0.x - v1.x, v0.y - v1.y);
    }
}

// signal[t][i][iz] = Re(x_i) / L for the first nv outputs of each transform
__global__ void k_tab_signal(const double2 *buf, int N, int nv, int nzp, double inv_len, int t0,
                             double *signal) {
    const int tr = blockIdx.y, t = t0 + tr / nzp, iz = tr % nzp;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nv; i += gridDim.x * blockDim.x)
        signal[((size_t) t * nv + i) * nzp + iz] = buf[(size_t) tr * N + i].x * inv_len;
}

// Nodes and weights of the 8-point Gauss-Legendre rule on [-1, 1] (Newton on P_8).
void gauss_legendre8(double *x, double *w) {
    const int n = 8;
    for (int i = 0; i < n; ++i) {
        double z = std::cos(kPi * (i + 0.75) / (n + 0.5)), pp = 0;
        for (int it = 0; it < 100; ++it) {
            double p1 = 1, p2 = 0;
            for (int j = 1; j <= n; ++j) {
                const double p3 = p2;
                p2 = p1;
                p1 = ((2. * j - 1.) * z * p2 - (j - 1.) * p3) / j;
            }
            pp = n * (z * p1 - p2) / (z * z - 1.);
            const double dz = p1 / pp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        x[n - 1 - i] = z;
        w[n - 1 - i] = 2. / ((1. - z * z) * pp * pp);
    }
}

struct DevMem {
    void *p = nullptr;
    ~DevMem() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, std::max<size_t>(n, 8)); }
    template <class T> T *as() { return static_cast<T *>(p); }
};

}  // namespace

}  // namespace lqg

using namespace lqg;

extern "C" int lqg_tables_generate(const lqg_bins *bins, int n_tables, const int *r_fwhm, const double *dv,
                                   int nv, double v_length, int nzp, const double *fid, int with_signal,
                                   double *deriv, double *signal, int device) {
    if (!bins || n_tables < 1 || !r_fwhm || !dv || nv < 2 || !(v_length > 0) || nzp < 2 || !deriv ||
        (with_signal && (!signal || !fid)) || bins->nk < 1 || bins->nz < 1 || !bins->k_edges ||
        !bins->z_centers || !(bins->z_bin_width > 0))
        return LQG_ERR_ARG;
    for (int t = 0; t < n_tables; ++t)
        if (r_fwhm[t] <= 0 || !(dv[t] > 0)) return LQG_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LQG_ERR_CUDA;
    const int nk = bins->nk;
    // quadrature nodes of every band: panels of width <= 3 / v_length
    double gx[8], gw[8];
    gauss_legendre8(gx, gw);
    const double width = 3.0 / std::max(v_length, 1.0);
    std::vector<double> nodes, weights;
    std::vector<int> band_off(1, 0);
    for (int kn = 0; kn < nk; ++kn) {
        const double a = bins->k_edges[kn], b = bins->k_edges[kn + 1];
        if (b > a) {
            const int npan = std::max(1, (int) std::ceil((b - a) / width));
            const double step = (b - a) / npan;
            for (int p = 0; p < npan; ++p) {
                const double e0 = a + step * p, e1 = (p == npan - 1) ? b : a + step * (p + 1);
                const double mid = (e0 + e1) / 2, h = e1 - e0;
                for (int q = 0; q < 8; ++q) {
                    nodes.push_back(mid + h / 2 * gx[q]);
                    weights.push_back(h / 2 * gw[q]);
                }
            }
        }
        band_off.push_back((int) nodes.size());
    }
    const int n_nodes = (int) nodes.size();
    std::vector<double> trk(n_tables);
    for (int t = 0; t < n_tables; ++t) trk[t] = kSpeedOfLight / r_fwhm[t] / kOneSigma2Fwhm;

    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return LQG_ERR_CUDA;
    struct StreamGuard { cudaStream_t s; ~StreamGuard() { cudaStreamDestroy(s); } } guard{st};
    DevMem d_nodes, d_weights, d_off, d_tdv, d_trk, d_wt, d_deriv;
    const size_t deriv_n = (size_t) n_tables * nk * nv;
    if (d_nodes.alloc(n_nodes * 8) || d_weights.alloc(n_nodes * 8) || d_off.alloc((nk + 1) * 4) ||
        d_tdv.alloc(n_tables * 8) || d_trk.alloc(n_tables * 8) || d_wt.alloc((size_t) n_tables * n_nodes * 8) ||
        d_deriv.alloc(deriv_n * 8))
        return LQG_ERR_NOMEM;
    cudaMemcpyAsync(d_nodes.p, nodes.data(), n_nodes * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_weights.p, weights.data(), n_nodes * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_off.p, band_off.data(), (nk + 1) * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_tdv.p, dv, n_tables * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_trk.p, trk.data(), n_tables * 8, cudaMemcpyHostToDevice, st);
    k_tab_weights<<<dim3(std::max(1, std::min(64, (n_nodes + 255) / 256)), n_tables), 256, 0, st>>>(
        d_nodes.as<double>(), d_weights.as<double>(), n_nodes, d_tdv.as<double>(), d_trk.as<double>(), n_tables,
        d_wt.as<double>());
    const double dv_grid = v_length / (nv - 1.);
    k_tab_deriv<<<dim3((nv + 127) / 128, nk, n_tables), 128, 0, st>>>(
        d_nodes.as<double>(), d_wt.as<double>(), d_off.as<int>(), n_nodes, nk, nv, dv_grid, d_deriv.as<double>());
    if (cudaMemcpyAsync(deriv, d_deriv.p, deriv_n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return LQG_ERR_CUDA;

    if (with_signal) {
        // RealField(nrft, dv_table / RFT_M): core/sq_table.cpp:222-228, mathtools/real_field.cpp:46-56
        const int nrft = (int) std::exp2(std::ceil(std::log2(2.0 * kRftM * nv)) + 1);
        const int N = nrft / 2;
        const double length = (dv_grid / kRftM) * nrft;
        const double z1 = bins->z_centers[0] - bins->z_bin_width;
        const double lenz = bins->z_bin_width * (bins->nz + 1);
        std::vector<double> zs(nzp);
        for (int j = 0; j < nzp; ++j) zs[j] = z1 + lenz / (nzp - 1.) * j;
        // transforms in groups of tables: at most ~1 GiB of complex buffers
        const int per_table = nzp;
        const size_t tr_bytes = (size_t) N * sizeof(double2);
        const int group = (int) std::max<size_t>(1, std::min<size_t>(n_tables, (512ull << 20) / (tr_bytes * per_table)));
        DevMem d_z, d_a, d_b, d_sig;
        const size_t sig_n = (size_t) n_tables * nv * nzp;
        if (d_z.alloc(nzp * 8) || d_a.alloc(tr_bytes * per_table * group) || d_b.alloc(tr_bytes * per_table * group) ||
            d_sig.alloc(sig_n * 8))
            return LQG_ERR_NOMEM;
        cudaMemcpyAsync(d_z.p, zs.data(), nzp * 8, cudaMemcpyHostToDevice, st);
        const Pd13 p{fid[0], fid[1], fid[2], fid[3], fid[4], fid[5]};
        const int gx_blocks = std::max(1, std::min(1024, (N / 2 + 255) / 256));
        for (int t0 = 0; t0 < n_tables; t0 += group) {
            const int ng = std::min(group, n_tables - t0), batch = ng * per_table;
            k_tab_spectrum<<<dim3(gx_blocks, batch), 256, 0, st>>>(nrft, length, d_tdv.as<double>(),
                                                                   d_trk.as<double>(), t0, d_z.as<double>(), nzp, p,
                                                                   d_a.as<double2>());
            double2 *src = d_a.as<double2>(), *dst = d_b.as<double2>();
            for (int ns = 1; ns < N; ns *= 2) {
                k_tab_fft_pass<<<dim3(gx_blocks, batch), 256, 0, st>>>(src, dst, N, ns);
                std::swap(src, dst);
            }
            k_tab_signal<<<dim3(std::max(1, (nv + 255) / 256), batch), 256, 0, st>>>(
                src, N, nv, nzp, 1.0 / length, t0, d_sig.as<double>());
        }
        if (cudaMemcpyAsync(signal, d_sig.p, sig_n * 8, cudaMemcpyDeviceToHost, st) != cudaSuccess)
            return LQG_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return LQG_ERR_CUDA;   // before the buffers go
    }
    if (cudaStreamSynchronize(st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return LQG_ERR_CUDA;
    return LQG_OK;
}
