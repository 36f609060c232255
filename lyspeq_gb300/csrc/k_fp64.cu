// Per-chunk QMLE kernels: matrix build, FP64 factorisation, FP64 products,
// trace reductions.  Matrices are ld x ld row-major (ld = n rounded up to 64);
// rows/columns >= n are padding (zero, identity on the diagonal of C~).
//
// Formulation.  The reference forms M = diag(ivar) C + I, inverts it by LU
// and right-scales by diag(ivar) (core/chunk_estimate.cpp:693-711).  Here
// C~ = D C D + I with D = diag(sqrt(ivar)) is factored by Cholesky and
// C^-1 = D C~^-1 D, the same matrix: (diag(ivar) C + I)^-1 diag(ivar)
// = D (D C D + I)^-1 D.  C~ is SPD for any ivar >= 0 and masked pixels
// (ivar = 0) get exact zero rows and columns in C^-1, as in the reference.
#include "lqg_internal.cuh"

#include <cfloat>

namespace lqg {

namespace {

constexpr int T64 = 64;   // tile edge of the element-wise kernels

__device__ __forceinline__ const ChunkDesc &chunk_of(const WaveArgs &a, int c) { return a.chunks[c]; }

template <class T> __device__ __forceinline__ T *ws_ptr(const WaveArgs &a, int64_t off) {
    return reinterpret_cast<T *>(a.ws + off);
}

// Velocity and redshift separations of pixels a <= b, as Chunk::_setVZMatrices
// (core/chunk_estimate.cpp:384-398), from per-pixel log(lambda) and sqrt(lambda).
__device__ __forceinline__ void vz_of(const double *logw, const double *sqw, int a, int b,
                                      double &v, double &z) {
    v = kSpeedOfLight * (logw[b] - logw[a]);
    z = sqw[a] * sqw[b] - 1.0;
}

// DiscreteInterpolation2D::evaluate (mathtools/discrete_interpolation.cpp:221-242),
// x = z (fastest), y = v.
__device__ __forceinline__ double signal_at(const double *tab, const TableGrid &g, double z,
                                            double v) {
    double xx = (z - g.z1) / g.dz, yy = (v - g.v1) / g.dv;
    int nx = (int) xx, ny = (int) yy;
    nx = nx < 0 ? 0 : (nx >= g.nzp - 1 ? g.nzp - 2 : nx);
    ny = ny < 0 ? 0 : (ny >= g.nv - 1 ? g.nv - 2 : ny);
    size_t ind = (size_t) nx + (size_t) g.nzp * ny;
    double dnx = xx - nx, dny = yy - ny;
    return tab[ind] * (1 - dnx) * (1 - dny) + tab[ind + 1] * dnx * (1 - dny)
         + tab[ind + g.nzp] * (1 - dnx) * dny + tab[ind + g.nzp + 1] * dnx * dny;
}

// Redshift weight of bin zm at z, element-wise form of bins::zBinTriangular1/2,
// zBinTriangular and zBinTopHat (core/global_numbers.cpp:393-471).
__device__ __forceinline__ double zweight(const DeviceBins &b, int zm, double z) {
    double zc = b.z_centers[zm], dz = b.dz;
    if (!b.triangular || b.nz == 1)
        return (z >= zc - dz / 2 && z <= zc + dz / 2) ? 1.0 : 0.0;
    if (zm == 0 && z < zc) return 1.0;
    if (zm == b.nz - 1 && z > zc) return 1.0;
    if (z >= zc - dz && z <= zc + dz) return 1.0 - fabs(z - zc) / dz;
    return 0.0;
}

// Linear interpolation of a derivative table row (discrete_interpolation.cpp:61-72);
// index and weight are shared by all k bands at one v.
__device__ __forceinline__ void vindex(const TableGrid &g, double v, int &n, double &dn) {
    double xx = (v - g.v1) / g.dv;
    n = (int) xx;
    n = n < 0 ? 0 : (n >= g.nv - 1 ? g.nv - 2 : n);
    dn = xx - n;
}

__device__ __forceinline__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int) (blockDim.x >> 5); ++i) s += red[i];
    return s;  // valid on thread 0
}

__device__ __forceinline__ double block_max(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int i = 0; i < (int) (blockDim.x >> 5); ++i) s = fmax(s, red[i]);
        red[32] = s;
    }
    __syncthreads();
    return red[32];
}

// ---------------------------------------------------------------------------
// K1a: S_fid and C~ = D (S + sum_s theta_s Q_s) D + I.
__global__ void k_build_s_c(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = chunk_of(a, c);
    const int ld = ch.ld, n = ch.n;
    const int tiles_per_row = ld / T64;
    if ((int) blockIdx.x >= tiles_per_row * tiles_per_row) return;
    const int ti = blockIdx.x / tiles_per_row, tj = blockIdx.x % tiles_per_row;
    double *S = ws_ptr<double>(a, ch.o_s), *C = ws_ptr<double>(a, ch.o_c);
    const double *logw = a.logw + ch.pix, *sqw = a.sqw + ch.pix, *iv = a.ivar + ch.pix;
    const double *stab = a.signal ? a.signal + (size_t) ch.res * a.grid.nv * a.grid.nzp : nullptr;
    const DeviceBins &bins = *a.bins;
    const bool use_theta = a.theta != nullptr;
    for (int e = threadIdx.x; e < T64 * T64; e += blockDim.x) {
        int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        size_t idx = (size_t) i * ld + j;
        if (i >= n || j >= n) {
            S[idx] = 0.0;
            C[idx] = (i == j) ? 1.0 : 0.0;
            continue;
        }
        int lo = i < j ? i : j, hi = i < j ? j : i;
        double v, z;
        vz_of(logw, sqw, lo, hi, v, z);
        double s = (stab && !a.turn_off_sfid) ? signal_at(stab, a.grid, z, v) : 0.0;
        S[idx] = s;
        double cv = a.turn_off_sfid ? 0.0 : s;
        if (use_theta) {
            int nidx;
            double dn;
            vindex(a.grid, v, nidx, dn);
            for (int sl = 0; sl < ch.ns; ++sl) {
                int iz = sl / ch.kbin_upp, kn = sl % ch.kbin_upp;
                int ikz = iz * bins.nk + kn;
                double th = a.theta[ch.fis + ikz];
                if (th == 0.0) continue;
                const double *row = a.deriv + ((size_t) ch.res * bins.nk + kn) * a.grid.nv;
                double q = row[nidx] * (1 - dn) + row[nidx + 1] * dn;
                q *= zweight(bins, ch.zb0 + iz, z);
                cv += th * q;
            }
        }
        double di = sqrt(iv[i]), dj = sqrt(iv[j]);
        C[idx] = di * cv * dj + (i == j ? 1.0 : 0.0);
    }
}

// ---------------------------------------------------------------------------
// K2: Cholesky C~ = L L^T, L^-1, C~^-1 = L^-T L^-1, C^-1 = D C~^-1 D,
// continuum marginalisation, y = C^-1 delta.  One CTA per chunk; FP64.
constexpr int NB = 32;
constexpr int FT = 256;   // threads of the factorisation kernel

__device__ void potrf_lower(double *A, int ld, int n32, double *sm, int *status) {
    double *Ld = sm;                  // 32 x 33
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int k0 = 0; k0 < n32; k0 += NB) {
        // (a) diagonal block, one warp: lane r keeps row r
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x)
            Ld[(e / NB) * 33 + e % NB] = A[(size_t) (k0 + e / NB) * ld + k0 + e % NB];
        __syncthreads();
        if (threadIdx.x < 32) {
            int r = threadIdx.x;
            double row[NB];
#pragma unroll
            for (int l = 0; l < NB; ++l) row[l] = Ld[r * 33 + l];
            bool ok = true;
#pragma unroll
            for (int j = 0; j < NB; ++j) {
                double piv = __shfl_sync(0xffffffffu, row[j], j);
                if (!(piv > 0.0) || !isfinite(piv)) ok = false;
                double ljj = sqrt(piv > 0.0 ? piv : 1.0);
                double lij = (r == j) ? ljj : (r > j ? row[j] / ljj : 0.0);
                row[j] = lij;
#pragma unroll
                for (int l = j + 1; l < NB; ++l) {
                    double llj = __shfl_sync(0xffffffffu, lij, l);
                    if (r >= l) row[l] -= lij * llj;
                }
            }
#pragma unroll
            for (int l = 0; l < NB; ++l) Ld[r * 33 + l] = (l <= r) ? row[l] : 0.0;
            if (!ok && r == 0) bad = 1;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x)
            A[(size_t) (k0 + e / NB) * ld + k0 + e % NB] = Ld[(e / NB) * 33 + e % NB];
        // (b) panel: L[i, k0:k0+32] = A[i, k0:k0+32] Ld^-T, one row per thread
        for (int i = k0 + NB + threadIdx.x; i < n32; i += blockDim.x) {
            double x[NB];
            double *Ai = A + (size_t) i * ld + k0;
#pragma unroll
            for (int cidx = 0; cidx < NB; ++cidx) {
                double s = Ai[cidx];
#pragma unroll
                for (int l = 0; l < cidx; ++l) s -= x[l] * Ld[cidx * 33 + l];
                x[cidx] = s / Ld[cidx * 33 + cidx];
            }
#pragma unroll
            for (int cidx = 0; cidx < NB; ++cidx) Ai[cidx] = x[cidx];
        }
        __syncthreads();
        // (c) trailing update of the lower triangle, 32x32 tiles, 2x2 per thread
        const int m0 = k0 + NB, nt = (n32 - m0) / NB;
        for (int ti = 0; ti < nt; ++ti)
        for (int tj = 0; tj <= ti; ++tj) {
            int i0 = m0 + ti * NB, j0 = m0 + tj * NB;
            int r = (threadIdx.x / 16) * 2, cc = (threadIdx.x % 16) * 2;
            double acc00 = 0, acc01 = 0, acc10 = 0, acc11 = 0;
            const double *Pi0 = A + (size_t) (i0 + r) * ld + k0, *Pi1 = Pi0 + ld;
            const double *Pj0 = A + (size_t) (j0 + cc) * ld + k0, *Pj1 = Pj0 + ld;
#pragma unroll 8
            for (int l = 0; l < NB; ++l) {
                double a0 = Pi0[l], a1 = Pi1[l], b0 = Pj0[l], b1 = Pj1[l];
                acc00 += a0 * b0; acc01 += a0 * b1; acc10 += a1 * b0; acc11 += a1 * b1;
            }
            double *T0 = A + (size_t) (i0 + r) * ld + j0 + cc, *T1 = T0 + ld;
            T0[0] -= acc00; T0[1] -= acc01; T1[0] -= acc10; T1[1] -= acc11;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0 && bad) *status = LQG_CHUNK_NOT_SPD;
    __syncthreads();
}

// In-place inverse of the lower triangular L (row blocks top to bottom).
// X[I, 0:I0] = -Ld_I^-1 (L[I, 0:I0] X[0:I0, 0:I0]), X[I, I] = Ld_I^-1.
__device__ void trtri_lower(double *A, int ld, int n32, double *scratch, double *sm) {
    double *Ld = sm;              // 32 x 33 diagonal block
    double *Xd = sm + NB * 33;    // 32 x 33 its inverse
    for (int I0 = 0; I0 < n32; I0 += NB) {
        // T = L[I, 0:I0] X[0:I0, 0:I0] into scratch (32 x I0); X lower: l >= c
        for (int e = threadIdx.x; e < NB * I0; e += blockDim.x) {
            int r = e / I0, c = e % I0;
            const double *Lr = A + (size_t) (I0 + r) * ld;
            double s = 0;
            for (int l = c; l < I0; ++l) s += Lr[l] * A[(size_t) l * ld + c];
            scratch[(size_t) r * I0 + c] = s;
        }
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x)
            Ld[(e / NB) * 33 + e % NB] = A[(size_t) (I0 + e / NB) * ld + I0 + e % NB];
        __syncthreads();
        // Xd = Ld^-1: column c solved by one thread
        if (threadIdx.x < NB) {
            int c = threadIdx.x;
            double x[NB];
#pragma unroll
            for (int r = 0; r < NB; ++r) {
                double s = (r == c) ? 1.0 : 0.0;
#pragma unroll
                for (int l = 0; l < r; ++l) s -= Ld[r * 33 + l] * x[l];
                x[r] = (r < c) ? 0.0 : s / Ld[r * 33 + r];
            }
#pragma unroll
            for (int r = 0; r < NB; ++r) Xd[r * 33 + c] = x[r];
        }
        __syncthreads();
        // X[I, c] = -Xd T[:, c]
        for (int e = threadIdx.x; e < NB * I0; e += blockDim.x) {
            int r = e / I0, c = e % I0;
            double s = 0;
            for (int l = 0; l <= r; ++l) s += Xd[r * 33 + l] * scratch[(size_t) l * I0 + c];
            A[(size_t) (I0 + r) * ld + c] = -s;
        }
        for (int e = threadIdx.x; e < NB * NB; e += blockDim.x)
            A[(size_t) (I0 + e / NB) * ld + I0 + e % NB] = Xd[(e / NB) * 33 + e % NB];
        __syncthreads();
    }
}

// C~^-1 = X^T X (X = L^-1 lower) in place, then C^-1 = D C~^-1 D, symmetric.
__device__ void lauum_scale(double *A, int ld, int n32, int n, const double *ivar) {
    const int nt = n32 / NB;
    for (int ti = 0; ti < nt; ++ti) {
        // tiles (ti, tj), tj < ti first, then the diagonal tile
        for (int pass = 0; pass < 2; ++pass) {
            int tj_lo = pass == 0 ? 0 : ti, tj_hi = pass == 0 ? ti : ti + 1;
            for (int tj = tj_lo; tj < tj_hi; ++tj) {
                int i0 = ti * NB, j0 = tj * NB;
                int r = (threadIdx.x / 16) * 2, cc = (threadIdx.x % 16) * 2;
                double acc[2][2] = {{0, 0}, {0, 0}};
                for (int l = i0; l < n32; ++l) {
                    const double *Xl = A + (size_t) l * ld;
                    double a0 = (l >= i0 + r) ? Xl[i0 + r] : 0.0;
                    double a1 = (l >= i0 + r + 1) ? Xl[i0 + r + 1] : 0.0;
                    double b0 = (l >= j0 + cc) ? Xl[j0 + cc] : 0.0;
                    double b1 = (l >= j0 + cc + 1) ? Xl[j0 + cc + 1] : 0.0;
                    acc[0][0] += a0 * b0; acc[0][1] += a0 * b1;
                    acc[1][0] += a1 * b0; acc[1][1] += a1 * b1;
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < 2; ++u)
#pragma unroll
                    for (int w = 0; w < 2; ++w) {
                        int i = i0 + r + u, j = j0 + cc + w;
                        if (j <= i) A[(size_t) i * ld + j] = acc[u][w];
                    }
                __syncthreads();
            }
        }
    }
    // scale and mirror; padding rows/cols -> 0
    for (size_t e = threadIdx.x; e < (size_t) ld * ld; e += blockDim.x) {
        int i = (int) (e / ld), j = (int) (e % ld);
        if (j > i) continue;
        double v = 0.0;
        if (i < n && j < n) v = sqrt(ivar[i]) * A[e] * sqrt(ivar[j]);
        A[e] = v;
        A[(size_t) j * ld + i] = v;
    }
    __syncthreads();
}

// Continuum marginalisation, Chunk::_addMarginalizations (core/chunk_estimate.cpp:576-665):
// template vectors, orthonormalised (their SVD is computed here from the r x r Gram
// matrix by Jacobi rotations), removed one by one by Sherman-Morrison.
__device__ void marginalize(double *A, int ld, int n, const double *wave, int logl, int lord,
                            double *smv /* >= (kMaxContVecs + 1) * ld */, double *red) {
    int nv = 0;
    double *V = smv;
    double *y = smv + kMaxContVecs * ld;
    // build unit vectors
    for (int i = threadIdx.x; i < n; i += blockDim.x) V[i] = 1.0 / sqrt((double) n);
    nv = 1;
    __shared__ double norm_s;
    for (int kind = 0; kind < 2; ++kind) {
        int order = kind == 0 ? logl : lord;
        for (int cmo = 1; cmo <= order && nv < kMaxContVecs; ++cmo) {
            double part = 0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double x = kind == 0 ? pow(log(wave[i]), (double) cmo) : pow(wave[i], (double) cmo);
                V[nv * ld + i] = x;
                part += x * x;
            }
            double s = block_sum(part, red);
            if (threadIdx.x == 0) norm_s = 1.0 / sqrt(s);
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x) V[nv * ld + i] *= norm_s;
            ++nv;
            __syncthreads();
        }
    }
    // One-sided Jacobi SVD of V (n x nv): rotate column pairs until they are
    // orthogonal; the column norms are then the singular values and the
    // normalised columns the left singular vectors (the reference takes them
    // from LAPACKE_dgesvd, mathtools/matrix_helper.cpp:437-447).  Working on V
    // directly keeps the accuracy of small singular values, which matter when
    // the templates are close to collinear.
    __shared__ double sv[kMaxContVecs], rot[2];
    __shared__ int order[kMaxContVecs], nuse_s, changed;
    for (int sweep = 0; sweep < 60; ++sweep) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int p = 0; p < nv; ++p)
            for (int q = p + 1; q < nv; ++q) {
                double app = 0, aqq = 0, apq = 0;
                for (int i = threadIdx.x; i < n; i += blockDim.x) {
                    double x = V[p * ld + i], y2 = V[q * ld + i];
                    app += x * x; aqq += y2 * y2; apq += x * y2;
                }
                app = block_sum(app, red);
                __syncthreads();
                aqq = block_sum(aqq, red);
                __syncthreads();
                apq = block_sum(apq, red);
                if (threadIdx.x == 0) {
                    rot[0] = 1.0; rot[1] = 0.0;
                    if (fabs(apq) > 1e-15 * sqrt(app * aqq)) {
                        double zeta = (aqq - app) / (2.0 * apq);
                        double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                        double cs = 1.0 / sqrt(1.0 + t * t);
                        rot[0] = cs; rot[1] = cs * t;
                        changed = 1;
                    }
                }
                __syncthreads();
                double cs = rot[0], sn = rot[1];
                if (sn != 0.0)
                    for (int i = threadIdx.x; i < n; i += blockDim.x) {
                        double x = V[p * ld + i], y2 = V[q * ld + i];
                        V[p * ld + i] = cs * x - sn * y2;
                        V[q * ld + i] = sn * x + cs * y2;
                    }
                __syncthreads();
            }
        if (!changed) break;
    }
    for (int p = 0; p < nv; ++p) {
        double part = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) part += V[p * ld + i] * V[p * ld + i];
        double s = block_sum(part, red);
        if (threadIdx.x == 0) sv[p] = sqrt(s);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        for (int p = 0; p < nv; ++p) order[p] = p;
        for (int p = 0; p < nv; ++p)
            for (int q = p + 1; q < nv; ++q)
                if (sv[order[q]] > sv[order[p]]) { int t = order[p]; order[p] = order[q]; order[q] = t; }
        int nuse = nv;
        while (nuse > 0 && !(sv[order[nuse - 1]] / sv[order[0]] > kDoubleEpsilon)) --nuse;
        nuse_s = nuse;
    }
    __syncthreads();
    const int nuse = nuse_s;
    double *U = y + ld;  // nuse x ld left singular vectors
    for (int u = 0; u < nuse; ++u) {
        int p = order[u];
        double inv = 1.0 / sv[p];
        for (int i = threadIdx.x; i < n; i += blockDim.x) U[u * ld + i] = V[p * ld + i] * inv;
    }
    __syncthreads();
    __shared__ double cnorm;
    for (int u = 0; u < nuse; ++u) {
        const double *vv = U + u * ld;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            double s = 0;
            const double *Ai = A + (size_t) i * ld;
            for (int j = 0; j < n; ++j) s += Ai[j] * vv[j];
            y[i] = s;
        }
        __syncthreads();
        double part = 0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) part += vv[i] * y[i];
        double s = block_sum(part, red);
        if (threadIdx.x == 0) cnorm = -1.0 / s;
        __syncthreads();
        for (size_t e = threadIdx.x; e < (size_t) n * ld; e += blockDim.x) {
            int i = (int) (e / ld), j = (int) (e % ld);
            if (j < n) A[e] += cnorm * y[i] * y[j];
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(FT) k_factor(WaveArgs a) {
    const int c = blockIdx.x;
    const ChunkDesc &ch = chunk_of(a, c);
    if (a.status[c] != LQG_CHUNK_OK) return;
    if (!LQG_IN_BOUNDS(a, ch.o_c + (int64_t) ch.ld * ch.ld * 8 <= a.ws_bytes &&
                              ch.o_part + 40 * (int64_t) ch.ld * 8 <= a.ws_bytes &&
                              ch.o_y + (int64_t) ch.ld * 8 <= a.ws_bytes, 7, c, ch.o_part))
        return;
    const int ld = ch.ld, n = ch.n, n32 = (n + NB - 1) / NB * NB;
    double *A = ws_ptr<double>(a, ch.o_c);
    double *scratch = ws_ptr<double>(a, ch.o_part);   // >= 32 * ld + (kMaxContVecs + 2) * ld doubles
    __shared__ double sm[2 * NB * 33];
    __shared__ double red[40];
    potrf_lower(A, ld, n32, sm, &a.status[c]);
    __syncthreads();
    if (a.status[c] != LQG_CHUNK_OK) return;
    trtri_lower(A, ld, n32, scratch, sm);
    __syncthreads();
    lauum_scale(A, ld, n32, n, a.ivar + ch.pix);
    int nvec_req = 0;
    if (a.cont_logl >= 0 || a.cont_l >= 0)
        nvec_req = 1 + (a.cont_logl > 0 ? a.cont_logl : 0) + (a.cont_l > 0 ? a.cont_l : 0);
    if (nvec_req > 0)
        marginalize(A, ld, n, a.wave + ch.pix, a.cont_logl, a.cont_l, scratch, red);
    // y = C^-1 delta (full symmetric matrix)
    double *y = ws_ptr<double>(a, ch.o_y);
    const double *dl = a.delta + ch.pix;
    for (int i = threadIdx.x; i < ld; i += blockDim.x) {
        double s = 0;
        if (i < n) {
            const double *Ai = A + (size_t) i * ld;
            for (int j = 0; j < n; ++j) s += Ai[j] * dl[j];
        }
        y[i] = s;
    }
    // scale bounds for the mixed path: max |C^-1| and max row sum of |C^-1|
    double mx = 0, rs = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double *Ai = A + (size_t) i * ld;
        double r = 0;
        for (int j = 0; j < n; ++j) { double v = fabs(Ai[j]); r += v; mx = fmax(mx, v); }
        rs = fmax(rs, r);
    }
    double gmx = block_max(mx, red);
    double grs = block_max(rs, red);
    if (threadIdx.x == 0) {
        double *sc = a.scales + 4 * c;
        sc[0] = gmx;
        sc[1] = grs;
    }
}

// ---------------------------------------------------------------------------
// K1b: stored derivative matrices Q_s (Chunk::_setQiMatrix + _applyRedshiftInterp,
// core/chunk_estimate.cpp:429-536), written as FP64 or as fp16 hi/lo planes, and
// the per-tile partial sums of d_s = y^T Q_s y (computePSbeforeFvector :754-759).
template <bool MIXED>
__global__ void k_build_q(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = chunk_of(a, c);
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    __shared__ double red[40];
    if (a.status[c] != LQG_CHUNK_OK) return;
    const DeviceBins &bins = *a.bins;
    const double *logw = a.logw + ch.pix, *sqw = a.sqw + ch.pix;
    const double *y = ws_ptr<double>(a, ch.o_y);
    constexpr int EPT = T64 * T64 / 256;   // elements per thread
    int nidx[EPT], ii[EPT], jj[EPT];
    double dn[EPT], zz[EPT], yy[EPT];
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
        int e = threadIdx.x + u * 256;
        int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        ii[u] = i; jj[u] = j;
        if (i < n && j < n) {
            int lo = i < j ? i : j, hi = i < j ? j : i;
            double v, z;
            vz_of(logw, sqw, lo, hi, v, z);
            vindex(a.grid, v, nidx[u], dn[u]);
            zz[u] = z;
            yy[u] = y[i] * y[j];
        } else {
            nidx[u] = -1; dn[u] = 0; zz[u] = 0; yy[u] = 0;
        }
    }
    double *dpart = ws_ptr<double>(a, ch.o_dpart) + (size_t) blockIdx.x * ch.ns;
    for (int s = 0; s < ch.ns; ++s) {
        const int iz = s / ch.kbin_upp, kn = s % ch.kbin_upp;
        const double *row = a.deriv + ((size_t) ch.res * bins.nk + kn) * a.grid.nv;
        const int zm = ch.zb0 + iz;
        double part = 0;
        double qs = MIXED ? a.scales[(size_t) 4 * a.n_chunks + ch.slot_q + s] : 0.0;
#pragma unroll
        for (int u = 0; u < EPT; ++u) {
            double q = 0.0;
            if (nidx[u] >= 0) {
                q = row[nidx[u]] * (1 - dn[u]) + row[nidx[u] + 1] * dn[u];
                q *= zweight(bins, zm, zz[u]);
                part += yy[u] * q;
            }
            size_t off = (size_t) (ch.slot_q + s) * ld * ld + (size_t) ii[u] * ld + jj[u];
            if (MIXED) {
                if (!LQG_IN_BOUNDS(a, off < (size_t) a.total_slots_q * ld * ld, 5, c, off)) continue;
                float xs = (float) (q * qs);
                __half h = __float2half_rn(xs);
                a.q_hi[off] = h;
                a.q_lo[off] = __float2half_rn(xs - __half2float(h));
            } else {
                ws_ptr<double>(a, ch.o_q)[(size_t) s * ld * ld + (size_t) ii[u] * ld + jj[u]] = q;
            }
        }
        double tot = block_sum(part, red);
        if (threadIdx.x == 0) dpart[s] = tot;
    }
}

// Mixed path: C^-1 and S to fp16 hi/lo planes, W_N = N C^-1 into its P slot.
__global__ void k_prep_mixed(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = chunk_of(a, c);
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr || a.status[c] != LQG_CHUNK_OK) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    const double *A = ws_ptr<double>(a, ch.o_c), *S = ws_ptr<double>(a, ch.o_s);
    const double *iv = a.ivar + ch.pix;
    const double *sc = a.scales + 4 * c;
    const double cs = sc[2], ws = sc[3];
    const double ss = a.scales[(size_t) 4 * a.n_chunks + ch.slot_q + ch.ns];
    for (int e = threadIdx.x; e < T64 * T64; e += blockDim.x) {
        int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        size_t idx = (size_t) i * ld + j;
        double cv = A[idx];
        float x = (float) (cv * cs);
        __half h = __float2half_rn(x);
        size_t coff = (size_t) c * ld * ld + idx;
        if (!LQG_IN_BOUNDS(a, coff < (size_t) a.n_chunks * ld * ld &&
                                  (size_t) (ch.slot_q + ch.ns) * ld * ld + idx < (size_t) a.total_slots_q * ld * ld &&
                                  (size_t) (ch.slot_p + ch.ns + 1) * ld * ld + idx < (size_t) a.total_slots_p * ld * ld,
                           6, c, coff))
            continue;
        a.c_hi[coff] = h;
        a.c_lo[coff] = __float2half_rn(x - __half2float(h));
        float xs = (float) (S[idx] * ss);
        __half hs = __float2half_rn(xs);
        size_t soff = (size_t) (ch.slot_q + ch.ns) * ld * ld + idx;
        a.q_hi[soff] = hs;
        a.q_lo[soff] = __float2half_rn(xs - __half2float(hs));
        double nw = (i < n && iv[i] != 0.0) ? 1.0 / iv[i] : 0.0;
        float xw = (float) (nw * cv * ws);
        __half hw = __float2half_rn(xw);
        size_t poff = (size_t) (ch.slot_p + ch.ns + 1) * ld * ld + idx;
        a.p_hi[poff] = hw;
        a.p_lo[poff] = __float2half_rn(xw - __half2float(hw));
    }
}

// FP64 path: W_N = N C^-1 (core/chunk_estimate.cpp:767-781) into its P slot.
__global__ void k_wn_fp64(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = chunk_of(a, c);
    const int ld = ch.ld, n = ch.n;
    if (a.status[c] != LQG_CHUNK_OK) return;
    const double *A = ws_ptr<double>(a, ch.o_c);
    const double *iv = a.ivar + ch.pix;
    double *P = ws_ptr<double>(a, ch.o_p) + (size_t) (ch.ns + 1) * ld * ld;
    for (size_t e = (size_t) blockIdx.x * blockDim.x + threadIdx.x; e < (size_t) ld * ld;
         e += (size_t) gridDim.x * blockDim.x) {
        int i = (int) (e / ld);
        double nw = (i < n && iv[i] != 0.0) ? 1.0 / iv[i] : 0.0;
        P[e] = nw * A[e];
    }
}

// ---------------------------------------------------------------------------
// K4 (FP64): A_s = C^-1 Q_s (s < ns) and A_S = C^-1 S; epilogue writes A_s to R
// (row-major) and A_s^T to P.  64x64 output tiles, 256 threads, 4x4 per thread.
constexpr int GT = 64, GK = 16;

__global__ void __launch_bounds__(256) k_dgemm(WaveArgs a, const int *jobs, int njobs) {
    const int job = blockIdx.y;
    if (job >= njobs) return;
    const int c = jobs[2 * job], s = jobs[2 * job + 1];
    const ChunkDesc &ch = chunk_of(a, c);
    if (a.status[c] != LQG_CHUNK_OK) return;
    const int ld = ch.ld, tpr = ld / GT;
    if ((int) blockIdx.x >= tpr * tpr) return;
    const int tm = blockIdx.x / tpr, tn = blockIdx.x % tpr;
    const double *A = ws_ptr<double>(a, ch.o_c);
    const double *B = (s < ch.ns) ? ws_ptr<double>(a, ch.o_q) + (size_t) s * ld * ld
                                  : ws_ptr<double>(a, ch.o_s);
    // operand tiles during the K loop, the output tile (for the transposed
    // store) afterwards: 64 x 65 doubles = 33 KB
    __shared__ double smem[GT * (GT + 1)];
    double (*As)[GT + 1] = reinterpret_cast<double (*)[GT + 1]>(smem);
    double (*Bs)[GT + 1] = reinterpret_cast<double (*)[GT + 1]>(smem + GK * (GT + 1));
    double (*Ot)[GT + 1] = reinterpret_cast<double (*)[GT + 1]>(smem);
    const int tr = (threadIdx.x / 16) * 4, tc = (threadIdx.x % 16) * 4;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < ld; k0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += blockDim.x) {
            int r = e / GK, kk = e % GK;
            As[kk][r] = A[(size_t) (tm * GT + r) * ld + k0 + kk];
            int kk2 = e / GT, cc = e % GT;
            Bs[kk2][cc] = B[(size_t) (k0 + kk2) * ld + tn * GT + cc];
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < GK; ++kk) {
            double av[4], bv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { av[u] = As[kk][tr + u]; bv[u] = Bs[kk][tc + u]; }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) acc[u][w] += av[u] * bv[w];
        }
        __syncthreads();
    }
    double *R = ws_ptr<double>(a, ch.o_r) + (size_t) s * ld * ld;
    double *P = ws_ptr<double>(a, ch.o_p) + (size_t) s * ld * ld;
    __syncthreads();   // the operand tiles are dead; Ot reuses their space
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            Ot[tr + u][tc + w] = acc[u][w];
            if (s < ch.ns) R[(size_t) (tm * GT + tr + u) * ld + tn * GT + tc + w] = acc[u][w];
        }
    __syncthreads();
    // transposed write: P[n][m] = A[m][n]
    for (int e = threadIdx.x; e < GT * GT; e += blockDim.x) {
        int nn = e / GT, mm = e % GT;
        P[(size_t) (tn * GT + nn) * ld + tm * GT + mm] = Ot[mm][nn];
    }
}

// K5 (FP64): Gram G[i][j] = <P_i, R_j> over a K split; rows i < ns + 2, cols j < ns.
constexpr int GR = 128;   // max rows / cols handled (ns + 2 <= 128)

__global__ void __launch_bounds__(256) k_dgram(WaveArgs a) {
    const int c = blockIdx.y, sp = blockIdx.x;
    const ChunkDesc &ch = chunk_of(a, c);
    if (a.status[c] != LQG_CHUNK_OK) return;
    const int64_t K = (int64_t) ch.ld * ch.ld;
    const int64_t kper = (K + a.gram_splits - 1) / a.gram_splits;
    const int64_t k_lo = sp * kper, k_hi = min(K, k_lo + kper);
    const int mi = ch.ns + 2, mj = ch.ns;
    const double *P = ws_ptr<double>(a, ch.o_p), *R = ws_ptr<double>(a, ch.o_r);
    __shared__ double Ps[8][GR + 1], Rs[8][GR + 1];
    const int tr = (threadIdx.x / 16) * 8, tc = (threadIdx.x % 16) * 8;
    double acc[8][8] = {};
    for (int64_t k0 = k_lo; k0 < k_hi; k0 += 8) {
        for (int e = threadIdx.x; e < GR * 8; e += blockDim.x) {
            int r = e / 8, kk = e % 8;
            int64_t k = k0 + kk;
            Ps[kk][r] = (r < mi && k < k_hi) ? P[(size_t) r * K + k] : 0.0;
            Rs[kk][r] = (r < mj && k < k_hi) ? R[(size_t) r * K + k] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
            double pv[8], rv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) { pv[u] = Ps[kk][tr + u]; rv[u] = Rs[kk][tc + u]; }
#pragma unroll
            for (int u = 0; u < 8; ++u)
#pragma unroll
                for (int w = 0; w < 8; ++w) acc[u][w] += pv[u] * rv[w];
        }
        __syncthreads();
    }
    double *out = ws_ptr<double>(a, ch.o_part) + (size_t) sp * GR * GR;
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int w = 0; w < 8; ++w) out[(tr + u) * GR + tc + w] = acc[u][w];
}

// ---------------------------------------------------------------------------
// K5b: per-chunk reduction of the Gram partials and d partials (fixed order)
// and the per-chunk results in the reference layout.
__global__ void k_finish(WaveArgs a, int mixed) {
    const int c = blockIdx.x;
    const ChunkDesc &ch = chunk_of(a, c);
    const DeviceBins &bins = *a.bins;
    const int nq = ch.nq;
    if (!LQG_IN_BOUNDS(a, ch.res_off + 3 * nq + (int64_t) nq * nq <= a.results_elems, 8, c, ch.res_off)) return;
    if (mixed && !LQG_IN_BOUNDS(a, (int64_t) (c + 1) * a.gram_splits * GR * GR <= a.gram_elems, 9, c, c)) return;
    double *res = a.results + ch.res_off;
    double *d = res, *b = res + nq, *t = res + 2 * nq, *F = res + 3 * nq;
    for (int e = threadIdx.x; e < 3 * nq + nq * nq; e += blockDim.x) res[e] = 0.0;
    __syncthreads();
    if (a.status[c] != LQG_CHUNK_OK) return;
    const int ns = ch.ns, tiles = (ch.ld / T64) * (ch.ld / T64);
    const double *dpart = ws_ptr<double>(a, ch.o_dpart);
    for (int s = threadIdx.x; s < ns; s += blockDim.x) {
        double acc = 0;
        for (int tl = 0; tl < tiles; ++tl) acc += dpart[(size_t) tl * ns + s];
        int ikz = (s / ch.kbin_upp) * bins.nk + s % ch.kbin_upp;
        d[ikz] = acc;
    }
    const int rows = ns + 2;
    for (int e = threadIdx.x; e < rows * ns; e += blockDim.x) {
        int i = e / ns, j = e % ns;
        double acc = 0;
        if (mixed) {
            const float *gp = a.gram_part + (size_t) c * a.gram_splits * GR * GR;
            for (int sp = 0; sp < a.gram_splits; ++sp) acc += (double) gp[(size_t) sp * GR * GR + i * GR + j];
            double si = a.scales[(size_t) 4 * a.n_chunks + a.total_slots_q + ch.slot_p + i];
            double sj = a.scales[(size_t) 4 * a.n_chunks + a.total_slots_q + a.total_slots_p + ch.slot_r + j];
            acc /= (si * sj);
        } else {
            const double *gp = ws_ptr<double>(a, ch.o_part);
            for (int sp = 0; sp < a.gram_splits; ++sp) acc += gp[(size_t) sp * GR * GR + i * GR + j];
        }
        int jkz = (j / ch.kbin_upp) * bins.nk + j % ch.kbin_upp;
        if (i < ns) {
            int ikz = (i / ch.kbin_upp) * bins.nk + i % ch.kbin_upp;
            if (ikz <= jkz && !a.skip_fisher) F[(size_t) ikz * nq + jkz] = acc;
        } else if (i == ns) {
            if (!a.turn_off_sfid) t[jkz] = acc;
        } else {
            b[jkz] = acc;
        }
    }
}

}  // namespace

void launch_build_s_c(WaveArgs &a, cudaStream_t st) {
    int tiles = (a.max_ld / T64) * (a.max_ld / T64);
    k_build_s_c<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
    a.launches++;
}

void launch_factor(WaveArgs &a, cudaStream_t st) {
    k_factor<<<a.n_chunks, FT, 0, st>>>(a);
    a.launches++;
}

void launch_build_q(WaveArgs &a, cudaStream_t st) {
    int tiles = (a.max_ld / T64) * (a.max_ld / T64);
    if (a.precision == LQG_PRECISION_MIXED) {
        k_prep_mixed<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
        k_build_q<true><<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
        a.launches += 2;
    } else {
        k_build_q<false><<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
        k_wn_fp64<<<dim3(64, a.n_chunks), 256, 0, st>>>(a);
        a.launches += 2;
    }
}

void launch_products_fp64(WaveArgs &a, cudaStream_t st, const int *d_jobs, int njobs) {
    int tiles = (a.max_ld / GT) * (a.max_ld / GT);
    k_dgemm<<<dim3(tiles, njobs), 256, 0, st>>>(a, d_jobs, njobs);
    if (a.mid_event) cudaEventRecord(a.mid_event, st);
    k_dgram<<<dim3(a.gram_splits, a.n_chunks), 256, 0, st>>>(a);
    a.launches += 2;
}

void launch_finish(WaveArgs &a, cudaStream_t st) {
    k_finish<<<a.n_chunks, 256, 0, st>>>(a, a.precision == LQG_PRECISION_MIXED);
    a.launches++;
}

}  // namespace lqg
