// Resolution-matrix path (UseResoMatrix): lyspeq evaluates the fiducial signal
// and the derivative matrices on the resolution matrix's grid and sandwiches
// them, M -> R M R^T (Chunk::_setFiducialSignalMatrix and _setQiMatrix,
// core/chunk_estimate.cpp:400-480; Resolution::sandwich,
// mathtools/matrix_helper.cpp:815-821, 877-903, 1075-1084).  The grid is the
// pixel grid for a diagonal (banded) matrix, or an oversampled grid linear in
// wavelength (Chunk::_initMatrices, core/chunk_estimate.cpp:927-938) for a
// matrix that Resolution::oversample has resampled.
//
// Host side: the per-spectrum preprocessing of the matrix (deconvolution and
// oversampling, core/one_qso_estimate.cpp:75-89).
// Device side: the S / C~ build of phase A and the Q_s build of phase B for
// chunks with a resolution matrix.  R is banded, row r having nelem weights at
// grid points r os + a - sh, so one 32 x 32 tile of R M R^T needs a block of
// at most 128 x 128 grid points of M.  The block is evaluated slab by slab into
// shared memory and contracted twice (T = M_block R_J^T, then R_I T): about
// 150 multiply-adds per output element for an x3-oversampled 11-diagonal
// matrix, and each grid point of M is evaluated once per tile.  Only tiles on
// or above the diagonal are computed; each writes its mirror tile too.
#include "lqg_internal.cuh"
#include "lqg_ff.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

// ---------------------------------------------------------------------------
// Host preprocessing

namespace {

// DiaMatrix::_getRowIndices (mathtools/matrix_helper.cpp:608-620): flat
// indices into values[ndiags][n] of row i, columns i - noff .. i + noff;
// entries beyond the matrix edge repeat the row's mirrored entry.
void dia_row_indices(int i, int n, int nd, std::vector<int> &idx) {
    const int noff = nd / 2;
    idx.clear();
    for (int j = nd - 1; j >= 0; --j) idx.push_back(j * n + (noff - j) + i);
    if (i < noff) {
        for (int j = 0; j < noff - i; ++j) idx[j] = idx[nd - 1 - j];
    } else if (i > n - noff - 1) {
        for (int j = 0; j < i - n + noff + 1; ++j) idx[nd - 1 - j] = idx[j];
    }
}

// Second derivatives of the natural cubic spline through (x, y).
void natural_spline(const std::vector<double> &x, const std::vector<double> &y, std::vector<double> &m) {
    const size_t n = x.size();
    m.assign(n, 0.0);
    if (n < 3) return;
    const size_t k = n - 2;
    std::vector<double> diag(k), upper(k), rhs(k);
    for (size_t j = 0; j < k; ++j) {
        const size_t i = j + 1;
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        diag[j] = 2.0 * (h0 + h1);
        upper[j] = h1;
        rhs[j] = 6.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
    }
    for (size_t j = 1; j < k; ++j) {
        const double f = (x[j + 1] - x[j]) / diag[j - 1];
        diag[j] -= f * upper[j - 1];
        rhs[j] -= f * rhs[j - 1];
    }
    m[k] = rhs[k - 1] / diag[k - 1];
    for (size_t j = k - 1; j-- > 0;) m[j + 1] = (rhs[j] - upper[j] * m[j + 2]) / diag[j];
}

double spline_eval(const std::vector<double> &x, const std::vector<double> &y, const std::vector<double> &m,
                   double t) {
    size_t lo = 0, hi = x.size() - 1;
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        if (x[mid] > t) hi = mid; else lo = mid;
    }
    const size_t i = lo;
    const double h = x[i + 1] - x[i], t1 = x[i + 1] - t, t0 = t - x[i];
    return (m[i] * t1 * t1 * t1 + m[i + 1] * t0 * t0 * t0) / (6.0 * h)
         + (y[i] / h - m[i] * h / 6.0) * t1 + (y[i + 1] / h - m[i + 1] * h / 6.0) * t0;
}

// nonzero_min_element (mathtools/matrix_helper.cpp:20-39): the smallest |x|
// above 1e-15 in the reference's scan order, at least 1e-15.
double nonzero_min_abs(const std::vector<double> &row) {
    double smallest = std::fabs(row[0]);
    for (size_t i = 1; i < row.size(); ++i) {
        const double tmp = std::fabs(row[i]);
        if (smallest < 1e-15) smallest = tmp;
        else if (tmp < smallest && tmp > 1e-15) smallest = tmp;
    }
    return smallest < 1e-15 ? 1e-15 : smallest;
}

}  // namespace

// DiaMatrix::deconvolve (mathtools/matrix_helper.cpp:653-682) with
// RealField::deconvolveSinc (mathtools/real_field.cpp:78-110): every row,
// zero-padded by 5 on each side, is divided by sinc(pi m k / size) in Fourier
// space (k >= 1).  The 21-point transforms are direct sums.
extern "C" int lqg_resomat_deconvolve(int n, int ndiags, double *values, double m) {
    if (n < 1 || ndiags < 1 || ndiags % 2 == 0 || !values || !(m > 0)) return LQG_ERR_ARG;
    const int pad = 5, size = ndiags + 2 * pad, nh = size / 2 + 1;
    std::vector<double> x(size), re(nh), im(nh), cs(size), sn(size);
    for (int j = 0; j < size; ++j) {
        cs[j] = std::cos(2.0 * lqg::kPi * j / size);
        sn[j] = std::sin(2.0 * lqg::kPi * j / size);
    }
    std::vector<int> idx;
    for (int i = 0; i < n; ++i) {
        dia_row_indices(i, n, ndiags, idx);
        std::fill(x.begin(), x.end(), 0.0);
        for (int p = 0; p < ndiags; ++p) x[p + pad] = values[idx[p]];
        for (int k = 0; k < nh; ++k) {
            double r = 0.0, s = 0.0;
            for (int j = 0; j < size; ++j) {
                const int w = (int) (((long long) j * k) % size);
                r += x[j] * cs[w];
                s -= x[j] * sn[w];
            }
            if (k >= 1) {
                const double a = lqg::kPi * m * k / size, sinc = std::sin(a) / a;
                r /= sinc;
                s /= sinc;
            }
            re[k] = r;
            im[k] = s;
        }
        for (int j = 0; j < size; ++j) {
            double v = re[0];
            for (int k = 1; k < nh; ++k) {
                const int w = (int) (((long long) j * k) % size);
                if (2 * k == size) v += re[k] * cs[w];
                else v += 2.0 * (re[k] * cs[w] - im[k] * sn[w]);
            }
            x[j] = v / size;
        }
        for (int p = 0; p < ndiags; ++p) values[idx[p]] = x[p + pad];
    }
    return LQG_OK;
}

// Resolution::oversample (mathtools/matrix_helper.cpp:1008-1073): each row's
// ndiags entries are shifted positive, log-transformed, passed through a
// natural cubic spline on the pixel offsets and evaluated osamp times finer;
// the exponentiated row is shifted back and normalised to unit sum.
extern "C" int lqg_resomat_oversample(int n, int ndiags, const double *values, int osamp, double dlambda,
                                      double *rows) {
    if (n < 1 || ndiags < 3 || ndiags % 2 == 0 || !values || !rows || osamp < 1 || !(dlambda > 0))
        return LQG_ERR_ARG;
    const int noff = ndiags / 2, nelem = 2 * noff * osamp + 1;
    std::vector<double> win(ndiags), wout(nelem), row(ndiags), m;
    for (int i = 0; i < ndiags; ++i) win[i] = (i - noff) * dlambda;
    for (int i = 0; i < nelem; ++i) wout[i] = (i * 1. / osamp - noff) * dlambda;
    std::vector<int> idx;
    for (int i = 0; i < n; ++i) {
        dia_row_indices(i, n, ndiags, idx);
        double mn = values[idx[0]];
        for (int p = 0; p < ndiags; ++p) {
            row[p] = values[idx[p]];
            mn = std::min(mn, row[p]);
        }
        const double shift = mn - nonzero_min_abs(row);
        for (auto &f : row) f = std::log(f - shift);
        natural_spline(win, row, m);
        double *out = rows + (size_t) i * nelem;
        double sum = 0.0;
        for (int jj = 0; jj < nelem; ++jj) {
            out[jj] = shift + std::exp(spline_eval(win, row, m, wout[jj]));
            sum += out[jj];
        }
        const double isum = 1. / sum;
        for (int jj = 0; jj < nelem; ++jj) out[jj] *= isum;
    }
    return LQG_OK;
}

// ---------------------------------------------------------------------------
// Device side

namespace lqg {

namespace {

constexpr int RT = kResoTile, RLF = kResoMaxFine, RME = kResoMaxElem;
constexpr int RSLAB = 32;          // grid rows of M evaluated per pass
constexpr int RTH = 256;           // threads; each owns 4 rows of one column of the tile

struct ResoShared {
    double wi[RT][RME + 1];        // weights of the tile's coarse rows
    double wj[RT][RME + 1];        // ... and columns
    double f[RSLAB][RLF + 1];      // a slab of M on the tile's grid block
    double t[RLF][RT + 1];         // T = M_block R_J^T
    double lwr[RLF], swr[RLF];     // ln w and sqrt w of the block's grid rows
    double lwc[RLF], swc[RLF];     // ... and grid columns
};

struct ResoGeom {
    int lf;                        // grid points spanned by the tile: (RT - 1) os + nelem
    int r0, c0;                    // first grid row / column of the block (may be < 0)
    int os, nelem, nf;
};

__device__ __forceinline__ double *fws_d(const WaveArgs &a, int64_t off) {
    return reinterpret_cast<double *>(a.fws + off);
}
__device__ __forceinline__ double *ws_d(const WaveArgs &a, int64_t off) {
    return reinterpret_cast<double *>(a.ws + off);
}

// Weights and grid values of tile (I, J) of chunk ch into shared memory.
__device__ ResoGeom reso_load(ResoShared &sm, const WaveArgs &a, const ChunkDesc &ch, int I, int J) {
    ResoGeom g;
    g.os = ch.os;
    g.nelem = ch.nelem;
    g.nf = ch.nf;
    g.lf = (RT - 1) * ch.os + ch.nelem;
    g.r0 = I * RT * ch.os - ch.sh;
    g.c0 = J * RT * ch.os - ch.sh;
    for (int e = threadIdx.x; e < RT * ch.nelem; e += blockDim.x) {
        const int r = e / ch.nelem, k = e % ch.nelem;
        const int ri = I * RT + r, rj = J * RT + r;
        sm.wi[r][k] = ri < ch.n ? a.rw[ch.rw_off + (int64_t) ri * ch.nelem + k] : 0.0;
        sm.wj[r][k] = rj < ch.n ? a.rw[ch.rw_off + (int64_t) rj * ch.nelem + k] : 0.0;
    }
    for (int e = threadIdx.x; e < g.lf; e += blockDim.x) {
        const int pr = g.r0 + e, pc = g.c0 + e;
        const bool okr = pr >= 0 && pr < ch.nf, okc = pc >= 0 && pc < ch.nf;
        sm.lwr[e] = okr ? a.flogw[ch.fpix + pr] : 0.0;
        sm.swr[e] = okr ? a.fsqw[ch.fpix + pr] : 0.0;
        sm.lwc[e] = okc ? a.flogw[ch.fpix + pc] : 0.0;
        sm.swc[e] = okc ? a.fsqw[ch.fpix + pc] : 0.0;
    }
    __syncthreads();
    return g;
}

// Velocity and redshift separations of grid points (block row fr, block
// column fc): v = c ln(w_hi / w_lo) >= 0 and z = sqrt(w_lo w_hi) - 1, the
// upper-triangle values the reference copies to the lower triangle
// (core/chunk_estimate.cpp:384-398, 414-416).  False outside the grid.
__device__ __forceinline__ bool grid_vz(const ResoShared &sm, const ResoGeom &g, int fr, int fc, double &v,
                                        double &z) {
    const int p = g.r0 + fr, q = g.c0 + fc;
    if (p < 0 || q < 0 || p >= g.nf || q >= g.nf) return false;
    if (p <= q) {
        v = kSpeedOfLight * (sm.lwc[fc] - sm.lwr[fr]);
        z = sm.swr[fr] * sm.swc[fc] - 1.0;
    } else {
        v = kSpeedOfLight * (sm.lwr[fr] - sm.lwc[fc]);
        z = sm.swc[fc] * sm.swr[fr] - 1.0;
    }
    return true;
}

// Tile of R M R^T: out[u] = (R M R^T)[I*RT + r8 + 8u][J*RT + j] for the
// calling thread (j = threadIdx.x % 32, r8 = threadIdx.x / 32), M given at
// block coordinates by ev(fr, fc).
template <class Eval>
__device__ void reso_sandwich(ResoShared &sm, const ResoGeom &g, Eval ev, double out[4]) {
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32;
    for (int s0 = 0; s0 < g.lf; s0 += RSLAB) {
        const int rows = min(RSLAB, g.lf - s0);
        for (int e = threadIdx.x; e < rows * g.lf; e += RTH) {
            const int fr = e / g.lf, fc = e % g.lf;
            sm.f[fr][fc] = ev(s0 + fr, fc);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < RSLAB / 8; ++u) {
            const int fr = r8 + 8 * u;
            if (fr < rows) {
                const double *frow = &sm.f[fr][j * g.os];
                double acc = 0.0;
                for (int b = 0; b < g.nelem; ++b) acc = fma(frow[b], sm.wj[j][b], acc);
                sm.t[s0 + fr][j] = acc;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = r8 + 8 * u;
        double acc = 0.0;
        for (int a = 0; a < g.nelem; ++a) acc = fma(sm.wi[i][a], sm.t[i * g.os + a][j], acc);
        out[u] = acc;
    }
    __syncthreads();
}

// DiscreteInterpolation2D::evaluate (mathtools/discrete_interpolation.cpp:221-242).
__device__ __forceinline__ double signal_at_r(const double *tab, const TableGrid &gr, double z, double v) {
    const double xx = (z - gr.z1) / gr.dz, yy = (v - gr.v1) / gr.dv;
    int nx = (int) xx, ny = (int) yy;
    nx = nx < 0 ? 0 : (nx >= gr.nzp - 1 ? gr.nzp - 2 : nx);
    ny = ny < 0 ? 0 : (ny >= gr.nv - 1 ? gr.nv - 2 : ny);
    const size_t ind = (size_t) nx + (size_t) gr.nzp * ny;
    const double dnx = xx - nx, dny = yy - ny;
    return tab[ind] * (1 - dnx) * (1 - dny) + tab[ind + 1] * dnx * (1 - dny)
         + tab[ind + gr.nzp] * (1 - dnx) * dny + tab[ind + gr.nzp + 1] * dnx * dny;
}

// Analytic band power derivative with a resolution matrix
// (core/chunk_estimate.cpp:444-454): (dk / pi) cos(k_c v) sin(x) / x, x = dk v / 2.
__device__ __forceinline__ double qband(double kc, double dk, double v) {
    if (v == 0) return dk / kPi;
    const double x = dk * v / 2;
    return (dk / kPi) * cos(kc * v) * (sin(x) / x);
}

// Phase A: S = R S_grid R^T into o_s and C~ = D (S + sum_s theta_s Q_s) D + I
// into o_c.  With theta, the Q_s term is formed per redshift bin m as
// w_m(z_ij) (R G_m R^T)_ij with G_m = sum_k theta_{k,m} Q_k on the grid (the
// sandwich is linear and the redshift weights act on the pixel grid after it,
// core/chunk_estimate.cpp:483-536).
__global__ void __launch_bounds__(RTH) k_build_s_c_reso(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    ResoShared &sm = *reinterpret_cast<ResoShared *>(smraw);
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    if (ch.nelem <= 0) return;
    const int ld = ch.ld, n = ch.n, nt = ld / RT;
    if ((int) blockIdx.x >= nt * nt) return;
    const int I = blockIdx.x / nt, J = blockIdx.x % nt;
    if (I > J) return;
    const ResoGeom g = reso_load(sm, a, ch, I, J);
    const DeviceBins &bins = *a.bins;
    const double *stab = (a.signal && !a.turn_off_sfid) ? a.signal + (size_t) ch.res * a.grid.nv * a.grid.nzp : nullptr;
    double s_out[4] = {0, 0, 0, 0}, c_out[4] = {0, 0, 0, 0};
    if (stab) {
        reso_sandwich(sm, g, [&](int fr, int fc) {
            double v, z;
            return grid_vz(sm, g, fr, fc, v, z) ? signal_at_r(stab, a.grid, z, v) : 0.0;
        }, s_out);
#pragma unroll
        for (int u = 0; u < 4; ++u) c_out[u] = s_out[u];
    }
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32;
    const int gj = J * RT + j;
    if (a.theta) {
        const int nzb = ch.ns / ch.kbin_upp;
        for (int iz = 0; iz < nzb; ++iz) {
            const double *th = a.theta + ch.fis + iz * bins.nk;
            bool any = false;
            for (int kn = 0; kn < ch.kbin_upp; ++kn) any |= th[kn] != 0.0;
            if (!any) continue;
            double gm[4];
            reso_sandwich(sm, g, [&](int fr, int fc) {
                double v, z;
                if (!grid_vz(sm, g, fr, fc, v, z)) return 0.0;
                double acc = 0.0;
                for (int kn = 0; kn < ch.kbin_upp; ++kn) {
                    if (th[kn] == 0.0) continue;
                    const double k1 = bins.k_edges[kn], k2 = bins.k_edges[kn + 1];
                    acc += th[kn] * qband((k1 + k2) / 2., k2 - k1, v);
                }
                return acc;
            }, gm);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int gi = I * RT + r8 + 8 * u;
                if (gi < n && gj < n) {
                    const int lo = min(gi, gj), hi = max(gi, gj);
                    const double z = a.sqw[ch.pix + lo] * a.sqw[ch.pix + hi] - 1.0;
                    c_out[u] += gm[u] * zfactor(bins, ch.zb0 + iz, z);
                }
            }
        }
    }
    double *S = fws_d(a, ch.o_s), *C = fws_d(a, ch.o_c);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int gi = I * RT + r8 + 8 * u;
        double sv = 0.0, cv = (gi == gj) ? 1.0 : 0.0;
        if (gi < n && gj < n) {
            sv = a.turn_off_sfid ? 0.0 : s_out[u];
            cv += a.sqiv[ch.pix + gi] * c_out[u] * a.sqiv[ch.pix + gj];
        }
        S[(size_t) gi * ld + gj] = sv;
        C[(size_t) gi * ld + gj] = cv;
        if (I != J) {
            S[(size_t) gj * ld + gi] = sv;
            C[(size_t) gj * ld + gi] = cv;
        }
    }
}

// Phase B, FP64 path: Q_s = w_m(z_ij) (R Q_k R^T)_ij for the chunk's stored
// (k, m) into the FP64 slots (ws o_q), and the per-block partial sums of
// d_s = y^T Q_s y.  d partial rows: each 64 x 64 tile of the plain build owns
// 8 rows; this tile's quarter writes its sum into the first of its two rows and
// zero into the other (tiles below the diagonal write zeros only).
__global__ void __launch_bounds__(RTH) k_build_q_reso(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    ResoShared &sm = *reinterpret_cast<ResoShared *>(smraw);
    __shared__ double red[RTH / 32];
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    if (ch.nelem <= 0 || a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int ld = ch.ld, n = ch.n, nt = ld / RT, t64 = ld / 64;
    if ((int) blockIdx.x >= nt * nt) return;
    const int I = blockIdx.x / nt, J = blockIdx.x % nt;
    const int parts = 8, share = parts / 4;
    double *dpart = ws_d(a, ch.o_dpart) +
                    ((size_t) ((I / 2) * t64 + J / 2) * parts + ((I % 2) * 2 + (J % 2)) * share) * ch.ns;
    if (I > J) {
        for (int e = threadIdx.x; e < share * ch.ns; e += blockDim.x) dpart[e] = 0.0;
        return;
    }
    const ResoGeom g = reso_load(sm, a, ch, I, J);
    const DeviceBins &bins = *a.bins;
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32, gj = J * RT + j;
    const int nzb = ch.ns / ch.kbin_upp;
    const double *y = fws_d(a, ch.o_y);
    // z_ij and y_i y_j of the thread's four elements
    double zz[4], yy[4];
    bool valid[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int gi = I * RT + r8 + 8 * u;
        valid[u] = gi < n && gj < n;
        yy[u] = valid[u] ? y[gi] * y[gj] : 0.0;
        const int lo = min(gi, gj), hi = max(gi, gj);
        zz[u] = valid[u] ? a.sqw[ch.pix + lo] * a.sqw[ch.pix + hi] - 1.0 : 0.0;
    }
    const double mult = (I == J) ? 1.0 : 2.0;   // the mirror tile's share of y^T Q y
    const size_t plane = (size_t) ld * ld;
    for (int kn = 0; kn < ch.kbin_upp; ++kn) {
        const double k1 = bins.k_edges[kn], k2 = bins.k_edges[kn + 1], kc = (k1 + k2) / 2., dk = k2 - k1;
        double b[4];
        reso_sandwich(sm, g, [&](int fr, int fc) {
            double v, z;
            return grid_vz(sm, g, fr, fc, v, z) ? qband(kc, dk, v) : 0.0;
        }, b);
        for (int iz = 0; iz < nzb; ++iz) {
            const int s = iz * ch.kbin_upp + kn;
            double part = 0.0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int gi = I * RT + r8 + 8 * u;
                const double q = valid[u] ? b[u] * zfactor(bins, ch.zb0 + iz, zz[u]) : 0.0;
                part += yy[u] * q;
                double *Q = ws_d(a, ch.o_q) + (size_t) s * plane;
                Q[(size_t) gi * ld + gj] = q;
                if (I != J) Q[(size_t) gj * ld + gi] = q;
            }
            for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
            if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = part;
            __syncthreads();
            if (threadIdx.x == 0) {
                double acc = 0.0;
                for (int w = 0; w < RTH / 32; ++w) acc += red[w];
                dpart[s] = mult * acc;
                for (int r = 1; r < share; ++r) dpart[(size_t) r * ch.ns + s] = 0.0;
            }
            __syncthreads();
        }
    }
}

// Mixed path, per grid point p and stored k band: (cos, sin)(k_c u_p) with
// u_p = c ln(w_p / w_0), in FP64.  cos(k_c v_pq) = C_p C_q + S_p S_q then
// needs no large-argument reduction on the FP32 pipe.
__global__ void k_reso_phases(WaveArgs a) {
    const ChunkDesc &ch = a.chunks[blockIdx.y];
    if (ch.nelem <= 0 || a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const DeviceBins &bins = *a.bins;
    float2 *ph = reinterpret_cast<float2 *>(a.ws + ch.o_ph);
    const double l0 = a.flogw[ch.fpix];
    const int total = ch.kbin_upp * ch.nf;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        const int kn = e / ch.nf, p = e % ch.nf;
        const double kc = (bins.k_edges[kn] + bins.k_edges[kn + 1]) / 2.;
        double sn, cs;
        sincos(kc * (kSpeedOfLight * (a.flogw[ch.fpix + p] - l0)), &sn, &cs);
        ph[e] = make_float2((float) cs, (float) sn);
    }
}

constexpr int FSLAB = 16;

struct ResoSharedF {
    float sinc[RLF][RLF + 1];      // sin(x) / x on the tile's grid block, x = dk v / 2, for one dk
    float fq[FSLAB * (RLF + 1)];   // a slab of Q_k on the block; later the 32 x 33 output tile
    float t[RLF][RT + 1];          // T = M_block R_J^T
    float wi[RT][RME + 1], wj[RT][RME + 1];
    float2 lwr[RLF], lwc[RLF];     // ln w of the block's grid rows / columns (double-float)
    float cr[RLF], sr[RLF], cc[RLF], sc[RLF];   // (cos, sin)(k_c u) of the rows / columns
    float qscale[kMaxGramBlocks * 128];
};

// Phase B, mixed path: the same Q_s as k_build_q_reso on the FP32 pipe, into
// fp16 hi/lo planes with the slot scale.  Q_k on the grid is
// (dk / pi) sinc(dk v / 2) (C_p C_q + S_p S_q): v from double-float ln w
// (relative error ~1e-7), the cosine from FP64 phases (absolute error ~1e-7);
// the sinc block is computed once per distinct dk.  Redshift weights in
// double-float arithmetic (as the plain mixed build).  d partial rows: 16 per
// 64 x 64 tile, 4 per quarter.
// NEL, OS > 0 fix the row width and oversampling of every chunk at compile
// time: each thread then keeps its column's weights, scaled by the column
// phases, in registers and reads the cached sinc block directly (no slab of
// Q_k is formed, one barrier per band).
//
// GR: the redshift-growth factor is applied (a separate instantiation: its
// code, even untaken, slows the register-bound loop of the others by a quarter).
template <int NEL, int OS, bool GR>
__global__ void __launch_bounds__(RTH, 2) k_build_q_reso_f32(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    ResoSharedF &sm = *reinterpret_cast<ResoSharedF *>(smraw);
    __shared__ double red[4 * (RTH / 32)];
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    if (ch.nelem <= 0 || a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int ld = ch.ld, n = ch.n, nt = ld / RT, t64 = ld / 64;
    if ((int) blockIdx.x >= nt * nt) return;
    const int I = blockIdx.x / nt, J = blockIdx.x % nt;
    const int parts = 16, share = parts / 4;
    double *dpart = ws_d(a, ch.o_dpart) +
                    ((size_t) ((I / 2) * t64 + J / 2) * parts + ((I % 2) * 2 + (J % 2)) * share) * ch.ns;
    if (I > J) {
        for (int e = threadIdx.x; e < share * ch.ns; e += blockDim.x) dpart[e] = 0.0;
        return;
    }
    const int os = NEL > 0 ? OS : ch.os, nel = NEL > 0 ? NEL : ch.nelem, lf = (RT - 1) * os + nel;
    const int r0 = I * RT * os - ch.sh, c0 = J * RT * os - ch.sh;
    for (int e = threadIdx.x; e < RT * nel; e += blockDim.x) {
        const int r = e / nel, k = e % nel;
        const int ri = I * RT + r, rj = J * RT + r;
        sm.wi[r][k] = ri < n ? (float) a.rw[ch.rw_off + (int64_t) ri * nel + k] : 0.f;
        sm.wj[r][k] = rj < n ? (float) a.rw[ch.rw_off + (int64_t) rj * nel + k] : 0.f;
    }

    for (int e = threadIdx.x; e < lf; e += blockDim.x) {
        const int pr = r0 + e, pc = c0 + e;
        const double lr = (pr >= 0 && pr < ch.nf) ? a.flogw[ch.fpix + pr] : 0.0;
        const double lc = (pc >= 0 && pc < ch.nf) ? a.flogw[ch.fpix + pc] : 0.0;
        sm.lwr[e] = make_float2((float) lr, (float) (lr - (double) (float) lr));
        sm.lwc[e] = make_float2((float) lc, (float) (lc - (double) (float) lc));
    }
    for (int t = threadIdx.x; t < ch.ns; t += blockDim.x)
        sm.qscale[t] = (float) a.scales[(size_t) 4 * a.n_chunks + ch.slot_q + t];
    __syncthreads();
    const DeviceBins &bins = *a.bins;
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32, gj = J * RT + j;
    const int nzb = ch.ns / ch.kbin_upp;
    const double *y = fws_d(a, ch.o_y);
    const float2 *sw2 = a.sqw2 + ch.pix;
    // per element: y_i y_j, 1 + z_ij as double-float, weights of the first 4 redshift bins
    float yy[4], zp[4], ze[4], zw[4][4];
    bool valid[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int gi = I * RT + r8 + 8 * u;
        valid[u] = gi < n && gj < n;
        yy[u] = valid[u] ? (float) (y[gi] * y[gj]) : 0.f;
        zp[u] = 0.f; ze[u] = 0.f;
        if (valid[u]) two_prod_ff(sw2[min(gi, gj)], sw2[max(gi, gj)], zp[u], ze[u]);
#pragma unroll
        for (int iz = 0; iz < 4; ++iz)
            zw[u][iz] = (valid[u] && iz < nzb) ? (GR ? zfactor_ff(bins, ch.zb0 + iz, zp[u], ze[u])
                                                     : zweight_ff(bins, ch.zb0 + iz, zp[u], ze[u]))
                                               : 0.f;
    }
    const float2 *ph = reinterpret_cast<const float2 *>(a.ws + ch.o_ph);
    const float mult = (I == J) ? 1.f : 2.f;
    const size_t plane = (size_t) ld * ld;
    float dk_cached = -1.f;
    float (*fs)[RLF + 1] = reinterpret_cast<float (*)[RLF + 1]>(sm.fq);
    for (int kn = 0; kn < ch.kbin_upp; ++kn) {
        const double k1 = bins.k_edges[kn], k2 = bins.k_edges[kn + 1];
        const float dkf = (float) (k2 - k1), coef = (float) ((k2 - k1) / kPi);
        // phases of the block's grid rows and columns for this band
        for (int e = threadIdx.x; e < lf; e += blockDim.x) {
            const int pr = r0 + e, pc = c0 + e;
            const float2 a1 = (pr >= 0 && pr < ch.nf) ? ph[(size_t) kn * ch.nf + pr] : make_float2(0.f, 0.f);
            const float2 a2 = (pc >= 0 && pc < ch.nf) ? ph[(size_t) kn * ch.nf + pc] : make_float2(0.f, 0.f);
            sm.cr[e] = a1.x; sm.sr[e] = a1.y;
            sm.cc[e] = a2.x; sm.sc[e] = a2.y;
        }
        if (dkf != dk_cached) {
            const float hdk = 0.5f * dkf;
            for (int e = threadIdx.x; e < lf * lf; e += RTH) {
                const int fr = e / lf, fc = e % lf;
                const int p = r0 + fr, q = c0 + fc;
                float v = 0.f;
                bool ok = p >= 0 && q >= 0 && p < ch.nf && q < ch.nf;
                if (ok) {
                    const float2 hi = p <= q ? sm.lwc[fc] : sm.lwr[fr], lo = p <= q ? sm.lwr[fr] : sm.lwc[fc];
                    v = __fmul_rn((float) kSpeedOfLight, __fadd_rn(__fsub_rn(hi.x, lo.x), __fsub_rn(hi.y, lo.y)));
                }
                const float x = hdk * v;
                sm.sinc[fr][fc] = !ok ? 0.f : (x == 0.f ? 1.f : __fdiv_rn(sinf(x), x));
            }
            dk_cached = dkf;
        }
        __syncthreads();
        if constexpr (NEL > 0) {
            // T[fr][j] = coef (C_fr X + S_fr Y) with X = sum_b sinc[fr][c] C_c w_jb and
            // Y likewise with S_c (c = j OS + b): the row phase factors leave the
            // sum, so the cached sinc block is read directly, one load per two FMAs
            float wc[NEL], wsn[NEL];
#pragma unroll
            for (int bb = 0; bb < NEL; ++bb) {
                const float w = sm.wj[j][bb];
                wc[bb] = sm.cc[j * OS + bb] * w;
                wsn[bb] = sm.sc[j * OS + bb] * w;
            }
            for (int fr = r8; fr < lf; fr += 8) {
                const float *srow = &sm.sinc[fr][j * OS];
                float x = 0.f, yv = 0.f;
#pragma unroll
                for (int bb = 0; bb < NEL; ++bb) {
                    const float sv = srow[bb];
                    x = fmaf(sv, wc[bb], x);
                    yv = fmaf(sv, wsn[bb], yv);
                }
                sm.t[fr][j] = coef * fmaf(sm.cr[fr], x, sm.sr[fr] * yv);
            }
            __syncthreads();
        } else {
            for (int s0 = 0; s0 < lf; s0 += FSLAB) {
                const int rows = min(FSLAB, lf - s0);
                for (int e = threadIdx.x; e < rows * lf; e += RTH) {
                    const int fr = e / lf, fc = e % lf;
                    const float cs = fmaf(sm.cr[s0 + fr], sm.cc[fc], sm.sr[s0 + fr] * sm.sc[fc]);
                    fs[fr][fc] = coef * sm.sinc[s0 + fr][fc] * cs;
                }
                __syncthreads();
#pragma unroll
                for (int u = 0; u < FSLAB / 8; ++u) {
                    const int fr = r8 + 8 * u;
                    if (fr < rows) {
                        const float *frow = &fs[fr][j * os];
                        float acc = 0.f;
                        for (int bb = 0; bb < nel; ++bb) acc = fmaf(frow[bb], sm.wj[j][bb], acc);
                        sm.t[s0 + fr][j] = acc;
                    }
                }
                __syncthreads();
            }
        }
        float b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int i = r8 + 8 * u;
            float acc = 0.f;
            for (int aa = 0; aa < nel; ++aa) acc = fmaf(sm.wi[i][aa], sm.t[i * os + aa][j], acc);
            b[u] = acc;
        }
        // Output of the band for up to 4 redshift bins at a time: Q_s tiles through
        // the T buffer (free once every thread holds its b) for the mirrored
        // stores, one block reduction of the d partials per group.
        float (*qts)[RT][RT + 1] = reinterpret_cast<float (*)[RT][RT + 1]>(&sm.t[0][0]);
        static_assert(4 * RT * (RT + 1) <= RLF * (RT + 1), "T buffer too small for 4 output tiles");
        for (int z0 = 0; z0 < nzb; z0 += 4) {
            const int nzg = min(4, nzb - z0);
            float part[4] = {0.f, 0.f, 0.f, 0.f};
            __syncthreads();   // T (stage 2) or the previous group's tiles are no longer read
            for (int g = 0; g < nzg; ++g) {
                const int iz = z0 + g, s = iz * ch.kbin_upp + kn;
                const float qs = sm.qscale[s];
                __half *qh = a.q_hi + (size_t) (ch.slot_q + s) * plane;
                __half *ql = a.q_lo + (size_t) (ch.slot_q + s) * plane;
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int i = r8 + 8 * u, gi = I * RT + i;
                    float w = 0.f;
                    if (valid[u])
                        w = iz < 4 ? zw[u][iz]
                                   : (GR ? zfactor_ff(bins, ch.zb0 + iz, zp[u], ze[u])
                                         : zweight_ff(bins, ch.zb0 + iz, zp[u], ze[u]));
                    const float q = b[u] * w;
                    part[g] = fmaf(yy[u], q, part[g]);
                    const float x = q * qs;
                    qts[g][i][j] = x;
                    const __half h = __float2half_rn(x);
                    qh[(size_t) gi * ld + gj] = h;
                    ql[(size_t) gi * ld + gj] = __float2half_rn(x - __half2float(h));
                }
            }
            for (int g = 0; g < nzg; ++g) {
                float v = part[g];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
                if (threadIdx.x % 32 == 0) red[g * (RTH / 32) + threadIdx.x / 32] = (double) v;
            }
            __syncthreads();
            if (I != J) {
                // mirror tile, row J*RT + r8 + 8u, column I*RT + j: element (j, r8 + 8u) of this tile
                for (int g = 0; g < nzg; ++g) {
                    const int s = (z0 + g) * ch.kbin_upp + kn;
                    __half *qh = a.q_hi + (size_t) (ch.slot_q + s) * plane;
                    __half *ql = a.q_lo + (size_t) (ch.slot_q + s) * plane;
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int rr = J * RT + r8 + 8 * u, cc2 = I * RT + j;
                        const float x = qts[g][j][r8 + 8 * u];
                        const __half h = __float2half_rn(x);
                        qh[(size_t) rr * ld + cc2] = h;
                        ql[(size_t) rr * ld + cc2] = __float2half_rn(x - __half2float(h));
                    }
                }
            }
            if (threadIdx.x < nzg) {
                const int g = threadIdx.x, s = (z0 + g) * ch.kbin_upp + kn;
                double acc = 0.0;
                for (int w = 0; w < RTH / 32; ++w) acc += red[g * (RTH / 32) + w];
                dpart[s] = mult * acc;
                for (int r = 1; r < share; ++r) dpart[(size_t) r * ch.ns + s] = 0.0;
            }
        }
        __syncthreads();   // before the next band overwrites the phases and the slab
    }
}

struct ResoSharedFF {
    float2 wi[RT][RME + 1], wj[RT][RME + 1];
    float2 f[RSLAB][RLF + 1];
    float2 t[RLF][RT + 1];
    float2 lwr[RLF], swr[RLF], lwc[RLF], swc[RLF];
};

// Tile of R M R^T in double-float: out[u] = (R M R^T)[I RT + r8 + 8u][J RT + j]
// for the calling thread, M given at grid rows fr in [0, lf) and columns fc of
// the tile's block by ev(fr, fc) (the same two stages as reso_sandwich).
template <class Eval>
__device__ void reso_sandwich_ff(ResoSharedFF &sm, int lf, int nel, int os, Eval ev, float2 out[4]) {
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32;
    for (int s0 = 0; s0 < lf; s0 += RSLAB) {
        const int rows = min(RSLAB, lf - s0);
        for (int e = threadIdx.x; e < rows * lf; e += RTH) {
            const int fr = e / lf, fc = e % lf;
            sm.f[fr][fc] = ev(s0 + fr, fc);
        }
        __syncthreads();
#pragma unroll
        for (int u = 0; u < RSLAB / 8; ++u) {
            const int fr = r8 + 8 * u;
            if (fr < rows) {
                float2 acc = make_float2(0.f, 0.f);
                for (int b = 0; b < nel; ++b) acc = ff_fma(sm.f[fr][j * os + b], sm.wj[j][b], acc);
                sm.t[s0 + fr][j] = acc;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = r8 + 8 * u;
        float2 acc = make_float2(0.f, 0.f);
        for (int aa = 0; aa < nel; ++aa) acc = ff_fma(sm.wi[i][aa], sm.t[i * os + aa][j], acc);
        out[u] = acc;
    }
    __syncthreads();
}

// G(v) = sum_{kn < K} theta[zm nk + kn] Q_kn(v), Q_kn the analytic band
// derivative with a resolution matrix (core/chunk_estimate.cpp:444-454),
// on nodes v = i h: G as a double-float pair and h G' as a float, for cubic
// Hermite interpolation between nodes.  One thread per (node, z bin, K).
__global__ void k_theta_reso_tables(const double *theta, const DeviceBins *bins, const int *ks, int nk, int nz,
                                    int64_t nn, double h, float4 *rtab) {
    const int64_t i = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    const int zm = blockIdx.y, kr = blockIdx.z;
    if (i >= nn) return;
    const int K = ks[kr];
    const double v = (double) i * h;
    double g = 0.0, dg = 0.0;
    for (int kn = 0; kn < K; ++kn) {
        const double th = theta[zm * nk + kn];
        if (th == 0.0) continue;
        const double k1 = bins->k_edges[kn], k2 = bins->k_edges[kn + 1], kc = (k1 + k2) / 2., dk = k2 - k1;
        double sn, cs, sx, cx;
        sincos(kc * v, &sn, &cs);
        const double x = dk * v / 2.;
        sincos(x, &sx, &cx);
        // sinc(x) and its derivative; the series below 1e-4 (error < 1e-17)
        const double sinc = fabs(x) < 1e-4 ? 1. - x * x / 6. : sx / x;
        const double dsinc = fabs(x) < 1e-4 ? -x / 3. : (x * cx - sx) / (x * x);
        g += th * (dk / kPi) * cs * sinc;
        dg += th * (dk / kPi) * (-kc * sn * sinc + cs * dsinc * (dk / 2.));
    }
    const float gh = (float) g;
    rtab[((int64_t) kr * nz + zm) * nn + i] = make_float4(gh, (float) (g - (double) gh), (float) (h * dg), 0.f);
}

// G at x = v / h (double-float) from a row of k_theta_reso_tables: the node
// value in double-float plus the cubic Hermite correction t (D0 + t (c2 +
// t c3)) in float, which is about h k_max = 1/20 of G: the interpolation
// error (h k)^4 / 384 and the float correction both stay near 1e-8 of G.
__device__ __forceinline__ float2 rtab_eval(const float4 *row, int64_t nn, float2 x) {
    int n;
    float2 t2;
    ff_index(x, (int) nn - 2, n, t2);
    const float4 a = row[n], b = row[n + 1];
    const float t = t2.x;
    const float dG = __fadd_rn(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y));
    const float c2 = 3.f * dG - 2.f * a.z - b.z, c3 = -2.f * dG + a.z + b.z;
    const float corr = t * (a.z + t * (c2 + t * c3));
    return ff_add(make_float2(a.x, a.y), make_float2(corr, 0.f));
}

// Phase A, mixed path: S = R S_grid R^T and C~ = D (S + sum_s theta_s Q_s) D + I
// in double-float arithmetic (about 48 significant bits) on the FP32 pipe;
// grid v, z, interpolation fractions and table values in double-float, the
// sandwich with double-float multiply-adds.  The theta term is formed per
// redshift bin m as w_m(z_ij) (R G_m R^T)_ij, G_m = sum_k theta_{k,m} Q_k on the
// grid from the node table of k_theta_reso_tables (G_m depends on v only; its
// nodes are shared by every chunk) instead of the band sum per grid element.
// Stored as double-float pairs.
__global__ void __launch_bounds__(RTH) k_build_s_c_reso_ff(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smraw[];
    ResoSharedFF &sm = *reinterpret_cast<ResoSharedFF *>(smraw);
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    if (ch.nelem <= 0) return;
    const int ld = ch.ld, n = ch.n, nt = ld / RT;
    if ((int) blockIdx.x >= nt * nt) return;
    const int I = blockIdx.x / nt, J = blockIdx.x % nt;
    if (I > J) return;
    const int os = ch.os, nel = ch.nelem, lf = (RT - 1) * os + nel;
    const int r0 = I * RT * os - ch.sh, c0 = J * RT * os - ch.sh;
    for (int e = threadIdx.x; e < RT * nel; e += blockDim.x) {
        const int r = e / nel, k = e % nel;
        const int ri = I * RT + r, rj = J * RT + r;
        sm.wi[r][k] = ri < n ? ff_of(a.rw[ch.rw_off + (int64_t) ri * nel + k]) : make_float2(0.f, 0.f);
        sm.wj[r][k] = rj < n ? ff_of(a.rw[ch.rw_off + (int64_t) rj * nel + k]) : make_float2(0.f, 0.f);
    }
    for (int e = threadIdx.x; e < lf; e += blockDim.x) {
        const int pr = r0 + e, pc = c0 + e;
        const bool okr = pr >= 0 && pr < ch.nf, okc = pc >= 0 && pc < ch.nf;
        sm.lwr[e] = okr ? ff_of(a.flogw[ch.fpix + pr]) : make_float2(0.f, 0.f);
        sm.swr[e] = okr ? ff_of(a.fsqw[ch.fpix + pr]) : make_float2(0.f, 0.f);
        sm.lwc[e] = okc ? ff_of(a.flogw[ch.fpix + pc]) : make_float2(0.f, 0.f);
        sm.swc[e] = okc ? ff_of(a.fsqw[ch.fpix + pc]) : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const TableGrid &gr = a.grid;
    const float2 *tab = (a.signal_ff && !a.turn_off_sfid) ? a.signal_ff + (size_t) ch.res * gr.nv * gr.nzp : nullptr;
    const int j = threadIdx.x % 32, r8 = threadIdx.x / 32, gj = J * RT + j;
    float2 sv[4] = {};
    if (tab) {
        const float2 kv = make_float2(gr.kv_hi, gr.kv_lo), z1p = make_float2(gr.z1p_hi, gr.z1p_lo);
        const float2 idz = make_float2(gr.idz_hi, gr.idz_lo), one = make_float2(1.f, 0.f);
        reso_sandwich_ff(sm, lf, nel, os, [&](int fr, int fc) {
            const int p = r0 + fr, q = c0 + fc;
            float2 val = make_float2(0.f, 0.f);
            if (p >= 0 && q >= 0 && p < ch.nf && q < ch.nf) {
                const bool up = p <= q;
                const float2 lh = up ? sm.lwc[fc] : sm.lwr[fr], ll = up ? sm.lwr[fr] : sm.lwc[fc];
                const float2 yy = ff_mul(ff_sub(lh, ll), kv);               // v / dv
                float zp, ze;
                two_prod_ff(sm.swr[fr], sm.swc[fc], zp, ze);                 // 1 + z
                const float2 xx = ff_mul(ff_sub(ff_norm(zp, ze), z1p), idz); // (z - z1) / dz
                int nx, ny;
                float2 fx, fy;
                ff_index(xx, gr.nzp - 2, nx, fx);
                ff_index(yy, gr.nv - 2, ny, fy);
                const size_t ind = (size_t) nx + (size_t) gr.nzp * ny;
                const float2 gx = ff_sub(one, fx), gy = ff_sub(one, fy);
                val = ff_mul(ff_mul(tab[ind], gx), gy);
                val = ff_fma(ff_mul(tab[ind + 1], fx), gy, val);
                val = ff_fma(ff_mul(tab[ind + gr.nzp], gx), fy, val);
                val = ff_fma(ff_mul(tab[ind + gr.nzp + 1], fx), fy, val);
            }
            return val;
        }, sv);
    }
    // sum_s theta_s Q_s on the pixel grid
    float2 tv[4] = {};
    if (a.theta && a.rtab && ch.tcombo >= 0) {
        const DeviceBins &bins = *a.bins;
        const int nzb = ch.ns / ch.kbin_upp;
        for (int iz = 0; iz < nzb; ++iz) {
            const double *th = a.theta + ch.fis + iz * bins.nk;
            bool any = false;
            for (int kn = 0; kn < ch.kbin_upp; ++kn) any |= th[kn] != 0.0;
            if (!any) continue;   // uniform over the block
            const float4 *row = a.rtab + ((int64_t) ch.tcombo * bins.nz + ch.zb0 + iz) * a.rtab_n;
            float2 gm[4];
            reso_sandwich_ff(sm, lf, nel, os, [&](int fr, int fc) {
                const int p = r0 + fr, q = c0 + fc;
                if (p < 0 || q < 0 || p >= ch.nf || q >= ch.nf) return make_float2(0.f, 0.f);
                const bool up = p <= q;
                const float2 lh = up ? sm.lwc[fc] : sm.lwr[fr], ll = up ? sm.lwr[fr] : sm.lwc[fc];
                return rtab_eval(row, a.rtab_n, ff_mul(ff_sub(lh, ll), a.rtab_x));   // v / h
            }, gm);
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int gi = I * RT + r8 + 8 * u;
                if (gi >= n || gj >= n) continue;
                float zp, ze;
                two_prod_ff(a.sqw2[ch.pix + gi], a.sqw2[ch.pix + gj], zp, ze);   // 1 + z_ij
                float2 w = zweight_dd(bins, ch.zb0 + iz, zp, ze);
                if (a.growth && w.x != 0.f) {
                    const double z1 = (double) zp + (double) ze;
                    w = ff_mul(w, ff_of(pow(z1 / (bins.z_centers[ch.zb0 + iz] + 1.0), bins.growth_b)));
                }
                tv[u] = ff_fma(gm[u], w, tv[u]);
            }
        }
    }
    // S and C~ as double-float pairs (c_is_ff: the form the mixed factorisation uses)
    float2 *S = reinterpret_cast<float2 *>(a.fws + ch.o_s), *C = reinterpret_cast<float2 *>(a.fws + ch.o_c);
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int gi = I * RT + r8 + 8 * u;
        float2 s2 = make_float2(0.f, 0.f), c2 = make_float2(gi == gj ? 1.f : 0.f, 0.f);
        if (gi < n && gj < n) {
            s2 = sv[u];
            const float2 cv = ff_mul(ff_mul(a.sqiv2[ch.pix + gi], ff_add(sv[u], tv[u])), a.sqiv2[ch.pix + gj]);
            c2 = (gi == gj) ? ff_add(cv, make_float2(1.f, 0.f)) : cv;
        }
        S[(size_t) gi * ld + gj] = s2;
        C[(size_t) gi * ld + gj] = c2;
        if (I != J) {
            S[(size_t) gj * ld + gi] = s2;
            C[(size_t) gj * ld + gi] = c2;
        }
    }
}

// Shared memory above the 48 KB default: once per device (the attribute is per device)
std::atomic<unsigned long long> reso_attr{0};

cudaError_t set_reso_attrs_now() {
    const int bytes = (int) sizeof(ResoShared), bytes_f = (int) sizeof(ResoSharedF), bytes_ff = (int) sizeof(ResoSharedFF);
    const cudaFuncAttribute at = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaError_t e = cudaFuncSetAttribute(k_build_s_c_reso, at, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_q_reso, at, bytes);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_q_reso_f32<0, 0, false>, at, bytes_f);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_q_reso_f32<0, 0, true>, at, bytes_f);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_q_reso_f32<31, 3, false>, at, bytes_f);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_q_reso_f32<11, 1, false>, at, bytes_f);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_build_s_c_reso_ff, at, bytes_ff);
    return e;
}

bool set_reso_attrs() {
    return once_per_device(reso_attr, [](int) { return set_reso_attrs_now(); });
}

}  // namespace

void launch_theta_reso_tables(const double *theta, const DeviceBins *bins, const int *ks, int n_ks, int nk, int nz,
                              int64_t nn, double h, float4 *rtab, cudaStream_t st) {
    k_theta_reso_tables<<<dim3((unsigned) ((nn + 255) / 256), nz, n_ks), 256, 0, st>>>(theta, bins, ks, nk, nz, nn, h,
                                                                                      rtab);
}

void launch_build_s_c_reso(WaveArgs &a, cudaStream_t st) {
    if (!set_reso_attrs()) {
        a.host_failed = 1;
        return;
    }
    const int nt = a.max_ld / RT;
    // mixed path: the double-float build (pairs, c_is_ff); FP64 path: FP64
    if (a.c_is_ff)
        k_build_s_c_reso_ff<<<dim3(nt * nt, a.n_chunks), RTH, sizeof(ResoSharedFF), st>>>(a);
    else
        k_build_s_c_reso<<<dim3(nt * nt, a.n_chunks), RTH, sizeof(ResoShared), st>>>(a);
    a.launches++;
}

void launch_build_q_reso(WaveArgs &a, cudaStream_t st) {
    if (!set_reso_attrs()) {
        a.host_failed = 1;
        return;
    }
    const int nt = a.max_ld / RT;
    if (a.precision == LQG_PRECISION_MIXED) {
        k_reso_phases<<<dim3(32, a.n_chunks), 256, 0, st>>>(a);
        // a fixed-width kernel when every resolution chunk of the batch has its shape
        const dim3 grid(nt * nt, a.n_chunks);
        if (a.growth)
            k_build_q_reso_f32<0, 0, true><<<grid, RTH, sizeof(ResoSharedF), st>>>(a);
        else if (a.reso_nelem == 31 && a.reso_os == 3)
            k_build_q_reso_f32<31, 3, false><<<grid, RTH, sizeof(ResoSharedF), st>>>(a);
        else if (a.reso_nelem == 11 && a.reso_os == 1)
            k_build_q_reso_f32<11, 1, false><<<grid, RTH, sizeof(ResoSharedF), st>>>(a);
        else
            k_build_q_reso_f32<0, 0, false><<<grid, RTH, sizeof(ResoSharedF), st>>>(a);
        a.launches += 2;
    } else {
        k_build_q_reso<<<dim3(nt * nt, a.n_chunks), RTH, sizeof(ResoShared), st>>>(a);
        a.launches++;
    }
}

}  // namespace lqg
