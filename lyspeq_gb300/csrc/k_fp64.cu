// Per-chunk QMLE kernels: matrix build, FP64 products, trace reductions.
// Matrices are ld x ld row-major (ld = n rounded up to 64); rows/columns >= n
// are padding (zero, identity on the diagonal of C~).  The FP64 factorisation
// of C~ is in k_factor.cu.
//
// Formulation.  The reference forms M = diag(ivar) C + I, inverts it by LU
// and right-scales by diag(ivar) (core/chunk_estimate.cpp:693-711).  Here
// C~ = D C D + I with D = diag(sqrt(ivar)) is factored by Cholesky and
// C^-1 = D C~^-1 D, the same matrix: (diag(ivar) C + I)^-1 diag(ivar)
// = D (D C D + I)^-1 D.  C~ is SPD for any ivar >= 0 and masked pixels
// (ivar = 0) get exact zero rows and columns in C^-1, as in the reference.
//
// The traces use the reference's own structure: A_s = C^-1 Q_s
// (core/chunk_estimate.cpp:721-736), F_ij = <A_i^T, A_j> (:815-832),
// b_j = <A_j, N C^-1> (:767-786), t_j = <A_j, S C^-1> (:789-804), written as one
// Gram product G = P R^T with rows P = [A_0^T .. A_{ns-1}^T, (C^-1 S)^T, N C^-1]
// and R = [A_0 .. A_{ns-1}].
#include "lqg_internal.cuh"
#include "lqg_ff.cuh"

namespace lqg {

namespace {

constexpr int T64 = 64;    // tile edge of the element-wise kernels
constexpr int GR = 128;    // Gram block edge

__device__ __forceinline__ double *fws_d(const WaveArgs &a, int64_t off) {
    return reinterpret_cast<double *>(a.fws + off);
}
__device__ __forceinline__ double *ws_d(const WaveArgs &a, int64_t off) {
    return reinterpret_cast<double *>(a.ws + off);
}

// Velocity and redshift separations of pixels p <= q, as Chunk::_setVZMatrices
// (core/chunk_estimate.cpp:384-398), from per-pixel log(lambda) and sqrt(lambda).
__device__ __forceinline__ void vz_of(const double *logw, const double *sqw, int p, int q,
                                      double &v, double &z) {
    v = kSpeedOfLight * (logw[q] - logw[p]);
    z = sqw[p] * sqw[q] - 1.0;
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

// Linear interpolation index of a derivative-table row (discrete_interpolation.cpp:61-72);
// shared by all k bands at one v.
__device__ __forceinline__ void vindex(const TableGrid &g, double v, int &n, double &dn) {
    double xx = (v - g.v1) / g.dv;
    n = (int) xx;
    n = n < 0 ? 0 : (n >= g.nv - 1 ? g.nv - 2 : n);
    dn = xx - n;
}

// Mixed-path element math on the FP32 pipe in double-float arithmetic (a
// value is hi + lo, two floats).  Differences of close operands are exact
// (Sterbenz), so v_ij, the interpolation fraction and the redshift weights
// keep ~1e-7 relative accuracy, down to the small weights at a bin's edge.

// Table index and fraction at v = c (ln w_hi - ln w_lo): xx = v / dv as p + e,
// then the reference's clamped linear-interpolation index
// (mathtools/discrete_interpolation.cpp:61-72, v1 = 0).
__device__ __forceinline__ void vindex_ff(const TableGrid &g, float2 lwh, float2 lwl, int &n, float &dn) {
    const float2 d = make_float2(__fsub_rn(lwh.x, lwl.x), __fsub_rn(lwh.y, lwl.y));
    float p, e;
    two_prod_ff(d, make_float2(g.kv_hi, g.kv_lo), p, e);
    int nn = (int) floorf(p);
    float f = __fadd_rn(__fsub_rn(p, (float) nn), e);
    if (f < 0.f) { --nn; f = __fadd_rn(f, 1.f); }
    else if (f >= 1.f) { ++nn; f = __fsub_rn(f, 1.f); }
    if (nn > g.nv - 2) { nn = g.nv - 2; f = __fadd_rn(__fsub_rn(p, (float) nn), e); }
    if (nn < 0) { nn = 0; f = __fadd_rn(p, e); }
    n = nn;
    dn = f;
}

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// theta-weighted derivative tables, one row per ((table, KBIN_UPP), z bin):
// ttab[(cb nz + zm) nv + v] = sum_{kn < KBIN_UPP} theta[zm nk + kn] deriv[table][kn][v];
// the mixed path also gets the rows as double-float pairs (ttab_ff non-null).
__global__ void k_theta_tables(const double *deriv, const double *theta, const int *combos, int nk, int nz,
                               int nv, double *ttab, float2 *ttab_ff) {
    const int v = blockIdx.x * blockDim.x + threadIdx.x, zm = blockIdx.y, cb = blockIdx.z;
    if (v >= nv) return;
    const int res = combos[2 * cb], kup = combos[2 * cb + 1];
    double acc = 0.0;
    for (int kn = 0; kn < kup; ++kn) {
        const double th = theta[zm * nk + kn];
        if (th != 0.0) acc += th * deriv[((size_t) res * nk + kn) * nv + v];
    }
    const size_t o = ((size_t) cb * nz + zm) * nv + v;
    ttab[o] = acc;
    if (ttab_ff) {
        const float h = (float) acc;
        ttab_ff[o] = make_float2(h, (float) (acc - (double) h));
    }
}

// ---------------------------------------------------------------------------
// Phase A, K1a: S_fid and C~ = D (S + sum_s theta_s Q_s) D + I.
__global__ void k_build_s_c(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n;
    const int tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr || ch.nelem > 0) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    if (!LQG_IN_BOUNDS(a, ch.o_s >= 0 && ch.o_c >= 0 && ch.o_s + (int64_t) ld * ld * 8 <= a.fws_bytes &&
                              ch.o_c + (int64_t) ld * ld * 8 <= a.fws_bytes && ch.pix >= 0 &&
                              ch.pix + n <= a.n_pix && ld % T64 == 0 && n <= ld,
                       11, c, ch.o_c))
        return;
    double *S = fws_d(a, ch.o_s), *C = fws_d(a, ch.o_c);
    const double *logw = a.logw + ch.pix, *sqw = a.sqw + ch.pix, *sq = a.sqiv + ch.pix;
    const double *stab = a.signal ? a.signal + (size_t) ch.res * a.grid.nv * a.grid.nzp : nullptr;
    const DeviceBins &bins = *a.bins;
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
        if (a.theta) {
            // sum_s theta_s Q_s (core/chunk_estimate.cpp:674-683): interpolation is
            // linear, so the k bands of one redshift bin come from one
            // theta-weighted table row, r_T(v) = sum_kn theta_kn r_kn(v)
            int nidx;
            double dn;
            vindex(a.grid, v, nidx, dn);
            const int nzb = ch.ns / ch.kbin_upp;
            for (int iz = 0; iz < nzb; ++iz) {
                const double *row = a.ttab + ((size_t) ch.tcombo * bins.nz + ch.zb0 + iz) * a.grid.nv;
                const double w = zfactor(bins, ch.zb0 + iz, z);
                if (w != 0.0) cv += (row[nidx] * (1 - dn) + row[nidx + 1] * dn) * w;
            }
        }
        const double di = sq[i], dj = sq[j];
        C[idx] = di * cv * dj + (i == j ? 1.0 : 0.0);
    }
}

// Phase A, mixed path without theta: S and C~ = D S D + I in double-float
// arithmetic on the FP32 pipe (48 significant bits; FP64 is 1/60 of the FP32
// rate here), written as (hi, lo) float pairs in the 8 bytes of each element,
// the form the mixed factorisation works in.  v_ij / dv, (z_ij - z1) / dz, the
// interpolation fractions and the table values are all double-float.
__global__ void k_build_s_c_ff(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr || ch.nelem > 0) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    float2 *S = reinterpret_cast<float2 *>(a.fws + ch.o_s), *C = reinterpret_cast<float2 *>(a.fws + ch.o_c);
    const float2 *lw = a.logw2 + ch.pix, *sw = a.sqw2 + ch.pix, *sq = a.sqiv2 + ch.pix;
    const TableGrid &gr = a.grid;
    const float2 *tab = (a.signal_ff && !a.turn_off_sfid) ? a.signal_ff + (size_t) ch.res * gr.nv * gr.nzp : nullptr;
    const float2 kv = make_float2(gr.kv_hi, gr.kv_lo), z1p = make_float2(gr.z1p_hi, gr.z1p_lo);
    const float2 idz = make_float2(gr.idz_hi, gr.idz_lo), one = make_float2(1.f, 0.f), zero = make_float2(0.f, 0.f);
    for (int e = threadIdx.x; e < T64 * T64; e += blockDim.x) {
        const int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        const size_t idx = (size_t) i * ld + j;
        if (i >= n || j >= n) {
            S[idx] = zero;
            C[idx] = (i == j) ? one : zero;
            continue;
        }
        float2 val = zero;
        if (tab) {
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            const float2 yy = ff_mul(ff_sub(lw[hi], lw[lo]), kv);               // v / dv
            float zp, ze;
            two_prod_ff(sw[lo], sw[hi], zp, ze);                                // 1 + z
            const float2 xx = ff_mul(ff_sub(ff_norm(zp, ze), z1p), idz);         // (z - z1) / dz
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
        S[idx] = val;
        float2 sv = a.turn_off_sfid ? zero : val;
        if (a.ttab_ff) {
            // sum_s theta_s Q_s from the theta-weighted rows (see k_build_s_c), in
            // double-float: the row interpolated at v (the signal table's v grid),
            // times the redshift weight (and growth factor)
            const int lo = i < j ? i : j, hi = i < j ? j : i;
            float2 fv;
            int nvx;
            ff_index(ff_mul(ff_sub(lw[hi], lw[lo]), kv), gr.nv - 2, nvx, fv);
            float zp, ze;
            two_prod_ff(sw[lo], sw[hi], zp, ze);
            const DeviceBins &bins = *a.bins;
            const int nzb = ch.ns / ch.kbin_upp;
            for (int iz = 0; iz < nzb; ++iz) {
                float2 w = zweight_dd(bins, ch.zb0 + iz, zp, ze);
                if (w.x == 0.f) continue;
                if (bins.growth) {
                    const double z1 = (double) zp + (double) ze;
                    w = ff_mul(w, ff_of(pow(z1 / (bins.z_centers[ch.zb0 + iz] + 1.0), bins.growth_b)));
                }
                const float2 *row = a.ttab_ff + ((size_t) ch.tcombo * bins.nz + ch.zb0 + iz) * gr.nv;
                const float2 r0 = row[nvx], r1 = row[nvx + 1];
                sv = ff_add(sv, ff_mul(ff_add(r0, ff_mul(ff_sub(r1, r0), fv)), w));
            }
        }
        float2 cv = ff_mul(ff_mul(sq[i], sv), sq[j]);
        if (i == j) cv = ff_add(cv, one);
        C[idx] = cv;
    }
}

// ---------------------------------------------------------------------------
// Phase B, K1b: stored derivative matrices Q_s (Chunk::_setQiMatrix and
// _applyRedshiftInterp, core/chunk_estimate.cpp:429-536) and per-warp partial
// sums of d_s = y^T Q_s y (computePSbeforeFvector, :754-759).  Q_s at
// (i, j) is the k-band row of the derivative table interpolated at v_ij times
// the redshift weight of bin iz at z_ij; the interpolation index and the
// interpolated row value are computed once per element and k band and reused
// by every redshift bin.
//
// FP64 variant: each thread owns 16 elements of a 64 x 64 tile.
constexpr int QEPT = T64 * T64 / 256;

__global__ void __launch_bounds__(256) k_build_q(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr || a.status[ch.gidx] != LQG_CHUNK_OK || ch.nelem > 0) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    const DeviceBins &bins = *a.bins;
    const double *logw = a.logw + ch.pix, *sqw = a.sqw + ch.pix;
    const double *y = fws_d(a, ch.o_y);
    const int nzb = ch.ns / ch.kbin_upp;
    int nidx[QEPT];
    double dn[QEPT], yy[QEPT], zz[QEPT];
    size_t off[QEPT];
    bool valid[QEPT];
#pragma unroll
    for (int u = 0; u < QEPT; ++u) {
        int e = threadIdx.x + u * 256;
        int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        off[u] = (size_t) i * ld + j;
        valid[u] = i < n && j < n;
        nidx[u] = 0; dn[u] = 0; zz[u] = 0; yy[u] = 0;
        if (valid[u]) {
            int lo = i < j ? i : j, hi = i < j ? j : i;
            double v, z;
            vz_of(logw, sqw, lo, hi, v, z);
            vindex(a.grid, v, nidx[u], dn[u]);
            zz[u] = z;
            yy[u] = y[i] * y[j];
        }
    }
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    double *dpart = ws_d(a, ch.o_dpart) + ((size_t) blockIdx.x * 8 + warp) * ch.ns;
    const size_t plane = (size_t) ld * ld;
    const double *rows = a.deriv + (size_t) ch.res * bins.nk * a.grid.nv;
    for (int kn = 0; kn < ch.kbin_upp; ++kn) {
        const double *row = rows + (size_t) kn * a.grid.nv;
        double base[QEPT];
#pragma unroll
        for (int u = 0; u < QEPT; ++u)
            base[u] = valid[u] ? row[nidx[u]] * (1 - dn[u]) + row[nidx[u] + 1] * dn[u] : 0.0;
        for (int iz = 0; iz < nzb; ++iz) {
            const int s = iz * ch.kbin_upp + kn, zm = ch.zb0 + iz;
            double *Q = ws_d(a, ch.o_q) + (size_t) s * plane;
            double part = 0.0;
#pragma unroll
            for (int u = 0; u < QEPT; ++u) {
                const double q = valid[u] ? base[u] * zfactor(bins, zm, zz[u]) : 0.0;
                part += yy[u] * q;
                Q[off[u]] = q;
            }
            part = warp_sum(part);
            if (lane == 0) dpart[s] = part;
        }
    }
}

// Mixed variant: Q_s straight to fp16 hi/lo planes with the slot's power-of-two
// scale.  The operands of a 22-bit split need no FP64: interpolation and
// weights run in FP32 (GB300's FP64 rate is 1/60 of its FP32 rate) from a
// float copy of the derivative table.  The redshift weights are evaluated from
// the FP64 z_ij (once per element and bin): a float z carries 2.4e-7 absolute
// error, which is 1e-4 relative on the small weights near a bin's edge.
// Each thread owns 4 column pairs of a
// 32 x 64 half tile (one row per warp and pair step, stores of 128 B per warp);
// redshift bins are taken kZGroup at a time with their weights in registers.
constexpr int QM_PAIRS = 4;
constexpr int kZGroup = 4;

// GR: with the redshift-growth factor (its own instantiation, so that the
// common case carries none of its code).
template <bool GR>
__global__ void __launch_bounds__(256, 2) k_build_q_mixed(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    const int tile = blockIdx.x >> 1, hrow = (blockIdx.x & 1) * 32;
    if (tile >= tpr * tpr || a.status[ch.gidx] != LQG_CHUNK_OK || ch.nelem > 0) return;
    const int ti = tile / tpr, tj = tile % tpr;
    const DeviceBins &bins = *a.bins;
    const float2 *lw2 = a.logw2 + ch.pix, *sw2 = a.sqw2 + ch.pix;
    const int nzb = ch.ns / ch.kbin_upp;
    constexpr int E = 2 * QM_PAIRS;
    int nidx[E];
    float dnf[E];
    float zp[E], ze[E];      // 1 + z_ij as double-float; zp = 0 marks padding
    size_t off[QM_PAIRS];    // element offset of each pair's first element
#pragma unroll
    for (int u = 0; u < QM_PAIRS; ++u) {
        const int p = threadIdx.x + 256 * u;
        const int i = ti * T64 + hrow + p / 32, j0 = tj * T64 + 2 * (p % 32);
        off[u] = (size_t) i * ld + j0;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int k = 2 * u + e, j = j0 + e;
            nidx[k] = 0; dnf[k] = 0.f; zp[k] = 0.f; ze[k] = 0.f;
            if (i < n && j < n) {
                const int lo = i < j ? i : j, hi = i < j ? j : i;
                vindex_ff(a.grid, lw2[hi], lw2[lo], nidx[k], dnf[k]);
                two_prod_ff(sw2[i], sw2[j], zp[k], ze[k]);
            }
        }
    }
    const size_t plane = (size_t) ld * ld;
    const float *rows = a.deriv_f + (size_t) ch.res * bins.nk * a.grid.nv;
    // slot scales as floats, converted once per block
    __shared__ float qscale[kMaxGramBlocks * 128];
    for (int t = threadIdx.x; t < ch.ns; t += blockDim.x)
        qscale[t] = (float) a.scales[(size_t) 4 * a.n_chunks + ch.slot_q + t];
    __syncthreads();
    for (int z0 = 0; z0 < nzb; z0 += kZGroup) {
        float w[kZGroup][E];
#pragma unroll
        for (int g = 0; g < kZGroup; ++g)
#pragma unroll
            for (int k = 0; k < E; ++k)
                w[g][k] = (z0 + g < nzb && zp[k] > 0.f) ? (GR ? zfactor_ff(bins, ch.zb0 + z0 + g, zp[k], ze[k])
                                                              : zweight_ff(bins, ch.zb0 + z0 + g, zp[k], ze[k]))
                                                         : 0.f;
        // the node pairs of band kn are loaded while band kn - 1 is stored
        float r0[E], r1[E];
#pragma unroll
        for (int k = 0; k < E; ++k) { r0[k] = rows[nidx[k]]; r1[k] = rows[nidx[k] + 1]; }
        for (int kn = 0; kn < ch.kbin_upp; ++kn) {
            float base[E];
#pragma unroll
            for (int k = 0; k < E; ++k) base[k] = fmaf(r1[k] - r0[k], dnf[k], r0[k]);
            if (kn + 1 < ch.kbin_upp) {
                const float *next = rows + (size_t) (kn + 1) * a.grid.nv;
#pragma unroll
                for (int k = 0; k < E; ++k) { r0[k] = next[nidx[k]]; r1[k] = next[nidx[k] + 1]; }
            }
#pragma unroll
            for (int g = 0; g < kZGroup; ++g) {
                if (z0 + g >= nzb) break;
                const int s = (z0 + g) * ch.kbin_upp + kn;
                const float qs = qscale[s];
                uint32_t *qh = reinterpret_cast<uint32_t *>(a.q_hi + (size_t) (ch.slot_q + s) * plane);
                uint32_t *ql = reinterpret_cast<uint32_t *>(a.q_lo + (size_t) (ch.slot_q + s) * plane);
#pragma unroll
                for (int u = 0; u < QM_PAIRS; ++u) {
                    const float q0 = base[2 * u] * w[g][2 * u], q1 = base[2 * u + 1] * w[g][2 * u + 1];
                    if (!LQG_IN_BOUNDS(a, (size_t) (ch.slot_q + s) * plane + off[u] + 1 <
                                              (size_t) a.total_slots_q * plane, 5, c, off[u]))
                        continue;
                    const __half2 hv = __floats2half2_rn(q0 * qs, q1 * qs);
                    const float2 hf = __half22float2(hv);
                    const __half2 lv = __floats2half2_rn(q0 * qs - hf.x, q1 * qs - hf.y);
                    qh[off[u] / 2] = *reinterpret_cast<const uint32_t *>(&hv);
                    ql[off[u] / 2] = *reinterpret_cast<const uint32_t *>(&lv);
                }
            }
        }
    }
}

// Mixed path, the d and x partials in double-float arithmetic on the FP32 pipe:
//   d_s = y^T Q_s y       (computePSbeforeFvector, core/chunk_estimate.cpp:754-759)
//   x_s = tr(Q_s C^-1) = sum_ij Q_s,ij C^-1_ij   (C^-1 marginalised, when cinv_m)
// over the upper triangle, off-diagonal elements counted twice.  k_finish_dx
// forms d - b - t = d - x + (F theta) from them (b_s + t_s = tr(C^-1 Q_s C^-1 (S +
// N)) with C^-1 C C^-1 = C^-1), a difference much smaller than its terms on
// high signal-to-noise chunks: a float Q_s (2^-24) or float y y^T - C^-1 already
// moves it by ~2e-7 of max |b| (CPU emulation on echelle-size chunks), so Q_s
// (table value, interpolation fraction and redshift weight), y_i y_j, C^-1_ij
// and the accumulation are all double-float (~48 bits).  No FP64 work in the
// slot loop (the FP64 pipe is 1/64 of the FP32 one).  The block's sums go
// through shared memory kDxBatch slots at a time: every thread stores its
// (d, x) double-float pair of each slot of the batch, then warp w adds slot w
// of the batch (each lane 8 of the 256 values in a fixed order, then a
// double-float warp sum), so one warp sum serves 256 values instead of 32.
// Each block (half tile) stores one (hi, lo) pair per slot in an 8-byte
// partial slot: part 2 tile + half.  Blocks of lower tiles write nothing.
constexpr int DX_E = 8;   // elements per thread: rows warp + 8u (u < 4), columns 2 lane, 2 lane + 1
constexpr int kDxBatch = 8;   // slots per shared-memory reduction (one per warp)

template <bool GR>
__global__ void __launch_bounds__(256, 2) k_dx_mixed(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    const int tile = blockIdx.x >> 1, hrow = (blockIdx.x & 1) * 32;
    if (tile >= tpr * tpr || a.status[ch.gidx] != LQG_CHUNK_OK || ch.nelem > 0) return;
    const int ti = tile / tpr, tj = tile % tpr;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const bool want_x = a.dbt_id && ch.cinv_m;
    double *dpart = ws_d(a, ch.o_dpart) + (size_t) blockIdx.x * ch.ns;
    double *xpart = want_x ? ws_d(a, ch.o_xpart) + (size_t) blockIdx.x * ch.ns : nullptr;
    if (ti > tj) return;   // counted through the mirrored upper tile; k_finish_dx skips these parts
    const DeviceBins &bins = *a.bins;
    const float2 *lw2 = a.logw2 + ch.pix, *sw2 = a.sqw2 + ch.pix;
    const double *y = fws_d(a, ch.o_y);
    const double *cm = want_x ? fws_d(a, ch.o_m) : nullptr;
    const int nzb = ch.ns / ch.kbin_upp;
    int nidx[DX_E];
    float2 dn[DX_E], yy[DX_E], cmv[DX_E];
    float zp[DX_E], ze[DX_E];   // 1 + z_ij as double-float; zp = 0: no element
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int i = ti * T64 + hrow + warp + 8 * u;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            const int k = 2 * u + e, j = tj * T64 + 2 * lane + e;
            nidx[k] = 0;
            dn[k] = yy[k] = cmv[k] = make_float2(0.f, 0.f);
            zp[k] = ze[k] = 0.f;
            // weight of the element in the full sum: 2 above the diagonal, 1 on it
            const double wt = (i < n && j < n) ? (i < j ? 2.0 : (i == j ? 1.0 : 0.0)) : 0.0;
            if (wt == 0.0) continue;
            vindex_dd(a.grid, lw2[j], lw2[i], nidx[k], dn[k]);
            two_prod_ff(sw2[i], sw2[j], zp[k], ze[k]);
            yy[k] = ff_of(wt * y[i] * y[j]);
            if (want_x) cmv[k] = ff_of(wt * cm[(size_t) i * ld + j]);
        }
    }
    const float4 *rows = a.deriv_ff + (size_t) ch.res * bins.nk * a.grid.nv;
    // (d hi, d lo, x hi, x lo) of every thread for the slots of one batch
    __shared__ float4 red[kDxBatch][256];
    for (int iz = 0; iz < nzb; ++iz) {
        float2 w[DX_E];
#pragma unroll
        for (int k = 0; k < DX_E; ++k) {
            w[k] = make_float2(0.f, 0.f);
            if (zp[k] > 0.f) {
                w[k] = zweight_dd(bins, ch.zb0 + iz, zp[k], ze[k]);
                if (GR && w[k].x != 0.f) {
                    const double z1 = (double) zp[k] + (double) ze[k];
                    w[k] = ff_mul(w[k], ff_of(pow(z1 / (bins.z_centers[ch.zb0 + iz] + 1.0), bins.growth_b)));
                }
            }
        }
        for (int kn = 0; kn < ch.kbin_upp; ++kn) {
            const float4 *row = rows + (size_t) kn * a.grid.nv;
            float sd = 0.f, cd = 0.f, sx = 0.f, cx = 0.f;
#pragma unroll
            for (int k = 0; k < DX_E; ++k) {
                if (w[k].x == 0.f) continue;
                // the reference's r0 (1 - dn) + r1 dn, as r0 + (r1 - r0) dn with
                // the node's difference stored: product (p, e), then two-sum
                const float4 r = row[nidx[k]];
                float p, e;
                two_prod_ff(make_float2(r.z, r.w), dn[k], p, e);
                const float2 s0 = ff_two_sum(r.x, p);
                const float2 base = make_float2(s0.x, __fadd_rn(s0.y, __fadd_rn(r.y, e)));
                float qp, qe;
                two_prod_ff(base, w[k], qp, qe);
                dd_mac(sd, cd, qp, qe, yy[k]);
                if (want_x) dd_mac(sx, cx, qp, qe, cmv[k]);
            }
            const int b = kn % kDxBatch;
            red[b][threadIdx.x] = make_float4(sd, cd, sx, cx);
            if (b != kDxBatch - 1 && kn != ch.kbin_upp - 1) continue;
            // the batch is complete: warp w adds the 256 values of its slot
            __syncthreads();
            if (warp <= b) {
                float2 dv = make_float2(0.f, 0.f), xv = make_float2(0.f, 0.f);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 v = red[warp][lane + 32 * q];
                    const float2 ds = ff_two_sum(dv.x, v.x), xs = ff_two_sum(xv.x, v.z);
                    dv = ff_norm(ds.x, __fadd_rn(ds.y, __fadd_rn(dv.y, v.y)));
                    xv = ff_norm(xs.x, __fadd_rn(xs.y, __fadd_rn(xv.y, v.w)));
                }
                const int s = iz * ch.kbin_upp + kn - b + warp;
                dv = warp_sum_ff(dv);
                if (lane == 0) reinterpret_cast<float2 *>(dpart)[s] = dv;
                if (want_x) {
                    xv = warp_sum_ff(xv);
                    if (lane == 0) reinterpret_cast<float2 *>(xpart)[s] = xv;
                }
            }
            __syncthreads();
        }
    }
}

// Mixed path: C^-1 and S to fp16 hi/lo planes, C^-1 N into its R slot.
__global__ void k_prep_mixed(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n, tpr = ld / T64;
    if ((int) blockIdx.x >= tpr * tpr || a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int ti = blockIdx.x / tpr, tj = blockIdx.x % tpr;
    const double *A = fws_d(a, ch.o_c), *S = fws_d(a, ch.o_s);
    const double *sc = a.scales + 4 * c;
    const double cs = sc[2], wsc = sc[3];
    const double ss = a.scales[(size_t) 4 * a.n_chunks + ch.slot_q + ch.ns];
    const size_t plane = (size_t) ld * ld;
    for (int e = threadIdx.x; e < T64 * T64; e += blockDim.x) {
        int i = ti * T64 + e / T64, j = tj * T64 + e % T64;
        size_t idx = (size_t) i * ld + j;
        if (!LQG_IN_BOUNDS(a, (size_t) c * plane + idx < (size_t) a.n_chunks * plane &&
                                  (size_t) (ch.slot_q + ch.ns) * plane + idx < (size_t) a.total_slots_q * plane &&
                                  (size_t) (ch.slot_r + ch.ns + 1) * plane + idx < (size_t) a.total_slots_r * plane,
                           6, c, idx))
            continue;
        double cv = A[idx];
        float x = (float) (cv * cs);
        __half h = __float2half_rn(x);
        a.c_hi[(size_t) c * plane + idx] = h;
        a.c_lo[(size_t) c * plane + idx] = __float2half_rn(x - __half2float(h));
        float xs;
        if (a.c_is_ff) {
            const float2 s2 = reinterpret_cast<const float2 *>(S)[idx];
            xs = __fadd_rn(s2.x, s2.y) * (float) ss;
        } else {
            xs = (float) (S[idx] * ss);
        }
        __half hs = __float2half_rn(xs);
        a.q_hi[(size_t) (ch.slot_q + ch.ns) * plane + idx] = hs;
        a.q_lo[(size_t) (ch.slot_q + ch.ns) * plane + idx] = __float2half_rn(xs - __half2float(hs));
        // C^-1 N (column j scaled by 1 / ivar_j) into R slot ns + 1
        const double nw = j < n ? a.niv[ch.pix + j] : 0.0;
        float xw = (float) (cv * nw * wsc);
        __half hw = __float2half_rn(xw);
        a.r_hi[(size_t) (ch.slot_r + ch.ns + 1) * plane + idx] = hw;
        a.r_lo[(size_t) (ch.slot_r + ch.ns + 1) * plane + idx] = __float2half_rn(xw - __half2float(hw));
    }
}

// FP64 path: W_N = N C^-1 (core/chunk_estimate.cpp:767-781) into its P slot.
__global__ void k_wn_fp64(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int ld = ch.ld, n = ch.n;
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const double *A = fws_d(a, ch.o_c);
    double *P = ws_d(a, ch.o_p) + (size_t) (ch.ns + 1) * ld * ld;
    for (size_t e = (size_t) blockIdx.x * blockDim.x + threadIdx.x; e < (size_t) ld * ld;
         e += (size_t) gridDim.x * blockDim.x) {
        int i = (int) (e / ld);
        const double nw = i < n ? a.niv[ch.pix + i] : 0.0;
        P[e] = nw * A[e];
    }
}

// ---------------------------------------------------------------------------
// FP64 products: A_s = C^-1 Q_s (s < ns) and A_S = C^-1 S; the epilogue writes
// A_s to R (row-major) and A_s^T to P.  64 x 64 output tiles, 4 x 4 per thread.
constexpr int GT = 64, GK = 16;

__global__ void __launch_bounds__(256) k_dgemm(WaveArgs a, const int *jobs, int njobs) {
    const int job = blockIdx.y;
    if (job >= njobs) return;
    const int c = jobs[2 * job], s = jobs[2 * job + 1];
    const ChunkDesc &ch = a.chunks[c];
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int ld = ch.ld, tpr = ld / GT;
    if ((int) blockIdx.x >= tpr * tpr) return;
    const int tm = blockIdx.x / tpr, tn = blockIdx.x % tpr;
    const double *A = fws_d(a, ch.o_c);
    const double *B = (s < ch.ns) ? ws_d(a, ch.o_q) + (size_t) s * ld * ld : fws_d(a, ch.o_s);
    // operand tiles during the K loop, the output tile (transposed store) afterwards
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
    double *R = ws_d(a, ch.o_r) + (size_t) s * ld * ld;
    double *P = ws_d(a, ch.o_p) + (size_t) s * ld * ld;
    __syncthreads();
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) {
            Ot[tr + u][tc + w] = acc[u][w];
            if (s < ch.ns) R[(size_t) (tm * GT + tr + u) * ld + tn * GT + tc + w] = acc[u][w];
        }
    __syncthreads();
    for (int e = threadIdx.x; e < GT * GT; e += blockDim.x) {
        int nn = e / GT, mm = e % GT;
        P[(size_t) (tn * GT + nn) * ld + tm * GT + mm] = Ot[mm][nn];
    }
}

// FP64 Gram, G[i][j] = <P_i, R_j> over one K split and one 128 x 128 block of (i, j).
__global__ void __launch_bounds__(256) k_dgram(WaveArgs a) {
    const int c = blockIdx.y, sp = blockIdx.x, blk = blockIdx.z;
    const ChunkDesc &ch = a.chunks[c];
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int bi = blk / a.gt, bj = blk % a.gt;
    const int mi = ch.ns + 2, mj = ch.ns;
    if (bi * GR >= mi || bj * GR >= mj) return;
    const int64_t K = (int64_t) ch.ld * ch.ld;
    const int64_t kper = (K + a.gram_splits - 1) / a.gram_splits;
    const int64_t k_lo = sp * kper, k_hi = min(K, k_lo + kper);
    const double *P = ws_d(a, ch.o_p), *R = ws_d(a, ch.o_r);
    __shared__ double Ps[8][GR + 1], Rs[8][GR + 1];
    const int tr = (threadIdx.x / 16) * 8, tc = (threadIdx.x % 16) * 8;
    double acc[8][8] = {};
    for (int64_t k0 = k_lo; k0 < k_hi; k0 += 8) {
        for (int e = threadIdx.x; e < GR * 8; e += blockDim.x) {
            int r = e / 8, kk = e % 8;
            int64_t k = k0 + kk;
            int ri = bi * GR + r, rj = bj * GR + r;
            Ps[kk][r] = (ri < mi && k < k_hi) ? P[(size_t) ri * K + k] : 0.0;
            Rs[kk][r] = (rj < mj && k < k_hi) ? R[(size_t) rj * K + k] : 0.0;
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
    double *out = ws_d(a, ch.o_part) + ((size_t) blk * a.gram_splits + sp) * GR * GR;
#pragma unroll
    for (int u = 0; u < 8; ++u)
#pragma unroll
        for (int w = 0; w < 8; ++w) out[(tr + u) * GR + tc + w] = acc[u][w];
}

// ---------------------------------------------------------------------------
// Element (i, j) of chunk c's trace Gram on the mixed path, from its fp32 split
// partials in fixed order, unscaled: F_ij (j < ns), t_i (j = ns), b_i (j = ns + 1).
__device__ __forceinline__ double gram_mixed(const WaveArgs &a, const ChunkDesc &ch, int c, int i, int j) {
    const double *psc = a.scales + (size_t) 4 * a.n_chunks + a.total_slots_q + ch.slot_p;
    const double *rsc = a.sym ? psc
                              : a.scales + (size_t) 4 * a.n_chunks + a.total_slots_q + a.total_slots_p + ch.slot_r;
    const size_t blkstride = (size_t) a.gram_splits * GR * GR;
    const int blk = (i / GR) * a.gt + j / GR, li = i % GR, lj = j % GR;
    const float *gp = a.gram_part + ((size_t) c * a.gt * a.gt + blk) * blkstride;
    double acc = 0;
    for (int sp = 0; sp < a.gram_splits; ++sp) acc += (double) gp[(size_t) sp * GR * GR + li * GR + lj];
    return acc / (psc[i] * rsc[j]);
}

// ---------------------------------------------------------------------------
// Per-chunk reduction of the Gram partials and d partials (fixed order), written
// in the reference's per-chunk layout (Chunk::dbt_estimate_before_fisher_vector
// and Chunk::fisher_matrix, upper triangle, not halved).
__global__ void k_finish(WaveArgs a, int mixed) {
    const int c = blockIdx.x;
    const ChunkDesc &ch = a.chunks[c];
    const DeviceBins &bins = *a.bins;
    const int nq = ch.nq;
    if (!LQG_IN_BOUNDS(a, ch.res_off + 3 * nq + (int64_t) nq * nq <= a.results_elems, 8, c, ch.res_off)) return;
    double *res = a.results + ch.res_off;
    double *d = res, *b = res + nq, *t = res + 2 * nq, *F = res + 3 * nq;
    for (int e = threadIdx.x; e < 3 * nq + nq * nq; e += blockDim.x) res[e] = 0.0;
    __syncthreads();
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    // d partials: 8 warps per 64 x 64 tile (FP64 build) or per 32 x 64 half tile (mixed)
    const int ns = ch.ns, parts = (ch.ld / T64) * (ch.ld / T64) * 8 * (mixed ? 2 : 1);
    const double *dpart = ws_d(a, ch.o_dpart);
    // the mixed path's table chunks: d (and d - b - t) in k_finish_dx
    if (!(mixed && ch.nelem == 0)) {
        // Sum of every slot's parts in a fixed order.  Thread t adds parts g, g + G,
        // ... of slot s0 + t % R (g = t / R, R slots per round, G = blockDim / R
        // groups), so that the threads of a group read consecutive slots of one
        // part; then the first R threads add the G group sums in order.
        __shared__ double red[256];
        const int R = min(ns, (int) blockDim.x), G = blockDim.x / R;
        const int g = threadIdx.x / R, sl = threadIdx.x % R;
        for (int s0 = 0; s0 < ns; s0 += R) {
            const int s = s0 + sl;
            if (g < G) {
                double acc = 0;
                if (s < ns)
                    for (int p = g; p < parts; p += G) acc += dpart[(size_t) p * ns + s];
                red[g * R + sl] = acc;
            }
            __syncthreads();
            if ((int) threadIdx.x < R && s0 + (int) threadIdx.x < ns) {
                double v = 0;
                for (int k = 0; k < G; ++k) v += red[k * R + threadIdx.x];
                const int sv = s0 + (int) threadIdx.x;
                d[(sv / ch.kbin_upp) * bins.nk + sv % ch.kbin_upp] = v;
            }
            __syncthreads();
        }
    }
    const size_t blkstride = (size_t) a.gram_splits * GR * GR;
    if (mixed) {
        // G = P R^T: P rows = A_i^T (i < ns), R rows = A_j (j < ns), C^-1 S, C^-1 N;
        // blocks bi <= bj only.  F_ij = G_ij (i <= j), t_i = G_{i,ns}, b_i = G_{i,ns+1}.
        // Whitened form: rows B_i of P on both sides (B_ns = W S W^T, B_{ns+1} = W N W^T).
        for (int e = threadIdx.x; e < ns * (ns + 2); e += blockDim.x) {
            const int i = e / (ns + 2), j = e % (ns + 2);
            if (j < ns && j < i) continue;
            const double g = gram_mixed(a, ch, c, i, j);
            const int ikz = (i / ch.kbin_upp) * bins.nk + i % ch.kbin_upp;
            if (j < ns) {
                const int jkz = (j / ch.kbin_upp) * bins.nk + j % ch.kbin_upp;
                if (!a.skip_fisher) F[(size_t) ikz * nq + jkz] = g;
            } else if (j == ns) {
                if (!a.turn_off_sfid) t[ikz] = g;
            } else {
                b[ikz] = g;
            }
        }
        return;
    }
    const int rows = ns + 2;
    for (int e = threadIdx.x; e < rows * ns; e += blockDim.x) {
        const int i = e / ns, j = e % ns;
        const int blk = (i / GR) * a.gt + j / GR, li = i % GR, lj = j % GR;
        double acc = 0;
        const double *gp = ws_d(a, ch.o_part) + blk * blkstride;
        for (int sp = 0; sp < a.gram_splits; ++sp) acc += gp[(size_t) sp * GR * GR + li * GR + lj];
        const int jkz = (j / ch.kbin_upp) * bins.nk + j % ch.kbin_upp;
        if (i < ns) {
            const int ikz = (i / ch.kbin_upp) * bins.nk + i % ch.kbin_upp;
            if (ikz <= jkz && !a.skip_fisher) F[(size_t) ikz * nq + jkz] = acc;
        } else if (i == ns) {
            if (!a.turn_off_sfid) t[jkz] = acc;
        } else {
            b[jkz] = acc;
        }
    }
}


// ---------------------------------------------------------------------------
// Mixed path, table chunks (after k_finish): d_s and x_s = tr(Q_s C^-1) from
// k_dx_mixed's (hi, lo) partials, one warp per slot.  The parts of a slot are
// the two half tiles of each upper 64 x 64 tile; a tile row's upper tiles are
// consecutive, so the lanes stride over them row by row, each lane adds its
// parts in order and the warp sums the lanes in a fixed tree.  Then d - b - t
// without the 22-bit traces: with C = S + N + sum_s theta_s Q_s (the stored
// slots) and the marginalised C^-1 (C^-1 C C^-1 = C^-1),
//   b_s + t_s = tr(C^-1 Q_s C^-1 (S + N)) = tr(Q_s C^-1) - sum_s' F_ss' theta_s',
// so e_s = d_s - b_s - t_s = d_s - x_s + (F theta)_s.  The larger of b_s and t_s
// (b_s alone without S_fid) takes the difference, so that d - b - t = e exactly
// and each keeps its own relative accuracy.
__global__ void __launch_bounds__(256) k_finish_dx(WaveArgs a) {
    const int c = blockIdx.y;
    const ChunkDesc &ch = a.chunks[c];
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int s = blockIdx.x * 8 + warp, ns = ch.ns, nq = ch.nq;
    if (ch.nelem > 0 || s >= ns || a.status[ch.gidx] != LQG_CHUNK_OK) return;
    if (!LQG_IN_BOUNDS(a, ch.res_off + 3 * nq + (int64_t) nq * nq <= a.results_elems, 8, c, ch.res_off)) return;
    const DeviceBins &bins = *a.bins;
    double *res = a.results + ch.res_off;
    double *d = res, *b = res + nq, *t = res + 2 * nq, *F = res + 3 * nq;
    const bool want_x = a.dbt_id && ch.cinv_m;
    const int tpr = ch.ld / T64;
    const float2 *dp = reinterpret_cast<const float2 *>(ws_d(a, ch.o_dpart));
    const float2 *xp = want_x ? reinterpret_cast<const float2 *>(ws_d(a, ch.o_xpart)) : nullptr;
    double dsum = 0, xsum = 0;
    for (int ti = 0; ti < tpr; ++ti) {
        const int p1 = (ti * tpr + tpr) * 2;
        for (int p = (ti * tpr + ti) * 2 + lane; p < p1; p += 32) {
            const float2 v = dp[(size_t) p * ns + s];
            dsum += (double) v.x + (double) v.y;
            if (want_x) {
                const float2 u = xp[(size_t) p * ns + s];
                xsum += (double) u.x + (double) u.y;
            }
        }
    }
    dsum = warp_sum(dsum);
    const int ikz = (s / ch.kbin_upp) * bins.nk + s % ch.kbin_upp;
    if (!want_x) {
        if (lane == 0) d[ikz] = dsum;
        return;
    }
    xsum = warp_sum(xsum);
    // (F theta)_s from F as k_finish wrote it (upper triangle), else from the Gram partials
    double ft = 0;
    if (a.theta)
        for (int s2 = lane; s2 < ns; s2 += 32) {
            const int jkz = (s2 / ch.kbin_upp) * bins.nk + s2 % ch.kbin_upp;
            const double th = a.theta[ch.fis + jkz];
            if (th == 0.0) continue;
            const int lo = min(ikz, jkz), hi = max(ikz, jkz);
            ft += th * (a.skip_fisher ? gram_mixed(a, ch, c, min(s, s2), max(s, s2)) : F[(size_t) lo * nq + hi]);
        }
    ft = warp_sum(ft);
    if (lane != 0) return;
    d[ikz] = dsum;
    const double e = dsum - xsum + ft, bt = dsum - e;
    if (a.turn_off_sfid) b[ikz] = bt;
    else if (fabs(b[ikz]) >= fabs(t[ikz])) b[ikz] = bt - t[ikz];
    else t[ikz] = bt - b[ikz];
}

}  // namespace

void launch_theta_tables(const double *deriv, const double *theta, const int *combos, int n_combos, int nk, int nz,
                         int nv, double *ttab, float2 *ttab_ff, cudaStream_t st) {
    k_theta_tables<<<dim3((nv + 255) / 256, nz, n_combos), 256, 0, st>>>(deriv, theta, combos, nk, nz, nv, ttab,
                                                                        ttab_ff);
}

void launch_build_s_c(WaveArgs &a, cudaStream_t st) {
    int tiles = (a.max_ld / T64) * (a.max_ld / T64);
    if (a.c_is_ff)
        k_build_s_c_ff<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
    else
        k_build_s_c<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
    a.launches++;
}

void launch_build_q(WaveArgs &a, cudaStream_t st) {
    int tiles = (a.max_ld / T64) * (a.max_ld / T64);
    if (a.precision == LQG_PRECISION_MIXED) {
        k_prep_mixed<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
        if (a.growth) {
            k_build_q_mixed<true><<<dim3(2 * tiles, a.n_chunks), 256, 0, st>>>(a);
            k_dx_mixed<true><<<dim3(2 * tiles, a.n_chunks), 256, 0, st>>>(a);
        } else {
            k_build_q_mixed<false><<<dim3(2 * tiles, a.n_chunks), 256, 0, st>>>(a);
            k_dx_mixed<false><<<dim3(2 * tiles, a.n_chunks), 256, 0, st>>>(a);
        }
        a.launches++;
    } else {
        k_build_q<<<dim3(tiles, a.n_chunks), 256, 0, st>>>(a);
        k_wn_fp64<<<dim3(64, a.n_chunks), 256, 0, st>>>(a);
    }
    a.launches += 2;
}

void launch_products_fp64(WaveArgs &a, cudaStream_t st, const int *d_jobs, int njobs) {
    int tiles = (a.max_ld / GT) * (a.max_ld / GT);
    k_dgemm<<<dim3(tiles, njobs), 256, 0, st>>>(a, d_jobs, njobs);
    if (a.mid_event) record_event(a.mid_event, st);
    k_dgram<<<dim3(a.gram_splits, a.n_chunks, a.gt * a.gt), 256, 0, st>>>(a);
    a.launches += 2;
}

void launch_finish(WaveArgs &a, cudaStream_t st) {
    k_finish<<<a.n_chunks, 256, 0, st>>>(a, a.precision == LQG_PRECISION_MIXED);
    a.launches++;
    if (a.precision == LQG_PRECISION_MIXED && a.max_ns > 0) {
        k_finish_dx<<<dim3((a.max_ns + 7) / 8, a.n_chunks), 256, 0, st>>>(a);
        a.launches++;
    }
}

}  // namespace lqg
