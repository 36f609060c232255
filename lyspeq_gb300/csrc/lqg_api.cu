// Host side of the C ABI declared in include/lqg.h.
#include "lqg_internal.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <numeric>

using namespace lqg;

struct lqg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    // binning
    int nk = 0, nz = 0, nkz = 0, triangular = 1;
    double dz = 0;
    std::vector<double> k_edges, k_centers, z_centers;
    // tables
    int n_tables = 0, nv = 0, nzp = 0;
    double lenv = 0;
    std::vector<int> r_fwhm;
    std::vector<double> tdv, qmax, smax;
    TableGrid grid{};
    DevBuf d_deriv, d_signal, d_bins;
    lqg_opts opts{};
    // batch
    struct HostChunk {
        int n, ld, nq, ns, kbin_upp, fis, res, zlow, zupp, input_index;
        int64_t pix, res_off;
    };
    std::vector<HostChunk> chunks;
    std::vector<double> h_wave, h_delta, h_ivar, h_logw, h_sqw;
    bool pix_dirty = true;
    DevBuf d_wave, d_delta, d_ivar, d_logw, d_sqw;
    int64_t results_size = 0;
    DevBuf d_results, d_status, d_theta, d_fisher, d_dbt, d_meta;
    // workspace
    DevBuf d_ws, d_desc, d_jobs, d_scales, d_halves, d_gram, d_wstat, d_check;
    std::vector<int> last_status;
    double timings[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int launches = 0;
    cudaEvent_t ev[8] = {};
};

namespace {

int set_err(lqg_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

double median_of(std::vector<double> v) {
    std::sort(v.begin(), v.end());
    size_t n = v.size();
    if (n == 0) return -1;
    return (n % 2 == 0) ? (v[n / 2 - 1] + v[n / 2]) / 2 : v[n / 2];
}

// bins::findRedshiftBin, core/global_numbers.cpp:344-355
int find_redshift_bin(const lqg_ctx *ctx, double z) {
    double zlow = ctx->z_centers[0] - ctx->dz / 2.0;
    if (z < zlow) return -1;
    int r = (int) ((z - zlow) / ctx->dz);
    return std::min(r, ctx->nz);
}

double pow2_scale(double bound, double target) {
    if (!(bound > 0) || !std::isfinite(bound)) return 1.0;
    return std::ldexp(1.0, (int) std::floor(std::log2(target / bound)));
}

}  // namespace

extern "C" int lqg_abi_version(void) { return LQG_ABI_VERSION; }

extern "C" const char *lqg_last_error(const lqg_ctx *ctx) {
    return ctx ? ctx->err.c_str() : "null context";
}

extern "C" int lqg_ctx_create(lqg_ctx **out, const lqg_bins *bins, const lqg_tables *tables,
                              const lqg_opts *opts, int device) {
    if (!out || !bins || !tables || !opts) return LQG_ERR_ARG;
    *out = nullptr;
    if (bins->nk <= 0 || bins->nz <= 0 || bins->nz > 64 || !bins->k_edges || !bins->z_centers ||
        !(bins->z_bin_width > 0))
        return LQG_ERR_ARG;
    if (tables->n_tables <= 0 || tables->nv < 2 || tables->nzp < 2 || !tables->deriv ||
        !tables->r_fwhm || !tables->dv || !(tables->v_length > 0))
        return LQG_ERR_ARG;
    if (!opts->turn_off_sfid && !tables->signal) return LQG_ERR_ARG;
    {
        // specifics::calcNvecs, core/global_numbers.cpp:78-90
        int nvec = 0;
        if (opts->cont_logl_order >= 0 || opts->cont_l_order >= 0)
            nvec = 1 + std::max(opts->cont_logl_order, 0) + std::max(opts->cont_l_order, 0);
        if (nvec > kMaxContVecs) return LQG_ERR_UNSUPPORTED;
    }
    if (!(opts->max_mean_pixel_size > 0) || !(opts->max_forest_length >= 0)) return LQG_ERR_ARG;
    auto ctx = std::make_unique<lqg_ctx>();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) return LQG_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return LQG_ERR_CUDA;
    for (auto &e : ctx->ev) cudaEventCreate(&e);
    ctx->nk = bins->nk;
    ctx->nz = bins->nz;
    ctx->nkz = bins->nk * bins->nz;
    ctx->dz = bins->z_bin_width;
    ctx->triangular = bins->triangular;
    ctx->k_edges.assign(bins->k_edges, bins->k_edges + bins->nk + 1);
    for (int k = 0; k < bins->nk; ++k)
        ctx->k_centers.push_back((ctx->k_edges[k] + ctx->k_edges[k + 1]) / 2.);
    ctx->z_centers.assign(bins->z_centers, bins->z_centers + bins->nz);
    ctx->n_tables = tables->n_tables;
    ctx->nv = tables->nv;
    ctx->nzp = tables->nzp;
    ctx->lenv = tables->v_length;
    ctx->r_fwhm.assign(tables->r_fwhm, tables->r_fwhm + tables->n_tables);
    ctx->tdv.assign(tables->dv, tables->dv + tables->n_tables);
    ctx->opts = *opts;
    // interpolation grids, core/sq_table.cpp:148-175 and :352-362
    ctx->grid.nv = tables->nv;
    ctx->grid.nzp = tables->nzp;
    ctx->grid.n_tables = tables->n_tables;
    ctx->grid.v1 = 0.0;
    ctx->grid.dv = tables->v_length / (tables->nv - 1.);
    ctx->grid.z1 = ctx->z_centers[0] - ctx->dz;
    ctx->grid.dz = ctx->dz * (ctx->nz + 1) / (tables->nzp - 1.);
    size_t nd = (size_t) tables->n_tables * bins->nk * tables->nv;
    size_t ns = (size_t) tables->n_tables * tables->nv * tables->nzp;
    lqg_ctx *c = ctx.get();
    if (ctx->d_deriv.alloc(nd * 8) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
    cudaMemcpy(ctx->d_deriv.p, tables->deriv, nd * 8, cudaMemcpyHostToDevice);
    ctx->qmax.assign((size_t) tables->n_tables * bins->nk, 0.0);
    for (int t = 0; t < tables->n_tables; ++t)
        for (int k = 0; k < bins->nk; ++k) {
            double m = 0;
            const double *row = tables->deriv + ((size_t) t * bins->nk + k) * tables->nv;
            for (int v = 0; v < tables->nv; ++v) m = std::max(m, std::fabs(row[v]));
            ctx->qmax[(size_t) t * bins->nk + k] = m;
        }
    ctx->smax.assign(tables->n_tables, 0.0);
    if (tables->signal) {
        if (ctx->d_signal.alloc(ns * 8) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
        cudaMemcpy(ctx->d_signal.p, tables->signal, ns * 8, cudaMemcpyHostToDevice);
        for (int t = 0; t < tables->n_tables; ++t) {
            double m = 0;
            const double *s = tables->signal + (size_t) t * tables->nv * tables->nzp;
            for (size_t e = 0; e < (size_t) tables->nv * tables->nzp; ++e) m = std::max(m, std::fabs(s[e]));
            ctx->smax[t] = m;
        }
    }
    DeviceBins db{};
    db.nk = ctx->nk;
    db.nz = ctx->nz;
    db.nkz = ctx->nkz;
    db.triangular = ctx->triangular;
    db.dz = ctx->dz;
    for (int z = 0; z < ctx->nz; ++z) db.z_centers[z] = ctx->z_centers[z];
    if (ctx->d_bins.alloc(sizeof(DeviceBins)) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "bins");
    cudaMemcpy(ctx->d_bins.p, &db, sizeof db, cudaMemcpyHostToDevice);
    if (ctx->d_fisher.alloc((size_t) ctx->nkz * ctx->nkz * 8) != cudaSuccess ||
        ctx->d_dbt.alloc((size_t) 3 * ctx->nkz * 8) != cudaSuccess ||
        ctx->d_theta.alloc((size_t) ctx->nkz * 8) != cudaSuccess)
        return set_err(c, LQG_ERR_NOMEM, "globals");
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(c, LQG_ERR_CUDA, cudaGetErrorString(e));
    *out = ctx.release();
    return LQG_OK;
}

extern "C" int lqg_ctx_destroy(lqg_ctx *ctx) {
    if (!ctx) return LQG_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LQG_OK;
}

extern "C" int lqg_batch_clear(lqg_ctx *ctx) {
    if (!ctx) return LQG_ERR_ARG;
    ctx->chunks.clear();
    ctx->h_wave.clear(); ctx->h_delta.clear(); ctx->h_ivar.clear();
    ctx->h_logw.clear(); ctx->h_sqw.clear();
    ctx->results_size = 0;
    ctx->pix_dirty = true;
    return LQG_OK;
}

extern "C" int lqg_batch_size(const lqg_ctx *ctx) { return ctx ? (int) ctx->chunks.size() : 0; }

extern "C" int lqg_batch_add(lqg_ctx *ctx, int n_chunks, const int64_t *offsets,
                             const double *lambda, const double *delta, const double *ivar,
                             const int *r_fwhm, int *status_out) {
    if (!ctx || n_chunks < 0 || (n_chunks > 0 && (!offsets || !lambda || !delta || !ivar || !r_fwhm)))
        return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add: bad arguments");
    const double max_v = ctx->opts.max_forest_length, min_v = 0.90 / 2 * max_v;
    for (int c = 0; c < n_chunks; ++c) {
        int64_t a = offsets[c], b = offsets[c + 1];
        int st = LQG_CHUNK_OK;
        if (b < a) return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add: offsets not increasing");
        // QSOFile::_cutMaskedBoundary (io/qso_file.cpp:139-157)
        while (a < b && ivar[a] == 0) ++a;
        while (b > a && ivar[b - 1] == 0) --b;
        int n = (int) (b - a);
        if (n <= 0) st = LQG_CHUNK_EMPTY;
        for (int64_t i = a; st == LQG_CHUNK_OK && i < b; ++i)
            if (!std::isfinite(lambda[i]) || !std::isfinite(delta[i]) || !std::isfinite(ivar[i]) ||
                ivar[i] < 0 || !(lambda[i] > 0))
                st = LQG_CHUNK_BAD_INPUT;
        if (st == LQG_CHUNK_OK && n > kMaxPixels) st = LQG_CHUNK_TOO_LARGE;
        if (st == LQG_CHUNK_OK && n < 2) st = LQG_CHUNK_SHORT;
        lqg_ctx::HostChunk hc{};
        if (st == LQG_CHUNK_OK) {
            int realsize = 0;
            for (int64_t i = a; i < b; ++i) realsize += ivar[i] != 0;
            // QSOFile::recalcDvDLam (io/qso_file.cpp:325-329)
            std::vector<double> dvs(n - 1);
            for (int i = 0; i < n - 1; ++i) dvs[i] = std::log(lambda[a + i + 1] / lambda[a + i]) * kSpeedOfLight;
            double dv = median_of(dvs);
            // Chunk::_copyQSOFile short-chunk rule (core/chunk_estimate.cpp:173-187)
            double lenv = kSpeedOfLight * std::log(lambda[b - 1] / lambda[a]);
            int minnopix = (int) (lenv / ctx->opts.max_mean_pixel_size);
            if (realsize < minnopix || lenv < min_v) st = LQG_CHUNK_SHORT;
            // SQLookupTable::findSpecResIndex (core/sq_table.cpp:388-397)
            int res = -1;
            if (st == LQG_CHUNK_OK) {
                double rounded = std::round(dv * 10) / 10;
                for (int t = 0; t < ctx->n_tables; ++t)
                    if (ctx->r_fwhm[t] == r_fwhm[c] && std::fabs(rounded - ctx->tdv[t]) < 0.01) { res = t; break; }
                if (res < 0) st = LQG_CHUNK_NO_TABLE;
            }
            if (st == LQG_CHUNK_OK) {
                double zmin = lambda[a] / kLyaRest - 1, zmax = lambda[b - 1] / kLyaRest - 1;
                // _getMaxKindex (core/chunk_estimate.cpp:32-39)
                int kup = (int) (std::lower_bound(ctx->k_centers.begin(), ctx->k_centers.end(),
                                                  0.85 * (kPi / dv)) - ctx->k_centers.begin());
                int zl = find_redshift_bin(ctx, zmin), zu = find_redshift_bin(ctx, zmax);
                // Chunk::_setNQandFisherIndex (core/chunk_estimate.cpp:240-257)
                int nq = zu - zl + 1, fis = ctx->nk * zl;
                if (ctx->triangular) {
                    if (zl >= 0 && zl < ctx->nz && zmin < ctx->z_centers[zl] && zl != 0) { ++nq; fis -= ctx->nk; }
                    if (zu >= 0 && zu < ctx->nz && ctx->z_centers[zu] < zmax && zu < ctx->nz - 1) ++nq;
                }
                nq *= ctx->nk;
                if (zl < 0 || zu >= ctx->nz || fis < 0 || fis + nq > ctx->nkz || kup <= 0)
                    st = LQG_CHUNK_OUT_OF_RANGE;
                hc.n = n;
                hc.ld = (int) align_up(n, kPad);
                hc.nq = nq;
                hc.kbin_upp = kup;
                hc.ns = (nq / ctx->nk) * kup;
                hc.fis = fis;
                hc.res = res;
                hc.zlow = zl;
                hc.zupp = zu;
                if (st == LQG_CHUNK_OK && hc.ns + 2 > 128)
                    st = LQG_CHUNK_TOO_LARGE;
            }
        }
        if (status_out) status_out[c] = st;
        if (st != LQG_CHUNK_OK) continue;
        hc.input_index = c;
        hc.pix = (int64_t) ctx->h_wave.size();
        hc.res_off = ctx->results_size;
        ctx->results_size += 3 * hc.nq + (int64_t) hc.nq * hc.nq;
        for (int64_t i = a; i < b; ++i) {
            double w = lambda[i] / kLyaRest;   // Chunk::_copyQSOFile divides by LYA_REST
            ctx->h_wave.push_back(w);
            ctx->h_logw.push_back(std::log(w));
            ctx->h_sqw.push_back(std::sqrt(w));
            ctx->h_delta.push_back(delta[i]);
            ctx->h_ivar.push_back(ivar[i]);
        }
        ctx->chunks.push_back(hc);
    }
    ctx->pix_dirty = true;
    return LQG_OK;
}

extern "C" int lqg_chunk_info(const lqg_ctx *ctx, int i, int *info) {
    if (!ctx || !info || i < 0 || i >= (int) ctx->chunks.size()) return LQG_ERR_ARG;
    const auto &h = ctx->chunks[i];
    int v[8] = {h.n, h.fis, h.nq, h.kbin_upp, h.res, h.zlow, h.zupp, h.input_index};
    std::memcpy(info, v, sizeof v);
    return LQG_OK;
}

namespace lqg {
void launch_accumulate(const ChunkDesc *chunks, int n_chunks, const double *results,
                       const int *status, int nkz, double *fisher, double *dbt, cudaStream_t st);
}

namespace {

struct WavePlan {
    std::vector<int> members;   // batch chunk indices
    int ld = 0;
};

int upload_pixels(lqg_ctx *ctx) {
    if (!ctx->pix_dirty) return LQG_OK;
    size_t np = ctx->h_wave.size();
    size_t bytes = std::max<size_t>(np, 1) * 8;
    if (ctx->d_wave.alloc(bytes) || ctx->d_delta.alloc(bytes) || ctx->d_ivar.alloc(bytes) ||
        ctx->d_logw.alloc(bytes) || ctx->d_sqw.alloc(bytes))
        return set_err(ctx, LQG_ERR_NOMEM, "pixel arrays");
    cudaStream_t s = ctx->stream;
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_wave.p, ctx->h_wave.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_delta.p, ctx->h_delta.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_ivar.p, ctx->h_ivar.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_logw.p, ctx->h_logw.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_sqw.p, ctx->h_sqw.data(), np * 8, cudaMemcpyHostToDevice, s));
    if (ctx->d_results.alloc(std::max<int64_t>(ctx->results_size, 1) * 8) ||
        ctx->d_status.alloc(std::max<size_t>(ctx->chunks.size(), 1) * 4))
        return set_err(ctx, LQG_ERR_NOMEM, "results");
    // batch-wide chunk metadata for the final accumulation
    std::vector<ChunkDesc> meta(ctx->chunks.size());
    for (size_t i = 0; i < ctx->chunks.size(); ++i) {
        const auto &h = ctx->chunks[i];
        ChunkDesc d{};
        d.n = h.n; d.nq = h.nq; d.fis = h.fis; d.res_off = h.res_off;
        meta[i] = d;
    }
    if (ctx->d_meta.alloc(std::max<size_t>(meta.size(), 1) * sizeof(ChunkDesc)))
        return set_err(ctx, LQG_ERR_NOMEM, "metadata");
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_meta.p, meta.data(), meta.size() * sizeof(ChunkDesc),
                                       cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(s));
    ctx->pix_dirty = false;
    return LQG_OK;
}

// Bytes of wave workspace one chunk needs (see the offsets set in run_wave).
int64_t chunk_ws_bytes(const lqg_ctx::HostChunk &h, int precision, int splits) {
    int64_t ld = h.ld, m = ld * ld * 8;
    int64_t tiles = (ld / 64) * (ld / 64);
    int64_t part = std::max<int64_t>((int64_t) splits * 128 * 128 * 8, 40 * ld * 8);
    int64_t base = align_up(m, 256) * 2 + align_up(ld * 8, 256) + align_up(tiles * h.ns * 8, 256) +
                   align_up(part, 256);
    if (precision == LQG_PRECISION_FP64)
        base += align_up(m * h.ns, 256) * 2 + align_up(m * (h.ns + 2), 256);
    else
        // halves: C (2 planes), Q (ns+1 slots), R (ns), P (ns+2), each 2 planes of ld^2 halves
        base += (int64_t) ld * ld * 2 * 2 * (1 + (h.ns + 1) + h.ns + (h.ns + 2)) + (int64_t) splits * 128 * 128 * 4;
    return base;
}

int gram_splits_for(int ld, int precision) {
    if (precision == LQG_PRECISION_MIXED) return gram_splits_mixed(ld);
    int64_t K = (int64_t) ld * ld;
    int64_t s = (K + 32767) / 32768;
    return (int) std::max<int64_t>(1, std::min<int64_t>(s, 256));
}

int run_wave(lqg_ctx *ctx, const WavePlan &w, int precision, bool use_theta) {
    cudaStream_t st = ctx->stream;
    const int nch = (int) w.members.size();
    const int ld = w.ld;
    const int splits = gram_splits_for(ld, precision);
    std::vector<ChunkDesc> desc(nch);
    int64_t off = 0;
    int slot_q = 0, slot_r = 0, slot_p = 0;
    const int64_t m = (int64_t) ld * ld * 8;
    const int64_t tiles = (ld / 64) * (ld / 64);
    for (int i = 0; i < nch; ++i) {
        const auto &h = ctx->chunks[w.members[i]];
        ChunkDesc &d = desc[i];
        d.n = h.n; d.ld = ld; d.nq = h.nq; d.ns = h.ns; d.kbin_upp = h.kbin_upp; d.fis = h.fis;
        d.res = h.res; d.zb0 = h.fis / ctx->nk; d.pix = h.pix; d.res_off = h.res_off;
        d.n_tiles = (int) tiles;
        d.o_s = off; off += align_up(m, 256);
        d.o_c = off; off += align_up(m, 256);
        d.o_y = off; off += align_up((int64_t) ld * 8, 256);
        d.o_dpart = off; off += align_up(tiles * h.ns * 8, 256);
        d.o_part = off; off += align_up(std::max<int64_t>((int64_t) splits * 128 * 128 * 8, 40 * (int64_t) ld * 8), 256);
        if (precision == LQG_PRECISION_FP64) {
            d.o_q = off; off += align_up(m * h.ns, 256);
            d.o_r = off; off += align_up(m * h.ns, 256);
            d.o_p = off; off += align_up(m * (h.ns + 2), 256);
        }
        d.slot_q = slot_q; slot_q += h.ns + 1;
        d.slot_r = slot_r; slot_r += h.ns;
        d.slot_p = slot_p; slot_p += h.ns + 2;
    }
    const int64_t fp64_bytes = off;
    int64_t half_bytes = 0;
    const int64_t plane = (int64_t) ld * ld * 2;
    if (precision == LQG_PRECISION_MIXED)
        half_bytes = plane * 2 * ((int64_t) nch + slot_q + slot_r + slot_p);
    if (ctx->d_ws.alloc(std::max<int64_t>(fp64_bytes, 256)))
        return set_err(ctx, LQG_ERR_NOMEM, "workspace");
    if (precision == LQG_PRECISION_MIXED) {
        if (ctx->d_halves.alloc(half_bytes + 1024) ||
            ctx->d_gram.alloc((int64_t) nch * splits * 128 * 128 * 4))
            return set_err(ctx, LQG_ERR_NOMEM, "mixed workspace");
    }
    int nscales = 4 * nch + slot_q + slot_p + slot_r;
    std::vector<double> scales(nscales, 1.0);
    if (precision == LQG_PRECISION_MIXED) {
        for (int i = 0; i < nch; ++i) {
            const auto &h = ctx->chunks[w.members[i]];
            for (int s = 0; s < h.ns; ++s)
                scales[4 * nch + desc[i].slot_q + s] =
                    pow2_scale(ctx->qmax[(size_t) h.res * ctx->nk + s % h.kbin_upp], 16384.0);
            scales[4 * nch + desc[i].slot_q + h.ns] = pow2_scale(ctx->smax[h.res], 16384.0);
        }
    }
    if (ctx->d_desc.alloc(nch * sizeof(ChunkDesc)) || ctx->d_scales.alloc(nscales * 8))
        return set_err(ctx, LQG_ERR_NOMEM, "descriptors");
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_desc.p, desc.data(), nch * sizeof(ChunkDesc), cudaMemcpyHostToDevice, st));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_scales.p, scales.data(), nscales * 8, cudaMemcpyHostToDevice, st));
    // jobs: (chunk, s) for s in [0, ns]
    std::vector<int> jobs;
    for (int i = 0; i < nch; ++i)
        for (int s = 0; s <= desc[i].ns; ++s) { jobs.push_back(i); jobs.push_back(s); }
    if (ctx->d_jobs.alloc(jobs.size() * 4)) return set_err(ctx, LQG_ERR_NOMEM, "jobs");
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_jobs.p, jobs.data(), jobs.size() * 4, cudaMemcpyHostToDevice, st));
    // wave-local status: starts OK
    if (ctx->d_wstat.alloc(nch * 4)) return set_err(ctx, LQG_ERR_NOMEM, "status");
    LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_wstat.p, 0, nch * 4, st));

    WaveArgs a{};
    a.chunks = ctx->d_desc.as<ChunkDesc>();
    a.n_chunks = nch;
    a.max_ld = ld;
    a.ws = ctx->d_ws.as<char>();
    a.wave = ctx->d_wave.as<double>(); a.delta = ctx->d_delta.as<double>(); a.ivar = ctx->d_ivar.as<double>();
    a.logw = ctx->d_logw.as<double>(); a.sqw = ctx->d_sqw.as<double>();
    a.deriv = ctx->d_deriv.as<double>();
    a.signal = ctx->d_signal.p ? ctx->d_signal.as<double>() : nullptr;
    a.theta = use_theta ? ctx->d_theta.as<double>() : nullptr;
    a.results = ctx->d_results.as<double>();
    a.status = ctx->d_wstat.as<int>();
    a.grid = ctx->grid;
    a.bins = ctx->d_bins.as<DeviceBins>();
    a.cont_logl = ctx->opts.cont_logl_order;
    a.cont_l = ctx->opts.cont_l_order;
    a.turn_off_sfid = ctx->opts.turn_off_sfid;
    a.skip_fisher = ctx->opts.skip_fisher;
    a.precision = precision;
    a.total_slots_q = slot_q; a.total_slots_r = slot_r; a.total_slots_p = slot_p;
    a.gram_splits = splits;
    a.scales = ctx->d_scales.as<double>();
    if (precision == LQG_PRECISION_MIXED) {
        __half *hb = ctx->d_halves.as<__half>();
        int64_t pl = (int64_t) ld * ld;
        a.c_hi = hb; hb += pl * nch;
        a.c_lo = hb; hb += pl * nch;
        a.q_hi = hb; hb += pl * slot_q;
        a.q_lo = hb; hb += pl * slot_q;
        a.r_hi = hb; hb += pl * slot_r;
        a.r_lo = hb; hb += pl * slot_r;
        a.p_hi = hb; hb += pl * slot_p;
        a.p_lo = hb; hb += pl * slot_p;
        a.gram_part = ctx->d_gram.as<float>();
    }
    a.mid_event = ctx->ev[4];
    a.ws_bytes = fp64_bytes;
    a.results_elems = ctx->results_size;
    a.gram_elems = precision == LQG_PRECISION_MIXED ? (int64_t) nch * splits * 128 * 128 : 0;
    if (ctx->d_check.alloc(4 * sizeof(unsigned long long))) return set_err(ctx, LQG_ERR_NOMEM, "check");
    LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_check.p, 0, 4 * sizeof(unsigned long long), st));
    a.check = ctx->d_check.as<unsigned long long>();
    // LQG_SYNC_EACH=1: synchronise after every kernel and name the one that failed
    static const bool sync_each = getenv("LQG_SYNC_EACH") && getenv("LQG_SYNC_EACH")[0] == '1';
    auto step = [&](const char *what) -> int {
        if (!sync_each) return LQG_OK;
        cudaError_t se = cudaStreamSynchronize(st);
        if (se == cudaSuccess) se = cudaGetLastError();
        if (se != cudaSuccess)
            return set_err(ctx, LQG_ERR_CUDA, std::string(what) + " (ld " + std::to_string(ld) + ", " +
                                                  std::to_string(nch) + " chunks): " + cudaGetErrorString(se));
        return LQG_OK;
    };
    int rc = LQG_OK;
    cudaEventRecord(ctx->ev[0], st);
    launch_build_s_c(a, st);
    if ((rc = step("build_s_c"))) return rc;
    cudaEventRecord(ctx->ev[1], st);
    launch_factor(a, st);
    if ((rc = step("factor"))) return rc;
    cudaEventRecord(ctx->ev[2], st);
    if (precision == LQG_PRECISION_MIXED) launch_scales_mixed(a, st);
    launch_build_q(a, st);
    if ((rc = step("build_q"))) return rc;
    cudaEventRecord(ctx->ev[3], st);
    if (precision == LQG_PRECISION_MIXED)
        launch_products_mixed(a, st, ctx->d_jobs.as<int>(), (int) jobs.size() / 2);
    else
        launch_products_fp64(a, st, ctx->d_jobs.as<int>(), (int) jobs.size() / 2);
    if ((rc = step("products"))) return rc;
    cudaEventRecord(ctx->ev[5], st);
    launch_finish(a, st);
    if ((rc = step("finish"))) return rc;
    cudaEventRecord(ctx->ev[6], st);
    unsigned long long chk[4] = {0, 0, 0, 0};
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(chk, ctx->d_check.p, sizeof chk, cudaMemcpyDeviceToHost, st));
    // scatter wave status into the batch status array
    std::vector<int> ws_host(nch);
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ws_host.data(), ctx->d_wstat.p, nch * 4, cudaMemcpyDeviceToHost, st));
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(st));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(ctx, LQG_ERR_CUDA, std::string("wave kernels: ") + cudaGetErrorString(e));
    if (chk[0] != 0)
        return set_err(ctx, LQG_ERR_STATE, "index check failed " + std::to_string(chk[0]) + " times: code " +
                                               std::to_string(chk[1]) + " chunk " + std::to_string(chk[2]) +
                                               " index " + std::to_string(chk[3]) + " (ld " + std::to_string(ld) + ")");
    // [0] S/C build, [1] factorisation, [2] Q build, [3] C^-1 Q products, [4] Gram, [5] finish
    static const int from[6] = {0, 1, 2, 3, 4, 5}, to[6] = {1, 2, 3, 4, 5, 6};
    for (int k = 0; k < 6; ++k) {
        float ms = 0;
        cudaEventElapsedTime(&ms, ctx->ev[from[k]], ctx->ev[to[k]]);
        ctx->timings[k] += ms;
    }
    for (int i = 0; i < nch; ++i) ctx->last_status[w.members[i]] = ws_host[i];
    ctx->launches += a.launches;
    return LQG_OK;
}

}  // namespace

extern "C" int lqg_nr_iteration(lqg_ctx *ctx, const double *theta, int precision) {
    if (!ctx) return LQG_ERR_ARG;
    if (precision != LQG_PRECISION_FP64 && precision != LQG_PRECISION_MIXED)
        return set_err(ctx, LQG_ERR_ARG, "unknown precision");
    if (precision == LQG_PRECISION_MIXED && !tc_available())
        return set_err(ctx, LQG_ERR_UNSUPPORTED, "mixed precision needs the sm_103a tensor-core kernels");
    cudaSetDevice(ctx->device);
    int rc = upload_pixels(ctx);
    if (rc) return rc;
    bool use_theta = false;
    if (theta) {
        for (int i = 0; i < ctx->nkz; ++i) use_theta |= theta[i] != 0.0;
        LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_theta.p, theta, ctx->nkz * 8, cudaMemcpyHostToDevice, ctx->stream));
    }
    const int nb = (int) ctx->chunks.size();
    ctx->last_status.assign(nb, LQG_CHUNK_OK);
    std::fill(ctx->timings, ctx->timings + 8, 0.0);
    ctx->launches = 0;
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    cudaEventRecord(t0, ctx->stream);
    // Size-bucketed waves: chunks grouped by their padded size, largest first,
    // each wave limited by the workspace budget.
    size_t budget = ctx->opts.workspace_bytes;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        budget = (size_t) (0.6 * (double) fr);
    }
    std::vector<int> order(nb);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return ctx->chunks[x].ld > ctx->chunks[y].ld; });
    std::vector<WavePlan> waves;
    int64_t used = 0;
    for (int idx : order) {
        const auto &h = ctx->chunks[idx];
        int64_t need = chunk_ws_bytes(h, precision, gram_splits_for(h.ld, precision));
        if (waves.empty() || waves.back().ld != h.ld || used + need > (int64_t) budget) {
            waves.push_back(WavePlan{});
            waves.back().ld = h.ld;
            used = 0;
        }
        waves.back().members.push_back(idx);
        used += need;
    }
    for (auto &w : waves) {
        rc = run_wave(ctx, w, precision, use_theta);
        if (rc) return rc;
    }
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_status.p, ctx->last_status.data(), nb * 4, cudaMemcpyHostToDevice, ctx->stream));
    cudaEventRecord(ctx->ev[7], ctx->stream);
    launch_accumulate(ctx->d_meta.as<ChunkDesc>(), nb, ctx->d_results.as<double>(), ctx->d_status.as<int>(),
                      ctx->nkz, ctx->d_fisher.as<double>(), ctx->d_dbt.as<double>(), ctx->stream);
    ctx->launches++;
    cudaEventRecord(t1, ctx->stream);
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(ctx->stream));
    float tt = 0, ta = 0;
    cudaEventElapsedTime(&tt, t0, t1);
    cudaEventElapsedTime(&ta, ctx->ev[7], t1);
    ctx->timings[6] = ta;
    ctx->timings[7] = tt;
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(ctx, LQG_ERR_CUDA, cudaGetErrorString(e));
    return LQG_OK;
}

extern "C" int lqg_download(lqg_ctx *ctx, double *d, double *b, double *t, double *fisher, int *chunk_status) {
    if (!ctx) return LQG_ERR_ARG;
    cudaStream_t s = ctx->stream;
    const int nkz = ctx->nkz;
    if (d) LQG_CUDA_CHECK_RET(cudaMemcpyAsync(d, ctx->d_dbt.as<double>(), nkz * 8, cudaMemcpyDeviceToHost, s));
    if (b) LQG_CUDA_CHECK_RET(cudaMemcpyAsync(b, ctx->d_dbt.as<double>() + nkz, nkz * 8, cudaMemcpyDeviceToHost, s));
    if (t) LQG_CUDA_CHECK_RET(cudaMemcpyAsync(t, ctx->d_dbt.as<double>() + 2 * nkz, nkz * 8, cudaMemcpyDeviceToHost, s));
    if (fisher) LQG_CUDA_CHECK_RET(cudaMemcpyAsync(fisher, ctx->d_fisher.p, (size_t) nkz * nkz * 8, cudaMemcpyDeviceToHost, s));
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(s));
    if (chunk_status)
        std::copy(ctx->last_status.begin(), ctx->last_status.end(), chunk_status);
    return LQG_OK;
}

extern "C" int lqg_chunk_result(lqg_ctx *ctx, int i, double *d, double *b, double *t, double *fisher) {
    if (!ctx || i < 0 || i >= (int) ctx->chunks.size()) return LQG_ERR_ARG;
    const auto &h = ctx->chunks[i];
    std::vector<double> buf(3 * h.nq + (size_t) h.nq * h.nq);
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(buf.data(), ctx->d_results.as<double>() + h.res_off, buf.size() * 8,
                                       cudaMemcpyDeviceToHost, ctx->stream));
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(ctx->stream));
    if (d) std::copy(buf.begin(), buf.begin() + h.nq, d);
    if (b) std::copy(buf.begin() + h.nq, buf.begin() + 2 * h.nq, b);
    if (t) std::copy(buf.begin() + 2 * h.nq, buf.begin() + 3 * h.nq, t);
    if (fisher) std::copy(buf.begin() + 3 * h.nq, buf.end(), fisher);
    return LQG_OK;
}

extern "C" int lqg_last_timings(const lqg_ctx *ctx, double *ms, int n) {
    if (!ctx || !ms) return 0;
    int k = std::min(n, 8);
    for (int i = 0; i < k; ++i) ms[i] = ctx->timings[i];
    return k;
}

extern "C" int lqg_last_launch_count(const lqg_ctx *ctx) { return ctx ? ctx->launches : 0; }

extern "C" int lqg_fisher_solve_n(int n, const double *fisher_sum, const double *dbt, double *fisher,
                                  double *solver, double *inverse, double *weighted, double *theta,
                                  int *damped, int *dof, double *damp_out);

extern "C" int lqg_fisher_solve(lqg_ctx *ctx, const double *fisher_sum, const double *dbt,
                                double *fisher, double *solver, double *inverse, double *weighted,
                                double *theta, int *damped, int *dof, double *damp) {
    if (!ctx) return LQG_ERR_ARG;
    int rc = lqg_fisher_solve_n(ctx->nkz, fisher_sum, dbt, fisher, solver, inverse, weighted, theta,
                                damped, dof, damp);
    if (rc) ctx->err = "Fisher matrix could not be inverted";
    return rc;
}
