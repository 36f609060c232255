// Host side of the C ABI declared in include/lqg.h.
#include "lqg_internal.cuh"

#include <algorithm>
#include <map>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <utility>
#include <numeric>

using namespace lqg;

namespace {

// Allocator whose value-initialisation leaves trivial elements unset: resize()
// of the batch's host arrays then costs no fill, each element being written
// once by the chunk it belongs to.
template <class T>
struct HostAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = HostAlloc<U>; };
    HostAlloc() = default;
    template <class U> HostAlloc(const HostAlloc<U> &) noexcept {}
    template <class U> void construct(U *p) noexcept { ::new ((void *) p) U; }
    template <class U, class... A> void construct(U *p, A &&...a) { ::new ((void *) p) U(std::forward<A>(a)...); }
};
template <class T> using HostVec = std::vector<T, HostAlloc<T>>;

}  // namespace

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
    DevBuf d_deriv, d_deriv_f, d_deriv_ff, d_signal, d_signal_ff, d_bins;
    lqg_opts opts{};
    uint64_t wait_ns = 0;   // lqg_set_wait_limit; 0: the kernels' 2 s
    int fisher_band = 0;    // lqg_set_fisher_optimization: banded chunk Fisher matrices
    int64_t h2d_bytes = 0;  // bytes the last iteration copied host to device (lqg_last_h2d_bytes)
    // LQG_PRECISION_MIXED_AUTO: per padded size ld, the mixed form, the drain
    // interval of the products and the Gram's K split (lqg_autotune)
    struct Tune {
        int sym = 1, drain = 8, gram_k = 32768, pair = 0;
    };
    std::map<int, Tune> tuning;
    // batch
    struct HostChunk {
        int n, ld, nq, ns, kbin_upp, fis, res, zlow, zupp, input_index;
        int64_t pix, res_off;
        int nelem, os, sh, nf;     // resolution matrix (nelem = 0: none)
        int64_t fpix, rw_off;
        double rw_sum;
    };
    std::vector<HostChunk> chunks;
    HostVec<double> h_wave, h_delta, h_ivar, h_logw, h_sqw;
    HostVec<float2> h_logw2, h_sqw2;
    HostVec<double> h_sqiv, h_niv;
    HostVec<float2> h_sqiv2;
    HostVec<double> h_flogw, h_fsqw, h_rw;   // resolution-matrix grids and weights
    bool has_reso = false;
    bool pix_dirty = true;
    DevBuf d_wave, d_delta, d_ivar, d_logw, d_sqw, d_logw2, d_sqw2, d_sqiv, d_niv;
    DevBuf d_flogw, d_fsqw, d_rw, d_sqiv2;
    int64_t results_size = 0;
    DevBuf d_results, d_status, d_theta, d_fisher, d_dbt, d_meta;
    // workspace
    DevBuf d_fws, d_ws, d_fbounds, d_desc, d_jobs, d_scales, d_halves, d_gram, d_check, d_ttab, d_ttab_ff, d_rtab;
    void *h_stage = nullptr;   // pinned staging of the per-iteration descriptors
    size_t h_stage_bytes = 0;
    std::vector<int> last_status;
    double timings[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int launches = 0;
    int waves = 0;
    bool have_results = false;   // an iteration has run on the current batch
    std::vector<cudaEvent_t> evpool;
    // CUDA graphs of iterations' launches: an iteration whose key (batch,
    // precision, theta use, device buffers, launch plan) was seen by one of the
    // last kKeyHistory iterations is captured, and replayed while the key holds.
    // A few graphs are kept, so that an NR loop alternating between keys (the
    // first iteration at theta = 0, the later ones with theta) replays each.
    struct GraphEntry {
        std::vector<uintptr_t> key;
        cudaGraphExec_t exec = nullptr;
        int launches = 0, waves = 0;
        std::vector<std::pair<size_t, int>> spans;
        size_t eacc = 0;
    };
    static constexpr size_t kMaxGraphs = 4, kKeyHistory = 8;
    uint64_t batch_version = 0;
    std::vector<std::vector<uintptr_t>> key_history;
    std::vector<GraphEntry> graphs;
    bool graph_failed = false;
    // an iteration enqueued by lqg_nr_iteration_async and not yet finished
    // (its statuses, index-check counters and timings are read by finish_pending)
    bool pending = false;
    cudaEvent_t ev_after = nullptr;   // orders the iteration after the caller's stream
    int pending_nb = 0;
    std::vector<std::pair<size_t, int>> pending_spans;
    size_t pending_eacc = 0;
};

namespace {

int set_err(lqg_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->err = msg;
    return code;
}

// The median of the sorted values (stats::medianOfSortedArray,
// mathtools/stats.cpp:8-16) from the order statistics n/2 and n/2 - 1, which
// nth_element places without sorting the rest: the same values, so the same
// result.
double median_of(std::vector<double> v) {
    const size_t n = v.size();
    if (n == 0) return -1;
    std::nth_element(v.begin(), v.begin() + n / 2, v.end());
    const double upper = v[n / 2];
    if (n % 2) return upper;
    const double lower = *std::max_element(v.begin(), v.begin() + n / 2);
    return (lower + upper) / 2;
}

// bins::findRedshiftBin, core/global_numbers.cpp:344-355
int find_redshift_bin(const lqg_ctx *ctx, double z) {
    double zlow = ctx->z_centers[0] - ctx->dz / 2.0;
    if (z < zlow) return -1;
    int r = (int) ((z - zlow) / ctx->dz);
    return std::min(r, ctx->nz);
}

// x as a double-float pair: hi = fl32(x), lo = fl32(x - hi)
float2 split_ff(double x) {
    const float h = (float) x;
    return make_float2(h, (float) (x - (double) h));
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

namespace {

// The context's binning, table list and options: everything Chunk::Chunk
// reads, all host-side (no CUDA call).
void set_host_fields(lqg_ctx *ctx, const lqg_bins *bins, const lqg_tables *tables, const lqg_opts *opts) {
    ctx->nk = bins->nk;
    ctx->nz = bins->nz;
    ctx->nkz = bins->nk * bins->nz;
    ctx->dz = bins->z_bin_width;
    ctx->triangular = bins->triangular;
    ctx->k_edges.assign(bins->k_edges, bins->k_edges + bins->nk + 1);
    ctx->k_centers.clear();
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
}

}  // namespace

extern "C" int lqg_ctx_create(lqg_ctx **out, const lqg_bins *bins, const lqg_tables *tables,
                              const lqg_opts *opts, int device) {
    cudaGetLastError();   // an error left by earlier work of the process is not this call's
    if (!out || !bins || !tables || !opts) return LQG_ERR_ARG;
    *out = nullptr;
    if (bins->nk <= 0 || bins->nk > kMaxKBands || bins->nz <= 0 || bins->nz > 64 || !bins->k_edges || !bins->z_centers ||
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
    if (opts->redshift_growth_on > 0 && !std::isfinite(opts->fid_redshift_power)) return LQG_ERR_ARG;
    auto ctx = std::make_unique<lqg_ctx>();
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) return LQG_ERR_CUDA;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
        return LQG_ERR_CUDA;
    set_host_fields(ctx.get(), bins, tables, opts);
    // interpolation grids, core/sq_table.cpp:148-175 and :352-362
    ctx->grid.nv = tables->nv;
    ctx->grid.nzp = tables->nzp;
    ctx->grid.n_tables = tables->n_tables;
    ctx->grid.v1 = 0.0;
    ctx->grid.dv = tables->v_length / (tables->nv - 1.);
    ctx->grid.z1 = ctx->z_centers[0] - ctx->dz;
    ctx->grid.dz = ctx->dz * (ctx->nz + 1) / (tables->nzp - 1.);
    {
        const float2 kv = split_ff(kSpeedOfLight / ctx->grid.dv);
        ctx->grid.kv_hi = kv.x;
        ctx->grid.kv_lo = kv.y;
        const float2 z1p = split_ff(1.0 + ctx->grid.z1), idz = split_ff(1.0 / ctx->grid.dz);
        ctx->grid.z1p_hi = z1p.x; ctx->grid.z1p_lo = z1p.y;
        ctx->grid.idz_hi = idz.x; ctx->grid.idz_lo = idz.y;
    }
    size_t nd = (size_t) tables->n_tables * bins->nk * tables->nv;
    size_t ns = (size_t) tables->n_tables * tables->nv * tables->nzp;
    lqg_ctx *c = ctx.get();
    if (ctx->d_deriv.alloc(nd * 8) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
    cudaMemcpy(ctx->d_deriv.p, tables->deriv, nd * 8, cudaMemcpyHostToDevice);
    {
        std::vector<float> df(tables->deriv, tables->deriv + nd);
        if (ctx->d_deriv_f.alloc(nd * 4) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
        cudaMemcpy(ctx->d_deriv_f.p, df.data(), nd * 4, cudaMemcpyHostToDevice);
        // double-float (value, difference to the next node) per node, for the
        // mixed path's interpolation r0 + (r1 - r0) dn in double-float
        std::vector<float4> dff(nd);
        for (size_t e = 0; e < nd; ++e) {
            const size_t v = e % (size_t) tables->nv;
            const double r = tables->deriv[e], dr = v + 1 < (size_t) tables->nv ? tables->deriv[e + 1] - r : 0.0;
            const float2 a = split_ff(r), b = split_ff(dr);
            dff[e] = make_float4(a.x, a.y, b.x, b.y);
        }
        if (ctx->d_deriv_ff.alloc(nd * 16) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
        cudaMemcpy(ctx->d_deriv_ff.p, dff.data(), nd * 16, cudaMemcpyHostToDevice);
    }
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
        {
            std::vector<float2> sf(ns);
            for (size_t e = 0; e < ns; ++e) sf[e] = split_ff(tables->signal[e]);
            if (ctx->d_signal_ff.alloc(ns * 8) != cudaSuccess) return set_err(c, LQG_ERR_NOMEM, "tables");
            cudaMemcpy(ctx->d_signal_ff.p, sf.data(), ns * 8, cudaMemcpyHostToDevice);
        }
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
    for (int k = 0; k <= ctx->nk; ++k) db.k_edges[k] = ctx->k_edges[k];
    for (int z = 0; z < ctx->nz; ++z) {
        db.z_centers[z] = ctx->z_centers[z];
        const float2 c1 = split_ff(1.0 + ctx->z_centers[z]);
        db.zc1_hi[z] = c1.x;
        db.zc1_lo[z] = c1.y;
    }
    {
        const float2 d = split_ff(ctx->dz), dh = split_ff(ctx->dz / 2);
        db.dz_hi = d.x; db.dz_lo = d.y; db.dzh_hi = dh.x; db.dzh_lo = dh.y;
        db.inv_dz = (float) (1.0 / ctx->dz);
        const float2 idz = split_ff(1.0 / ctx->dz);
        db.idz_hi = idz.x; db.idz_lo = idz.y;
    }
    db.growth = opts->redshift_growth_on > 0;
    db.growth_b = opts->fid_redshift_power;
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
    for (auto &g : ctx->graphs) cudaGraphExecDestroy(g.exec);
    for (auto &e : ctx->evpool) cudaEventDestroy(e);
    if (ctx->ev_after) cudaEventDestroy(ctx->ev_after);
    if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return LQG_OK;
}

extern "C" int lqg_batch_clear(lqg_ctx *ctx) {
    if (!ctx) return LQG_ERR_ARG;
    ctx->chunks.clear();
    ctx->h_wave.clear(); ctx->h_delta.clear(); ctx->h_ivar.clear();
    ctx->h_logw.clear(); ctx->h_sqw.clear();
    ctx->h_logw2.clear(); ctx->h_sqw2.clear();
    ctx->h_sqiv.clear(); ctx->h_niv.clear(); ctx->h_sqiv2.clear();
    ctx->h_flogw.clear(); ctx->h_fsqw.clear(); ctx->h_rw.clear();
    ctx->has_reso = false;
    ctx->have_results = false;
    ctx->results_size = 0;
    ctx->pix_dirty = true;
    ctx->batch_version++;
    return LQG_OK;
}

extern "C" int lqg_batch_size(const lqg_ctx *ctx) { return ctx ? (int) ctx->chunks.size() : 0; }

namespace {

// One chunk of an lqg_batch_add / lqg_batch_add_reso call after Chunk::Chunk:
// its status, its description and (resolution matrix) its weights and grid.
struct ChunkSetup {
    int st = LQG_CHUNK_OK;
    int64_t a = 0, b = 0;        // pixel range after the masked edges are cut
    lqg_ctx::HostChunk hc{};
    std::vector<double> rw, fgrid;   // the diagonal form's weights, built here; the grid
    const double *rw_src = nullptr;  // the weights: the caller's rows (oversampled) or rw
    size_t rw_len = 0;
};

// Chunk::Chunk for chunk c.  resomat == NULL: table lookup by (R, dv).
// Otherwise the chunk's resolution matrix, per pixel: nelem weights of its
// oversampled row (reso_os > 0) or its column's entries on the ndiags = nelem
// diagonals (reso_os <= 0).  Reads the context, writes only `out`.
void setup_chunk(const lqg_ctx *ctx, int c, const int64_t *offsets, const double *lambda,
                 const double *delta, const double *ivar, const int *r_fwhm, int reso_os, int reso_nelem,
                 const double *resomat, ChunkSetup &out) {
    const double max_v = ctx->opts.max_forest_length, min_v = 0.90 / 2 * max_v;
    const bool reso = resomat != nullptr;
    lqg_ctx::HostChunk &hc = out.hc;
    std::vector<double> &fgrid = out.fgrid;
    int64_t a = offsets[c], b = offsets[c + 1];
    int st = LQG_CHUNK_OK;
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
        // SQLookupTable::findSpecResIndex (core/sq_table.cpp:388-397); with a
        // resolution matrix RES_INDEX = 0 (core/chunk_estimate.cpp:189-193)
        int res = reso ? 0 : -1;
        if (st == LQG_CHUNK_OK && !reso) {
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
            if (st == LQG_CHUNK_OK && hc.ns + 2 > 128 * kMaxGramBlocks)
                st = LQG_CHUNK_TOO_LARGE;
        }
    }
    // resolution matrix of the chunk: weights per coarse row and its grid
    if (st == LQG_CHUNK_OK && reso) {
        const int nel = reso_nelem;
        hc.nelem = nel;
        if (reso_os > 0) {
            // OversampledMatrix rows; grid of Chunk::_initMatrices
            // (core/chunk_estimate.cpp:927-938): w_0 + (p - nelem/2) dlambda / LYA / os,
            // dlambda the chunk's median pixel width (io/qso_file.cpp:86-88, 325-329)
            hc.os = reso_os;
            hc.sh = 0;
            hc.nf = n * reso_os + nel - 1;
            out.rw_src = resomat + a * nel;
            out.rw_len = (size_t) n * nel;
            std::vector<double> dl(n - 1);
            for (int i = 0; i < n - 1; ++i) dl[i] = lambda[a + i + 1] - lambda[a + i];
            const double fine = median_of(dl) / kLyaRest / reso_os, w0 = lambda[a] / kLyaRest;
            const int disp = nel / 2;
            fgrid.resize(hc.nf);
            for (int p = 0; p < hc.nf; ++p) fgrid[p] = w0 + (p - disp) * fine;
        } else {
            // DiaMatrix: row r has entries at columns r + off, off = a - nel/2,
            // held on diagonal d = nel - 1 - a (mathtools/matrix_helper.cpp:503-520,
            // 684-813); columns outside the chunk drop out
            hc.os = 1;
            hc.sh = nel / 2;
            hc.nf = n;
            std::vector<double> &rw = out.rw;
            rw.assign((size_t) n * nel, 0.0);
            for (int r = 0; r < n; ++r)
                for (int k = 0; k < nel; ++k) {
                    const int col = r - hc.sh + k;
                    if (col >= 0 && col < n) rw[(size_t) r * nel + k] = resomat[(a + col) * nel + (nel - 1 - k)];
                }
            out.rw_src = rw.data();
            out.rw_len = rw.size();
            for (int64_t i = a; i < b; ++i) fgrid.push_back(lambda[i] / kLyaRest);
        }
        hc.rw_sum = 0;
        for (int r = 0; r < n; ++r) {
            double sum = 0;
            for (int k = 0; k < nel; ++k) {
                const double w = out.rw_src[(size_t) r * nel + k];
                if (!std::isfinite(w)) st = LQG_CHUNK_BAD_INPUT;
                sum += std::fabs(w);
            }
            hc.rw_sum = std::max(hc.rw_sum, sum);
        }
        for (double w : fgrid)
            if (!(w > 0) || !std::isfinite(w)) st = LQG_CHUNK_BAD_INPUT;
    }
    out.st = st;
    out.a = a;
    out.b = b;
}

// Chunk::Chunk for every chunk of an lqg_batch_add / lqg_batch_add_reso call.
// The chunks are set up and their pixel arrays filled on the host's cores;
// the accepted ones join the batch in input order, each at the offsets a
// serial walk over the call's chunks gives them.  Offsets that decrease
// reject the whole call before anything is added.
int add_chunks(lqg_ctx *ctx, int n_chunks, const int64_t *offsets, const double *lambda,
               const double *delta, const double *ivar, const int *r_fwhm, int reso_os, int reso_nelem,
               const double *resomat, int *status_out) {
    for (int c = 0; c < n_chunks; ++c)
        if (offsets[c + 1] < offsets[c]) return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add: offsets not increasing");
    const bool reso = resomat != nullptr;
    std::vector<ChunkSetup> set(n_chunks);
    host_parallel_for(n_chunks, 16, [&](int c) {
        setup_chunk(ctx, c, offsets, lambda, delta, ivar, r_fwhm, reso_os, reso_nelem, resomat, set[c]);
    });
    std::vector<int> accepted;
    size_t np = ctx->h_wave.size(), nfp = ctx->h_flogw.size(), nrw = ctx->h_rw.size();
    for (int c = 0; c < n_chunks; ++c) {
        ChunkSetup &u = set[c];
        if (status_out) status_out[c] = u.st;
        if (u.st != LQG_CHUNK_OK) continue;
        lqg_ctx::HostChunk &hc = u.hc;
        if (reso) {
            ctx->has_reso = true;
            hc.fpix = (int64_t) nfp;
            hc.rw_off = (int64_t) nrw;
            nfp += u.fgrid.size();
            nrw += u.rw_len;
        }
        hc.input_index = c;
        hc.pix = (int64_t) np;
        np += (size_t) (u.b - u.a);
        hc.res_off = ctx->results_size;
        ctx->results_size += 3 * hc.nq + (int64_t) hc.nq * hc.nq;
        accepted.push_back(c);
    }
    for (auto *v : {&ctx->h_wave, &ctx->h_logw, &ctx->h_sqw, &ctx->h_delta, &ctx->h_ivar, &ctx->h_sqiv,
                    &ctx->h_niv})
        v->resize(np);
    for (auto *v : {&ctx->h_logw2, &ctx->h_sqw2, &ctx->h_sqiv2}) v->resize(np);
    ctx->h_flogw.resize(nfp);
    ctx->h_fsqw.resize(nfp);
    ctx->h_rw.resize(nrw);
    host_parallel_for((int) accepted.size(), 8, [&](int j) {
        const ChunkSetup &u = set[accepted[j]];
        const lqg_ctx::HostChunk &hc = u.hc;
        if (reso) {
            for (size_t p = 0; p < u.fgrid.size(); ++p) {
                ctx->h_flogw[hc.fpix + p] = std::log(u.fgrid[p]);
                ctx->h_fsqw[hc.fpix + p] = std::sqrt(u.fgrid[p]);
            }
            std::copy(u.rw_src, u.rw_src + u.rw_len, ctx->h_rw.begin() + hc.rw_off);
        }
        // SmoothNoiseWeights: C takes the smoothed ivar, N the raw one
        const int64_t a = u.a, n = u.b - u.a;
        std::vector<double> ivc(ivar + a, ivar + u.b);
        if (ctx->opts.smooth_noise_weights >= 0)
            smooth_ivar((int) n, ivar + a, ctx->opts.smooth_noise_weights, ivc.data());
        for (int64_t i = 0; i < n; ++i) {
            const int64_t q = hc.pix + i;
            const double w = lambda[a + i] / kLyaRest;   // Chunk::_copyQSOFile divides by LYA_REST
            ctx->h_wave[q] = w;
            ctx->h_logw[q] = std::log(w);
            ctx->h_sqw[q] = std::sqrt(w);
            ctx->h_logw2[q] = split_ff(ctx->h_logw[q]);
            ctx->h_sqw2[q] = split_ff(ctx->h_sqw[q]);
            ctx->h_delta[q] = delta[a + i];
            ctx->h_ivar[q] = ivc[i];
            ctx->h_sqiv[q] = std::sqrt(ivc[i]);
            ctx->h_sqiv2[q] = split_ff(ctx->h_sqiv[q]);
            ctx->h_niv[q] = ivar[a + i] != 0 ? 1.0 / ivar[a + i] : 0.0;
        }
    });
    for (int c : accepted) ctx->chunks.push_back(set[c].hc);
    ctx->pix_dirty = true;
    ctx->have_results = false;
    ctx->batch_version++;
    return LQG_OK;
}

}  // namespace

extern "C" int lqg_batch_add(lqg_ctx *ctx, int n_chunks, const int64_t *offsets,
                             const double *lambda, const double *delta, const double *ivar,
                             const int *r_fwhm, int *status_out) {
    if (!ctx || n_chunks < 0 || (n_chunks > 0 && (!offsets || !lambda || !delta || !ivar || !r_fwhm)))
        return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add: bad arguments");
    return add_chunks(ctx, n_chunks, offsets, lambda, delta, ivar, r_fwhm, 0, 0, nullptr, status_out);
}

extern "C" int lqg_batch_add_reso(lqg_ctx *ctx, int n_chunks, const int64_t *offsets,
                                  const double *lambda, const double *delta, const double *ivar,
                                  int oversampling, int nelem, const double *resomat, int *status_out) {
    if (!ctx || n_chunks < 0 || (n_chunks > 0 && (!offsets || !lambda || !delta || !ivar || !resomat)))
        return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add_reso: bad arguments");
    if (nelem < 1 || nelem % 2 == 0)
        return set_err(ctx, LQG_ERR_ARG, "lqg_batch_add_reso: nelem must be odd and positive");
    const int os = oversampling > 0 ? oversampling : 1;
    if (nelem > kResoMaxElem || (kResoTile - 1) * os + nelem > kResoMaxFine)
        return set_err(ctx, LQG_ERR_UNSUPPORTED, "lqg_batch_add_reso: resolution matrix wider than the "
                                                 "engine's tile (31 oversampling + nelem <= 128, nelem <= 48)");
    return add_chunks(ctx, n_chunks, offsets, lambda, delta, ivar, nullptr, oversampling, nelem, resomat,
                      status_out);
}

extern "C" int lqg_chunk_plan(const lqg_bins *bins, const lqg_tables *tables, const lqg_opts *opts,
                              int n_chunks, const int64_t *offsets, const double *lambda, const double *delta,
                              const double *ivar, const int *r_fwhm, int oversampling, int nelem,
                              const double *resomat, int *status_out, int *info_out) {
    const bool reso = resomat != nullptr;
    if (!bins || !tables || !opts || n_chunks < 0 || !status_out || !info_out ||
        (n_chunks > 0 && (!offsets || !lambda || !delta || !ivar || (!reso && !r_fwhm))))
        return LQG_ERR_ARG;
    if (reso) {
        // the checks of lqg_batch_add_reso
        const int os = oversampling > 0 ? oversampling : 1;
        if (nelem < 1 || nelem % 2 == 0) return LQG_ERR_ARG;
        if (nelem > kResoMaxElem || (kResoTile - 1) * os + nelem > kResoMaxFine) return LQG_ERR_UNSUPPORTED;
    }
    if (bins->nk <= 0 || bins->nk > kMaxKBands || bins->nz <= 0 || bins->nz > 64 || !bins->k_edges ||
        !bins->z_centers || !(bins->z_bin_width > 0) || tables->n_tables <= 0 || !tables->r_fwhm || !tables->dv ||
        !(opts->max_mean_pixel_size > 0) || !(opts->max_forest_length >= 0))
        return LQG_ERR_ARG;
    for (int c = 0; c < n_chunks; ++c)
        if (offsets[c + 1] < offsets[c]) return LQG_ERR_ARG;
    lqg_ctx host;   // binning and tables only: nothing on a device
    set_host_fields(&host, bins, tables, opts);
    host_parallel_for(n_chunks, 16, [&](int c) {
        ChunkSetup u;
        setup_chunk(&host, c, offsets, lambda, delta, ivar, r_fwhm, reso ? oversampling : 0, reso ? nelem : 0,
                    resomat, u);
        status_out[c] = u.st;
        int *info = info_out + 8 * (size_t) c;
        if (u.st != LQG_CHUNK_OK) {
            std::fill(info, info + 8, 0);
            return;
        }
        const auto &h = u.hc;
        const int v[8] = {h.n, h.fis, h.nq, h.kbin_upp, h.res, h.zlow, h.zupp, c};
        std::copy(v, v + 8, info);
    });
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
void launch_fisher_band(const ChunkDesc *chunks, int n_chunks, double *results, int64_t results_elems, int nk,
                        cudaStream_t st);
}

namespace {

int upload_pixels(lqg_ctx *ctx) {
    if (!ctx->pix_dirty) return LQG_OK;
    size_t np = ctx->h_wave.size();
    size_t bytes = std::max<size_t>(np, 1) * 8;
    if (ctx->d_wave.alloc(bytes) || ctx->d_delta.alloc(bytes) || ctx->d_ivar.alloc(bytes) ||
        ctx->d_logw.alloc(bytes) || ctx->d_sqw.alloc(bytes) || ctx->d_logw2.alloc(bytes) ||
        ctx->d_sqw2.alloc(bytes) || ctx->d_sqiv.alloc(bytes) || ctx->d_niv.alloc(bytes))
        return set_err(ctx, LQG_ERR_NOMEM, "pixel arrays");
    cudaStream_t s = ctx->stream;
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_wave.p, ctx->h_wave.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_delta.p, ctx->h_delta.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_ivar.p, ctx->h_ivar.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_logw.p, ctx->h_logw.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_sqw.p, ctx->h_sqw.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_logw2.p, ctx->h_logw2.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_sqiv.p, ctx->h_sqiv.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_niv.p, ctx->h_niv.data(), np * 8, cudaMemcpyHostToDevice, s));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_sqw2.p, ctx->h_sqw2.data(), np * 8, cudaMemcpyHostToDevice, s));
    if (ctx->d_sqiv2.alloc(bytes)) return set_err(ctx, LQG_ERR_NOMEM, "pixel arrays");
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_sqiv2.p, ctx->h_sqiv2.data(), np * 8, cudaMemcpyHostToDevice, s));
    const size_t nfp = ctx->h_flogw.size(), nrw = ctx->h_rw.size();
    if (ctx->d_flogw.alloc(std::max<size_t>(nfp, 1) * 8) || ctx->d_fsqw.alloc(std::max<size_t>(nfp, 1) * 8) ||
        ctx->d_rw.alloc(std::max<size_t>(nrw, 1) * 8))
        return set_err(ctx, LQG_ERR_NOMEM, "resolution-matrix arrays");
    if (nfp) {
        LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_flogw.p, ctx->h_flogw.data(), nfp * 8, cudaMemcpyHostToDevice, s));
        LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_fsqw.p, ctx->h_fsqw.data(), nfp * 8, cudaMemcpyHostToDevice, s));
    }
    if (nrw) LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_rw.p, ctx->h_rw.data(), nrw * 8, cudaMemcpyHostToDevice, s));
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
    ctx->h2d_bytes += (int64_t) (np * 8 * 10 + nfp * 16 + nrw * 8 + meta.size() * sizeof(ChunkDesc));
    ctx->pix_dirty = false;
    return LQG_OK;
}

// The plan's choices for chunks of padded size ld under a requested precision
// mode: the kernels' defaults for the fixed modes, the context's table for
// LQG_PRECISION_MIXED_AUTO (defaults where it has no entry).
lqg_ctx::Tune form_for(const lqg_ctx *ctx, int mode, int ld) {
    lqg_ctx::Tune t;
    if (mode == LQG_PRECISION_FP64 || mode == LQG_PRECISION_MIXED_DIRECT) t.sym = 0;
    if (mode == LQG_PRECISION_MIXED_AUTO) {
        auto it = ctx->tuning.find(ld);
        if (it != ctx->tuning.end()) t = it->second;
    }
    return t;
}

int gram_splits_for(int ld, int precision, bool sym, int gram_k) {
    if (precision == LQG_PRECISION_MIXED) return gram_splits_mixed(sym ? sym_plane(ld) : (int64_t) ld * ld, gram_k);
    int64_t K = (int64_t) ld * ld;
    int64_t s = (K + 32767) / 32768;
    return (int) std::max<int64_t>(1, std::min<int64_t>(s, 256));
}

int gram_blocks(int ns) { return (ns + 2 + 127) / 128; }

// Factor workspace of one chunk: S_fid, C~ (becomes C^-1), y and 64 ld of scratch;
// the whitened mixed form adds the marginalised C^-1 next to W.
int64_t chunk_fws_bytes(int64_t ld, bool cinv_m) {
    return align_up(ld * ld * 8, 256) * (cinv_m ? 3 : 2) + align_up(ld * 8, 256) + align_up(64 * ld * 8, 256);
}

// Mixed path: d - b - t from the x partials (k_finish_dx).  It rests on C = S + N +
// sum theta Q with the N of b, which smoothed noise weights break (C takes the
// smoothed ivar, N the raw one); the Gram's b and t stand alone then.
bool dbt_identity(const lqg_ctx *ctx, int precision) {
    return precision == LQG_PRECISION_MIXED && ctx->opts.smooth_noise_weights < 0;
}

// Wave workspace of one chunk in a wave with the given Gram blocking.
int64_t chunk_ws_bytes(int64_t ld, int ns, int precision, bool sym, int splits, int gt) {
    const int64_t m = ld * ld * 8, tiles = (ld / 64) * (ld / 64);
    int64_t b = align_up(tiles * 16 * ns * 8, 256) * (precision == LQG_PRECISION_MIXED ? 2 : 1);
    const int64_t gblk = (int64_t) gt * gt * splits * 128 * 128;
    if (precision == LQG_PRECISION_FP64)
        b += align_up(gblk * 8, 256) + align_up(m * ns, 256) * 2 + align_up(m * (ns + 2), 256);
    else if (!sym)
        // fp16 hi/lo planes of C^-1, Q (ns + 1 slots), R (ns + 2) and P (ns), and fp32 Gram partials
        b += ld * ld * 2 * 2 * (int64_t) (1 + (ns + 1) + ns + (ns + 2)) + gblk * 4;
    else
        // W, Q (ns + 1), X (ns + 2) planes of ld^2 and the compact B slots (ns + 2)
        b += ld * ld * 2 * 2 * (int64_t) (1 + (ns + 1) + (ns + 2)) + sym_plane((int) ld) * 2 * 2 * (ns + 2) +
             gblk * 4;
    return b;
}

struct WavePlan {
    std::vector<int> members;   // batch chunk indices
    int ld = 0, gt = 1, splits = 1;
    int sym = 0, drain = 8;     // mixed form and products drain interval (one per ld)
    int pair = 0;               // products on CTA pairs
    int max_ns = 0;             // largest stored-slot count
    int slot_q = 0, slot_r = 0, slot_p = 0;
    int64_t ws_bytes = 0, half_bytes = 0;
    size_t desc_off = 0, jobs_off = 0, scales_off = 0, jobs2_off = 0;
    int njobs = 0, nscales = 0, njobs2 = 0;
};

struct GroupPlan {
    std::vector<int> members;   // batch chunk indices, largest first
    int max_ld = 0;
    int64_t fws_bytes = 0;
    size_t desc_off = 0;
    std::vector<WavePlan> waves;
};

cudaEvent_t pool_event(lqg_ctx *ctx, size_t i) {
    while (ctx->evpool.size() <= i) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ctx->evpool.push_back(e);
    }
    return ctx->evpool[i];
}

// Plans the iteration: groups of chunks whose factor workspaces fit together
// (phase A: S, C~ and the factorisation of every chunk of the group), each
// split into waves of equal padded size (phase B: Q_s, products, traces).
// Descriptors, jobs and host-known scales of every launch are packed into
// single arrays, uploaded once.
int plan_iteration(lqg_ctx *ctx, int precision, int mode, std::vector<GroupPlan> &groups, std::vector<ChunkDesc> &desc,
                   std::vector<int> &jobs, std::vector<double> &scales, int64_t &max_fws, int64_t &max_ws,
                   int64_t &max_half, int64_t &max_gram, int &n_combos, int &n_rks) {
    const int nb = (int) ctx->chunks.size();
    size_t budget = ctx->opts.workspace_bytes;
    if (budget == 0) {
        // 60 % of the memory that is free or already held as workspace
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        const size_t held = ctx->d_fws.bytes + ctx->d_ws.bytes + ctx->d_halves.bytes + ctx->d_gram.bytes;
        budget = (size_t) (0.6 * (double) (fr + held));
    }
    std::vector<int> order(nb);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const auto &a = ctx->chunks[x], &b = ctx->chunks[y];
        if (a.ld != b.ld) return a.ld > b.ld;
        return gram_blocks(a.ns) > gram_blocks(b.ns);
    });
    const int64_t fws_limit = (int64_t) (0.35 * (double) budget);
    const bool ident = dbt_identity(ctx, precision);
    auto own_m = [&](const lqg_ctx::HostChunk &h) {
        return ident && form_for(ctx, mode, h.ld).sym && h.nelem == 0;
    };
    int64_t fsum = 0;
    for (int idx : order) {
        const int64_t need = chunk_fws_bytes(ctx->chunks[idx].ld, own_m(ctx->chunks[idx]));
        // gridDim.y carries the chunk index of a launch: at most 65535 per launch
        if (groups.empty() || fsum + need > fws_limit || groups.back().members.size() >= 65535) {
            groups.emplace_back();
            fsum = 0;
        }
        groups.back().members.push_back(idx);
        fsum += need;
        groups.back().fws_bytes = fsum;
    }
    max_fws = max_ws = max_half = max_gram = 0;
    // (table, KBIN_UPP) pairs of the batch: one theta-weighted table row block
    // each, as (res, kbin_upp) ints at the front of jobs
    std::vector<std::pair<int, int>> combos;
    for (const auto &h : ctx->chunks)
        if (h.res >= 0 && h.nelem == 0) combos.push_back({h.res, h.kbin_upp});
    std::sort(combos.begin(), combos.end());
    combos.erase(std::unique(combos.begin(), combos.end()), combos.end());
    n_combos = (int) combos.size();
    for (const auto &cb : combos) { jobs.push_back(cb.first); jobs.push_back(cb.second); }
    // KBIN_UPP values of the resolution-matrix chunks: one theta node table row
    // block each (the mixed path with theta), after the pairs in jobs
    std::vector<int> rks;
    for (const auto &h : ctx->chunks)
        if (h.nelem > 0) rks.push_back(h.kbin_upp);
    std::sort(rks.begin(), rks.end());
    rks.erase(std::unique(rks.begin(), rks.end()), rks.end());
    n_rks = (int) rks.size();
    for (int k : rks) jobs.push_back(k);
    for (auto &g : groups) {
        max_fws = std::max(max_fws, g.fws_bytes);
        g.desc_off = desc.size();
        int64_t off = 0;
        for (int idx : g.members) {
            const auto &h = ctx->chunks[idx];
            ChunkDesc d{};
            d.tcombo = -1;
            if (h.res >= 0 && h.nelem == 0)
                d.tcombo = (int) (std::lower_bound(combos.begin(), combos.end(), std::make_pair(h.res, h.kbin_upp)) -
                                  combos.begin());
            if (h.nelem > 0)
                d.tcombo = (int) (std::lower_bound(rks.begin(), rks.end(), h.kbin_upp) - rks.begin());
            d.n = h.n; d.ld = h.ld; d.nq = h.nq; d.ns = h.ns; d.kbin_upp = h.kbin_upp; d.fis = h.fis;
            d.res = h.res; d.zb0 = h.fis / ctx->nk; d.pix = h.pix; d.res_off = h.res_off; d.gidx = idx;
            d.nelem = h.nelem; d.os = h.os; d.sh = h.sh; d.nf = h.nf; d.fpix = h.fpix; d.rw_off = h.rw_off;
            d.rw_sum = h.rw_sum;
            d.sym = precision == LQG_PRECISION_MIXED ? form_for(ctx, mode, h.ld).sym : 0;
            const int64_t m = (int64_t) h.ld * h.ld * 8;
            d.o_s = off; off += align_up(m, 256);
            d.o_c = off; off += align_up(m, 256);
            d.o_y = off; off += align_up((int64_t) h.ld * 8, 256);
            d.o_fscr = off; off += align_up(64 * (int64_t) h.ld * 8, 256);
            // the marginalised C^-1: its own buffer next to W (whitened form), or
            // C^-1 itself (direct form); not formed for resolution-matrix chunks
            d.cinv_m = ident && h.nelem == 0 ? 1 : 0;
            d.o_m = d.o_c;
            if (own_m(h)) { d.o_m = off; off += align_up(m, 256); }
            g.max_ld = std::max(g.max_ld, h.ld);
            desc.push_back(d);
        }
    }
    // the wave budget is what the largest factor workspace leaves
    const int64_t wlimit = std::max<int64_t>((int64_t) budget - max_fws, 1);
    for (auto &g : groups) {
        for (size_t k = 0; k < g.members.size(); ++k) {
            const int idx = g.members[k];
            const auto &h = ctx->chunks[idx];
            const lqg_ctx::Tune tn = form_for(ctx, mode, h.ld);
            const bool sym = precision == LQG_PRECISION_MIXED && tn.sym;
            const int gt = gram_blocks(h.ns), splits = gram_splits_for(h.ld, precision, sym, tn.gram_k);
            int64_t need = chunk_ws_bytes(h.ld, h.ns, precision, sym, splits, gt);
            if (precision == LQG_PRECISION_MIXED && h.nelem > 0)
                need += align_up((int64_t) h.kbin_upp * h.nf * 8, 256);   // grid-point phases
            bool fresh = g.waves.empty() || g.waves.back().ld != h.ld || g.waves.back().gt != gt;
            if (!fresh) {
                const auto &w = g.waves.back();
                fresh = w.ws_bytes + need > wlimit || w.slot_q + h.ns + 1 > 65535;
            }
            if (fresh) {
                g.waves.emplace_back();
                g.waves.back().ld = h.ld;
                g.waves.back().gt = gt;
                g.waves.back().splits = splits;
                g.waves.back().sym = sym ? 1 : 0;
                g.waves.back().drain = tn.drain;
                g.waves.back().pair = precision == LQG_PRECISION_MIXED ? tn.pair : 0;
            }
            WavePlan &w = g.waves.back();
            w.members.push_back((int) k);   // index within the group
            w.ws_bytes += need;             // refined below
            w.slot_q += h.ns + 1;           // product jobs, one launch row each (reset below)
        }
        for (auto &w : g.waves) {
            const int ld = w.ld;
            const bool sym = w.sym != 0;
            w.slot_q = 0;
            const int64_t m = (int64_t) ld * ld * 8, tiles = (ld / 64) * (ld / 64);
            const int64_t gblk = (int64_t) w.gt * w.gt * w.splits * 128 * 128;
            w.desc_off = desc.size();
            int64_t off = 0;
            for (int k : w.members) {
                ChunkDesc d = desc[g.desc_off + k];
                d.o_dpart = off; off += align_up(tiles * 16 * d.ns * 8, 256);
                if (precision == LQG_PRECISION_MIXED) {
                    d.o_xpart = off; off += align_up(tiles * 16 * d.ns * 8, 256);
                }
                if (precision == LQG_PRECISION_MIXED && d.nelem > 0) {
                    d.o_ph = off; off += align_up((int64_t) d.kbin_upp * d.nf * 8, 256);
                }
                if (precision == LQG_PRECISION_FP64) {
                    d.o_part = off; off += align_up(gblk * 8, 256);
                    d.o_q = off; off += align_up(m * d.ns, 256);
                    d.o_r = off; off += align_up(m * d.ns, 256);
                    d.o_p = off; off += align_up(m * (d.ns + 2), 256);
                }
                d.slot_q = w.slot_q; w.slot_q += d.ns + 1;
                w.max_ns = std::max(w.max_ns, d.ns);
                // trace-Gram operand stacks.  FP64: P = [A_s^T, (C^-1 S)^T, N C^-1],
                // R = [A_s].  Mixed: P = [A_s^T], R = [A_s, C^-1 S, C^-1 N].  Whitened
                // form: R = [X_s, W S, W N], P = [B_s, W S W^T, W N W^T] (compact).
                const bool mixed = precision == LQG_PRECISION_MIXED;
                d.slot_r = w.slot_r; w.slot_r += mixed ? d.ns + 2 : d.ns;
                d.slot_p = w.slot_p; w.slot_p += mixed ? (sym ? d.ns + 2 : d.ns) : d.ns + 2;
                desc.push_back(d);
            }
            const int nch = (int) w.members.size();
            w.ws_bytes = std::max<int64_t>(off, 256);
            w.half_bytes = 0;
            int64_t gram = 0;
            if (precision == LQG_PRECISION_MIXED) {
                const int64_t pp = sym ? sym_plane(ld) : (int64_t) ld * ld;
                w.half_bytes = (int64_t) ld * ld * 2 * 2 * ((int64_t) nch + w.slot_q + w.slot_r) + pp * 2 * 2 * w.slot_p;
                gram = (int64_t) nch * gblk;
            }
            max_ws = std::max(max_ws, w.ws_bytes);
            max_half = std::max(max_half, w.half_bytes);
            max_gram = std::max(max_gram, gram);
            w.jobs_off = jobs.size();
            for (int i = 0; i < nch; ++i)
                for (int s = 0; s <= desc[w.desc_off + i].ns; ++s) { jobs.push_back(i); jobs.push_back(s); }
            w.njobs = (int) (jobs.size() - w.jobs_off) / 2;
            // whitened form, second product: B_s for s <= ns + 1 (CTA pairs: slots
            // s and s + 1 from one job of even s)
            w.jobs2_off = jobs.size();
            if (sym)
                for (int i = 0; i < nch; ++i)
                    for (int s = 0; s <= desc[w.desc_off + i].ns + 1; s += w.pair ? 2 : 1) {
                        jobs.push_back(i);
                        jobs.push_back(s);
                    }
            w.njobs2 = (int) (jobs.size() - w.jobs2_off) / 2;
            w.scales_off = scales.size();
            w.nscales = 4 * nch + w.slot_q + w.slot_p + w.slot_r;
            scales.resize(scales.size() + w.nscales, 1.0);
            if (precision == LQG_PRECISION_MIXED) {
                for (int i = 0; i < nch; ++i) {
                    const ChunkDesc &d = desc[w.desc_off + i];
                    double *q = scales.data() + w.scales_off + 4 * nch + d.slot_q;
                    if (d.nelem > 0) {
                        // |R M R^T| <= max|M| (largest row sum of |R|)^2; the
                        // resolution-matrix Q_k peaks at dk / pi (v = 0)
                        const double r2 = d.rw_sum * d.rw_sum;
                        for (int s = 0; s < d.ns; ++s) {
                            const int kn = s % d.kbin_upp;
                            q[s] = pow2_scale((ctx->k_edges[kn + 1] - ctx->k_edges[kn]) / kPi * r2, 16384.0);
                        }
                        q[d.ns] = pow2_scale(ctx->smax[d.res] * r2, 16384.0);
                    } else {
                        for (int s = 0; s < d.ns; ++s)
                            q[s] = pow2_scale(ctx->qmax[(size_t) d.res * ctx->nk + s % d.kbin_upp], 16384.0);
                        q[d.ns] = pow2_scale(ctx->smax[d.res], 16384.0);
                    }
                }
            }
        }
    }
    return LQG_OK;
}

}  // namespace

namespace {

// Waits for the last enqueued iteration and reads what it left on the host
// side: per-chunk statuses, the index-check counters and the phase timings.
int finish_pending(lqg_ctx *ctx) {
    if (!ctx->pending) return LQG_OK;
    ctx->pending = false;
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(ctx->stream));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_err(ctx, LQG_ERR_CUDA, std::string("iteration kernels: ") + cudaGetErrorString(e));
    const char *hs = static_cast<const char *>(ctx->h_stage);
    const unsigned long long *chk = reinterpret_cast<const unsigned long long *>(hs);
    const int *st = reinterpret_cast<const int *>(hs + 4 * sizeof(unsigned long long));
    ctx->last_status.assign(st, st + ctx->pending_nb);
    if (chk[0] != 0)
        return set_err(ctx, LQG_ERR_STATE, "index check failed " + std::to_string(chk[0]) + " times: code " +
                                               std::to_string(chk[1]) + " chunk " + std::to_string(chk[2]) +
                                               " index " + std::to_string(chk[3]));
    // [0] S/C build, [1] factorisation, [2] Q build, [3] products, [4] Gram, [5] finish,
    // [6] accumulation, [7] whole iteration
    for (auto &sp : ctx->pending_spans) {
        float ms = 0;
        if (cudaEventElapsedTime(&ms, ctx->evpool[sp.first], ctx->evpool[sp.first + 1]) == cudaSuccess)
            ctx->timings[sp.second] += ms;
    }
    float ta = 0, tt = 0;
    if (cudaEventElapsedTime(&ta, ctx->evpool[ctx->pending_eacc], ctx->evpool[1]) != cudaSuccess) ta = 0;
    if (cudaEventElapsedTime(&tt, ctx->evpool[0], ctx->evpool[1]) != cudaSuccess) tt = 0;
    cudaGetLastError();   // a timing query that failed leaves no error behind
    ctx->timings[6] = ta;
    ctx->timings[7] = tt;
    ctx->have_results = true;
    return LQG_OK;
}

// Plans and enqueues one iteration on the context's stream, ordered after
// `after` (a caller's stream) when given; finish_pending completes it.
int enqueue_iteration(lqg_ctx *ctx, const double *theta, int precision, cudaStream_t after) {
    if (precision != LQG_PRECISION_FP64 && precision != LQG_PRECISION_MIXED &&
        precision != LQG_PRECISION_MIXED_DIRECT && precision != LQG_PRECISION_MIXED_AUTO)
        return set_err(ctx, LQG_ERR_ARG, "unknown precision");
    // the mixed forms share the kernels up to the products; the plan picks the
    // form per padded size (whitened or direct) from the requested mode
    const int mode = precision;
    if (precision != LQG_PRECISION_FP64) precision = LQG_PRECISION_MIXED;
    if (precision == LQG_PRECISION_MIXED && !tc_available())
        return set_err(ctx, LQG_ERR_UNSUPPORTED, "mixed precision needs the sm_103a tensor-core kernels");
    cudaSetDevice(ctx->device);
    int rc = finish_pending(ctx);
    if (rc) return rc;
    ctx->h2d_bytes = 0;
    if ((rc = upload_pixels(ctx))) return rc;
    cudaStream_t st = ctx->stream;
    if (after && after != st) {
        // inputs the caller produced on its stream come first
        if (!ctx->ev_after && cudaEventCreateWithFlags(&ctx->ev_after, cudaEventDisableTiming) != cudaSuccess)
            return set_err(ctx, LQG_ERR_CUDA, "event");
        LQG_CUDA_CHECK_RET(cudaEventRecord(ctx->ev_after, after));
        LQG_CUDA_CHECK_RET(cudaStreamWaitEvent(st, ctx->ev_after, 0));
    }
    bool use_theta = false;
    if (theta) {
        for (int i = 0; i < ctx->nkz; ++i) use_theta |= theta[i] != 0.0;
        LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_theta.p, theta, ctx->nkz * 8, cudaMemcpyHostToDevice, st));
        ctx->h2d_bytes += (int64_t) ctx->nkz * 8;
    }
    const int nb = (int) ctx->chunks.size();
    ctx->last_status.assign(nb, LQG_CHUNK_OK);
    std::fill(ctx->timings, ctx->timings + 8, 0.0);
    ctx->launches = 0;
    ctx->waves = 0;
    if (nb == 0) {
        // an empty batch contributes nothing: zero sums, as the reference's
        // accumulators stay when no chunk is processed
        LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_fisher.p, 0, (size_t) ctx->nkz * ctx->nkz * 8, st));
        LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_dbt.p, 0, (size_t) 3 * ctx->nkz * 8, st));
        LQG_CUDA_CHECK_RET(cudaStreamSynchronize(st));
        ctx->have_results = true;
        return LQG_OK;
    }

    std::vector<GroupPlan> groups;
    std::vector<ChunkDesc> desc;
    std::vector<int> jobs;
    std::vector<double> scales;
    int64_t max_fws = 0, max_ws = 0, max_half = 0, max_gram = 0;
    int n_combos = 0, n_rks = 0;
    if ((rc = plan_iteration(ctx, precision, mode, groups, desc, jobs, scales, max_fws, max_ws, max_half, max_gram,
                             n_combos, n_rks)))
        return rc;
    const size_t ttab_bytes = (size_t) n_combos * ctx->nz * ctx->grid.nv * 8;
    if (use_theta && n_combos > 0 &&
        (ctx->d_ttab.alloc(ttab_bytes) || (precision == LQG_PRECISION_MIXED && ctx->d_ttab_ff.alloc(ttab_bytes))))
        return set_err(ctx, LQG_ERR_NOMEM, "theta tables");
    // Mixed path with theta and resolution-matrix chunks: node tables of
    // G(v) = sum_k theta_k Q_k(v) on [0, v_max] (the widest fine grid's v) at
    // h = 1 / (20 k_max), so that the cubic Hermite interpolation's (h k)^4 / 384
    // stays below 2e-8 of G
    bool reso_theta = use_theta && precision == LQG_PRECISION_MIXED && n_rks > 0;
    int64_t rtab_n = 0;
    double rtab_h = 0.0;
    if (reso_theta) {
        double span = 0.0;
        int kmax = 0;
        for (const auto &h : ctx->chunks) {
            if (h.nelem <= 0 || h.nf < 2) continue;
            span = std::max(span, ctx->h_flogw[h.fpix + h.nf - 1] - ctx->h_flogw[h.fpix]);
            kmax = std::max(kmax, h.kbin_upp);
        }
        rtab_h = 0.05 / ctx->k_edges[std::max(kmax, 1)];
        rtab_n = (int64_t) std::ceil(kSpeedOfLight * span / rtab_h) + 4;
        // a binning whose tables would pass 1 GiB (very high k over very long
        // chunks) keeps the FP64 build of C for its resolution chunks instead
        const double bytes = (double) n_rks * ctx->nz * (double) rtab_n * sizeof(float4);
        if (!(bytes <= 1073741824.0) || rtab_n > INT32_MAX) {
            reso_theta = false;
            rtab_n = 0;
        } else if (ctx->d_rtab.alloc((size_t) bytes)) {
            return set_err(ctx, LQG_ERR_NOMEM, "theta node tables");
        }
    }
    ctx->d_fws.trim(std::max<int64_t>(max_fws, 256));
    ctx->d_ws.trim(std::max<int64_t>(max_ws, 256));
    ctx->d_halves.trim(precision == LQG_PRECISION_MIXED ? max_half + 1024 : 0);
    ctx->d_gram.trim(precision == LQG_PRECISION_MIXED ? std::max<int64_t>(max_gram, 1) * 4 : 0);
    if (ctx->d_fws.alloc(std::max<int64_t>(max_fws, 256)) || ctx->d_ws.alloc(std::max<int64_t>(max_ws, 256)) ||
        ctx->d_fbounds.alloc(std::max(4 * nb, 1) * 8))
        return set_err(ctx, LQG_ERR_NOMEM, "workspace");
    if (precision == LQG_PRECISION_MIXED &&
        (ctx->d_halves.alloc(max_half + 1024) || ctx->d_gram.alloc(std::max<int64_t>(max_gram, 1) * 4)))
        return set_err(ctx, LQG_ERR_NOMEM, "mixed workspace");
    if (ctx->d_desc.alloc(std::max<size_t>(desc.size(), 1) * sizeof(ChunkDesc)) ||
        ctx->d_jobs.alloc(std::max<size_t>(jobs.size(), 1) * 4) ||
        ctx->d_scales.alloc(std::max<size_t>(scales.size(), 1) * 8) ||
        ctx->d_check.alloc(4 * sizeof(unsigned long long)))
        return set_err(ctx, LQG_ERR_NOMEM, "descriptors");
    // pinned staging, so that the uploads below are asynchronous
    const size_t stage = std::max(desc.size() * sizeof(ChunkDesc) + jobs.size() * 4 + scales.size() * 8,
                                  4 * sizeof(unsigned long long) + (size_t) nb * 4);
    if (ctx->h_stage_bytes < stage) {
        if (ctx->h_stage) cudaFreeHost(ctx->h_stage);
        ctx->h_stage = nullptr;
        ctx->h_stage_bytes = 0;
        LQG_CUDA_CHECK_RET(cudaMallocHost(&ctx->h_stage, stage));
        ctx->h_stage_bytes = stage;
    }
    // the previous iteration's uploads must have left the staging buffer
    LQG_CUDA_CHECK_RET(cudaStreamSynchronize(st));
    char *hs = static_cast<char *>(ctx->h_stage);
    std::memcpy(hs, desc.data(), desc.size() * sizeof(ChunkDesc));
    std::memcpy(hs + desc.size() * sizeof(ChunkDesc), jobs.data(), jobs.size() * 4);
    std::memcpy(hs + desc.size() * sizeof(ChunkDesc) + jobs.size() * 4, scales.data(), scales.size() * 8);
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_desc.p, hs, desc.size() * sizeof(ChunkDesc), cudaMemcpyHostToDevice, st));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_jobs.p, hs + desc.size() * sizeof(ChunkDesc), jobs.size() * 4,
                                       cudaMemcpyHostToDevice, st));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(ctx->d_scales.p, hs + desc.size() * sizeof(ChunkDesc) + jobs.size() * 4,
                                       scales.size() * 8, cudaMemcpyHostToDevice, st));
    ctx->h2d_bytes += (int64_t) (desc.size() * sizeof(ChunkDesc) + jobs.size() * 4 + scales.size() * 8);
    LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_status.p, 0, std::max(nb, 1) * 4, st));
    LQG_CUDA_CHECK_RET(cudaMemsetAsync(ctx->d_check.p, 0, 4 * sizeof(unsigned long long), st));

    WaveArgs base{};
    base.fws = ctx->d_fws.as<char>();
    base.ws = ctx->d_ws.as<char>();
    base.fbounds = ctx->d_fbounds.as<double>();
    base.wave = ctx->d_wave.as<double>(); base.delta = ctx->d_delta.as<double>(); base.ivar = ctx->d_ivar.as<double>();
    base.logw = ctx->d_logw.as<double>(); base.sqw = ctx->d_sqw.as<double>();
    base.logw2 = ctx->d_logw2.as<float2>(); base.sqw2 = ctx->d_sqw2.as<float2>();
    base.sqiv = ctx->d_sqiv.as<double>(); base.niv = ctx->d_niv.as<double>();
    base.sqiv2 = ctx->d_sqiv2.as<float2>();
    // mixed path: S and C~ built in double-float, handed over as pairs (with
    // theta too, unless resolution-matrix chunks need their FP64 theta sandwiches)
    // the double-float S/C build; with theta, resolution chunks need their node tables
    base.c_is_ff = (precision == LQG_PRECISION_MIXED && ctx->d_signal_ff.p &&
                    (!use_theta || !ctx->has_reso || reso_theta)) ? 1 : 0;
    base.flogw = ctx->d_flogw.as<double>(); base.fsqw = ctx->d_fsqw.as<double>(); base.rw = ctx->d_rw.as<double>();
    base.n_fpix = (int64_t) ctx->h_flogw.size();
    base.reso_nelem = base.reso_os = 0;
    base.growth = ctx->opts.redshift_growth_on > 0;
    base.sym = 0;   // per wave (and per chunk in the factorisation)
    base.dbt_id = dbt_identity(ctx, precision) ? 1 : 0;
    // W = T is lower triangular unless the continuum projector makes it full
    const bool no_marg = ctx->opts.cont_logl_order < 0 && ctx->opts.cont_l_order < 0;
    base.w_tri = 0;
    {
        int ne = -1, os = -1;
        bool uniform = true;
        for (const auto &h : ctx->chunks) {
            if (h.nelem <= 0) continue;
            if (ne < 0) { ne = h.nelem; os = h.os; }
            uniform &= h.nelem == ne && h.os == os;
        }
        if (uniform && ne > 0) { base.reso_nelem = ne; base.reso_os = os; }
    }
    base.n_rw = (int64_t) ctx->h_rw.size();
    base.deriv = ctx->d_deriv.as<double>();
    base.deriv_f = ctx->d_deriv_f.as<float>();
    base.deriv_ff = ctx->d_deriv_ff.as<float4>();
    base.signal = ctx->d_signal.p ? ctx->d_signal.as<double>() : nullptr;
    base.signal_ff = ctx->d_signal_ff.p ? ctx->d_signal_ff.as<float2>() : nullptr;
    base.theta = use_theta ? ctx->d_theta.as<double>() : nullptr;
    base.ttab = use_theta && n_combos > 0 ? ctx->d_ttab.as<double>() : nullptr;
    base.ttab_ff = base.ttab && base.c_is_ff ? ctx->d_ttab_ff.as<float2>() : nullptr;
    base.rtab = reso_theta ? ctx->d_rtab.as<float4>() : nullptr;
    base.rtab_n = rtab_n;
    if (reso_theta) {
        const double x = kSpeedOfLight / rtab_h;
        base.rtab_x = make_float2((float) x, (float) (x - (double) (float) x));
    }
    base.results = ctx->d_results.as<double>();
    base.status = ctx->d_status.as<int>();
    base.grid = ctx->grid;
    base.bins = ctx->d_bins.as<DeviceBins>();
    base.cont_logl = ctx->opts.cont_logl_order;
    base.cont_l = ctx->opts.cont_l_order;
    base.turn_off_sfid = ctx->opts.turn_off_sfid;
    base.skip_fisher = ctx->opts.skip_fisher;
    base.precision = precision;
    base.results_elems = ctx->results_size;
    base.n_pix = (int64_t) ctx->h_wave.size();
    base.check = ctx->d_check.as<unsigned long long>();
    base.wait_ns = ctx->wait_ns;

    // LQG_SYNC_EACH=1: synchronise after every kernel and name the one that failed
    static const bool sync_each = getenv("LQG_SYNC_EACH") && getenv("LQG_SYNC_EACH")[0] == '1';
    auto step = [&](const char *what, int ld, int nch) -> int {
        if (!sync_each) return LQG_OK;
        cudaError_t se = cudaStreamSynchronize(st);
        if (se == cudaSuccess) se = cudaGetLastError();
        if (se != cudaSuccess)
            return set_err(ctx, LQG_ERR_CUDA, std::string(what) + " (ld " + std::to_string(ld) + ", " +
                                                  std::to_string(nch) + " chunks): " + cudaGetErrorString(se));
        return LQG_OK;
    };
    // events: [0] start, then 3 per group and 5 per wave, [1] end
    std::vector<std::pair<size_t, int>> spans;   // (first event, timing slot) of each measured span
    size_t eacc = 0;
    cudaEvent_t ev_start = pool_event(ctx, 0), ev_end = pool_event(ctx, 1);
    auto launch_all = [&]() -> int {
        int rc = LQG_OK;
        size_t nev = 2;
        record_event(ev_start, st);
        if (base.ttab) {
            launch_theta_tables(base.deriv, base.theta, ctx->d_jobs.as<int>(), n_combos, ctx->nk, ctx->nz,
                                ctx->grid.nv, ctx->d_ttab.as<double>(), const_cast<float2 *>(base.ttab_ff), st);
            ctx->launches++;
        }
        if (base.rtab) {
            launch_theta_reso_tables(base.theta, base.bins, ctx->d_jobs.as<int>() + 2 * n_combos, n_rks, ctx->nk,
                                     ctx->nz, rtab_n, rtab_h, ctx->d_rtab.as<float4>(), st);
            ctx->launches++;
        }
        for (auto &g : groups) {
            WaveArgs a = base;
            a.chunks = ctx->d_desc.as<ChunkDesc>() + g.desc_off;
            a.n_chunks = (int) g.members.size();
            a.max_ld = g.max_ld;
            a.fws_bytes = g.fws_bytes;
            const size_t e0 = nev;
            nev += 3;
            record_event(pool_event(ctx, e0), st);
            launch_build_s_c(a, st);
            if (ctx->has_reso) launch_build_s_c_reso(a, st);
            if ((rc = step("build_s_c", g.max_ld, a.n_chunks))) return rc;
            record_event(pool_event(ctx, e0 + 1), st);
            launch_factor_all(a, st);
            if (a.host_failed)
                return set_err(ctx, LQG_ERR_CUDA, "factorisation: kernel attribute setup failed");
            if ((rc = step("factor", g.max_ld, a.n_chunks))) return rc;
            record_event(pool_event(ctx, e0 + 2), st);
            spans.push_back({e0, 0});
            spans.push_back({e0 + 1, 1});
            ctx->launches += a.launches;
            for (auto &w : g.waves) {
                WaveArgs b = base;
                const int nch = (int) w.members.size();
                b.chunks = ctx->d_desc.as<ChunkDesc>() + w.desc_off;
                b.n_chunks = nch;
                b.max_ld = w.ld;
                b.max_ns = w.max_ns;
                b.gt = w.gt;
                b.fws_bytes = g.fws_bytes;
                b.ws_bytes = w.ws_bytes;
                b.total_slots_q = w.slot_q; b.total_slots_r = w.slot_r; b.total_slots_p = w.slot_p;
                b.gram_splits = w.splits;
                b.sym = w.sym;
                b.w_tri = w.sym && no_marg;
                b.gemm_drain = w.drain;
                b.gemm_pair = w.pair;
                b.scales = ctx->d_scales.as<double>() + w.scales_off;
                if (precision == LQG_PRECISION_MIXED) {
                    __half *hb = ctx->d_halves.as<__half>();
                    const int64_t pl = (int64_t) w.ld * w.ld;
                    b.c_hi = hb; hb += pl * nch;
                    b.c_lo = hb; hb += pl * nch;
                    b.q_hi = hb; hb += pl * w.slot_q;
                    b.q_lo = hb; hb += pl * w.slot_q;
                    b.r_hi = hb; hb += pl * w.slot_r;
                    b.r_lo = hb; hb += pl * w.slot_r;
                    b.p_plane = w.sym ? sym_plane(w.ld) : pl;
                    b.p_hi = hb; hb += b.p_plane * w.slot_p;
                    b.p_lo = hb; hb += b.p_plane * w.slot_p;
                    b.gram_part = ctx->d_gram.as<float>();
                    b.gram_elems = (int64_t) nch * w.gt * w.gt * w.splits * 128 * 128;
                }
                const size_t w0 = nev;
                nev += 5;
                b.mid_event = pool_event(ctx, w0 + 2);
                const int *d_jobs = ctx->d_jobs.as<int>() + w.jobs_off;
                record_event(pool_event(ctx, w0), st);
                if (precision == LQG_PRECISION_MIXED) launch_scales_mixed(b, st);
                launch_build_q(b, st);
                if (ctx->has_reso) launch_build_q_reso(b, st);
                if ((rc = step("build_q", w.ld, nch))) return rc;
                record_event(pool_event(ctx, w0 + 1), st);
                if (precision == LQG_PRECISION_MIXED)
                    launch_products_mixed(b, st, d_jobs, w.njobs, ctx->d_jobs.as<int>() + w.jobs2_off, w.njobs2);
                else
                    launch_products_fp64(b, st, d_jobs, w.njobs);
                if (b.host_failed)
                    return set_err(ctx, LQG_ERR_CUDA,
                                   "products: kernel attribute setup or TMA descriptor encoding "
                                   "(cuTensorMapEncodeTiled) failed");
                if ((rc = step("products", w.ld, nch))) return rc;
                record_event(pool_event(ctx, w0 + 3), st);
                launch_finish(b, st);
                if ((rc = step("finish", w.ld, nch))) return rc;
                record_event(pool_event(ctx, w0 + 4), st);
                spans.push_back({w0, 2});
                spans.push_back({w0 + 1, 3});
                spans.push_back({w0 + 2, 4});
                spans.push_back({w0 + 3, 5});
                ctx->launches += b.launches;
                ctx->waves++;
            }
        }
        eacc = nev++;
        record_event(pool_event(ctx, eacc), st);
        if (ctx->fisher_band) {
            launch_fisher_band(ctx->d_meta.as<ChunkDesc>(), nb, ctx->d_results.as<double>(), ctx->results_size,
                               ctx->nk, st);
            ctx->launches++;
        }
        launch_accumulate(ctx->d_meta.as<ChunkDesc>(), nb, ctx->d_results.as<double>(), ctx->d_status.as<int>(),
                          ctx->nkz, ctx->d_fisher.as<double>(), ctx->d_dbt.as<double>(), st);
        ctx->launches++;
        record_event(ev_end, st);
        return LQG_OK;
    };
    // the key of everything a captured iteration would bake in
    std::vector<uintptr_t> key = {
        (uintptr_t) ctx->batch_version, (uintptr_t) precision, (uintptr_t) mode, (uintptr_t) use_theta,
        (uintptr_t) base.c_is_ff, (uintptr_t) ctx->d_fws.p, (uintptr_t) ctx->d_ws.p, (uintptr_t) ctx->d_halves.p,
        (uintptr_t) ctx->d_gram.p, (uintptr_t) ctx->d_desc.p, (uintptr_t) ctx->d_jobs.p, (uintptr_t) ctx->d_scales.p,
        (uintptr_t) ctx->d_fbounds.p, (uintptr_t) ctx->d_check.p, (uintptr_t) ctx->d_results.p,
        (uintptr_t) ctx->d_status.p, (uintptr_t) ctx->d_meta.p, (uintptr_t) ctx->d_wave.p, (uintptr_t) ctx->d_flogw.p,
        (uintptr_t) ctx->d_rw.p, (uintptr_t) ctx->d_sqiv2.p, (uintptr_t) ctx->d_niv.p, (uintptr_t) ctx->d_ttab.p,
        (uintptr_t) ctx->d_ttab_ff.p, (uintptr_t) ctx->wait_ns, (uintptr_t) n_combos, (uintptr_t) ctx->d_rtab.p,
        (uintptr_t) rtab_n, (uintptr_t) n_rks, (uintptr_t) ctx->fisher_band};
    // the launch plan: grid sizes and the by-value kernel arguments follow from these
    for (const auto &g : groups) {
        key.insert(key.end(), {(uintptr_t) g.members.size(), (uintptr_t) g.max_ld, (uintptr_t) g.fws_bytes,
                               (uintptr_t) g.desc_off, (uintptr_t) g.waves.size()});
        for (const auto &w : g.waves)
            key.insert(key.end(), {(uintptr_t) w.members.size(), (uintptr_t) w.ld, (uintptr_t) w.gt,
                                   (uintptr_t) w.splits, (uintptr_t) w.slot_q, (uintptr_t) w.slot_r,
                                   (uintptr_t) w.slot_p, (uintptr_t) w.ws_bytes, (uintptr_t) w.desc_off,
                                   (uintptr_t) w.jobs_off, (uintptr_t) w.scales_off, (uintptr_t) w.jobs2_off,
                                   (uintptr_t) w.njobs, (uintptr_t) w.njobs2, (uintptr_t) w.sym,
                                   (uintptr_t) w.drain, (uintptr_t) w.pair, (uintptr_t) w.max_ns});
    }
    auto cached = std::find_if(ctx->graphs.begin(), ctx->graphs.end(),
                               [&](const lqg_ctx::GraphEntry &g) { return g.key == key; });
    if (cached != ctx->graphs.end()) {
        LQG_CUDA_CHECK_RET(cudaGraphLaunch(cached->exec, st));
        ctx->launches = cached->launches;
        ctx->waves = cached->waves;
        spans = cached->spans;
        eacc = cached->eacc;
    } else {
        const bool seen = std::find(ctx->key_history.begin(), ctx->key_history.end(), key) != ctx->key_history.end();
        const bool capture = !sync_each && !ctx->graph_failed && seen;
        bool captured = false;
        if (capture && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            rc = launch_all();
            cudaGraph_t g = nullptr;
            const cudaError_t ec = cudaStreamEndCapture(st, &g);
            cudaGraphExec_t ge = nullptr;
            if (rc != LQG_OK) {
                // a launcher refused on the host (no kernel ran): report it and
                // keep capturing later iterations; the graph itself did not fail
                if (g) cudaGraphDestroy(g);
                cudaGetLastError();
                return rc;
            }
            if (ec == cudaSuccess && g && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess) {
                captured = true;
                if (ctx->graphs.size() >= lqg_ctx::kMaxGraphs) {
                    // the oldest entry goes; nothing of it can be in flight (the
                    // previous iteration synchronised)
                    cudaGraphExecDestroy(ctx->graphs.front().exec);
                    ctx->graphs.erase(ctx->graphs.begin());
                }
                lqg_ctx::GraphEntry ent;
                ent.key = key;
                ent.exec = ge;
                ent.launches = ctx->launches;
                ent.waves = ctx->waves;
                ent.spans = spans;
                ent.eacc = eacc;
                ctx->graphs.push_back(std::move(ent));
            } else {
                ctx->graph_failed = true;
            }
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            if (captured) {
                LQG_CUDA_CHECK_RET(cudaGraphLaunch(ge, st));
            }
        }
        if (!captured) {
            spans.clear();
            ctx->launches = 0;
            ctx->waves = 0;
            if ((rc = launch_all())) return rc;
        }
    }
    if (std::find(ctx->key_history.begin(), ctx->key_history.end(), key) == ctx->key_history.end()) {
        ctx->key_history.push_back(key);
        if (ctx->key_history.size() > lqg_ctx::kKeyHistory) ctx->key_history.erase(ctx->key_history.begin());
    }
    // index-check counters and statuses into the pinned staging buffer (the
    // uploads from it were enqueued before), read by finish_pending
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(hs, ctx->d_check.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    LQG_CUDA_CHECK_RET(cudaMemcpyAsync(hs + 4 * sizeof(unsigned long long), ctx->d_status.p, nb * 4,
                                       cudaMemcpyDeviceToHost, st));
    if (after && after != st) {
        // the caller's later work waits for the iteration's results
        cudaEvent_t ev = pool_event(ctx, eacc + 1);
        LQG_CUDA_CHECK_RET(cudaEventRecord(ev, st));
        LQG_CUDA_CHECK_RET(cudaStreamWaitEvent(after, ev, 0));
    }
    ctx->pending = true;
    ctx->pending_nb = nb;
    ctx->pending_spans = spans;
    ctx->pending_eacc = eacc;
    return LQG_OK;
}

}  // namespace

extern "C" int lqg_nr_iteration(lqg_ctx *ctx, const double *theta, int precision) {
    if (!ctx) return LQG_ERR_ARG;
    const int rc = enqueue_iteration(ctx, theta, precision, nullptr);
    if (rc) return rc;
    return finish_pending(ctx);
}

extern "C" int lqg_nr_iteration_async(lqg_ctx *ctx, const double *theta, int precision, void *stream) {
    if (!ctx) return LQG_ERR_ARG;
    return enqueue_iteration(ctx, theta, precision, static_cast<cudaStream_t>(stream));
}

extern "C" int lqg_download(lqg_ctx *ctx, double *d, double *b, double *t, double *fisher, int *chunk_status) {
    if (!ctx) return LQG_ERR_ARG;
    if (int rc = finish_pending(ctx)) return rc;
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
    if (int rc = finish_pending(ctx)) return rc;
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

namespace lqg {
int run_fast_bootstrap(cudaStream_t st, const ChunkDesc *d_meta, const double *d_results, int nkz, int n_chunks,
                       int n_qso, const int *qso_offsets, int nboots, unsigned long long seed,
                       const double *solver, double *mean, double *cov, double *fisher_cov, double *realizations,
                       std::string &err);
int run_complete_bootstrap(cudaStream_t st, const ChunkDesc *d_meta, const double *d_results, int nkz,
                           int n_chunks, const int *chunk_fis, const int *chunk_nq, int n_qso,
                           const int *qso_offsets, int nboots, unsigned long long seed, double *mean, double *cov,
                           double *realizations, int *n_valid, std::string &err);
int draw_coefficients(unsigned long long seed, int n_qso, int nboots, bool per_realization, unsigned char *p,
                      std::string &err);
}

extern "C" int lqg_bootstrap(lqg_ctx *ctx, int n_qso, const int *qso_offsets, int nboots, unsigned long long seed,
                             const double *solver_invfisher, double *mean, double *cov, double *fisher_cov,
                             double *realizations) {
    if (ctx) {
        if (int rc = finish_pending(ctx)) return rc;
    }
    if (!ctx || n_qso < 0 || !qso_offsets || nboots < 2)
        return set_err(ctx, LQG_ERR_ARG, "lqg_bootstrap: bad arguments");
    if (!ctx->have_results) return set_err(ctx, LQG_ERR_STATE, "lqg_bootstrap: no iteration on this batch yet");
    cudaSetDevice(ctx->device);
    return lqg::run_fast_bootstrap(ctx->stream, ctx->d_meta.as<ChunkDesc>(), ctx->d_results.as<double>(), ctx->nkz,
                                   (int) ctx->chunks.size(), n_qso, qso_offsets, nboots, seed, solver_invfisher,
                                   mean, cov, fisher_cov, realizations, ctx->err);
}

extern "C" int lqg_bootstrap_complete(lqg_ctx *ctx, int n_qso, const int *qso_offsets, int nboots,
                                      unsigned long long seed, double *mean, double *cov, double *realizations,
                                      int *n_valid) {
    if (ctx) {
        if (int rc = finish_pending(ctx)) return rc;
    }
    if (!ctx || n_qso < 0 || !qso_offsets || nboots < 2)
        return set_err(ctx, LQG_ERR_ARG, "lqg_bootstrap_complete: bad arguments");
    if (!ctx->have_results)
        return set_err(ctx, LQG_ERR_STATE, "lqg_bootstrap_complete: no iteration on this batch yet");
    cudaSetDevice(ctx->device);
    std::vector<int> fis(ctx->chunks.size()), nq(ctx->chunks.size());
    for (size_t c = 0; c < ctx->chunks.size(); ++c) {
        fis[c] = ctx->chunks[c].fis;
        nq[c] = ctx->chunks[c].nq;
    }
    return lqg::run_complete_bootstrap(ctx->stream, ctx->d_meta.as<ChunkDesc>(), ctx->d_results.as<double>(),
                                       ctx->nkz, (int) ctx->chunks.size(), fis.data(), nq.data(), n_qso,
                                       qso_offsets, nboots, seed, mean, cov, realizations, n_valid, ctx->err);
}

extern "C" int lqg_bootstrap_coefficients(int n_qso, int nboots, unsigned long long seed, int per_realization,
                                          unsigned char *p) {
    if (n_qso < 0 || nboots < 0 || !p) return LQG_ERR_ARG;
    std::string err;
    return lqg::draw_coefficients(seed, n_qso, nboots, per_realization != 0, p, err);
}

extern "C" int lqg_last_wave_count(const lqg_ctx *ctx) { return ctx ? ctx->waves : 0; }

extern "C" int lqg_last_h2d_bytes(const lqg_ctx *ctx, int64_t *bytes) {
    if (!ctx || !bytes) return LQG_ERR_ARG;
    *bytes = ctx->h2d_bytes;
    return LQG_OK;
}

extern "C" int lqg_set_wait_limit(lqg_ctx *ctx, double seconds) {
    if (!ctx || !(seconds >= 0.0) || seconds > 60.0) return LQG_ERR_ARG;
    ctx->wait_ns = (uint64_t) (seconds * 1e9);
    return LQG_OK;
}

extern "C" int lqg_set_fisher_optimization(lqg_ctx *ctx, int on) {
    if (!ctx || (on != 0 && on != 1)) return LQG_ERR_ARG;
    ctx->fisher_band = on;
    return LQG_OK;
}

extern "C" int lqg_sync(lqg_ctx *ctx) {
    if (!ctx) return LQG_ERR_ARG;
    cudaSetDevice(ctx->device);
    return finish_pending(ctx);
}

namespace {

// One iteration over a subset of the batch (the tuner's samples): the chunk
// list is swapped for the subset and restored; per-chunk results land at the
// chunks' own result offsets, the global sums are not meaningful.
int iterate_subset(lqg_ctx *ctx, const std::vector<int> &subset, int mode, double *ms) {
    std::vector<lqg_ctx::HostChunk> full;
    full.swap(ctx->chunks);
    for (int i : subset) ctx->chunks.push_back(full[i]);
    const uint64_t ver = ctx->batch_version;
    // the sample's own batch version, for the graph cache: a hash (FNV-1a) of
    // the batch's version and the sample's indices, so that repeats of one
    // sample replay its graph and no other sample or batch matches it; bit 62
    // keeps it apart from the counter of real batches
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](uint64_t v) {
        for (int k = 0; k < 8; ++k) { h ^= (v >> (8 * k)) & 0xff; h *= 1099511628211ull; }
    };
    mix(ver);
    mix(subset.size());
    for (int i : subset) mix((uint64_t) i);
    ctx->batch_version = ((uint64_t) 1 << 62) | (h & (((uint64_t) 1 << 62) - 1));
    int rc = enqueue_iteration(ctx, nullptr, mode, nullptr);
    if (rc == LQG_OK) rc = finish_pending(ctx);
    if (ms) *ms = ctx->timings[7];
    for (int s : ctx->last_status)
        if (rc == LQG_OK && s != LQG_CHUNK_OK) rc = set_err(ctx, LQG_ERR_STATE, "autotune: a sample chunk failed");
    ctx->chunks.swap(full);
    ctx->batch_version = ver;
    ctx->have_results = false;
    ctx->last_status.assign(ctx->chunks.size(), LQG_CHUNK_OK);
    return rc;
}

// Per-chunk results (3 nq + nq^2 doubles each) of the chunks at their offsets.
int read_results(lqg_ctx *ctx, const std::vector<int> &subset, std::vector<std::vector<double>> &out) {
    out.clear();
    for (int i : subset) {
        const auto &h = ctx->chunks[i];
        std::vector<double> buf(3 * h.nq + (size_t) h.nq * h.nq);
        LQG_CUDA_CHECK_RET(cudaMemcpy(buf.data(), ctx->d_results.as<double>() + h.res_off, buf.size() * 8,
                                      cudaMemcpyDeviceToHost));
        out.push_back(std::move(buf));
    }
    return LQG_OK;
}

// Largest error of mixed against FP64 over the chunks: d, b, t normwise, F
// per element normalised by sqrt(F_ii F_jj).
double max_error(const lqg_ctx *ctx, const std::vector<int> &subset, const std::vector<std::vector<double>> &mix,
                 const std::vector<std::vector<double>> &ref) {
    double worst = 0;
    for (size_t c = 0; c < subset.size(); ++c) {
        const int nq = ctx->chunks[subset[c]].nq;
        const double *x = mix[c].data(), *r = ref[c].data();
        for (int v = 0; v < 3; ++v) {
            double scale = 0, err = 0;
            for (int i = 0; i < nq; ++i) {
                scale = std::max(scale, std::fabs(r[v * nq + i]));
                err = std::max(err, std::fabs(x[v * nq + i] - r[v * nq + i]));
            }
            if (scale > 0) worst = std::max(worst, err / scale);
        }
        const double *f = x + 3 * nq, *fr = r + 3 * nq;
        for (int i = 0; i < nq; ++i)
            for (int j = i; j < nq; ++j) {
                double den = std::sqrt(std::fabs(fr[i * nq + i] * fr[j * nq + j]));
                if (den == 0) den = 1;
                worst = std::max(worst, std::fabs(f[i * nq + j] - fr[i * nq + j]) / den);
            }
    }
    return worst;
}

}  // namespace

extern "C" int lqg_autotune(lqg_ctx *ctx, double max_rel_err, int max_chunks, int flags) {
    if (!ctx) return LQG_ERR_ARG;
    if (!tc_available()) return set_err(ctx, LQG_ERR_UNSUPPORTED, "autotune: mixed path unavailable");
    cudaSetDevice(ctx->device);
    if (int rc = finish_pending(ctx)) return rc;
    if (max_rel_err <= 0) max_rel_err = 1e-5;
    if (max_chunks <= 0) max_chunks = 48;
    if (flags == 0) flags = 15;
    // the batch-wide buffers (statuses, metadata, results) are sized by the
    // whole batch before the sample iterations swap in their subsets
    if (int rc = upload_pixels(ctx)) return rc;
    std::map<int, std::vector<int>> buckets;   // padded size -> batch indices (table chunks only)
    for (int i = 0; i < (int) ctx->chunks.size(); ++i)
        if (ctx->chunks[i].nelem == 0) buckets[ctx->chunks[i].ld].push_back(i);
    if (buckets.empty()) return set_err(ctx, LQG_ERR_STATE, "autotune: no chunk in the batch");
    const std::map<int, lqg_ctx::Tune> saved = ctx->tuning;
    for (auto &bk : buckets) {
        const int ld = bk.first;
        std::vector<int> timing(bk.second.begin(), bk.second.begin() + std::min<size_t>(bk.second.size(), max_chunks));
        std::vector<int> acc(timing.begin(), timing.begin() + std::min<size_t>(timing.size(), 4));
        std::vector<std::vector<double>> ref, mix;
        int rc = iterate_subset(ctx, acc, LQG_PRECISION_FP64, nullptr);
        if (!rc) rc = read_results(ctx, acc, ref);
        if (rc) { ctx->tuning = saved; return rc; }
        lqg_ctx::Tune best;
        double best_ms = -1, best_err = 1e300;
        lqg_ctx::Tune best_any;   // the most accurate, if no candidate meets the bound
        for (int sym = 1; sym >= ((flags & 1) ? 0 : 1); --sym)
            for (int drain : {8, 4, 16}) {
                if (!(flags & 2) && drain != 8) continue;
                lqg_ctx::Tune t;
                t.sym = sym;
                t.drain = drain;
                ctx->tuning[ld] = t;
                rc = iterate_subset(ctx, acc, LQG_PRECISION_MIXED_AUTO, nullptr);
                if (!rc) rc = read_results(ctx, acc, mix);
                if (rc) { ctx->tuning = saved; return rc; }
                const double err = max_error(ctx, acc, mix, ref);
                if (err < best_err) { best_err = err; best_any = t; }
                // a margin on the sample leaves room for the chunks not sampled
                if (!(err <= 0.8 * max_rel_err)) continue;
                double ms = 0;
                // twice: the second replays the captured graph
                rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (!rc) rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (rc) { ctx->tuning = saved; return rc; }
                if (best_ms < 0 || ms < best_ms) { best_ms = ms; best = t; }
            }
        if (best_ms < 0) best = best_any;
        if ((flags & 8) && best_ms >= 0) {
            // the products on CTA pairs: the same arithmetic but for the drain
            // interval of slot ns - 1 (paired with S), so checked and timed again
            lqg_ctx::Tune t = best;
            t.pair = 1;
            ctx->tuning[ld] = t;
            rc = iterate_subset(ctx, acc, LQG_PRECISION_MIXED_AUTO, nullptr);
            if (!rc) rc = read_results(ctx, acc, mix);
            if (rc) { ctx->tuning = saved; return rc; }
            if (max_error(ctx, acc, mix, ref) <= 0.8 * max_rel_err) {
                double ms = 0;
                rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (!rc) rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (rc) { ctx->tuning = saved; return rc; }
                if (ms < best_ms) best = t;
            }
        }
        if (flags & 4) {
            double bms = -1;
            int bk_k = best.gram_k;
            for (int gk : {32768, 16384, 65536}) {
                lqg_ctx::Tune t = best;
                t.gram_k = gk;
                ctx->tuning[ld] = t;
                double ms = 0;
                rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (!rc) rc = iterate_subset(ctx, timing, LQG_PRECISION_MIXED_AUTO, &ms);
                if (rc) { ctx->tuning = saved; return rc; }
                if (bms < 0 || ms < bms) { bms = ms; bk_k = gk; }
            }
            best.gram_k = bk_k;
        }
        ctx->tuning[ld] = best;
    }
    return LQG_OK;
}

extern "C" int lqg_tuning_get(const lqg_ctx *ctx, int *entries, int n) {
    if (!ctx) return LQG_ERR_ARG;
    int k = 0;
    for (const auto &e : ctx->tuning) {
        if (entries && k < n) {
            int *r = entries + LQG_TUNING_FIELDS * k;
            r[0] = e.first;
            r[1] = e.second.sym;
            r[2] = e.second.drain;
            r[3] = e.second.gram_k;
            r[4] = e.second.pair;
        }
        ++k;
    }
    return k;
}

extern "C" int lqg_tuning_set(lqg_ctx *ctx, const int *entries, int n) {
    if (!ctx || n < 0 || (n > 0 && !entries)) return LQG_ERR_ARG;
    std::map<int, lqg_ctx::Tune> t;
    for (int k = 0; k < n; ++k) {
        const int *r = entries + LQG_TUNING_FIELDS * k;
        const int ld = r[0], sym = r[1], drain = r[2], gk = r[3], pair = r[4];
        if (ld <= 0 || ld % kPad || (sym != 0 && sym != 1) || drain < 1 || drain > 64 || gk < 4096 || gk % 64 ||
            (pair != 0 && pair != 1))
            return set_err(ctx, LQG_ERR_ARG, "lqg_tuning_set: bad entry " + std::to_string(k));
        lqg_ctx::Tune e;
        e.sym = sym;
        e.drain = drain;
        e.gram_k = gk;
        e.pair = pair;
        t[ld] = e;
    }
    ctx->tuning = t;
    return LQG_OK;
}

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
