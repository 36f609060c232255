// Internal declarations shared by the engine's translation units.
#pragma once

#include <algorithm>
#include <atomic>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lqg.h"

namespace lqg {

constexpr double kSpeedOfLight = 299792.458;   // core/global_numbers.hpp:17-22
constexpr double kLyaRest = 1215.67;
constexpr double kPi = 3.14159265358979323846;
constexpr double kDoubleEpsilon = 1e-15;

constexpr int kPad = 64;          // matrices are stored with a leading dimension that is a multiple of 64
constexpr int kMaxPixels = 8192;  // largest chunk the engine accepts
constexpr int kMaxContVecs = 4;
constexpr int kMaxGramBlocks = 4; // ns + 2 <= 128 kMaxGramBlocks stored matrices per chunk

// One chunk of the batch: what Chunk::Chunk computes (core/chunk_estimate.cpp:141-257)
// plus the device offsets of its data and workspace.
struct ChunkDesc {
    int n;                // pixels (size())
    int ld;               // leading dimension of its N x N matrices (n rounded up to kPad)
    int nq;               // N_Q_MATRICES
    int ns;               // number of stored derivative matrices (kn < KBIN_UPP)
    int kbin_upp;         // KBIN_UPP
    int fis;              // fisher_index_start
    int res;              // table index (RES_INDEX)
    int zb0;              // first redshift bin of the chunk's matrices = fis / nk
    int64_t pix;          // offset of the pixel arrays
    int64_t res_off;      // offset of the per-chunk results (3 nq + nq^2 doubles)
    // Factor workspace (bytes, relative to WaveArgs::fws): S_fid, C~ -> C^-1, y and
    // the factorisation scratch (64 ld doubles), kept for the whole iteration.
    int64_t o_s, o_c, o_y, o_fscr;
    // Mixed path: the marginalised C^-1 in FP64 at o_m when cinv_m is set (its
    // own buffer in the whitened form, o_c in the direct form), read by
    // k_dx_mixed for the partials of x_s = tr(Q_s C^-1).
    int64_t o_m;
    int cinv_m;
    // Wave workspace (bytes, relative to WaveArgs::ws): FP64 product stacks, per-tile
    // d partials (and x partials, mixed path) and FP64 Gram partials.
    int64_t o_q, o_r, o_p, o_part, o_dpart, o_xpart;
    int slot_q, slot_r, slot_p;  // first matrix slot of this chunk in the stacked operand buffers
    int gidx;             // index of the chunk in the batch (factor bounds, status)
    int status;
    // Resolution matrix (UseResoMatrix; nelem = 0 without one).  Coarse row r
    // has weights rw[rw_off + r * nelem + a] at grid point r * os + a - sh of
    // a grid of nf points (the oversampled grid, or the pixels themselves for
    // a diagonal matrix), whose ln(lambda) and sqrt(lambda) start at fpix.
    int nelem, os, sh, nf;
    int64_t fpix, rw_off;
    int64_t o_ph;         // wave workspace: cos, sin of k_c u at each grid point (mixed path)
    int tcombo;           // row block of this chunk's (table, KBIN_UPP) in WaveArgs::ttab, or of a
                          // resolution-matrix chunk's KBIN_UPP in WaveArgs::rtab
    int sym;              // mixed path: whitened symmetric form (else direct)
    double rw_sum;        // largest sum of |weights| of a row (bound of R M R^T)
};

constexpr int kMaxKBands = 256;   // largest NUMBER_OF_K_BANDS

struct DeviceBins {
    int nk, nz, nkz, triangular;
    double dz;
    double z_centers[64];
    double k_edges[kMaxKBands + 1];
    // double-float (hi + lo) forms for the FP32-pipe element math of the
    // mixed path: 1 + z_c per bin, dz, dz / 2, and 1 / dz
    float zc1_hi[64], zc1_lo[64];
    float dz_hi, dz_lo, dzh_hi, dzh_lo, inv_dz;
    float idz_hi, idz_lo;   // 1 / dz as double-float
    // RedshiftGrowthOn: Q_k of bin m scaled by ((1 + z_ij) / (1 + z_m))^B
    int growth;
    double growth_b;
};

// Redshift weight of bin zm at z, element-wise form of bins::zBinTriangular1/2,
// zBinTriangular and zBinTopHat (core/global_numbers.cpp:393-471); on the
// sorted rows the reference walks these conditions select the same elements.
// With the growth option on, times ((1 + z) / (1 + z_m))^B
// (Chunk::_scaleDerivativesWithRedshiftGrowth, core/chunk_estimate.cpp:539-573,
// which takes 1 + z_ij as z_ij + 1 and 1 + z_m as ZBIN_CENTERS[m] + 1).
__device__ __forceinline__ double zfactor(const DeviceBins &b, int zm, double z) {
    const double zc = b.z_centers[zm], dz = b.dz;
    double w;
    if (!b.triangular || b.nz == 1) w = (z >= zc - dz / 2 && z <= zc + dz / 2) ? 1.0 : 0.0;
    else if (zm == 0 && z < zc) w = 1.0;
    else if (zm == b.nz - 1 && z > zc) w = 1.0;
    else if (z >= zc - dz && z <= zc + dz) w = 1.0 - fabs(z - zc) / dz;
    else w = 0.0;
    if (b.growth && w != 0.0) w *= pow((z + 1.0) / (zc + 1), b.growth_b);
    return w;
}

struct TableGrid {
    int nv, nzp, n_tables;
    double v1, dv, z1, dz;
    float kv_hi, kv_lo;   // speed of light / dv as double-float
    float z1p_hi, z1p_lo; // 1 + z1 as double-float
    float idz_hi, idz_lo; // 1 / dz as double-float
};

// Thin RAII for device allocations owned by the context.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    ~DevBuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) {
        if (p && bytes >= n) return cudaSuccess;
        if (p) { cudaFree(p); p = nullptr; bytes = 0; }
        if (n == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) bytes = n;
        return e;
    }
    // Release the buffer when it is much larger than n: the iteration planner
    // counts held buffers as free memory, so an oversized one (from a larger
    // plan, e.g. the FP64 path before the mixed one) must go before the
    // other buffers of the new plan are allocated.
    void trim(size_t n) {
        if (p && bytes > n + n / 4) { cudaFree(p); p = nullptr; bytes = 0; }
    }
    template <class T> T *as() const { return static_cast<T *>(p); }
};

inline int64_t align_up(int64_t x, int64_t a) { return (x + a - 1) / a * a; }

// ---- kernel launchers (defined in the .cu files) ----
struct WaveArgs {
    const ChunkDesc *chunks;     // device
    int n_chunks;
    int max_ld;
    int max_ns;                  // largest stored-slot count of the wave
    char *ws;                    // wave workspace base
    char *fws;                   // factor workspace base
    double *fbounds;             // per batch chunk: max |C^-1|, largest row sum of |C^-1|
    int gt;                      // Gram blocks of 128 per dimension (ns + 2 <= 128 gt)
    const double *wave, *delta, *ivar, *logw, *sqw;  // pixel arrays
    const float2 *logw2, *sqw2;                      // ln w and sqrt w as double-float (hi, lo)
    const double *sqiv, *niv;                        // sqrt(ivar), and 1 / ivar (0 where ivar = 0)
    const float2 *sqiv2;                             // sqrt(ivar) as double-float
    int c_is_ff;                                     // S and C~ written as double-float pairs (mixed, no theta)
    const double *flogw, *fsqw, *rw;                 // resolution-matrix grids and weights
    int reso_nelem, reso_os;                         // shape shared by every resolution chunk, else 0
    int growth;                                      // RedshiftGrowthOn (as DeviceBins::growth)
    int sym;                                         // mixed path in the whitened symmetric form
    int dbt_id;                                      // mixed path: d - b - t from the x partials (see k_finish)
    int w_tri;                                       // W lower triangular (no marginalisation)
    int gemm_drain;                                  // K blocks per drained hi*hi partial of the products; 0: 8
    int gemm_pair;                                   // products on CTA pairs (k_tc_gemm_pair)
    int64_t p_plane;                                 // elements of one P slot
    const double *deriv, *signal, *qmax;             // tables
    const float *deriv_f;                            // float copy of deriv (mixed path)
    const float4 *deriv_ff;                          // per node: deriv and (next - this) as double-floats
    const float2 *signal_ff;                         // signal table as double-float (mixed path)
    const double *theta;                             // device, nkz
    // theta-weighted derivative tables: ttab[(tcombo nz + zm) nv + v] =
    // sum_{kn < KBIN_UPP} theta[zm nk + kn] deriv[table][kn][v] (nullptr without theta)
    const double *ttab;
    const float2 *ttab_ff;                           // the same rows as double-float (mixed path)
    // resolution-matrix chunks, mixed path with theta: G(v) = sum_{kn < KBIN_UPP}
    // theta[zm nk + kn] Q_kn(v) (the analytic band derivative) at v = i h, row
    // (tcombo nz + zm) of rtab_n nodes (G hi, G lo, h G', 0) (nullptr otherwise)
    const float4 *rtab;
    int64_t rtab_n;
    float2 rtab_x;                                   // c / h as double-float
    double *results;                                 // per-chunk results
    int *status;                                     // per-chunk status (wave-local)
    TableGrid grid;
    DeviceBins *bins;                                // device pointer
    int cont_logl, cont_l, turn_off_sfid, skip_fisher;
    int precision;
    int total_slots_q, total_slots_r, total_slots_p;
    __half *q_hi, *q_lo, *r_hi, *r_lo, *p_hi, *p_lo, *c_hi, *c_lo;  // mixed operand planes
    float *gram_part;
    int gram_splits;
    double *scales;              // per-slot scales (mixed): q [slots], r, p and c
    int launches;
    int host_failed;             // set by a launcher that could not launch (host side)
    cudaEvent_t mid_event;       // recorded between the product and the Gram kernels
    // extents of the buffers above, used by the LQG_CHECKED build to validate indices
    int64_t ws_bytes, fws_bytes, results_elems, gram_elems, n_pix, n_fpix, n_rw;
    int ext_cy;                  // C and y are caller buffers (o_c, o_y may fall outside fws)
    uint64_t wait_ns;            // limit of the tensor-core pipeline waits; 0: 2 s
    unsigned long long *check;   // [0] violations, [1] first code, [2] first chunk, [3] first index
};

// Self-checking build (-DLQG_CHECKED): an index that would leave its buffer is
// counted and the access skipped, so that a bad launch reports instead of faulting.
#ifdef LQG_CHECKED
__device__ __forceinline__ bool lqg_in_bounds(const WaveArgs &a, bool ok, int code, int chunk,
                                              long long idx) {
    if (!ok && a.check) {
        if (atomicAdd(&a.check[0], 1ull) == 0ull) {
            a.check[1] = (unsigned long long) code;
            a.check[2] = (unsigned long long) chunk;
            a.check[3] = (unsigned long long) idx;
        }
    }
    return ok;
}
#define LQG_IN_BOUNDS(a, cond, code, chunk, idx) lqg_in_bounds((a), (cond), (code), (chunk), (long long) (idx))
#else
#define LQG_IN_BOUNDS(a, cond, code, chunk, idx) true
#endif

// Phase A (all chunks of a group): S_fid and C~, then the FP64 factorisation.
void launch_build_s_c(WaveArgs &a, cudaStream_t st);
// The theta-weighted tables of an iteration (before the groups' S/C builds).
void launch_theta_tables(const double *deriv, const double *theta, const int *combos, int n_combos, int nk, int nz,
                         int nv, double *ttab, float2 *ttab_ff, cudaStream_t st);
void launch_theta_reso_tables(const double *theta, const DeviceBins *bins, const int *ks, int n_ks, int nk, int nz,
                              int64_t nn, double h, float4 *rtab, cudaStream_t st);
// The same two matrix builds for chunks with a resolution matrix (lqg_reso.cu);
// each kind of kernel skips the chunks of the other kind.
void launch_build_s_c_reso(WaveArgs &a, cudaStream_t st);
void launch_build_q_reso(WaveArgs &a, cudaStream_t st);
constexpr int kResoTile = 32;     // coarse tile edge of the resolution-matrix kernels
constexpr int kResoMaxFine = 128; // largest fine extent of a tile: (kResoTile - 1) os + nelem
constexpr int kResoMaxElem = 48;  // largest number of weights per row
void launch_factor_all(WaveArgs &a, cudaStream_t st);
size_t factor_smem_bytes();
// Phase B (per wave): Q_k, products, traces, per-chunk results.
void launch_build_q(WaveArgs &a, cudaStream_t st);
void launch_products_fp64(WaveArgs &a, cudaStream_t st, const int *d_jobs, int njobs);
void launch_products_mixed(WaveArgs &a, cudaStream_t st, const int *d_jobs, int njobs, const int *d_jobs2,
                           int njobs2);
void launch_scales_mixed(WaveArgs &a, cudaStream_t st);
void launch_finish(WaveArgs &a, cudaStream_t st);

// Timing event on the stream; inside a stream capture it becomes an external
// event record node, which (unlike the default internal one) can be timed
// (the external flag is refused outside a capture)
inline void record_event(cudaEvent_t e, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusActive)
        cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
    else
        cudaEventRecord(e, st);
}

// Per-device one-time setup for a launcher: true once fn() has returned
// cudaSuccess on the current device.  Kernel attributes (dynamic shared memory
// above 48 KB) are per device; two host threads that race here both run fn,
// which only sets attributes, so the race is harmless.  A device index beyond
// the mask runs fn on every call.
template <class Fn>
inline bool once_per_device(std::atomic<unsigned long long> &done, Fn fn) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return true;
    if (fn(dev) != cudaSuccess) return false;
    if (bit) done.fetch_or(bit, std::memory_order_release);
    return true;
}

// fn(i) for i in [0, n) on up to 16 host threads (the calling one included),
// handed out `grain` at a time; serial when n <= grain.  fn must not throw
// and must write no state that another i writes.  A thread the system does
// not grant is simply not used: the others take its share.
template <class Fn>
inline void host_parallel_for(int n, int grain, Fn fn) {
    if (n <= 0) return;
    const unsigned hw = std::thread::hardware_concurrency();
    const int nt = (int) std::min<long long>({16ll, hw ? (long long) hw : 1ll, (n + (long long) grain - 1) / grain});
    if (nt <= 1) {
        for (int i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<int> next{0};
    auto worker = [&] {
        for (int i0; (i0 = next.fetch_add(grain, std::memory_order_relaxed)) < n;)
            for (int i = i0; i < std::min(n, i0 + grain); ++i) fn(i);
    };
    std::vector<std::thread> pool;
    pool.reserve(nt - 1);
    for (int t = 1; t < nt; ++t) {
        try {
            pool.emplace_back(worker);
        } catch (...) {
            break;
        }
    }
    worker();
    for (auto &th : pool) th.join();
}

bool tc_available();
int gram_splits_mixed(int64_t K, int gram_k);
// Elements of one compact upper-triangle slot of the whitened form: the
// ceil(ld / 128) (ceil(ld / 128) + 1) / 2 tiles of 128 x 128 on and above the diagonal
inline int64_t sym_plane(int ld) {
    const int64_t mt = (ld + 127) / 128;
    return mt * (mt + 1) / 2 * 128 * 128;
}
// Smoother::smoothIvar on the host (lqg_smooth.cu)
int smooth_ivar(int n, const double *ivar, int sigmapix, double *out);

}  // namespace lqg

#define LQG_CUDA_CHECK_RET(expr)                                               \
    do {                                                                       \
        cudaError_t _e = (expr);                                               \
        if (_e != cudaSuccess) {                                               \
            ctx->err = std::string(#expr) + ": " + cudaGetErrorString(_e);     \
            return LQG_ERR_CUDA;                                               \
        }                                                                      \
    } while (0)
