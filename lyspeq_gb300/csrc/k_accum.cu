// Global accumulation of the per-chunk results (core/chunk_estimate.cpp:893-903
// and the MPI allreduce at core/quadratic_estimate.cpp:469-475, which on one GPU
// is this on-device reduction).  Every output element is owned by one thread,
// which adds the chunks in batch order: the sum is deterministic.
#include "lqg_internal.cuh"

namespace lqg {

namespace {

__global__ void k_accumulate(const ChunkDesc *chunks, int n_chunks, const double *results,
                             const int *status, int nkz, double *fisher, double *dbt) {
    extern __shared__ int smeta[];   // fis, nq, status per chunk of the current block of chunks
    const int64_t total = (int64_t) nkz * nkz + 3 * nkz;
    const int64_t e = (int64_t) blockIdx.x * blockDim.x + threadIdx.x;
    int r = -1, c = -1, which = -1;
    if (e < (int64_t) nkz * nkz) { r = (int) (e / nkz); c = (int) (e % nkz); }
    else if (e < total) { which = (int) ((e - (int64_t) nkz * nkz) / nkz); r = (int) ((e - (int64_t) nkz * nkz) % nkz); }
    double acc = 0.0;
    const int CH = 1024;
    for (int base = 0; base < n_chunks; base += CH) {
        int cnt = min(CH, n_chunks - base);
        __syncthreads();
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            smeta[3 * i] = chunks[base + i].fis;
            smeta[3 * i + 1] = chunks[base + i].nq;
            smeta[3 * i + 2] = status[base + i];
        }
        __syncthreads();
        if (e >= total) continue;
        for (int i = 0; i < cnt; ++i) {
            int fis = smeta[3 * i], nq = smeta[3 * i + 1];
            if (smeta[3 * i + 2] != LQG_CHUNK_OK) continue;
            const double *res = results + chunks[base + i].res_off;
            if (which < 0) {
                if (r < fis || c < r || c >= fis + nq) continue;
                acc += res[3 * nq + (int64_t) (r - fis) * nq + (c - fis)];
            } else {
                if (r < fis || r >= fis + nq) continue;
                acc += res[which * nq + (r - fis)];
            }
        }
    }
    if (e < (int64_t) nkz * nkz) fisher[e] = acc;
    else if (e < total) dbt[which * nkz + r] = acc;
}

// lyspeq built with FISHER_OPTIMIZATION (./configure --enable-fisher-optimization)
// computes of a chunk's Fisher matrix only the pairs i <= j of local kz indices
// with j - i <= 5 or |j - i - Nk| <= 2 (core/chunk_estimate.cpp:823-827); the
// others stay 0.  One block per chunk zeroes them in the chunk's results
// (upper triangle; the lower one is 0 already), before the accumulation.
__global__ void k_fisher_band(const ChunkDesc *chunks, int n_chunks, double *results, int64_t results_elems,
                              int nk) {
    const int c = blockIdx.x;
    if (c >= n_chunks) return;
    const int nq = chunks[c].nq;
    const int64_t off = chunks[c].res_off + 3 * (int64_t) nq;
    if (nq <= 0 || chunks[c].res_off < 0 || off + (int64_t) nq * nq > results_elems) return;
    double *f = results + off;
    for (int64_t e = threadIdx.x; e < (int64_t) nq * nq; e += blockDim.x) {
        const int diff = (int) (e % nq) - (int) (e / nq);
        if (diff > 5 && abs(diff - nk) > 2) f[e] = 0.0;
    }
}

}  // namespace

void launch_fisher_band(const ChunkDesc *chunks, int n_chunks, double *results, int64_t results_elems, int nk,
                        cudaStream_t st) {
    if (n_chunks <= 0) return;
    k_fisher_band<<<n_chunks, 256, 0, st>>>(chunks, n_chunks, results, results_elems, nk);
}

void launch_accumulate(const ChunkDesc *chunks, int n_chunks, const double *results,
                       const int *status, int nkz, double *fisher, double *dbt, cudaStream_t st) {
    int64_t total = (int64_t) nkz * nkz + 3 * nkz;
    int blocks = (int) ((total + 255) / 256);
    k_accumulate<<<blocks, 256, 3 * 1024 * sizeof(int), st>>>(chunks, n_chunks, results, status, nkz,
                                                               fisher, dbt);
}

}  // namespace lqg
