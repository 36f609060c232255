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

}  // namespace

void launch_accumulate(const ChunkDesc *chunks, int n_chunks, const double *results,
                       const int *status, int nkz, double *fisher, double *dbt, cudaStream_t st) {
    int64_t total = (int64_t) nkz * nkz + 3 * nkz;
    int blocks = (int) ((total + 255) / 256);
    k_accumulate<<<blocks, 256, 3 * 1024 * sizeof(int), st>>>(chunks, n_chunks, results, status, nkz,
                                                               fisher, dbt);
}

}  // namespace lqg
