// Throughput probe of the FP64 pipe, the denominator of the FP64 kernels'
// rooflines (the measured-peak file has HBM and tensor-core figures only).
// No counterpart in the reference.
#include "lqg_internal.cuh"

#include <algorithm>

namespace lqg {

namespace {

constexpr int kProbeChains = 8;      // independent FMA chains per thread
constexpr int kProbeIters = 4096;    // FMAs per chain

// Every thread runs kProbeChains independent DFMA chains of kProbeIters steps
// on values that stay finite (|x| < 1: x <- x a + b with |a| < 1, |b| small);
// the sum is stored so that nothing is optimised away.
__global__ void __launch_bounds__(256) k_probe_dfma(double a, double b, double *out) {
    double x[kProbeChains];
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) x[c] = 1e-3 * (threadIdx.x + c);
    for (int i = 0; i < kProbeIters; ++i)
#pragma unroll
        for (int c = 0; c < kProbeChains; ++c) x[c] = fma(x[c], a, b);
    double s = 0;
#pragma unroll
    for (int c = 0; c < kProbeChains; ++c) s += x[c];
    if (s == 12345.678) out[0] = s;   // never true; keeps the chains live
}

}  // namespace

}  // namespace lqg

using namespace lqg;

extern "C" int lqg_probe_fp64_rate(int device, double *tflops) {
    if (!tflops) return LQG_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) return LQG_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0)
        return LQG_ERR_CUDA;
    double *out = nullptr;
    if (cudaMalloc(&out, 8) != cudaSuccess) return LQG_ERR_NOMEM;
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = LQG_OK;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess)
        rc = LQG_ERR_CUDA;
    const int blocks = sms * 8, threads = 256;
    const double flops = 2.0 * kProbeChains * kProbeIters * (double) blocks * threads;
    double best = 0;
    for (int rep = 0; rep < 6 && rc == LQG_OK; ++rep) {
        cudaEventRecord(e0, st);
        k_probe_dfma<<<blocks, threads, 0, st>>>(0.999999, 1e-7, out);
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) { rc = LQG_ERR_CUDA; break; }
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);   // first: warm-up
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(out);
    if (rc == LQG_OK && cudaGetLastError() != cudaSuccess) rc = LQG_ERR_CUDA;
    *tflops = best;
    return rc;
}
