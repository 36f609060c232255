// lqg_factor_noalloc: the covariance factorisation of one chunk for callers
// that must not allocate device memory.
//
// lqg_nr_iteration sizes its workspaces from the batch and allocates them
// with cudaMalloc.  Some callers cannot let that happen inside their loop: a
// host thread with a latency budget cannot afford the device-wide
// synchronisation cudaMalloc and cudaFree may imply, a caller that owns a
// fixed memory pool must not have a library allocate behind its back, and a
// sequence of enqueued launches cannot be interrupted by a call that blocks.
// This entry point does the one step of the path whose scratch has a fixed
// bound for a given maximum chunk size: C~ = D C D + I, its Cholesky
// factorisation and inverse, C^-1 = D C~^-1 D, the continuum marginalisation
// and y = C^-1 delta.  Its scratch is a file-scope device array; every other
// buffer belongs to the caller, and nothing is allocated, freed or copied
// from the host.
#include "lqg_internal.cuh"

#include <algorithm>

namespace lqg {

namespace {

constexpr int kNoallocMaxLd = 4096;                     // largest padded chunk size
constexpr size_t kNoallocDescBytes = 256;               // ChunkDesc
constexpr size_t kNoallocBoundsOff = 256;               // 4 doubles: max |C^-1|, max row sum, 2 unused
constexpr size_t kNoallocScratchOff = 1024;             // 64 ld doubles of factorisation scratch
constexpr size_t kNoallocBytes = kNoallocScratchOff + (size_t) 64 * kNoallocMaxLd * sizeof(double);
static_assert(sizeof(ChunkDesc) <= kNoallocDescBytes, "descriptor slot too small");

// 2 MiB + 1 KiB per device.  Nothing in it needs to start at zero: the
// descriptor is written by k_noalloc_setup at the start of every call, and the
// factorisation writes each scratch row before it reads it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

__global__ void k_noalloc_setup(ChunkDesc d, ChunkDesc *slot, int *status) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *slot = d;
        *status = LQG_CHUNK_OK;
    }
}

// C~ = D C D + I in place (D = diag(sqrt(ivar))); padding rows and columns
// become the identity, so the factorisation sees an SPD ld x ld matrix.
__global__ void k_noalloc_whiten(double *cov, int n, int ld, const double *ivar) {
    const size_t total = (size_t) ld * ld;
    for (size_t e = (size_t) blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t) gridDim.x * blockDim.x) {
        const int i = (int) (e / ld), j = (int) (e % ld);
        double v = (i == j) ? 1.0 : 0.0;
        if (i < n && j < n) v += sqrt(ivar[i]) * cov[e] * sqrt(ivar[j]);
        cov[e] = v;
    }
}

}  // namespace

}  // namespace lqg

using namespace lqg;

extern "C" int lqg_factor_noalloc(int n, int ld, double *cov, const double *wave, const double *delta,
                                  const double *ivar, int cont_logl_order, int cont_l_order, double *y,
                                  int *status, void *stream) {
    if (n < 1 || ld < n || ld % kPad != 0 || !cov || !wave || !delta || !ivar || !y || !status)
        return LQG_ERR_ARG;
    if (ld > kNoallocMaxLd) return LQG_ERR_TOO_LARGE;
    int nvec = 0;
    if (cont_logl_order >= 0 || cont_l_order >= 0)
        nvec = 1 + (cont_logl_order > 0 ? cont_logl_order : 0) + (cont_l_order > 0 ? cont_l_order : 0);
    if (nvec > kMaxContVecs) return LQG_ERR_UNSUPPORTED;
    // the scratch's address on the current device, looked up on every call
    // (it allocates nothing, and a reset context reloads the module at
    // another address)
    void *sym = nullptr;
    if (cudaGetSymbolAddress(&sym, g_noalloc_scratch) != cudaSuccess || !sym) return LQG_ERR_CUDA;
    unsigned char *scratch = static_cast<unsigned char *>(sym);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    // Offsets of the caller's buffers relative to the scratch base, which the
    // factorisation kernel takes as its workspace base.
    const intptr_t base = reinterpret_cast<intptr_t>(scratch);
    ChunkDesc d{};
    d.n = n;
    d.ld = ld;
    d.pix = 0;
    d.gidx = 0;
    d.o_c = (int64_t) (reinterpret_cast<intptr_t>(cov) - base);
    d.o_y = (int64_t) (reinterpret_cast<intptr_t>(y) - base);
    d.o_fscr = (int64_t) kNoallocScratchOff;
    ChunkDesc *slot = reinterpret_cast<ChunkDesc *>(scratch);

    k_noalloc_setup<<<1, 32, 0, st>>>(d, slot, status);
    const int blocks = (int) std::min<size_t>(((size_t) ld * ld + 255) / 256, 4096);
    k_noalloc_whiten<<<blocks, 256, 0, st>>>(cov, n, ld, ivar);

    WaveArgs a{};
    a.chunks = slot;
    a.n_chunks = 1;
    a.max_ld = ld;
    a.fws = reinterpret_cast<char *>(scratch);
    a.fws_bytes = (int64_t) kNoallocBytes;
    a.ext_cy = 1;   // C^-1 and y live in the caller's buffers, outside the scratch
    a.fbounds = reinterpret_cast<double *>(scratch + kNoallocBoundsOff);
    a.status = status;
    a.wave = wave;
    a.delta = delta;
    a.ivar = ivar;
    a.cont_logl = cont_logl_order;
    a.cont_l = cont_l_order;
    a.precision = LQG_PRECISION_FP64;
    a.n_pix = n;
    a.check = nullptr;
    launch_factor_all(a, st);
    if (a.host_failed) return LQG_ERR_CUDA;
    return cudaGetLastError() == cudaSuccess ? LQG_OK : LQG_ERR_CUDA;
}
