// Tensor-core kernels of the mixed-precision path (sm_103a, tcgen05 + TMA).
//
// Every FP64 operand X is stored as two fp16 planes, hi = fp16(s X) and
// lo = fp16(s X - hi), with a power-of-two scale s chosen so |s X| <= 2^14;
// hi + lo carries 22 significant bits.  A product is taken as
//     A B ~= A_hi B_hi + A_hi B_lo + A_lo B_hi
// (three tcgen05.mma kind::f16 per K step, fp32 accumulation in tensor
// memory); the dropped A_lo B_lo term is below 2^-22 relative.
//
// k_tc_gemm:  A_s = C^-1 Q_s for every stored derivative matrix and A_S = C^-1 S
//             (Chunk::_getWeightedMatrix, core/chunk_estimate.cpp:721-736, and
//             the S_fid C^-1 product at :796-799).  The epilogue writes A_s as
//             hi/lo planes twice: row-major into R and transposed into P.  The
//             whitened form's two stages (X_s = W Q_s, B_s = X_s W^T) are
//             stages 1 and 2 of the same persistent kernel.
// k_tc_gemm_pair: the same products on CTA pairs (cta_group::2, 256 x 128
//             tiles), an autotuned alternative per padded size.
// k_tc_gram:  G = P R^T over K = ld^2 (or the whitened form's compact upper
//             tiles), split over K; per-split fp32 partial tiles are reduced in
//             FP64 by k_finish.  Rows of P are A_s^T, A_S^T = S C^-1 and
//             N C^-1, so G holds F_ij = <A_i^T, A_j>, t_j and b_j
//             (core/chunk_estimate.cpp:783-832).
//
// Warp roles (320 threads): warp 0 issues TMA loads, warp 1 owns tensor memory
// and issues the MMAs, warps 2-9 drain the accumulators.  Every wait on an
// mbarrier is bounded by a wall-clock limit; on timeout the kernel records an
// error in the chunk status and leaves after its own work has drained.
#include "lqg_internal.cuh"

#include <algorithm>
#include <cuda.h>
#include <cudaTypedefs.h>

namespace lqg {

namespace {

constexpr uint64_t kWaitLimitNs = 2000000000ull;   // 2 s per wait

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Bounded wait for the phase of the given parity to complete.  The pipeline
// waits take the iteration's limit (lqg_set_wait_limit; 2 s unless set); the
// waits of a CTA's exit for its own copies and MMAs always take 2 s.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
    uint64_t t0 = 0;
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        uint64_t t = now_ns();
        if (t0 == 0) t0 = t;
        else if (t - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
        "%4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(z)
        : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
        "%4}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

// Shared-memory matrix descriptor of a K-major tile written by TMA with
// 128-byte swizzle: rows of 64 fp16 (128 B), 8-row groups 1024 B apart.
__device__ __forceinline__ uint64_t sw128_desc(const void *tile) {
    uint64_t addr = smem_u32(tile);
    uint64_t d = (addr & 0x3FFFF) >> 4;      // start address
    d |= (uint64_t) 1 << 16;                  // leading byte offset (unused with this swizzle)
    d |= (uint64_t) (1024 >> 4) << 32;        // stride byte offset
    d |= (uint64_t) 1 << 46;                  // descriptor version
    d |= (uint64_t) 2 << 61;                  // 128-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: fp16 A and B (K-major), fp32 D.
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
    return (1u << 4) | ((uint32_t) (n >> 3) << 17) | ((uint32_t) (m >> 4) << 24);
}

__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// The .sync.aligned tcgen05 instructions below must be executed by all 32
// lanes of a converged warp; callers reach them after divergent waits and
// branches, so each helper re-converges the warp first.
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive fp32 columns of this warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
        "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
        "%30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]),
          "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]),
          "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 64 consecutive fp32 columns of this warp's 32 lanes: one load, one wait.
__device__ __forceinline__ void tmem_ld64(uint32_t taddr, float (&v)[64]) {
    uint32_t r[64];
    __syncwarp();
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
        "%13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, "
        "%32, %33, %34, %35, %36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, "
        "%51, %52, %53, %54, %55, %56, %57, %58, %59, %60, %61, %62, %63}, [%64];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31]), "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]),
          "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]), "=r"(r[40]), "=r"(r[41]), "=r"(r[42]),
          "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]), "=r"(r[48]), "=r"(r[49]),
          "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]), "=r"(r[56]),
          "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}

// Store 32 consecutive fp32 columns of this warp's 32 lanes (waits for completion).
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const float (&v)[32]) {
    __syncwarp();
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
        "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
        "%30, %31, %32};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
        "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
        "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
        "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
        "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
        "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

// ---- CTA pairs (cta_group::2): a cluster of two CTAs on one TPC ------------
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Address in the cluster's shared window of this CTA's variable p in CTA rank.
__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
    return r;
}

__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_cluster(uint32_t caddr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}

// TMA load into this CTA's shared memory that completes on the mbarrier at
// cluster address bar_cl, in this CTA or the other CTA of the pair.
__device__ __forceinline__ void tma_load_3d_pair(void *dst, const CUtensorMap *map, uint32_t bar_cl, int x, int y,
                                                 int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
        "%4, %5}], [%2];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cl), "r"(x), "r"(y), "r"(z)
        : "memory");
}

__device__ __forceinline__ void st_cluster_u32(uint32_t caddr, uint32_t v) {
    asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(caddr), "r"(v) : "memory");
}

// mbar_wait for barriers that the other CTA of the pair (or its MMAs) arrive on.
__device__ __forceinline__ bool mbar_wait_cl(uint64_t *bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
    uint64_t t0 = 0;
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(ok)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (ok) return true;
        uint64_t t = now_ns();
        if (t0 == 0) t0 = t;
        else if (t - t0 > limit_ns) return false;
    }
}

// One MMA of the pair, issued by the even CTA: D (128 lanes of each CTA's
// tensor memory) += A (128 rows from each CTA) B^T (N / 2 rows from each CTA),
// all at the same shared-memory and tensor-memory offsets in both CTAs.
__device__ __forceinline__ void umma_f16_pair(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                              uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

// Arrive on the barrier at this offset in both CTAs once the pair's MMAs so far complete.
__device__ __forceinline__ void umma_commit_pair(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
            smem_u32(bar)),
        "h"((unsigned short) 3)
        : "memory");
}

// Tensor memory of a pair: the same columns in both CTAs, allocated and freed
// by one warp of each.
__device__ __forceinline__ void tmem_alloc_pair(uint32_t *dst, uint32_t ncols) {
    __syncwarp();
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols) {
    __syncwarp();
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ double pow2_floor(double x) {
    if (!(x > 0) || !isfinite(x)) return 1.0;
    int e;
    frexp(x, &e);
    return ldexp(1.0, e - 1);
}

constexpr int BK = 64;                      // fp16 elements per K step (128 bytes)
constexpr int G_BM = 128, G_BN = 128, G_STAGES = 3;
constexpr int G_TILE_A = G_BM * BK * 2, G_TILE_B = G_BN * BK * 2;
constexpr int G_STAGE_BYTES = 2 * G_TILE_A + 2 * G_TILE_B;
constexpr int kStoreStage = 2048;                        // per epilogue warp: 32 rows x 64 bytes
constexpr int kStoreStages = 8 * kStoreStage;
constexpr int G_SMEM = G_STAGES * G_STAGE_BYTES + kStoreStages + 1024 + 256;
constexpr int R_BM = 128, R_BN = 128, R_STAGES = 3;
constexpr int R_TILE = R_BM * BK * 2;
constexpr int R_STAGE_BYTES = 4 * R_TILE;
constexpr int kGramBox = 32;                      // rows per TMA box of the Gram operands
constexpr int kGramBoxBytes = kGramBox * BK * 2;  // 4 KB: whole 1024-byte swizzle groups
constexpr int R_SMEM = R_STAGES * R_STAGE_BYTES + 1024 + 256;
constexpr int TC_THREADS = 320;             // producer, MMA, 8 epilogue warps
constexpr int R_THREADS = TC_THREADS;
constexpr int kGramK = 32768;               // K elements per Gram split
constexpr int kGemmDrain = 8;               // K blocks per drained hi*hi partial: products
constexpr int kGemmDrainST = 2;             // the whitened form's S and N slots
constexpr int kGramDrain = 2;               // and traces

// Accumulation: the tensor cores round every fp32 accumulation of an MMA, with a
// bias that grows with the number of accumulations into one accumulator.  The
// hi*hi products and the (2^11 times smaller) cross products therefore go to
// separate TMEM accumulators, and the hi*hi accumulator is drained every DRAIN
// K blocks (4 DRAIN MMAs of K = 16: 32 in the products, 8 in the traces) into
// fp32 sums held in registers: a ping-pong pair of hi*hi accumulators lets the
// MMAs continue while one is drained.
//
// TMEM columns: hi*hi ping [0, 128), pong [128, 256), cross [256, 384).
// Epilogue warps 2..9: warp w reads TMEM lanes 32 (w % 4) .. +31 and the 64
// columns 64 ((w - 2) / 4) .. +63 of each accumulator.

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// MMA issuer, one output tile: for each drain group (DRAIN K blocks)
// accumulate hi*hi into hi*hi buffer (g_all & 1) of [thh, thh + 2 BN), fresh
// per group, and the cross terms into tx, fresh at the tile's first K block.
// kb_all (shared-memory stage ring) and g_all (hi*hi buffers) run on across
// the tiles of a persistent CTA.  Commits `done` after the tile's last MMA.
// Returns false after a timed-out wait (abort flag set).
// Stage layout: A hi, A lo, B hi, B lo.
template <int STAGES, int STAGE_BYTES, int TILE_A, int TILE_B, int BN>
__device__ __forceinline__ bool mma_tile(uint32_t thh, uint32_t tx, unsigned char *smem, uint64_t *full,
                                         uint64_t *empty, uint64_t *dfull, uint64_t *dempty, uint64_t *done,
                                         int kblocks, int DRAIN, uint32_t idesc, int &kb_all, int &g_all,
                                         int *abort_flag, uint64_t lim) {
    const int ngroups = (kblocks + DRAIN - 1) / DRAIN;
    for (int g = 0; g < ngroups; ++g) {
        const int b = g_all & 1;
        if (g_all >= 2 && !mbar_wait(&dempty[b], ((g_all >> 1) - 1) & 1, lim)) { *abort_flag = 1; return false; }
        fence_after();
        const uint32_t th = thh + b * BN;
        const int kb_end = min(kblocks, (g + 1) * DRAIN);
        for (int kb = g * DRAIN; kb < kb_end; ++kb) {
            const int st = kb_all % STAGES;
            if (!mbar_wait(&full[st], (kb_all / STAGES) & 1, lim)) { *abort_flag = 1; return false; }
            fence_after();
            unsigned char *sb = smem + st * STAGE_BYTES;
            const uint64_t ah = sw128_desc(sb), al = sw128_desc(sb + TILE_A);
            const uint64_t bh = sw128_desc(sb + 2 * TILE_A), bl = sw128_desc(sb + 2 * TILE_A + TILE_B);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
                const uint64_t adv = (uint64_t) (kk * 32) >> 4;
                umma_f16(th, ah + adv, bh + adv, idesc, (kb > g * DRAIN || kk > 0));
                umma_f16(tx, ah + adv, bl + adv, idesc, (kb | kk) != 0);
                umma_f16(tx, al + adv, bh + adv, idesc, 1);
            }
            umma_commit(&empty[st]);
            ++kb_all;
        }
        umma_commit(&dfull[b]);
        ++g_all;
    }
    umma_commit(done);
    return true;
}

// Epilogue side of the drains of one tile: adds every drained hi*hi partial
// of this warp's 32 lanes x 64 columns into sum, in plain fp32 or
// Kahan-compensated with the compensation kept in TMEM columns [384, 512)
// (registers are the limit: ten warps leave 168 per thread).  g_all runs on
// across tiles like the issuer's.  Returns false (warp-uniform) if a wait
// timed out or the CTA aborted.
template <bool KAHAN>
__device__ __forceinline__ bool drain_tile(uint32_t tmem, uint32_t lane_addr, int col0, uint64_t *dfull,
                                           uint64_t *dempty, int kblocks, int DRAIN, float (&sum)[64], int &g_all,
                                           int *abort_flag, uint64_t lim) {
    const int ngroups = (kblocks + DRAIN - 1) / DRAIN;
    bool alive = true;
    for (int g = 0; g < ngroups; ++g) {
        const int b = g_all & 1;
        alive = __all_sync(0xffffffffu, alive && mbar_wait(&dfull[b], (g_all >> 1) & 1, lim)) && !*abort_flag;
        if (!alive) break;
        fence_after();
        if (!KAHAN) {
            float v[64];
            tmem_ld64(tmem + lane_addr + b * 128 + col0, v);
#pragma unroll
            for (int j = 0; j < 64; ++j) sum[j] += v[j];
        }
#pragma unroll
        for (int h = 0; h < 2 && KAHAN; ++h) {
            float v[32];
            tmem_ld32(tmem + lane_addr + b * 128 + col0 + h * 32, v);
            {
                const uint32_t ca = tmem + lane_addr + 384 + col0 + h * 32;
                float cp[32];
                if (g == 0) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) cp[j] = 0.f;
                } else {
                    tmem_ld32(ca, cp);
                }
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    const float yv = v[j] - cp[j];
                    const float t = sum[h * 32 + j] + yv;
                    cp[j] = (t - sum[h * 32 + j]) - yv;
                    sum[h * 32 + j] = t;
                }
                tmem_st32(ca, cp);
            }
        }
        fence_before();
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive(&dempty[b]);
        ++g_all;
    }
    return alive;
}

// ---------------------------------------------------------------------------
// Persistent GEMM: one CTA per SM walks the tiles t = blockIdx.x + i gridDim.x
// of the wave (tile t: job t / tiles_per_job, i.e. (chunk, slot), and one
// 128 x 128 output tile of A_s).  The TMA ring, the hi*hi drain groups and
// their barrier parities run on across tiles; the cross-term accumulator
// alternates between two TMEM buffers, so that the epilogue of tile t
// (conversion and stores) overlaps the MMAs of tile t + 1.
// TMEM: hi*hi ping [0, 128), pong [128, 256), cross [256, 384) and [384, 512).
//
// STAGE selects the product (all three share the pipeline):
//   0  A_s = C^-1 Q_s: every 128 x 128 tile, written row-major to R and
//      transposed to P;
//   1  X_s = W Q_s (whitened path, W in the C planes): written row-major to R;
//   2  B_s = X_s W^T (X_s from R, W as the second operand): tiles on and above
//      the diagonal only, weighted for the trace Gram (off-diagonal elements
//      times sqrt 2, the lower half of a diagonal tile zero) and stored as
//      compact 128 x 128 tiles in P.
// Stages 1 and 2 stop the K loop where W's lower triangle ends (a.w_tri).
struct GemmTile {
    int c, s, m0, n0, tu;   // tu: compact index of an upper tile (stage 2)
};

template <int STAGE>
__device__ __forceinline__ GemmTile gemm_tile(const int *jobs, long long t, int mt) {
    const long long tpj = STAGE == 2 ? (long long) mt * (mt + 1) / 2 : (long long) mt * mt;
    const int job = (int) (t / tpj), tix = (int) (t % tpj);
    if (STAGE != 2) return GemmTile{jobs[2 * job], jobs[2 * job + 1], (tix % mt) * G_BM, (tix / mt) * G_BN, 0};
    // upper tiles row by row: row I holds tiles J = I .. mt - 1
    int I = 0, r = tix;
    while (r >= mt - I) { r -= mt - I; ++I; }
    return GemmTile{jobs[2 * job], jobs[2 * job + 1], I * G_BM, (I + r) * G_BN, tix};
}

// K blocks of a tile: the whole row, or up to the end of W's lower triangle
template <int STAGE>
__device__ __forceinline__ int tile_kblocks(const WaveArgs &a, const GemmTile &tl, int kblocks) {
    if (STAGE == 0 || !a.w_tri) return kblocks;
    const int end = ((STAGE == 1 ? tl.m0 : tl.n0) + G_BM) / BK;
    return min(kblocks, end);
}

// hi*hi drain interval of a tile: the whitened signal and noise slots (B_ns =
// W S W^T, B_{ns+1} = W N W^T, two of ns + 2 slots, which enter every t_k and
// b_k) drain every 2 K blocks: their accumulation, not the operands, sets the
// error of t and b (2 blocks for every slot cut b, t from 6e-6, 9e-6 to 1e-6,
// 2e-6 on DESI-like chunks, at 28 % more product time)
template <int STAGE>
__device__ __forceinline__ int tile_drain(const WaveArgs &a, const GemmTile &tl) {
    return (STAGE != 0 && tl.s >= a.chunks[tl.c].ns) ? kGemmDrainST : (a.gemm_drain > 0 ? a.gemm_drain : kGemmDrain);
}

// Row-major stores of a warp's 32 rows x 32 fp16 columns of one plane (w:
// this lane's row, 16 words), coalesced through the warp's 2 KB shared-memory
// stage: each lane writes its row's four 16-byte chunks (chunk c at position
// c ^ ((row >> 1) & 3): no bank conflicts), then stores row 8q + lane / 4,
// chunk lane % 4 for q = 0..3, four lanes covering one row's 64 contiguous
// bytes (a lane per row would make every 16-byte store its own request).
__device__ __forceinline__ void store_rows(uint4 *stg, const uint32_t (&w)[16], __half *row0, size_t pitch,
                                           int lane) {
    __syncwarp();   // the previous plane's reads of the stage are done
#pragma unroll
    for (int c = 0; c < 4; ++c)
        stg[lane * 4 + (c ^ ((lane >> 1) & 3))] = make_uint4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        const int r = 8 * q + lane / 4, c = lane % 4;
        *reinterpret_cast<uint4 *>(row0 + (size_t) r * pitch + 8 * c) = stg[r * 4 + (c ^ ((r >> 1) & 3))];
    }
}

// Epilogue of one products tile (epilogue warp quad, columns col0 .. col0 + 63):
// the drained hi*hi sums plus the cross terms at tcross, scaled to fp16 hi/lo
// planes.  Stage 0: A_s row-major to R and transposed to P; stage 1: X_s to R;
// stage 2: B_s weighted into its compact upper tile of P.  A tile with live =
// false (the padding half of a CTA pair) reads TMEM but writes nothing.
// release() runs once the warp's last read of the cross buffer has completed,
// before its second half of the global stores: the MMAs of the tile after next
// may take the buffer while the stores drain (the stores hold the epilogue
// longer than the MMAs of a tile take).
template <int STAGE, class Release>
__device__ __forceinline__ void store_tile(const WaveArgs &a, const GemmTile &tl, bool live, uint32_t tcross,
                                           uint32_t lane_addr, int quad, int lane, int col0, const float (&sum)[64],
                                           uint4 *stg, Release &&release) {
    const int ld = a.max_ld;
    const size_t plane = (size_t) ld * ld;
    const int nq4 = 4 * a.n_chunks;
    const ChunkDesc &ch = a.chunks[tl.c];
    if (STAGE == 2) {
        // B_s = (R scale X_s)(C scale W)^T: to the P scale, weighted, compact upper tile
        const int s = tl.s;
        const double rs = a.scales[nq4 + a.total_slots_q + a.total_slots_p + ch.slot_r + s];
        const double bs = a.scales[nq4 + a.total_slots_q + ch.slot_p + s];
        const float mult = (float) (bs / (rs * a.scales[4 * tl.c + 2]));
        const int rt = quad * 32 + lane;   // row within the tile
        // this warp's first row of the compact tile
        const size_t tbase = (size_t) (ch.slot_p + s) * a.p_plane + (size_t) tl.tu * (G_BM * G_BN) +
                             (size_t) (quad * 32) * G_BN;
        const bool ok = live && LQG_IN_BOUNDS(a, ch.slot_p + s < a.total_slots_p &&
                                             (size_t) tl.tu * (G_BM * G_BN) + G_BM * G_BN <= a.p_plane,
                                      2, tl.c, s);
        const float sqrt2 = 1.41421356237309515f;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int cb = col0 + h * 32;   // column within the tile
            float xv[32];
            tmem_ld32(tcross + lane_addr + cb, xv);
            if (h == 1) release();
            if (!ok) continue;
            uint32_t hp[16], lp[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                float v[2];
#pragma unroll
                for (int e2 = 0; e2 < 2; ++e2) {
                    const int cc = cb + 2 * j + e2;
                    float wgt = sqrt2;
                    if (tl.m0 == tl.n0) wgt = cc > rt ? sqrt2 : (cc == rt ? 1.f : 0.f);
                    v[e2] = (sum[h * 32 + 2 * j + e2] + xv[2 * j + e2]) * mult * wgt;
                }
                const __half2 hv = __floats2half2_rn(v[0], v[1]);
                const float2 hf = __half22float2(hv);
                const __half2 lv = __floats2half2_rn(v[0] - hf.x, v[1] - hf.y);
                hp[j] = *reinterpret_cast<const uint32_t *>(&hv);
                lp[j] = *reinterpret_cast<const uint32_t *>(&lv);
            }
            store_rows(stg, hp, a.p_hi + tbase + cb, G_BN, lane);
            store_rows(stg, lp, a.p_lo + tbase + cb, G_BN, lane);
        }
        return;
    }
    const int row = tl.m0 + quad * 32 + lane;
    const int s = tl.s;
    const double sc = a.scales[4 * tl.c + 2];
    const double qs = a.scales[nq4 + ch.slot_q + s];
    // R scale (equal to the P scale of the same slot for s < ns)
    const double ps = a.scales[nq4 + a.total_slots_q + a.total_slots_p + ch.slot_r + s];
    const float mult = (float) (ps / (sc * qs));
    __half *Rh = a.r_hi + (size_t) (ch.slot_r + s) * plane, *Rl = a.r_lo + (size_t) (ch.slot_r + s) * plane;
    __half *Ph = a.p_hi + (size_t) (ch.slot_p + s) * plane, *Pl = a.p_lo + (size_t) (ch.slot_p + s) * plane;
    // A_s (s < ns) goes to R and, transposed, to P; C^-1 S (s = ns) to R only
    // (stage 1: every X_s to R only)
    const bool write_p = STAGE == 0 && s < ch.ns;
    const bool slots_ok = live && LQG_IN_BOUNDS(a, ch.slot_r + s < a.total_slots_r &&
                                             (!write_p || ch.slot_p + s < a.total_slots_p), 2, tl.c, s);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int cb = tl.n0 + col0 + h * 32;
        float xv[32];
        tmem_ld32(tcross + lane_addr + col0 + h * 32, xv);
        if (h == 1) release();
        // warp-uniform: ld is a multiple of 64, so a warp's 32 rows are all
        // inside the matrix or all padding
        if (!slots_ok || cb >= ld || tl.m0 + quad * 32 >= ld) continue;
        // hi/lo pairs packed in registers (two halves per 32-bit word)
        uint32_t hp[16], lp[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float v0 = (sum[h * 32 + 2 * j] + xv[2 * j]) * mult;
            const float v1 = (sum[h * 32 + 2 * j + 1] + xv[2 * j + 1]) * mult;
            const __half2 hv = __floats2half2_rn(v0, v1);
            const float2 hf = __half22float2(hv);
            const __half2 lv = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
            hp[j] = *reinterpret_cast<const uint32_t *>(&hv);
            lp[j] = *reinterpret_cast<const uint32_t *>(&lv);
        }
        store_rows(stg, hp, Rh + (size_t) (row - lane) * ld + cb, ld, lane);
        store_rows(stg, lp, Rl + (size_t) (row - lane) * ld + cb, ld, lane);
        if (!write_p) continue;
        unsigned short *ph = reinterpret_cast<unsigned short *>(Ph) + row;
        unsigned short *pl = reinterpret_cast<unsigned short *>(Pl) + row;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            ph[(size_t) (cb + 2 * j) * ld] = (unsigned short) (hp[j] & 0xffffu);
            ph[(size_t) (cb + 2 * j + 1) * ld] = (unsigned short) (hp[j] >> 16);
            pl[(size_t) (cb + 2 * j) * ld] = (unsigned short) (lp[j] & 0xffffu);
            pl[(size_t) (cb + 2 * j + 1) * ld] = (unsigned short) (lp[j] >> 16);
        }
    }
}

template <int STAGE>
__global__ void __launch_bounds__(TC_THREADS, 1)
k_tc_gemm(WaveArgs a, const int *jobs, int njobs, const __grid_constant__ CUtensorMap mc_hi,
          const __grid_constant__ CUtensorMap mc_lo, const __grid_constant__ CUtensorMap mq_hi,
          const __grid_constant__ CUtensorMap mq_lo) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t) 1023);
    uint4 *stg_all = reinterpret_cast<uint4 *>(smem + G_STAGES * G_STAGE_BYTES);   // epilogue store stages
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + G_STAGES * G_STAGE_BYTES + kStoreStages);
    uint64_t *empty = full + G_STAGES;
    uint64_t *dfull = empty + G_STAGES;
    uint64_t *dempty = dfull + 2;
    uint64_t *xfull = dempty + 2;
    uint64_t *xempty = xfull + 2;
    uint64_t *mdone = xempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

    const int ld = a.max_ld;
    const int mt = (ld + G_BM - 1) / G_BM;
    const long long total = (long long) njobs * (STAGE == 2 ? mt * (mt + 1) / 2 : mt * mt);
    const int kblocks = ld / BK;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t lim = a.wait_ns ? a.wait_ns : kWaitLimitNs;

    if (threadIdx.x == 0) {
        for (int i = 0; i < G_STAGES; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], 1); }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&dfull[i], 1);
            mbar_init(&dempty[i], 8);
            mbar_init(&xfull[i], 1);
            mbar_init(&xempty[i], 8);
        }
        mbar_init(mdone, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(tmem_slot, 512);
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        // TMA producer
        int kb_all = 0;
        for (long long t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x) {
            const GemmTile tl = gemm_tile<STAGE>(jobs, t, mt);
            // stages 0, 1: A = C planes of the chunk, B = Q slot; stage 2: A = R slot, B = C planes
            const int aidx = STAGE == 2 ? a.chunks[tl.c].slot_r + tl.s : tl.c;
            const int bidx = STAGE == 2 ? tl.c : a.chunks[tl.c].slot_q + tl.s;
            const bool idx_ok = STAGE == 2 ? (aidx >= 0 && aidx < a.total_slots_r)
                                           : (bidx >= 0 && bidx < a.total_slots_q);
            if (!LQG_IN_BOUNDS(a, tl.c >= 0 && tl.c < a.n_chunks && idx_ok && tl.m0 < ld && tl.n0 < ld &&
                                      a.chunks[tl.c].ld == ld,
                               1, tl.c, STAGE == 2 ? aidx : bidx)) {
                *abort_flag = 1;
                break;
            }
            const int kbt = tile_kblocks<STAGE>(a, tl, kblocks);
            for (int kb = 0; kb < kbt; ++kb) {
                const int st = kb_all % G_STAGES;
                if (!mbar_wait(&empty[st], ((kb_all / G_STAGES) & 1) ^ 1, lim)) { *abort_flag = 1; break; }
                unsigned char *sb = smem + st * G_STAGE_BYTES;
                mbar_expect_tx(&full[st], G_STAGE_BYTES);
                tma_load_3d(sb, &mc_hi, &full[st], kb * BK, tl.m0, aidx);
                tma_load_3d(sb + G_TILE_A, &mc_lo, &full[st], kb * BK, tl.m0, aidx);
                tma_load_3d(sb + 2 * G_TILE_A, &mq_hi, &full[st], kb * BK, tl.n0, bidx);
                tma_load_3d(sb + 2 * G_TILE_A + G_TILE_B, &mq_lo, &full[st], kb * BK, tl.n0, bidx);
                ++kb_all;
            }
        }
        // every issued stage must land before the CTA may leave
        for (int k = (kb_all > G_STAGES ? kb_all - G_STAGES : 0); k < kb_all; ++k)
            mbar_wait(&full[k % G_STAGES], (k / G_STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        int kb_all = 0, g_all = 0, lt = 0;
        for (long long t = blockIdx.x; t < total && !*abort_flag; t += gridDim.x, ++lt) {
            const int x = lt & 1;
            if (lt >= 2 && !mbar_wait(&xempty[x], ((lt >> 1) - 1) & 1, lim)) { *abort_flag = 1; break; }
            fence_after();
            const GemmTile tl = gemm_tile<STAGE>(jobs, t, mt);
            const int kbt = tile_kblocks<STAGE>(a, tl, kblocks);
            if (!mma_tile<G_STAGES, G_STAGE_BYTES, G_TILE_A, G_TILE_B, G_BN>(
                    tmem, tmem + 2 * G_BN + x * G_BN, smem, full, empty, dfull, dempty, &xfull[x], kbt,
                    tile_drain<STAGE>(a, tl), idesc_f16(G_BM, G_BN), kb_all, g_all, abort_flag, lim))
                break;
        }
        // every MMA of this CTA completes before its tensor memory is freed
        umma_commit(mdone);
        mbar_wait(mdone, 0);
    } else if (warp >= 2) {
        // epilogue: drained sums + cross terms -> scaled fp16 hi/lo planes,
        // row-major (R) and transposed (P)
        const int quad = warp % 4, col0 = 64 * ((warp - 2) / 4);
        const uint32_t lane_addr = (uint32_t) (quad * 32) << 16;
        int g_all = 0, lt = 0;
        for (long long t = blockIdx.x; t < total; t += gridDim.x, ++lt) {
            const GemmTile tl = gemm_tile<STAGE>(jobs, t, mt);
            float sum[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) sum[j] = 0.f;
            bool got = drain_tile<false>(tmem, lane_addr, col0, dfull, dempty, tile_kblocks<STAGE>(a, tl, kblocks),
                                         tile_drain<STAGE>(a, tl), sum, g_all, abort_flag, lim);
            const int x = lt & 1;
            got = __all_sync(0xffffffffu, got && mbar_wait(&xfull[x], (lt >> 1) & 1, lim)) && !*abort_flag;
            if (!got) break;
            fence_after();
            // the cross buffer may be taken by tile lt + 2 once read
            store_tile<STAGE>(a, tl, true, tmem + 2 * G_BN + x * G_BN, lane_addr, quad, lane, col0, sum,
                              stg_all + (warp - 2) * (kStoreStage / 16), [&] {
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&xempty[x]);
            });
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (threadIdx.x == 0 && *abort_flag)
        for (long long t = blockIdx.x; t < total; t += gridDim.x)
            atomicExch(&a.status[a.chunks[gemm_tile<STAGE>(jobs, t, mt).c].gidx], LQG_CHUNK_TIMEOUT);
}

// ---------------------------------------------------------------------------
// The same three products on CTA pairs (a cluster of two CTAs on one TPC,
// tcgen05 cta_group::2): one MMA of M = 256, N = 128, K = 16 per instruction,
// each CTA holding 128 rows of A and 64 of the 128 rows of B.  Per SM and MMA
// the shared memory then serves 6 KB of operands instead of 8 KB, and the TMA
// writes 48 KB instead of 64 KB per K block: the single-CTA kernel is bound
// by that bandwidth (operand reads plus TMA writes) at ~60 % tensor-pipe
// activity, the pair kernel at ~80 %.
//
// Pairing: stages 0 and 1 take row blocks 2P and 2P + 1 of the same output
// column block (an odd row-block count leaves the last pair's second half as
// padding: rows past ld read as zeros and are not written); stage 2 takes
// slots s0 and s0 + 1 (jobs list even s0 only) of the same upper tile, the
// second half padding when s0 + 1 > ns + 1.  Each CTA's tensor memory holds
// its own 128 rows in the single-CTA kernel's layout, so the drains and the
// epilogue are the same code.
//
// Roles: warp 0 of each CTA loads its own operands, both CTAs' copies
// completing on the even CTA's full barrier (which expects both halves);
// warp 1 of the even CTA issues every MMA of the pair and commits to both
// CTAs' barriers (empty stages, drains, cross buffers); the epilogue warps of
// both arrive on the even CTA's dempty/xempty (16 arrivals).  Before leaving,
// the even CTA waits for its last stages to land and the odd CTA for its last
// stages to be consumed (the MMAs read them after they landed), both bounded;
// then both pass a cluster barrier after the even CTA's MMAs have completed.
constexpr int P_STAGES = 4;
constexpr int P_TILE_A = 128 * BK * 2;                       // this CTA's 128 rows of A
constexpr int P_TILE_B = 64 * BK * 2;                        // its 64 rows of B
constexpr int P_STAGE_BYTES = 2 * P_TILE_A + 2 * P_TILE_B;   // 48 KB
constexpr int P_SMEM = P_STAGES * P_STAGE_BYTES + kStoreStages + 1024 + 256;

struct PairTile {
    GemmTile tl;   // this CTA's tile
    bool live;     // false: the padding half of the pair
    int kbt;       // K blocks of the pair
    int drain;     // hi*hi drain interval of the pair
};

template <int STAGE>
__device__ __forceinline__ PairTile pair_tile(const WaveArgs &a, const int *jobs, long long t, int mt, int kblocks,
                                              int rank) {
    PairTile p;
    const int defdrain = a.gemm_drain > 0 ? a.gemm_drain : kGemmDrain;
    if (STAGE != 2) {
        const int mh = (mt + 1) / 2;
        const long long tpj = (long long) mh * mt;
        const int job = (int) (t / tpj), tix = (int) (t % tpj);
        const int P = tix % mh, J = tix / mh;
        p.tl = GemmTile{jobs[2 * job], jobs[2 * job + 1], (2 * P + rank) * G_BM, J * G_BN, 0};
        p.live = p.tl.m0 < a.max_ld;
        // stage 1 with a triangular W: the K range of the pair's lower row block
        p.kbt = (STAGE == 1 && a.w_tri) ? min(kblocks, ((2 * P + 1) * G_BM + G_BM) / BK) : kblocks;
        p.drain = (STAGE == 1 && p.tl.s >= a.chunks[p.tl.c].ns) ? kGemmDrainST : defdrain;
        return p;
    }
    const long long tpj = (long long) mt * (mt + 1) / 2;
    const int job = (int) (t / tpj), tix = (int) (t % tpj);
    int I = 0, r = tix;
    while (r >= mt - I) { r -= mt - I; ++I; }
    const int c = jobs[2 * job], s0 = jobs[2 * job + 1];
    const int ns = a.chunks[c].ns;
    const int s = s0 + rank;
    p.live = s <= ns + 1;
    p.tl = GemmTile{c, p.live ? s : s0, I * G_BM, (I + r) * G_BN, tix};
    p.kbt = a.w_tri ? min(kblocks, (p.tl.n0 + G_BM) / BK) : kblocks;
    // the S and N slots drain more often; a pair holding one drains at its interval
    p.drain = s0 + 1 >= ns ? kGemmDrainST : defdrain;
    return p;
}

// Epilogue drains of one tile, as drain_tile<false>, arriving on the even CTA's dempty.
__device__ __forceinline__ bool drain_tile_pair(uint32_t tmem, uint32_t lane_addr, int col0, uint64_t *dfull,
                                                uint32_t dempty_cl, int kblocks, int DRAIN, float (&sum)[64],
                                                int &g_all, const volatile int *abort_flag, uint64_t lim) {
    const int ngroups = (kblocks + DRAIN - 1) / DRAIN;
    bool alive = true;
    for (int g = 0; g < ngroups; ++g) {
        const int b = g_all & 1;
        alive = __all_sync(0xffffffffu, alive && mbar_wait(&dfull[b], (g_all >> 1) & 1, lim)) && !*abort_flag;
        if (!alive) break;
        fence_after();
        float v[64];
        tmem_ld64(tmem + lane_addr + b * 128 + col0, v);
#pragma unroll
        for (int j = 0; j < 64; ++j) sum[j] += v[j];
        fence_before();
        __syncwarp();
        if ((threadIdx.x & 31) == 0) mbar_arrive_cluster(dempty_cl + 8 * b);
        ++g_all;
    }
    return alive;
}

template <int STAGE>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(TC_THREADS, 1)
k_tc_gemm_pair(WaveArgs a, const int *jobs, int njobs, const __grid_constant__ CUtensorMap ma_hi,
               const __grid_constant__ CUtensorMap ma_lo, const __grid_constant__ CUtensorMap mb_hi,
               const __grid_constant__ CUtensorMap mb_lo) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // the same offset in both CTAs: the MMAs address both with one descriptor
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t) 1023);
    uint4 *stg_all = reinterpret_cast<uint4 *>(smem + P_STAGES * P_STAGE_BYTES);   // epilogue store stages
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + P_STAGES * P_STAGE_BYTES + kStoreStages);   // even CTA: both halves
    uint64_t *empty = full + P_STAGES;
    uint64_t *dfull = empty + P_STAGES;
    uint64_t *dempty = dfull + 2;
    uint64_t *xfull = dempty + 2;
    uint64_t *xempty = xfull + 2;
    uint64_t *mdone = xempty + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int rank = (int) cluster_rank();
    const int cid = blockIdx.x >> 1, ncl = gridDim.x >> 1;
    const int ld = a.max_ld;
    const int mt = (ld + G_BM - 1) / G_BM, mh = (mt + 1) / 2;
    const long long total = (long long) njobs * (STAGE == 2 ? (long long) mt * (mt + 1) / 2 : (long long) mh * mt);
    const int kblocks = ld / BK;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t lim = a.wait_ns ? a.wait_ns : kWaitLimitNs;

    if (threadIdx.x == 0) {
        for (int i = 0; i < P_STAGES; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&dfull[i], 1);
            mbar_init(&dempty[i], 16);
            mbar_init(&xfull[i], 1);
            mbar_init(&xempty[i], 16);
        }
        mbar_init(mdone, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc_pair(tmem_slot, 512);
    fence_before();
    __syncthreads();
    cluster_sync();   // both CTAs' barriers exist before either arrives on the other's
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t full_cl = cluster_addr(full, 0), dempty_cl = cluster_addr(dempty, 0),
                   xempty_cl = cluster_addr(xempty, 0);
    const uint32_t peer_abort = cluster_addr((const void *) abort_flag, rank ^ 1);
    auto set_abort = [&]() {
        *abort_flag = 1;
        st_cluster_u32(peer_abort, 1);
    };

    if (warp == 0 && lane == 0) {
        // TMA producer of this CTA's operands
        int kb_all = 0;
        for (long long t = cid; t < total && !*abort_flag; t += ncl) {
            const PairTile p = pair_tile<STAGE>(a, jobs, t, mt, kblocks, rank);
            const GemmTile &tl = p.tl;
            const int aidx = STAGE == 2 ? a.chunks[tl.c].slot_r + tl.s : tl.c;
            const int bidx = STAGE == 2 ? tl.c : a.chunks[tl.c].slot_q + tl.s;
            const bool idx_ok = STAGE == 2 ? (aidx >= 0 && aidx < a.total_slots_r)
                                           : (bidx >= 0 && bidx < a.total_slots_q);
            if (!LQG_IN_BOUNDS(a, tl.c >= 0 && tl.c < a.n_chunks && idx_ok && tl.n0 < ld &&
                                      a.chunks[tl.c].ld == ld,
                               1, tl.c, STAGE == 2 ? aidx : bidx)) {
                set_abort();
                break;
            }
            for (int kb = 0; kb < p.kbt; ++kb) {
                const int st = kb_all % P_STAGES;
                if (!mbar_wait(&empty[st], ((kb_all / P_STAGES) & 1) ^ 1, lim)) { set_abort(); break; }
                unsigned char *sb = smem + st * P_STAGE_BYTES;
                // the even CTA's barrier expects both CTAs' bytes of the stage
                if (rank == 0) mbar_expect_tx(&full[st], 2 * P_STAGE_BYTES);
                const uint32_t bar = full_cl + 8 * st;
                tma_load_3d_pair(sb, &ma_hi, bar, kb * BK, tl.m0, aidx);
                tma_load_3d_pair(sb + P_TILE_A, &ma_lo, bar, kb * BK, tl.m0, aidx);
                tma_load_3d_pair(sb + 2 * P_TILE_A, &mb_hi, bar, kb * BK, tl.n0 + 64 * rank, bidx);
                tma_load_3d_pair(sb + 2 * P_TILE_A + P_TILE_B, &mb_lo, bar, kb * BK, tl.n0 + 64 * rank, bidx);
                ++kb_all;
            }
        }
        // this CTA's copies land before it leaves: the even CTA waits for its
        // last stages to complete, the odd CTA for them to be consumed.  After
        // an abort these phases may never complete (a stage the other CTA did
        // not load, MMAs not issued); the copies themselves land within
        // microseconds, so the wait is cut to 10 ms then.
        for (int k = (kb_all > P_STAGES ? kb_all - P_STAGES : 0); k < kb_all; ++k) {
            const uint64_t tail = *abort_flag ? 10000000ull : kWaitLimitNs;
            if (rank == 0) mbar_wait(&full[k % P_STAGES], (k / P_STAGES) & 1, tail);
            else mbar_wait(&empty[k % P_STAGES], (k / P_STAGES) & 1, tail);
        }
    } else if (warp == 1 && lane == 0 && rank == 0) {
        // MMA issuer of the pair
        const uint32_t idesc = idesc_f16(2 * G_BM, G_BN);
        int kb_all = 0, g_all = 0, lt = 0;
        bool ok = true;
        for (long long t = cid; t < total && ok && !*abort_flag; t += ncl, ++lt) {
            const int x = lt & 1;
            if (lt >= 2 && !mbar_wait_cl(&xempty[x], ((lt >> 1) - 1) & 1, lim)) { ok = false; break; }
            fence_after();
            const PairTile p = pair_tile<STAGE>(a, jobs, t, mt, kblocks, rank);
            const uint32_t tx = tmem + 2 * G_BN + x * G_BN;
            const int ngroups = (p.kbt + p.drain - 1) / p.drain;
            for (int g = 0; g < ngroups && ok; ++g) {
                const int b = g_all & 1;
                if (g_all >= 2 && !mbar_wait_cl(&dempty[b], ((g_all >> 1) - 1) & 1, lim)) { ok = false; break; }
                fence_after();
                const uint32_t th = tmem + b * G_BN;
                const int kb_end = min(p.kbt, (g + 1) * p.drain);
                for (int kb = g * p.drain; kb < kb_end; ++kb) {
                    const int st = kb_all % P_STAGES;
                    const uint32_t par = (kb_all / P_STAGES) & 1;
                    if (!mbar_wait(&full[st], par, lim)) { ok = false; break; }
                    fence_after();
                    unsigned char *sb = smem + st * P_STAGE_BYTES;
                    const uint64_t ah = sw128_desc(sb), al = sw128_desc(sb + P_TILE_A);
                    const uint64_t bh = sw128_desc(sb + 2 * P_TILE_A), bl = sw128_desc(sb + 2 * P_TILE_A + P_TILE_B);
#pragma unroll
                    for (int kk = 0; kk < BK / 16; ++kk) {
                        const uint64_t adv = (uint64_t) (kk * 32) >> 4;
                        umma_f16_pair(th, ah + adv, bh + adv, idesc, (kb > g * p.drain || kk > 0));
                        umma_f16_pair(tx, ah + adv, bl + adv, idesc, (kb | kk) != 0);
                        umma_f16_pair(tx, al + adv, bh + adv, idesc, 1);
                    }
                    umma_commit_pair(&empty[st]);
                    ++kb_all;
                }
                if (!ok) break;
                umma_commit_pair(&dfull[b]);
                ++g_all;
            }
            if (!ok) break;
            umma_commit_pair(&xfull[x]);
        }
        if (!ok) set_abort();
        // every MMA of the pair completes before either CTA frees its tensor memory
        umma_commit_pair(mdone);
        mbar_wait_cl(mdone, 0);
    } else if (warp >= 2) {
        // epilogue of this CTA's 128 rows
        const int quad = warp % 4, col0 = 64 * ((warp - 2) / 4);
        const uint32_t lane_addr = (uint32_t) (quad * 32) << 16;
        int g_all = 0, lt = 0;
        for (long long t = cid; t < total; t += ncl, ++lt) {
            const PairTile p = pair_tile<STAGE>(a, jobs, t, mt, kblocks, rank);
            float sum[64];
#pragma unroll
            for (int j = 0; j < 64; ++j) sum[j] = 0.f;
            bool got = drain_tile_pair(tmem, lane_addr, col0, dfull, dempty_cl, p.kbt, p.drain, sum, g_all,
                                       abort_flag, lim);
            const int x = lt & 1;
            got = __all_sync(0xffffffffu, got && mbar_wait(&xfull[x], (lt >> 1) & 1, lim)) && !*abort_flag;
            if (!got) break;
            fence_after();
            store_tile<STAGE>(a, p.tl, p.live, tmem + 2 * G_BN + x * G_BN, lane_addr, quad, lane, col0, sum,
                              stg_all + (warp - 2) * (kStoreStage / 16), [&] {
                fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive_cluster(xempty_cl + 8 * x);
            });
        }
    }
    fence_before();
    __syncthreads();
    cluster_sync();   // the pair's MMAs are complete (even CTA) and neither CTA has copies in flight
    if (warp == 1) {
        fence_after();
        tmem_dealloc_pair(tmem, 512);
    }
    if (threadIdx.x == 0 && *abort_flag)
        for (long long t = cid; t < total; t += ncl)
            atomicExch(&a.status[a.chunks[pair_tile<STAGE>(a, jobs, t, mt, kblocks, rank).tl.c].gidx],
                       LQG_CHUNK_TIMEOUT);
}

// ---------------------------------------------------------------------------
// Gram block (bi, bj) of one chunk over one K split.
__global__ void __launch_bounds__(TC_THREADS, 1)
k_tc_gram(WaveArgs a, const __grid_constant__ CUtensorMap mp_hi, const __grid_constant__ CUtensorMap mp_lo,
          const __grid_constant__ CUtensorMap mr_hi, const __grid_constant__ CUtensorMap mr_lo) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *smem = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t) 1023);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + R_STAGES * R_STAGE_BYTES);
    uint64_t *empty = full + R_STAGES;
    uint64_t *dfull = empty + R_STAGES;      // [2] hi*hi buffer ready to drain
    uint64_t *dempty = dfull + 2;            // [2] hi*hi buffer drained
    uint64_t *accum = dempty + 2;
    uint64_t *mdone = accum + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(mdone + 1);
    int *abort_flag = reinterpret_cast<int *>(tmem_slot + 1);

    const int c = blockIdx.y, sp = blockIdx.x, blk = blockIdx.z;
    const ChunkDesc &ch = a.chunks[c];
    if (a.status[ch.gidx] != LQG_CHUNK_OK || sp >= a.gram_splits) return;
    // P rows: the ns A_s^T; R rows: ns A_s, C^-1 S, C^-1 N.  F is symmetric, so
    // only blocks bi <= bj are formed (they hold every F_ij with i <= j and the
    // t, b columns ns and ns + 1).
    const int bi = blk / a.gt, bj = blk % a.gt;
    if (bi > bj || bi * R_BM >= ch.ns || bj * R_BN >= ch.ns + 2) return;
    const int64_t K = a.sym ? a.p_plane : (int64_t) ch.ld * ch.ld;
    const int64_t kper = ((K + a.gram_splits - 1) / a.gram_splits + BK - 1) / BK * BK;
    const int64_t k_lo = sp * kper, k_hi = min(K, k_lo + kper);
    const int kblocks = k_hi > k_lo ? (int) ((k_hi - k_lo) / BK) : 0;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const uint64_t lim = a.wait_ns ? a.wait_ns : kWaitLimitNs;
    // whitened form: both operands are the B_s rows of P (B_0 .. B_{ns+1})
    const int prow = ch.slot_p + bi * R_BM, rrow = (a.sym ? ch.slot_p : ch.slot_r) + bj * R_BN;
    // Rows of this block that belong to the chunk (P: ns, or ns + 2 in the
    // whitened form; R: ns + 2), loaded as 32-row boxes: the rows past them
    // are the next chunk's and are not fetched (16-row boxes fetch less but
    // cost more TMA issue than they save).  The shared-memory rows left
    // unloaded hold stale data that only reaches G's rows >= ns and columns
    // >= ns + 2, which nothing reads.
    const int prows = min(R_BM, (a.sym ? ch.ns + 2 : ch.ns) - bi * R_BM), rrows = min(R_BN, ch.ns + 2 - bj * R_BN);
    const int pboxes = (prows + kGramBox - 1) / kGramBox, rboxes = (rrows + kGramBox - 1) / kGramBox;

    if (threadIdx.x == 0) {
        for (int i = 0; i < R_STAGES; ++i) { mbar_init(&full[i], 1); mbar_init(&empty[i], 1); }
        for (int i = 0; i < 2; ++i) { mbar_init(&dfull[i], 1); mbar_init(&dempty[i], 8); }
        mbar_init(accum, 1);
        mbar_init(mdone, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tmem_alloc(tmem_slot, 512);   // hi*hi ping [0,128), pong [128,256), cross [256,384)
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0 && lane == 0) {
        int issued = 0;
        if (!LQG_IN_BOUNDS(a, prow >= 0 && prow < a.total_slots_p && rrow >= 0 &&
                                  rrow < (a.sym ? a.total_slots_p : a.total_slots_r) && k_hi <= K, 3, c, prow))
            *abort_flag = 1;
        for (int kb = 0; kb < kblocks && !*abort_flag; ++kb) {
            const int st = kb % R_STAGES;
            if (!mbar_wait(&empty[st], ((kb / R_STAGES) & 1) ^ 1, lim)) { *abort_flag = 1; break; }
            unsigned char *sb = smem + st * R_STAGE_BYTES;
            const int x = (int) (k_lo + (int64_t) kb * BK);
            mbar_expect_tx(&full[st], 2 * (pboxes + rboxes) * kGramBoxBytes);
            for (int q = 0; q < pboxes; ++q) {
                tma_load_2d(sb + q * kGramBoxBytes, &mp_hi, &full[st], x, prow + q * kGramBox);
                tma_load_2d(sb + R_TILE + q * kGramBoxBytes, &mp_lo, &full[st], x, prow + q * kGramBox);
            }
            for (int q = 0; q < rboxes; ++q) {
                tma_load_2d(sb + 2 * R_TILE + q * kGramBoxBytes, &mr_hi, &full[st], x, rrow + q * kGramBox);
                tma_load_2d(sb + 3 * R_TILE + q * kGramBoxBytes, &mr_lo, &full[st], x, rrow + q * kGramBox);
            }
            ++issued;
        }
        for (int kb = (issued > R_STAGES ? issued - R_STAGES : 0); kb < issued; ++kb)
            mbar_wait(&full[kb % R_STAGES], (kb / R_STAGES) & 1);
    } else if (warp == 1 && lane == 0) {
        int kb_all = 0, g_all = 0;
        mma_tile<R_STAGES, R_STAGE_BYTES, R_TILE, R_TILE, R_BN>(tmem, tmem + 2 * R_BN, smem, full, empty, dfull,
                                                               dempty, accum, kblocks, kGramDrain,
                                                               idesc_f16(R_BM, R_BN), kb_all, g_all, abort_flag, lim);
        // every MMA completes before the tensor memory is freed
        umma_commit(mdone);
        mbar_wait(mdone, 0);
    } else if (warp >= 2) {
        // 8 epilogue warps: lane quadrant warp % 4, columns 64 * ((warp - 2) / 4) + [0, 64)
        const int quad = warp % 4, half = (warp - 2) / 4;
        const uint32_t lane_addr = (uint32_t) (quad * 32) << 16;
        float sum[64];
#pragma unroll
        for (int j = 0; j < 64; ++j) sum[j] = 0.f;
        int g_all = 0;
        const bool alive = drain_tile<true>(tmem, lane_addr, half * 64, dfull, dempty, kblocks, kGramDrain, sum,
                                            g_all, abort_flag, lim);
        const bool got = __all_sync(0xffffffffu, alive && mbar_wait(accum, 0, lim)) && !*abort_flag;
        fence_after();
        if (got) {
            const int row = quad * 32 + lane;
            const size_t obase = (((size_t) c * a.gt * a.gt + blk) * a.gram_splits + sp) * R_BM * R_BN +
                                 (size_t) row * R_BN + half * 64;
            const bool out_ok = LQG_IN_BOUNDS(a, (int64_t) (obase + 64) <= a.gram_elems, 4, c, obase);
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float x[32], cp[32];
                tmem_ld32(tmem + lane_addr + 2 * R_BN + half * 64 + h * 32, x);
                if (kblocks > 0) {
                    tmem_ld32(tmem + lane_addr + 384 + half * 64 + h * 32, cp);
                } else {
#pragma unroll
                    for (int j = 0; j < 32; ++j) { x[j] = 0.f; cp[j] = 0.f; }
                }
                if (!out_ok) continue;
                float4 *o = reinterpret_cast<float4 *>(a.gram_part + obase + h * 32);
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    float r4[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int j = h * 32 + 4 * q + e;
                        r4[e] = (sum[j] - cp[4 * q + e]) + x[4 * q + e];
                    }
                    o[q] = make_float4(r4[0], r4[1], r4[2], r4[3]);
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (threadIdx.x == 0 && *abort_flag) atomicExch(&a.status[ch.gidx], LQG_CHUNK_TIMEOUT);
}

// Operand scales of the mixed path (powers of two), from the FP64 bounds the
// factorisation left per chunk: max |C^-1| and the largest row sum of |C^-1|
// (of W in the whitened form).
__global__ void k_scales(WaveArgs a) {
    const int c = blockIdx.x;
    const ChunkDesc &ch = a.chunks[c];
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    __shared__ double red[32];
    double mx = 0;
    const double *iv = a.niv + ch.pix;
    for (int i = threadIdx.x; i < ch.n; i += blockDim.x)
        mx = fmax(mx, iv[i]);   // 1 / ivar, 0 where masked
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_down_sync(0xffffffffu, mx, o));
    if (threadIdx.x % 32 == 0) red[threadIdx.x / 32] = mx;
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int i = 1; i < (int) blockDim.x / 32; ++i) mx = fmax(mx, red[i]);
    double *sc = a.scales + 4 * c;
    const double maxc = a.fbounds[4 * ch.gidx], rowsum = a.fbounds[4 * ch.gidx + 1];
    const double target = 16384.0;
    sc[0] = maxc;
    sc[1] = rowsum;
    sc[2] = pow2_floor(target / maxc);
    sc[3] = pow2_floor(target / (maxc * mx));
    const int nq4 = 4 * a.n_chunks;
    double *qsc = a.scales + nq4 + ch.slot_q;
    double *psc = a.scales + nq4 + a.total_slots_q + ch.slot_p;
    double *rsc = a.scales + nq4 + a.total_slots_q + a.total_slots_p + ch.slot_r;
    for (int s = 0; s <= ch.ns; ++s) {
        // |C^-1 B| <= rowsum * max|B| and max|B| <= target / (B scale); the
        // same bound for X_s = W Q_s in the whitened form
        double r = pow2_floor(qsc[s] / rowsum);
        rsc[s] = r;
        if (s < ch.ns && !a.sym) psc[s] = r;
    }
    rsc[ch.ns + 1] = sc[3];   // C^-1 N, or X_N = W N
    if (a.sym)
        // |B_s| = |X_s W^T| <= max|X_s| rowsum, and sqrt 2 for the off-diagonal weight
        for (int s = 0; s <= ch.ns + 1; ++s) psc[s] = pow2_floor(rsc[s] / (2.0 * rowsum));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point, so that the
// library links without libcuda.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

CUtensorMap make_map(void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides,
                     const cuuint32_t *box, bool *ok) {
    CUtensorMap m{};
    cuuint32_t es[3] = {1, 1, 1};
    auto enc = encode_fn();
    if (!enc) { *ok = false; return m; }
    CUresult r = enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, rank, base, dims, strides, box,
                                        es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) *ok = false;
    return m;
}

}  // namespace

bool tc_available() { return true; }

void launch_scales_mixed(WaveArgs &a, cudaStream_t st) {
    k_scales<<<a.n_chunks, 256, 0, st>>>(a);
    a.launches++;
}

void launch_products_mixed(WaveArgs &a, cudaStream_t st, const int *d_jobs, int njobs, const int *d_jobs2,
                           int njobs2) {
    // shared memory above the 48 KB default, and the SM count: once per device
    static std::atomic<unsigned long long> attr{0};
    static int n_sm_dev[64], n_pair_dev[64];
    const bool ready = once_per_device(attr, [](int dev) {
        cudaError_t e = cudaFuncSetAttribute(k_tc_gemm<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tc_gemm<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tc_gemm<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, G_SMEM);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(k_tc_gram, cudaFuncAttributeMaxDynamicSharedMemorySize, R_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_gemm_pair<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_gemm_pair<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_tc_gemm_pair<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, P_SMEM);
        int sms = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess && dev >= 0 && dev < 64) n_sm_dev[dev] = sms > 0 ? sms : 1;
        // CTA pairs resident at once (the persistent pair kernels' grid): the
        // cluster placement need not reach every TPC
        int pairs = 0;
        if (e == cudaSuccess) {
            cudaLaunchConfig_t cfg{};
            cfg.gridDim = dim3(2 * std::max(sms / 2, 1));
            cfg.blockDim = dim3(TC_THREADS);
            cfg.dynamicSmemBytes = P_SMEM;
            if (cudaOccupancyMaxActiveClusters(&pairs, k_tc_gemm_pair<1>, &cfg) != cudaSuccess || pairs <= 0) {
                cudaGetLastError();
                pairs = std::max(sms / 2, 1);
            }
        }
        if (e == cudaSuccess && dev >= 0 && dev < 64) n_pair_dev[dev] = pairs;
        return e;
    });
    if (!ready) {
        a.host_failed = 1;
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    int n_sm = (dev >= 0 && dev < 64) ? n_sm_dev[dev] : 0;
    if (n_sm <= 0 && (cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n_sm <= 0))
        n_sm = 1;
    const int n_pairs = (dev >= 0 && dev < 64 && n_pair_dev[dev] > 0) ? n_pair_dev[dev] : std::max(n_sm / 2, 1);
    const int ld = a.max_ld;
    const cuuint64_t plane = (cuuint64_t) ld * ld;
    bool ok = true;
    cuuint64_t d3c[3] = {(cuuint64_t) ld, (cuuint64_t) ld, (cuuint64_t) a.n_chunks};
    cuuint64_t d3q[3] = {(cuuint64_t) ld, (cuuint64_t) ld, (cuuint64_t) a.total_slots_q};
    cuuint64_t s3[2] = {(cuuint64_t) ld * 2, plane * 2};
    cuuint32_t boxa[3] = {BK, G_BM, 1}, boxb[3] = {BK, G_BN, 1};
    CUtensorMap mch = make_map(a.c_hi, 3, d3c, s3, boxa, &ok);
    CUtensorMap mcl = make_map(a.c_lo, 3, d3c, s3, boxa, &ok);
    CUtensorMap mqh = make_map(a.q_hi, 3, d3q, s3, boxb, &ok);
    CUtensorMap mql = make_map(a.q_lo, 3, d3q, s3, boxb, &ok);
    const cuuint64_t pplane = (cuuint64_t) a.p_plane;
    cuuint64_t d2p[2] = {pplane, (cuuint64_t) a.total_slots_p};
    cuuint64_t d2r[2] = {plane, (cuuint64_t) a.total_slots_r};
    cuuint64_t s2p[1] = {pplane * 2}, s2[1] = {plane * 2};
    cuuint32_t box2[2] = {BK, kGramBox};
    CUtensorMap mph = make_map(a.p_hi, 2, d2p, s2p, box2, &ok);
    CUtensorMap mpl = make_map(a.p_lo, 2, d2p, s2p, box2, &ok);
    // whitened form: the Gram's second operand is P as well
    CUtensorMap mrh = a.sym ? mph : make_map(a.r_hi, 2, d2r, s2, box2, &ok);
    CUtensorMap mrl = a.sym ? mpl : make_map(a.r_lo, 2, d2r, s2, box2, &ok);
    // whitened form, second product: A = X_s (R planes), B = W (C planes)
    cuuint64_t d3r[3] = {(cuuint64_t) ld, (cuuint64_t) ld, (cuuint64_t) a.total_slots_r};
    CUtensorMap mxh{}, mxl{}, mwh{}, mwl{};
    if (a.sym) {
        mxh = make_map(a.r_hi, 3, d3r, s3, boxa, &ok);
        mxl = make_map(a.r_lo, 3, d3r, s3, boxa, &ok);
        mwh = make_map(a.c_hi, 3, d3c, s3, boxb, &ok);
        mwl = make_map(a.c_lo, 3, d3c, s3, boxb, &ok);
    }
    // CTA pairs: each CTA loads 64 of the 128 B rows of a tile
    CUtensorMap mqh2{}, mql2{}, mwh2{}, mwl2{};
    if (a.gemm_pair) {
        cuuint32_t boxh[3] = {BK, 64, 1};
        mqh2 = make_map(a.q_hi, 3, d3q, s3, boxh, &ok);
        mql2 = make_map(a.q_lo, 3, d3q, s3, boxh, &ok);
        if (a.sym) {
            mwh2 = make_map(a.c_hi, 3, d3c, s3, boxh, &ok);
            mwl2 = make_map(a.c_lo, 3, d3c, s3, boxh, &ok);
        }
    }
    if (!ok) {
        // nothing launched: the caller turns this into an error return
        a.host_failed = 1;
        return;
    }
    // persistent: one CTA per SM (one fits: 197 KB of shared memory)
    const long long mt = (ld + G_BM - 1) / G_BM;
    if (a.gemm_pair) {
        // one cluster of two CTAs per TPC
        const long long mh = (mt + 1) / 2, pairs_max = n_pairs;
        const long long p1 = mh * mt * njobs;
        const int grid = 2 * (int) std::min<long long>(p1, pairs_max);
        if (!a.sym) {
            k_tc_gemm_pair<0><<<grid, TC_THREADS, P_SMEM, st>>>(a, d_jobs, njobs, mch, mcl, mqh2, mql2);
        } else {
            k_tc_gemm_pair<1><<<grid, TC_THREADS, P_SMEM, st>>>(a, d_jobs, njobs, mch, mcl, mqh2, mql2);
            const long long p2 = mt * (mt + 1) / 2 * njobs2;
            const int grid2 = 2 * (int) std::min<long long>(p2, pairs_max);
            k_tc_gemm_pair<2><<<grid2, TC_THREADS, P_SMEM, st>>>(a, d_jobs2, njobs2, mxh, mxl, mwh2, mwl2);
            a.launches++;
        }
        if (a.mid_event) record_event(a.mid_event, st);
        k_tc_gram<<<dim3(a.gram_splits, a.n_chunks, a.gt * a.gt), R_THREADS, R_SMEM, st>>>(a, mph, mpl, mrh, mrl);
        a.launches += 2;
        return;
    }
    const long long tiles = mt * mt * njobs;
    const int grid = (int) std::min<long long>(tiles, n_sm);
    if (!a.sym) {
        k_tc_gemm<0><<<grid, TC_THREADS, G_SMEM, st>>>(a, d_jobs, njobs, mch, mcl, mqh, mql);
    } else {
        k_tc_gemm<1><<<grid, TC_THREADS, G_SMEM, st>>>(a, d_jobs, njobs, mch, mcl, mqh, mql);
        const long long tiles2 = mt * (mt + 1) / 2 * njobs2;
        const int grid2 = (int) std::min<long long>(tiles2, n_sm);
        k_tc_gemm<2><<<grid2, TC_THREADS, G_SMEM, st>>>(a, d_jobs2, njobs2, mxh, mxl, mwh, mwl);
        a.launches++;
    }
    if (a.mid_event) record_event(a.mid_event, st);
    k_tc_gram<<<dim3(a.gram_splits, a.n_chunks, a.gt * a.gt), R_THREADS, R_SMEM, st>>>(a, mph, mpl, mrh, mrl);
    a.launches += 2;
}

int gram_splits_mixed(int64_t K, int gram_k) {
    const int64_t k = gram_k > 0 ? gram_k : kGramK;
    return (int) ((K + k - 1) / k);
}

}  // namespace lqg
