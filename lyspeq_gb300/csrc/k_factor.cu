// FP64 factorisation of every chunk's covariance, one CTA per chunk, all
// chunks of the batch in one launch (largest first):
//   C~ = L L^T (blocked right-looking Cholesky),  X = L^-1 (blocked, row block
//   by row block),  C~^-1 = X^T X,  C^-1 = D C~^-1 D  (D = diag(sqrt(ivar))),
// then the continuum marginalisation (Chunk::_addMarginalizations,
// core/chunk_estimate.cpp:576-665) and y = C^-1 delta (:747-750).
// The reference inverts N^-1 C + I by LU instead (mathtools/matrix_helper.cpp:184-204);
// both give the same C^-1 (see k_fp64.cu).
//
// Every O(n^3) step is a sequence of 64 x 64 x 64 tile products staged in
// shared memory (two K-major tiles), 256 threads with a 4 x 4 register block
// each; rows {ti + 16u}, columns {tj + 16w} per thread keep shared-memory
// reads conflict-free.  The tile products run in FP64 for the FP64 path and
// in double-float (df64, 48 bits) on the FP32 pipe for the mixed path.
#include "lqg_internal.cuh"

namespace lqg {

namespace {

constexpr int FB = 64;             // tile edge
constexpr int FP = FB + 1;         // padded row of a shared tile
constexpr int FTH = 256;           // threads per CTA

__device__ __forceinline__ double block_sum_all(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int i = 0; i < FTH / 32; ++i) s += red[i];
    __syncthreads();
    return s;
}

__device__ __forceinline__ double block_max_all(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    for (int i = 0; i < FTH / 32; ++i) s = fmax(s, red[i]);
    __syncthreads();
    return s;
}

// Shared tile loaders.  K-major layout: t[k * FP + m].
// direct: t[k][m] = G[(r0 + k) * ld + c0 + m]  (rows of G are k)
template <class T>
__device__ __forceinline__ void load_direct(T *t, const T *G, int ld, int r0, int c0) {
    for (int e = threadIdx.x; e < FB * FB; e += FTH) {
        int k = e / FB, m = e % FB;
        t[k * FP + m] = G[(size_t) (r0 + k) * ld + c0 + m];
    }
}
// transposed: t[k][m] = G[(r0 + m) * ld + c0 + k]  (rows of G are m)
template <class T>
__device__ __forceinline__ void load_trans(T *t, const T *G, int ld, int r0, int c0) {
    for (int e = threadIdx.x; e < FB * FB; e += FTH) {
        int m = e / FB, k = e % FB;
        t[k * FP + m] = G[(size_t) (r0 + m) * ld + c0 + k];
    }
}

// acc[u][w] += sum_k A[k][ti + 16u] * B[k][tj + 16w]
__device__ __forceinline__ void tile_mma(double (&acc)[4][4], const double *A, const double *B, int klen) {
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
#pragma unroll 4
    for (int k = 0; k < klen; ++k) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { a[u] = A[k * FP + ti + 16 * u]; b[u] = B[k * FP + tj + 16 * u]; }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) acc[u][w] = fma(a[u], b[w], acc[u][w]);
    }
}

// ---------------------------------------------------------------------------
// Double-float (df64) arithmetic for the mixed path: a value is hi + lo (two
// floats, 48 significant bits), the matrix is kept in this form in memory
// between the steps, and the O(n^3) tile products run on the FP32 pipe
// (GB300's FP32 rate is 60x its FP64 rate).  The _rn intrinsics keep the
// compiler from contracting the error-free transformations.
__device__ __forceinline__ float2 to_df(double v) {
    const float h = __double2float_rn(v);
    return make_float2(h, __double2float_rn(v - (double) h));
}
__device__ __forceinline__ double df_to_d(float2 v) { return (double) v.x + (double) v.y; }

// Knuth's two-sum: a + b = s + e exactly
__device__ __forceinline__ float2 df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
// a - (bh + bl), renormalised
__device__ __forceinline__ float2 df_sub(float2 a, float bh, float bl) {
    const float2 s = df_two_sum(a.x, -bh);
    return df_two_sum(s.x, __fadd_rn(s.y, __fsub_rn(a.y, bl)));
}

// A tile of doubles already in shared memory, to df64 in place.
__device__ __forceinline__ void tile_to_df(double *t) {
    for (int e = threadIdx.x; e < FB * FB; e += FTH) {
        const int idx = (e / FB) * FP + e % FB;
        const double v = t[idx];
        reinterpret_cast<float2 *>(t)[idx] = to_df(v);
    }
}

struct DfAcc {
    float h[4][4], l[4][4];
};
__device__ __forceinline__ void df_zero(DfAcc &c) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) { c.h[u][w] = 0.f; c.l[u][w] = 0.f; }
}

// c[u][w] += sum_k A[k][ti + 16u] * B[k][tj + 16w] in df64: each product
// a * b = p + e up to the dropped lo * lo term (p = fl(hi * hi), e from FMAs),
// p added to the running hi by two-sum, the errors summed in lo.
__device__ __forceinline__ void tile_mma_df(DfAcc &c, const float2 *A2, const float2 *B2) {
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
#pragma unroll 2
    for (int k = 0; k < FB; ++k) {
        float2 a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) { a[u] = A2[k * FP + ti + 16 * u]; b[u] = B2[k * FP + tj + 16 * u]; }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int w = 0; w < 4; ++w) {
                const float p = __fmul_rn(a[u].x, b[w].x);
                float e = __fmaf_rn(a[u].x, b[w].x, -p);
                e = __fmaf_rn(a[u].x, b[w].y, e);
                e = __fmaf_rn(a[u].y, b[w].x, e);
                const float2 s2 = df_two_sum(c.h[u][w], p);
                c.h[u][w] = s2.x;
                c.l[u][w] = __fadd_rn(c.l[u][w], __fadd_rn(s2.y, e));
            }
    }
}

__device__ __forceinline__ void zero_acc(double (&acc)[4][4]) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int w = 0; w < 4; ++w) acc[u][w] = 0.0;
}

// In-shared-memory Cholesky of a 64 x 64 block stored row-major in d[r * FP + c]
// (lower triangle is used); returns false if a pivot is not positive.
__device__ bool chol_block(double *d, int *flag) {
    if (threadIdx.x == 0) *flag = 0;
    __syncthreads();
    for (int j = 0; j < FB; ++j) {
        const double piv = d[j * FP + j];
        if (threadIdx.x == 0 && (!(piv > 0.0) || !isfinite(piv))) *flag = 1;
        const double ljj = sqrt(piv > 0.0 ? piv : 1.0);
        __syncthreads();
        // column j below the diagonal
        for (int i = j + 1 + threadIdx.x; i < FB; i += FTH) d[i * FP + j] /= ljj;
        __syncthreads();
        if (threadIdx.x == 0) d[j * FP + j] = ljj;
        // rank-1 update of the trailing lower triangle
        const int m = FB - j - 1;
        for (int e = threadIdx.x; e < m * m; e += FTH) {
            int i = j + 1 + e / m, l = j + 1 + e % m;
            if (l <= i) d[i * FP + l] -= d[i * FP + j] * d[l * FP + j];
        }
        __syncthreads();
    }
    return *flag == 0;
}

// Inverse of the lower-triangular 64 x 64 block d (row-major) into x (row-major,
// zero above the diagonal).  Column c is solved by thread c.
__device__ void tri_inv_block(const double *d, double *x) {
    if (threadIdx.x < FB) {
        const int c = threadIdx.x;
        for (int r = 0; r < FB; ++r) {
            double s = (r == c) ? 1.0 : 0.0;
            if (r >= c) {
                for (int l = c; l < r; ++l) s -= d[r * FP + l] * x[l * FP + c];
                s /= d[r * FP + r];
            } else {
                s = 0.0;
            }
            x[r * FP + c] = s;
        }
    }
    __syncthreads();
}

struct FactorSmem {
    double a[FB * FP];
    double b[FB * FP];
    double red[FTH / 32];
    int flag;
};

// Blocked Cholesky in place (lower triangle of A, ld x ld, first nb*64 rows).
__device__ bool potrf_blocked(double *A, int ld, int nb, FactorSmem &s) {
    for (int kb = 0; kb < nb; ++kb) {
        const int k0 = kb * FB;
        // diagonal block
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            s.a[(e / FB) * FP + e % FB] = A[(size_t) (k0 + e / FB) * ld + k0 + e % FB];
        __syncthreads();
        if (!chol_block(s.a, &s.flag)) return false;
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            A[(size_t) (k0 + e / FB) * ld + k0 + e % FB] = s.a[(e / FB) * FP + e % FB];
        // b = (L_kk^-1)^T in K-major form: b[k][j] = Linv[j][k]
        tri_inv_block(s.a, s.b);           // s.b row-major inverse
        // transpose in place into K-major (b[k * FP + j] = Linv[j][k])
        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
            int r = e / FB, c = e % FB;
            if (c < r) {
                double t = s.b[r * FP + c];
                s.b[r * FP + c] = s.b[c * FP + r];
                s.b[c * FP + r] = t;
            }
        }
        __syncthreads();
        // panel: L_ik = A_ik L_kk^-T, tile by tile
        for (int ib = kb + 1; ib < nb; ++ib) {
            const int i0 = ib * FB;
            load_trans(s.a, A, ld, i0, k0);     // a[k][m] = A[i0 + m][k0 + k]
            __syncthreads();
            double acc[4][4];
            zero_acc(acc);
            // acc[m][j] = sum_k A[m][k] Linv[j][k]  with b[k][j] = Linv[j][k]
            tile_mma(acc, s.a, s.b, FB);
            __syncthreads();
            const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    A[(size_t) (i0 + ti + 16 * u) * ld + k0 + tj + 16 * w] = acc[u][w];
            __syncthreads();
        }
        // trailing update: A_ij -= L_ik L_jk^T for kb < jb <= ib
        for (int ib = kb + 1; ib < nb; ++ib)
            for (int jb = kb + 1; jb <= ib; ++jb) {
                const int i0 = ib * FB, j0 = jb * FB;
                load_trans(s.a, A, ld, i0, k0);
                load_trans(s.b, A, ld, j0, k0);
                __syncthreads();
                double acc[4][4];
                zero_acc(acc);
                tile_mma(acc, s.a, s.b, FB);
                const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w)
                        A[(size_t) (i0 + ti + 16 * u) * ld + j0 + tj + 16 * w] -= acc[u][w];
                __syncthreads();
            }
    }
    return true;
}

// In-place X = L^-1 (lower), row block by row block:
//   X_II = L_II^-1;  X_IC = -X_II sum_{J=C}^{I-1} L_IJ X_JC   for C < I.
// T = sum_J L_IJ X_JC is accumulated per column block into scratch (64 x ld).
__device__ void trtri_blocked(double *A, int ld, int nb, double *T, FactorSmem &s) {
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    for (int ib = 0; ib < nb; ++ib) {
        const int i0 = ib * FB;
        // T[:, C] for every C < I (reads L_I* and already inverted X rows above)
        for (int cb = 0; cb < ib; ++cb) {
            double acc[4][4];
            zero_acc(acc);
            for (int jb = cb; jb < ib; ++jb) {
                load_trans(s.a, A, ld, i0, jb * FB);       // a[k][m] = L[i0+m][j0+k]
                load_direct(s.b, A, ld, jb * FB, cb * FB);  // b[k][c] = X[j0+k][c0+c]
                __syncthreads();
                tile_mma(acc, s.a, s.b, FB);
                __syncthreads();
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) T[(size_t) (ti + 16 * u) * ld + cb * FB + tj + 16 * w] = acc[u][w];
        }
        __syncthreads();
        // X_II = L_II^-1 in s.b (row-major), then as K-major operand
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            s.a[(e / FB) * FP + e % FB] = A[(size_t) (i0 + e / FB) * ld + i0 + e % FB];
        __syncthreads();
        tri_inv_block(s.a, s.b);
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            A[(size_t) (i0 + e / FB) * ld + i0 + e % FB] = s.b[(e / FB) * FP + e % FB];
        // a[k][m] = X_II[m][k]
        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
            int m = e / FB, k = e % FB;
            s.a[k * FP + m] = s.b[m * FP + k];
        }
        __syncthreads();
        // X_IC = -X_II T_C
        for (int cb = 0; cb < ib; ++cb) {
            load_direct(s.b, T, ld, 0, cb * FB);           // b[k][c] = T[k][c0+c]
            __syncthreads();
            double acc[4][4];
            zero_acc(acc);
            tile_mma(acc, s.a, s.b, FB);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    A[(size_t) (i0 + ti + 16 * u) * ld + cb * FB + tj + 16 * w] = -acc[u][w];
            __syncthreads();
        }
    }
}

// In place: M = X^T X (lower tiles, row block by row block; within a row block the
// off-diagonal tiles first), then C^-1 = D M D symmetric in the full ld x ld.
__device__ void lauum_blocked(double *A, int ld, int nb, int n, const double *ivar, double *sq, FactorSmem &s) {
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    for (int ib = 0; ib < nb; ++ib) {
        for (int pass = 0; pass < 2; ++pass) {
            const int jlo = pass == 0 ? 0 : ib, jhi = pass == 0 ? ib : ib + 1;
            for (int jb = jlo; jb < jhi; ++jb) {
                double acc[4][4];
                zero_acc(acc);
                for (int lb = ib; lb < nb; ++lb) {
                    load_direct(s.a, A, ld, lb * FB, ib * FB);   // a[l][i] = X[l0+l][i0+i]
                    load_direct(s.b, A, ld, lb * FB, jb * FB);   // b[l][j] = X[l0+l][j0+j]
                    __syncthreads();
                    // X is lower triangular: zero its upper part inside the diagonal tiles
                    if (lb == ib)
                        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
                            int l = e / FB, i = e % FB;
                            if (l < i) s.a[l * FP + i] = 0.0;
                        }
                    if (lb == jb)
                        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
                            int l = e / FB, j = e % FB;
                            if (l < j) s.b[l * FP + j] = 0.0;
                        }
                    __syncthreads();
                    tile_mma(acc, s.a, s.b, FB);
                    __syncthreads();
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w)
                        A[(size_t) (ib * FB + ti + 16 * u) * ld + jb * FB + tj + 16 * w] = acc[u][w];
                __syncthreads();
            }
        }
    }
    for (int i = threadIdx.x; i < n; i += FTH) sq[i] = sqrt(ivar[i]);
    __syncthreads();
    for (size_t e = threadIdx.x; e < (size_t) ld * ld; e += FTH) {
        int i = (int) (e / ld), j = (int) (e % ld);
        if (j > i) continue;
        double v = 0.0;
        if (i < n && j < n) v = sq[i] * A[e] * sq[j];
        A[e] = v;
        A[(size_t) j * ld + i] = v;
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// The same three steps with the matrix held as df64 pairs (A2, the same bytes
// as the FP64 matrix).  The 64 x 64 diagonal-block Cholesky and inverse run in
// FP64 (O(64^3) per block) and are converted at their boundaries; every tile
// product, load and store is FP32-pipe work.

__device__ bool potrf_df(float2 *A2, int ld, int nb, FactorSmem &s) {
    float2 *sa2 = reinterpret_cast<float2 *>(s.a), *sb2 = reinterpret_cast<float2 *>(s.b);
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    for (int kb = 0; kb < nb; ++kb) {
        const int k0 = kb * FB;
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            s.a[(e / FB) * FP + e % FB] = df_to_d(A2[(size_t) (k0 + e / FB) * ld + k0 + e % FB]);
        __syncthreads();
        if (!chol_block(s.a, &s.flag)) return false;
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            A2[(size_t) (k0 + e / FB) * ld + k0 + e % FB] = to_df(s.a[(e / FB) * FP + e % FB]);
        tri_inv_block(s.a, s.b);           // s.b row-major inverse
        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
            int r = e / FB, c = e % FB;
            if (c < r) {
                double t = s.b[r * FP + c];
                s.b[r * FP + c] = s.b[c * FP + r];
                s.b[c * FP + r] = t;
            }
        }
        __syncthreads();
        tile_to_df(s.b);                   // b[k][j] = Linv[j][k] as df64
        __syncthreads();
        for (int ib = kb + 1; ib < nb; ++ib) {
            const int i0 = ib * FB;
            load_trans(sa2, A2, ld, i0, k0);
            __syncthreads();
            DfAcc c;
            df_zero(c);
            tile_mma_df(c, sa2, sb2);
            __syncthreads();
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    A2[(size_t) (i0 + ti + 16 * u) * ld + k0 + tj + 16 * w] = df_two_sum(c.h[u][w], c.l[u][w]);
            __syncthreads();
        }
        for (int ib = kb + 1; ib < nb; ++ib)
            for (int jb = kb + 1; jb <= ib; ++jb) {
                const int i0 = ib * FB, j0 = jb * FB;
                load_trans(sa2, A2, ld, i0, k0);
                load_trans(sb2, A2, ld, j0, k0);
                __syncthreads();
                DfAcc c;
                df_zero(c);
                tile_mma_df(c, sa2, sb2);
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w) {
                        float2 &dst = A2[(size_t) (i0 + ti + 16 * u) * ld + j0 + tj + 16 * w];
                        dst = df_sub(dst, c.h[u][w], c.l[u][w]);
                    }
                __syncthreads();
            }
    }
    return true;
}

__device__ void trtri_df(float2 *A2, int ld, int nb, float2 *T2, FactorSmem &s) {
    float2 *sa2 = reinterpret_cast<float2 *>(s.a), *sb2 = reinterpret_cast<float2 *>(s.b);
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    for (int ib = 0; ib < nb; ++ib) {
        const int i0 = ib * FB;
        for (int cb = 0; cb < ib; ++cb) {
            DfAcc c;
            df_zero(c);
            for (int jb = cb; jb < ib; ++jb) {
                load_trans(sa2, A2, ld, i0, jb * FB);
                load_direct(sb2, A2, ld, jb * FB, cb * FB);
                __syncthreads();
                tile_mma_df(c, sa2, sb2);
                __syncthreads();
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    T2[(size_t) (ti + 16 * u) * ld + cb * FB + tj + 16 * w] = df_two_sum(c.h[u][w], c.l[u][w]);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            s.a[(e / FB) * FP + e % FB] = df_to_d(A2[(size_t) (i0 + e / FB) * ld + i0 + e % FB]);
        __syncthreads();
        tri_inv_block(s.a, s.b);
        for (int e = threadIdx.x; e < FB * FB; e += FTH)
            A2[(size_t) (i0 + e / FB) * ld + i0 + e % FB] = to_df(s.b[(e / FB) * FP + e % FB]);
        // a[k][m] = X_II[m][k]: s.a is free (tri_inv_block ended with a barrier)
        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
            int m = e / FB, k = e % FB;
            sa2[k * FP + m] = to_df(s.b[m * FP + k]);
        }
        __syncthreads();
        for (int cb = 0; cb < ib; ++cb) {
            load_direct(sb2, T2, ld, 0, cb * FB);
            __syncthreads();
            DfAcc c;
            df_zero(c);
            tile_mma_df(c, sa2, sb2);
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int w = 0; w < 4; ++w) {
                    const float2 v = df_two_sum(c.h[u][w], c.l[u][w]);
                    A2[(size_t) (i0 + ti + 16 * u) * ld + cb * FB + tj + 16 * w] = make_float2(-v.x, -v.y);
                }
            __syncthreads();
        }
    }
}

// M = X^T X, then C^-1 = D M D symmetric as FP64 (the matrix leaves df64 form).
__device__ void lauum_df(float2 *A2, int ld, int nb, int n, const double *ivar, double *sq, FactorSmem &s) {
    float2 *sa2 = reinterpret_cast<float2 *>(s.a), *sb2 = reinterpret_cast<float2 *>(s.b);
    const int ti = threadIdx.x / 16, tj = threadIdx.x % 16;
    for (int ib = 0; ib < nb; ++ib) {
        for (int pass = 0; pass < 2; ++pass) {
            const int jlo = pass == 0 ? 0 : ib, jhi = pass == 0 ? ib : ib + 1;
            for (int jb = jlo; jb < jhi; ++jb) {
                DfAcc c;
                df_zero(c);
                for (int lb = ib; lb < nb; ++lb) {
                    load_direct(sa2, A2, ld, lb * FB, ib * FB);
                    load_direct(sb2, A2, ld, lb * FB, jb * FB);
                    __syncthreads();
                    if (lb == ib)
                        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
                            int l = e / FB, i = e % FB;
                            if (l < i) sa2[l * FP + i] = make_float2(0.f, 0.f);
                        }
                    if (lb == jb)
                        for (int e = threadIdx.x; e < FB * FB; e += FTH) {
                            int l = e / FB, j = e % FB;
                            if (l < j) sb2[l * FP + j] = make_float2(0.f, 0.f);
                        }
                    __syncthreads();
                    tile_mma_df(c, sa2, sb2);
                    __syncthreads();
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int w = 0; w < 4; ++w)
                        A2[(size_t) (ib * FB + ti + 16 * u) * ld + jb * FB + tj + 16 * w] =
                            df_two_sum(c.h[u][w], c.l[u][w]);
                __syncthreads();
            }
        }
    }
    for (int i = threadIdx.x; i < n; i += FTH) sq[i] = sqrt(ivar[i]);
    __syncthreads();
    double *A = reinterpret_cast<double *>(A2);
    // lower elements are read (as df64) and written (as FP64) by the same
    // thread; upper elements are only written
    for (size_t e = threadIdx.x; e < (size_t) ld * ld; e += FTH) {
        int i = (int) (e / ld), j = (int) (e % ld);
        if (j > i) continue;
        double v = 0.0;
        if (i < n && j < n) v = sq[i] * df_to_d(A2[e]) * sq[j];
        A[e] = v;
        A[(size_t) j * ld + i] = v;
    }
    __syncthreads();
}

// x^m for integer m >= 1 by repeated multiplication
__device__ __forceinline__ double ipow(double x, int m) {
    double r = x;
    for (int i = 1; i < m; ++i) r *= x;
    return r;
}

// Continuum templates [1/sqrt(n), (ln w)^m, w^m] (each of unit norm) and their
// left singular vectors by one-sided Jacobi on the n x nv matrix; vectors with
// s_i / s_0 <= 1e-15 are dropped (Chunk::_addMarginalizations,
// core/chunk_estimate.cpp:605-665).  The nuse vectors are left at U[u * ld].
__device__ int cont_basis(int ld, int n, const double *wave, int logl, int lord, double *V, double *U,
                          FactorSmem &s) {
    __shared__ double sv[kMaxContVecs], rot[2];
    __shared__ int order[kMaxContVecs], nuse_s, changed;
    int nv = 0;
    for (int i = threadIdx.x; i < n; i += FTH) V[i] = 1.0 / sqrt((double) n);
    nv = 1;
    for (int kind = 0; kind < 2; ++kind) {
        const int ordr = kind == 0 ? logl : lord;
        for (int cmo = 1; cmo <= ordr && nv < kMaxContVecs; ++cmo) {
            double part = 0;
            for (int i = threadIdx.x; i < n; i += FTH) {
                double x = ipow(kind == 0 ? log(wave[i]) : wave[i], cmo);
                V[nv * ld + i] = x;
                part += x * x;
            }
            const double inv = 1.0 / sqrt(block_sum_all(part, s.red));
            for (int i = threadIdx.x; i < n; i += FTH) V[nv * ld + i] *= inv;
            ++nv;
            __syncthreads();
        }
    }
    for (int sweep = 0; sweep < 60; ++sweep) {
        if (threadIdx.x == 0) changed = 0;
        __syncthreads();
        for (int p = 0; p < nv; ++p)
            for (int q = p + 1; q < nv; ++q) {
                double app = 0, aqq = 0, apq = 0;
                for (int i = threadIdx.x; i < n; i += FTH) {
                    double x = V[p * ld + i], z = V[q * ld + i];
                    app += x * x; aqq += z * z; apq += x * z;
                }
                app = block_sum_all(app, s.red);
                aqq = block_sum_all(aqq, s.red);
                apq = block_sum_all(apq, s.red);
                if (threadIdx.x == 0) {
                    rot[0] = 1.0; rot[1] = 0.0;
                    if (fabs(apq) > 1e-15 * sqrt(app * aqq)) {
                        double zeta = (aqq - app) / (2.0 * apq);
                        double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                        double cs = 1.0 / sqrt(1.0 + t * t);
                        rot[0] = cs; rot[1] = cs * t;
                        changed = 1;
                    }
                }
                __syncthreads();
                const double cs = rot[0], sn = rot[1];
                if (sn != 0.0)
                    for (int i = threadIdx.x; i < n; i += FTH) {
                        double x = V[p * ld + i], z = V[q * ld + i];
                        V[p * ld + i] = cs * x - sn * z;
                        V[q * ld + i] = sn * x + cs * z;
                    }
                __syncthreads();
            }
        // every thread takes the flag before thread 0 may reset it for the
        // next sweep: all threads must leave the loop at the same sweep
        const int again = changed;
        __syncthreads();
        if (!again) break;
    }
    for (int p = 0; p < nv; ++p) {
        double part = 0;
        for (int i = threadIdx.x; i < n; i += FTH) part += V[p * ld + i] * V[p * ld + i];
        double ss = block_sum_all(part, s.red);
        if (threadIdx.x == 0) sv[p] = sqrt(ss);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int p = 0; p < nv; ++p) order[p] = p;
        for (int p = 0; p < nv; ++p)
            for (int q = p + 1; q < nv; ++q)
                if (sv[order[q]] > sv[order[p]]) { int t = order[p]; order[p] = order[q]; order[q] = t; }
        int nuse = nv;
        while (nuse > 0 && !(sv[order[nuse - 1]] / sv[order[0]] > kDoubleEpsilon)) --nuse;
        nuse_s = nuse;
    }
    __syncthreads();
    const int nuse = nuse_s;
    for (int u = 0; u < nuse; ++u) {
        const int p = order[u];
        const double inv = 1.0 / sv[p];
        for (int i = threadIdx.x; i < n; i += FTH) U[u * ld + i] = V[p * ld + i] * inv;
    }
    __syncthreads();
    return nuse;
}

// Continuum marginalisation of C^-1: sequential rank-1 removal
// C^-1 <- C^-1 - (C^-1 v)(C^-1 v)^T / (v^T C^-1 v) over the basis above.
__device__ void marginalize_all(double *A, int ld, int n, const double *wave, int logl, int lord,
                                double *V /* (2 kMaxContVecs + 1) * ld */, FactorSmem &s) {
    double *y = V + kMaxContVecs * ld, *U = y + ld;
    const int nuse = cont_basis(ld, n, wave, logl, lord, V, U, s);
    for (int u = 0; u < nuse; ++u) {
        const double *vv = U + u * ld;
        for (int i = threadIdx.x; i < n; i += FTH) {
            double acc = 0;
            const double *Ai = A + (size_t) i * ld;
            for (int j = 0; j < n; ++j) acc += Ai[j] * vv[j];
            y[i] = acc;
        }
        __syncthreads();
        double part = 0;
        for (int i = threadIdx.x; i < n; i += FTH) part += vv[i] * y[i];
        const double cnorm = -1.0 / block_sum_all(part, s.red);
        for (size_t e = threadIdx.x; e < (size_t) n * ld; e += FTH) {
            int i = (int) (e / ld), j = (int) (e % ld);
            if (j < n) A[e] += cnorm * y[i] * y[j];
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// Whitened factor of the mixed path.  With C~ = L L^T and D = diag(sqrt(ivar)),
// C^-1 = T^T T for T = L^-1 D (lower triangular), and the marginalised inverse
// is T^T P T with P = I - U U^T, U the orthonormal basis of {T v} for the
// continuum templates v taken in the reference's order (the sequential
// rank-1 removals of _addMarginalizations are Gram-Schmidt in this space).
// The mixed products then work with W = P T, C^-1 = W^T W: F_ij =
// tr(C^-1 Q_i C^-1 Q_j) = <W Q_i W^T, W Q_j W^T>_F.  Without marginalisation
// W = T is lower triangular and the products skip its zero tiles.
//
// T from the df64 inverse factor, as FP64: A[i][j] = L^-1_ij sqrt(ivar_j) on
// and below the diagonal, 0 elsewhere (padding included).
__device__ void form_t_df(float2 *A2, int ld, int n, const double *ivar, double *sq) {
    for (int i = threadIdx.x; i < n; i += FTH) sq[i] = sqrt(ivar[i]);
    __syncthreads();
    double *A = reinterpret_cast<double *>(A2);
    for (size_t e = threadIdx.x; e < (size_t) ld * ld; e += FTH) {
        const int i = (int) (e / ld), j = (int) (e % ld);
        double v = 0.0;
        if (j <= i && i < n) v = df_to_d(A2[e]) * sq[j];
        A[e] = v;
    }
    __syncthreads();
}

// W = P T in place for the nuse plain-space template vectors U[u * ld]:
// w_u = T U_u, orthonormalised in order (modified Gram-Schmidt) into Wh,
// then W = T - Wh (Wh^T T).  Scratch: Wh and Z, nuse * ld each.  (Applying P
// afterwards as rank-r corrections of the traces instead cancels most of the
// low-k Fisher elements and loses their precision; W itself carries none.)
__device__ void project_w(double *A, int ld, int n, const double *U, int nuse, double *Wh, double *Z,
                          FactorSmem &s) {
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    for (int u = 0; u < nuse; ++u) {
        // w = T U_u, one warp per row (T is lower triangular)
        for (int i = warp; i < n; i += FTH / 32) {
            double acc = 0;
            const double *Ai = A + (size_t) i * ld;
            for (int j = lane; j <= i; j += 32) acc += Ai[j] * U[u * ld + j];
            for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
            if (lane == 0) Wh[u * ld + i] = acc;
        }
        __syncthreads();
        for (int v = 0; v < u; ++v) {
            double part = 0;
            for (int i = threadIdx.x; i < n; i += FTH) part += Wh[v * ld + i] * Wh[u * ld + i];
            const double c = block_sum_all(part, s.red);
            for (int i = threadIdx.x; i < n; i += FTH) Wh[u * ld + i] -= c * Wh[v * ld + i];
            __syncthreads();
        }
        double part = 0;
        for (int i = threadIdx.x; i < n; i += FTH) part += Wh[u * ld + i] * Wh[u * ld + i];
        const double nrm = sqrt(block_sum_all(part, s.red));
        const double inv = nrm > 0 ? 1.0 / nrm : 0.0;
        for (int i = threadIdx.x; i < n; i += FTH) Wh[u * ld + i] *= inv;
        __syncthreads();
    }
    // Z = Wh^T T: thread per column, rows j .. n - 1 (coalesced along the row)
    for (int j = threadIdx.x; j < n; j += FTH) {
        double z[kMaxContVecs] = {0, 0, 0, 0};
        for (int i = j; i < n; ++i) {
            const double t = A[(size_t) i * ld + j];
            for (int u = 0; u < nuse; ++u) z[u] += Wh[u * ld + i] * t;
        }
        for (int u = 0; u < nuse; ++u) Z[u * ld + j] = z[u];
    }
    __syncthreads();
    for (size_t e = threadIdx.x; e < (size_t) n * ld; e += FTH) {
        const int i = (int) (e / ld), j = (int) (e % ld);
        if (j >= n) continue;
        double v = A[e];
        for (int u = 0; u < nuse; ++u) v -= Wh[u * ld + i] * Z[u * ld + j];
        A[e] = v;
    }
    __syncthreads();
}

// The rest of the whitened factor: W (T, or P T with marginalisation) in A,
// y = W^T W delta, and the bounds max |W| and largest row sum of |W|
// (fbounds[4 gidx], [4 gidx + 1]).
__device__ void whitened_factor(const WaveArgs &a, const ChunkDesc &ch, float2 *A2, double *scratch,
                                FactorSmem &s) {
    const int ld = ch.ld, n = ch.n;
    double *A = reinterpret_cast<double *>(A2);
    form_t_df(A2, ld, n, a.ivar + ch.pix, scratch);
    int nuse = 0;
    if (a.cont_logl >= 0 || a.cont_l >= 0) {
        double *V = scratch, *U = V + kMaxContVecs * ld, *Wh = U + kMaxContVecs * ld, *Z = Wh + kMaxContVecs * ld;
        nuse = cont_basis(ld, n, a.wave + ch.pix, a.cont_logl, a.cont_l, V, U, s);
        project_w(A, ld, n, U, nuse, Wh, Z, s);
    }
    // t = W delta (warp per row), y = W^T t (thread per column)
    double *t = scratch;
    double *y = reinterpret_cast<double *>(a.fws + ch.o_y);
    const double *dl = a.delta + ch.pix;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    double mx = 0, rs = 0;
    for (int i = warp; i < ld; i += FTH / 32) {
        double acc = 0, r = 0;
        if (i < n) {
            const double *Ai = A + (size_t) i * ld;
            for (int j = lane; j < n; j += 32) {
                const double v = Ai[j];
                acc += v * dl[j];
                r += fabs(v);
                mx = fmax(mx, fabs(v));
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_down_sync(0xffffffffu, acc, o);
            r += __shfl_down_sync(0xffffffffu, r, o);
        }
        if (lane == 0) {
            t[i] = acc;
            rs = fmax(rs, r);
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < ld; j += FTH) {
        double acc = 0;
        if (j < n)
            for (int i = 0; i < n; ++i) acc += A[(size_t) i * ld + j] * t[i];
        y[j] = acc;
    }
    mx = block_max_all(mx, s.red);
    rs = block_max_all(rs, s.red);
    if (threadIdx.x == 0) {
        a.fbounds[4 * ch.gidx] = mx;
        a.fbounds[4 * ch.gidx + 1] = rs;
        a.fbounds[4 * ch.gidx + 2] = nuse;
        a.fbounds[4 * ch.gidx + 3] = 0.0;
    }
}

// The marginalised C^-1 of the whitened form in FP64 at o_m, from the df64
// inverse factor X = L^-1 (left in place for W): a copy of X, C^-1 = D X^T X D
// (lauum_df) and the reference's rank-1 removals.  k_dx_mixed contracts it
// with every Q_s for x_s = tr(Q_s C^-1), from which k_finish_dx forms
// d_s - b_s - t_s without the 22-bit trace products.
__device__ void marginal_inverse_df(const WaveArgs &a, const ChunkDesc &ch, const float2 *X2, int nb,
                                    double *scratch, FactorSmem &s) {
    const int ld = ch.ld, n = ch.n;
    float2 *M2 = reinterpret_cast<float2 *>(a.fws + ch.o_m);
    for (size_t e = threadIdx.x; e < (size_t) nb * FB * ld; e += FTH) M2[e] = X2[e];
    __syncthreads();
    lauum_df(M2, ld, nb, n, a.ivar + ch.pix, scratch, s);
    if (a.cont_logl >= 0 || a.cont_l >= 0)
        marginalize_all(reinterpret_cast<double *>(M2), ld, n, a.wave + ch.pix, a.cont_logl, a.cont_l, scratch, s);
}

template <bool DF>
__global__ void __launch_bounds__(FTH, 3) k_factor_tiled(WaveArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    FactorSmem &s = *reinterpret_cast<FactorSmem *>(smem_raw);
    const int c = blockIdx.x;
    const ChunkDesc &ch = a.chunks[c];
    if (a.status[ch.gidx] != LQG_CHUNK_OK) return;
    const int ld = ch.ld, n = ch.n, nb = (n + FB - 1) / FB;
    if (!LQG_IN_BOUNDS(a, (a.ext_cy || (ch.o_c >= 0 && ch.o_c + (int64_t) ld * ld * 8 <= a.fws_bytes &&
                                         ch.o_y >= 0 && ch.o_y + (int64_t) ld * 8 <= a.fws_bytes)) &&
                              ch.o_fscr >= 0 && ch.o_fscr + (int64_t) FB * ld * 8 <= a.fws_bytes &&
                              nb * FB <= ld && ch.pix >= 0 && ch.pix + n <= a.n_pix &&
                              (!ch.cinv_m || (ch.o_m >= 0 && ch.o_m + (int64_t) ld * ld * 8 <= a.fws_bytes)),
                       10, c, ch.o_fscr)) {
        // only the self-checking build gets here: skip the chunk, visibly
        if (threadIdx.x == 0) a.status[ch.gidx] = LQG_CHUNK_INDEX_CHECK;
        return;
    }
    double *A = reinterpret_cast<double *>(a.fws + ch.o_c);
    double *scratch = reinterpret_cast<double *>(a.fws + ch.o_fscr);
    const double *iv = a.ivar + ch.pix;
    if (DF) {
        // C~ to df64 in place (the pair occupies the double's 8 bytes), unless
        // the matrix build already wrote it in that form
        if (!a.c_is_ff) {
            for (size_t e = threadIdx.x; e < (size_t) ld * ld; e += FTH) {
                const double v = A[e];
                reinterpret_cast<float2 *>(A)[e] = to_df(v);
            }
            __syncthreads();
        }
        float2 *A2 = reinterpret_cast<float2 *>(A);
        if (!potrf_df(A2, ld, nb, s)) {
            if (threadIdx.x == 0) a.status[ch.gidx] = LQG_CHUNK_NOT_SPD;
            return;
        }
        __syncthreads();
        trtri_df(A2, ld, nb, reinterpret_cast<float2 *>(scratch), s);
        __syncthreads();
        if (ch.sym) {
            if (ch.cinv_m) {
                marginal_inverse_df(a, ch, A2, nb, scratch, s);
                __syncthreads();
            }
            whitened_factor(a, ch, A2, scratch, s);
            return;
        }
        lauum_df(A2, ld, nb, n, iv, scratch, s);
    } else {
        if (!potrf_blocked(A, ld, nb, s)) {
            if (threadIdx.x == 0) a.status[ch.gidx] = LQG_CHUNK_NOT_SPD;
            return;
        }
        __syncthreads();
        trtri_blocked(A, ld, nb, scratch, s);
        __syncthreads();
        lauum_blocked(A, ld, nb, n, iv, scratch, s);
    }
    if (a.cont_logl >= 0 || a.cont_l >= 0)
        marginalize_all(A, ld, n, a.wave + ch.pix, a.cont_logl, a.cont_l, scratch, s);
    // y = C^-1 delta, and the bounds max |C^-1| and max row sum of |C^-1|:
    // one warp per row, lanes along the row (coalesced)
    double *y = reinterpret_cast<double *>(a.fws + ch.o_y);
    const double *dl = a.delta + ch.pix;
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    double mx = 0, rs = 0;
    for (int i = warp; i < ld; i += FTH / 32) {
        double acc = 0, r = 0;
        if (i < n) {
            const double *Ai = A + (size_t) i * ld;
            for (int j = lane; j < n; j += 32) {
                const double v = Ai[j];
                acc += v * dl[j];
                r += fabs(v);
                mx = fmax(mx, fabs(v));
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            acc += __shfl_down_sync(0xffffffffu, acc, o);
            r += __shfl_down_sync(0xffffffffu, r, o);
        }
        if (lane == 0) {
            y[i] = acc;
            rs = fmax(rs, r);
        }
    }
    mx = block_max_all(mx, s.red);
    rs = block_max_all(rs, s.red);
    if (threadIdx.x == 0) {
        a.fbounds[4 * ch.gidx] = mx;
        a.fbounds[4 * ch.gidx + 1] = rs;
    }
}

}  // namespace

size_t factor_smem_bytes() { return sizeof(FactorSmem); }

// The FP64 path factors in FP64 throughout; the mixed path runs the tile
// products in df64 on the FP32 pipe (the diagonal-block Cholesky and inverse,
// the scaling and the marginalisation stay FP64).
void launch_factor_all(WaveArgs &a, cudaStream_t st) {
    // FactorSmem is above the 48 KB default: the attribute, once per device
    static std::atomic<unsigned long long> attr{0};
    const bool ready = once_per_device(attr, [](int) {
        cudaError_t e = cudaFuncSetAttribute(k_factor_tiled<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int) sizeof(FactorSmem));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_factor_tiled<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int) sizeof(FactorSmem));
        return e;
    });
    if (!ready) {
        a.host_failed = 1;
        return;
    }
    if (a.precision == LQG_PRECISION_MIXED)
        k_factor_tiled<true><<<a.n_chunks, FTH, sizeof(FactorSmem), st>>>(a);
    else
        k_factor_tiled<false><<<a.n_chunks, FTH, sizeof(FactorSmem), st>>>(a);
    a.launches++;
}

}  // namespace lqg
