// Double-float helpers (a value is hi + lo, two floats) shared by the
// FP32-pipe element math of the mixed path.
#pragma once

#include "lqg_internal.cuh"

namespace lqg {

// a * b for double-float a, b: p + e (the lo * lo term is below 2^-46)
__device__ __forceinline__ void two_prod_ff(float2 a, float2 b, float &p, float &e) {
    p = __fmul_rn(a.x, b.x);
    e = __fmaf_rn(a.x, b.x, -p);
    e = __fmaf_rn(a.x, b.y, e);
    e = __fmaf_rn(a.y, b.x, e);
}

// Redshift weight of bin zm at 1 + z = P + E (zweight's rules): u = z - z_c
// as u_hi (exact) + u_lo, and dz - |u| formed before any rounding.
__device__ __forceinline__ float zweight_ff(const DeviceBins &b, int zm, float P, float E) {
    const float u_hi = __fsub_rn(P, b.zc1_hi[zm]);
    const float u_lo = __fsub_rn(E, b.zc1_lo[zm]);
    const float u = __fadd_rn(u_hi, u_lo);
    const float au_hi = fabsf(u_hi);
    const float au_lo = u_hi > 0.f ? u_lo : (u_hi < 0.f ? -u_lo : fabsf(u_lo));
    if (!b.triangular || b.nz == 1) {
        const float r = __fadd_rn(__fsub_rn(b.dzh_hi, au_hi), __fsub_rn(b.dzh_lo, au_lo));
        return r >= 0.f ? 1.f : 0.f;
    }
    if (zm == 0 && u < 0.f) return 1.f;
    if (zm == b.nz - 1 && u > 0.f) return 1.f;
    const float r = __fadd_rn(__fsub_rn(b.dz_hi, au_hi), __fsub_rn(b.dz_lo, au_lo));
    return r >= 0.f ? r * b.inv_dz : 0.f;
}

}  // namespace lqg
