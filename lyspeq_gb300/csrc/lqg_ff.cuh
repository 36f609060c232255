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

// ((1 + z) / (1 + z_m))^B in FP32 (the ratio is within 1e-7 relative, as the
// 22-bit operands need).
__device__ __forceinline__ float growth_ff(const DeviceBins &b, int zm, float P, float E) {
    return powf(__fdiv_rn(__fadd_rn(P, E), __fadd_rn(b.zc1_hi[zm], b.zc1_lo[zm])), (float) b.growth_b);
}

// zweight_ff times, with the growth option on, the growth factor.
__device__ __forceinline__ float zfactor_ff(const DeviceBins &b, int zm, float P, float E) {
    float w = zweight_ff(b, zm, P, E);
    if (b.growth && w != 0.f) w *= growth_ff(b, zm, P, E);
    return w;
}

// ---- double-float arithmetic on the FP32 pipe (value = hi + lo) ----
__device__ __forceinline__ float2 ff_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    return make_float2(s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb)));
}
__device__ __forceinline__ float2 ff_norm(float s, float e) {
    const float h = __fadd_rn(s, e);
    return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}
__device__ __forceinline__ float2 ff_add(float2 a, float2 b) {
    const float2 s = ff_two_sum(a.x, b.x);
    return ff_norm(s.x, __fadd_rn(s.y, __fadd_rn(a.y, b.y)));
}
__device__ __forceinline__ float2 ff_sub(float2 a, float2 b) { return ff_add(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 ff_mul(float2 a, float2 b) {
    float p, e;
    two_prod_ff(a, b, p, e);
    return ff_norm(p, e);
}
__device__ __forceinline__ float2 ff_fma(float2 a, float2 b, float2 c) { return ff_add(ff_mul(a, b), c); }
__device__ __forceinline__ float2 ff_of(double x) {
    const float h = (float) x;
    return make_float2(h, (float) (x - (double) h));
}

// Clamped interpolation index and fraction of x (a double-float >= any
// negative value), the reference's rule (discrete_interpolation.cpp:61-72,
// 221-242): n = trunc(x) clamped to [0, nmax], fraction x - n.
__device__ __forceinline__ void ff_index(float2 x, int nmax, int &n, float2 &frac) {
    int nn = (int) floorf(x.x);
    float2 f = ff_norm(__fsub_rn(x.x, (float) nn), x.y);
    if (f.x < 0.f) { --nn; f = ff_add(f, make_float2(1.f, 0.f)); }
    else if (f.x >= 1.f) { ++nn; f = ff_sub(f, make_float2(1.f, 0.f)); }
    // trunc rather than floor below zero (the reference casts to int)
    if (nn < 0) nn = (x.x < 0.f && x.x > -1.f) ? 0 : nn;
    if (nn > nmax) nn = nmax;
    if (nn < 0) nn = 0;
    f = ff_norm(__fsub_rn(x.x, (float) nn), x.y);
    n = nn;
    frac = f;
}

// Redshift weight of bin zm at 1 + z = P + E as a double-float (zweight's
// rules, zweight_ff's exact u_hi = P - (1 + z_c)_hi): w = (dz - |u|) / dz.
__device__ __forceinline__ float2 zweight_dd(const DeviceBins &b, int zm, float P, float E) {
    const float u_hi = __fsub_rn(P, b.zc1_hi[zm]);
    const float u_lo = __fsub_rn(E, b.zc1_lo[zm]);
    const float u = __fadd_rn(u_hi, u_lo);
    const float au_hi = fabsf(u_hi);
    const float au_lo = u_hi > 0.f ? u_lo : (u_hi < 0.f ? -u_lo : fabsf(u_lo));
    if (!b.triangular || b.nz == 1) {
        const float r = __fadd_rn(__fsub_rn(b.dzh_hi, au_hi), __fsub_rn(b.dzh_lo, au_lo));
        return make_float2(r >= 0.f ? 1.f : 0.f, 0.f);
    }
    if (zm == 0 && u < 0.f) return make_float2(1.f, 0.f);
    if (zm == b.nz - 1 && u > 0.f) return make_float2(1.f, 0.f);
    const float2 r = ff_add(make_float2(b.dz_hi, b.dz_lo), make_float2(-au_hi, -au_lo));
    if (r.x < 0.f) return make_float2(0.f, 0.f);
    return ff_mul(r, make_float2(b.idz_hi, b.idz_lo));
}

// Table index and fraction at v = c (ln w_hi - ln w_lo) with the fraction as a
// double-float (vindex_ff keeps it as one float).
__device__ __forceinline__ void vindex_dd(const TableGrid &g, float2 lwh, float2 lwl, int &n, float2 &dn) {
    const float2 d = make_float2(__fsub_rn(lwh.x, lwl.x), __fsub_rn(lwh.y, lwl.y));
    float p, e;
    two_prod_ff(d, make_float2(g.kv_hi, g.kv_lo), p, e);
    ff_index(ff_norm(p, e), g.nv - 2, n, dn);
}

// Sum over the warp of a double-float value (hi, lo) by double-float additions;
// every lane gets the total.
__device__ __forceinline__ float2 warp_sum_ff(float2 v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float h = __shfl_xor_sync(0xffffffffu, v.x, o), l = __shfl_xor_sync(0xffffffffu, v.y, o);
        const float2 s = ff_two_sum(v.x, h);
        v = ff_norm(s.x, __fadd_rn(s.y, __fadd_rn(v.y, l)));
    }
    return v;
}

// (s, c) += (ah + al)(bh + bl): the product as p + e (p = fl(ah bh), e its
// error and the cross terms), p added to the running sum s by two-sum, every
// error collected in c (Ogita-Rump-Oishi Sum2 with exact products).
__device__ __forceinline__ void dd_mac(float &s, float &c, float ah, float al, float2 b) {
    const float p = __fmul_rn(ah, b.x);
    float e = __fmaf_rn(ah, b.x, -p);
    e = __fmaf_rn(ah, b.y, e);
    e = __fmaf_rn(al, b.x, e);
    const float t = __fadd_rn(s, p);
    const float bb = __fsub_rn(t, s);
    const float err = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s = t;
    c = __fadd_rn(c, __fadd_rn(err, e));
}

}  // namespace lqg
