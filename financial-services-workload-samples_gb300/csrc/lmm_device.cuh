// Device helpers shared by the LMM kernels: PTX fast math, Philox4x32-10,
// Box-Muller, warp reductions.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "lmm_internal.h"

// 1: the FP32 kernels' 32-path column sums are TwoSum-compensated before
// they reach their FP64 accumulators (two_sum_acc); 0: plain FP32 sums.
// GB300, 80/40 fused kernel at 4,194,304 paths: 10.87 ms plain, 11.04 ms
// compensated, with the same largest errors against FP64.
#ifndef LMM_COMP_SUMS
#define LMM_COMP_SUMS 1
#endif

// 1: the long-tenor (160/120) forwards share one MUFU reciprocal between the
// cells of one step at rates 2m and 2m+1 (rcp_pair), as the 80/40 forwards do
// with LMM_FWD_RCP2. Shared by the fused kernel (lmm_f32_tpp.cu) and the
// thread pair of the forward/backward API (lmm_f32_tp2.cu), which must round
// alike. GB300, fused 160/120 kernel at 1,048,576 paths: 14.19 ms without,
// 18.8 ms with (its 255-register forward pass does not take the pairs'
// extra live values), so it is off.
#ifndef LMM_FWD_RCP2_LONG
#define LMM_FWD_RCP2_LONG 0
#endif

namespace lmm {

// MUFU approximations issued directly (PTX ISA: rcp.approx.ftz.f32,
// ex2.approx.ftz.f32). Both are within a few ulp in FP32.
__device__ __forceinline__ float rcp_approx(float x)
{
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ float ex2_approx(float x)
{
    float r;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// Two reciprocals from one: 1/a = b/(ab), 1/b = a/(ab). The forward's a, b
// are 1/L + delta >= delta; ab overflows FP32 only if both rates fall below
// about 5e-20 (from L0 >= 1e-3, more than 30 standard deviations of the
// log-rate's spread over 40 steps at lambda = 0.35), so the product stays
// far inside the range.
__device__ __forceinline__ void rcp_pair(float a, float b, float &ta, float &tb)
{
    const float r = rcp_approx(a * b);
    ta = b * r;
    tb = a * r;
}

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): multipliers 0xD2511F53,
// 0xCD9E8D57 and Weyl key increments 0x9E3779B9, 0xBB67AE85, ten rounds.
struct U4 {
    uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r > 0) {
            k0 += 0x9E3779B9u;
            k1 += 0xBB67AE85u;
        }
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}

// The counter layout of the library: normals 4q..4q+3 of global path p.
__device__ __forceinline__ U4 philox_quad(uint64_t seed, uint64_t path, uint32_t q)
{
    return philox4x32_10(U4{q, 0u, (uint32_t)path, (uint32_t)(path >> 32)}, (uint32_t)seed,
                         (uint32_t)(seed >> 32));
}

// FP32 Box-Muller on 24-bit uniforms: u1 = ((a>>8)+1)/2^24 in (0,1],
// u2 = (b>>8)/2^24 in [0,1); z0 = r cos(2 pi u2), z1 = r sin(2 pi u2).
__device__ __forceinline__ void box_muller_f32(uint32_t a, uint32_t b, float &z0, float &z1)
{
    const float u1 = (float)((a >> 8) + 1u) * 5.9604644775390625e-8f;
    const float u2 = (float)(b >> 8) * 5.9604644775390625e-8f;
    const float r = sqrtf(-2.0f * logf(u1));
    float s, c;
    sincospif(2.0f * u2, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__device__ __forceinline__ void normals_quad_f32(uint64_t seed, uint64_t path, uint32_t q,
                                                 float z[4])
{
    const U4 x = philox_quad(seed, path, q);
    box_muller_f32(x.x, x.y, z[0], z[1]);
    box_muller_f32(x.z, x.w, z[2], z[3]);
}

// FP64 Box-Muller on 32-bit uniforms (the FP64 spec of the library).
__device__ __forceinline__ void box_muller_f64(uint32_t a, uint32_t b, double &z0, double &z1)
{
    const double u1 = ((double)a + 1.0) * 2.3283064365386962890625e-10;
    const double u2 = (double)b * 2.3283064365386962890625e-10;
    const double r = sqrt(-2.0 * log(u1));
    const double th = 6.283185307179586476925286766559 * u2;
    double s, c;
    sincos(th, &s, &c);
    z0 = r * c;
    z1 = r * s;
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Double-FP32 ("float-float") numbers hi + lo, |lo| <= ulp(hi)/2, for the
// payoff's discount and annuity products and the swap values. They use the
// error-free transforms TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and the FMA form
// of Dekker's product, about 48 significant bits. On GB300 an FP64 warp
// instruction occupies its pipe about as long as 64 FP32 instructions, so
// these run on the FP32 pipe. Every step is an explicitly rounded intrinsic,
// so the compiler cannot contract or reorder the error terms.
struct F2 {
    float hi, lo;
};

// a + b as F2, given |a| >= |b| or a == 0 (Fast2Sum).
__device__ __forceinline__ F2 f2_fast(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ F2 f2_mul(F2 x, float y)
{
    const float p = __fmul_rn(x.hi, y);
    return f2_fast(p, __fmaf_rn(x.lo, y, __fmaf_rn(x.hi, y, -p)));
}

__device__ __forceinline__ F2 f2_mul(F2 x, F2 y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    float e = __fmaf_rn(x.hi, y.hi, -p);
    e = __fmaf_rn(x.hi, y.lo, e);
    e = __fmaf_rn(x.lo, y.hi, e);
    return f2_fast(p, e);
}

__device__ __forceinline__ F2 f2_add(F2 x, F2 y)
{
    const float s = __fadd_rn(x.hi, y.hi);
    const float v = __fsub_rn(s, x.hi);
    const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, v)), __fsub_rn(y.hi, v));
    return f2_fast(s, __fadd_rn(e, __fadd_rn(x.lo, y.lo)));
}

__device__ __forceinline__ F2 f2_add(F2 x, float y) { return f2_add(x, F2{y, 0.0f}); }

// Compensated FP32 summation: s + c carries the running sum, s its rounded
// value and c the accumulated rounding errors of the additions, each
// recovered exactly by TwoSum (Knuth, TAOCP vol. 2, 4.2.2). The result is
// about as accurate as an FP64 sum of the same FP32 terms.
__device__ __forceinline__ void two_sum_acc(float &s, float &c, float x)
{
    const float t = __fadd_rn(s, x);
    const float v = __fsub_rn(t, s);
    c = __fadd_rn(c, __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(x, v)));
    s = t;
}

// The F2 nearest a double (host data staged once per block).
__device__ __forceinline__ F2 f2_from(double x)
{
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}

// Swap value (:145) K*s + b - 1 from the F2 annuity sum (sb = s/delta, kd =
// K*delta) and annuity factor b, rounded once to FP32. For a high part in
// [1/2, 2] subtracting 1 is exact (Sterbenz); outside it the swap value is
// far from 0 and one more rounding does not matter.
__device__ __forceinline__ float f2_swap_value(F2 kd, F2 sb, F2 b)
{
    const F2 t = f2_add(f2_mul(sb, kd), b);
    return __fadd_rn(__fsub_rn(t.hi, 1.0f), t.lo);
}


// Four consecutive normals n = 4q..4q+3 of one path: read from memory (16-byte
// aligned since nmat % 4 == 0) or generated by Philox.
template <bool PHILOX, int NMAT>
__device__ __forceinline__ float4 zquad(const float *zp, uint64_t seed, uint64_t gpath, int q)
{
    if (PHILOX) {
        float g[4];
        normals_quad_f32(seed, gpath, (uint32_t)q, g);
        return make_float4(g[0], g[1], g[2], g[3]);
    } else {
        return __ldg(reinterpret_cast<const float4 *>(zp) + q);
    }
}

// The bond ratio 1/(1+delta L) from the inverse rate il = 1/L and
// t = 1/(il + delta) (MUFU reciprocal, within 1 ulp): 1 - delta t while
// delta L < 1 (within 0.5 + delta L ulp), il t above (within 2.5 ulp).
__device__ __forceinline__ float bond_ratio_t(float il, float delta, float t)
{
    return il > delta ? fmaf(-delta, t, 1.0f) : il * t;
}

__device__ __forceinline__ float bond_ratio(float il, float delta)
{
    return bond_ratio_t(il, delta, rcp_approx(il + delta));
}

}  // namespace lmm
