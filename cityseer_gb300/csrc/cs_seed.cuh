// cs_seed.cuh -- the beta-weighted Brandes seed exp(-beta * cost) to f64 accuracy on the FP32 pipe.
//
// The reference seeds the beta-weighted betweenness with pair * exp(-(beta as f64) * (cost as f64))
// in f64 (rust/src/centrality.rs:1806-1808, 2508-2510).  GB300 runs f64 arithmetic at 1/64 of the
// f32 rate, and one library exp(double) per reached (target, threshold) pair cost more than the
// rest of the backward sweep.  This header evaluates the same value to about 1e-14 relative error
// (the reference's own libm exp is within 1.1e-16) with double-float arithmetic (pairs of f32,
// error-free transformations with FMA, Dekker 1971 / Knuth TAOCP 4.2.2) on the f32 pipe:
//
//   y = beta * cost exactly, as the pair (yh, yl) = two_prod(beta, cost) (both operands are f32,
//       so their product has at most 48 significant bits, as in the reference's f64 product);
//   y = j / 256 + t with j = floor(256 yh) and 0 <= t < 1/256 (yh - j / 256 is exact);
//   exp(-y) = T[j] * exp(-t), T[j] = exp(-j / 256) tabulated once per call by seed_table_kernel
//       with the library's f64 exp and split into a double-float pair;
//   exp(-t) = 1 - t + t^2 / 2 + q, q = -t^3 / 6 + t^4 / 24 - t^5 / 120 (|q| < 1.1e-8, taken in f32:
//       its error is below 3e-15), the Taylor series of exp truncated after t^5 (the remainder is
//       below t^6 / 720 < 5e-18 for t < 1/256).
// Arguments y outside [0, 8) (betas that are not 4 / d over costs beyond the threshold) take the
// library's f64 exp.  cs_debug_seed_exp checks the result against the f64 exp on the device.
#pragma once
#include "cs_common.cuh"

namespace cs {

constexpr int SEED_TAB = 2048;  // exp(-j / 256) for j < 2048: arguments below 8
// Each translation unit that includes this header has its own copy, filled by seed_table_kernel
// (launched on the call's stream before the kernels that read it).
static __device__ float2 seed_tab[SEED_TAB];

static __global__ void seed_table_kernel() {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < SEED_TAB; j += gridDim.x * blockDim.x) {
        const double e = exp(-(double)j / 256.0);
        const float hi = __double2float_rn(e);
        const float lo = __double2float_rn(e - (double)hi);
        seed_tab[j] = make_float2(hi, lo);
    }
}

struct dfloat {
    float h, l;
};

__device__ __forceinline__ dfloat df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ dfloat df_fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dfloat df_two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ dfloat df_add(dfloat a, dfloat b) {
    dfloat s = df_two_sum(a.h, b.h);
    const dfloat t = df_two_sum(a.l, b.l);
    s.l = __fadd_rn(s.l, t.h);
    s = df_fast_two_sum(s.h, s.l);
    s.l = __fadd_rn(s.l, t.l);
    return df_fast_two_sum(s.h, s.l);
}
__device__ __forceinline__ dfloat df_mul(dfloat a, dfloat b) {
    dfloat p = df_two_prod(a.h, b.h);
    p.l = __fmaf_rn(a.h, b.l, p.l);
    p.l = __fmaf_rn(a.l, b.h, p.l);
    return df_fast_two_sum(p.h, p.l);
}

// exp(-(beta * cost)) as a double-float pair, the product beta * cost taken exactly.  Returns false
// (r untouched) when the argument lies outside [0, 8): the caller then takes the f64 exp.
__device__ __forceinline__ bool seed_exp_df(float beta, float cost, dfloat &r) {
    const dfloat y = df_two_prod(beta, cost);
    if (!(y.h >= 0.0f && y.h < 8.0f)) return false;
    const int j = min((int)__fmul_rn(y.h, 256.0f), SEED_TAB - 1);
    const dfloat t = df_two_sum(__fsub_rn(y.h, __fmul_rn((float)j, 1.0f / 256.0f)), y.l);
    const float tf = t.h;
    const float q = __fmul_rn(__fmul_rn(__fmul_rn(tf, tf), tf),
                              __fmaf_rn(tf, __fmaf_rn(tf, -1.0f / 120.0f, 1.0f / 24.0f), -1.0f / 6.0f));
    dfloat t2 = df_mul(t, t);
    t2.h = __fmul_rn(t2.h, 0.5f);
    t2.l = __fmul_rn(t2.l, 0.5f);
    dfloat e = df_add({1.0f, 0.0f}, {-t.h, -t.l});
    e = df_add(e, t2);
    e = df_add(e, {q, 0.0f});
    const float2 tj = seed_tab[j];
    r = df_mul({tj.x, tj.y}, e);
    return true;
}

// w * exp(-(beta * cost)) as f64, for a pair weight w (0.5 or 1 for centrality, a trip weight for
// origin-destination betweenness); the product with w is taken in double-float.
__device__ __forceinline__ double seed_exp(float w, float beta, float cost) {
    dfloat r;
    if (!seed_exp_df(beta, cost, r)) {
        const dfloat y = df_two_prod(beta, cost);
        return (double)w * exp(-((double)y.h + (double)y.l));
    }
    if (w != 1.0f) r = df_mul(r, {w, 0.0f});
    return f2d(r.h) + f2d(r.l);
}

}  // namespace cs
