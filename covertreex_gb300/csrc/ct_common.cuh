// ct_common.cuh — shared device helpers for the GB300 residual-correlation
// cover-tree engine (sm_103a).
//
// Arithmetic conventions of the plain FP32 form: every multiply and add is a
// separately rounded IEEE binary32 operation (__fmul_rn / __fadd_rn), so the
// compiler cannot contract them into FMAs.  That is the arithmetic of the
// reference's x86-64 build of src/metric.rs (covertreex), whose
// `wide::f32x8::mul_add` is a separate multiply and add without the FMA
// target feature.  exp() is `ct_expf` below, shared bit for bit with the CPU
// restatement used as the parity oracle.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#define CT_OK 0
#define CT_ERR_ARG 1
#define CT_ERR_CUDA 2
#define CT_ERR_STATE 3
#define CT_ERR_UNSUPPORTED 4
#define CT_ERR_TIMEOUT 5
#define CT_ERR_NOMEM 6

#define CT_FLT_MAX 3.402823466e+38f

namespace ct {

// exp(x): Cody-Waite reduction x = n*ln2 + r (|r| <= ln2/2) with a two-part
// ln2, then the degree-7 Taylor polynomial of e^r in Horner form (fmaf), then
// scaling by 2^n.  |error| <= 1 ulp against the correctly rounded value.
__device__ __forceinline__ float expf_ct(float x) {
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return __int_as_float(0x7f800000);
    const float log2e = 1.44269504088896341f;
    const float ln2_hi = 0.693145751953125f;
    const float ln2_lo = 1.42860682030941723e-6f;
    float n = rintf(__fmul_rn(x, log2e));
    float r = __fmaf_rn(-n, ln2_hi, x);
    r = __fmaf_rn(-n, ln2_lo, r);
    float p = 1.98412698412698413e-4f;
    p = __fmaf_rn(p, r, 1.38888888888888889e-3f);
    p = __fmaf_rn(p, r, 8.33333333333333333e-3f);
    p = __fmaf_rn(p, r, 4.16666666666666667e-2f);
    p = __fmaf_rn(p, r, 1.66666666666666667e-1f);
    p = __fmaf_rn(p, r, 0.5f);
    p = __fmaf_rn(p, r, 1.0f);
    p = __fmaf_rn(p, r, 1.0f);
    // p in [0.7, 1.42] and n in [-126, 127]: scale through the exponent field
    // in two exact steps (no subnormal results are reachable for x >= -87).
    int ni = (int)n;
    int h = ni >> 1;
    float s1 = __int_as_float((h + 127) << 23);
    float s2 = __int_as_float((ni - h + 127) << 23);
    return __fmul_rn(__fmul_rn(p, s1), s2);
}

// Residual kernel value from the squared scaled distance d2 (the batch path of
// src/metric.rs:456-465).  kernel_type 0 = RBF, 1 = Matern 5/2.
__device__ __forceinline__ float kernel_value_batch(float d2, float var, int kernel_type) {
    if (kernel_type == 0) {
        return __fmul_rn(var, expf_ct(__fmul_rn(-0.5f, d2)));
    }
    float r = __fsqrt_rn(d2);
    float a = __fmul_rn(2.2360679775f, r);
    float poly = __fadd_rn(__fadd_rn(1.0f, a), __fmul_rn(__fmul_rn(a, a), 0.3333333333f));
    return __fmul_rn(__fmul_rn(var, poly), expf_ct(-a));
}

// Final residual distance from the kernel value, the V dot product and the two
// residual variances (src/metric.rs:467-485): denom = sqrt(max(pq*pc, 1e-18)),
// rho clamped to [-1, 1], d = sqrt(1 - |rho|).
__device__ __forceinline__ float residual_from_parts(float kval, float dot_v, float pq, float pc) {
    const float ee = __int_as_float(0x219392ee);  // 1e-9f * 1e-9f rounded to binary32
    float pp = __fmul_rn(pq, pc);
    float denom = __fsqrt_rn(pp > ee ? pp : ee);
    float rho = __fdiv_rn(__fsub_rn(kval, dot_v), denom);
    rho = rho > -1.0f ? rho : -1.0f;
    rho = rho < 1.0f ? rho : 1.0f;
    float ds = __fsub_rn(1.0f, fabsf(rho));
    return ds > 0.0f ? __fsqrt_rn(ds) : 0.0f;
}

// Squared scaled coordinate distance, batch path (src/metric.rs:439-454):
// D == 3 is the unrolled left-to-right sum, otherwise a loop from 0.
__device__ __forceinline__ float coord_d2_batch(const float* xq, const float* xc, int d, float nq, float nc) {
    float dot;
    if (d == 3) {
        dot = __fadd_rn(__fadd_rn(__fmul_rn(xq[0], xc[0]), __fmul_rn(xq[1], xc[1])), __fmul_rn(xq[2], xc[2]));
    } else {
        dot = 0.0f;
        for (int c = 0; c < d; ++c) dot = __fadd_rn(dot, __fmul_rn(xq[c], xc[c]));
    }
    float d2 = __fsub_rn(__fadd_rn(nq, nc), __fmul_rn(2.0f, dot));
    return d2 < 0.0f ? 0.0f : d2;
}

// (dist, idx) lexicographic order used for every selection in the engine.
__device__ __forceinline__ bool nb_less(float da, int64_t ia, float db, int64_t ib) {
    return da < db || (da == db && ia < ib);
}

}  // namespace ct
