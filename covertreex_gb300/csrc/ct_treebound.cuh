// ct_treebound.cuh — certified error bounds that make the cover-tree prune exact.
//
// The plain FP32 forms evaluate d32(q, x) = sqrt(1 - |rho32|) from the stored f32 V,
// p and coordinates in the reference's batch-path arithmetic.  That FP32 function is
// not itself a metric (rounding breaks the triangle inequality, badly where p is
// tiny), so a cover radius alone cannot prune exactly.  The bounds here relate it to
// an ideal metric d* that does satisfy the triangle inequality:
//
//   rho*(q, x) = C(q, x) / sqrt(C(q, q) C(x, x)),  C = K - V V^T,
//
// with K the kernel of the original coordinates and V = K_xm (K_mm + jitter I)^-1/2
// in exact arithmetic.  C is a posterior covariance (positive semi-definite), so rho*
// is a correlation and d* = sqrt(1 - |rho*|) = min over s = +-1 of |a - s b| / sqrt(2)
// for unit feature vectors a, b: a metric.  For every pair,
//
//   |d32^2 - d*^2| <= delta(q, x),
//   delta = [eK + c_dot |v_q| |v_x| + u var] / sqrt(p_q p_x) + (r_q + r_x) / 2 + 8 u,
//
// where u = 2^-24 and
//   eK     kernel-value error: the coordinate squared distance from the scaled f32
//          coordinates and norms (|x_q|^2 + |x_x|^2 - 2 x_q.x_x, (D + 8) u per unit of
//          the norms, including the 1/l scaling), the exp / Matern evaluation (16 u var);
//   c_dot  the V dot product: the 16-lane order (m/16 + 6 roundings, doubled), the f32
//          rounding of V itself (3 u) and the FP64 construction error (2 eta, eta =
//          2^-28 relative, generous for the jittered Cholesky solve);
//   r      the relative error of p against C(x, x): the f32 rounding (u) plus the FP64
//          evaluation of var - |v|^2 ((m + 2) 2^-53 (var + |v|^2)) and the V error
//          (2 eta |v|^2), divided by p.
// Rows with 1/sqrt(p) above kSideIsp are kept out of the tree (see ct_build.cu); a query
// with 1/sqrt(p_q) above kNoPruneIsp prunes nothing.  Every bound below is evaluated in
// FP32 with its own rounding covered by small relative and absolute margins.
#pragma once
#include <cuda_runtime.h>

namespace ct {

constexpr float kSideIsp = 32.f;       // p < 1/1024: rows scored by every query, outside the tree
constexpr float kNoPruneIsp = 1.0e4f;  // p < 1e-8: the query is scored against every node

struct BoundModel {
    float ck;    // eK per unit of (|x_q|^2 + |x_x|^2)
    float ck0;   // eK floor
    float cdot;  // V-dot error per unit of |v_q| |v_x|
    float cvar;  // rounding of K - dot
    float cpa;   // p error: (cpa (var + |v|^2) + cpb |v|^2) / p
    float cpb;
    float var;
    float vmax, nmax;  // dataset maxima of |v| and of the scaled squared norms
};

inline BoundModel make_bound_model(int m, int d, int kernel_type, float var, float vmax, float nmax) {
    const double u = 1.0 / 16777216.0;
    const double eta = 1.0 / 268435456.0;
    BoundModel B;
    const double kc = kernel_type == 0 ? 1.0 : 2.0;  // Matern: |dK/dd2| <= (5/6) var
    B.ck = (float)(var * kc * (d + 8) * u * 1.01);
    B.ck0 = (float)(var * 16.0 * u);
    B.cdot = (float)(((m / 8.0 + 12.0) * u + 2.0 * eta) * 1.01);
    B.cvar = (float)(var * u * 2.0);
    B.cpa = (float)((m + 2) * 1.2e-16);
    B.cpb = (float)(2.0 * eta);
    B.var = var;
    B.vmax = vmax;
    B.nmax = nmax;
    return B;
}

// delta(q, x) of the header, in units of d^2.
__host__ __device__ __forceinline__ float pair_delta(const BoundModel& B, float nq, float nx, float vq, float vx,
                                                     float isq, float isx) {
    const float a = (B.ck * (nq + nx) + B.ck0 + B.cdot * vq * vx + B.cvar) * isq * isx;
    const float rq = 6.0e-8f + (B.cpa * (B.var + vq * vq) + B.cpb * vq * vq) * isq * isq;
    const float rx = 6.0e-8f + (B.cpa * (B.var + vx * vx) + B.cpb * vx * vx) * isx * isx;
    return (a + 0.55f * (rq + rx)) * 1.0001f + 5.0e-7f;
}

// Certified upper / lower bounds of d* from an FP32 distance and its delta.
__host__ __device__ __forceinline__ float dist_upper(float d32, float delta) {
    const float s = d32 * d32 + delta + 5.0e-7f;
    return sqrtf(s < 1.f ? s : 1.f) * (1.f + 5.0e-7f);
}
__host__ __device__ __forceinline__ float dist_lower(float d, float delta) {
    const float s = d * d - delta - 5.0e-7f;
    return s > 0.f ? sqrtf(s) * (1.f - 5.0e-7f) : 0.f;
}

}  // namespace ct
