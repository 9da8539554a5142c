// ct_euclid.cu — exact Euclidean kNN (the reference's Euclidean cover-tree path,
// CoverTreeWrapper.insert / knn_query, src/lib.rs:207-223,331 and
// src/algo.rs:179-323, which prunes with 2^(level+1) radii the greedy batch
// insert does not guarantee; this search is exhaustive and exact).
//
// One warp per query, eight queries per CTA.  Candidate points are staged
// through shared memory in tiles shared by the CTA's warps; lane l of a warp
// scores the tile's candidates l, l + 32, ... and keeps its own k best
// (d^2, index) in registers, sorted, inserting only candidates that beat its
// current k-th (a lane sees its candidates in increasing index, so a tie keeps
// the lower index).  At the end the warp merges its 32 sorted lists with k
// rounds of a warp-wide (d^2, index) minimum.  d^2 is the left-to-right sum of
// squared differences, as `Euclidean::distance_sq` (src/metric.rs:33-41); the
// returned distance is its square root.
#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {
namespace {

constexpr int kEWarps = 8;
constexpr int kEThreads = 32 * kEWarps;
constexpr int kETile = 1024;
constexpr int kEMaxK = 64;
constexpr int kEMaxD = 16;

__device__ __forceinline__ bool dl_less(float da, int ia, float db, int ib) {
    return da < db || (da == db && ia < ib);
}

template <int K>
__global__ void __launch_bounds__(kEThreads) euclid_knn_kernel(const float* __restrict__ pts, long long n, int d,
                                                               const float* __restrict__ qry, long long nq, int k,
                                                               int predecessor, long long* __restrict__ out_idx,
                                                               float* __restrict__ out_dist) {
    extern __shared__ float tile[];  // kETile * d floats
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long qi = (long long)blockIdx.x * kEWarps + warp;
    const bool active = qi < nq;
    float q[kEMaxD];
#pragma unroll
    for (int c = 0; c < kEMaxD; ++c) q[c] = (active && c < d) ? qry[qi * d + c] : 0.f;
    float bd[K];
    int bi[K];
#pragma unroll
    for (int j = 0; j < K; ++j) { bd[j] = CT_FLT_MAX; bi[j] = 0x7fffffff; }
    const long long limit = predecessor ? (active ? qi : 0) : n;
    // the CTA needs candidates below the largest limit of its queries
    const long long block_limit =
        predecessor ? min(n, ((long long)blockIdx.x + 1) * kEWarps) : n;
    for (long long t0 = 0; t0 < block_limit; t0 += kETile) {
        const int tn = (int)min((long long)kETile, block_limit - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < tn * d; e += kEThreads) tile[e] = pts[t0 * d + e];
        __syncthreads();
        if (!active) continue;
        const int jn = (int)min((long long)tn, limit - t0);
        for (int j = lane; j < jn; j += 32) {
            float s = 0.f;
            for (int c = 0; c < d; ++c) {
                const float df = q[c] - tile[j * d + c];
                s += df * df;
            }
            if (s < bd[K - 1]) {  // strict: an equal distance seen later has a larger index
                const int gj = (int)(t0 + j);
                // register insertion: shift the entries above s up by one
#pragma unroll
                for (int p = K - 1; p > 0; --p) {
                    const bool up = s < bd[p - 1];
                    const bool here = !up && s < bd[p];
                    bd[p] = up ? bd[p - 1] : (here ? s : bd[p]);
                    bi[p] = up ? bi[p - 1] : (here ? gj : bi[p]);
                }
                if (s < bd[0]) { bd[0] = s; bi[0] = gj; }
            }
        }
    }
    if (!active) return;
    // k rounds of a warp-wide minimum over the lanes' list heads
    int head = 0;
    for (int r = 0; r < k; ++r) {
        float hd = CT_FLT_MAX;
        int hi = 0x7fffffff;
#pragma unroll
        for (int j = 0; j < K; ++j)
            if (j == head) { hd = bd[j]; hi = bi[j]; }
        float md = hd;
        int mi = hi;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, md, off);
            const int oi = __shfl_xor_sync(0xffffffffu, mi, off);
            if (dl_less(od, oi, md, mi)) { md = od; mi = oi; }
        }
        if (hd == md && hi == mi && hi != 0x7fffffff) ++head;
        if (lane == 0) {
            const bool ok = mi != 0x7fffffff && md < CT_FLT_MAX;
            out_idx[qi * k + r] = ok ? (long long)mi : -1LL;
            out_dist[qi * k + r] = ok ? sqrtf(md) : CT_FLT_MAX;
        }
    }
}

template <int K>
cudaError_t launch_k(const float* pts, long long n, int d, const float* qry, long long nq, int k, int predecessor,
                     long long* out_idx, float* out_dist, cudaStream_t st) {
    const size_t smem = sizeof(float) * kETile * (size_t)d;
    cudaError_t e = cudaFuncSetAttribute(euclid_knn_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    euclid_knn_kernel<K><<<(unsigned)((nq + kEWarps - 1) / kEWarps), kEThreads, smem, st>>>(
        pts, n, d, qry, nq, k, predecessor, out_idx, out_dist);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_euclid_knn(const float* pts, long long n, int d, const float* qry, long long nq, int k,
                              int predecessor, long long* out_idx, float* out_dist, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    if (k <= 16) return launch_k<16>(pts, n, d, qry, nq, k, predecessor, out_idx, out_dist, st);
    if (k <= 32) return launch_k<32>(pts, n, d, qry, nq, k, predecessor, out_idx, out_dist, st);
    return launch_k<64>(pts, n, d, qry, nq, k, predecessor, out_idx, out_dist, st);
}

int euclid_max_k() { return kEMaxK; }
int euclid_max_d() { return kEMaxD; }

}  // namespace ct
