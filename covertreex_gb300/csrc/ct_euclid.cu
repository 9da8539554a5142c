// ct_euclid.cu — exact Euclidean kNN (the reference's Euclidean cover-tree path,
// CoverTreeWrapper.insert / knn_query, src/lib.rs:207-223,331 and
// src/algo.rs:179-323, which prunes with 2^(level+1) radii the greedy batch
// insert does not guarantee; this search is exhaustive and exact).
//
// One thread per query; candidate points are staged through shared memory in
// tiles; each thread keeps its k best (d^2, index) pairs sorted in local memory
// and inserts only candidates that beat the current k-th.  d^2 is the
// left-to-right sum of squared differences, as `Euclidean::distance_sq`
// (src/metric.rs:33-41); the returned distance is its square root.
#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {
namespace {

constexpr int kEThreads = 128;
constexpr int kETile = 512;
constexpr int kEMaxK = 64;
constexpr int kEMaxD = 16;

__global__ void __launch_bounds__(kEThreads) euclid_knn_kernel(const float* __restrict__ pts, long long n, int d,
                                                                const float* __restrict__ qry, long long nq, int k,
                                                                int predecessor, long long* __restrict__ out_idx,
                                                                float* __restrict__ out_dist) {
    __shared__ float tile[kETile * kEMaxD];
    const long long qi = (long long)blockIdx.x * kEThreads + threadIdx.x;
    const bool active = qi < nq;
    float q[kEMaxD];
#pragma unroll
    for (int c = 0; c < kEMaxD; ++c) q[c] = (active && c < d) ? qry[qi * d + c] : 0.f;
    float bd[kEMaxK];
    int bi[kEMaxK];
    int cnt = 0;
    const long long limit = predecessor ? (active ? qi : 0) : n;
    // the block needs candidates below the largest limit of its queries
    long long block_limit = predecessor ? (long long)min((long long)n, ((long long)blockIdx.x + 1) * kEThreads) : n;
    for (long long t0 = 0; t0 < block_limit; t0 += kETile) {
        const int tn = (int)min((long long)kETile, block_limit - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < tn * d; e += kEThreads) tile[e] = pts[t0 * d + e];
        __syncthreads();
        if (!active) continue;
        for (int j = 0; j < tn; ++j) {
            const long long gj = t0 + j;
            if (gj >= limit) break;
            float s = 0.f;
            for (int c = 0; c < d; ++c) {
                float df = q[c] - tile[j * d + c];
                s += df * df;
            }
            if (cnt < k || s < bd[k - 1]) {
                int pos = cnt < k ? cnt : k - 1;
                while (pos > 0 && bd[pos - 1] > s) {  // equal distances keep the lower index first
                    bd[pos] = bd[pos - 1];
                    bi[pos] = bi[pos - 1];
                    --pos;
                }
                bd[pos] = s;
                bi[pos] = (int)gj;
                if (cnt < k) ++cnt;
            }
        }
    }
    if (!active) return;
    for (int j = 0; j < k; ++j) {
        const bool ok = j < cnt;
        out_idx[qi * k + j] = ok ? (long long)bi[j] : -1LL;
        out_dist[qi * k + j] = ok ? sqrtf(bd[j]) : CT_FLT_MAX;
    }
}

}  // namespace

cudaError_t launch_euclid_knn(const float* pts, long long n, int d, const float* qry, long long nq, int k,
                              int predecessor, long long* out_idx, float* out_dist, cudaStream_t st) {
    if (nq <= 0) return cudaSuccess;
    euclid_knn_kernel<<<(unsigned)((nq + kEThreads - 1) / kEThreads), kEThreads, 0, st>>>(
        pts, n, d, qry, nq, k, predecessor, out_idx, out_dist);
    return cudaGetLastError();
}

int euclid_max_k() { return kEMaxK; }
int euclid_max_d() { return kEMaxD; }

}  // namespace ct
