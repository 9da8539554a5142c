// ct_brute.cu — plain FP32 residual-correlation kNN, dense form for one tree.
//
// One CTA owns a tile of QT queries and sweeps every candidate (or, in
// predecessor mode, every candidate with a smaller dataset index than the
// tile's largest query).  The tile itself (dot-product order, distance
// epilogue, top-k merge) is dense::run_tile in ct_dense.cuh, shared with the
// batched persistent kernel.
#include "ct_common.cuh"
#include "ct_dense.cuh"
#include "ct_internal.h"

namespace ct {

namespace {

using dense::kThreads;

template <int QT>
__global__ void __launch_bounds__(kThreads, 1) brute_knn_kernel(BruteParams P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    dense::Tile J;
    J.vperm = P.vperm; J.xs = P.xs; J.norms = P.norms; J.p = P.p;
    J.n = P.n; J.m = P.m; J.d = P.d; J.k = P.k; J.kernel_type = P.kernel_type; J.predecessor = P.predecessor;
    J.var = P.var;
    J.qids = P.qids; J.qv = nullptr; J.qcoords = nullptr; J.qp = nullptr; J.inv_ls = nullptr;
    J.nq = P.nq;
    // heavy tiles (large query ids in predecessor mode) first
    J.q0 = ((long long)gridDim.x - 1 - blockIdx.x) * QT;
    J.cbeg = P.cbeg; J.cend = P.cend > 0 ? P.cend : P.n;
    J.out_idx = P.out_idx; J.out_dist = P.out_dist; J.out_stride = P.k;
    dense::run_tile<QT>(J, smem_raw);
}

}  // namespace

size_t brute_smem_bytes(int qt, int m, int d, int k) { return dense::layout(qt, m, d, k).total; }

int brute_pick_qt(int m, int d, int k, size_t smem_limit) {
    const int qts[3] = {64, 32, 16};
    for (int t = 0; t < 3; ++t)
        if (dense::layout(qts[t], m, d, k).total <= smem_limit) return qts[t];
    return 0;
}

cudaError_t launch_brute_knn(const BruteParams& P, int qt, cudaStream_t stream) {
    const size_t smem = dense::layout(qt, P.m, P.d, P.k).total;
    const long long tiles = (P.nq + qt - 1) / qt;
    if (tiles <= 0) return cudaSuccess;
    dim3 grid((unsigned)tiles), block(kThreads);
    cudaError_t e;
    switch (qt) {
        case 64:
            e = cudaFuncSetAttribute(brute_knn_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            brute_knn_kernel<64><<<grid, block, smem, stream>>>(P);
            break;
        case 32:
            e = cudaFuncSetAttribute(brute_knn_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            brute_knn_kernel<32><<<grid, block, smem, stream>>>(P);
            break;
        default:
            e = cudaFuncSetAttribute(brute_knn_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return e;
            brute_knn_kernel<16><<<grid, block, smem, stream>>>(P);
            break;
    }
    return cudaGetLastError();
}

}  // namespace ct
