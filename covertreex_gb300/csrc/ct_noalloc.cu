// ct_noalloc.cu — an allocation-free variant of the plain FP32 dense residual
// kNN (ct_knn_residual with CT_FORM_DENSE).
//
// Who needs it: callers that must not allocate device memory themselves or let
// a library do it — e.g. an application whose framework owns every byte of the
// GPU through its own pool and forbids other allocators, or a latency-critical
// loop that cannot afford the implicit device synchronisation of
// cudaMalloc/cudaFree.  They pass inputs and outputs; everything the dense
// kernel needs beyond them (the residue-major V copy, scaled coordinates, norms,
// p copy, 1/lengthscale) lives in one file-scope __device__ array of fixed size,
// reserved when the library is loaded and held by every GPU that loads it until
// the process exits.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <mutex>

#include "../../include/covertree_cuda.h"
#include "ct_common.cuh"
#include "ct_internal.h"

namespace {

constexpr size_t kScratchBytes = (size_t)CT_NOALLOC_SCRATCH_BYTES;
__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device addresses of g_noalloc_scratch, looked up once per device.
std::mutex g_mu;
void* g_scratch_addr[128] = {nullptr};

struct InvLs {
    float v[64];
};

__global__ void write_inv_ls_kernel(InvLs ls, int d, float* out) {
    int i = threadIdx.x;
    if (i < d) out[i] = ls.v[i];
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

size_t ct_noalloc_bytes_needed(long long n, int m, int d) {
    return align256((size_t)n * m * 4) + align256((size_t)n * d * 4) + align256((size_t)n * 4) +
           align256((size_t)n * 4) + align256(64 * 4);
}

// Scratch address for the current device: cudaGetSymbolAddress on first use
// (with that device current), cached afterwards.
static int noalloc_scratch(void** out, char* err, size_t errlen) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { snprintf(err, errlen, "cudaGetDevice: %s", cudaGetErrorString(e)); return CT_ERR_CUDA; }
    if (dev < 0 || dev >= 128) { snprintf(err, errlen, "device ordinal %d out of range", dev); return CT_ERR_ARG; }
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            snprintf(err, errlen, "cudaGetSymbolAddress(no-allocation scratch): %s", cudaGetErrorString(e));
            return CT_ERR_CUDA;
        }
        g_scratch_addr[dev] = ptr;
    }
    *out = g_scratch_addr[dev];
    return CT_OK;
}

int ct_noalloc_dense_impl(const float* v, const float* p, const float* coords, long long n, int m, int d,
                          float variance, const float* lengthscale, int n_lengthscale, int kernel_type,
                          const long long* q_ids, long long nq, int k, int predecessor, long long* out_idx,
                          float* out_dist, cudaStream_t st, char* err, size_t errlen) {
    const size_t need = ct_noalloc_bytes_needed(n, m, d);
    if (need > kScratchBytes) {
        snprintf(err, errlen,
                 "n=%lld, m=%d, d=%d needs %zu bytes of scratch; the no-allocation entry point holds %zu "
                 "(use ct_build_residual + ct_knn_residual)", n, m, d, need, kScratchBytes);
        return CT_ERR_UNSUPPORTED;
    }
    void* base = nullptr;
    int rc = noalloc_scratch(&base, err, errlen);
    if (rc != CT_OK) return rc;
    int dev = 0;
    cudaGetDevice(&dev);
    int smem_optin = 0;
    cudaError_t e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) { snprintf(err, errlen, "device attribute: %s", cudaGetErrorString(e)); return CT_ERR_CUDA; }
    const int qt = ct::brute_pick_qt(m, d, k, (size_t)smem_optin);
    if (qt == 0) { snprintf(err, errlen, "m=%d, k=%d exceed shared memory", m, k); return CT_ERR_UNSUPPORTED; }
    // carve the scratch: every byte is written below before it is read, so
    // nothing has to be cleared between calls
    unsigned char* b = (unsigned char*)base;
    float* vperm = (float*)b; b += align256((size_t)n * m * 4);
    float* xs = (float*)b; b += align256((size_t)n * d * 4);
    float* norms = (float*)b; b += align256((size_t)n * 4);
    float* pc = (float*)b; b += align256((size_t)n * 4);
    float* inv_ls = (float*)b;
    InvLs ils;
    const float fallback = (lengthscale && n_lengthscale > 0) ? lengthscale[0] : 1.0f;
    for (int i = 0; i < 64; ++i) ils.v[i] = 1.0f;
    for (int i = 0; i < d; ++i) {
        const float raw = (lengthscale && i < n_lengthscale) ? lengthscale[i] : fallback;
        const float safe = fabsf(raw) < 1e-6f ? 1e-6f : raw;
        ils.v[i] = 1.0f / safe;  // ResidualMetric::new, src/metric.rs:93-101
    }
    write_inv_ls_kernel<<<1, 64, 0, st>>>(ils, d, inv_ls);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = ct::launch_metric_setup(v, p, coords, n, m, d, inv_ls, vperm, xs, norms, pc, st);
    if (e == cudaSuccess) {
        ct::BruteParams P;
        P.vperm = vperm; P.xs = xs; P.norms = norms; P.p = pc;
        P.qids = q_ids; P.n = n; P.nq = nq; P.m = m; P.d = d; P.k = k;
        P.kernel_type = kernel_type == 1 ? 1 : 0; P.predecessor = predecessor ? 1 : 0; P.var = variance;
        P.out_idx = out_idx; P.out_dist = out_dist;
        e = ct::launch_brute_knn(P, qt, st);
    }
    if (e != cudaSuccess) { snprintf(err, errlen, "%s", cudaGetErrorString(e)); return CT_ERR_CUDA; }
    return CT_OK;
}
