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
#include <cuda.h>
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

// Device addresses of g_noalloc_scratch, looked up once per CUDA context and kept
// under the context's unique id (cuCtxGetId ids are never reused), so that a context
// destroyed by cudaDeviceReset, or a caller's own non-primary context on the same
// device, gets its own lookup instead of a stale address.
std::mutex g_mu;
constexpr int kCacheSlots = 64;
unsigned long long g_ctx_id[kCacheSlots] = {0};
void* g_scratch_addr[kCacheSlots] = {nullptr};
int g_next_slot = 0;

struct InvLs {
    float v[64];
};

__global__ void write_inv_ls_kernel(InvLs ls, int d, float* out) {
    int i = threadIdx.x;
    if (i < d) out[i] = ls.v[i];
}

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

// Scratch bytes a call needs: five pieces, each rounded up to a multiple of 256
// bytes — V in residue-major order (4 n m), scaled coordinates (4 n d), squared norms
// (4 n), p (4 n) and the inverse lengthscales (256).
size_t ct_noalloc_bytes_needed(long long n, int m, int d) {
    return align256((size_t)n * m * 4) + align256((size_t)n * d * 4) + align256((size_t)n * 4) +
           align256((size_t)n * 4) + align256(64 * 4);
}

// Unique id of the calling thread's current CUDA context (0 if none or unknown).  The
// two driver functions are fetched through the runtime, so the library does not link
// the driver library itself (it still loads on machines without a GPU driver).
static unsigned long long current_context_id() {
    typedef CUresult (*get_current_fn)(CUcontext*);
    typedef CUresult (*get_id_fn)(CUcontext, unsigned long long*);
    static get_current_fn get_current = nullptr;
    static get_id_fn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* a = nullptr;
        void* b = nullptr;
        cudaDriverEntryPointQueryResult qa, qb;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) == cudaSuccess &&
            qa == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) == cudaSuccess &&
            qb == cudaDriverEntryPointSuccess) {
            get_current = (get_current_fn)a;
            get_id = (get_id_fn)b;
        }
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current && get_id && get_current(&ctx) == CUDA_SUCCESS && ctx && get_id(ctx, &id) == CUDA_SUCCESS)
        return id;
    return 0;
}

// Scratch address in the calling thread's current context: cudaGetSymbolAddress on
// the first call in a context (which also creates the device's primary context when
// none is current), cached by context id afterwards.
static int noalloc_scratch(void** out, char* err, size_t errlen) {
    unsigned long long id = current_context_id();
    if (id) {
        std::lock_guard<std::mutex> lock(g_mu);
        for (int i = 0; i < kCacheSlots; ++i)
            if (g_ctx_id[i] == id) { *out = g_scratch_addr[i]; return CT_OK; }
    }
    void* ptr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || !ptr) {
        snprintf(err, errlen, "cudaGetSymbolAddress(no-allocation scratch): %s", cudaGetErrorString(e));
        return CT_ERR_CUDA;
    }
    // the lookup made the runtime's context current if none was: key the cache by it
    id = current_context_id();
    if (id) {
        std::lock_guard<std::mutex> lock(g_mu);
        g_ctx_id[g_next_slot] = id;
        g_scratch_addr[g_next_slot] = ptr;
        g_next_slot = (g_next_slot + 1) % kCacheSlots;
    }
    *out = ptr;
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
