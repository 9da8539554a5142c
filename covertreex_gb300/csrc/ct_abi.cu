// ct_abi.cu — extern "C" entry points of libcovertree_cuda.so (declared in
// include/covertree_cuda.h).  No torch types cross this boundary: plain device
// pointers, sizes and a cudaStream_t.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <new>

#include "../../include/covertree_cuda.h"
#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_tree.h"
#include "ct_vmatrix.h"

int ct_screen_debug_dots(ct_tree* T, const int* rows_a, const int* rows_b, float* out, cudaStream_t st);
int ct_noalloc_dense_impl(const float* v, const float* p, const float* coords, long long n, int m, int d,
                          float variance, const float* lengthscale, int n_lengthscale, int kernel_type,
                          const long long* q_ids, long long nq, int k, int predecessor, long long* out_idx,
                          float* out_dist, cudaStream_t st, char* err, size_t errlen);

namespace {

thread_local char g_last_error[512] = "";
thread_local bool g_timing = false;
thread_local int g_cta_budget = 0;  // cap on the grid of the FP64 embed kernels (0 = none)

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char* where) {
    return fail(CT_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

// The engine's per-call buffers come from the stream-ordered allocator; let the
// device's default pool keep freed memory for reuse (this process only) instead of
// returning it at every synchronisation.
void keep_pool_memory() {
    static bool done[64] = {false};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long keep = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[dev] = true;
}

}  // namespace

namespace ct {
bool timing_enabled() { return g_timing; }
int batch_fail(const char* where, const char* msg, int code) { return fail(code, "%s: %s", where, msg); }
}  // namespace ct

#define CT_CUDA(call, where)                          \
    do {                                              \
        cudaError_t e_ = (call);                      \
        if (e_ != cudaSuccess) return cuda_fail(e_, where); \
    } while (0)

namespace {
// rows[i] of src (w floats per row) -> row i of dst
__global__ void gather_f32_rows_kernel(const float* __restrict__ src, const int64_t* __restrict__ rows, long long n,
                                       int w, float* __restrict__ dst) {
    const long long total = n * (long long)w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / w;
        dst[e] = src[rows[r] * w + (e - r * w)];
    }
}
__global__ void check_rows_kernel(const int64_t* __restrict__ rows, long long n, long long limit, int* __restrict__ bad) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n && (rows[i] < 0 || rows[i] >= limit || (i > 0 && rows[i] <= rows[i - 1]))) atomicOr(bad, 1);
}
}  // namespace

extern "C" {

int ct_version(void) { return 10000; }

int ct_set_timing(int enable) {
    g_timing = enable != 0;
    return CT_OK;
}

int ct_set_cta_budget(int32_t ctas) {
    if (ctas < 0) return fail(CT_ERR_ARG, "ct_set_cta_budget: ctas < 0");
    g_cta_budget = ctas;
    return CT_OK;
}

const char* ct_last_error(void) { return g_last_error; }

int ct_build_residual(const float* v, const float* p, const float* coords, int64_t n, int32_t m, int32_t d,
                      float variance, const float* lengthscale, int32_t n_lengthscale, int32_t kernel_type,
                      int32_t chunk, int32_t order, uint64_t seed, int32_t flags, void* stream, ct_tree** out) {
    if (!out) return fail(CT_ERR_ARG, "ct_build_residual: out is NULL");
    *out = nullptr;
    if (n <= 0 || n >= (1LL << 31)) return fail(CT_ERR_ARG, "ct_build_residual: n=%lld outside [1, 2^31)", (long long)n);
    if (m <= 0 || (m % 16) != 0) return fail(CT_ERR_UNSUPPORTED, "ct_build_residual: m=%d must be a positive multiple of 16", m);
    if (d <= 0 || d > 64) return fail(CT_ERR_ARG, "ct_build_residual: d=%d outside [1, 64]", d);
    if (!v || !p || !coords) return fail(CT_ERR_ARG, "ct_build_residual: NULL input pointer");
    if (kernel_type != CT_KERNEL_RBF && kernel_type != CT_KERNEL_MATERN52) kernel_type = CT_KERNEL_RBF;
    cudaStream_t st = (cudaStream_t)stream;
    keep_pool_memory();

    ct_tree* T = new (std::nothrow) ct_tree();
    if (!T) return fail(CT_ERR_NOMEM, "ct_build_residual: host allocation failed");
    T->n = n; T->m = m; T->d = d; T->var = variance; T->kernel_type = kernel_type;
    T->chunk = chunk > 0 ? chunk : 512; T->order_mode = order; T->seed = seed;
    T->slab_rows = (flags & CT_BUILD_QUERY_SLAB) ? 4096 : 0;

    // inverse lengthscales exactly as ResidualMetric::new (src/metric.rs:93-101)
    float inv_ls[64];
    float fallback = (lengthscale && n_lengthscale > 0) ? lengthscale[0] : 1.0f;
    for (int i = 0; i < d; ++i) {
        float raw = (lengthscale && i < n_lengthscale) ? lengthscale[i] : fallback;
        float safe = fabsf(raw) < 1e-6f ? 1e-6f : raw;
        inv_ls[i] = 1.0f / safe;
        T->inv_ls_host64[i] = 1.0 / (double)safe;
    }
    int rc = T->alloc_metric();
    if (rc != CT_OK) { const char* msg = T->err; int r = fail(rc, "ct_build_residual: %s", msg); delete T; return r; }
    cudaError_t e = cudaMemcpyAsync(T->inv_ls, inv_ls, sizeof(float) * d, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->vnat, v, sizeof(float) * (size_t)n * m, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(T->coords_raw, coords, sizeof(float) * (size_t)n * d, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess)
        e = ct::launch_metric_setup(v, p, coords, n, m, d, T->inv_ls, T->vperm, T->xs, T->norms, T->p, st);
    if (e == cudaSuccess && !(flags & CT_BUILD_METRIC_ONLY)) {
        rc = T->build_tree(v, coords, st);
        if (rc != CT_OK) { int r = fail(rc, "ct_build_residual: tree build: %s", T->err); delete T; return r; }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { int r = cuda_fail(e, "ct_build_residual"); delete T; return r; }
    *out = T;
    return CT_OK;
}

int ct_tree_subset(const ct_tree* B, const int64_t* rows, int64_t n_keep, void* stream, ct_tree** out) {
    if (!out) return fail(CT_ERR_ARG, "ct_tree_subset: out is NULL");
    *out = nullptr;
    if (!B) return fail(CT_ERR_ARG, "ct_tree_subset: base tree is NULL");
    if (n_keep <= 0) return fail(CT_ERR_ARG, "ct_tree_subset: n_keep must be positive");
    if (!rows) return fail(CT_ERR_ARG, "ct_tree_subset: rows is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const long long m = B->m, d = B->d;
    float *v = nullptr, *p = nullptr, *c = nullptr;
    int* bad = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&v, sizeof(float) * n_keep * m, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&p, sizeof(float) * n_keep, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&c, sizeof(float) * n_keep * d, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&bad, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
    int hbad = 0;
    if (e == cudaSuccess) {
        check_rows_kernel<<<(unsigned)((n_keep + 255) / 256), 256, 0, st>>>(rows, n_keep, B->n, bad);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    int rc = CT_OK;
    if (e == cudaSuccess && hbad) rc = fail(CT_ERR_ARG, "ct_tree_subset: rows must be ascending ids in [0, %lld)", (long long)B->n);
    if (e == cudaSuccess && rc == CT_OK) {
        gather_f32_rows_kernel<<<152 * 8, 256, 0, st>>>(B->vnat, rows, n_keep, (int)m, v);
        gather_f32_rows_kernel<<<(unsigned)((n_keep + 255) / 256), 256, 0, st>>>(B->p, rows, n_keep, 1, p);
        gather_f32_rows_kernel<<<(unsigned)((n_keep * d + 255) / 256), 256, 0, st>>>(B->coords_raw, rows, n_keep, (int)d, c);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess && rc == CT_OK) {
        // the base's lengthscales, recovered exactly from their inverses
        float ls[64];
        for (int i = 0; i < d; ++i) ls[i] = (float)(1.0 / B->inv_ls_host64[i]);
        const int flags = (B->has_tree ? 0 : CT_BUILD_METRIC_ONLY) | (B->slab_rows > 0 ? CT_BUILD_QUERY_SLAB : 0);
        rc = ct_build_residual(v, p, c, n_keep, (int32_t)m, (int32_t)d, B->var, ls, (int32_t)d, B->kernel_type,
                               B->chunk, B->order_mode, B->seed, flags, stream, out);
    }
    cudaFreeAsync(v, st); cudaFreeAsync(p, st); cudaFreeAsync(c, st); cudaFreeAsync(bad, st);
    if (e != cudaSuccess) return cuda_fail(e, "ct_tree_subset");
    return rc;
}

int ct_tree_extend(const ct_tree* B, const float* v, const float* p, const float* coords, int64_t n_new, void* stream,
                   ct_tree** out) {
    if (!out) return fail(CT_ERR_ARG, "ct_tree_extend: out is NULL");
    *out = nullptr;
    if (!B) return fail(CT_ERR_ARG, "ct_tree_extend: base tree is NULL");
    if (n_new < 0) return fail(CT_ERR_ARG, "ct_tree_extend: n_new < 0");
    if (n_new > 0 && (!v || !p || !coords)) return fail(CT_ERR_ARG, "ct_tree_extend: NULL input pointer");
    if (B->n + n_new > INT32_MAX) return fail(CT_ERR_UNSUPPORTED, "ct_tree_extend: more than 2^31 - 1 rows");
    cudaStream_t st = (cudaStream_t)stream;
    keep_pool_memory();
    ct_tree* T = new (std::nothrow) ct_tree();
    if (!T) return fail(CT_ERR_NOMEM, "ct_tree_extend: host allocation failed");
    const long long nb = B->n, m = B->m, d = B->d;
    T->n = nb + n_new; T->m = B->m; T->d = B->d; T->var = B->var; T->kernel_type = B->kernel_type;
    T->chunk = B->chunk; T->order_mode = B->order_mode; T->seed = B->seed; T->slab_rows = B->slab_rows;
    for (int i = 0; i < 64; ++i) T->inv_ls_host64[i] = B->inv_ls_host64[i];
    int rc = T->alloc_metric();
    if (rc != CT_OK) { const char* msg = T->err; int r = fail(rc, "ct_tree_extend: %s", msg); delete T; return r; }
    // the base's rows and their derived data are copied on the device; only the new rows
    // go through the metric setup
    cudaError_t e = cudaMemcpyAsync(T->inv_ls, B->inv_ls, sizeof(float) * 64, cudaMemcpyDeviceToDevice, st);
    auto D2D = [&](void* dst, const void* src, size_t bytes) {
        if (e == cudaSuccess && bytes) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, st);
    };
    D2D(T->vnat, B->vnat, sizeof(float) * nb * m);
    D2D(T->coords_raw, B->coords_raw, sizeof(float) * nb * d);
    D2D(T->vperm, B->vperm, sizeof(float) * nb * m);
    D2D(T->xs, B->xs, sizeof(float) * nb * d);
    D2D(T->norms, B->norms, sizeof(float) * nb);
    D2D(T->p, B->p, sizeof(float) * nb);
    D2D(T->vnat + nb * m, v, sizeof(float) * n_new * m);
    D2D(T->coords_raw + nb * d, coords, sizeof(float) * n_new * d);
    if (e == cudaSuccess)
        e = ct::launch_metric_setup(v, p, coords, n_new, (int)m, (int)d, T->inv_ls, T->vperm + nb * m, T->xs + nb * d,
                                    T->norms + nb, T->p + nb, st);
    if (e == cudaSuccess && B->has_tree) {
        rc = T->grow_tree(B, st);
        if (rc != CT_OK) { int r = fail(rc, "ct_tree_extend: tree: %s", T->err); delete T; return r; }
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { int r = cuda_fail(e, "ct_tree_extend"); delete T; return r; }
    *out = T;
    return CT_OK;
}

int ct_knn_residual(ct_tree* T, const int64_t* q_ids, int64_t nq, int32_t k, int32_t predecessor, int32_t form,
                    int64_t* out_idx, float* out_dist, ct_stats* stats, void* stream) {
    if (!T) return fail(CT_ERR_ARG, "ct_knn_residual: tree is NULL");
    if (nq < 0) return fail(CT_ERR_ARG, "ct_knn_residual: nq < 0");
    if (k <= 0) return fail(CT_ERR_ARG, "ct_knn_residual: k=%d must be positive", k);
    if (k > 128) return fail(CT_ERR_UNSUPPORTED, "ct_knn_residual: k=%d above the supported maximum 128", k);
    if (nq == 0) return CT_OK;
    if (!q_ids || !out_idx || !out_dist) return fail(CT_ERR_ARG, "ct_knn_residual: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    if (stats) memset(stats, 0, sizeof(*stats));
    switch (form) {
        case CT_FORM_DENSE: {
            int dev = 0;
            CT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
            int smem_optin = 0;
            CT_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev), "smem attr");
            int qt = ct::brute_pick_qt(T->m, T->d, k, (size_t)smem_optin);
            if (qt == 0) return fail(CT_ERR_UNSUPPORTED, "ct_knn_residual: m=%d, k=%d exceed shared memory", T->m, k);
            ct::BruteParams P;
            P.vperm = T->vperm; P.xs = T->xs; P.norms = T->norms; P.p = T->p;
            P.qids = (const long long*)q_ids; P.n = T->n; P.nq = nq; P.m = T->m; P.d = T->d; P.k = k;
            P.kernel_type = T->kernel_type; P.predecessor = predecessor ? 1 : 0; P.var = T->var;
            P.out_idx = (long long*)out_idx; P.out_dist = out_dist;
            cudaEvent_t e0 = nullptr, e1 = nullptr;
            if (g_timing) {
                CT_CUDA(cudaEventCreate(&e0), "event");
                CT_CUDA(cudaEventCreate(&e1), "event");
                CT_CUDA(cudaEventRecord(e0, st), "event record");
            }
            CT_CUDA(ct::launch_brute_knn(P, qt, st), "dense kNN launch");
            if (g_timing) {
                float ms = 0.f;
                CT_CUDA(cudaEventRecord(e1, st), "event record");
                CT_CUDA(cudaEventSynchronize(e1), "event sync");
                CT_CUDA(cudaEventElapsedTime(&ms, e0, e1), "event time");
                cudaEventDestroy(e0); cudaEventDestroy(e1);
                if (stats) { stats->device_ms = ms; stats->screen_ms = ms; }
            }
            if (stats) {
                stats->kernel_launches = 1;
                stats->distance_evals = predecessor ? -1 : nq * T->n;
            }
            return CT_OK;
        }
        case CT_FORM_TREE:
            return T->knn_tree(q_ids, nq, k, predecessor, out_idx, out_dist, stats, st)
                       ? fail(CT_ERR_STATE, "ct_knn_residual: tree form: %s", T->err)
                       : CT_OK;
        case CT_FORM_SCREENED:
            return T->knn_screened(q_ids, nq, k, predecessor, out_idx, out_dist, stats, st)
                       ? fail(CT_ERR_STATE, "ct_knn_residual: screened form: %s", T->err)
                       : CT_OK;
        default:
            return fail(CT_ERR_ARG, "ct_knn_residual: unknown form %d", form);
    }
}

int ct_tree_arrays(const ct_tree* T, int64_t* parents, int32_t* levels, float* si, int64_t* node_to_dataset,
                   int64_t* subtree_min, void* stream) {
    if (!T) return fail(CT_ERR_ARG, "ct_tree_arrays: tree is NULL");
    if (!T->has_tree) return fail(CT_ERR_STATE, "ct_tree_arrays: tree was built with CT_BUILD_METRIC_ONLY");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)T->n;
    if (parents) CT_CUDA(cudaMemcpyAsync(parents, T->parents, n * 8, cudaMemcpyDeviceToDevice, st), "copy parents");
    if (levels) CT_CUDA(cudaMemcpyAsync(levels, T->levels, n * 4, cudaMemcpyDeviceToDevice, st), "copy levels");
    if (si) CT_CUDA(cudaMemcpyAsync(si, T->si, n * 4, cudaMemcpyDeviceToDevice, st), "copy si");
    if (node_to_dataset) CT_CUDA(cudaMemcpyAsync(node_to_dataset, T->order, n * 8, cudaMemcpyDeviceToDevice, st), "copy order");
    if (subtree_min) CT_CUDA(cudaMemcpyAsync(subtree_min, T->sub_min, n * 8, cudaMemcpyDeviceToDevice, st), "copy subtree_min");
    return CT_OK;
}

int ct_debug_screen_dots(ct_tree* T, const int32_t* rows_a, const int32_t* rows_b, float* out, void* stream) {
    if (!T || !rows_a || !rows_b || !out) return fail(CT_ERR_ARG, "ct_debug_screen_dots: NULL argument");
    int rc = ct_screen_debug_dots(T, rows_a, rows_b, out, (cudaStream_t)stream);
    return rc ? fail(rc, "ct_debug_screen_dots: %s", T->err) : CT_OK;
}

int ct_knn_euclidean(const float* points, int64_t n, int32_t d, const float* queries, int64_t nq, int32_t k,
                     int32_t predecessor, int64_t* out_idx, float* out_dist, void* stream) {
    if (n < 0 || nq < 0) return fail(CT_ERR_ARG, "ct_knn_euclidean: negative size");
    if (k <= 0) return fail(CT_ERR_ARG, "ct_knn_euclidean: k=%d must be positive", k);
    if (k > ct::euclid_max_k()) return fail(CT_ERR_UNSUPPORTED, "ct_knn_euclidean: k=%d above %d", k, ct::euclid_max_k());
    if (d <= 0 || d > ct::euclid_max_d()) return fail(CT_ERR_UNSUPPORTED, "ct_knn_euclidean: d=%d outside [1, %d]", d, ct::euclid_max_d());
    if (nq == 0) return CT_OK;
    if (!points || !queries || !out_idx || !out_dist) return fail(CT_ERR_ARG, "ct_knn_euclidean: NULL pointer");
    CT_CUDA(ct::launch_euclid_knn(points, n, d, queries, nq, k, predecessor ? 1 : 0, (long long*)out_idx, out_dist,
                                  (cudaStream_t)stream), "euclidean kNN launch");
    return CT_OK;
}

int ct_knn_residual_dense_noalloc(const float* v, const float* p, const float* coords, int64_t n, int32_t m,
                                  int32_t d, float variance, const float* lengthscale, int32_t n_lengthscale,
                                  int32_t kernel_type, const int64_t* q_ids, int64_t nq, int32_t k,
                                  int32_t predecessor, int64_t* out_idx, float* out_dist, void* stream) {
    if (n <= 0 || n >= (1LL << 31)) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: n=%lld outside [1, 2^31)", (long long)n);
    if (m <= 0 || (m % 16) != 0) return fail(CT_ERR_UNSUPPORTED, "ct_knn_residual_dense_noalloc: m=%d must be a positive multiple of 16", m);
    if (d <= 0 || d > 64) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: d=%d outside [1, 64]", d);
    if (k <= 0 || k > 128) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: k=%d outside [1, 128]", k);
    if (nq < 0) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: nq < 0");
    if (!v || !p || !coords) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: NULL input pointer");
    if (nq > 0 && (!q_ids || !out_idx || !out_dist)) return fail(CT_ERR_ARG, "ct_knn_residual_dense_noalloc: NULL pointer");
    char msg[400];
    int rc = ct_noalloc_dense_impl(v, p, coords, n, m, d, variance, lengthscale, n_lengthscale, kernel_type,
                                   (const long long*)q_ids, nq, k, predecessor, (long long*)out_idx, out_dist,
                                   (cudaStream_t)stream, msg, sizeof(msg));
    return rc == CT_OK ? CT_OK : fail(rc, "ct_knn_residual_dense_noalloc: %s", msg);
}

namespace {
__global__ void widen_order_kernel(const int* __restrict__ in, long long n, long long* __restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}
__global__ void iota_kernel(long long n, long long* __restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = i;
}
}  // namespace

int ct_batch_order(const float* coords, int64_t n, int32_t d, int32_t mode, int64_t* out_perm, void* stream) {
    if (n < 0 || n >= (1LL << 31)) return fail(CT_ERR_ARG, "ct_batch_order: n=%lld outside [0, 2^31)", (long long)n);
    if (d <= 0 || d > 64) return fail(CT_ERR_ARG, "ct_batch_order: d=%d outside [1, 64]", d);
    if (mode != CT_ORDER_NATURAL && mode != CT_ORDER_HILBERT && mode != CT_ORDER_MORTON)
        return fail(CT_ERR_ARG, "ct_batch_order: unknown mode %d", mode);
    if (n == 0) return CT_OK;
    if (!coords || !out_perm) return fail(CT_ERR_ARG, "ct_batch_order: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((n + 255) / 256);
    // the reference's Morton order is defined for D = 3 only and is the identity otherwise
    if (mode == CT_ORDER_NATURAL || (mode == CT_ORDER_MORTON && d != 3)) {
        iota_kernel<<<grid, 256, 0, st>>>(n, (long long*)out_perm);
        CT_CUDA(cudaGetLastError(), "ct_batch_order");
        return CT_OK;
    }
    int* order32 = nullptr;
    CT_CUDA(cudaMallocAsync((void**)&order32, sizeof(int) * (size_t)n, st), "ct_batch_order allocation");
    cudaError_t e = ct::compute_order(coords, n, d, mode == CT_ORDER_MORTON ? 2 : 1, order32, st);
    if (e == cudaSuccess) {
        widen_order_kernel<<<grid, 256, 0, st>>>(order32, n, (long long*)out_perm);
        e = cudaGetLastError();
    }
    cudaFreeAsync(order32, st);
    if (e != cudaSuccess) return cuda_fail(e, "ct_batch_order");
    return CT_OK;
}

int ct_luby_mis(const int64_t* indptr, const int64_t* indices, int64_t n, uint64_t seed, int8_t* out_sel,
                int32_t* iterations, void* stream) {
    if (iterations) *iterations = 0;
    if (n < 0) return fail(CT_ERR_ARG, "ct_luby_mis: n < 0");
    if (n == 0) return CT_OK;
    if (!indptr || !out_sel) return fail(CT_ERR_ARG, "ct_luby_mis: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    bool valid = false;
    CT_CUDA(ct::csr_graph_valid((const long long*)indptr, (const long long*)indices, n, &valid, st), "ct_luby_mis");
    if (!valid)
        return fail(CT_ERR_ARG, "ct_luby_mis: indptr must start at 0 and not decrease, indices must lie in [0, n)");
    int it = 0;
    CT_CUDA(ct::luby_mis_csr((const long long*)indptr, (const long long*)indices, n, seed, (signed char*)out_sel, &it,
                             st),
            "ct_luby_mis");
    if (iterations) *iterations = it;
    return CT_OK;
}

int ct_tree_inputs(const ct_tree* T, float* v, float* p, float* coords, void* stream) {
    if (!T) return fail(CT_ERR_ARG, "ct_tree_inputs: tree is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t n = (size_t)T->n;
    if (v) CT_CUDA(cudaMemcpyAsync(v, T->vnat, n * T->m * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy v");
    if (p) CT_CUDA(cudaMemcpyAsync(p, T->p, n * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy p");
    if (coords) CT_CUDA(cudaMemcpyAsync(coords, T->coords_raw, n * T->d * sizeof(float), cudaMemcpyDeviceToDevice, st), "copy coords");
    return CT_OK;
}

int ct_prepare_screened(ct_tree* T, void* stream) {
    if (!T) return fail(CT_ERR_ARG, "ct_prepare_screened: tree is NULL");
    int rc = T->prepare_screened((cudaStream_t)stream);
    return rc ? fail(rc, "ct_prepare_screened: %s", T->err) : CT_OK;
}

int ct_tree_device_bytes(const ct_tree* T, int64_t* bytes) {
    if (!T || !bytes) return fail(CT_ERR_ARG, "ct_tree_device_bytes: NULL argument");
    *bytes = T->device_bytes();
    return CT_OK;
}

int ct_tree_build_info(const ct_tree* T, int64_t* groups, int64_t* conflict_edges, int64_t* selected,
                       int64_t* side_rows, int64_t* roots, double* build_ms) {
    if (!T) return fail(CT_ERR_ARG, "ct_tree_build_info: tree is NULL");
    if (!T->has_tree) return fail(CT_ERR_STATE, "ct_tree_build_info: tree was built with CT_BUILD_METRIC_ONLY");
    if (groups) *groups = T->build_groups;
    if (conflict_edges) *conflict_edges = T->build_conflict_edges;
    if (selected) *selected = T->build_selected;
    if (side_rows) *side_rows = T->n_side;
    if (roots) *roots = T->n_roots;
    if (build_ms) *build_ms = T->build_ms;
    return CT_OK;
}

int ct_tree_shape(const ct_tree* T, int64_t* n, int32_t* m, int32_t* d) {
    if (!T) return fail(CT_ERR_ARG, "ct_tree_shape: tree is NULL");
    if (n) *n = T->n;
    if (m) *m = T->m;
    if (d) *d = T->d;
    return CT_OK;
}

int ct_free(ct_tree* T) {
    if (!T) return CT_OK;
    delete T;
    return CT_OK;
}

int ct_knn_residual_points(ct_tree* T, const float* qv, const float* qp, const float* qcoords, int64_t nq, int32_t k,
                           int32_t form, int64_t* out_idx, float* out_dist, ct_stats* stats, void* stream) {
    // one cached batch object per calling thread and device
    thread_local ct_batch* tb = nullptr;
    thread_local int tb_dev = -1;
    if (!T) return fail(CT_ERR_ARG, "ct_knn_residual_points: tree is NULL");
    if (nq < 0) return fail(CT_ERR_ARG, "ct_knn_residual_points: nq < 0");
    if (k <= 0) return fail(CT_ERR_ARG, "ct_knn_residual_points: k=%d must be positive", k);
    if (k > 128) return fail(CT_ERR_UNSUPPORTED, "ct_knn_residual_points: k=%d above the supported maximum 128", k);
    if (nq > 0 && (!qv || !qp || !qcoords || !out_idx || !out_dist))
        return fail(CT_ERR_ARG, "ct_knn_residual_points: NULL pointer");
    if (form == CT_FORM_SCREENED) {
        if (stats) memset(stats, 0, sizeof(*stats));
        return T->knn_screened_points(qv, qp, qcoords, nq, k, out_idx, out_dist, stats, (cudaStream_t)stream)
                   ? fail(CT_ERR_STATE, "ct_knn_residual_points: screened form: %s", T->err)
                   : CT_OK;
    }
    if (form != CT_FORM_DENSE) return fail(CT_ERR_ARG, "ct_knn_residual_points: form %d (dense or screened)", form);
    int dev = 0;
    CT_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (tb && tb_dev != dev) { ct_batch_free(tb); tb = nullptr; }
    if (!tb) {
        int rc = ct_batch_create(&tb);
        if (rc != CT_OK) return rc;
        tb_dev = dev;
    }
    ct_batch_clear(tb);
    int rc = ct_batch_add_points(tb, T, qv, qp, qcoords, nq, k, out_idx, out_dist);
    if (rc == CT_OK) rc = ct_batch_run(tb, 0, stats, stream);
    ct_batch_clear(tb);
    return rc;
}

int ct_vfactor_create(const double* z, int32_t m, int32_t d, int32_t kernel_type, double variance,
                      double lengthscale, void* stream, ct_vfactor** out) {
    if (!out) return fail(CT_ERR_ARG, "ct_vfactor_create: out is NULL");
    *out = nullptr;
    if (m <= 0 || m > 16384) return fail(CT_ERR_ARG, "ct_vfactor_create: m=%d outside [1, 16384]", m);
    if (d <= 0 || d > 64) return fail(CT_ERR_ARG, "ct_vfactor_create: d=%d outside [1, 64]", d);
    if (!z) return fail(CT_ERR_ARG, "ct_vfactor_create: z is NULL");
    if (kernel_type != CT_KERNEL_RBF && kernel_type != CT_KERNEL_MATERN52) kernel_type = CT_KERNEL_RBF;
    cudaStream_t st = (cudaStream_t)stream;
    keep_pool_memory();
    ct_vfactor* F = new (std::nothrow) ct_vfactor();
    if (!F) return fail(CT_ERR_NOMEM, "ct_vfactor_create: host allocation failed");
    F->m = m; F->d = d; F->kernel_type = kernel_type; F->variance = variance; F->lengthscale = lengthscale;
    cudaGetDevice(&F->device);
    const size_t mm = (size_t)m * m;
    int* status = nullptr;
    int hs = 0;
    cudaError_t e = cudaMalloc((void**)&F->z, sizeof(double) * (size_t)m * d);
    if (e == cudaSuccess) e = cudaMalloc((void**)&F->L, sizeof(double) * mm);
    if (e == cudaSuccess) e = cudaMalloc((void**)&F->Li, sizeof(double) * mm);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&status, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(F->z, z, sizeof(double) * (size_t)m * d, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = ct::vmatrix_factor(F->z, m, d, kernel_type, variance, lengthscale, F->L, F->Li, status, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (status) cudaFreeAsync(status, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) { int r = cuda_fail(e, "ct_vfactor_create"); ct_vfactor_free(F); return r; }
    if (hs) {
        ct_vfactor_free(F);
        return fail(CT_ERR_ARG, "ct_vfactor_create: K(Z,Z) + jitter is not positive definite");
    }
    *out = F;
    return CT_OK;
}

int ct_vfactor_embed(ct_vfactor* F, const double* x, int64_t n, float* v_out, float* p_out, void* stream) {
    if (!F) return fail(CT_ERR_ARG, "ct_vfactor_embed: factor is NULL");
    if (n < 0) return fail(CT_ERR_ARG, "ct_vfactor_embed: n < 0");
    if (n == 0) return CT_OK;
    if (!x || !v_out || !p_out) return fail(CT_ERR_ARG, "ct_vfactor_embed: NULL pointer");
    cudaStream_t st = (cudaStream_t)stream;
    // scratch is stream-ordered and private to the call: embeds on one factor may
    // run concurrently on different streams (the factor itself is read-only)
    const long long chunk = ct::vmatrix_chunk_rows(n, F->m);
    double *kc = nullptr, *vc = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&kc, sizeof(double) * (size_t)chunk * F->m, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&vc, sizeof(double) * (size_t)chunk * F->m, st);
    if (e == cudaSuccess)
        e = ct::vmatrix_embed(x, n, F->d, F->z, F->m, F->kernel_type, F->variance, F->lengthscale, F->Li, kc, vc,
                              chunk, v_out, p_out, st, nullptr, g_cta_budget);
    if (kc) cudaFreeAsync(kc, st);
    if (vc) cudaFreeAsync(vc, st);
    if (e != cudaSuccess) return cuda_fail(e, "ct_vfactor_embed");
    return CT_OK;
}

int ct_vfactor_chol(const ct_vfactor* F, double* l_out, void* stream) {
    if (!F || !l_out) return fail(CT_ERR_ARG, "ct_vfactor_chol: NULL argument");
    CT_CUDA(cudaMemcpyAsync(l_out, F->L, sizeof(double) * (size_t)F->m * F->m, cudaMemcpyDeviceToDevice,
                            (cudaStream_t)stream),
            "ct_vfactor_chol copy");
    return CT_OK;
}

int ct_vfactor_free(ct_vfactor* F) {
    if (!F) return CT_OK;
    if (F->z) cudaFree(F->z);
    if (F->L) cudaFree(F->L);
    if (F->Li) cudaFree(F->Li);
    delete F;
    return CT_OK;
}

}  // extern "C"
