// ct_batch.cu — batching form: many trees and query sets of uneven N, D and k
// in ONE persistent launch that drains a device work queue.
//
// Work item = (problem, query tile, candidate chunk).  A problem is one query
// set against one resident tree: dataset ids (the reference's
// knn_query_residual, src/lib.rs:370-507) or new points (V rows from
// ct_vfactor_embed).  Items are numbered problem by problem (problems sorted by
// per-tile work, heaviest first; tiles of a problem in reverse so the long
// predecessor tiles start early); persistent CTAs take the next item with one
// atomicAdd on a device counter.  Every item runs dense::run_tile, the same
// code and arithmetic as the single-tree dense kernel, so each problem's
// result is bit-identical to running it alone.
//
// When a problem has fewer tiles than the GPU has slots, its candidate range is
// split into chunks; each chunk writes an exact partial top-k, and the CTA that
// completes a tile's last chunk (a per-tile atomic counter; no CTA ever waits
// for another) merges the partial lists with a warp-wide k-way merge.  The
// counters return themselves to zero (the merging CTA clears its tile's
// counter, the last CTA to leave clears the queue counter), so a launch needs
// no memset and the launch sequence can be replayed as a CUDA graph:
// [copy descriptors from pinned host memory, persistent kernel].
//
// The autotuner (ct_batch_autotune) times the candidate launch shapes —
// queries per CTA tile (QT = 64 / 32 / 16), CTAs per SM, and the candidate split
// target (work items per SM slot) — on the batch itself and keeps the fastest.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <new>
#include <vector>

#include "../../include/covertree_cuda.h"
#include "ct_common.cuh"
#include "ct_dense.cuh"
#include "ct_internal.h"
#include "ct_tree.h"

namespace ct {
namespace batch {

struct Problem {
    dense::Tile base;     // q0 / cbeg / cend / out_* are set per item
    long long tiles;      // query tiles of QT
    long long chunk;      // candidates per chunk (multiple of dense::kCT)
    long long item_base;  // first work item of the problem
    long long* part_idx;  // [nq][split][k] partial lists (split > 1)
    float* part_dist;
    int* tile_done;       // [tiles] chunk completion counters (split > 1)
    int split;            // candidate chunks per tile (1..kMaxSplit)
    int pad_;
};

struct Header {
    long long total_items;
    int nprob;
    int qt;
};

constexpr size_t kHeaderBytes = 64;

// Merge a tile's `split` sorted partial lists per query into the final top-k.
// One warp per query; lane l owns lists l, l+32, l+64 and l+96 and offers the
// smallest of their heads to a warp-wide (dist, idx) minimum.
constexpr int kMaxSplit = 128;
__device__ void merge_partials(const Problem& B, long long tile, int QT) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = B.base.k, S = B.split;
    const float kInf = __int_as_float(0x7f800000);
    for (int qi = warp; qi < QT; qi += dense::kThreads / 32) {
        const long long g = tile * QT + qi;
        if (g >= B.base.nq) continue;
        int pos[4] = {0, 0, 0, 0};
        float hd[4];
        long long hi[4];
        auto load = [&](int h) {
            const int list = lane + 32 * h;
            hd[h] = kInf;
            hi[h] = LLONG_MAX;
            if (list < S && pos[h] < k) {
                const long long off = (g * S + list) * k + pos[h];
                const long long i = __ldcg(B.part_idx + off);
                if (i >= 0) { hi[h] = i; hd[h] = __ldcg(B.part_dist + off); }
            }
        };
#pragma unroll
        for (int h = 0; h < 4; ++h) load(h);
        for (int j = 0; j < k; ++j) {
            int bh = 0;
#pragma unroll
            for (int h = 1; h < 4; ++h)
                if (nb_less(hd[h], hi[h], hd[bh], hi[bh])) bh = h;
            float bd = hd[bh];
            long long bi = hi[bh];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const float od = __shfl_xor_sync(0xffffffffu, bd, o);
                const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (nb_less(od, oi, bd, bi)) { bd = od; bi = oi; }
            }
            if (lane == 0) {
                const bool pad = bi == LLONG_MAX;
                B.base.out_idx[g * k + j] = pad ? -1LL : bi;
                B.base.out_dist[g * k + j] = pad ? CT_FLT_MAX : bd;
            }
            if (bi != LLONG_MAX && hi[bh] == bi) { ++pos[bh]; load(bh); }
        }
    }
}

template <int QT, int MINB>
__global__ void __launch_bounds__(dense::kThreads, MINB)
    batch_kernel(const unsigned char* __restrict__ desc, unsigned long long* __restrict__ ctr) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ dense::Tile sJ;
    __shared__ long long s_item;
    __shared__ int s_prob, s_last;
    const Header* H = (const Header*)desc;
    const Problem* probs = (const Problem*)(desc + kHeaderBytes);
    const long long total = H->total_items;
    const int np = H->nprob;
    for (;;) {
        if (threadIdx.x == 0) {
            const long long it = (long long)atomicAdd(&ctr[0], 1ull);
            s_item = it;
            if (it < total) {
                int lo = 0, hi = np - 1;  // last problem with item_base <= it
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (probs[mid].item_base <= it) lo = mid; else hi = mid - 1;
                }
                s_prob = lo;
                const Problem& B = probs[lo];
                const long long local = it - B.item_base;
                const long long tile = B.tiles - 1 - local / B.split;
                const int chunk = (int)(local % B.split);
                dense::Tile J = B.base;
                J.q0 = tile * QT;
                J.cbeg = (long long)chunk * B.chunk;
                J.cend = J.cbeg + B.chunk < J.n ? J.cbeg + B.chunk : J.n;
                if (B.split > 1) {
                    J.out_idx = B.part_idx + (long long)chunk * J.k;
                    J.out_dist = B.part_dist + (long long)chunk * J.k;
                    J.out_stride = (long long)B.split * J.k;
                } else {
                    J.out_stride = J.k;
                }
                sJ = J;
            }
        }
        __syncthreads();
        const long long it = s_item;
        if (it >= total) break;
        dense::run_tile<QT>(sJ, smem_raw);
        const Problem& B = probs[s_prob];
        if (B.split > 1) {
            __threadfence();
            __syncthreads();
            const long long tile = sJ.q0 / QT;
            if (threadIdx.x == 0) {
                const int prev = atomicAdd(&B.tile_done[tile], 1);
                s_last = prev == B.split - 1;
            }
            __syncthreads();
            if (s_last) {
                __threadfence();
                merge_partials(B, tile, QT);
                if (threadIdx.x == 0) B.tile_done[tile] = 0;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        // every CTA has made its last queue access before it counts itself out
        const unsigned long long out = atomicAdd(&ctr[1], 1ull);
        if (out == gridDim.x - 1) {
            ctr[0] = 0ull;
            ctr[1] = 0ull;
            __threadfence();
        }
    }
}

typedef void (*KernelFn)(const unsigned char*, unsigned long long*);

struct Shape {
    int qt, cps;
};

KernelFn kernel_for(int qt, int cps) {
    if (qt == 64) return batch_kernel<64, 1>;
    if (qt == 32) return batch_kernel<32, 1>;
    return cps >= 2 ? batch_kernel<16, 2> : batch_kernel<16, 1>;
}

}  // namespace batch
}  // namespace ct

using namespace ct;
using namespace ct::batch;

struct BatchReq {
    ct_tree* tree;
    const int64_t* qids;
    const float* qv;
    const float* qp;
    const float* qcoords;
    long long nq;
    int k, predecessor;
    int64_t* out_idx;
    float* out_dist;
};

struct ct_batch {
    int device = 0, num_sms = 0;
    size_t smem_optin = 0, smem_per_sm = 0;
    std::vector<BatchReq> reqs;
    int cfg_qt = 0, cfg_cps = 0, cfg_ips = 0;  // 0 = automatic
    int res_m = 16, res_d = 1, res_k = 1;      // shared memory is sized for at least these
    // device and pinned buffers
    unsigned char* d_desc = nullptr;
    unsigned char* h_desc = nullptr;
    std::vector<unsigned char*> old_pinned;  // replaced pinned descriptor buffers, freed with the batch
    size_t desc_cap = 0;
    unsigned long long* d_ctr = nullptr;
    int* d_done = nullptr;
    size_t done_cap = 0;  // ints
    unsigned char* d_part = nullptr;
    size_t part_cap = 0;  // bytes
    // graph of [descriptor copy, kernel]
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int g_qt = 0, g_cps = 0, g_grid = 0;
    size_t g_smem = 0, g_cap = 0;
    cudaEvent_t staged = nullptr;
    bool staged_pending = false;
    // last run
    long long last_items = 0, last_pairs = 0;
    int last_qt = 0, last_cps = 0, last_ips = 0, last_grid = 0;
    char err[256] = "";

    int set_err(int code, const char* msg) {
        snprintf(err, sizeof(err), "%s", msg);
        return code;
    }
    int cuda_err(cudaError_t e, const char* where) {
        snprintf(err, sizeof(err), "%s: %s", where, cudaGetErrorString(e));
        return CT_ERR_CUDA;
    }
    ~ct_batch() {
        if (staged) cudaEventDestroy(staged);
        if (gexec) cudaGraphExecDestroy(gexec);
        if (cap_stream) cudaStreamDestroy(cap_stream);
        if (d_desc) cudaFree(d_desc);
        if (h_desc) cudaFreeHost(h_desc);
        for (unsigned char* h : old_pinned) cudaFreeHost(h);
        if (d_ctr) cudaFree(d_ctr);
        if (d_done) cudaFree(d_done);
        if (d_part) cudaFree(d_part);
    }
};

namespace {

int batch_init(ct_batch* B) {
    cudaError_t e = cudaGetDevice(&B->device);
    int v = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&B->num_sms, cudaDevAttrMultiProcessorCount, B->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, B->device);
    B->smem_optin = (size_t)v;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerMultiprocessor, B->device);
    B->smem_per_sm = (size_t)v;
    if (e == cudaSuccess) e = cudaMalloc((void**)&B->d_ctr, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(B->d_ctr, 0, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&B->cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B->staged, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    return e == cudaSuccess ? CT_OK : B->cuda_err(e, "ct_batch_create");
}

// static shared memory of the batch kernel (sJ and the item scalars)
constexpr size_t kStaticSmem = sizeof(dense::Tile) + 64;

size_t smem_for(const ct_batch* B, int qt) {
    int m = B->res_m, d = B->res_d, k = B->res_k;
    for (const BatchReq& r : B->reqs) {
        m = std::max(m, r.tree->m);
        d = std::max(d, r.tree->d);
        k = std::max(k, r.k);
    }
    return dense::layout(qt, m, d, k).total;
}

bool shape_fits(const ct_batch* B, int qt, int cps) {
    const size_t s = smem_for(B, qt);
    if (s + kStaticSmem > B->smem_optin) return false;
    if (cps >= 2 && (qt != 16 || 2 * (s + kStaticSmem + 1024) > B->smem_per_sm)) return false;
    return true;
}

struct Plan {
    std::vector<Problem> probs;
    long long total_items = 0, pairs = 0;
    size_t part_bytes = 0, done_ints = 0;
};

// Order problems, choose each problem's candidate split and lay out its scratch.
void make_plan(const ct_batch* B, int qt, int cps, int ips, Plan& P) {
    const int nr = (int)B->reqs.size();
    std::vector<int> ord;
    std::vector<double> tile_work(nr, 0.0);
    double total_work = 0.0;
    long long total_tiles = 0;
    for (int i = 0; i < nr; ++i) {
        const BatchReq& r = B->reqs[i];
        if (r.nq <= 0) continue;
        const long long tiles = (r.nq + qt - 1) / qt;
        const double per_pair = (double)r.tree->m + 4.0 * r.tree->d + 16.0;
        tile_work[i] = (double)r.tree->n * (r.predecessor ? 0.5 : 1.0) * qt * per_pair;
        total_work += tile_work[i] * tiles;
        total_tiles += tiles;
        ord.push_back(i);
    }
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return tile_work[a] > tile_work[b]; });
    const double slots = (double)B->num_sms * cps;
    const double target_items = slots * ips;
    size_t part_off = 0, done_off = 0;
    long long item = 0;
    for (int i : ord) {
        const BatchReq& r = B->reqs[i];
        ct_tree* T = r.tree;
        Problem pr;
        memset(&pr, 0, sizeof(pr));
        dense::Tile& J = pr.base;
        J.vperm = T->vperm; J.xs = T->xs; J.norms = T->norms; J.p = T->p;
        J.n = T->n; J.m = T->m; J.d = T->d; J.k = r.k; J.kernel_type = T->kernel_type;
        J.predecessor = r.predecessor; J.var = T->var;
        J.qids = (const long long*)r.qids;
        J.qv = r.qv; J.qcoords = r.qcoords; J.qp = r.qp; J.inv_ls = T->inv_ls;
        J.nq = r.nq;
        J.out_idx = (long long*)r.out_idx; J.out_dist = r.out_dist; J.out_stride = r.k;
        pr.tiles = (r.nq + qt - 1) / qt;
        // split so that the batch has about target_items items, in proportion to work
        int split = 1;
        if ((double)total_tiles < target_items && total_work > 0) {
            const double want = target_items * (tile_work[i] * pr.tiles / total_work) / (double)pr.tiles;
            split = (int)std::min((double)kMaxSplit, std::max(1.0, want));
        }
        long long chunk = (T->n + split - 1) / split;
        chunk = ((chunk + dense::kCT - 1) / dense::kCT) * dense::kCT;
        if (chunk < dense::kCT) chunk = dense::kCT;
        split = (int)((T->n + chunk - 1) / chunk);
        pr.split = split;
        pr.chunk = chunk;
        pr.item_base = item;
        item += pr.tiles * split;
        if (split > 1) {
            const size_t entries = (size_t)r.nq * split * r.k;
            pr.part_idx = (long long*)(uintptr_t)part_off;  // offsets until the arena is known
            part_off += (entries * 8 + 255) & ~size_t(255);
            pr.part_dist = (float*)(uintptr_t)part_off;
            part_off += (entries * 4 + 255) & ~size_t(255);
            pr.tile_done = (int*)(uintptr_t)(done_off * sizeof(int));
            done_off += (size_t)pr.tiles;
        }
        P.pairs += (long long)((r.predecessor ? 0.5 : 1.0) * (double)r.nq * (double)T->n);
        P.probs.push_back(pr);
    }
    P.total_items = item;
    P.part_bytes = part_off;
    P.done_ints = done_off;
}

// Growth is stream-ordered: the old buffers are released on the run's stream after the
// previous run (its staging event), the new ones come from the stream-ordered allocator,
// so a growing batch never synchronises the device (a serving step would otherwise wait
// for every build and screened request in flight).  Old pinned descriptor buffers are kept
// until the batch is freed (freeing pinned memory synchronises).
int ensure_capacity(ct_batch* B, const Plan& P, cudaStream_t st) {
    cudaError_t e = cudaSuccess;
    const size_t need_desc = kHeaderBytes + sizeof(Problem) * std::max<size_t>(P.probs.size(), 1);
    const bool grow = need_desc > B->desc_cap || P.part_bytes > B->part_cap || P.done_ints > B->done_cap;
    if (grow && B->staged_pending) e = cudaStreamWaitEvent(st, B->staged, 0);
    if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: ordering a buffer growth");
    if (need_desc > B->desc_cap) {
        if (B->staged_pending) cudaEventSynchronize(B->staged);  // the pinned buffer's last copy
        B->staged_pending = false;
        size_t cap = std::max<size_t>(need_desc * 2, 16384);
        if (B->d_desc) cudaFreeAsync(B->d_desc, st);
        if (B->h_desc) B->old_pinned.push_back(B->h_desc);
        B->d_desc = nullptr; B->h_desc = nullptr; B->desc_cap = 0;
        e = cudaMallocAsync((void**)&B->d_desc, cap, st);
        if (e == cudaSuccess) e = cudaMallocHost((void**)&B->h_desc, cap);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: descriptor buffers");
        B->desc_cap = cap;
    }
    if (P.part_bytes > B->part_cap) {
        if (B->d_part) cudaFreeAsync(B->d_part, st);
        B->d_part = nullptr; B->part_cap = 0;
        const size_t cap = std::max<size_t>(P.part_bytes * 2, (size_t)1 << 20);
        e = cudaMallocAsync((void**)&B->d_part, cap, st);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: partial-list scratch");
        B->part_cap = cap;
    }
    if (P.done_ints > B->done_cap) {
        if (B->d_done) cudaFreeAsync(B->d_done, st);
        B->d_done = nullptr; B->done_cap = 0;
        const size_t cap = std::max<size_t>(P.done_ints * 2, 4096);
        e = cudaMallocAsync((void**)&B->d_done, cap * sizeof(int), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(B->d_done, 0, cap * sizeof(int), st);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: tile counters");
        B->done_cap = cap;
    }
    return CT_OK;
}

int run_shape(ct_batch* B, int qt, int cps, int ips, bool use_graph, cudaStream_t st) {
    Plan P;
    make_plan(B, qt, cps, ips, P);
    B->last_items = P.total_items;
    B->last_pairs = P.pairs;
    B->last_qt = qt; B->last_cps = cps; B->last_ips = ips;
    if (P.total_items == 0) return CT_OK;
    int rc = ensure_capacity(B, P, st);
    if (rc != CT_OK) return rc;
    for (Problem& pr : P.probs) {
        if (pr.split > 1) {
            pr.part_idx = (long long*)(B->d_part + (uintptr_t)pr.part_idx);
            pr.part_dist = (float*)(B->d_part + (uintptr_t)pr.part_dist);
            pr.tile_done = (int*)((unsigned char*)B->d_done + (uintptr_t)pr.tile_done);
        }
    }
    // the previous run's descriptor copy must have left the pinned buffer
    if (B->staged_pending) {
        cudaError_t e = cudaEventSynchronize(B->staged);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: staging event");
        B->staged_pending = false;
    }
    Header h;
    memset(&h, 0, sizeof(h));
    h.total_items = P.total_items;
    h.nprob = (int)P.probs.size();
    h.qt = qt;
    memcpy(B->h_desc, &h, sizeof(h));
    memcpy(B->h_desc + kHeaderBytes, P.probs.data(), sizeof(Problem) * P.probs.size());
    const size_t copy_bytes = kHeaderBytes + sizeof(Problem) * P.probs.size();

    const size_t smem = smem_for(B, qt);
    KernelFn fn = kernel_for(qt, cps);
    cudaError_t e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: shared-memory attribute");
    long long grid = (long long)B->num_sms * cps;
    // a graph keeps one grid for every batch (CTAs without items leave at once)
    if (!use_graph && grid > P.total_items) grid = P.total_items;
    B->last_grid = (int)grid;

    if (use_graph) {
        if (!B->gexec || B->g_qt != qt || B->g_cps != cps || B->g_grid != (int)grid || B->g_smem != smem ||
            B->g_cap != B->desc_cap) {
            if (B->gexec) { cudaGraphExecDestroy(B->gexec); B->gexec = nullptr; }
            cudaGraph_t g = nullptr;
            e = cudaStreamBeginCapture(B->cap_stream, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: begin capture");
            // the whole descriptor buffer is copied: the graph is reusable for any batch that fits
            cudaMemcpyAsync(B->d_desc, B->h_desc, B->desc_cap, cudaMemcpyHostToDevice, B->cap_stream);
            fn<<<(unsigned)grid, dense::kThreads, smem, B->cap_stream>>>(B->d_desc, B->d_ctr);
            e = cudaStreamEndCapture(B->cap_stream, &g);
            if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: end capture");
            e = cudaGraphInstantiate(&B->gexec, g, 0);
            cudaGraphDestroy(g);
            if (e != cudaSuccess) { B->gexec = nullptr; return B->cuda_err(e, "ct_batch: graph instantiate"); }
            B->g_qt = qt; B->g_cps = cps; B->g_grid = (int)grid; B->g_smem = smem; B->g_cap = B->desc_cap;
        }
        e = cudaGraphLaunch(B->gexec, st);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: graph launch");
    } else {
        e = cudaMemcpyAsync(B->d_desc, B->h_desc, copy_bytes, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: descriptor copy");
        fn<<<(unsigned)grid, dense::kThreads, smem, st>>>(B->d_desc, B->d_ctr);
        e = cudaGetLastError();
        if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: kernel launch");
    }
    e = cudaEventRecord(B->staged, st);
    if (e != cudaSuccess) return B->cuda_err(e, "ct_batch: staging event");
    B->staged_pending = true;
    return CT_OK;
}

void default_shape(const ct_batch* B, int& qt, int& cps, int& ips) {
    qt = B->cfg_qt;
    cps = B->cfg_cps > 0 ? B->cfg_cps : 1;
    ips = B->cfg_ips > 0 ? B->cfg_ips : 4;
    if (qt == 0) {
        // the tile height whose padded work, weighted by the measured per-pair cost of
        // the narrower tiles (more shared-memory traffic per multiply), is smallest
        const int order[3] = {64, 32, 16};
        const double cost[3] = {1.0, 1.6, 2.6};
        double best = -1.0;
        qt = 16;
        for (int t = 0; t < 3; ++t) {
            if (!shape_fits(B, order[t], 1)) continue;
            double w = 0.0;
            for (const BatchReq& r : B->reqs)
                w += (double)((r.nq + order[t] - 1) / order[t]) * order[t] * (double)r.tree->n * cost[t];
            if (best < 0.0 || w < best) { best = w; qt = order[t]; }
        }
    }
    if (!shape_fits(B, qt, cps)) cps = 1;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
namespace ct {
int batch_fail(const char* where, const char* msg, int code);  // ct_abi.cu
}

extern "C" {

int ct_batch_create(ct_batch** out) {
    if (!out) return ct::batch_fail("ct_batch_create", "out is NULL", CT_ERR_ARG);
    *out = nullptr;
    ct_batch* B = new (std::nothrow) ct_batch();
    if (!B) return ct::batch_fail("ct_batch_create", "host allocation failed", CT_ERR_NOMEM);
    int rc = batch_init(B);
    if (rc != CT_OK) {
        ct::batch_fail("ct_batch_create", B->err, rc);
        delete B;
        return rc;
    }
    *out = B;
    return CT_OK;
}

int ct_batch_clear(ct_batch* B) {
    if (!B) return ct::batch_fail("ct_batch_clear", "batch is NULL", CT_ERR_ARG);
    B->reqs.clear();
    return CT_OK;
}

static int add_req(ct_batch* B, ct_tree* T, const int64_t* q_ids, const float* qv, const float* qp,
                   const float* qcoords, int64_t nq, int32_t k, int32_t predecessor, int64_t* out_idx,
                   float* out_dist, const char* where) {
    if (!B || !T) return ct::batch_fail(where, "batch or tree is NULL", CT_ERR_ARG);
    if (nq < 0) return ct::batch_fail(where, "nq < 0", CT_ERR_ARG);
    if (k <= 0) return ct::batch_fail(where, "k must be positive", CT_ERR_ARG);
    if (k > 128) return ct::batch_fail(where, "k above the supported maximum 128", CT_ERR_UNSUPPORTED);
    if (nq > 0 && (!out_idx || !out_dist)) return ct::batch_fail(where, "NULL output", CT_ERR_ARG);
    BatchReq r;
    r.tree = T; r.qids = q_ids; r.qv = qv; r.qp = qp; r.qcoords = qcoords; r.nq = nq; r.k = k;
    r.predecessor = predecessor ? 1 : 0; r.out_idx = out_idx; r.out_dist = out_dist;
    B->reqs.push_back(r);
    return CT_OK;
}

int ct_batch_add_ids(ct_batch* B, ct_tree* T, const int64_t* q_ids, int64_t nq, int32_t k, int32_t predecessor,
                     int64_t* out_idx, float* out_dist) {
    if (nq > 0 && !q_ids) return ct::batch_fail("ct_batch_add_ids", "q_ids is NULL", CT_ERR_ARG);
    return add_req(B, T, q_ids, nullptr, nullptr, nullptr, nq, k, predecessor, out_idx, out_dist,
                   "ct_batch_add_ids");
}

int ct_batch_add_points(ct_batch* B, ct_tree* T, const float* qv, const float* qp, const float* qcoords,
                        int64_t nq, int32_t k, int64_t* out_idx, float* out_dist) {
    if (nq > 0 && (!qv || !qp || !qcoords))
        return ct::batch_fail("ct_batch_add_points", "NULL query rows", CT_ERR_ARG);
    return add_req(B, T, nullptr, qv, qp, qcoords, nq, k, 0, out_idx, out_dist, "ct_batch_add_points");
}

int ct_batch_set_shape(ct_batch* B, int32_t qt, int32_t ctas_per_sm, int32_t items_per_slot) {
    if (!B) return ct::batch_fail("ct_batch_set_shape", "batch is NULL", CT_ERR_ARG);
    if (qt != 0 && qt != 16 && qt != 32 && qt != 64)
        return ct::batch_fail("ct_batch_set_shape", "qt must be 0, 16, 32 or 64", CT_ERR_ARG);
    if (ctas_per_sm < 0 || ctas_per_sm > 2)
        return ct::batch_fail("ct_batch_set_shape", "ctas_per_sm must be 0, 1 or 2", CT_ERR_ARG);
    if (items_per_slot < 0 || items_per_slot > 64)
        return ct::batch_fail("ct_batch_set_shape", "items_per_slot must be in [0, 64]", CT_ERR_ARG);
    B->cfg_qt = qt; B->cfg_cps = ctas_per_sm; B->cfg_ips = items_per_slot;
    return CT_OK;
}

int ct_batch_reserve(ct_batch* B, int32_t m, int32_t d, int32_t k) {
    if (!B) return ct::batch_fail("ct_batch_reserve", "batch is NULL", CT_ERR_ARG);
    if (m < 16 || m % 16 != 0 || d < 1 || d > 64 || k < 1 || k > 128)
        return ct::batch_fail("ct_batch_reserve", "need m a positive multiple of 16, 1 <= d <= 64, 1 <= k <= 128",
                              CT_ERR_ARG);
    B->res_m = m; B->res_d = d; B->res_k = k;
    return CT_OK;
}

int ct_batch_get_shape(const ct_batch* B, int32_t* qt, int32_t* ctas_per_sm, int32_t* items_per_slot,
                       int32_t* grid, int64_t* items) {
    if (!B) return ct::batch_fail("ct_batch_get_shape", "batch is NULL", CT_ERR_ARG);
    if (qt) *qt = B->last_qt;
    if (ctas_per_sm) *ctas_per_sm = B->last_cps;
    if (items_per_slot) *items_per_slot = B->last_ips;
    if (grid) *grid = B->last_grid;
    if (items) *items = B->last_items;
    return CT_OK;
}

int ct_batch_run(ct_batch* B, int32_t use_graph, ct_stats* stats, void* stream) {
    if (!B) return ct::batch_fail("ct_batch_run", "batch is NULL", CT_ERR_ARG);
    if (stats) memset(stats, 0, sizeof(*stats));
    for (const BatchReq& r : B->reqs)
        if (r.tree->m % 16 != 0) return ct::batch_fail("ct_batch_run", "tree rank m must be a multiple of 16", CT_ERR_UNSUPPORTED);
    int qt, cps, ips;
    default_shape(B, qt, cps, ips);
    if (!shape_fits(B, qt, cps))
        return ct::batch_fail("ct_batch_run", "the batch's largest m, d, k exceed shared memory", CT_ERR_UNSUPPORTED);
    cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool timing = ct::timing_enabled() && stats;
    if (timing) {
        cudaEventCreate(&e0); cudaEventCreate(&e1);
        cudaEventRecord(e0, st);
    }
    int rc = run_shape(B, qt, cps, ips, use_graph != 0, st);
    if (rc != CT_OK) {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return ct::batch_fail("ct_batch_run", B->err, rc);
    }
    if (stats) {
        stats->kernel_launches = B->last_items > 0 ? 1 : 0;
        stats->distance_evals = B->last_pairs;
        stats->screen_pairs_main = B->last_items;
    }
    if (timing) {
        float ms = 0.f;
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        stats->device_ms = ms;
        cudaEventDestroy(e0); cudaEventDestroy(e1);
    }
    return CT_OK;
}

int ct_batch_autotune(ct_batch* B, int32_t reps, void* stream, int32_t* qt_out, int32_t* cps_out, int32_t* ips_out) {
    if (!B) return ct::batch_fail("ct_batch_autotune", "batch is NULL", CT_ERR_ARG);
    cudaStream_t st = (cudaStream_t)stream;
    if (reps <= 0) reps = 1;
    const Shape shapes[4] = {{64, 1}, {32, 1}, {16, 1}, {16, 2}};
    const int ipss[3] = {1, 4, 16};
    float best = 3.4e38f;
    int bq = 0, bc = 0, bi = 0;
    bool primed = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const Shape& s : shapes) {
        if (!shape_fits(B, s.qt, s.cps)) continue;
        std::vector<std::vector<int>> seen;  // split patterns already timed for this shape
        for (int ips : ipss) {
            Plan P;
            make_plan(B, s.qt, s.cps, ips, P);
            std::vector<int> splits;
            for (const Problem& pr : P.probs) splits.push_back(pr.split);
            if (std::find(seen.begin(), seen.end(), splits) != seen.end()) continue;  // same launch
            seen.push_back(splits);
            int rc = CT_OK;
            if (!primed) { rc = run_shape(B, s.qt, s.cps, ips, false, st); primed = true; }  // first-touch costs
            if (rc == CT_OK) cudaEventRecord(e0, st);
            for (int r = 0; r < reps && rc == CT_OK; ++r) rc = run_shape(B, s.qt, s.cps, ips, false, st);
            if (rc != CT_OK) {
                cudaEventDestroy(e0); cudaEventDestroy(e1);
                return ct::batch_fail("ct_batch_autotune", B->err, rc);
            }
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms < best) { best = ms; bq = s.qt; bc = s.cps; bi = ips; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (bq == 0) return ct::batch_fail("ct_batch_autotune", "no launch shape fits shared memory", CT_ERR_UNSUPPORTED);
    B->cfg_qt = bq; B->cfg_cps = bc; B->cfg_ips = bi;
    if (qt_out) *qt_out = bq;
    if (cps_out) *cps_out = bc;
    if (ips_out) *ips_out = bi;
    return CT_OK;
}

int ct_batch_free(ct_batch* B) {
    if (!B) return CT_OK;
    if (B->staged_pending) cudaEventSynchronize(B->staged);
    delete B;
    return CT_OK;
}

}  // extern "C"
