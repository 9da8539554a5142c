// ct_traverse.cu — plain FP32 form, cover-tree traversal (the query of
// single_residual_knn_query, src/algo.rs:612-1242, in its exhaustive parity
// mode, without the budget ladder).
//
// One warp owns one query (persistent grid, queries strided over warps).  The
// warp keeps its top-k (distance, dataset id) list sorted in shared memory and a
// depth-first stack of (node, lower bound) in shared memory.  Children of a
// popped node are scored two at a time, one per half-warp, with the
// reference's batch-path f32 distance (bit-identical to the dense form): the
// query's V row stays in registers (lane l holds elements 16c + (l mod 16)),
// candidate rows stream through coalesced 64-byte half-warp loads.  A child is
// pruned when d(q, child) - max(si[child], 1e-3) > kth (the reference's cover
// radius test with its 1e-3 floor, src/algo.rs:814-818, 1113-1142); in
// predecessor mode a subtree whose minimum dataset id is >= the query's is
// skipped without a distance (src/algo.rs:900-916).
#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_tree.h"

namespace ct {
namespace trav {

constexpr int kWarps = 4;
constexpr int kStack = 1024;
constexpr int kTopK = 64;
constexpr float kRadiusFloor = 1e-3f;

struct Params {
    const float* v;      // node-order natural V
    const float* xs;
    const float* norms;
    const float* p;
    const long long* order;  // node -> dataset id
    const long long* inv;    // dataset id -> node
    const long long* child_off;
    const long long* child_idx;
    const float* si;
    const long long* sub_min;
    const long long* roots;
    long long n_roots;
    const long long* q_ids;
    long long nq, n;
    int m, d, k, kernel_type, predecessor;
    float var;
    long long* out_idx;
    float* out_dist;
    unsigned long long* evals;
    int* overflow;
};

template <int MAXC>
__device__ __forceinline__ float half_dist_q(const Params& P, const float (&vq)[MAXC], const float* xq, float nq,
                                             float pq, int qnode, int b) {
    const int l = threadIdx.x & 15;
    const unsigned hmask = (threadIdx.x & 16) ? 0xffff0000u : 0x0000ffffu;
    const float* vb = P.v + (size_t)b * P.m;
    const int mc = P.m >> 4;
    float acc = 0.f;
#pragma unroll
    for (int c = 0; c < MAXC; ++c)
        if (c < mc) acc = __fadd_rn(__fmul_rn(vq[c], __ldg(vb + 16 * c + l)), acc);
    float t = __shfl_down_sync(hmask, acc, 8, 16);
    float comb = __fadd_rn(acc, t);
    t = __shfl_down_sync(hmask, comb, 4, 16);
    float s = __fadd_rn(comb, t);
    t = __shfl_down_sync(hmask, s, 2, 16);
    float u = __fadd_rn(s, t);
    t = __shfl_down_sync(hmask, u, 1, 16);
    float dot = __fadd_rn(u, t);
    dot = __shfl_sync(hmask, dot, 0, 16);
    if (b == qnode) return 0.f;
    const float d2 = coord_d2_batch(xq, P.xs + (size_t)b * P.d, P.d, nq, P.norms[b]);
    const float kv = kernel_value_batch(d2, P.var, P.kernel_type);
    return residual_from_parts(kv, dot, pq, P.p[b]);
}

// Insert (d, id) into the warp's sorted top-k list if it beats the k-th entry.
__device__ __forceinline__ void topk_offer(float* td, int* ti, int& cnt, int k, float d, int id) {
    const int lane = threadIdx.x & 31;
    const bool full = cnt >= k;
    if (full && !nb_less(d, id, td[k - 1], ti[k - 1])) return;
    // position = number of entries that precede (d, id)
    int below = 0;
    for (int j = lane; j < cnt; j += 32) below += nb_less(td[j], ti[j], d, id) ? 1 : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) below += __shfl_xor_sync(0xffffffffu, below, off);
    const int last = full ? k - 1 : cnt;  // entries [pos, last) shift right by one
    float sd[2];
    int si2[2];
    int ns = 0;
    for (int j = below + lane; j < last; j += 32) { sd[ns] = td[j]; si2[ns] = ti[j]; ++ns; }
    __syncwarp();
    ns = 0;
    for (int j = below + lane; j < last; j += 32) { td[j + 1] = sd[ns]; ti[j + 1] = si2[ns]; ++ns; }
    __syncwarp();
    if (lane == 0) { td[below] = d; ti[below] = id; }
    __syncwarp();
    if (!full) ++cnt;
}

template <int MAXC>
__global__ void __launch_bounds__(32 * kWarps) traverse_kernel(Params P) {
    __shared__ int s_node[kWarps][kStack];
    __shared__ float s_lb[kWarps][kStack];
    __shared__ float s_td[kWarps][kTopK];
    __shared__ int s_ti[kWarps][kTopK];
    __shared__ float s_xq[kWarps][64];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = (lane >> 4) & 1;
    const long long nwarps = (long long)gridDim.x * kWarps;
    int* stn = s_node[wi];
    float* stl = s_lb[wi];
    float* td = s_td[wi];
    int* ti = s_ti[wi];
    float* xq = s_xq[wi];
    unsigned long long evals = 0;
    for (long long qi = (long long)blockIdx.x * kWarps + wi; qi < P.nq; qi += nwarps) {
        const long long qd = P.q_ids[qi];
        int cnt = 0;
        if (qd >= 0 && qd < P.n && !(P.predecessor && qd == 0)) {
            const int qn = (int)P.inv[qd];
            float vq[MAXC];
#pragma unroll
            for (int c = 0; c < MAXC; ++c) vq[c] = (c < (P.m >> 4)) ? P.v[(size_t)qn * P.m + 16 * c + (lane & 15)] : 0.f;
            for (int c = lane; c < P.d; c += 32) xq[c] = P.xs[(size_t)qn * P.d + c];
            __syncwarp();
            const float nq = P.norms[qn], pq = P.p[qn];
            int sp = 0;
            bool overflowed = false;
            // score a node (per half); returns through the warp in pairs
            auto visit_pair = [&](int nodeA, int nodeB) {
                const int mine = half ? nodeB : nodeA;
                float dd = CT_FLT_MAX;
                bool ok = mine >= 0;
                if (ok) dd = half_dist_q<MAXC>(P, vq, xq, nq, pq, qn, mine);
                const float d0 = __shfl_sync(0xffffffffu, dd, 0);
                const float d1 = __shfl_sync(0xffffffffu, dd, 16);
                for (int h = 0; h < 2; ++h) {
                    const int nd = h ? nodeB : nodeA;
                    if (nd < 0) continue;
                    const float dist = h ? d1 : d0;
                    const long long ds = P.order[nd];
                    ++evals;
                    if (!P.predecessor || ds < qd) topk_offer(td, ti, cnt, P.k, dist, (int)ds);
                    const long long c0 = P.child_off[nd], c1 = P.child_off[nd + 1];
                    if (c1 > c0) {
                        const float lb = dist - fmaxf(P.si[nd], kRadiusFloor);
                        const float kth = cnt >= P.k ? td[P.k - 1] : CT_FLT_MAX;
                        if (lb <= kth) {
                            if (sp < kStack) {
                                if (lane == 0) { stn[sp] = nd; stl[sp] = lb; }
                                ++sp;
                            } else {
                                overflowed = true;
                            }
                        }
                    }
                    __syncwarp();
                }
            };
            // roots
            for (long long r = 0; r < P.n_roots; r += 2) {
                int a = (int)P.roots[r];
                int b = r + 1 < P.n_roots ? (int)P.roots[r + 1] : -1;
                if (P.predecessor) {
                    if (P.sub_min[a] >= qd) a = -1;
                    if (b >= 0 && P.sub_min[b] >= qd) b = -1;
                }
                if (a < 0 && b < 0) continue;
                visit_pair(a, b);
            }
            while (sp > 0) {
                --sp;
                const int nd = stn[sp];
                const float lb = stl[sp];
                __syncwarp();
                const float kth = cnt >= P.k ? td[P.k - 1] : CT_FLT_MAX;
                if (lb > kth) continue;
                const long long c0 = P.child_off[nd], c1 = P.child_off[nd + 1];
                int pending = -1;
                for (long long c = c0; c < c1; ++c) {
                    int ch = (int)P.child_idx[c];
                    if (P.predecessor && P.sub_min[ch] >= qd) continue;
                    if (pending < 0) { pending = ch; continue; }
                    visit_pair(pending, ch);
                    pending = -1;
                }
                if (pending >= 0) visit_pair(pending, -1);
            }
            if (overflowed && lane == 0) atomicAdd(P.overflow, 1);
        }
        for (int j = lane; j < P.k; j += 32) {
            const bool ok = j < cnt;
            P.out_idx[qi * P.k + j] = ok ? (long long)ti[j] : -1LL;
            P.out_dist[qi * P.k + j] = ok ? td[j] : CT_FLT_MAX;
        }
        __syncwarp();
    }
    if (lane == 0 && P.evals) atomicAdd(P.evals, evals);
}

}  // namespace trav
}  // namespace ct

using namespace ct::trav;

int ct_tree::knn_tree(const int64_t* q_ids, int64_t nq, int k, int predecessor, int64_t* out_idx, float* out_dist,
                      ct_stats* stats, cudaStream_t st) {
    if (!has_tree) return set_err(CT_ERR_STATE, "%s", "tree form needs a tree (built without CT_BUILD_METRIC_ONLY)");
    if (k > kTopK) return set_err(CT_ERR_UNSUPPORTED, "tree form supports k <= %d", kTopK);
    if (m > 1024 || d > 64) return set_err(CT_ERR_UNSUPPORTED, "%s", "tree form supports m <= 1024, d <= 64");
    unsigned long long* evals = nullptr;
    int* overflow = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&evals, 8, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&overflow, 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(evals, 0, 8, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(overflow, 0, 4, st);
    Params P{};
    P.v = tvnat; P.xs = txs; P.norms = tnorms; P.p = tp; P.order = order; P.inv = inv;
    P.child_off = child_off; P.child_idx = child_idx; P.si = si; P.sub_min = sub_min;
    P.roots = roots; P.n_roots = n_roots; P.q_ids = (const long long*)q_ids; P.nq = nq; P.n = n;
    P.m = m; P.d = d; P.k = k; P.kernel_type = kernel_type; P.predecessor = predecessor ? 1 : 0; P.var = var;
    P.out_idx = (long long*)out_idx; P.out_dist = out_dist; P.evals = evals; P.overflow = overflow;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    long long blocks = (nq + kWarps - 1) / kWarps;
    if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool timing = ct::timing_enabled();
    if (timing) { cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventRecord(e0, st); }
    if (e == cudaSuccess) {
        if (m <= 512) traverse_kernel<32><<<(unsigned)blocks, 32 * kWarps, 0, st>>>(P);
        else traverse_kernel<64><<<(unsigned)blocks, 32 * kWarps, 0, st>>>(P);
        e = cudaGetLastError();
    }
    unsigned long long he = 0;
    int ho = 0;
    float ms = 0.f;
    if (timing && e == cudaSuccess) { cudaEventRecord(e1, st); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1); }
    if (timing) { cudaEventDestroy(e0); cudaEventDestroy(e1); }
    if (e == cudaSuccess && stats) {
        e = cudaMemcpyAsync(&he, evals, 8, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&ho, overflow, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFreeAsync(evals, st);
    cudaFreeAsync(overflow, st);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "tree traversal: %s", cudaGetErrorString(e));
    if (stats) {
        stats->distance_evals = (long long)he;
        stats->kernel_launches = 1;
        stats->device_ms = ms;
        stats->screen_ms = ms;
        stats->overflow_queries = ho;
    }
    if (ho > 0) return set_err(CT_ERR_STATE, "tree traversal: %d queries overflowed the %d-entry stack", ho, kStack);
    return CT_OK;
}
