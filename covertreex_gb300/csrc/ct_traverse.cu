// ct_traverse.cu — plain FP32 form, cover-tree traversal (the query of
// single_residual_knn_query, src/algo.rs:612-1242, in its exhaustive parity mode,
// without the budget ladder), exact: it returns the dense form's neighbour lists
// bit for bit.
//
// One warp owns one query (persistent grid, queries strided over warps).  The warp
// keeps its top-k (distance, dataset id) list sorted in shared memory and a
// depth-first stack of (node, bound) in shared memory.  Candidate lists (the roots,
// then the children of each expanded node) are filtered 32 at a time with a ballot
// (predecessor mode: a subtree whose minimum dataset id is not below the query's is
// skipped without a distance, src/algo.rs:900-916), and the surviving candidates are
// scored 4 at a time: their V rows are staged in shared memory with 16-byte cp.async
// copies, then each half-warp scores 2 rows with the reference's batch-path f32
// distance (lane l sums elements 16c + l, bit-identical to the dense form) against
// the query row held in registers.
//
// Prune (certified, ct_treebound.cuh): the subtree below a node a cannot hold a
// neighbour when
//   L = lower(d32(q, a), delta(q, a)) - si_up[a] > 0  and
//   lower(L, delta_max(q, subtree a)) > kth,
// where lower() is a certified lower bound of the ideal metric, si_up[a] a certified
// upper bound of the ideal distance from a to any descendant, and delta_max the FP32
// error bound of any pair (q, x) in the subtree (through sub_isp[a], the subtree's
// largest 1/sqrt(p)).  By the ideal metric's triangle inequality every x below a then
// has d32(q, x) > kth, so the pruned subtree cannot change the list: the result equals
// the dense form's.  The reference's own test, d(q, a) - max(si[a], 1e-3) > kth on
// FP32 values (src/algo.rs:814-818, 1113-1142), has no such guarantee.
#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_tree.h"
#include "ct_treebound.cuh"

namespace ct {
namespace trav {

constexpr int kWarps = 8;
constexpr int kChunk = 8;                    // list entries a frame hands out per step
// per tree level the stack holds at most one chunk's children; 40 levels (levels fall strictly
// from 0 to -30, and only duplicate points share the floor level)
constexpr int kStack = kChunk * 40 + 1;
constexpr int kTopK = 64;
constexpr int kRows = 4;  // candidate rows staged per batch (2 per half-warp)

struct Params {
    const float* v;      // node-order natural V
    const float* xs;
    const float* norms;
    const float* p;
    const float* isp;    // node order: 1/sqrt(p), |v| (rounded up)
    const float* vn;
    const long long* order;  // node -> dataset id
    const long long* inv;    // dataset id -> node
    const long long* child_off;
    const long long* child_idx;
    const float* si_up;
    const float* sub_isp;
    const long long* sub_min;
    const long long* roots;
    long long n_roots;
    const long long* q_ids;
    long long nq, n;
    int m, d, k, kernel_type, predecessor;
    float var;
    BoundModel bound;
    long long* out_idx;
    float* out_dist;
    unsigned long long* evals;
    int* overflow;
};

// Insert (d, id) into the warp's sorted top-k list if it beats the k-th entry.
__device__ __forceinline__ void topk_offer(float* td, int* ti, int& cnt, int k, float d, int id) {
    const int lane = threadIdx.x & 31;
    const bool full = cnt >= k;
    if (full && !nb_less(d, id, td[k - 1], ti[k - 1])) return;
    int below = 0;
    for (int j = lane; j < cnt; j += 32) below += nb_less(td[j], ti[j], d, id) ? 1 : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) below += __shfl_xor_sync(0xffffffffu, below, off);
    const int last = full ? k - 1 : cnt;  // entries [below, last) shift right by one
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

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc));
}

template <int MAXC>
__global__ void __launch_bounds__(32 * kWarps) traverse_kernel(Params P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_node[kWarps][kStack];
    __shared__ int s_cur[kWarps][kStack];
    __shared__ float s_lb[kWarps][kStack];
    __shared__ float s_td[kWarps][kTopK];
    __shared__ int s_ti[kWarps][kTopK];
    __shared__ float s_xq[kWarps][64];
    __shared__ int s_cand[kWarps][32];
    const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int half = (lane >> 4) & 1, l16 = lane & 15;
    const unsigned hmask = half ? 0xffff0000u : 0x0000ffffu;
    const long long nwarps = (long long)gridDim.x * kWarps;
    const int m = P.m, mc = P.m >> 4;
    float* rows = (float*)smem_raw + (size_t)wi * kRows * m;
    int* stn = s_node[wi];
    int* stc = s_cur[wi];
    float* stl = s_lb[wi];
    float* td = s_td[wi];
    int* ti = s_ti[wi];
    float* xq = s_xq[wi];
    int* cand = s_cand[wi];
    unsigned long long evals = 0;
    for (long long qi = (long long)blockIdx.x * kWarps + wi; qi < P.nq; qi += nwarps) {
        const long long qd = P.q_ids[qi];
        int cnt = 0;
        if (qd >= 0 && qd < P.n && !(P.predecessor && qd == 0)) {
            const int qn = (int)P.inv[qd];
            float vq[MAXC];
#pragma unroll
            for (int c = 0; c < MAXC; ++c) vq[c] = c < mc ? P.v[(size_t)qn * m + 16 * c + l16] : 0.f;
            for (int c = lane; c < P.d; c += 32) xq[c] = P.xs[(size_t)qn * P.d + c];
            const float nq = P.norms[qn], pq = P.p[qn], isq = P.isp[qn], vnq = P.vn[qn];
            const bool may_prune = isq <= kNoPruneIsp;
            bool overflowed = false;
            // Depth-first over frames (node, cursor, bound): node -1 is the list of roots.
            // A frame hands out its candidates kChunk at a time; expandable candidates
            // become frames on top of it, so the stack holds at most kChunk frames per tree
            // level; a deeper tree is reported as an overflow error, never read past.
            int sp = 0;
            if (lane == 0) { stn[0] = -1; stc[0] = 0; stl[0] = 0.f; }
            sp = 1;
            __syncwarp();
            while (sp > 0) {
                const int top = sp - 1;
                const int nd = stn[top];
                const int cur = stc[top];
                const float lbf = stl[top];
                __syncwarp();
                const long long b0 = nd < 0 ? 0 : P.child_off[nd];
                const long long e0 = nd < 0 ? P.n_roots : P.child_off[nd + 1];
                const long long* ids = nd < 0 ? P.roots : P.child_idx;
                const float kth0 = cnt >= P.k ? td[P.k - 1] : CT_FLT_MAX;
                const long long base = b0 + cur;
                if (base >= e0 || lbf > kth0) {  // frame done, or its whole subtree pruned
                    --sp;
                    continue;
                }
                if (lane == 0) stc[top] = cur + kChunk;
                const long long gi = base + lane;
                int c = (lane < kChunk && gi < e0) ? (int)ids[gi] : -1;
                if (c >= 0 && P.predecessor && P.sub_min[c] >= qd) c = -1;
                const unsigned ok = __ballot_sync(0xffffffffu, c >= 0);
                if (c >= 0) cand[__popc(ok & ((1u << lane) - 1u))] = c;
                __syncwarp();
                const int nc = __popc(ok);
                for (int c0 = 0; c0 < nc; c0 += kRows) {
                    const int nr = min(kRows, nc - c0);
                    // stage nr rows: 16-byte pieces spread over the warp
                    const int pieces = m >> 2;  // per row
                    for (int t = lane; t < nr * pieces; t += 32) {
                        const int r = t / pieces, q4 = t - r * pieces;
                        cp_async16(rows + (size_t)r * m + 4 * q4, P.v + (size_t)cand[c0 + r] * m + 4 * q4);
                    }
                    asm volatile("cp.async.commit_group;\n" ::);
                    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                    __syncwarp();
                    float dist[kRows / 2];
#pragma unroll
                    for (int r = 0; r < kRows / 2; ++r) {
                        const int rr = half * (kRows / 2) + r;
                        dist[r] = CT_FLT_MAX;
                        if (rr < nr) {
                            const float* row = rows + (size_t)rr * m;
                            float acc = 0.f;
#pragma unroll
                            for (int cc = 0; cc < MAXC; ++cc)
                                if (cc < mc) acc = __fadd_rn(__fmul_rn(vq[cc], row[16 * cc + l16]), acc);
                            float t = __shfl_down_sync(hmask, acc, 8, 16);
                            const float comb = __fadd_rn(acc, t);
                            t = __shfl_down_sync(hmask, comb, 4, 16);
                            const float s2 = __fadd_rn(comb, t);
                            t = __shfl_down_sync(hmask, s2, 2, 16);
                            const float u2 = __fadd_rn(s2, t);
                            t = __shfl_down_sync(hmask, u2, 1, 16);
                            float dot = __fadd_rn(u2, t);
                            dot = __shfl_sync(hmask, dot, 0, 16);
                            const int node = cand[c0 + rr];
                            if (node == qn) {
                                dist[r] = 0.f;
                            } else {
                                const float d2 = coord_d2_batch(xq, P.xs + (size_t)node * P.d, P.d, nq, P.norms[node]);
                                const float kv = kernel_value_batch(d2, P.var, P.kernel_type);
                                dist[r] = residual_from_parts(kv, dot, pq, P.p[node]);
                            }
                        }
                    }
                    __syncwarp();
#pragma unroll
                    for (int rr = 0; rr < kRows; ++rr) {
                        if (rr < nr) {
                            const float dd = __shfl_sync(0xffffffffu, dist[rr % (kRows / 2)], rr < kRows / 2 ? 0 : 16);
                            const int node = cand[c0 + rr];
                            const long long ds = P.order[node];
                            ++evals;
                            if (!P.predecessor || ds < qd) topk_offer(td, ti, cnt, P.k, dd, (int)ds);
                            if (P.child_off[node + 1] > P.child_off[node]) {
                                float lb = 0.f;
                                if (may_prune) {
                                    const float dqa = pair_delta(P.bound, nq, P.norms[node], vnq, P.vn[node], isq,
                                                                 P.isp[node]);
                                    const float L = (dist_lower(dd, dqa) - P.si_up[node]) * (1.f - 5.0e-7f);
                                    if (L > 0.f) {
                                        const float dmax = pair_delta(P.bound, nq, P.bound.nmax, vnq, P.bound.vmax,
                                                                      isq, P.sub_isp[node]);
                                        lb = dist_lower(L, dmax);
                                    }
                                }
                                const float kth = cnt >= P.k ? td[P.k - 1] : CT_FLT_MAX;
                                if (!(lb > kth)) {
                                    if (sp < kStack) {
                                        if (lane == 0) { stn[sp] = node; stc[sp] = 0; stl[sp] = lb; }
                                        ++sp;
                                    } else {
                                        overflowed = true;
                                    }
                                }
                            }
                            __syncwarp();
                        }
                    }
                }
                __syncwarp();
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
    P.v = tvnat; P.xs = txs; P.norms = tnorms; P.p = tp; P.isp = tisp; P.vn = tvn; P.order = order; P.inv = inv;
    P.child_off = child_off; P.child_idx = child_idx; P.si_up = si_up; P.sub_isp = sub_isp; P.sub_min = sub_min;
    P.roots = roots; P.n_roots = n_roots; P.q_ids = (const long long*)q_ids; P.nq = nq; P.n = n;
    P.m = m; P.d = d; P.k = k; P.kernel_type = kernel_type; P.predecessor = predecessor ? 1 : 0; P.var = var;
    P.bound = bound;
    P.out_idx = (long long*)out_idx; P.out_dist = out_dist; P.evals = evals; P.overflow = overflow;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const size_t smem = sizeof(float) * (size_t)kWarps * kRows * m;
    long long blocks = (nq + kWarps - 1) / kWarps;
    if (blocks > (long long)sms * 16) blocks = (long long)sms * 16;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const bool timing = ct::timing_enabled();
    if (timing) { cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventRecord(e0, st); }
    if (e == cudaSuccess) {
        if (m <= 512) {
            e = cudaFuncSetAttribute(traverse_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) traverse_kernel<32><<<(unsigned)blocks, 32 * kWarps, smem, st>>>(P);
        } else {
            e = cudaFuncSetAttribute(traverse_kernel<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) traverse_kernel<64><<<(unsigned)blocks, 32 * kWarps, smem, st>>>(P);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    unsigned long long he = 0;
    int ho = 0;
    float ms = 0.f;
    if (timing && e == cudaSuccess) { cudaEventRecord(e1, st); cudaEventSynchronize(e1); cudaEventElapsedTime(&ms, e0, e1); }
    if (timing) { cudaEventDestroy(e0); cudaEventDestroy(e1); }
    if (e == cudaSuccess) {
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
