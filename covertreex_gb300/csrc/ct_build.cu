// ct_build.cu — device cover-tree build (the batch build of the reference's
// build_pcct2_residual_tree, src/lib.rs:1374-1564, and of the Python PCCT path,
// covertreex/algo/batch/insert.py:43-803), re-designed level-synchronous for a GPU.
//
//  1. Batch order: Hilbert keys + LSD radix sort (ct_order.cu); node i of the
//     tree is the point at sorted position i, and V / coordinates are copied
//     into that order so subtrees are contiguous in memory.
//  2. Coarsening, finest radius first.  The active set S starts as all nodes.
//     At radius r (2^-9, 2^-8, ..., 1, then 1 again until |S| <= 64):
//       * conflict graph: an edge joins two active nodes within kWindow positions
//         of each other (in S's Hilbert order) whose residual distance is <= r;
//       * seeded Luby MIS on that graph with warp ballots (hash priorities of
//         covertreex/algo/_mis_numba.py:19-28, lower index wins ties); a
//         maximal independent set keeps every non-selected node next to a
//         selected one;
//       * every non-selected node attaches to its nearest selected neighbour
//         (its parent; its level is log2 r); the selected nodes form the next S.
//     The nodes left at the end are the roots.
//  3. Cover radii: si[a] = max over descendants x of d(a, x), computed exactly
//     by walking each node's ancestor chain (the reference's
//     compute_si_cache_residual, src/algo.rs:52-106, stores the looser
//     sum d(node, child) + si[child]); subtree_min[a] = min dataset id below a
//     (compute_subtree_index_bounds, src/tree.rs:144-185).
//  4. Children in CSR (child_off / child_idx), roots listed separately.
//
// Distances use the reference's batch-path f32 arithmetic (the same device
// functions as the dense form), evaluated by half-warps: lane l of a half owns
// the accumulator of elements 16c + l, so a pair's value is bit-identical to
// the dense form's.
#include <climits>

#include <algorithm>
#include <vector>

#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_tree.h"

namespace ct {
namespace treeb {

constexpr int kWindow = 32;  // neighbours on each side in the active order
constexpr int kMaxRoots = 64;

struct TreeData {
    const float* v;    // n x m natural layout, node order
    const float* xs;   // n x d scaled coords, node order
    const float* norms;
    const float* p;
    int m, d, kernel_type;
    float var;
};

// Half-warp residual distance between nodes a and b (reference batch-path order).
// Every lane of the half returns the value.
__device__ __forceinline__ float half_dist(const TreeData& T, int a, int b) {
    const int l = threadIdx.x & 15;
    const unsigned hmask = (threadIdx.x & 16) ? 0xffff0000u : 0x0000ffffu;
    if (a == b) return 0.f;
    const float* va = T.v + (size_t)a * T.m;
    const float* vb = T.v + (size_t)b * T.m;
    float acc = 0.f;
    for (int c = 0; c < T.m / 16; ++c) acc = __fadd_rn(__fmul_rn(va[16 * c + l], vb[16 * c + l]), acc);
    float t = __shfl_down_sync(hmask, acc, 8, 16);
    float comb = __fadd_rn(acc, t);
    t = __shfl_down_sync(hmask, comb, 4, 16);
    float s = __fadd_rn(comb, t);
    t = __shfl_down_sync(hmask, s, 2, 16);
    float u = __fadd_rn(s, t);
    t = __shfl_down_sync(hmask, u, 1, 16);
    float dot = __fadd_rn(u, t);
    dot = __shfl_sync(hmask, dot, 0, 16);
    const float d2 = coord_d2_batch(T.xs + (size_t)a * T.d, T.xs + (size_t)b * T.d, T.d, T.norms[a], T.norms[b]);
    const float kv = kernel_value_batch(d2, T.var, T.kernel_type);
    return residual_from_parts(kv, dot, T.p[a], T.p[b]);
}

__device__ __forceinline__ double hash_priority(unsigned node, unsigned seed, unsigned iteration) {
    unsigned x = node ^ seed;
    x ^= (unsigned)((unsigned long long)iteration * 0x9E3779B9ULL);
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return ((double)x + 1.0) / 4294967296.0;
}

// adjacency: bit w of mask[i] <-> neighbour at active position i + (w - kWindow) (w != kWindow)
__global__ void conflict_edges_kernel(TreeData T, const int* __restrict__ act, int na, float r,
                                      unsigned long long* __restrict__ mask) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int half = (threadIdx.x >> 4) & 1;
    const int lane16 = threadIdx.x & 15;
    if (warp >= na) return;
    const int i = warp;
    unsigned long long bits = 0;
    for (int w = half; w < 2 * kWindow + 1; w += 2) {
        const int j = i + w - kWindow;
        if (w == kWindow || j < 0 || j >= na) continue;
        const float dd = half_dist(T, act[i], act[j]);
        if (dd <= r) bits |= 1ULL << w;
    }
    // combine the two halves' bits
    bits |= __shfl_xor_sync(0xffffffffu, bits, 16);
    if ((threadIdx.x & 31) == 0) mask[i] = bits;
    (void)lane16;
}

// One Luby round: an active node wins if no active neighbour has a higher
// (priority, lower index) rank.  A warp handles 32 nodes; lanes test their
// node's neighbours and the warp ballots on the outcome.
__global__ void luby_round_kernel(const unsigned long long* __restrict__ mask, int na, unsigned seed, unsigned round,
                                  unsigned char* __restrict__ state, int* __restrict__ any_active) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool win = false;
    if (i < na && state[i] == 0) {
        const double pi = hash_priority((unsigned)i, seed, round);
        win = true;
        unsigned long long b = mask[i];
        while (b) {
            const int w = __ffsll((long long)b) - 1;
            b &= b - 1;
            const int j = i + w - kWindow;
            if (state[j] != 0 && state[j] != 3) continue;  // 3 = winning this round, still active
            const double pj = hash_priority((unsigned)j, seed, round);
            if (pj > pi || (pj == pi && j < i)) { win = false; break; }
        }
    }
    const unsigned wins = __ballot_sync(0xffffffffu, win);
    if (win) state[i] = 3;  // tentatively selected this round
    if ((threadIdx.x & 31) == 0 && wins) atomicOr(any_active, 1);
}

// Commit a round: winners become selected (1), their neighbours excluded (2).
__global__ void luby_commit_kernel(const unsigned long long* __restrict__ mask, int na,
                                   unsigned char* __restrict__ state, int* __restrict__ remaining) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= na) return;
    if (state[i] == 3) { state[i] = 1; return; }
    if (state[i] != 0) return;
    unsigned long long b = mask[i];
    while (b) {
        const int w = __ffsll((long long)b) - 1;
        b &= b - 1;
        const int j = i + w - kWindow;
        if (state[j] == 3 || state[j] == 1) { state[i] = 2; return; }
    }
    atomicAdd(remaining, 1);
}

// Non-selected nodes attach to their nearest selected neighbour (one warp per node).
__global__ void attach_kernel(TreeData T, const int* __restrict__ act, int na, const unsigned long long* __restrict__ mask,
                              const unsigned char* __restrict__ state, int level, long long* __restrict__ parents,
                              int* __restrict__ levels) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int half = (threadIdx.x >> 4) & 1;
    if (warp >= na) return;
    const int i = warp;
    if (state[i] != 2) return;  // selected (or undecided, kept as selected) nodes do not attach
    float best = CT_FLT_MAX;
    int bj = -1;
    for (int w = half; w < 2 * kWindow + 1; w += 2) {
        const int j = i + w - kWindow;
        if (!((mask[i] >> w) & 1ULL) || state[j] != 1) continue;
        const float dd = half_dist(T, act[i], act[j]);
        if (dd < best || (dd == best && j < bj)) { best = dd; bj = j; }
    }
    const float ob = __shfl_xor_sync(0xffffffffu, best, 16);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, 16);
    if (oj >= 0 && (ob < best || (ob == best && (bj < 0 || oj < bj)))) { best = ob; bj = oj; }
    if ((threadIdx.x & 31) == 0 && bj >= 0) {
        parents[act[i]] = act[bj];
        levels[act[i]] = level;
    }
}

// Stream compaction of the selected nodes (one block; order preserved).
__global__ void __launch_bounds__(1024) compact_selected_kernel(const int* __restrict__ act, int na,
                                                                const unsigned char* __restrict__ state,
                                                                int* __restrict__ out, int* __restrict__ nout) {
    // selected (1) and, should the round limit ever be hit, undecided (0) nodes
    __shared__ int warp_tot[32];
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (int c0 = 0; c0 < na; c0 += 1024) {
        const int i = c0 + threadIdx.x;
        const bool sel = i < na && (state[i] == 1 || state[i] == 0);  // undecided nodes stay active
        const unsigned bal = __ballot_sync(0xffffffffu, sel);
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        if (lane == 0) warp_tot[wid] = __popc(bal);
        __syncthreads();
        int before = 0;
        for (int w = 0; w < wid; ++w) before += warp_tot[w];
        if (sel) out[base + before + __popc(bal & ((1u << lane) - 1u))] = act[i];
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < 32; ++w) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *nout = base;
}

// si and subtree_min by walking every node's ancestor chain (one half-warp per node).
__global__ void ancestors_kernel(TreeData T, int n, const long long* __restrict__ parents,
                                 const long long* __restrict__ order, unsigned* __restrict__ si_bits,
                                 long long* __restrict__ sub_min) {
    const int hw = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    if (hw >= n) return;
    const int x = hw;
    const long long ds = order[x];
    long long a = parents[x];
    int guard = 0;
    while (a >= 0 && guard < 4096) {
        const float dd = half_dist(T, (int)a, x);
        if ((threadIdx.x & 15) == 0) {
            atomicMax(&si_bits[a], __float_as_uint(dd));
            atomicMin((unsigned long long*)&sub_min[a], (unsigned long long)ds);
        }
        a = parents[a];
        ++guard;
    }
}

__global__ void init_tree_kernel(int n, long long* parents, int* levels, unsigned* si_bits, long long* sub_min,
                                 const long long* order, int* act) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    parents[i] = -1;
    levels[i] = INT_MIN;
    si_bits[i] = 0u;
    sub_min[i] = order[i];
    act[i] = i;
}

__global__ void gather_rows_kernel(const float* __restrict__ src, const long long* __restrict__ order, long long n,
                                   int w, float* __restrict__ dst) {
    const long long total = n * (long long)w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / w;
        dst[e] = src[order[r] * w + (e - r * w)];
    }
}

__global__ void to_i64_kernel(const int* in, long long n, long long* out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

__global__ void inverse_kernel(const long long* order, long long n, long long* inv) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) inv[order[i]] = i;
}

}  // namespace treeb
}  // namespace ct

using namespace ct::treeb;

static inline unsigned gridn(long long n, int b) { return (unsigned)((n + b - 1) / b); }

int ct_tree::build_tree(const float* /*v_dataset*/, const float* /*coords_dataset*/, cudaStream_t st) {
    const long long N = n;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** ptr, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(ptr, bytes ? bytes : 16); };
    A((void**)&order, 8 * N); A((void**)&inv, 8 * N); A((void**)&parents, 8 * N); A((void**)&levels, 4 * N);
    A((void**)&si, 4 * N); A((void**)&sub_min, 8 * N); A((void**)&child_off, 8 * (N + 1)); A((void**)&child_idx, 8 * N);
    A((void**)&roots, 8 * kMaxRoots * 64);
    A((void**)&tvnat, sizeof(float) * N * m); A((void**)&txs, sizeof(float) * N * d);
    A((void**)&tnorms, sizeof(float) * N); A((void**)&tp, sizeof(float) * N);
    int *order32 = nullptr, *act = nullptr, *act2 = nullptr, *counters = nullptr;
    unsigned long long* mask = nullptr;
    unsigned char* state = nullptr;
    A((void**)&order32, 4 * N); A((void**)&act, 4 * N); A((void**)&act2, 4 * N); A((void**)&counters, 16);
    A((void**)&mask, 8 * N); A((void**)&state, N);
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "tree build allocation: %s", cudaGetErrorString(e));

    // 1. batch order
    if (order_mode == CT_ORDER_NATURAL) {
        std::vector<int> id(N);
        for (long long i = 0; i < N; ++i) id[i] = (int)i;
        e = cudaMemcpyAsync(order32, id.data(), 4 * N, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    } else {
        e = ct::compute_order(coords_raw, N, d, (d == 3 && order_mode == 2) ? 2 : 1, order32, st);
    }
    if (e == cudaSuccess) {
        to_i64_kernel<<<gridn(N, 256), 256, 0, st>>>(order32, N, order);
        inverse_kernel<<<gridn(N, 256), 256, 0, st>>>(order, N, inv);
        // node-order copies (natural-layout V for the half-warp distances)
        gather_rows_kernel<<<152 * 8, 256, 0, st>>>(vnat, order, N, m, tvnat);
        gather_rows_kernel<<<152 * 8, 256, 0, st>>>(xs, order, N, d, txs);
        gather_rows_kernel<<<gridn(N, 256), 256, 0, st>>>(norms, order, N, 1, tnorms);
        gather_rows_kernel<<<gridn(N, 256), 256, 0, st>>>(p, order, N, 1, tp);
        init_tree_kernel<<<gridn(N, 256), 256, 0, st>>>((int)N, parents, levels, (unsigned*)si, sub_min, order, act);
        e = cudaGetLastError();
    }
    TreeData TD{tvnat, txs, tnorms, tp, m, d, kernel_type, var};
    // 2. coarsening
    long long na = N;
    int level = -9;
    int guard = 0;
    unsigned mis_seed = (unsigned)(seed & 0xffffffffu);
    while (e == cudaSuccess && na > kMaxRoots && guard < 64) {
        ++guard;
        const float r = ldexpf(1.0f, level < 0 ? level : 0);
        conflict_edges_kernel<<<gridn(na * 32, 256), 256, 0, st>>>(TD, act, (int)na, r, mask);
        e = cudaMemsetAsync(state, 0, na, st);
        int rounds = 0;
        while (e == cudaSuccess && rounds < 256) {
            ++rounds;
            e = cudaMemsetAsync(counters, 0, 16, st);
            if (e != cudaSuccess) break;
            luby_round_kernel<<<gridn(na, 256), 256, 0, st>>>(mask, (int)na, mis_seed, (unsigned)rounds, state, counters);
            luby_commit_kernel<<<gridn(na, 256), 256, 0, st>>>(mask, (int)na, state, counters + 1);
            int h[2] = {0, 0};
            e = cudaMemcpyAsync(h, counters, 8, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (h[1] == 0) break;  // no undecided node left
        }
        if (e != cudaSuccess) break;
        attach_kernel<<<gridn(na * 32, 256), 256, 0, st>>>(TD, act, (int)na, mask, state, level, parents, levels);
        compact_selected_kernel<<<1, 1024, 0, st>>>(act, (int)na, state, act2, counters + 2);
        int nn = 0;
        e = cudaMemcpyAsync(&nn, counters + 2, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        std::swap(act, act2);
        if (nn == na) {  // no progress at this radius: widen (radius capped at 1)
            if (level >= 0) break;
        }
        na = nn;
        if (level < 0) ++level;
    }
    // roots
    std::vector<int> rootsv(na > 0 ? na : 0);
    if (e == cudaSuccess && na > 0) e = cudaMemcpyAsync(rootsv.data(), act, 4 * na, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    n_roots = na;
    std::vector<long long> rl(rootsv.begin(), rootsv.end());
    if (e == cudaSuccess && na > 0) {
        if (na > kMaxRoots * 64) return set_err(CT_ERR_STATE, "tree build left %lld roots", (long long)na);
        e = cudaMemcpyAsync(roots, rl.data(), 8 * na, cudaMemcpyHostToDevice, st);
    }
    // 3. radii and subtree bounds
    if (e == cudaSuccess) {
        ancestors_kernel<<<gridn(N * 16, 256), 256, 0, st>>>(TD, (int)N, parents, order, (unsigned*)si, sub_min);
        e = cudaGetLastError();
    }
    // 4. children CSR (host assembles: n parents is a few MB)
    std::vector<long long> par(N);
    if (e == cudaSuccess) e = cudaMemcpyAsync(par.data(), parents, 8 * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
        std::vector<long long> off(N + 1, 0), idx(N > 0 ? N : 1);
        for (long long i = 0; i < N; ++i) if (par[i] >= 0) ++off[par[i] + 1];
        for (long long i = 0; i < N; ++i) off[i + 1] += off[i];
        std::vector<long long> fillp(off.begin(), off.end() - 1);
        for (long long i = 0; i < N; ++i) if (par[i] >= 0) idx[fillp[par[i]]++] = i;
        e = cudaMemcpyAsync(child_off, off.data(), 8 * (N + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(child_idx, idx.data(), 8 * N, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFree(order32); cudaFree(act); cudaFree(act2); cudaFree(counters); cudaFree(mask); cudaFree(state);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "tree build: %s", cudaGetErrorString(e));
    has_tree = true;
    return CT_OK;
}
