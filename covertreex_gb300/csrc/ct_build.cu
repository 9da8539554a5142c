// ct_build.cu — device cover-tree build: the batch insert of the reference's
// PCCT path (prefix-doubling groups, covertreex/algo/batch/insert.py:671-803 with
// prefix_slices, algo/order/helpers.py:59-71; traversal level and parent, conflict
// graph, MIS, selected / dominated insertion, insert.py:43-640) and of its Rust
// build_pcct2_residual_tree (far-set conflicts at radius 2^l, MIS, leaders and
// attached non-leaders, src/algo/batch/mod.rs:447-999), re-designed for one GPU.
//
//  1. Node order: Hilbert keys + LSD radix sort (ct_order.cu).  Rows whose residual
//     variance is tiny (p < 1/kSideIsp^2: the inducing rows, p ~ 1e-6) are moved to
//     the end and kept out of the tree: their distances carry errors of order 1 in
//     FP32 and no cover radius could prune a subtree holding one; every query scores
//     them directly (they are roots without children, like the reference's dropped
//     points).  The first remaining node is the root, at level 0 (radius 2^0 = 1
//     covers every residual distance).
//  2. Prefix doubling: the other nodes are inserted in groups [1,2), [2,4), [4,8), ...
//     (prefix_slices).  For a group G inserted into the tree T built so far:
//       * traversal: each x in G finds its nearest node t(x) in T (dense exact FP32
//         search, ct_dense.cuh) and the level l(x) = min(ceil(log2 d) - 1, level(t) - 1),
//         so that d(x, t) <= 2^(l+1) whenever the parent's level allows it;
//       * conflict graph: x and y in G conflict when d(x, y) <= 2^min(l(x), l(y)); the
//         candidate pairs are each point's kConflictK nearest group members (the degree
//         cap of the reference's conflict_degree_cap), made symmetric without duplicates;
//       * seeded Luby MIS on the device (ct_mis.cu, the reference's _mis_numba rules);
//       * selected points join at level l(x) under t(x); every dominated point joins
//         under its nearest selected neighbour at level min(l(x) - 1, level(parent) - 1,
//         floor(log2 d)) (insert.py:586-640).
//  3. Radii: si[a] = max over descendants x of the FP32 distance d(a, x) (exact, by
//     walking every node's ancestor chain); si_up[a] = max of a certified upper bound
//     of the ideal metric's d(a, x) (the FP32 value plus its error bound, see
//     ct_traverse.cu); sub_isp[a] = max over the subtree of 1/sqrt(p); subtree_min[a]
//     = min dataset id below a (compute_subtree_index_bounds, src/tree.rs:144-185).
//  4. Children in CSR (child_off / child_idx); roots (the root and the side rows).
//
// Distances use the reference's batch-path f32 arithmetic (the dense form's device
// functions), so every distance the build evaluates is bit-identical to the one the
// dense form and the traversal evaluate for the same pair.
#include <climits>
#include <cmath>

#include <algorithm>
#include <vector>

#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_tree.h"
#include "ct_treebound.cuh"

namespace ct {
namespace treeb {

constexpr int kLevelTop = 0;
constexpr int kLevelMin = -30;
constexpr int kConflictK = 16;

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

// Smallest L with d <= 2^L (d > 0), as an integer; kLevelMin + 1 for d == 0.
__device__ __forceinline__ int ceil_log2(float d) {
    if (!(d > 0.f)) return kLevelMin + 1;
    int e;
    const float f = frexpf(d, &e);  // d = f 2^e, f in [0.5, 1)
    return f == 0.5f ? e - 1 : e;
}
// Largest L with 2^L <= d (d > 0); kLevelMin for d == 0.
__device__ __forceinline__ int floor_log2(float d) {
    if (!(d > 0.f)) return kLevelMin;
    int e;
    frexpf(d, &e);
    return e - 1;
}

// Traversal level of the group's points: t[i] = nearest tree node, td[i] its distance.
__global__ void group_level_kernel(long long s, long long g, const long long* __restrict__ t,
                                   const float* __restrict__ td, const int* __restrict__ levels,
                                   int* __restrict__ lvl) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g) return;
    const long long pnt = t[i];
    const int pl = pnt >= 0 ? levels[pnt] : kLevelTop;
    int l = ceil_log2(td[i]) - 1;
    if (l > pl - 1) l = pl - 1;
    if (l < kLevelMin) l = kLevelMin;
    lvl[i] = l;
}

__device__ __forceinline__ bool lists_member(const long long* __restrict__ cidx, int kc, long long row, long long x) {
    for (int j = 0; j < kc; ++j)
        if (cidx[row * kc + j] == x) return true;
    return false;
}

// Conflict edges from the group's kNN lists (node ids): x -- y when y is among x's
// nearest group members and d(x, y) <= 2^min(l(x), l(y)).  x's row always gets y;
// y's row gets x only when x is not on y's own list (y adds it itself otherwise), so
// no edge is stored twice.  pass 0 counts, pass 1 fills (with the distances).
__global__ void conflict_edges_kernel(long long s, long long g, const long long* __restrict__ cidx,
                                      const float* __restrict__ cd, int kc, const int* __restrict__ lvl,
                                      int pass, int* __restrict__ deg, int* __restrict__ cursor,
                                      long long* __restrict__ indices, float* __restrict__ w) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g) return;
    const long long x = s + i;
    for (int j = 0; j < kc; ++j) {
        const long long y = cidx[i * kc + j];
        if (y < s || y >= s + g || y == x) continue;
        const long long yi = y - s;
        const int l = min(lvl[i], lvl[yi]);
        const float dd = cd[i * kc + j];
        if (!(dd <= ldexpf(1.f, l))) continue;
        const bool reverse = !lists_member(cidx, kc, yi, x);
        if (pass == 0) {
            atomicAdd(&deg[i], 1);
            if (reverse) atomicAdd(&deg[yi], 1);
        } else {
            const int a = atomicAdd(&cursor[i], 1);
            indices[a] = yi;
            w[a] = dd;
            if (reverse) {
                const int b = atomicAdd(&cursor[yi], 1);
                indices[b] = i;
                w[b] = dd;
            }
        }
    }
}

// Selected points join under their traversal parent; dominated points under their
// nearest selected neighbour (ties to the lower node), one level below it at most.
__global__ void group_assign_kernel(long long s, long long g, const signed char* __restrict__ sel,
                                    const long long* __restrict__ indptr, const long long* __restrict__ indices,
                                    const float* __restrict__ w, const long long* __restrict__ t,
                                    const int* __restrict__ lvl, long long* __restrict__ parents,
                                    int* __restrict__ levels, int* __restrict__ selected_count) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= g) return;
    const long long x = s + i;
    if (sel[i]) {
        parents[x] = t[i];
        levels[x] = lvl[i];
        atomicAdd(selected_count, 1);
        return;
    }
    float best = CT_FLT_MAX;
    long long bj = -1;
    for (long long o = indptr[i]; o < indptr[i + 1]; ++o) {
        const long long j = indices[o];
        if (!sel[j]) continue;
        if (w[o] < best || (w[o] == best && j < bj)) { best = w[o]; bj = j; }
    }
    if (bj < 0) {  // cannot happen for a maximal independent set; keep the traversal parent
        parents[x] = t[i];
        levels[x] = lvl[i];
        return;
    }
    int l = lvl[i] - 1;
    l = min(l, lvl[bj] - 1);
    l = min(l, floor_log2(best));
    if (l < kLevelMin) l = kLevelMin;
    parents[x] = s + bj;
    levels[x] = l;
}

// Per node: 1/sqrt(p) rounded up and ||v|| rounded up (inputs of the certified bounds).
__global__ void node_scalars_kernel(TreeData T, long long n, float* __restrict__ isp, float* __restrict__ vn) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float* v = T.v + (size_t)r * T.m;
    double s = 0.0;
    for (int c = 0; c < T.m; ++c) s += (double)v[c] * (double)v[c];
    vn[r] = (float)(sqrt(s) * (1.0 + 1e-6));
    const double pr = (double)T.p[r];
    isp[r] = pr > 0.0 ? (float)(1.0 / sqrt(pr) * (1.0 + 1e-6)) : 3.0e38f;
}

// si, si_up, subtree_min and sub_isp by walking every node's ancestor chain (one
// half-warp per node); atomicMax on the bits of non-negative floats orders them.
__global__ void ancestors_kernel(TreeData T, BoundModel B, int n, const long long* __restrict__ parents,
                                 const long long* __restrict__ order, const float* __restrict__ isp,
                                 const float* __restrict__ vn, unsigned* __restrict__ si_bits,
                                 unsigned* __restrict__ si_up_bits, unsigned* __restrict__ sub_isp_bits,
                                 long long* __restrict__ sub_min) {
    const int hw = (blockIdx.x * blockDim.x + threadIdx.x) >> 4;
    if (hw >= n) return;
    const int x = hw;
    const long long ds = order[x];
    const float ispx = isp[x];
    long long a = parents[x];
    int guard = 0;
    while (a >= 0 && guard < 4096) {
        const float dd = half_dist(T, (int)a, x);
        if ((threadIdx.x & 15) == 0) {
            const float delta = pair_delta(B, T.norms[a], T.norms[x], vn[a], vn[x], isp[a], ispx);
            const float up = dist_upper(dd, delta);
            atomicMax(&si_bits[a], __float_as_uint(dd));
            atomicMax(&si_up_bits[a], __float_as_uint(up));
            atomicMax(&sub_isp_bits[a], __float_as_uint(ispx));
            atomicMin((unsigned long long*)&sub_min[a], (unsigned long long)ds);
        }
        a = parents[a];
        ++guard;
    }
}

__global__ void init_tree_kernel(long long n, long long* parents, int* levels, unsigned* si_bits,
                                 unsigned* si_up_bits, unsigned* sub_isp_bits, const float* isp, long long* sub_min,
                                 const long long* order) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    parents[i] = -1;
    levels[i] = INT_MIN;
    si_bits[i] = 0u;
    si_up_bits[i] = 0u;
    sub_isp_bits[i] = __float_as_uint(isp[i]);
    sub_min[i] = order[i];
}

__global__ void gather_rows_kernel(const float* __restrict__ src, const long long* __restrict__ order, long long n,
                                   int w, float* __restrict__ dst) {
    const long long total = n * (long long)w;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / w;
        dst[e] = src[order[r] * w + (e - r * w)];
    }
}

__global__ void iota_kernel(long long s, long long g, long long* out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < g) out[i] = s + i;
}

__global__ void inverse_kernel(const long long* order, long long n, long long* inv) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) inv[order[i]] = i;
}

__global__ void widen_kernel(const int* in, long long n, long long* out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}

__global__ void set_root_kernel(long long* parents, int* levels) {
    parents[0] = -1;
    levels[0] = kLevelTop;
}

}  // namespace treeb
}  // namespace ct

using namespace ct::treeb;

static inline unsigned gridn(long long n, int b) { return (unsigned)((n + b - 1) / b); }

int ct_tree::build_tree(const float* /*v_dataset*/, const float* /*coords_dataset*/, cudaStream_t st) {
    return grow_tree(nullptr, st);
}

// base == nullptr: the build described at the top of this file.  Otherwise this handle
// holds base's rows followed by new rows (ct_tree_extend): base's tree nodes keep their
// node numbers, parents and levels, the new rows (ordered among themselves) follow them
// and are inserted by the same prefix-doubling groups (the batch insert of the reference's
// CoverTree.insert, api/pcct.py:171-197), and the tiny-p rows of both come last.
int ct_tree::grow_tree(const ct_tree* base, cudaStream_t st) {
    const long long N = n;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** ptr, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(ptr, bytes ? bytes : 16); };
    A((void**)&order, 8 * N); A((void**)&inv, 8 * N); A((void**)&parents, 8 * N); A((void**)&levels, 4 * N);
    A((void**)&si, 4 * N); A((void**)&si_up, 4 * N); A((void**)&sub_isp, 4 * N); A((void**)&sub_min, 8 * N);
    A((void**)&child_off, 8 * (N + 1)); A((void**)&child_idx, 8 * N); A((void**)&roots, 8 * N);
    A((void**)&tvnat, sizeof(float) * N * m); A((void**)&txs, sizeof(float) * N * d);
    A((void**)&tnorms, sizeof(float) * N); A((void**)&tp, sizeof(float) * N);
    A((void**)&tisp, sizeof(float) * N); A((void**)&tvn, sizeof(float) * N);
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "tree build allocation: %s", cudaGetErrorString(e));

    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaEventCreate(&ev0);
    cudaEventCreate(&ev1);
    cudaEventRecord(ev0, st);

    // 1. node order: Hilbert (or natural), then rows with tiny p moved to the end
    const long long nb = base ? base->n : 0;               // rows of the base handle
    const long long n_tree_base = base ? base->n - base->n_side : 0;
    const long long nr = N - nb;                           // rows ordered here
    int* order32 = nullptr;
    A((void**)&order32, 4 * (nr > 0 ? nr : 1));
    if (e == cudaSuccess && nr > 0) {
        if (order_mode == CT_ORDER_NATURAL) {
            std::vector<int> id(nr);
            for (long long i = 0; i < nr; ++i) id[i] = (int)i;
            e = cudaMemcpyAsync(order32, id.data(), 4 * nr, cudaMemcpyHostToDevice, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        } else {
            e = ct::compute_order(coords_raw + (size_t)nb * d, nr, d, (d == 3 && order_mode == CT_ORDER_MORTON) ? 2 : 1,
                                  order32, st);
        }
    }
    std::vector<int> ord(nr > 0 ? nr : 1);
    std::vector<float> ph(nr > 0 ? nr : 1);
    std::vector<long long> bord(nb > 0 ? nb : 1);
    if (e == cudaSuccess && nr > 0) e = cudaMemcpyAsync(ord.data(), order32, 4 * nr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nr > 0) e = cudaMemcpyAsync(ph.data(), p + nb, 4 * nr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && nb > 0) e = cudaMemcpyAsync(bord.data(), base->order, 8 * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    std::vector<long long> ord64;
    n_side = 0;
    if (e == cudaSuccess) {
        ord64.reserve(N);
        const float pside = 1.f / (ct::kSideIsp * ct::kSideIsp);
        for (long long i = 0; i < n_tree_base; ++i) ord64.push_back(bord[i]);
        for (long long i = 0; i < nr; ++i) if (!(ph[ord[i]] < pside)) ord64.push_back(nb + ord[i]);
        const long long n_tree = (long long)ord64.size();
        for (long long i = n_tree_base; i < nb; ++i) ord64.push_back(bord[i]);
        for (long long i = 0; i < nr; ++i) if (ph[ord[i]] < pside) ord64.push_back(nb + ord[i]);
        n_side = N - n_tree;
        e = cudaMemcpyAsync(order, ord64.data(), 8 * N, cudaMemcpyHostToDevice, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // ord64 is a host buffer
    cudaFree(order32);
    const long long n_tree = N - n_side;
    if (e == cudaSuccess) {
        inverse_kernel<<<gridn(N, 256), 256, 0, st>>>(order, N, inv);
        gather_rows_kernel<<<152 * 8, 256, 0, st>>>(vnat, order, N, m, tvnat);
        gather_rows_kernel<<<152 * 8, 256, 0, st>>>(xs, order, N, d, txs);
        gather_rows_kernel<<<gridn(N, 256), 256, 0, st>>>(norms, order, N, 1, tnorms);
        gather_rows_kernel<<<gridn(N, 256), 256, 0, st>>>(p, order, N, 1, tp);
        e = cudaGetLastError();
    }
    TreeData TD{tvnat, txs, tnorms, tp, m, d, kernel_type, var};
    if (e == cudaSuccess) {
        node_scalars_kernel<<<gridn(N, 256), 256, 0, st>>>(TD, N, tisp, tvn);
        init_tree_kernel<<<gridn(N, 256), 256, 0, st>>>(N, parents, levels, (unsigned*)si, (unsigned*)si_up,
                                                        (unsigned*)sub_isp, tisp, sub_min, order);
        e = cudaGetLastError();
    }
    // the base tree's nodes keep their parents and levels (node numbers below n_tree_base)
    if (e == cudaSuccess && n_tree_base > 0) {
        e = cudaMemcpyAsync(parents, base->parents, 8 * n_tree_base, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(levels, base->levels, 4 * n_tree_base, cudaMemcpyDeviceToDevice, st);
    }
    // bound model of the tree: dataset maxima of ||v|| and of the scaled norms
    if (e == cudaSuccess) {
        std::vector<float> hv(N), hn(N);
        e = cudaMemcpyAsync(hv.data(), tvn, 4 * N, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hn.data(), tnorms, 4 * N, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        float vmax = 0.f, nmax = 0.f;
        for (long long i = 0; i < N; ++i) { vmax = std::max(vmax, hv[i]); nmax = std::max(nmax, hn[i]); }
        bound = ct::make_bound_model(m, d, kernel_type, var, vmax, nmax);
    }

    // node-order residue-major V for the dense searches of the build (freed at the end)
    float* tvperm = nullptr;
    A((void**)&tvperm, sizeof(float) * N * m);
    if (e == cudaSuccess) {
        gather_rows_kernel<<<152 * 8, 256, 0, st>>>(vperm, order, N, m, tvperm);
        e = cudaGetLastError();
    }

    // 2. prefix-doubling groups over nodes [1, n_tree) (over the new nodes [n_tree_base,
    //    n_tree) when growing a base tree)
    build_groups = base ? base->build_groups : 0;
    build_conflict_edges = base ? base->build_conflict_edges : 0;
    build_selected = base ? base->build_selected : 0;
    long long gmax = n_tree > 1 ? (n_tree - 1 + 1) / 2 + 1 : 1;
    long long *gq = nullptr, *t_idx = nullptr, *c_idx = nullptr, *indptr = nullptr, *indices = nullptr;
    float *t_d = nullptr, *c_d = nullptr, *w = nullptr;
    int *lvl = nullptr, *deg = nullptr, *cursor = nullptr, *counters = nullptr;
    signed char* sel = nullptr;
    const int kc = (int)std::min<long long>(kConflictK + 1, std::max<long long>(gmax, 1));
    A((void**)&gq, 8 * gmax); A((void**)&t_idx, 8 * gmax); A((void**)&t_d, 4 * gmax);
    A((void**)&c_idx, 8 * gmax * kc); A((void**)&c_d, 4 * gmax * kc);
    A((void**)&lvl, 4 * gmax); A((void**)&deg, 4 * (gmax + 1)); A((void**)&cursor, 4 * (gmax + 1));
    A((void**)&indptr, 8 * (gmax + 1)); A((void**)&indices, 8 * gmax * 2 * kc); A((void**)&w, 4 * gmax * 2 * kc);
    A((void**)&sel, gmax); A((void**)&counters, 16);
    int smem_optin = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess && n_tree > 0 && n_tree_base == 0) {
        set_root_kernel<<<1, 1, 0, st>>>(parents, levels);
        e = cudaGetLastError();
    }
    ct::BruteParams BP;
    BP.vperm = tvperm; BP.xs = txs; BP.norms = tnorms; BP.p = tp; BP.n = N; BP.m = m; BP.d = d;
    BP.kernel_type = kernel_type; BP.predecessor = 0; BP.var = var;
    long long s = n_tree_base > 0 ? n_tree_base : 1;
    long long size = n_tree_base > 0 ? std::max<long long>(1, std::min(s, n_tree - s)) : 1;
    while (e == cudaSuccess && s < n_tree) {
        const long long g = std::min(size, n_tree - s);
        ++build_groups;
        iota_kernel<<<gridn(g, 256), 256, 0, st>>>(s, g, gq);
        // traversal: nearest node of the tree built so far, nodes [0, s)
        BP.qids = gq; BP.nq = g; BP.k = 1; BP.cbeg = 0; BP.cend = s; BP.out_idx = t_idx; BP.out_dist = t_d;
        int qt = ct::brute_pick_qt(m, d, 1, (size_t)smem_optin);
        if (qt == 0) { e = cudaErrorInvalidValue; break; }
        e = ct::launch_brute_knn(BP, qt, st);
        if (e != cudaSuccess) break;
        group_level_kernel<<<gridn(g, 256), 256, 0, st>>>(s, g, t_idx, t_d, levels, lvl);
        // conflict candidates: nearest group members (the point itself among them)
        const int kk = (int)std::min<long long>(kc, g);
        BP.k = kk; BP.cbeg = s; BP.cend = s + g; BP.out_idx = c_idx; BP.out_dist = c_d;
        qt = ct::brute_pick_qt(m, d, kk, (size_t)smem_optin);
        if (qt == 0) { e = cudaErrorInvalidValue; break; }
        e = ct::launch_brute_knn(BP, qt, st);
        if (e != cudaSuccess) break;
        e = cudaMemsetAsync(deg, 0, 4 * (g + 1), st);
        if (e != cudaSuccess) break;
        conflict_edges_kernel<<<gridn(g, 256), 256, 0, st>>>(s, g, c_idx, c_d, kk, lvl, 0, deg, nullptr, nullptr,
                                                             nullptr);
        // exclusive scan of the degrees into indptr (g + 1 entries; g <= 2^30)
        std::vector<int> hdeg(g + 1);
        e = cudaMemcpyAsync(hdeg.data(), deg, 4 * g, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) break;
        std::vector<long long> hptr(g + 1, 0);
        std::vector<int> hcur(g);
        for (long long i = 0; i < g; ++i) { hptr[i + 1] = hptr[i] + hdeg[i]; hcur[i] = (int)hptr[i]; }
        build_conflict_edges += hptr[g];
        e = cudaMemcpyAsync(indptr, hptr.data(), 8 * (g + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(cursor, hcur.data(), 4 * g, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) break;
        conflict_edges_kernel<<<gridn(g, 256), 256, 0, st>>>(s, g, c_idx, c_d, kk, lvl, 1, nullptr, cursor, indices,
                                                             w);
        e = cudaGetLastError();
        if (e != cudaSuccess) break;
        int iters = 0;
        e = ct::luby_mis_csr(indptr, indices, g, (unsigned long long)(seed + (unsigned long long)build_groups), sel,
                             &iters, st);
        if (e != cudaSuccess) break;
        e = cudaMemsetAsync(counters, 0, 16, st);
        if (e != cudaSuccess) break;
        group_assign_kernel<<<gridn(g, 256), 256, 0, st>>>(s, g, sel, indptr, indices, w, t_idx, lvl, parents, levels,
                                                           counters);
        int hs = 0;
        e = cudaMemcpyAsync(&hs, counters, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // keeps the host vectors alive until copied
        build_selected += hs;
        s += g;
        size = std::min(2 * size, n_tree - s);
        if (size <= 0) size = 1;
    }
    cudaFree(gq); cudaFree(t_idx); cudaFree(t_d); cudaFree(c_idx); cudaFree(c_d); cudaFree(lvl); cudaFree(deg);
    cudaFree(cursor); cudaFree(indptr); cudaFree(indices); cudaFree(w); cudaFree(sel); cudaFree(counters);
    cudaFree(tvperm);

    // 3. radii and subtree bounds
    if (e == cudaSuccess) {
        ancestors_kernel<<<gridn(N * 16, 256), 256, 0, st>>>(TD, bound, (int)N, parents, order, tisp, tvn,
                                                             (unsigned*)si, (unsigned*)si_up, (unsigned*)sub_isp,
                                                             sub_min);
        e = cudaGetLastError();
    }
    // 4. children CSR and roots (host assembles: n parents is a few MB)
    std::vector<long long> par(N);
    if (e == cudaSuccess) e = cudaMemcpyAsync(par.data(), parents, 8 * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) {
        std::vector<long long> off(N + 1, 0), idx(N > 0 ? N : 1), rl;
        for (long long i = 0; i < N; ++i) if (par[i] >= 0) ++off[par[i] + 1]; else rl.push_back(i);
        for (long long i = 0; i < N; ++i) off[i + 1] += off[i];
        std::vector<long long> fillp(off.begin(), off.end() - 1);
        for (long long i = 0; i < N; ++i) if (par[i] >= 0) idx[fillp[par[i]]++] = i;
        n_roots = (int64_t)rl.size();
        e = cudaMemcpyAsync(child_off, off.data(), 8 * (N + 1), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(child_idx, idx.data(), 8 * N, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess && !rl.empty()) e = cudaMemcpyAsync(roots, rl.data(), 8 * rl.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    float ms = 0.f;
    if (e == cudaSuccess) {
        cudaEventRecord(ev1, st);
        cudaEventSynchronize(ev1);
        cudaEventElapsedTime(&ms, ev0, ev1);
    }
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    build_ms = ms;
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "tree build: %s", cudaGetErrorString(e));
    has_tree = true;
    return CT_OK;
}
