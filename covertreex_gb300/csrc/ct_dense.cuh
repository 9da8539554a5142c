// ct_dense.cuh — the plain FP32 dense tile shared by the single-tree kernel
// (ct_brute.cu) and the batched persistent kernel (ct_batch.cu).
//
// A tile is QT queries x a candidate range [cbeg, cend).  Each thread holds a
// (QT/16) x 4 block of query x candidate pairs.  The V dot product of a pair is
// evaluated in the exact order of the reference's `dot_f32_simd_inline`
// (src/metric.rs:601-643): sixteen lane accumulators, lane l summing elements
// 16c+l in c order with a separately rounded multiply and add, then
// comb[l] = acc0[l] + acc1[l] and the horizontal tree
// ((c0+c4)+(c2+c6)) + ((c1+c5)+(c3+c7)).  V is stored residue-major (column
// l*(m/16)+c holds element 16c+l) so every lane accumulator is a contiguous dot
// product over m/16 elements.  The epilogue is the batch-path distance of
// src/metric.rs:439-485.  Top-k lists live in shared memory in (dist, idx)
// order; a candidate tile's entries that beat the k-th are merged by rank.
//
// Queries are either dataset rows named by id (qids) or external rows (new
// points: natural-layout V, raw coordinates and p), which the tile permutes,
// scales by the tree's inverse lengthscales and normalises while loading, with
// the arithmetic of the dataset's own setup (ct_setup.cu).
#pragma once
#include "ct_common.cuh"

namespace ct {
namespace dense {

constexpr int kThreads = 256;
constexpr int kCT = 64;  // candidates per candidate tile

// residue visiting order: (acc0[l], acc1[l]) pairs in reduction-tree order
__device__ __forceinline__ int residue_order(int s) {
    // {0, 8, 4, 12, 2, 10, 6, 14, 1, 9, 5, 13, 3, 11, 7, 15}: bit-reversal of s
    return (int)(__brev((unsigned)s) >> 28);
}

struct Smem {
    // byte offsets
    size_t a, b, ds, ld, li, tmp, xq, xc, nq, nc, pq, pc, qid, cnt, total;
};

__host__ __device__ inline Smem layout(int qt, int m, int d, int k) {
    Smem L;
    const int m16 = m / 16;
    size_t off = 0;
    auto take = [&](size_t bytes) { size_t o = off; off += (bytes + 15) & ~size_t(15); return o; };
    // row strides: m + 4 / m16 + 4 floats (16-byte rows for the vector path); the
    // scalar path uses m + 1 / m16 + 1 inside the same space
    L.a = take(sizeof(float) * qt * (m + 4));
    L.b = take(sizeof(float) * 2 * kCT * (m16 + 4));
    L.ds = take(sizeof(float) * qt * (kCT + 1));
    L.ld = take(sizeof(float) * qt * k);
    L.li = take(sizeof(int) * qt * k);
    L.tmp = take(sizeof(float) * 8 * 2 * 64 + sizeof(int) * 8 * 2 * 64);
    L.xq = take(sizeof(float) * qt * d);
    L.xc = take(sizeof(float) * kCT * d);
    L.nq = take(sizeof(float) * qt);
    L.nc = take(sizeof(float) * kCT);
    L.pq = take(sizeof(float) * qt);
    L.pc = take(sizeof(float) * kCT);
    L.qid = take(sizeof(long long) * qt);
    L.cnt = take(sizeof(int) * qt);
    L.total = off;
    return L;
}

__device__ __forceinline__ void cp_async16(void* smem_dst, const void* gsrc) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc));
}
__device__ __forceinline__ void cp_async4(void* smem_dst, const void* gsrc) {
    unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

// Merge the passing candidates of one tile into query qi's sorted list.
// Called by one full warp.  Lane's two slots are candidates lane and lane+32.
__device__ inline void merge_tile_into_list(float* ld, int* li, int& cnt, int k, float d0, int i0, bool p0, float d1,
                                            int i1, bool p1, float* td, int* ti, float* sd, int* si) {
    const int lane = threadIdx.x & 31;
    unsigned m0 = __ballot_sync(0xffffffffu, p0);
    unsigned m1 = __ballot_sync(0xffffffffu, p1);
    int n0 = __popc(m0);
    int nnew = n0 + __popc(m1);
    unsigned below = (1u << lane) - 1u;
    if (p0) { int pos = __popc(m0 & below); td[pos] = d0; ti[pos] = i0; }
    if (p1) { int pos = n0 + __popc(m1 & below); td[pos] = d1; ti[pos] = i1; }
    __syncwarp();
    // rank new entries among themselves -> sorted copy in sd/si
    for (int e = lane; e < nnew; e += 32) {
        float de = td[e]; int ie = ti[e];
        int r = 0;
        for (int f = 0; f < nnew; ++f) r += nb_less(td[f], ti[f], de, ie) ? 1 : 0;
        sd[r] = de; si[r] = ie;
    }
    __syncwarp();
    const int L = cnt;
    // gather final positions in registers first, then write
    float outd[4]; int outi[4]; int outp[4]; int no = 0;
    float outd2[4]; int outi2[4]; int outp2[4]; int no2 = 0;
    for (int e = lane; e < nnew; e += 32) {
        float de = sd[e]; int ie = si[e];
        int lo = 0, hi = L;  // #list entries < new
        while (lo < hi) { int mid = (lo + hi) >> 1; if (nb_less(ld[mid], li[mid], de, ie)) lo = mid + 1; else hi = mid; }
        outd[no] = de; outi[no] = ie; outp[no] = e + lo; ++no;
    }
    for (int e = lane; e < L; e += 32) {
        float de = ld[e]; int ie = li[e];
        int lo = 0, hi = nnew;  // #new entries < list entry
        while (lo < hi) { int mid = (lo + hi) >> 1; if (nb_less(sd[mid], si[mid], de, ie)) lo = mid + 1; else hi = mid; }
        outd2[no2] = de; outi2[no2] = ie; outp2[no2] = e + lo; ++no2;
    }
    __syncwarp();
    for (int t = 0; t < no; ++t) if (outp[t] < k) { ld[outp[t]] = outd[t]; li[outp[t]] = outi[t]; }
    for (int t = 0; t < no2; ++t) if (outp2[t] < k) { ld[outp2[t]] = outd2[t]; li[outp2[t]] = outi2[t]; }
    __syncwarp();
    cnt = min(k, L + nnew);
}

struct Tile {
    // candidates: the tree's device-resident metric (ct_setup.cu layout)
    const float* vperm;
    const float* xs;
    const float* norms;
    const float* p;
    long long n;
    int m, d, k, kernel_type, predecessor;
    float var;
    // queries: dataset ids (qids != nullptr) or external rows
    const long long* qids;
    const float* qv;       // external: nq x m, natural column order
    const float* qcoords;  // external: nq x d, unscaled
    const float* qp;       // external: nq
    const float* inv_ls;   // external: d inverse lengthscales of the tree
    long long nq;
    long long q0;          // first query of the tile
    long long cbeg, cend;  // candidate range
    long long* out_idx;    // row g writes out_*[g * out_stride + j], j < k
    float* out_dist;
    long long out_stride;
};

// VEC = 4: shared-memory rows padded to 16 bytes, operands moved and read 4 floats at
// a time (m a multiple of 64); VEC = 1: scalar (any m multiple of 16).  Both add the
// products in the same order, so both give the same bits.
template <int QT, int VEC>
__device__ __forceinline__ void run_tile_v(const Tile& P, unsigned char* smem_raw) {
    const Smem S = layout(QT, P.m, P.d, P.k);
    float* As = (float*)(smem_raw + S.a);
    float* Bs = (float*)(smem_raw + S.b);
    float* Ds = (float*)(smem_raw + S.ds);
    float* Ld = (float*)(smem_raw + S.ld);
    int* Li = (int*)(smem_raw + S.li);
    float* Td = (float*)(smem_raw + S.tmp);
    int* Ti = (int*)(Td + 8 * 2 * 64);
    float* Xq = (float*)(smem_raw + S.xq);
    float* Xc = (float*)(smem_raw + S.xc);
    float* Nq = (float*)(smem_raw + S.nq);
    float* Nc = (float*)(smem_raw + S.nc);
    float* Pq = (float*)(smem_raw + S.pq);
    float* Pc = (float*)(smem_raw + S.pc);
    long long* Qid = (long long*)(smem_raw + S.qid);
    int* Cnt = (int*)(smem_raw + S.cnt);

    constexpr int QPT = QT / 16;  // queries per thread
    const int tid = threadIdx.x;
    const int lane = tid & 31, warp = tid >> 5;
    const int tq = tid >> 4, tc = tid & 15;
    const int m = P.m, m16 = m / 16, d = P.d, k = P.k;
    const int AST = VEC == 4 ? m + 4 : m + 1, BST = VEC == 4 ? m16 + 4 : m16 + 1;
    const long long n = P.n;
    const bool ext = P.qids == nullptr;
    const long long q0 = P.q0;
    const long long cl = P.cend < n ? P.cend : n;  // candidate limit

    // ---- load query tile.  Qid: dataset id (internal), row (external), -1 = padding
    for (int qi = tid; qi < QT; qi += kThreads) {
        long long g = q0 + qi;
        long long id;
        if (ext) {
            id = g < P.nq ? g : -1;
        } else {
            id = g < P.nq ? P.qids[g] : -1;
            if (id >= P.n) id = -1;  // ids outside [0, n) give an all-padding row
            if (id < 0) id = -1;
        }
        Qid[qi] = id;
        Cnt[qi] = 0;
        if (ext) {
            float s = 0.f;
            for (int c = 0; c < d; ++c) {
                float x = id >= 0 ? __fmul_rn(P.qcoords[id * d + c], P.inv_ls[c]) : 0.f;
                Xq[qi * d + c] = x;
                s = __fadd_rn(s, __fmul_rn(x, x));
            }
            Nq[qi] = s;
            Pq[qi] = id >= 0 ? P.qp[id] : 1.f;
        } else {
            Nq[qi] = id >= 0 ? P.norms[id] : 0.f;
            Pq[qi] = id >= 0 ? P.p[id] : 1.f;
        }
    }
    __syncthreads();
    if (ext) {
        for (int e = tid; e < QT * m; e += kThreads) {
            int qi = e / m, col = e - qi * m;  // natural column 16c + l -> residue-major l*m16 + c
            long long id = Qid[qi];
            As[qi * AST + (col & 15) * m16 + (col >> 4)] = id >= 0 ? P.qv[id * m + col] : 0.f;
        }
    } else {
        for (int e = tid; e < QT * m; e += kThreads) {
            int qi = e / m, c = e - qi * m;
            long long id = Qid[qi];
            As[qi * AST + c] = id >= 0 ? P.vperm[id * m + c] : 0.f;
        }
        for (int e = tid; e < QT * d; e += kThreads) {
            int qi = e / d, c = e - qi * d;
            long long id = Qid[qi];
            Xq[e] = id >= 0 ? P.xs[id * d + c] : 0.f;
        }
    }
    long long jend = cl;
    if (P.predecessor && !ext) {
        long long mx = 0;
        for (int qi = 0; qi < QT; ++qi) mx = Qid[qi] > mx ? Qid[qi] : mx;
        jend = mx < cl ? mx : cl;
    }
    __syncthreads();

    for (long long j0 = P.cbeg; j0 < jend; j0 += kCT) {
        // candidate scalars
        for (int cj = tid; cj < kCT; cj += kThreads) {
            long long g = j0 + cj;
            Nc[cj] = g < cl ? P.norms[g] : 0.f;
            Pc[cj] = g < cl ? P.p[g] : 1.f;
        }
        for (int e = tid; e < kCT * d; e += kThreads) {
            int cj = e / d, c = e - cj * d;
            long long g = j0 + cj;
            Xc[e] = g < cl ? P.xs[g * d + c] : 0.f;
        }
        auto stage = [&](int s, int buf) {
            const int l = residue_order(s);
            float* dst = Bs + buf * kCT * BST;
            if (VEC == 4) {
                const int m4 = m16 >> 2;
                for (int e = tid; e < kCT * m4; e += kThreads) {
                    int cj = e / m4, c = (e - cj * m4) << 2;
                    long long g = j0 + cj;
                    if (g < cl) cp_async16(dst + cj * BST + c, P.vperm + g * m + l * m16 + c);
                    else *(float4*)(dst + cj * BST + c) = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            } else {
                for (int e = tid; e < kCT * m16; e += kThreads) {
                    int cj = e / m16, c = e - cj * m16;
                    long long g = j0 + cj;
                    if (g < cl) cp_async4(dst + cj * BST + c, P.vperm + g * m + l * m16 + c);
                    else dst[cj * BST + c] = 0.f;
                }
            }
            cp_async_commit();
        };
        stage(0, 0);

        float h[QPT][4], cA[QPT][4], sA[QPT][4], t0[QPT][4];
        for (int s = 0; s < 16; ++s) {
            cp_async_wait_all();
            __syncthreads();
            if (s + 1 < 16) stage(s + 1, (s + 1) & 1);
            const int l = residue_order(s);
            const float* Bb = Bs + (s & 1) * kCT * BST;
            float acc[QPT][4];
#pragma unroll
            for (int a = 0; a < QPT; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
            const float* Ab = As + l * m16;
            if (VEC == 4) {
#pragma unroll 2
                for (int c = 0; c < m16; c += 4) {
                    float4 av[QPT], bv[4];
#pragma unroll
                    for (int a = 0; a < QPT; ++a) av[a] = *(const float4*)(Ab + (tq + 16 * a) * AST + c);
#pragma unroll
                    for (int b = 0; b < 4; ++b) bv[b] = *(const float4*)(Bb + (tc + 16 * b) * BST + c);
#pragma unroll
                    for (int a = 0; a < QPT; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) {
                            float t = acc[a][b];
                            t = __fadd_rn(__fmul_rn(av[a].x, bv[b].x), t);
                            t = __fadd_rn(__fmul_rn(av[a].y, bv[b].y), t);
                            t = __fadd_rn(__fmul_rn(av[a].z, bv[b].z), t);
                            t = __fadd_rn(__fmul_rn(av[a].w, bv[b].w), t);
                            acc[a][b] = t;
                        }
                }
            } else {
#pragma unroll 4
                for (int c = 0; c < m16; ++c) {
                    float av[QPT], bv[4];
#pragma unroll
                    for (int a = 0; a < QPT; ++a) av[a] = Ab[(tq + 16 * a) * AST + c];
#pragma unroll
                    for (int b = 0; b < 4; ++b) bv[b] = Bb[(tc + 16 * b) * BST + c];
#pragma unroll
                    for (int a = 0; a < QPT; ++a)
#pragma unroll
                        for (int b = 0; b < 4; ++b) acc[a][b] = __fadd_rn(__fmul_rn(av[a], bv[b]), acc[a][b]);
                }
            }
            // fold into the reduction tree
#pragma unroll
            for (int a = 0; a < QPT; ++a)
#pragma unroll
                for (int b = 0; b < 4; ++b) {
                    float v = acc[a][b];
                    switch (s) {
                        case 0: case 2: case 4: case 6: case 8: case 10: case 12: case 14:
                            h[a][b] = v; break;
                        case 1: case 5: case 9: case 13:
                            cA[a][b] = __fadd_rn(h[a][b], v); break;
                        case 3: case 11:
                            sA[a][b] = __fadd_rn(cA[a][b], __fadd_rn(h[a][b], v)); break;
                        case 7:
                            t0[a][b] = __fadd_rn(sA[a][b], __fadd_rn(cA[a][b], __fadd_rn(h[a][b], v))); break;
                        case 15: {
                            float s3 = __fadd_rn(cA[a][b], __fadd_rn(h[a][b], v));
                            float t1 = __fadd_rn(sA[a][b], s3);
                            h[a][b] = __fadd_rn(t0[a][b], t1);  // final dot in h
                        } break;
                    }
                }
        }
        // ---- epilogue: distances into Ds
#pragma unroll
        for (int a = 0; a < QPT; ++a) {
            const int qi = tq + 16 * a;
            const long long gq = Qid[qi];
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int cj = tc + 16 * b;
                const long long gc = j0 + cj;
                float dist = __int_as_float(0x7f800000);
                bool valid = gq >= 0 && gc < cl && (ext || !P.predecessor || gc < gq);
                if (valid) {
                    if (!ext && gq == gc) {
                        dist = 0.f;
                    } else {
                        float d2 = coord_d2_batch(Xq + qi * d, Xc + cj * d, d, Nq[qi], Nc[cj]);
                        float kv = kernel_value_batch(d2, P.var, P.kernel_type);
                        dist = residual_from_parts(kv, h[a][b], Pq[qi], Pc[cj]);
                    }
                }
                Ds[qi * (kCT + 1) + cj] = dist;
            }
        }
        __syncthreads();
        // ---- selection: warp w owns queries w, w+8, ...
        float* td = Td + warp * 2 * 64;
        int* ti = Ti + warp * 2 * 64;
        for (int qi = warp; qi < QT; qi += kThreads / 32) {
            if (Qid[qi] < 0) continue;
            int cnt = Cnt[qi];
            float* ld = Ld + qi * k;
            int* li = Li + qi * k;
            float taud = cnt >= k ? ld[k - 1] : __int_as_float(0x7f800000);
            int taui = cnt >= k ? li[k - 1] : 0x7fffffff;
            float d0 = Ds[qi * (kCT + 1) + lane];
            float d1 = Ds[qi * (kCT + 1) + lane + 32];
            int i0 = (int)(j0 + lane), i1 = (int)(j0 + lane + 32);
            bool p0 = d0 < __int_as_float(0x7f800000) && (cnt < k || nb_less(d0, i0, taud, taui));
            bool p1 = d1 < __int_as_float(0x7f800000) && (cnt < k || nb_less(d1, i1, taud, taui));
            if (__any_sync(0xffffffffu, p0 || p1)) {
                merge_tile_into_list(ld, li, cnt, k, d0, i0, p0, d1, i1, p1, td, ti, td + 64, ti + 64);
                if (lane == 0) Cnt[qi] = cnt;
            }
        }
        __syncthreads();
    }

    // ---- write results (dataset ids; -1 / FLT_MAX padding)
    for (int e = tid; e < QT * k; e += kThreads) {
        int qi = e / k, j = e - qi * k;
        long long g = q0 + qi;
        if (g >= P.nq) continue;
        int cnt = Cnt[qi];
        bool ok = j < cnt;
        P.out_idx[g * P.out_stride + j] = ok ? (long long)Li[qi * k + j] : -1LL;
        P.out_dist[g * P.out_stride + j] = ok ? Ld[qi * k + j] : CT_FLT_MAX;
    }
}

template <int QT>
__device__ __forceinline__ void run_tile(const Tile& P, unsigned char* smem_raw) {
    if ((P.m & 63) == 0) run_tile_v<QT, 4>(P, smem_raw);
    else run_tile_v<QT, 1>(P, smem_raw);
}

}  // namespace dense
}  // namespace ct
