/*
 * ct_oracle.c — CPU restatement of covertreex's residual-correlation cover-tree
 * hot path (the `covertreex_backend` Rust crate), used ONLY as test
 * infrastructure: the parity checker for the CUDA engine and the timed CPU
 * baseline in bench.py.  Nothing in the product links or calls this file.
 *
 * Each function names the reference file:line it follows (paths inside the
 * covertreex project).  Arithmetic is plain IEEE binary32 with no FMA
 * contraction (compiled with -ffp-contract=off), matching the x86-64 baseline
 * build of the reference, whose `wide::f32x8::mul_add` lowers to a separate
 * multiply and add when the target has no FMA feature.
 *
 * Two deliberate, documented deviations from the reference:
 *   1. exp(): the reference calls the platform libm expf.  Here `ct_expf`
 *      (Cody-Waite reduction + degree-7 Taylor polynomial, fmaf Horner) is used
 *      so that the CUDA engine, which uses the same function, is bit-identical.
 *      It differs from a correctly-rounded expf by at most 1 ulp.
 *   2. Result heap ties: Rust's BinaryHeap orders neighbours by distance only;
 *      here ties are broken by the lower node index (the engine's contract).
 *   3. The horizontal sum of `wide::f32x8::reduce_add` is taken as the tree
 *      ((l0+l4)+(l2+l6)) + ((l1+l5)+(l3+l7)); the crate's own order is not
 *      vendored in the reference, so this boundary is unpinned.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <limits.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define CT_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* exp: Cody-Waite range reduction (x = n ln2 + r, |r| <= ln2/2) followed by a
 * degree-7 Taylor polynomial in Horner form with fmaf.  Shared verbatim (as
 * arithmetic) with the device version in the CUDA engine.                   */
/* ------------------------------------------------------------------------- */
CT_EXPORT float ct_expf(float x) {
    if (x < -87.0f) return 0.0f;
    if (x > 88.0f) return INFINITY;
    const float log2e = 1.44269504088896341f;
    const float ln2_hi = 0.693145751953125f;        /* 11 significant bits: n*ln2_hi exact */
    const float ln2_lo = 1.42860682030941723e-6f;   /* ln2 - ln2_hi */
    float n = rintf(x * log2e);
    float r = fmaf(-n, ln2_hi, x);
    r = fmaf(-n, ln2_lo, r);
    /* 1/k! for k = 7..0 */
    float p = 1.98412698412698413e-4f;
    p = fmaf(p, r, 1.38888888888888889e-3f);
    p = fmaf(p, r, 8.33333333333333333e-3f);
    p = fmaf(p, r, 4.16666666666666667e-2f);
    p = fmaf(p, r, 1.66666666666666667e-1f);
    p = fmaf(p, r, 0.5f);
    p = fmaf(p, r, 1.0f);
    p = fmaf(p, r, 1.0f);
    return ldexpf(p, (int)n);
}

/* ------------------------------------------------------------------------- */
/* Dot products (src/metric.rs)                                              */
/* ------------------------------------------------------------------------- */

/* wide::f32x8::reduce_add, see header note 3. */
static inline float reduce8(const float c[8]) {
    float s0 = c[0] + c[4], s1 = c[1] + c[5], s2 = c[2] + c[6], s3 = c[3] + c[7];
    return (s0 + s2) + (s1 + s3);
}

/* dot_f32_simd_inline, src/metric.rs:601-643: two 8-lane accumulators over
 * 16-element strides, odd trailing chunk into acc0, lane-wise combine,
 * horizontal reduce, scalar tail. */
CT_EXPORT float ct_dot_simd_inline(const float* a, const float* b, int len) {
    int chunks = len / 8, tail = chunks * 8;
    float acc0[8] = {0}, acc1[8] = {0};
    int i = 0;
    for (int dc = 0; dc < chunks / 2; ++dc) {
        for (int l = 0; l < 8; ++l) acc0[l] = a[i + l] * b[i + l] + acc0[l];
        for (int l = 0; l < 8; ++l) acc1[l] = a[i + 8 + l] * b[i + 8 + l] + acc1[l];
        i += 16;
    }
    if (chunks % 2 == 1)
        for (int l = 0; l < 8; ++l) acc0[l] = a[i + l] * b[i + l] + acc0[l];
    float comb[8];
    for (int l = 0; l < 8; ++l) comb[l] = acc0[l] + acc1[l];
    float r = reduce8(comb);
    for (int j = tail; j < len; ++j) r += a[j] * b[j];
    return r;
}

/* dot_product_simd_slice (f32 branch), src/metric.rs:693-733: per 8-chunk
 * horizontal reduce accumulated into a scalar, scalar tail. */
CT_EXPORT float ct_dot_simd_slice(const float* a, const float* b, int len) {
    int chunks = len / 8, tail = chunks * 8;
    float acc = 0.0f;
    for (int c = 0; c < chunks; ++c) {
        float prod[8];
        for (int l = 0; l < 8; ++l) prod[l] = a[8 * c + l] * b[8 * c + l];
        acc += reduce8(prod);
    }
    for (int j = tail; j < len; ++j) acc += a[j] * b[j];
    return acc;
}

/* dot_parity_f32, src/metric.rs:664-668: f64 accumulation, cast to f32. */
static inline float dot_parity(const float* a, const float* b, int len) {
    double s = 0.0;
    for (int j = 0; j < len; ++j) s += (double)a[j] * (double)b[j];
    return (float)s;
}

/* ------------------------------------------------------------------------- */
/* Residual metric (src/metric.rs:84-177, :180-199, :376-563)                */
/* ------------------------------------------------------------------------- */
typedef struct {
    int64_t n;
    int m, d;
    const float* v;      /* n x m, row-major */
    const float* p;      /* n */
    float* xs;           /* scaled coords n x d (owned) */
    float* norms;        /* n (owned) */
    float var;
    int kernel_type;     /* 0 RBF, 1 Matern52 */
    int parity;          /* COVERTREEX_RESIDUAL_PARITY */
} ct_metric;

/* ResidualMetric::new, src/metric.rs:84-120: inv_ls = 1/ls (|ls|<1e-6 -> 1e-6),
 * scaled coords x*inv_ls, squared norms summed left to right. */
static void metric_init(ct_metric* M, const float* v, const float* p, const float* coords,
                        int64_t n, int m, int d, float var, const float* ls, int n_ls,
                        int kernel_type, int parity) {
    M->n = n; M->m = m; M->d = d; M->v = v; M->p = p; M->var = var;
    M->kernel_type = kernel_type == 1 ? 1 : 0; M->parity = parity;
    M->xs = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1) * (size_t)(d > 0 ? d : 1));
    M->norms = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    float inv_ls[64];
    float fallback = n_ls > 0 ? ls[0] : 1.0f;
    for (int i = 0; i < d && i < 64; ++i) {
        float raw = i < n_ls ? ls[i] : fallback;
        float safe = fabsf(raw) < 1e-6f ? 1e-6f : raw;
        inv_ls[i] = 1.0f / safe;
    }
    for (int64_t r = 0; r < n; ++r) {
        float s = 0.0f;
        for (int c = 0; c < d; ++c) {
            float x = coords[r * d + c] * inv_ls[c];
            M->xs[r * d + c] = x;
            s += x * x;
        }
        M->norms[r] = s;
    }
}

static void metric_free(ct_metric* M) { free(M->xs); free(M->norms); M->xs = NULL; M->norms = NULL; }

/* Batch-path distance, distances_f32_batch_idx_into_with_kth,
 * src/metric.rs:376-487.  Returns sqrt(1-|rho|). */
static float dist_batch(const ct_metric* M, int64_t q, int64_t j) {
    if (q == j) return 0.0f;
    const int d = M->d, m = M->m;
    const float* qc = M->xs + q * d;
    const float* pc = M->xs + j * d;
    float dot_c = 0.0f;
    if (d == 3) {
        dot_c = qc[0] * pc[0] + qc[1] * pc[1] + qc[2] * pc[2];
    } else {
        for (int c = 0; c < d; ++c) dot_c += qc[c] * pc[c];
    }
    float d2 = M->norms[q] + M->norms[j] - 2.0f * dot_c;
    if (d2 < 0.0f) d2 = 0.0f;
    float kval;
    if (M->kernel_type == 0) {
        kval = M->var * ct_expf(-0.5f * d2);
    } else {
        float r = sqrtf(d2);
        float a = 2.2360679775f * r;
        float poly = 1.0f + a + (a * a) * 0.3333333333f;
        kval = M->var * poly * ct_expf(-a);
    }
    const float eps = 1e-9f;
    float pp = M->p[q] * M->p[j];
    float ee = eps * eps;
    float denom = sqrtf(pp > ee ? pp : ee);
    float dot_v = ct_dot_simd_inline(M->v + q * m, M->v + j * m, m);
    float rho = (kval - dot_v) / denom;
    rho = rho > -1.0f ? rho : -1.0f;   /* max(-1) */
    rho = rho < 1.0f ? rho : 1.0f;     /* min(1)  */
    float ds = 1.0f - fabsf(rho);
    return ds > 0.0f ? sqrtf(ds) : 0.0f;
}

/* Scalar-path squared distance, distance_sq_idx_f32, src/metric.rs:489-563.
 * Returns 1-|rho| (the value the build compares with radius^2). */
static float dist_sq_idx(const ct_metric* M, int64_t i, int64_t j) {
    if (i == j) return 0.0f;
    const int d = M->d, m = M->m;
    const float* x = M->xs + i * d;
    const float* y = M->xs + j * d;
    float dot_s = M->parity ? dot_parity(x, y, d) : ct_dot_simd_slice(x, y, d);
    float d2 = M->norms[i] + M->norms[j] - 2.0f * dot_s;
    if (d2 < 0.0f) d2 = 0.0f;
    float kval;
    if (M->kernel_type == 0) {
        kval = M->var * ct_expf(-0.5f * d2);
    } else {
        float r = sqrtf(d2);
        float a = 2.2360679775f * r;
        float poly = 1.0f + a + (a * a) / 3.0f;
        kval = M->var * poly * ct_expf(-a);
    }
    const float eps = 1e-9f;
    float pp = M->p[i] * M->p[j];
    float ee = eps * eps;
    float denom = sqrtf(pp > ee ? pp : ee);
    const float* v1 = M->v + i * m;
    const float* v2 = M->v + j * m;
    float dot = M->parity ? dot_parity(v1, v2, m) : ct_dot_simd_slice(v1, v2, m);
    float rho = denom > 0.0f ? (kval - dot) / denom : 0.0f;
    rho = rho > -1.0f ? rho : -1.0f;
    rho = rho < 1.0f ? rho : 1.0f;
    float ds = 1.0f - fabsf(rho);
    return ds > 0.0f ? ds : 0.0f;
}

/* distance_idx, src/metric.rs:565-567. */
static inline float dist_idx(const ct_metric* M, int64_t i, int64_t j) {
    return sqrtf(dist_sq_idx(M, i, j));
}

/* ------------------------------------------------------------------------- */
/* Morton order, src/pcct.rs:3-67                                            */
/* ------------------------------------------------------------------------- */
static inline uint64_t part1by2(uint64_t n) {
    n &= 0x1fffffULL;
    n = (n | (n << 32)) & 0x1f00000000ffffULL;
    n = (n | (n << 16)) & 0x1f0000ff0000ffULL;
    n = (n | (n << 8)) & 0x100f00f00f00f00fULL;
    n = (n | (n << 4)) & 0x10c30c30c30c30c3ULL;
    n = (n | (n << 2)) & 0x1249249249249249ULL;
    return n;
}

CT_EXPORT uint64_t ct_morton3(uint32_t x, uint32_t y, uint32_t z) {
    return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2);
}

typedef struct { uint64_t key; int64_t idx; } key_idx;
static int cmp_key_idx(const void* a, const void* b) {
    const key_idx* x = (const key_idx*)a; const key_idx* y = (const key_idx*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return x->idx < y->idx ? -1 : (x->idx > y->idx);
}

/* hilbert_like_order, src/pcct.rs:27-67 (stable sort by code). */
CT_EXPORT void ct_morton_order(const float* coords, int64_t n, int d, int64_t* order, uint64_t* codes_out) {
    if (n <= 0) return;
    if (d != 3) {
        for (int64_t i = 0; i < n; ++i) { order[i] = i; if (codes_out) codes_out[i] = 0; }
        return;
    }
    float mins[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, maxs[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int64_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            float v = coords[i * 3 + a];
            if (v < mins[a]) mins[a] = v;
            if (v > maxs[a]) maxs[a] = v;
        }
    key_idx* ki = (key_idx*)malloc(sizeof(key_idx) * (size_t)n);
    const float scale = (float)(1u << 21) - 1.0f;
    for (int64_t i = 0; i < n; ++i) {
        uint32_t q[3];
        for (int a = 0; a < 3; ++a) {
            float denom = fabsf(maxs[a] - mins[a]);
            if (denom < 1e-9f) denom = 1e-9f;
            float nv = (coords[i * 3 + a] - mins[a]) / denom;
            nv = nv < 0.0f ? 0.0f : (nv > 1.0f ? 1.0f : nv);
            q[a] = (uint32_t)(nv * scale);
        }
        ki[i].key = ct_morton3(q[0], q[1], q[2]);
        ki[i].idx = i;
        if (codes_out) codes_out[i] = ki[i].key;
    }
    qsort(ki, (size_t)n, sizeof(key_idx), cmp_key_idx);
    for (int64_t i = 0; i < n; ++i) order[i] = ki[i].idx;
    free(ki);
}

/* ------------------------------------------------------------------------- */
/* Tree storage, src/tree.rs:6-125                                           */
/* ------------------------------------------------------------------------- */
typedef struct {
    int64_t n, cap;
    int64_t* parents;
    int64_t* children;   /* first child */
    int64_t* next;       /* next sibling */
    int32_t* levels;
    float* si;
    int32_t min_level, max_level;
} ct_tree_data;

static void tree_init(ct_tree_data* T, int64_t cap) {
    memset(T, 0, sizeof(*T));
    T->cap = cap > 0 ? cap : 1;
    T->parents = (int64_t*)malloc(sizeof(int64_t) * T->cap);
    T->children = (int64_t*)malloc(sizeof(int64_t) * T->cap);
    T->next = (int64_t*)malloc(sizeof(int64_t) * T->cap);
    T->levels = (int32_t*)malloc(sizeof(int32_t) * T->cap);
    T->si = (float*)calloc((size_t)T->cap, sizeof(float));
    T->min_level = -20; T->max_level = 20;
}

static void tree_free(ct_tree_data* T) {
    free(T->parents); free(T->children); free(T->next); free(T->levels); free(T->si);
    memset(T, 0, sizeof(*T));
}

/* link_child, src/tree.rs:165-170: prepend to the parent's child list. */
static inline void link_child(ct_tree_data* T, int64_t parent, int64_t child) {
    int64_t old = T->children[parent];
    T->children[parent] = child;
    T->next[child] = old;
}

static inline void set_level(ct_tree_data* T, int64_t idx, int32_t level) {
    T->levels[idx] = level;
    if (level > T->max_level) T->max_level = level;
    if (level < T->min_level) T->min_level = level;
}

static inline void set_parent(ct_tree_data* T, int64_t idx, int64_t parent) {
    T->parents[idx] = parent;
    if (parent >= 0) link_child(T, parent, idx);
}

/* ------------------------------------------------------------------------- */
/* Metric dispatch for the build: residual (index payload) or Euclidean.     */
/* ------------------------------------------------------------------------- */
typedef struct {
    int kind;                 /* 0 residual, 1 euclidean */
    const ct_metric* res;
    const float* pts;         /* euclidean points n x d */
    int d;
} build_metric;

/* Metric::distance_sq: residual -> distance_sq_idx (src/metric.rs:586-590);
 * Euclidean -> sum of squared differences (src/metric.rs:33-41). */
static inline float bm_dist_sq(const build_metric* B, int64_t i, int64_t j) {
    if (B->kind == 0) return dist_sq_idx(B->res, i, j);
    const float* a = B->pts + i * B->d;
    const float* b = B->pts + j * B->d;
    float s = 0.0f;
    for (int c = 0; c < B->d; ++c) { float df = a[c] - b[c]; s += df * df; }
    return s;
}

/* ------------------------------------------------------------------------- */
/* Grid conflicts, src/algo/batch/mod.rs:212-327                             */
/* Cells are floor(coord*scale) over all D axes; neighbour cells differ by   */
/* -1/0/+1 on the first min(D,3) axes and are only matched when D <= 3 (the  */
/* reference builds 3-component neighbour keys, which never equal a longer   */
/* key).  Edges are emitted into the caller's adjacency bitmap.              */
/* ------------------------------------------------------------------------- */
typedef struct { int64_t key[8]; int dim; int pos; } cell_entry;
static int cmp_cell(const void* a, const void* b) {
    const cell_entry* x = (const cell_entry*)a; const cell_entry* y = (const cell_entry*)b;
    for (int i = 0; i < x->dim; ++i) if (x->key[i] != y->key[i]) return x->key[i] < y->key[i] ? -1 : 1;
    return x->pos - y->pos;
}

static int cell_key_eq(const int64_t* a, const int64_t* b, int dim) {
    for (int i = 0; i < dim; ++i) if (a[i] != b[i]) return 0;
    return 1;
}

/* adjacency as dense bitmap over far candidates (n_far <= chunk size) */
static inline void adj_set(uint8_t* adj, int n, int u, int v) { adj[(size_t)u * n + v] = 1; adj[(size_t)v * n + u] = 1; }

static void grid_conflicts(const float* coords_batch, int d, const int64_t* far, int n_far,
                           int64_t start_idx, float scale, uint8_t* adj) {
    if (n_far == 0) return;
    int kd = d < 8 ? d : 8;
    cell_entry* cells = (cell_entry*)malloc(sizeof(cell_entry) * (size_t)n_far);
    for (int pos = 0; pos < n_far; ++pos) {
        int64_t local = far[pos] - start_idx;
        cells[pos].dim = kd; cells[pos].pos = pos;
        for (int c = 0; c < kd; ++c) {
            float s = coords_batch[local * d + c] * scale;
            cells[pos].key[c] = (int64_t)floorf(s);
        }
    }
    qsort(cells, (size_t)n_far, sizeof(cell_entry), cmp_cell);
    /* same-cell pairs */
    int g0 = 0;
    while (g0 < n_far) {
        int g1 = g0 + 1;
        while (g1 < n_far && cell_key_eq(cells[g1].key, cells[g0].key, kd)) ++g1;
        for (int a = g0; a < g1; ++a)
            for (int b = a + 1; b < g1; ++b) adj_set(adj, n_far, cells[a].pos, cells[b].pos);
        g0 = g1;
    }
    /* neighbour-cell pairs (only reachable when d <= 3) */
    if (d <= 3 && d > 0) {
        for (int a = 0; a < n_far; ++a)
            for (int b = 0; b < n_far; ++b) {
                if (cell_key_eq(cells[a].key, cells[b].key, kd)) continue;
                int ok = 1;
                for (int c = 0; c < kd; ++c) {
                    int64_t df = cells[a].key[c] - cells[b].key[c];
                    if (df < -1 || df > 1) { ok = 0; break; }
                }
                if (ok) adj_set(adj, n_far, cells[a].pos, cells[b].pos);
            }
    }
    free(cells);
}

/* ------------------------------------------------------------------------- */
/* Batch insert, src/algo/batch/mod.rs:447-800 (with compute_mis_greedy,     */
/* src/algo/batch/mis.rs:9-59: all priorities 1.0 -> index order).          */
/* Points of the batch are nodes [start, start+len) already appended.        */
/* ------------------------------------------------------------------------- */
static void batch_insert(ct_tree_data* T, int64_t start_idx, int64_t end_idx, const build_metric* B,
                         const float* coords_batch, int coord_d, float grid_scale) {
    /* append with dummy level (mod.rs:511-513) */
    for (int64_t i = start_idx; i < end_idx; ++i) {
        T->parents[i] = -1; T->children[i] = -1; T->next[i] = -1;
        T->levels[i] = INT32_MIN; T->si[i] = 0.0f;
    }
    T->n = end_idx;
    int64_t ncand = end_idx - start_idx;
    if (ncand <= 0) return;
    int64_t* cand = (int64_t*)malloc(sizeof(int64_t) * ncand);
    int64_t* cover = (int64_t*)malloc(sizeof(int64_t) * ncand);   /* active set (single node) */
    int64_t nc = 0;
    int64_t first = start_idx;
    if (start_idx == 0) {   /* bootstrap root (mod.rs:523-531) */
        T->min_level = -10; T->max_level = 10;
        set_level(T, 0, 10);
        first = 1;
    }
    for (int64_t i = first; i < end_idx; ++i) { cand[nc] = i; cover[nc] = 0; ++nc; }
    if (nc == 0) { free(cand); free(cover); return; }

    int32_t level = T->max_level - 1;
    const int32_t min_level = T->min_level;
    int64_t* next_cand = (int64_t*)malloc(sizeof(int64_t) * ncand);
    int64_t* next_cover = (int64_t*)malloc(sizeof(int64_t) * ncand);
    uint8_t* is_near = (uint8_t*)malloc((size_t)ncand);
    int64_t* best = (int64_t*)malloc(sizeof(int64_t) * ncand);
    int64_t* far = (int64_t*)malloc(sizeof(int64_t) * ncand);
    int64_t* far_orig = (int64_t*)malloc(sizeof(int64_t) * ncand);

    while (level >= min_level) {
        float radius = ldexpf(1.0f, level);
        float radius_sq = radius * radius;
        /* near / far filter (mod.rs:580-627) */
        #pragma omp parallel for schedule(dynamic, 16)
        for (int64_t c = 0; c < nc; ++c) {
            int64_t q = cand[c];
            float best_d = FLT_MAX; int64_t bn = -1; int near = 0;
            int64_t pnode = cover[c];
            float dp = bm_dist_sq(B, q, pnode);
            if (dp <= radius_sq) { if (dp < best_d) { best_d = dp; bn = pnode; } near = 1; }
            int64_t child = T->children[pnode];
            while (child != -1) {
                float dc = bm_dist_sq(B, q, child);
                if (dc <= radius_sq) { if (dc < best_d) { best_d = dc; bn = child; } near = 1; }
                int64_t nx = T->next[child];
                if (nx == child) break;
                child = nx;
                if (child == T->children[pnode]) break;
            }
            is_near[c] = (uint8_t)near; best[c] = bn;
        }
        int64_t nn = 0, nf = 0;
        for (int64_t c = 0; c < nc; ++c) {
            if (is_near[c]) { next_cand[nn] = cand[c]; next_cover[nn] = best[c]; ++nn; }
            else { far[nf] = cand[c]; far_orig[nf] = c; ++nf; }
        }
        if (nf > 0) {
            int n_far = (int)nf;
            uint8_t* adj = (uint8_t*)calloc((size_t)n_far * (size_t)n_far, 1);
            if (coords_batch) grid_conflicts(coords_batch, coord_d, far, n_far, start_idx, grid_scale, adj);
            /* pairwise conflicts (mod.rs:370-400) */
            #pragma omp parallel for schedule(dynamic, 8)
            for (int i = 0; i < n_far; ++i)
                for (int j = i + 1; j < n_far; ++j)
                    if (bm_dist_sq(B, far[i], far[j]) <= radius_sq) { adj[(size_t)i * n_far + j] = 1; adj[(size_t)j * n_far + i] = 1; }
            /* greedy MIS in index order (mis.rs:281-310) */
            int8_t* state = (int8_t*)calloc((size_t)n_far, 1);
            for (int i = 0; i < n_far; ++i) {
                if (state[i] != 0) continue;
                state[i] = 1;
                for (int j = 0; j < n_far; ++j) if (adj[(size_t)i * n_far + j] && state[j] == 0) state[j] = -1;
            }
            /* leaders (mod.rs:694-714) */
            int64_t* leaders = (int64_t*)malloc(sizeof(int64_t) * n_far);
            int nl = 0;
            for (int i = 0; i < n_far; ++i) {
                if (state[i] != 1) continue;
                int64_t q = far[i];
                leaders[nl++] = q;
                set_level(T, q, level);
                set_parent(T, q, cover[far_orig[i]]);
            }
            /* non-leaders attach to nearest leader within radius (mod.rs:733-769) */
            int64_t* attach = (int64_t*)malloc(sizeof(int64_t) * n_far);
            #pragma omp parallel for schedule(dynamic, 8)
            for (int i = 0; i < n_far; ++i) {
                attach[i] = -1;
                if (state[i] == 1) continue;
                float bd = FLT_MAX; int64_t bl = -1;
                for (int l = 0; l < nl; ++l) {
                    float dd = bm_dist_sq(B, far[i], leaders[l]);
                    if (dd <= radius_sq && dd < bd) { bd = dd; bl = leaders[l]; }
                }
                attach[i] = bl;
            }
            for (int i = 0; i < n_far; ++i) {
                if (state[i] == 1) continue;
                if (attach[i] >= 0) { next_cand[nn] = far[i]; next_cover[nn] = attach[i]; ++nn; }
                /* else: dropped -> stays an orphan root (level INT32_MIN, parent -1) */
            }
            free(attach); free(leaders); free(state); free(adj);
        }
        memcpy(cand, next_cand, sizeof(int64_t) * nn);
        memcpy(cover, next_cover, sizeof(int64_t) * nn);
        nc = nn;
        level -= 1;
    }
    /* survivors (mod.rs:791-800) */
    for (int64_t c = 0; c < nc; ++c) {
        set_level(T, cand[c], min_level);
        set_parent(T, cand[c], cover[c]);
    }
    free(cand); free(cover); free(next_cand); free(next_cover); free(is_near); free(best); free(far); free(far_orig);
}

/* ------------------------------------------------------------------------- */
/* Separation cache, compute_si_cache_residual, src/algo.rs:52-106           */
/* Post-order DFS from node 0 only (explicit stack).                         */
/* ------------------------------------------------------------------------- */
static void compute_si_cache(ct_tree_data* T, const ct_metric* M) {
    int64_t n = T->n;
    for (int64_t i = 0; i < n; ++i) T->si[i] = 0.0f;
    if (n == 0) return;
    int64_t* stack = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    uint8_t* expanded = (uint8_t*)calloc((size_t)n, 1);
    int64_t sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        int64_t node = stack[sp - 1];
        if (!expanded[node]) {
            expanded[node] = 1;
            int64_t child = T->children[node];
            while (child != -1) {
                stack[sp++] = child;
                int64_t nx = T->next[child];
                if (nx == -1 || nx == child) break;
                child = nx;
                if (child == T->children[node]) break;
            }
            continue;
        }
        --sp;
        float max_r = 0.0f;
        int64_t child = T->children[node];
        while (child != -1) {
            float dd = dist_idx(M, node, child);
            float bound = dd + T->si[child];
            if (bound > max_r) max_r = bound;
            int64_t nx = T->next[child];
            if (nx == -1 || nx == child) break;
            child = nx;
            if (child == T->children[node]) break;
        }
        T->si[node] = max_r;
    }
    free(stack); free(expanded);
}

/* compute_subtree_index_bounds, src/tree.rs:144-185 (relaxation to a fixed point). */
CT_EXPORT void ct_subtree_bounds(const int64_t* parents, const int64_t* n2d, int64_t n,
                                 int64_t* min_b, int64_t* max_b) {
    for (int64_t i = 0; i < n; ++i) { min_b[i] = n2d[i]; max_b[i] = n2d[i]; }
    int changed = 1; int64_t it = 0;
    while (changed && it < n) {
        changed = 0; ++it;
        for (int64_t node = 0; node < n; ++node) {
            int64_t p = parents[node];
            if (p >= 0) {
                if (min_b[node] < min_b[p]) { min_b[p] = min_b[node]; changed = 1; }
                if (max_b[node] > max_b[p]) { max_b[p] = max_b[node]; changed = 1; }
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* Residual tree handle, mirrors CoverTreeWrapper + build_pcct2_residual_tree */
/* (src/lib.rs:1374-1564).                                                    */
/* ------------------------------------------------------------------------- */
typedef struct {
    ct_tree_data T;
    ct_metric M;
    float* v;       /* reordered copies (CachedResidualData) */
    float* p;
    float* coords;
    int64_t* order; /* node -> dataset */
    int64_t* inv;   /* dataset -> node */
    int64_t n;
    int m, d;
} ct_otree;

CT_EXPORT ct_otree* ct_oracle_build_residual(const float* v, const float* p, const float* coords,
                                             int64_t n, int m, int d, float var, const float* ls, int n_ls,
                                             int kernel_type, int64_t chunk, int order_mode,
                                             float grid_scale, int parity) {
    ct_otree* H = (ct_otree*)calloc(1, sizeof(ct_otree));
    H->n = n; H->m = m; H->d = d;
    H->order = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    H->inv = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    if (order_mode == 1) ct_morton_order(coords, n, d, H->order, NULL);
    else for (int64_t i = 0; i < n; ++i) H->order[i] = i;
    for (int64_t i = 0; i < n; ++i) H->inv[H->order[i]] = i;
    H->v = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1) * (size_t)m);
    H->p = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    H->coords = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1) * (size_t)(d > 0 ? d : 1));
    for (int64_t i = 0; i < n; ++i) {
        int64_t s = H->order[i];
        memcpy(H->v + i * m, v + s * m, sizeof(float) * m);
        memcpy(H->coords + i * d, coords + s * d, sizeof(float) * d);
        H->p[i] = p[s];
    }
    metric_init(&H->M, H->v, H->p, H->coords, n, m, d, var, ls, n_ls, kernel_type, parity);
    tree_init(&H->T, n);
    build_metric B = {0, &H->M, NULL, d};
    if (chunk <= 0) chunk = n;
    for (int64_t s = 0; s < n; s += chunk) {
        int64_t e = s + chunk < n ? s + chunk : n;
        batch_insert(&H->T, s, e, &B, H->coords + s * d, d, grid_scale);
    }
    compute_si_cache(&H->T, &H->M);
    return H;
}

CT_EXPORT void ct_oracle_free(ct_otree* H) {
    if (!H) return;
    tree_free(&H->T); metric_free(&H->M);
    free(H->v); free(H->p); free(H->coords); free(H->order); free(H->inv);
    free(H);
}

CT_EXPORT void ct_oracle_tree_arrays(const ct_otree* H, int64_t* parents, int64_t* children, int64_t* next,
                                     int32_t* levels, float* si, int64_t* order) {
    int64_t n = H->n;
    if (parents) memcpy(parents, H->T.parents, sizeof(int64_t) * n);
    if (children) memcpy(children, H->T.children, sizeof(int64_t) * n);
    if (next) memcpy(next, H->T.next, sizeof(int64_t) * n);
    if (levels) memcpy(levels, H->T.levels, sizeof(int32_t) * n);
    if (si) memcpy(si, H->T.si, sizeof(float) * n);
    if (order) memcpy(order, H->order, sizeof(int64_t) * n);
}

/* ------------------------------------------------------------------------- */
/* Result heap: max-heap on (dist, idx) lexicographic.                       */
/* ------------------------------------------------------------------------- */
typedef struct { float d; int64_t i; } nb;
static inline int nb_less(nb a, nb b) { return a.d < b.d || (a.d == b.d && a.i < b.i); }
typedef struct { nb* a; int n, k; } nheap;
static void nh_push(nheap* h, nb x) {
    int c = h->n++;
    h->a[c] = x;
    while (c > 0) { int p = (c - 1) / 2; if (nb_less(h->a[p], h->a[c])) { nb t = h->a[p]; h->a[p] = h->a[c]; h->a[c] = t; c = p; } else break; }
}
static void nh_pop(nheap* h) {
    h->a[0] = h->a[--h->n];
    int c = 0;
    for (;;) {
        int l = 2 * c + 1, r = l + 1, g = c;
        if (l < h->n && nb_less(h->a[g], h->a[l])) g = l;
        if (r < h->n && nb_less(h->a[g], h->a[r])) g = r;
        if (g == c) break;
        nb t = h->a[g]; h->a[g] = h->a[c]; h->a[c] = t; c = g;
    }
}
/* push then trim to k (BinaryHeap push/pop pattern in src/algo.rs:1152-1158) */
static inline void nh_offer(nheap* h, nb x) { nh_push(h, x); if (h->n > h->k) nh_pop(h); }
static int cmp_nb(const void* a, const void* b) {
    nb x = *(const nb*)a, y = *(const nb*)b;
    if (nb_less(x, y)) return -1;
    if (nb_less(y, x)) return 1;
    return 0;
}

/* ------------------------------------------------------------------------- */
/* single_residual_knn_query, src/algo.rs:612-1242.                          */
/* parity=1: stream tile 1, visited set, no budget, min-lb early stop.       */
/* parity=0: budget ladder [32,64,96], up 0.015, down 0.002, dynamic tile    */
/*           (16/32/64/128 capped at stream tile 64), level cap 2.0.         */
/* ------------------------------------------------------------------------- */
typedef struct { int64_t node; float dist; } fentry;

typedef struct {
    float* cached_lb; uint64_t* visited;
    fentry* frontier; fentry* next_frontier; int64_t fcap;
    int64_t* ch_nodes; float* ch_lb; int64_t ccap;
    nb* heap_buf; nb* tile_buf;
} qctx;

static void qctx_init(qctx* c, int64_t n, int k) {
    c->cached_lb = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1));
    c->visited = (uint64_t*)calloc((size_t)((n + 63) / 64 + 1), sizeof(uint64_t));
    c->fcap = n + 1;
    c->frontier = (fentry*)malloc(sizeof(fentry) * (size_t)c->fcap);
    c->next_frontier = (fentry*)malloc(sizeof(fentry) * (size_t)c->fcap);
    c->ccap = n + 1;
    c->ch_nodes = (int64_t*)malloc(sizeof(int64_t) * (size_t)c->ccap);
    c->ch_lb = (float*)malloc(sizeof(float) * (size_t)c->ccap);
    c->heap_buf = (nb*)malloc(sizeof(nb) * (size_t)(n + k + 2));   /* roots are pushed untrimmed */
    c->tile_buf = (nb*)malloc(sizeof(nb) * 160);
}
static void qctx_free(qctx* c) {
    free(c->cached_lb); free(c->visited); free(c->frontier); free(c->next_frontier);
    free(c->ch_nodes); free(c->ch_lb); free(c->heap_buf); free(c->tile_buf);
}

typedef struct { float lb; float dist; int64_t node; int64_t pos; } tile_item;
static int cmp_tile_item(const void* a, const void* b) {
    const tile_item* x = (const tile_item*)a; const tile_item* y = (const tile_item*)b;
    if (x->dist < y->dist) return -1;
    if (x->dist > y->dist) return 1;
    return x->pos < y->pos ? -1 : (x->pos > y->pos);   /* stable, as Rust sort_by */
}

static inline float node_radius(const ct_tree_data* T, int64_t node, int parity) {
    float r = T->si[node];
    if (!parity && r > 2.0f) r = 2.0f;   /* apply_level_cap with cap_default 2.0, metric.rs:202-213 */
    if (r < 1e-3f) r = 1e-3f;            /* radius floor, algo.rs:814-818 */
    return r;
}

static int single_query(const ct_otree* H, qctx* ctx, int64_t q_node, int k, int64_t max_idx /* -1 none */,
                        const int64_t* n2d, const int64_t* sub_min, int parity,
                        int64_t* out_idx, float* out_dist, int64_t* evals) {
    const ct_tree_data* T = &H->T;
    const ct_metric* M = &H->M;
    int64_t n = T->n;
    nheap heap = {ctx->heap_buf, 0, k};
    if (n == 0) return 0;
    if (max_idx == 0) return 0;
    for (int64_t i = 0; i < n; ++i) ctx->cached_lb[i] = FLT_MAX;
    static const int64_t schedule[3] = {32, 64, 96};
    int64_t budget_limit = parity ? INT64_MAX : schedule[0];
    int budget_idx = 0;
    const double budget_up = 0.015, budget_down = 0.002;
    int64_t survivors = 0; int low_yield = 0;
    float kth = FLT_MAX;
    int all_prunable = 1;
    int64_t nf = 0;
    /* root scan (algo.rs:688-734) */
    for (int64_t r = 0; r < n; ++r) {
        if (T->parents[r] != -1) continue;
        int64_t rds = n2d[r];
        int valid = max_idx < 0 || rds < max_idx;
        float rd = dist_idx(M, q_node, r);
        ctx->frontier[nf].node = r; ctx->frontier[nf].dist = rd; ++nf;
        if (valid) {
            nb x = {rd, r};
            nh_push(&heap, x);   /* roots are pushed without trimming */
            ++survivors;
            if (rd < kth) kth = rd;
        }
        if (max_idx >= 0 && sub_min) { if (sub_min[r] < max_idx) all_prunable = 0; }
        else all_prunable = 0;
    }
    if (all_prunable && max_idx >= 0) goto finish;
    if (parity) {
        memset(ctx->visited, 0, sizeof(uint64_t) * (size_t)((n + 63) / 64 + 1));
        for (int64_t r = 0; r < n; ++r) if (T->parents[r] == -1) ctx->visited[r >> 6] |= 1ULL << (r & 63);
    }
    const int64_t stream_tile = parity ? 1 : 64;
    while (nf > 0 && (survivors < budget_limit || (max_idx >= 0 && heap.n < k))) {
        if (parity && heap.n == k) {
            float min_lb = FLT_MAX;
            for (int64_t f = 0; f < nf; ++f) {
                float lb = ctx->frontier[f].dist - node_radius(T, ctx->frontier[f].node, 1);
                if (lb < min_lb) min_lb = lb;
            }
            if (min_lb > kth) break;
        }
        int64_t nch = 0, nnext = 0;
        /* gather children (algo.rs:862-995) */
        for (int64_t f = 0; f < nf; ++f) {
            int64_t parent = ctx->frontier[f].node;
            float pr = node_radius(T, parent, parity);
            float plb = ctx->frontier[f].dist - pr;
            if (heap.n == k && plb > kth) continue;
            int64_t child = T->children[parent];
            while (child != -1) {
                int64_t c = child;
                int skip_sibling = 0;
                if (max_idx >= 0 && sub_min && sub_min[c] >= max_idx) {
                    skip_sibling = 1;
                } else {
                    int pred_ok = max_idx < 0 || n2d[c] < max_idx;
                    if (!pred_ok) {
                        int sub_valid = sub_min ? (sub_min[c] < max_idx) : 1;
                        if (sub_valid) {
                            float dd = dist_idx(M, q_node, c);
                            ctx->next_frontier[nnext].node = c; ctx->next_frontier[nnext].dist = dd; ++nnext;
                        }
                        skip_sibling = 1;
                    }
                }
                if (skip_sibling) {
                    int64_t nx = T->next[c];
                    if (nx == c || nx == -1) break;
                    child = nx;
                    if (child == T->children[parent]) break;
                    continue;
                }
                int add = 1;
                if (parity) {
                    if (ctx->visited[c >> 6] & (1ULL << (c & 63))) add = 0;
                    else ctx->visited[c >> 6] |= 1ULL << (c & 63);
                }
                if (add) {
                    ctx->ch_nodes[nch] = c; ctx->ch_lb[nch] = plb; ++nch;
                    if (ctx->cached_lb[c] > plb) ctx->cached_lb[c] = plb;
                }
                int64_t nx = T->next[c];
                if (nx == c) break;
                child = nx;
                if (child == T->children[parent]) break;
            }
        }
        /* tiles (algo.rs:997-1222) */
        int64_t start = 0;
        int stop_all = 0;
        while (start < nch && (survivors < budget_limit || (max_idx >= 0 && heap.n < k))) {
            int64_t active = nch - start;
            int64_t tile;
            if (!parity) {
                int64_t wave = nf > 1 ? nf : 1;
                int64_t comb = active + wave;
                tile = comb <= 32 ? 16 : comb <= 128 ? 32 : comb <= 512 ? 64 : 128;
                if (tile > stream_tile) tile = stream_tile;
            } else {
                tile = stream_tile;
            }
            int64_t end = start + tile < nch ? start + tile : nch;
            if (heap.n == k) {
                float mlb = FLT_MAX;
                for (int64_t j = start; j < end; ++j) if (ctx->ch_lb[j] < mlb) mlb = ctx->ch_lb[j];
                if (mlb > kth) { start = end; continue; }
            }
            tile_item items[160];
            int nit = 0;
            for (int64_t j = start; j < end; ++j) {
                int64_t c = ctx->ch_nodes[j];
                if (heap.n == k && ctx->cached_lb[c] > kth) continue;
                float dd = dist_batch(M, q_node, c);
                if (evals) ++*evals;
                items[nit].dist = dd; items[nit].node = c; items[nit].lb = ctx->ch_lb[j]; items[nit].pos = j - start;
                ++nit;
            }
            qsort(items, (size_t)nit, sizeof(tile_item), cmp_tile_item);
            int64_t added = 0;
            for (int t = 0; t < nit; ++t) {
                int64_t c = items[t].node;
                float dd = items[t].dist;
                float cr = node_radius(T, c, parity);
                if (heap.n == k) {
                    float lb = items[t].lb < dd - cr ? items[t].lb : dd - cr;
                    if (lb > kth) continue;
                }
                float nlb = dd - cr;
                if (nlb < ctx->cached_lb[c]) ctx->cached_lb[c] = nlb;
                nb x = {dd, c};
                nh_offer(&heap, x);
                kth = heap.a[0].d;
                ++survivors; ++added;
                int cont = survivors < budget_limit || (max_idx >= 0 && heap.n < k);
                if (cont) {
                    int sub_valid = (max_idx >= 0 && sub_min) ? (sub_min[c] < max_idx) : 1;
                    if (sub_valid) { ctx->next_frontier[nnext].node = c; ctx->next_frontier[nnext].dist = dd; ++nnext; }
                } else {
                    break;
                }
            }
            if (!parity && end > start) {
                double ratio = (double)added / (double)(end - start);
                if (ratio >= budget_up) {
                    if (budget_idx + 1 < 3) { ++budget_idx; budget_limit = schedule[budget_idx]; }
                    low_yield = 0;
                } else if (ratio < budget_down) {
                    ++low_yield;
                    int need_more = max_idx >= 0 && heap.n < k;
                    if (low_yield >= 2 && !need_more) { stop_all = 1; break; }
                } else {
                    low_yield = 0;
                }
            }
            start = end;
        }
        (void)stop_all;
        fentry* t = ctx->frontier; ctx->frontier = ctx->next_frontier; ctx->next_frontier = t;
        nf = nnext;
    }
finish:;
    /* into_sorted_vec (algo.rs:1232-1241) */
    int cnt = heap.n;
    qsort(heap.a, (size_t)cnt, sizeof(nb), cmp_nb);
    int outn = cnt < k ? cnt : k;
    for (int j = 0; j < outn; ++j) { out_idx[j] = n2d[heap.a[j].i]; out_dist[j] = heap.a[j].d; }
    return outn;
}

/* knn_query_residual cached path, src/lib.rs:370-507 + to_py_arrays :907-938.
 * queries are dataset ids; out-of-range ids map to node 0 (lib.rs:414-418).
 * Output rows padded with -1 / FLT_MAX, ascending by (dist, idx).           */
CT_EXPORT int64_t ct_oracle_knn_residual(const ct_otree* H, const int64_t* queries, int64_t nq, int k,
                                         int predecessor, const int64_t* sub_min_in, int parity,
                                         int64_t* out_idx, float* out_dist, int n_threads) {
    int64_t n = H->n;
    /* node_to_dataset for constraint checks: the order when predecessor mode is
     * on; identity otherwise with a final remap (lib.rs:436-499). */
    int64_t* ident = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    for (int64_t i = 0; i < n; ++i) ident[i] = i;
    const int64_t* n2d = predecessor ? H->order : ident;
    const int64_t* sub_min = predecessor ? sub_min_in : NULL;
    int64_t total_evals = 0;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    #pragma omp parallel reduction(+:total_evals)
    {
        qctx ctx; qctx_init(&ctx, n, k);
        int64_t* tmp_i = (int64_t*)malloc(sizeof(int64_t) * (size_t)(k > 0 ? k : 1));
        float* tmp_d = (float*)malloc(sizeof(float) * (size_t)(k > 0 ? k : 1));
        #pragma omp for schedule(dynamic, 64)
        for (int64_t qi = 0; qi < nq; ++qi) {
            int64_t qd = queries[qi];
            int64_t qn = (qd >= 0 && qd < n) ? H->inv[qd] : 0;
            int64_t max_idx = predecessor ? qd : -1;
            int64_t ev = 0;
            int cnt = single_query(H, &ctx, qn, k, max_idx, n2d, sub_min, parity, tmp_i, tmp_d, &ev);
            total_evals += ev;
            for (int j = 0; j < k; ++j) {
                int64_t idx = -1; float dd = FLT_MAX;
                if (j < cnt) {
                    idx = tmp_i[j]; dd = tmp_d[j];
                    if (!predecessor && idx >= 0 && idx < n) idx = H->order[idx];
                }
                out_idx[qi * k + j] = idx; out_dist[qi * k + j] = dd;
            }
        }
        free(tmp_i); free(tmp_d);
        qctx_free(&ctx);
    }
    free(ident);
    return total_evals;
}

/* ------------------------------------------------------------------------- */
/* Brute force over the batch-path f32 distance: the exact answer the        */
/* traversal approximates (ties by lower dataset index).  Dataset numbering. */
/* ------------------------------------------------------------------------- */
/* New points against a dataset: query row i is (qv[i], qp[i], qcoords[i]) and is
 * scaled, normalised and compared exactly like one more dataset row would be
 * (metric_init + dist_batch above); candidates are the n dataset rows.  The
 * reference has no new-point query; this is the f32 oracle of the serving path. */
CT_EXPORT void ct_oracle_brute_points_f32(const float* v, const float* p, const float* coords, int64_t n, int m,
                                          int d, float var, const float* ls, int n_ls, int kernel_type,
                                          const float* qv, const float* qp, const float* qcoords, int64_t nq,
                                          int k, int64_t* out_idx, float* out_dist, int n_threads) {
    const int64_t nt = n + nq;
    float* av = (float*)malloc(sizeof(float) * (size_t)(nt > 0 ? nt : 1) * (size_t)m);
    float* ap = (float*)malloc(sizeof(float) * (size_t)(nt > 0 ? nt : 1));
    float* ac = (float*)malloc(sizeof(float) * (size_t)(nt > 0 ? nt : 1) * (size_t)d);
    memcpy(av, v, sizeof(float) * (size_t)n * m);
    memcpy(av + (size_t)n * m, qv, sizeof(float) * (size_t)nq * m);
    memcpy(ap, p, sizeof(float) * (size_t)n);
    memcpy(ap + n, qp, sizeof(float) * (size_t)nq);
    memcpy(ac, coords, sizeof(float) * (size_t)n * d);
    memcpy(ac + (size_t)n * d, qcoords, sizeof(float) * (size_t)nq * d);
    ct_metric M;
    metric_init(&M, av, ap, ac, nt, m, d, var, ls, n_ls, kernel_type, 0);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    #pragma omp parallel
    {
        nb* buf = (nb*)malloc(sizeof(nb) * (size_t)(k + 2));
        #pragma omp for schedule(dynamic, 16)
        for (int64_t qi = 0; qi < nq; ++qi) {
            nheap h = {buf, 0, k};
            for (int64_t j = 0; j < n; ++j) {
                nb x = {dist_batch(&M, n + qi, j), j};
                if (h.n < k) nh_push(&h, x);
                else if (nb_less(x, h.a[0])) { h.a[0] = x; int c = 0; for (;;) { int l = 2*c+1, r = l+1, g = c; if (l < h.n && nb_less(h.a[g], h.a[l])) g = l; if (r < h.n && nb_less(h.a[g], h.a[r])) g = r; if (g == c) break; nb t = h.a[g]; h.a[g] = h.a[c]; h.a[c] = t; c = g; } }
            }
            qsort(h.a, (size_t)h.n, sizeof(nb), cmp_nb);
            for (int j = 0; j < k; ++j) {
                out_idx[qi * k + j] = j < h.n ? h.a[j].i : -1;
                out_dist[qi * k + j] = j < h.n ? h.a[j].d : FLT_MAX;
            }
        }
        free(buf);
    }
    metric_free(&M);
    free(av); free(ap); free(ac);
}

CT_EXPORT void ct_oracle_brute_f32(const float* v, const float* p, const float* coords, int64_t n, int m, int d,
                                   float var, const float* ls, int n_ls, int kernel_type,
                                   const int64_t* queries, int64_t nq, int k, int predecessor,
                                   int64_t* out_idx, float* out_dist, int n_threads) {
    ct_metric M;
    metric_init(&M, v, p, coords, n, m, d, var, ls, n_ls, kernel_type, 0);
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    #pragma omp parallel
    {
        nb* buf = (nb*)malloc(sizeof(nb) * (size_t)(k + 2));
        #pragma omp for schedule(dynamic, 16)
        for (int64_t qi = 0; qi < nq; ++qi) {
            int64_t q = queries[qi];
            nheap h = {buf, 0, k};
            int64_t lim = predecessor ? q : n;
            for (int64_t j = 0; j < lim; ++j) {
                float dd = dist_batch(&M, q, j);
                nb x = {dd, j};
                if (h.n < k) nh_push(&h, x);
                else if (nb_less(x, h.a[0])) { h.a[0] = x; int c = 0; for (;;) { int l = 2*c+1, r = l+1, g = c; if (l < h.n && nb_less(h.a[g], h.a[l])) g = l; if (r < h.n && nb_less(h.a[g], h.a[r])) g = r; if (g == c) break; nb t = h.a[g]; h.a[g] = h.a[c]; h.a[c] = t; c = g; } }
            }
            qsort(h.a, (size_t)h.n, sizeof(nb), cmp_nb);
            for (int j = 0; j < k; ++j) {
                out_idx[qi * k + j] = j < h.n ? h.a[j].i : -1;
                out_dist[qi * k + j] = j < h.n ? h.a[j].d : FLT_MAX;
            }
        }
        free(buf);
    }
    metric_free(&M);
}

/* Pairwise batch-path distances for given (i, j) pairs (dataset numbering). */
CT_EXPORT void ct_oracle_pair_dist(const float* v, const float* p, const float* coords, int64_t n, int m, int d,
                                   float var, const float* ls, int n_ls, int kernel_type,
                                   const int64_t* qi, const int64_t* cj, int64_t npairs, float* out, int scalar_path) {
    ct_metric M;
    metric_init(&M, v, p, coords, n, m, d, var, ls, n_ls, kernel_type, 0);
    for (int64_t t = 0; t < npairs; ++t)
        out[t] = scalar_path ? dist_sq_idx(&M, qi[t], cj[t]) : dist_batch(&M, qi[t], cj[t]);
    metric_free(&M);
}

/* ------------------------------------------------------------------------- */
/* Euclidean path: CoverTreeWrapper.insert -> batch_insert (Euclidean metric, */
/* no grid edges) and single_knn_query best-first, src/algo.rs:179-323.      */
/* ------------------------------------------------------------------------- */
typedef struct { ct_tree_data T; float* pts; int64_t n; int d; } ct_oetree;

CT_EXPORT ct_oetree* ct_oracle_build_euclidean(const float* pts, int64_t n, int d, int64_t chunk) {
    ct_oetree* E = (ct_oetree*)calloc(1, sizeof(ct_oetree));
    E->n = n; E->d = d;
    E->pts = (float*)malloc(sizeof(float) * (size_t)(n > 0 ? n : 1) * (size_t)d);
    memcpy(E->pts, pts, sizeof(float) * (size_t)n * (size_t)d);
    tree_init(&E->T, n);
    build_metric B = {1, NULL, E->pts, d};
    if (chunk <= 0) chunk = n;
    for (int64_t s = 0; s < n; s += chunk) {
        int64_t e = s + chunk < n ? s + chunk : n;
        batch_insert(&E->T, s, e, &B, NULL, d, 1.0f);
    }
    return E;
}

CT_EXPORT void ct_oracle_free_euclidean(ct_oetree* E) {
    if (!E) return;
    tree_free(&E->T); free(E->pts); free(E);
}

CT_EXPORT void ct_oracle_euclidean_arrays(const ct_oetree* E, int64_t* parents, int32_t* levels) {
    if (parents) memcpy(parents, E->T.parents, sizeof(int64_t) * E->n);
    if (levels) memcpy(levels, E->T.levels, sizeof(int32_t) * E->n);
}

/* candidate min-heap on distance (Candidate Ord is reversed, algo.rs:138-142) */
typedef struct { float d; int64_t i; } cand_t;

CT_EXPORT void ct_oracle_knn_euclidean(const ct_oetree* E, const float* queries, int64_t nq, int k, int predecessor,
                                       int64_t* out_idx, float* out_dist) {
    const ct_tree_data* T = &E->T;
    int64_t n = E->n; int d = E->d;
    #pragma omp parallel
    {
        cand_t* ch = (cand_t*)malloc(sizeof(cand_t) * (size_t)(n + 1));
        nb* rb = (nb*)malloc(sizeof(nb) * (size_t)(k + 2));
        #pragma omp for schedule(dynamic, 16)
        for (int64_t qi = 0; qi < nq; ++qi) {
            const float* q = queries + qi * d;
            int64_t max_idx = predecessor ? qi : -1;
            nheap res = {rb, 0, k};
            int nc = 0;
            int done = (n == 0) || (max_idx == 0);
            #define DIST(node) ({ const float* pp_ = E->pts + (node) * d; float s_ = 0.0f; for (int c_ = 0; c_ < d; ++c_) { float df_ = q[c_] - pp_[c_]; s_ += df_ * df_; } sqrtf(s_); })
            #define CH_PUSH(dd_, ii_) do { int c_ = nc++; ch[c_].d = (dd_); ch[c_].i = (ii_); while (c_ > 0) { int p_ = (c_ - 1) / 2; if (ch[c_].d < ch[p_].d || (ch[c_].d == ch[p_].d && ch[c_].i < ch[p_].i)) { cand_t t_ = ch[p_]; ch[p_] = ch[c_]; ch[c_] = t_; c_ = p_; } else break; } } while (0)
            if (!done) {
                for (int64_t r = 0; r < n; ++r) if (T->parents[r] == -1) { float dd = DIST(r); CH_PUSH(dd, r); }
            }
            float kth = FLT_MAX;
            while (!done && nc > 0) {
                cand_t top = ch[0];
                ch[0] = ch[--nc];
                { int c = 0; for (;;) { int l = 2*c+1, r = l+1, g = c;
                    if (l < nc && (ch[l].d < ch[g].d || (ch[l].d == ch[g].d && ch[l].i < ch[g].i))) g = l;
                    if (r < nc && (ch[r].d < ch[g].d || (ch[r].d == ch[g].d && ch[r].i < ch[g].i))) g = r;
                    if (g == c) break;
                    cand_t t = ch[g]; ch[g] = ch[c]; ch[c] = t; c = g; } }
                int can_prune = res.n >= k;
                if (can_prune) {
                    float radius = ldexpf(1.0f, T->levels[top.i] + 1);
                    if (top.d - radius > kth) continue;
                }
                int ok = max_idx < 0 || top.i < max_idx;
                if (ok) {
                    nb x = {top.d, top.i};
                    nh_offer(&res, x);
                    if (res.n == k) kth = res.a[0].d;
                }
                int64_t child = T->children[top.i];
                while (child != -1) {
                    float dd = DIST(child);
                    CH_PUSH(dd, child);
                    int64_t nx = T->next[child];
                    if (nx == child) break;
                    child = nx;
                    if (child == T->children[top.i]) break;
                }
            }
            #undef DIST
            #undef CH_PUSH
            qsort(res.a, (size_t)res.n, sizeof(nb), cmp_nb);
            for (int j = 0; j < k; ++j) {
                out_idx[qi * k + j] = j < res.n ? res.a[j].i : -1;
                out_dist[qi * k + j] = j < res.n ? res.a[j].d : FLT_MAX;
            }
        }
        free(ch); free(rb);
    }
}

/* ------------------------------------------------------------------------- */
/* Seeded Luby MIS, covertreex/algo/_mis_numba.py:19-131 (degree <= 8 ->     */
/* deterministic greedy; else hash priorities with lower-index tie-break).   */
/* ------------------------------------------------------------------------- */
CT_EXPORT double ct_hash_priority(int64_t node, int64_t seed, int64_t iteration) {
    uint32_t x = (uint32_t)node ^ (uint32_t)seed;
    x ^= (uint32_t)((uint64_t)iteration * 0x9E3779B9ULL);
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return ((double)x + 1.0) / 4294967296.0;
}

CT_EXPORT int ct_oracle_luby_mis(const int64_t* indptr, const int64_t* indices, int64_t n, int64_t seed, int8_t* selected) {
    int64_t max_deg = 0;
    for (int64_t v = 0; v < n; ++v) { int64_t dg = indptr[v + 1] - indptr[v]; if (dg > max_deg) max_deg = dg; }
    uint8_t* active = (uint8_t*)malloc((size_t)(n > 0 ? n : 1));
    memset(active, 1, (size_t)(n > 0 ? n : 1));
    for (int64_t v = 0; v < n; ++v) selected[v] = 0;
    if (max_deg <= 8) {
        for (int64_t v = 0; v < n; ++v) {
            if (!active[v]) continue;
            selected[v] = 1;
            for (int64_t o = indptr[v]; o < indptr[v + 1]; ++o) active[indices[o]] = 0;
            active[v] = 0;
        }
        free(active);
        return 1;
    }
    double* pr = (double*)malloc(sizeof(double) * (size_t)n);
    uint8_t* win = (uint8_t*)malloc((size_t)n);
    uint8_t* dom = (uint8_t*)malloc((size_t)n);
    int it = 0;
    for (;;) {
        int any = 0;
        for (int64_t v = 0; v < n; ++v) if (active[v]) { any = 1; break; }
        if (!any) break;
        ++it;
        for (int64_t v = 0; v < n; ++v) pr[v] = ct_hash_priority(v, seed, it);
        memset(win, 0, (size_t)n);
        int anyw = 0;
        for (int64_t v = 0; v < n; ++v) {
            if (!active[v]) continue;
            int bestf = 1;
            for (int64_t o = indptr[v]; o < indptr[v + 1]; ++o) {
                int64_t u = indices[o];
                if (!active[u]) continue;
                if (pr[u] > pr[v] || (pr[u] == pr[v] && u < v)) { bestf = 0; break; }
            }
            if (bestf) { win[v] = 1; anyw = 1; }
        }
        if (!anyw) for (int64_t v = 0; v < n; ++v) if (active[v]) { win[v] = 1; break; }
        memset(dom, 0, (size_t)n);
        for (int64_t v = 0; v < n; ++v) if (win[v]) for (int64_t o = indptr[v]; o < indptr[v + 1]; ++o) dom[indices[o]] = 1;
        for (int64_t v = 0; v < n; ++v) { if (win[v]) selected[v] = 1; if (win[v] || dom[v]) active[v] = 0; }
    }
    free(pr); free(win); free(dom); free(active);
    return it;
}

/* ------------------------------------------------------------------------- */
/* Hilbert keys, covertreex/algo/order/strategy.py:38-100 (Skilling's        */
/* axes-to-transpose, bits = clamp(64 / D, 1, 16), round-half-even quantise). */
/* ------------------------------------------------------------------------- */
CT_EXPORT void ct_hilbert_codes(const double* pts, int64_t n, int d, uint64_t* codes) {
    if (n <= 0) return;
    int bits = 64 / (d > 0 ? d : 1);
    if (bits > 16) bits = 16;
    if (bits < 1) bits = 1;
    double lo[64], hi[64];
    for (int c = 0; c < d; ++c) { lo[c] = pts[c]; hi[c] = pts[c]; }
    for (int64_t i = 0; i < n; ++i) for (int c = 0; c < d; ++c) {
        double v = pts[i * d + c]; if (v < lo[c]) lo[c] = v; if (v > hi[c]) hi[c] = v;
    }
    const uint64_t maxv = (1ULL << bits) - 1;
    for (int64_t i = 0; i < n; ++i) {
        uint64_t X[64];
        for (int c = 0; c < d; ++c) {
            double span = hi[c] - lo[c]; if (span < 1e-9) span = 1e-9;
            double s = (pts[i * d + c] - lo[c]) / span;
            double r = nearbyint(s * (double)maxv);
            if (r < 0) r = 0;
            if (r > (double)maxv) r = (double)maxv;
            X[c] = (uint64_t)r;
        }
        uint64_t M = 1ULL << (bits - 1);
        for (uint64_t Q = M; Q > 1; Q >>= 1) {
            uint64_t P = Q - 1;
            for (int c = 0; c < d; ++c) {
                if (X[c] & Q) X[0] ^= P;
                else { uint64_t t = (X[0] ^ X[c]) & P; X[0] ^= t; X[c] ^= t; }
            }
        }
        for (int c = 1; c < d; ++c) X[c] ^= X[c - 1];
        uint64_t t = 0;
        for (uint64_t Q = M; Q > 1; Q >>= 1) if (X[d - 1] & Q) t ^= Q - 1;
        for (int c = 0; c < d; ++c) X[c] ^= t;
        uint64_t idx = 0;
        for (int b = bits - 1; b >= 0; --b) {
            uint64_t w = 0;
            for (int c = 0; c < d; ++c) w = (w << 1) | ((X[c] >> b) & 1ULL);
            idx = (idx << d) | w;
        }
        codes[i] = idx;
    }
}

/* ------------------------------------------------------------------------- */
/* FP64 brute force (ground truth for the precision form at full size).       */
/* Same formula as oracle.py's residual_dist_f64 over the stored f32 inputs:  */
/* x/l in FP64, K = var exp(-d2/2) (RBF) or var (1+a+a^2/3) e^-a, a = sqrt(5  */
/* d2) (Matern 5/2), rho = clamp((K - v_q.v_c) / sqrt(max(p_q p_c, 1e-18)),   */
/* +-1), d = sqrt(1-|rho|), d(q,q) = 0 (src/metric.rs:376-487 in FP64).       */
/* Queries are processed in blocks of BQ that share each candidate row, the   */
/* dot products of f32 inputs are exact products summed in FP64.  Results are */
/* ascending by (d, idx); rows with fewer than k candidates pad -1 / +inf.    */
/* cand_limit: candidates are rows [0, cand_limit) (rows beyond it are new    */
/* query points stored after the dataset).                                    */
/* ------------------------------------------------------------------------- */
#define BQ64 16
typedef struct { double d; int64_t i; } nb64;
static inline int nb64_less(nb64 a, nb64 b) { return a.d < b.d || (a.d == b.d && a.i < b.i); }

CT_EXPORT void ct_oracle_brute_f64(const float* v, const float* p, const float* coords, int64_t n, int m, int d,
                                   double var, const float* ls, int n_ls, int kernel_type,
                                   const int64_t* queries, int64_t nq, int k, int predecessor, int64_t cand_limit,
                                   int64_t* out_idx, double* out_dist, int n_threads) {
    const int64_t nc = cand_limit > 0 && cand_limit < n ? cand_limit : n;
    double inv_ls[64];
    for (int c = 0; c < d; ++c) {
        float raw = (ls && n_ls > 0) ? ls[c < n_ls ? c : 0] : 1.0f;
        inv_ls[c] = 1.0 / (double)raw;
    }
    /* query blocks in ascending id order (predecessor mode scores [0, max id) only) */
    int64_t* ord = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
    for (int64_t i = 0; i < nq; ++i) ord[i] = i;
    {
        /* bottom-up merge sort of the rows by query id (stable) */
        int64_t* tmp = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
        for (int64_t w = 1; w < nq; w *= 2) {
            for (int64_t lo = 0; lo < nq; lo += 2 * w) {
                int64_t mid = lo + w < nq ? lo + w : nq, hi = lo + 2 * w < nq ? lo + 2 * w : nq;
                int64_t a = lo, b = mid, o = lo;
                while (a < mid && b < hi) tmp[o++] = queries[ord[b]] < queries[ord[a]] ? ord[b++] : ord[a++];
                while (a < mid) tmp[o++] = ord[a++];
                while (b < hi) tmp[o++] = ord[b++];
            }
            memcpy(ord, tmp, sizeof(int64_t) * (size_t)nq);
        }
        free(tmp);
    }
    const int64_t nblk = (nq + BQ64 - 1) / BQ64;
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#else
    (void)n_threads;
#endif
    #pragma omp parallel
    {
        double* vqt = (double*)malloc(sizeof(double) * (size_t)m * BQ64);   /* [m][BQ64] */
        nb64* heap = (nb64*)malloc(sizeof(nb64) * (size_t)BQ64 * (size_t)(k + 1));
        int hn[BQ64];
        #pragma omp for schedule(dynamic, 1)
        for (int64_t blk = 0; blk < nblk; ++blk) {
            const int64_t b0 = blk * BQ64;
            const int nb = (int)(nq - b0 < BQ64 ? nq - b0 : BQ64);
            int64_t qid[BQ64];
            double xq[BQ64][64], pq[BQ64];
            int64_t hi = 0;
            for (int t = 0; t < BQ64; ++t) {
                const int64_t q = t < nb ? queries[ord[b0 + t]] : -1;
                qid[t] = q;
                hn[t] = 0;
                const int ok = q >= 0 && q < n;
                for (int j = 0; j < m; ++j) vqt[(size_t)j * BQ64 + t] = ok ? (double)v[(size_t)q * m + j] : 0.0;
                for (int c = 0; c < d; ++c) xq[t][c] = ok ? (double)coords[(size_t)q * d + c] * inv_ls[c] : 0.0;
                pq[t] = ok ? (double)p[q] : 1.0;
                const int64_t lim = !ok ? 0 : (predecessor ? (q < nc ? q : nc) : nc);
                if (lim > hi) hi = lim;
            }
            for (int64_t c = 0; c < hi; ++c) {
                double acc[BQ64];
                for (int t = 0; t < BQ64; ++t) acc[t] = 0.0;
                const float* vc = v + (size_t)c * m;
                for (int j = 0; j < m; ++j) {
                    const double x = (double)vc[j];
                    const double* row = vqt + (size_t)j * BQ64;
                    for (int t = 0; t < BQ64; ++t) acc[t] += row[t] * x;
                }
                double xc[64];
                for (int a = 0; a < d; ++a) xc[a] = (double)coords[(size_t)c * d + a] * inv_ls[a];
                const double pc = (double)p[c];
                for (int t = 0; t < nb; ++t) {
                    const int64_t q = qid[t];
                    if (q < 0 || q >= n) continue;
                    if (predecessor ? c >= q : 0) continue;
                    double dd;
                    if (c == q) {
                        dd = 0.0;
                    } else {
                        double d2 = 0.0;
                        for (int a = 0; a < d; ++a) { const double df = xq[t][a] - xc[a]; d2 += df * df; }
                        double K;
                        if (kernel_type == 1) {
                            const double aa = sqrt(5.0) * sqrt(d2);
                            K = var * (1.0 + aa + aa * aa / 3.0) * exp(-aa);
                        } else {
                            K = var * exp(-0.5 * d2);
                        }
                        double pp = pq[t] * pc;
                        if (pp < 1e-18) pp = 1e-18;
                        double rho = (K - acc[t]) / sqrt(pp);
                        if (rho > 1.0) rho = 1.0;
                        if (rho < -1.0) rho = -1.0;
                        const double om = 1.0 - fabs(rho);
                        dd = sqrt(om > 0.0 ? om : 0.0);
                    }
                    /* bounded max-heap of the k best (d, idx) */
                    nb64* h = heap + (size_t)t * (k + 1);
                    const nb64 x = {dd, c};
                    if (hn[t] < k) {
                        int i = hn[t]++;
                        while (i > 0) { int pa = (i - 1) / 2; if (!nb64_less(h[pa], x)) break; h[i] = h[pa]; i = pa; }
                        h[i] = x;
                    } else if (nb64_less(x, h[0])) {
                        int i = 0;
                        for (;;) {
                            int l = 2 * i + 1, r = l + 1, g = i;
                            nb64 hg = x;
                            if (l < k && nb64_less(hg, h[l])) { g = l; hg = h[l]; }
                            if (r < k && nb64_less(hg, h[r])) { g = r; }
                            if (g == i) break;
                            h[i] = h[g];
                            i = g;
                        }
                        h[i] = x;
                    }
                }
            }
            for (int t = 0; t < nb; ++t) {
                nb64* h = heap + (size_t)t * (k + 1);
                /* heap sort ascending */
                for (int e = hn[t] - 1; e > 0; --e) {
                    nb64 top = h[0];
                    nb64 x = h[e];
                    int i = 0;
                    for (;;) {
                        int l = 2 * i + 1, r = l + 1, g = i;
                        nb64 hg = x;
                        if (l < e && nb64_less(hg, h[l])) { g = l; hg = h[l]; }
                        if (r < e && nb64_less(hg, h[r])) { g = r; }
                        if (g == i) break;
                        h[i] = h[g];
                        i = g;
                    }
                    h[i] = x;
                    h[e] = top;
                }
                const int64_t row = ord[b0 + t];
                for (int j = 0; j < k; ++j) {
                    out_idx[row * k + j] = j < hn[t] ? h[j].i : -1;
                    out_dist[row * k + j] = j < hn[t] ? h[j].d : INFINITY;
                }
            }
        }
        free(vqt);
        free(heap);
    }
    free(ord);
}
