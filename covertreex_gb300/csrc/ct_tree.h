// ct_tree.h — the opaque ct_tree handle behind the C ABI: device-resident
// residual metric data, the cover tree, and the buffers of the search forms.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/covertree_cuda.h"
#include "ct_treebound.cuh"

struct ct_tree {
    // shape and metric parameters
    int64_t n = 0;
    int m = 0, d = 0;
    float var = 1.f;
    int kernel_type = 0;
    int chunk = 512, order_mode = CT_ORDER_HILBERT;
    long long slab_rows = 0;  // rows reserved past n in vnat / xs / coords_raw / p for new points
    uint64_t seed = 0;

    // metric data (dataset order), see ct_setup.cu
    float* vperm = nullptr;
    float* xs = nullptr;
    float* norms = nullptr;
    float* p = nullptr;
    float* inv_ls = nullptr;
    float* vnat = nullptr;        // V in natural layout (dataset order), for operand prep / rescoring
    float* coords_raw = nullptr;  // unscaled coordinates (dataset order)
    double inv_ls_host64[64] = {0};

    // cover tree (node order = build order; node i holds dataset row order[i])
    bool has_tree = false;
    long long* order = nullptr;     // node -> dataset
    long long* inv = nullptr;       // dataset -> node
    long long* parents = nullptr;   // node numbering, -1 for roots
    int32_t* levels = nullptr;
    float* si = nullptr;          // cover radius: max FP32 distance to any descendant
    float* si_up = nullptr;       // certified upper bound of the ideal-metric cover radius
    float* sub_isp = nullptr;     // max 1/sqrt(p) over the subtree (node itself included)
    long long* sub_min = nullptr;   // min dataset id in the subtree (node itself included)
    long long* child_off = nullptr; // CSR children: child_off[n+1], child_idx[n]
    long long* child_idx = nullptr;
    long long* roots = nullptr;     // root nodes
    int64_t n_roots = 0;
    float* tvnat = nullptr;       // node-order copies for the build and traversal (natural-layout V)
    float* txs = nullptr;
    float* tnorms = nullptr;
    float* tp = nullptr;
    float* tisp = nullptr;        // node order: 1/sqrt(p) and ||v||, both rounded up
    float* tvn = nullptr;
    int64_t n_side = 0;           // rows kept out of the tree (tiny p), the last n_side nodes
    ct::BoundModel bound{};       // error model of the certified prune (ct_treebound.cuh)
    // build telemetry
    int64_t build_groups = 0, build_conflict_edges = 0, build_selected = 0;
    float build_ms = 0.f;

    // screened form (BF16 operands, built lazily)
    void* screen = nullptr;

    char err[256] = "";

    int alloc_metric();
    int build_tree(const float* v_dataset, const float* coords_dataset, cudaStream_t st);
    int grow_tree(const ct_tree* base, cudaStream_t st);  // base's tree + this handle's extra rows
    int knn_tree(const int64_t* q_ids, int64_t nq, int k, int predecessor, int64_t* out_idx, float* out_dist,
                 ct_stats* stats, cudaStream_t st);
    // id_limit: query ids must lie in [0, id_limit) (default n; rows >= n are the query slab)
    int knn_screened(const int64_t* q_ids, int64_t nq, int k, int predecessor, int64_t* out_idx, float* out_dist,
                     ct_stats* stats, cudaStream_t st, long long id_limit = -1);
    int knn_screened_points(const float* qv, const float* qp, const float* qcoords, int64_t nq, int k,
                            int64_t* out_idx, float* out_dist, ct_stats* stats, cudaStream_t st);
    int prepare_screened(cudaStream_t st);  // build the screened form's operands now
    long long device_bytes() const;          // device memory held by the handle
    void release_screen();
    ~ct_tree();

    template <typename... A>
    int set_err(int code, const char* fmt, A... a) {
        snprintf(err, sizeof(err), fmt, a...);
        return code;
    }
};
