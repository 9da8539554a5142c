// ct_internal.h — internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace ct {

// per-thread timing switch (ct_set_timing)
bool timing_enabled();

struct BruteParams {
    const float* vperm;   // n x m, residue-major columns (see ct_setup.cu)
    const float* xs;      // n x d scaled coordinates
    const float* norms;   // n squared scaled norms
    const float* p;       // n residual variances
    const long long* qids;
    long long n, nq;
    int m, d, k, kernel_type, predecessor;
    float var;
    long long* out_idx;
    float* out_dist;
    // candidate rows [cbeg, cend); cend <= 0 means n (every row)
    long long cbeg = 0, cend = 0;
};

size_t brute_smem_bytes(int qt, int m, int d, int k);
int brute_pick_qt(int m, int d, int k, size_t smem_limit);
cudaError_t launch_brute_knn(const BruteParams& P, int qt, cudaStream_t stream);

// ct_setup.cu
cudaError_t launch_metric_setup(const float* v, const float* p, const float* coords, long long n, int m, int d,
                                const float* inv_ls_dev, float* vperm, float* xs, float* norms, float* pcopy,
                                cudaStream_t stream);

// ct_order.cu
cudaError_t compute_order(const float* coords, long long n, int d, int mode, int* order_out, cudaStream_t st,
                          unsigned long long* keys_by_id = nullptr, double* bounds_out = nullptr);
cudaError_t hilbert_keys_bounded(const float* coords, long long n, int d, const double* bounds,
                                 unsigned long long* keys, int* scratch_vals, cudaStream_t st);
int radix_sort_launches(long long n, int kbits);
cudaError_t radix_sort_pairs(unsigned long long* keys, int* vals, unsigned long long* ktmp, int* vtmp, long long n,
                             int kbits, unsigned* hist, void* scan_tmp, size_t scan_tmp_bytes, cudaStream_t st,
                             bool* result_in_tmp);
int radix_num_blocks(long long n);

// ct_mis.cu
cudaError_t csr_graph_valid(const long long* indptr, const long long* indices, long long n, bool* valid,
                            cudaStream_t st);
cudaError_t luby_mis_csr(const long long* indptr, const long long* indices, long long n, unsigned long long seed,
                         signed char* sel, int* iterations, cudaStream_t st);

// ct_euclid.cu
cudaError_t launch_euclid_knn(const float* pts, long long n, int d, const float* qry, long long nq, int k,
                              int predecessor, long long* out_idx, float* out_dist, cudaStream_t st);
int euclid_max_k();
int euclid_max_d();

}  // namespace ct
