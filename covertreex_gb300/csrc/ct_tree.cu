// ct_tree.cu — handle memory management; the cover-tree build and traversal
// live in ct_build.cu and ct_traverse.cu.
#include "ct_tree.h"

#include "ct_common.cuh"

namespace {
template <typename T>
cudaError_t dalloc(T** p, size_t count) {
    return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}
template <typename T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}
}  // namespace

int ct_tree::alloc_metric() {
    const size_t rows = (size_t)(n + slab_rows);  // query-side arrays carry the slab
    cudaError_t e = dalloc(&vperm, (size_t)n * m);
    if (e == cudaSuccess) e = dalloc(&xs, rows * d);
    if (e == cudaSuccess) e = dalloc(&norms, (size_t)n);
    if (e == cudaSuccess) e = dalloc(&p, rows);
    if (e == cudaSuccess) e = dalloc(&inv_ls, (size_t)64);
    if (e == cudaSuccess) e = dalloc(&vnat, rows * m);
    if (e == cudaSuccess) e = dalloc(&coords_raw, rows * d);
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "device allocation of %lld x %d metric rows failed: %s",
                                         (long long)n, m, cudaGetErrorString(e));
    return CT_OK;
}

ct_tree::~ct_tree() {
    release_screen();
    dfree(vperm); dfree(xs); dfree(norms); dfree(p); dfree(inv_ls); dfree(vnat); dfree(coords_raw);
    dfree(order); dfree(inv); dfree(parents); dfree(levels); dfree(si); dfree(si_up); dfree(sub_isp);
    dfree(sub_min); dfree(child_off); dfree(child_idx); dfree(roots);
    dfree(tvnat); dfree(txs); dfree(tnorms); dfree(tp); dfree(tisp); dfree(tvn);
}
