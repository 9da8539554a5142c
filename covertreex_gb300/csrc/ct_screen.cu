// ct_screen.cu — BF16 tcgen05 screening form (placeholder).
#include "ct_tree.h"
#include "ct_common.cuh"

int ct_tree::knn_screened(const int64_t*, int64_t, int, int, int64_t*, float*, ct_stats*, cudaStream_t) {
    return set_err(CT_ERR_UNSUPPORTED, "%s", "screened form not available in this build");
}

void ct_tree::release_screen() { screen = nullptr; }
