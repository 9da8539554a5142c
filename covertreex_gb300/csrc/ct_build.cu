// ct_build.cu — device cover-tree build (placeholder until the level-synchronous
// batch insert lands).
#include "ct_tree.h"
#include "ct_common.cuh"

int ct_tree::build_tree(const float*, const float*, cudaStream_t) {
    return set_err(CT_ERR_UNSUPPORTED, "%s", "cover-tree build not available in this build");
}

int ct_tree::knn_tree(const int64_t*, int64_t, int, int, int64_t*, float*, ct_stats*, cudaStream_t) {
    return set_err(CT_ERR_UNSUPPORTED, "%s", "tree traversal not available in this build");
}
