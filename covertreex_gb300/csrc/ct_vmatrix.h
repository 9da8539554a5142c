// ct_vmatrix.h — FP64 residual-backend construction (ct_vmatrix.cu) and the
// factor handle behind the ct_vfactor_* entry points.
#pragma once
#include <cuda_runtime.h>

namespace ct {

// L = chol(K(Z,Z) + 1e-6 var I) and Li = L^-1 (both m x m, lower, device FP64).
// *status_dev is set non-zero when a pivot is not positive.
cudaError_t vmatrix_factor(const double* z, int m, int d, int kt, double var, double ls, double* L, double* Li,
                           int* status_dev, cudaStream_t st);

// Rows per chunk of the embed step (scratch kc and vc hold chunk x m doubles each;
// at most about 256 MB each).
long long vmatrix_chunk_rows(long long n, int m);

// V [n x m] f32 and p [n] f32 for points x [n x d] (device FP64).  max_ctas > 0 caps the
// grid of the kernel-matrix and GEMM kernels (their blocks then loop).
cudaError_t vmatrix_embed(const double* x, long long n, int d, const double* z, int m, int kt, double var, double ls,
                          const double* Li, double* kc, double* vc, long long chunk, float* V, float* p,
                          cudaStream_t st, int* launches, int max_ctas = 0);

}  // namespace ct

struct ct_vfactor {
    int device = 0;
    int m = 0, d = 0, kernel_type = 0;
    double variance = 1.0, lengthscale = 1.0;
    double* z = nullptr;   // m x d inducing points
    double* L = nullptr;   // m x m Cholesky factor (lower)
    double* Li = nullptr;  // m x m inverse of L (lower)
};
