// ct_setup.cu — device-resident residual metric data (the GPU counterpart of
// ResidualMetric::new, src/metric.rs:84-177, and of the reordered caches of
// build_pcct2_residual_tree, src/lib.rs:1404-1439).
//
// HBM layout written here:
//   vperm [n x m] f32  residue-major V: column l*(m/16)+c holds V[:, 16c+l]
//   xs    [n x d] f32  coords * (1/lengthscale), rounded exactly as the reference
//   norms [n]     f32  sum of xs^2, left to right
//   p     [n]     f32  residual variances (copy)
#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {
namespace {

__global__ void setup_rows_kernel(const float* __restrict__ coords, const float* __restrict__ p, long long n, int d,
                                  const float* __restrict__ inv_ls, float* __restrict__ xs, float* __restrict__ norms,
                                  float* __restrict__ pcopy) {
    long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    float s = 0.f;
    for (int c = 0; c < d; ++c) {
        float x = __fmul_rn(coords[r * d + c], inv_ls[c]);
        xs[r * d + c] = x;
        s = __fadd_rn(s, __fmul_rn(x, x));
    }
    norms[r] = s;
    pcopy[r] = p[r];
}

// vperm[r, l*m16 + c] = v[r, 16c + l]
__global__ void permute_v_kernel(const float* __restrict__ v, long long n, int m, float* __restrict__ vperm) {
    const int m16 = m / 16;
    long long total = n * (long long)m;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        long long r = e / m;
        int col = (int)(e - r * m);
        int l = col / m16, c = col - l * m16;
        vperm[e] = v[r * m + 16 * c + l];
    }
}

}  // namespace

cudaError_t launch_metric_setup(const float* v, const float* p, const float* coords, long long n, int m, int d,
                                const float* inv_ls_dev, float* vperm, float* xs, float* norms, float* pcopy,
                                cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    setup_rows_kernel<<<(unsigned)((n + 255) / 256), 256, 0, stream>>>(coords, p, n, d, inv_ls_dev, xs, norms, pcopy);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    long long total = n * (long long)m;
    long long blocks = (total + 255) / 256;
    if (blocks > 152 * 64) blocks = 152 * 64;
    permute_v_kernel<<<(unsigned)blocks, 256, 0, stream>>>(v, n, m, vperm);
    return cudaGetLastError();
}

}  // namespace ct
