// ct_vmatrix.cu — residual-backend construction on the GPU in FP64
// (covertreex/metrics/residual/host_backend.py:165-246).
//
//   Kmm = K(Z, Z) + 1e-6 var I      kernels of host_backend.py:14-43, FP64 from
//                                    pairwise differences of FP64 coordinates
//   L   = chol(Kmm)                  blocked right-looking (32-column panels):
//                                    diagonal factor / panel solve / trailing update
//   Li  = L^-1                       column-wise forward substitution, one warp
//                                    per column
//   V   = K(X, Z) Li^T               in row chunks: K(X_c, Z) evaluated into a
//                                    scratch buffer, then an FP64 GEMM that only
//                                    visits t <= j (Li is lower triangular)
//   p   = max(var - ||v||^2, 1e-9)   FP64 in a fixed order, then V and p cast to f32
//
// The reference solves L V^T = K(X,Z)^T with LAPACK; multiplying by the explicit
// inverse has the same forward-error order (cond(L) * eps64), far below the f32
// rounding of the outputs.  Serving uses the same embed step for new points:
// v_x = Li k(Z, x), p_x = var - ||v_x||^2.
//
// FP64 on GB300 runs on the CUDA cores only (about two DFMA per clock per SM), so
// the GEMM is register-tiled 64 x 64 with 4 x 4 outputs per thread and is bound by
// the DFMA rate; N m^2 FMAs for N rows.
#include <cuda_runtime.h>

#include <algorithm>
#include <math.h>

#include "ct_vmatrix.h"

namespace ct {
namespace vmat {

__device__ __forceinline__ double kernel_f64(const double* __restrict__ x, const double* __restrict__ z, int d,
                                             int kt, double var, double ls) {
    double sq = 0.0;
    for (int c = 0; c < d; ++c) {
        const double t = x[c] - z[c];
        sq += t * t;
    }
    const double denom = ls > 1e-12 ? ls : 1e-12;
    if (kt == 1) {
        const double a = sqrt(5.0) * (sqrt(sq) / denom);
        return var * (1.0 + a + (a * a) / 3.0) * exp(-a);
    }
    return var * exp(-0.5 * sq / (denom * denom));
}

// A[i][j] = K(z_i, z_j), plus 1e-6 var on the diagonal (host_backend.py:210-211).
__global__ void kmm_kernel(const double* __restrict__ z, int m, int d, int kt, double var, double ls,
                           double* __restrict__ A) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)m * m) return;
    const int i = (int)(e / m), j = (int)(e - (long long)i * m);
    double v = kernel_f64(z + (size_t)i * d, z + (size_t)j * d, d, kt, var, ls);
    if (i == j) v += 1e-6 * var;
    A[e] = v;
}

constexpr int CB = 32;  // Cholesky panel width

// Factor the diagonal block A[p0:p0+b, p0:p0+b] in place (lower, upper part of the
// block zeroed).  status |= 1 on a non-positive pivot (the matrix is not SPD).
__global__ void __launch_bounds__(1024) potrf_diag_kernel(double* __restrict__ A, int m, int p0, int b,
                                                          int* __restrict__ status) {
    __shared__ double S[CB][CB + 1];
    const int c = threadIdx.x, r = threadIdx.y;
    if (r < b && c < b) S[r][c] = A[(size_t)(p0 + r) * m + p0 + c];
    __syncthreads();
    for (int j = 0; j < b; ++j) {
        if (r == 0 && c == 0) {
            const double a = S[j][j];
            if (!(a > 0.0)) atomicOr(status, 1);
            S[j][j] = a > 0.0 ? sqrt(a) : 1.0;
        }
        __syncthreads();
        if (r == 0 && c > j && c < b) S[c][j] /= S[j][j];
        __syncthreads();
        if (c > j && r >= c && r < b) S[r][c] -= S[r][j] * S[c][j];
        __syncthreads();
    }
    if (r < b && c < b) A[(size_t)(p0 + r) * m + p0 + c] = c <= r ? S[r][c] : 0.0;
}

// Panel solve: rows r >= p0+b get L[r][p0:p0+b] = A[r][p0:p0+b] L_pp^-T.
__global__ void trsm_panel_kernel(double* __restrict__ A, int m, int p0, int b) {
    __shared__ double P[CB][CB + 1];
    for (int e = threadIdx.x; e < CB * CB; e += blockDim.x) {
        const int rr = e / CB, cc = e - rr * CB;
        P[rr][cc] = (rr < b && cc < b) ? A[(size_t)(p0 + rr) * m + p0 + cc] : 0.0;
    }
    __syncthreads();
    const int r = p0 + b + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    double x[CB];
    double* row = A + (size_t)r * m + p0;
#pragma unroll
    for (int c = 0; c < CB; ++c) {
        if (c < b) {
            double s = row[c];
            for (int t = 0; t < c; ++t) s -= x[t] * P[c][t];
            x[c] = s / P[c][c];
            row[c] = x[c];
        }
    }
}

// Trailing update: A[r][c] -= sum_t L[r][p0+t] L[c][p0+t] for p0+b <= c <= r < m.
__global__ void __launch_bounds__(1024) syrk_update_kernel(double* __restrict__ A, int m, int p0, int b) {
    const int base = p0 + b;
    const int bi = blockIdx.y, bj = blockIdx.x;
    if (bj > bi) return;  // strictly upper tile
    __shared__ double Lr[CB][CB + 1];
    __shared__ double Lc[CB][CB + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int r = base + bi * CB + ty, cr = base + bj * CB + ty;
    Lr[ty][tx] = (r < m && tx < b) ? A[(size_t)r * m + p0 + tx] : 0.0;
    Lc[ty][tx] = (cr < m && tx < b) ? A[(size_t)cr * m + p0 + tx] : 0.0;
    __syncthreads();
    const int c = base + bj * CB + tx;
    if (r >= m || c >= m || c > r) return;
    double s = 0.0;
#pragma unroll 8
    for (int t = 0; t < CB; ++t) s += Lr[ty][t] * Lc[tx][t];
    A[(size_t)r * m + c] -= s;
}

__global__ void zero_upper_kernel(double* __restrict__ A, int m) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= (long long)m * m) return;
    const int i = (int)(e / m), j = (int)(e - (long long)i * m);
    if (j > i) A[e] = 0.0;
}

// Li = L^-1 (lower triangular): warp c solves L x = e_c by forward substitution.
// The lanes split each row's dot product (lane l takes t = c + l, c + l + 32, ...,
// then a butterfly sum) and x stays in shared memory, so a column costs m - c
// short steps instead of (m - c)^2 / 2 dependent FMAs on one thread.
__global__ void __launch_bounds__(128) trinv_kernel(const double* __restrict__ L, int m, double* __restrict__ Li) {
    extern __shared__ double trinv_x[];  // [warps per block][m]
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int c = blockIdx.x * (blockDim.x >> 5) + wib;
    if (c >= m) return;
    double* x = trinv_x + (size_t)wib * m;
    for (int i = lane; i < m; i += 32) x[i] = 0.0;
    __syncwarp();
    for (int i = c; i < m; ++i) {
        const double* Lrow = L + (size_t)i * m;
        double s = 0.0;
        for (int t = c + lane; t < i; t += 32) s = fma(Lrow[t], x[t], s);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const double xi = ((i == c ? 1.0 : 0.0) - s) / Lrow[i];
        if (lane == 0) x[i] = xi;
        __syncwarp();
    }
    for (int i = lane; i < m; i += 32) Li[(size_t)i * m + c] = x[i];
}

// Kc[r][t] = K(x_{r0+r}, z_t) for r < rows (grid-stride: the grid may be capped).
__global__ void kxm_kernel(const double* __restrict__ x, long long r0, long long rows, const double* __restrict__ z,
                           int m, int d, int kt, double var, double ls, double* __restrict__ Kc) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < rows * m;
         e += (long long)gridDim.x * blockDim.x) {
        const long long r = e / m;
        const int t = (int)(e - r * m);
        Kc[e] = kernel_f64(x + (size_t)(r0 + r) * d, z + (size_t)t * d, d, kt, var, ls);
    }
}

// Vc[r][j] = sum_{t <= j} Kc[r][t] Li[j][t]; 32 x 32 tiles, 256 threads, 2 x 2 each, a
// block looping over tiles when the grid is capped.  GB300's FP64 rate is low (one block
// of eight warps fills an SM's FP64 pipe), so a serving build runs these kernels on a
// capped grid (ct_set_cta_budget): the other SMs stay free of build blocks, whose shared
// memory would keep the screened form's large blocks off an SM.
constexpr int GT = 32;
constexpr int GK = 32;
__device__ __forceinline__ void dgemm_lt_tile(const double* __restrict__ Kc, long long rows,
                                              const double* __restrict__ Li, int m, double* __restrict__ Vc,
                                              double (*As)[GT + 1], double (*Bs)[GT + 1], long long r0, int j0) {
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[2][2];
#pragma unroll
    for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int w = 0; w < 2; ++w) acc[u][w] = 0.0;
    const int kend = min(m, j0 + GT);  // Li[j][t] = 0 for t > j
    for (int t0 = 0; t0 < kend; t0 += GK) {
        for (int e = threadIdx.x; e < GT * GK; e += 256) {
            const int rr = e / GK, tt = e - rr * GK;
            const int t = t0 + tt;
            const long long row = r0 + rr;
            As[tt][rr] = (row < rows && t < m) ? Kc[row * m + t] : 0.0;
            const int j = j0 + rr;
            Bs[tt][rr] = (j < m && t < m) ? Li[(size_t)j * m + t] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int tt = 0; tt < GK; ++tt) {
            double a[2], b[2];
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                a[u] = As[tt][ty + 16 * u];
                b[u] = Bs[tt][tx + 16 * u];
            }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
                for (int w = 0; w < 2; ++w) acc[u][w] = fma(a[u], b[w], acc[u][w]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
        const long long row = r0 + ty + 16 * u;
        if (row >= rows) continue;
#pragma unroll
        for (int w = 0; w < 2; ++w) {
            const int j = j0 + tx + 16 * w;
            if (j < m) Vc[row * m + j] = acc[u][w];
        }
    }
}

__global__ void __launch_bounds__(256) dgemm_lt_kernel(const double* __restrict__ Kc, long long rows,
                                                       const double* __restrict__ Li, int m,
                                                       double* __restrict__ Vc) {
    __shared__ double As[GK][GT + 1];
    __shared__ double Bs[GK][GT + 1];
    const int tiles_j = (m + GT - 1) / GT;
    const long long tiles = tiles_j * ((rows + GT - 1) / GT);
    for (long long tile = blockIdx.x; tile < tiles; tile += gridDim.x)  // grid-stride: the grid may be capped
        dgemm_lt_tile(Kc, rows, Li, m, Vc, As, Bs, (tile / tiles_j) * GT, (int)(tile % tiles_j) * GT);
}

// One warp per row: p = max(var - ||v||^2, 1e-9) in FP64 (fixed summation order),
// V and p cast to f32.
__global__ void finalize_rows_kernel(const double* __restrict__ Vc, long long rows, int m, double var,
                                     float* __restrict__ V, float* __restrict__ p) {
    const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (row >= rows) return;
    const double* src = Vc + row * m;
    float* dst = V + row * m;
    double s = 0.0;
    for (int j = lane; j < m; j += 32) {
        const double v = src[j];
        s = fma(v, v, s);
        dst[j] = (float)v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        const double q = var - s;
        p[row] = (float)(q > 1e-9 ? q : 1e-9);
    }
}

}  // namespace vmat

using namespace vmat;

cudaError_t vmatrix_factor(const double* z, int m, int d, int kt, double var, double ls, double* L, double* Li,
                           int* status_dev, cudaStream_t st) {
    const long long mm = (long long)m * m;
    cudaError_t e = cudaMemsetAsync(status_dev, 0, sizeof(int), st);
    if (e != cudaSuccess) return e;
    kmm_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(z, m, d, kt, var, ls, L);
    for (int p0 = 0; p0 < m; p0 += CB) {
        const int b = m - p0 < CB ? m - p0 : CB;
        potrf_diag_kernel<<<1, dim3(CB, CB), 0, st>>>(L, m, p0, b, status_dev);
        const int rest = m - p0 - b;
        if (rest > 0) {
            trsm_panel_kernel<<<(rest + 127) / 128, 128, 0, st>>>(L, m, p0, b);
            const int nt = (rest + CB - 1) / CB;
            syrk_update_kernel<<<dim3(nt, nt), dim3(CB, CB), 0, st>>>(L, m, p0, b);
        }
    }
    zero_upper_kernel<<<(unsigned)((mm + 255) / 256), 256, 0, st>>>(L, m);
    // up to 4 warps per block, each with an m-double column in shared memory (m <= 16384)
    const int tw = (int)std::max<size_t>(1, std::min<size_t>(4, (200 * 1024) / (sizeof(double) * (size_t)m)));
    const size_t tsm = sizeof(double) * tw * (size_t)m;
    if (tsm > 48 * 1024) {
        e = cudaFuncSetAttribute(trinv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsm);
        if (e != cudaSuccess) return e;
    }
    trinv_kernel<<<(m + tw - 1) / tw, 32 * tw, tsm, st>>>(L, m, Li);
    return cudaGetLastError();
}

long long vmatrix_chunk_rows(long long n, int m) {
    // two FP64 buffers of rows x m (K(X_c, Z) and V_c), about 512 MB together
    long long c = (256ll << 20) / ((long long)m * 8);
    c = c < 64 ? 64 : (c / 64) * 64;
    return n < c ? n : c;
}

cudaError_t vmatrix_embed(const double* x, long long n, int d, const double* z, int m, int kt, double var, double ls,
                          const double* Li, double* kc, double* vc, long long chunk, float* V, float* p,
                          cudaStream_t st, int* launches, int max_ctas) {
    int nl = 0;
    auto capped = [&](long long blocks) {
        if (max_ctas > 0 && blocks > max_ctas) blocks = max_ctas;
        return (unsigned)(blocks > 0 ? blocks : 1);
    };
    for (long long r0 = 0; r0 < n; r0 += chunk) {
        const long long rows = n - r0 < chunk ? n - r0 : chunk;
        const long long el = rows * m;
        kxm_kernel<<<capped((el + 255) / 256), 256, 0, st>>>(x, r0, rows, z, m, d, kt, var, ls, kc);
        const long long tiles = (long long)((m + GT - 1) / GT) * ((rows + GT - 1) / GT);
        dgemm_lt_kernel<<<capped(tiles), 256, 0, st>>>(kc, rows, Li, m, vc);
        finalize_rows_kernel<<<(unsigned)((rows * 32 + 255) / 256), 256, 0, st>>>(vc, rows, m, var, V + r0 * m,
                                                                               p + r0);
        nl += 3;
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (launches) *launches += nl;
    return cudaSuccess;
}

}  // namespace ct
