// ct_order.cu — device batch ordering: Hilbert keys and an LSD radix sort.
//
// Hilbert keys restate covertreex/algo/order/strategy.py:38-100 (the Python
// PCCT path's true Hilbert curve; the Rust crate's "hilbert" is a 3-D Morton
// code, src/pcct.rs:27-67, also provided): per-axis min/max, quantisation to
// `bits = clamp(64 / D, 1, 16)` bits with round-half-even, Skilling's
// axes-to-transpose, bit interleave.  Order = stable sort by (key, index).
//
// Up to 4096 pairs sort in one block (bitonic, by key then position).  Larger sets
// take a least-significant-digit radix sort over 8-bit digits: per pass
// a per-block histogram, one exclusive scan over (digit, block), and a stable
// scatter in which each block ranks its keys with warp ballots.  No
// inter-block waiting, so nothing can spin.
#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {
namespace {

constexpr int kSortThreads = 256;
constexpr int kItemsPerThread = 8;
constexpr int kTile = kSortThreads * kItemsPerThread;  // keys per block per pass

__global__ void minmax_kernel(const float* __restrict__ coords, long long n, int d, double* __restrict__ mm) {
    // mm[2*c] = min, mm[2*c+1] = max, initialised by the host to +inf/-inf.
    __shared__ double smin[64], smax[64];
    for (int c = threadIdx.x; c < d; c += blockDim.x) { smin[c] = 1e300; smax[c] = -1e300; }
    __syncthreads();
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        for (int c = 0; c < d; ++c) {
            double v = coords[r * d + c];
            // shared-memory atomics on doubles via CAS loops
            unsigned long long* pmn = (unsigned long long*)&smin[c];
            unsigned long long old = *pmn, assumed;
            while (__longlong_as_double(old) > v) {
                assumed = old;
                old = atomicCAS(pmn, assumed, __double_as_longlong(v));
                if (old == assumed) break;
            }
            unsigned long long* pmx = (unsigned long long*)&smax[c];
            old = *pmx;
            while (__longlong_as_double(old) < v) {
                assumed = old;
                old = atomicCAS(pmx, assumed, __double_as_longlong(v));
                if (old == assumed) break;
            }
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < d; c += blockDim.x) {
        unsigned long long* gmn = (unsigned long long*)&mm[2 * c];
        unsigned long long* gmx = (unsigned long long*)&mm[2 * c + 1];
        unsigned long long old = *gmn, assumed;
        while (__longlong_as_double(old) > smin[c]) {
            assumed = old;
            old = atomicCAS(gmn, assumed, __double_as_longlong(smin[c]));
            if (old == assumed) break;
        }
        old = *gmx;
        while (__longlong_as_double(old) < smax[c]) {
            assumed = old;
            old = atomicCAS(gmx, assumed, __double_as_longlong(smax[c]));
            if (old == assumed) break;
        }
    }
}

__global__ void hilbert_keys_kernel(const float* __restrict__ coords, long long n, int d, const double* __restrict__ mm,
                                    unsigned long long* __restrict__ keys, int* __restrict__ vals) {
    long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    int bits = 64 / (d > 0 ? d : 1);
    bits = bits > 16 ? 16 : (bits < 1 ? 1 : bits);
    const unsigned long long maxv = (1ULL << bits) - 1ULL;
    unsigned long long X[64];
    for (int c = 0; c < d; ++c) {
        double lo = mm[2 * c], hi = mm[2 * c + 1];
        double span = hi - lo;
        if (span < 1e-9) span = 1e-9;
        double s = ((double)coords[r * d + c] - lo) / span;
        double q = rint(s * (double)maxv);
        if (q < 0) q = 0;
        if (q > (double)maxv) q = (double)maxv;
        X[c] = (unsigned long long)q;
    }
    const unsigned long long M = 1ULL << (bits - 1);
    for (unsigned long long Q = M; Q > 1; Q >>= 1) {
        unsigned long long P = Q - 1;
        for (int c = 0; c < d; ++c) {
            if (X[c] & Q) {
                X[0] ^= P;
            } else {
                unsigned long long t = (X[0] ^ X[c]) & P;
                X[0] ^= t;
                X[c] ^= t;
            }
        }
    }
    for (int c = 1; c < d; ++c) X[c] ^= X[c - 1];
    unsigned long long t = 0;
    for (unsigned long long Q = M; Q > 1; Q >>= 1)
        if (X[d - 1] & Q) t ^= Q - 1;
    for (int c = 0; c < d; ++c) X[c] ^= t;
    unsigned long long key = 0;
    for (int b = bits - 1; b >= 0; --b) {
        unsigned long long w = 0;
        for (int c = 0; c < d; ++c) w = (w << 1) | ((X[c] >> b) & 1ULL);
        key = (key << d) | w;
    }
    keys[r] = key;
    vals[r] = (int)r;
}

// 3-D Morton key of src/pcct.rs:27-67 (21 bits/axis, float32 quantisation).
__device__ __forceinline__ unsigned long long part1by2(unsigned long long n) {
    n &= 0x1fffffULL;
    n = (n | (n << 32)) & 0x1f00000000ffffULL;
    n = (n | (n << 16)) & 0x1f0000ff0000ffULL;
    n = (n | (n << 8)) & 0x100f00f00f00f00fULL;
    n = (n | (n << 4)) & 0x10c30c30c30c30c3ULL;
    n = (n | (n << 2)) & 0x1249249249249249ULL;
    return n;
}

__global__ void morton_keys_kernel(const float* __restrict__ coords, long long n, const double* __restrict__ mm,
                                   unsigned long long* __restrict__ keys, int* __restrict__ vals) {
    long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    const float scale = (float)(1u << 21) - 1.0f;
    unsigned q[3];
    for (int a = 0; a < 3; ++a) {
        float mn = (float)mm[2 * a], mx = (float)mm[2 * a + 1];
        float denom = fabsf(__fsub_rn(mx, mn));
        if (denom < 1e-9f) denom = 1e-9f;
        float nv = __fdiv_rn(__fsub_rn(coords[r * 3 + a], mn), denom);
        nv = nv < 0.f ? 0.f : (nv > 1.f ? 1.f : nv);
        q[a] = (unsigned)__fmul_rn(nv, scale);
    }
    keys[r] = part1by2(q[0]) | (part1by2(q[1]) << 1) | (part1by2(q[2]) << 2);
    vals[r] = (int)r;
}

// ---------------------------------------------------------------- radix sort
__global__ void radix_hist_kernel(const unsigned long long* __restrict__ keys, long long n, int shift,
                                  unsigned* __restrict__ hist, int nblocks) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    long long base = (long long)blockIdx.x * kTile;
    for (int i = threadIdx.x; i < kTile; i += blockDim.x) {
        long long g = base + i;
        if (g < n) atomicAdd(&h[(keys[g] >> shift) & 255ULL], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[(size_t)i * nblocks + blockIdx.x] = h[i];
}

// Stable scatter: the block walks its tile in rounds of 256 consecutive keys;
// within a round warp w holds keys [32w, 32w+32), so ranking by (warp, lane)
// preserves input order and equal digits stay stable across rounds.
__global__ void radix_scatter_kernel(const unsigned long long* __restrict__ kin, const int* __restrict__ vin,
                                     unsigned long long* __restrict__ kout, int* __restrict__ vout, long long n,
                                     int shift, const unsigned* __restrict__ offsets, int nblocks) {
    __shared__ unsigned base[256];
    __shared__ unsigned warp_counts[kSortThreads / 32][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) base[i] = offsets[(size_t)i * nblocks + blockIdx.x];
    __syncthreads();
    const long long tile0 = (long long)blockIdx.x * kTile;
    for (int round = 0; round < kItemsPerThread; ++round) {
        for (int i = threadIdx.x; i < (kSortThreads / 32) * 256; i += blockDim.x) (&warp_counts[0][0])[i] = 0;
        __syncthreads();
        long long g = tile0 + (long long)round * kSortThreads + threadIdx.x;
        bool valid = g < n;
        unsigned long long key = valid ? kin[g] : 0ULL;
        int val = valid ? vin[g] : 0;
        unsigned digit = (unsigned)((key >> shift) & 255ULL);
        unsigned peers = __match_any_sync(0xffffffffu, valid ? digit : 0x100u);
        unsigned rank_in_warp = __popc(peers & ((1u << lane) - 1u));
        if (valid && rank_in_warp == 0) warp_counts[warp][digit] = __popc(peers);
        __syncthreads();
        if (valid) {
            unsigned before = 0;
            for (int w = 0; w < warp; ++w) before += warp_counts[w][digit];
            unsigned pos = base[digit] + before + rank_in_warp;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        for (int dgt = threadIdx.x; dgt < 256; dgt += blockDim.x) {
            unsigned tot = 0;
            for (int w = 0; w < kSortThreads / 32; ++w) tot += warp_counts[w][dgt];
            base[dgt] += tot;
        }
        __syncthreads();
    }
}

// Exclusive scan of `len` counters in place by one block of 1024 threads
// (len = 256 x blocks of the sort, at most a few hundred thousand).
__global__ void __launch_bounds__(1024) scan_exclusive_kernel(unsigned* __restrict__ data, int len) {
    __shared__ unsigned partial[1024];
    const int t = threadIdx.x;
    const int per = (len + 1023) / 1024;
    const int b = t * per, e = min(len, b + per);
    unsigned s = 0;
    for (int i = b; i < e; ++i) s += data[i];
    partial[t] = s;
    __syncthreads();
    for (int off = 1; off < 1024; off <<= 1) {
        unsigned v = t >= off ? partial[t - off] : 0u;
        __syncthreads();
        partial[t] += v;
        __syncthreads();
    }
    unsigned run = t > 0 ? partial[t - 1] : 0u;
    for (int i = b; i < e; ++i) {
        unsigned v = data[i];
        data[i] = run;
        run += v;
    }
}

// Up to kSmallSort pairs: one block, a bitonic sort in shared memory by (key, val).
// The values are the input positions (ascending), so this is the stable order by key
// that the radix passes give, in one launch instead of three per digit.
constexpr int kSmallSort = 4096;
__global__ void __launch_bounds__(1024) small_sort_pairs_kernel(unsigned long long* __restrict__ keys,
                                                                int* __restrict__ vals, int n) {
    __shared__ unsigned long long sk[kSmallSort];
    __shared__ int sv[kSmallSort];
    int np = 2;
    while (np < n) np <<= 1;
    for (int i = threadIdx.x; i < np; i += blockDim.x) {
        sk[i] = i < n ? keys[i] : ~0ULL;
        sv[i] = i < n ? vals[i] : 0x7fffffff;
    }
    __syncthreads();
    for (int size = 2; size <= np; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int i = threadIdx.x; i < np / 2; i += blockDim.x) {
                const int lo = 2 * i - (i & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const unsigned long long ka = sk[lo], kb = sk[hi];
                const int va = sv[lo], vb = sv[hi];
                const bool gt = ka > kb || (ka == kb && va > vb);
                if (gt == up) {
                    sk[lo] = kb; sk[hi] = ka;
                    sv[lo] = vb; sv[hi] = va;
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        keys[i] = sk[i];
        vals[i] = sv[i];
    }
}

}  // namespace

int radix_sort_launches(long long n, int kbits) { return n <= kSmallSort ? 1 : 3 * ((kbits + 7) / 8); }

// Sort (keys, vals) ascending by key, stable (vals must be the input positions when n
// is at most kSmallSort).  `kbits` = number of key bits used.
cudaError_t radix_sort_pairs(unsigned long long* keys, int* vals, unsigned long long* ktmp, int* vtmp, long long n,
                             int kbits, unsigned* hist, void* scan_tmp, size_t scan_tmp_bytes, cudaStream_t st,
                             bool* result_in_tmp) {
    if (n <= kSmallSort) {
        if (n > 1) small_sort_pairs_kernel<<<1, 1024, 0, st>>>(keys, vals, (int)n);
        *result_in_tmp = false;
        return cudaGetLastError();
    }
    const int nblocks = (int)((n + kTile - 1) / kTile);
    unsigned long long *ka = keys, *kb = ktmp;
    int *va = vals, *vb = vtmp;
    int passes = (kbits + 7) / 8;
    for (int p = 0; p < passes; ++p) {
        int shift = 8 * p;
        radix_hist_kernel<<<nblocks, kSortThreads, 0, st>>>(ka, n, shift, hist, nblocks);
        scan_exclusive_kernel<<<1, 1024, 0, st>>>(hist, 256 * nblocks);
        radix_scatter_kernel<<<nblocks, kSortThreads, 0, st>>>(ka, va, kb, vb, n, shift, hist, nblocks);
        unsigned long long* tk = ka; ka = kb; kb = tk;
        int* tv = va; va = vb; vb = tv;
    }
    *result_in_tmp = (passes % 2) == 1;
    return cudaGetLastError();
}

size_t radix_scan_tmp_bytes(long long) { return 16; }

int radix_num_blocks(long long n) { return (int)((n + kTile - 1) / kTile); }

// Compute the batch order of `coords` (n x d, f32): order[i] = dataset row of
// sorted position i.  mode 1 = Hilbert (D-generic), 2 = Morton (D == 3 only).
cudaError_t compute_order(const float* coords, long long n, int d, int mode, int* order_out, cudaStream_t st,
                          unsigned long long* keys_by_id, double* bounds_out) {
    if (n <= 0) return cudaSuccess;
    double* mm = nullptr;
    unsigned long long *keys = nullptr, *ktmp = nullptr;
    int* vtmp = nullptr;
    unsigned* hist = nullptr;
    void* scan = nullptr;
    size_t scan_bytes = radix_scan_tmp_bytes(n);
    const int nb = radix_num_blocks(n);
    cudaError_t e = cudaMallocAsync((void**)&mm, sizeof(double) * 2 * 64, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&keys, sizeof(unsigned long long) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&ktmp, sizeof(unsigned long long) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&vtmp, sizeof(int) * n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&hist, sizeof(unsigned) * 256 * (size_t)nb, st);
    if (e == cudaSuccess) e = cudaMallocAsync(&scan, scan_bytes > 0 ? scan_bytes : 16, st);
    if (e == cudaSuccess) {
        double init[128];
        for (int c = 0; c < 64; ++c) { init[2 * c] = 1e300; init[2 * c + 1] = -1e300; }
        e = cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // `init` is a stack buffer
    }
    if (e == cudaSuccess) {
        minmax_kernel<<<152 * 4, 256, 0, st>>>(coords, n, d, mm);
        int kbits;
        if (mode == 2 && d == 3) {
            morton_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(coords, n, mm, keys, order_out);
            kbits = 63;
        } else {
            hilbert_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(coords, n, d, mm, keys, order_out);
            int bits = 64 / (d > 0 ? d : 1);
            bits = bits > 16 ? 16 : (bits < 1 ? 1 : bits);
            kbits = bits * d;
        }
        e = cudaGetLastError();
        if (e == cudaSuccess && keys_by_id)
            e = cudaMemcpyAsync(keys_by_id, keys, sizeof(unsigned long long) * n, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess && bounds_out)
            e = cudaMemcpyAsync(bounds_out, mm, sizeof(double) * 2 * 64, cudaMemcpyDeviceToDevice, st);
        bool in_tmp = false;
        if (e == cudaSuccess) e = radix_sort_pairs(keys, order_out, ktmp, vtmp, n, kbits, hist, scan, scan_bytes, st, &in_tmp);
        if (e == cudaSuccess && in_tmp) e = cudaMemcpyAsync(order_out, vtmp, sizeof(int) * n, cudaMemcpyDeviceToDevice, st);
    }
    cudaFreeAsync(mm, st); cudaFreeAsync(keys, st); cudaFreeAsync(ktmp, st); cudaFreeAsync(vtmp, st);
    cudaFreeAsync(hist, st); cudaFreeAsync(scan, st);
    return e;
}

// Hilbert keys of points in the frame of bounds computed by compute_order for
// another point set (coordinates outside it clamp to the edge cells).
cudaError_t hilbert_keys_bounded(const float* coords, long long n, int d, const double* bounds,
                                 unsigned long long* keys, int* scratch_vals, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    hilbert_keys_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(coords, n, d, bounds, keys, scratch_vals);
    return cudaGetLastError();
}

}  // namespace ct
