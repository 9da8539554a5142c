// ct_mis.cu — maximal independent set of a CSR conflict graph on the device, with
// the semantics of the reference's seeded Luby MIS (covertreex/algo/_mis_numba.py:
// 19-131, run_mis_numba :134-140):
//
//   * max degree <= 8: the deterministic greedy in index order
//     (_greedy_low_degree), reported as one iteration;
//   * otherwise Luby rounds r = 1, 2, ...: every node gets the priority
//     hash(node ^ seed ^ r * 0x9E3779B9) (xorshift 13/17/5, (x + 1) / 2^32); an active
//     node wins when no active neighbour has a higher priority, equal priorities going
//     to the lower index; if no node wins, the lowest-index active node does; winners
//     are selected and they and their neighbours leave the active set.
//
// The greedy runs as rounds too: an active node is selected once none of its
// lower-index neighbours is active.  That selects exactly the nodes the sequential
// greedy selects (a node is decided only after all its lower neighbours are, and a
// higher neighbour cannot be selected while it is active), in as many rounds as the
// longest chain of such dependencies.
//
// One thread per node and round; the host reads one counter per round (the number of
// nodes still active), so every loop ends after at most n rounds.
#include <climits>

#include "ct_common.cuh"
#include "ct_internal.h"

namespace ct {
namespace {

__device__ __forceinline__ double mis_priority(unsigned long long node, unsigned long long seed, unsigned iteration) {
    unsigned x = (unsigned)node ^ (unsigned)seed;
    x ^= (unsigned)((unsigned long long)iteration * 0x9E3779B9ULL);
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    return ((double)x + 1.0) / 4294967296.0;
}

__global__ void mis_init_kernel(long long n, const long long* __restrict__ indptr, unsigned char* __restrict__ active,
                                signed char* __restrict__ sel, int* __restrict__ maxdeg) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    active[i] = 1;
    sel[i] = 0;
    const long long deg = indptr[i + 1] - indptr[i];
    atomicMax(maxdeg, (int)(deg < INT_MAX ? deg : INT_MAX));
}

// Winners of one round.  greedy != 0: no active lower-index neighbour; else Luby.
__global__ void mis_round_kernel(long long n, const long long* __restrict__ indptr,
                                 const long long* __restrict__ indices, const unsigned char* __restrict__ active,
                                 unsigned char* __restrict__ win, unsigned long long seed, unsigned iteration,
                                 int greedy, int* __restrict__ any_win, unsigned long long* __restrict__ min_active) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    win[i] = 0;
    if (!active[i]) return;
    atomicMin(min_active, (unsigned long long)i);
    bool best = true;
    if (greedy) {
        for (long long o = indptr[i]; o < indptr[i + 1]; ++o) {
            const long long j = indices[o];
            if (j < i && active[j]) { best = false; break; }
        }
    } else {
        const double pi = mis_priority((unsigned long long)i, seed, iteration);
        for (long long o = indptr[i]; o < indptr[i + 1]; ++o) {
            const long long j = indices[o];
            if (!active[j]) continue;
            const double pj = mis_priority((unsigned long long)j, seed, iteration);
            if (pj > pi || (pj == pi && j < i)) { best = false; break; }
        }
    }
    if (best) {
        win[i] = 1;
        atomicOr(any_win, 1);
    }
}

// No winner: the lowest-index active node wins (the reference's fallback).
__global__ void mis_fallback_kernel(const int* __restrict__ any_win, const unsigned long long* __restrict__ min_active,
                                    long long n, unsigned char* __restrict__ win) {
    if (threadIdx.x == 0 && blockIdx.x == 0 && *any_win == 0 && *min_active < (unsigned long long)n)
        win[*min_active] = 1;
}

__global__ void mis_dominate_kernel(long long n, const long long* __restrict__ indptr,
                                    const long long* __restrict__ indices, const unsigned char* __restrict__ win,
                                    unsigned char* __restrict__ dom) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n || !win[i]) return;
    for (long long o = indptr[i]; o < indptr[i + 1]; ++o) dom[indices[o]] = 1;
}

__global__ void mis_update_kernel(long long n, const unsigned char* __restrict__ win, unsigned char* __restrict__ dom,
                                  unsigned char* __restrict__ active, signed char* __restrict__ sel,
                                  int* __restrict__ remaining) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (win[i]) sel[i] = 1;
    if (win[i] || dom[i]) active[i] = 0;
    dom[i] = 0;
    if (active[i]) atomicAdd(remaining, 1);
}

// Rejects graphs the kernels would read out of bounds: indptr not starting at 0 or
// not non-decreasing, or a neighbour index outside [0, n).
__global__ void mis_validate_kernel(long long n, const long long* __restrict__ indptr,
                                    const long long* __restrict__ indices, long long nnz, int* __restrict__ bad) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n && (indptr[t] > indptr[t + 1] || indptr[t] < 0 || indptr[t + 1] > nnz)) atomicOr(bad, 1);
    if (t == 0 && indptr[0] != 0) atomicOr(bad, 1);
    for (long long o = t; o < nnz; o += (long long)gridDim.x * blockDim.x)
        if (indices[o] < 0 || indices[o] >= n) atomicOr(bad, 2);
}

inline unsigned grid_of(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

// Checks the CSR arrays on the device; *valid <- false if a kernel would read out of
// bounds.  Synchronises `st`.
cudaError_t csr_graph_valid(const long long* indptr, const long long* indices, long long n, bool* valid,
                            cudaStream_t st) {
    *valid = false;
    long long nnz = 0;
    int* bad = nullptr;
    cudaError_t e = cudaMemcpyAsync(&nnz, indptr + n, sizeof(long long), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess || nnz < 0) return e;
    if (nnz > 0 && !indices) return cudaSuccess;
    e = cudaMallocAsync((void**)&bad, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(bad, 0, sizeof(int), st);
    if (e == cudaSuccess) {
        mis_validate_kernel<<<grid_of(n > 0 ? n : 1), 256, 0, st>>>(n, indptr, indices, nnz, bad);
        e = cudaGetLastError();
    }
    int hb = 1;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (bad) cudaFreeAsync(bad, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    *valid = e == cudaSuccess && hb == 0;
    return e;
}

// sel[n] (device int8) <- the independent set; *iterations <- the reference's count.
// The graph must have passed csr_graph_valid.  Synchronises `st` once per round.
cudaError_t luby_mis_csr(const long long* indptr, const long long* indices, long long n, unsigned long long seed,
                         signed char* sel, int* iterations, cudaStream_t st) {
    if (iterations) *iterations = 0;
    if (n <= 0) return cudaSuccess;
    unsigned char *active = nullptr, *win = nullptr, *dom = nullptr;
    int* counters = nullptr;  // int [0] maxdeg, [1] any_win, [2] remaining, [3] pad; u64 at byte 16: min_active
    cudaError_t e = cudaMallocAsync((void**)&active, (size_t)n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&win, (size_t)n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&dom, (size_t)n, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&counters, 32, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(dom, 0, (size_t)n, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(counters, 0, 32, st);
    if (e == cudaSuccess) {
        mis_init_kernel<<<grid_of(n), 256, 0, st>>>(n, indptr, active, sel, counters);
        e = cudaGetLastError();
    }
    int maxdeg = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&maxdeg, counters, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    const int greedy = maxdeg <= 8;
    unsigned long long* min_active = (unsigned long long*)(counters + 4);
    int rounds = 0;
    while (e == cudaSuccess && rounds < n + 1) {
        ++rounds;
        e = cudaMemsetAsync(counters + 1, 0, 3 * sizeof(int), st);            // any_win, remaining, pad
        if (e == cudaSuccess) e = cudaMemsetAsync(min_active, 0xff, sizeof(unsigned long long), st);
        if (e != cudaSuccess) break;
        mis_round_kernel<<<grid_of(n), 256, 0, st>>>(n, indptr, indices, active, win, seed, (unsigned)rounds, greedy,
                                                     counters + 1, min_active);
        mis_fallback_kernel<<<1, 32, 0, st>>>(counters + 1, min_active, n, win);
        mis_dominate_kernel<<<grid_of(n), 256, 0, st>>>(n, indptr, indices, win, dom);
        mis_update_kernel<<<grid_of(n), 256, 0, st>>>(n, win, dom, active, sel, counters + 2);
        int remaining = 0;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&remaining, counters + 2, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (remaining == 0) break;
    }
    if (iterations) *iterations = greedy ? 1 : rounds;
    cudaFreeAsync(active, st);
    cudaFreeAsync(win, st);
    cudaFreeAsync(dom, st);
    cudaFreeAsync(counters, st);
    return e;
}

}  // namespace ct
