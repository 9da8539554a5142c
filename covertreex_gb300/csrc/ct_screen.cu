// ct_screen.cu — precision form: BF16 tcgen05 screening with certified bounds,
// then FP64-grade rescoring of the survivors.
//
// Pipeline of one ct_knn_residual(form = CT_FORM_SCREENED) call:
//   1. Operands.  V is split as v = hi + lo (hi = bf16(v), lo = bf16(v - hi)) and
//      stored in the UMMA "blocked" layout: for each K-chunk of 32 columns and
//      each group of 8 rows, one 512-byte block of four 8x8 core matrices.  A
//      K-chunk of a 128- or 256-row tile is therefore one contiguous span that a
//      single 1-D bulk copy (TMA) moves into shared memory.
//   2. Pass A (threshold).  Query tiles in Hilbert order meet the W candidate
//      tiles around them in Hilbert order.  s = hi.hi + hi.lo + lo.hi is
//      accumulated in TMEM by tcgen05.mma (kind::f16, M=128, N=256, K=16); the
//      epilogue turns s into a certified upper bound of each squared residual
//      distance, and tau_q^2 is the k-th smallest bound among valid candidates,
//      an upper bound of the true k-th distance.
//   3. Pass B (screen).  Query tiles in dataset order sweep the candidate tiles
//      (the lower triangle in predecessor mode); every candidate whose certified
//      lower bound is <= tau_q^2 is appended to the query's survivor list.
//   4. Rescore.  Each survivor's distance is recomputed from the f32 inputs with
//      a compensated FP32 dot product (TwoProd/TwoSum) and an FP64 kernel value
//      and normalisation; the k best (distance, index) pairs are written out.
//      Queries whose list overflowed are rescored against every valid candidate.
//
// Error bound of the screened dot (per pair), with u = 2^-8 (bf16) and
// v = hi + lo + r, |r| <= u^2 |v|:  |s - v_q.v_c| <= c_split ||v_q|| ||v_c|| with
// c_split = 3.1 u^2 + (3 m / 16 + 17) 2^-22, the second term covering FP32
// accumulation inside the tensor core (one rounding per MMA step plus the
// step's internal alignment), both relative to sum |v_qi v_ci| <= ||v_q|| ||v_c||.
#include <cuda_bf16.h>

#include <cmath>
#include <vector>

#include "ct_common.cuh"
#include "ct_internal.h"
#include "ct_sm100.cuh"
#include "ct_tree.h"

namespace ct {
namespace screen {

using bf16 = __nv_bfloat16;
namespace sm = ct::sm100;

constexpr int TQ = 128;
constexpr int TC = 256;
constexpr int KC = 32;
constexpr int STAGES = 3;
constexpr int CHUNK_A = TQ * KC * 2;  // bytes
constexpr int CHUNK_B = TC * KC * 2;
constexpr int STAGE_BYTES = 2 * CHUNK_A + 2 * CHUNK_B;
constexpr int kEpiWarps = 8;
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kMaxD = 8;
constexpr int WINDOW_TILES = 4;
constexpr int SURV_CAP = 1024;
constexpr int RBUF = 1024;  // rescoring sort buffer (power of two)

enum Mode { MODE_DEBUG = 0, MODE_WINDOW = 1, MODE_FILTER = 2 };

// element offset of (row, col) in a blocked matrix with G = rows_pad / 8 row groups
__host__ __device__ inline size_t blocked_offset(long long row, int col, long long G) {
    int c = col >> 5, j = (col >> 3) & 3, e = col & 7;
    long long g = row >> 3;
    int rr = (int)(row & 7);
    return ((size_t)c * (size_t)G + (size_t)g) * 256 + (size_t)j * 64 + (size_t)rr * 8 + e;
}

struct Job {
    int qtile, ctile, slot, pad;
};

struct MMAParams {
    const bf16* a_hi; const bf16* a_lo; long long a_groups;
    const bf16* b_hi; const bf16* b_lo; long long b_groups;
    int m;
    const Job* jobs; int njobs;
    const int* a_slot;   // A row -> query slot (or -1)
    const int* slot_id;  // query slot -> dataset id
    const int* b_id;     // B row -> dataset id (or -1)
    const float* xs; int d;
    const float* vn; const float* isp; const float* xmax;
    float var; int kernel_type; int predecessor;
    float err_coef;
    int mode;
    float* out_f; int out_stride;
    const float* tau2;   // per slot
    int* surv; int* surv_cnt;
    int* status;
};

struct SmemLayout {
    size_t stages, cand, bars, tmem_slot, total;
};
__host__ __device__ inline SmemLayout smem_layout() {
    SmemLayout L;
    size_t off = 0;
    L.stages = off; off += (size_t)STAGES * STAGE_BYTES;
    L.cand = off;
    L.bars = off; off += (size_t)(2 * STAGES + 4 + 1) * 8;
    L.tmem_slot = off; off += 16;
    L.total = off + 1024;  // alignment slack
    return L;
}

// Certified squared-distance bounds of one pair from the screened dot s.
// xc: candidate scaled coordinates, vnc = ||v_c|| (rounded up), isc = 1/sqrt(p_c),
// xmc = max |xs_c|.
__device__ __forceinline__ void pair_bounds(float s, const float (&xq)[kMaxD], float vnq, float isq, float xmq,
                                            const float (&xc)[kMaxD], float vnc, float isc, float xmc, int d,
                                            float var, int kt, float err_coef, float& dl2, float& du2) {
    float d2 = 0.f, sabs = 0.f;
#pragma unroll
    for (int c = 0; c < kMaxD; ++c) {
        if (c < d) {
            float t = xq[c] - xc[c];
            d2 = fmaf(t, t, d2);
            sabs += fabsf(t);
        }
    }
    // error of d2: rounding of the sum of squares + rounding of the scaled coordinates
    float ed2 = (float)(d + 2) * 5.97e-8f * d2 + 2.39e-7f * sabs * (xmq + xmc);
    float kv, ek;
    if (kt == 0) {
        kv = var * expf(-0.5f * d2);
        ek = kv * (1e-6f + 0.5f * ed2);
    } else {
        float r = sqrtf(d2);
        float a = 2.2360679775f * r;
        float ea = expf(-a);
        kv = var * (1.f + a + a * a * 0.33333334f) * ea;
        // |dK/dd2| = var (5/6)(1+a) e^-a ; rounding of a, poly and exp bounded by 1e-6 K + a^2 term
        ek = kv * 1e-6f + var * (0.8334f * ed2 + 1e-7f * a * a) * (1.f + a) * ea;
    }
    float R = fabsf(kv - s);
    float e = err_coef * vnq * vnc + ek + R * 1.2e-7f + 1e-30f;
    float sc = isq * isc;
    float rho_hi = (R + e) * sc * (1.f + 1e-6f);
    float rho_lo = fmaxf(R - e, 0.f) * sc * (1.f - 1e-6f);
    dl2 = 1.f - fminf(rho_hi, 1.f);
    du2 = 1.f - fminf(rho_lo, 1.f);
}

__global__ void __launch_bounds__(kThreads, 1) screen_mma_kernel(MMAParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const SmemLayout L = smem_layout();
    unsigned char* stage_base = smem + L.stages;
    uint64_t* full = (uint64_t*)(smem + L.bars);
    uint64_t* empty = full + STAGES;
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* done = acce + 2;
    uint32_t* tmem_slot = (uint32_t*)(smem + L.tmem_slot);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = P.m / KC;
    const uint32_t idesc = sm::idesc_bf16_f32(TQ, TC);

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) { sm::mbar_init(&full[s], 1); sm::mbar_init(&empty[s], 1); }
        for (int a = 0; a < 2; ++a) { sm::mbar_init(&accf[a], 1); sm::mbar_init(&acce[a], kEpiWarps); }
        sm::mbar_init(done, 1);
        sm::fence_barrier_init();
    }
    if (warp == 1) {
        sm::tmem_alloc(tmem_slot, 512);
        sm::tmem_relinquish();
    }
    sm::tc_fence_before();
    __syncthreads();
    sm::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            long long it = 0;
            for (int j = blockIdx.x; j < P.njobs; j += gridDim.x) {
                const Job jb = P.jobs[j];
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int s = (int)(it % STAGES);
                    const unsigned ph = (unsigned)((it / STAGES) & 1);
                    if (!sm::mbar_wait(&empty[s], ph ^ 1u, P.status, 11)) goto producer_done;
                    unsigned char* dst = stage_base + (size_t)s * STAGE_BYTES;
                    sm::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                    const size_t aoff = blocked_offset((long long)jb.qtile * TQ, c * KC, P.a_groups);
                    const size_t boff = blocked_offset((long long)jb.ctile * TC, c * KC, P.b_groups);
                    sm::bulk_g2s(dst, P.a_hi + aoff, CHUNK_A, &full[s]);
                    sm::bulk_g2s(dst + CHUNK_A, P.a_lo + aoff, CHUNK_A, &full[s]);
                    sm::bulk_g2s(dst + 2 * CHUNK_A, P.b_hi + boff, CHUNK_B, &full[s]);
                    sm::bulk_g2s(dst + 2 * CHUNK_A + CHUNK_B, P.b_lo + boff, CHUNK_B, &full[s]);
                }
            }
        producer_done:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            long long it = 0;
            int lt = 0;
            for (int j = blockIdx.x; j < P.njobs; j += gridDim.x, ++lt) {
                const int acc = lt & 1;
                const unsigned aph = (unsigned)((lt >> 1) & 1);
                if (!sm::mbar_wait(&acce[acc], aph ^ 1u, P.status, 12)) break;
                sm::tc_fence_after();
                const uint32_t dt = tmem_base + (uint32_t)(acc * TC);
                bool ok = true;
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int s = (int)(it % STAGES);
                    const unsigned ph = (unsigned)((it / STAGES) & 1);
                    if (!sm::mbar_wait(&full[s], ph, P.status, 13)) { ok = false; break; }
                    sm::tc_fence_after();
                    unsigned char* st = stage_base + (size_t)s * STAGE_BYTES;
#pragma unroll
                    for (int kk = 0; kk < KC / 16; ++kk) {
                        const uint64_t ahi = sm::smem_desc(st + kk * 256, 128, 512);
                        const uint64_t alo = sm::smem_desc(st + CHUNK_A + kk * 256, 128, 512);
                        const uint64_t bhi = sm::smem_desc(st + 2 * CHUNK_A + kk * 256, 128, 512);
                        const uint64_t blo = sm::smem_desc(st + 2 * CHUNK_A + CHUNK_B + kk * 256, 128, 512);
                        sm::mma_bf16(dt, ahi, bhi, idesc, !(c == 0 && kk == 0));
                        sm::mma_bf16(dt, ahi, blo, idesc, true);
                        sm::mma_bf16(dt, alo, bhi, idesc, true);
                    }
                    sm::mma_commit(&empty[s]);
                }
                if (!ok) break;
                sm::mma_commit(&accf[acc]);
            }
            // drain: every MMA issued by this thread has completed once `done` flips
            sm::mma_commit(done);
            sm::mbar_wait(done, 0, P.status, 14);
        }
    } else {
        // ------------------------------------------------------------ epilogue
        const int quarter = warp & 3;        // TMEM lanes 32*quarter ..
        const int half = (warp - 2) >> 2;    // columns half*128 ..
        const int row = quarter * 32 + lane;
        int lt = 0;
        for (int j = blockIdx.x; j < P.njobs; j += gridDim.x, ++lt) {
            const Job jb = P.jobs[j];
            const int acc = lt & 1;
            const unsigned aph = (unsigned)((lt >> 1) & 1);
            const long long arow = (long long)jb.qtile * TQ + row;
            const int slot = P.mode != MODE_DEBUG ? P.a_slot[arow] : -1;
            const int qid = slot >= 0 ? P.slot_id[slot] : -1;
            float xq[kMaxD];
            float vnq = 0.f, isq = 0.f, xmq = 0.f, tau2 = -1.f;
#pragma unroll
            for (int c = 0; c < kMaxD; ++c) xq[c] = 0.f;
            if (qid >= 0) {
                vnq = P.vn[qid]; isq = P.isp[qid]; xmq = P.xmax[qid];
#pragma unroll
                for (int c = 0; c < kMaxD; ++c) if (c < P.d) xq[c] = P.xs[(size_t)qid * P.d + c];
                if (P.mode == MODE_FILTER) tau2 = P.tau2[slot];
            }
            if (!sm::mbar_wait(&accf[acc], aph, P.status, 15)) break;
            sm::tc_fence_after();
            for (int cc = 0; cc < 4; ++cc) {
                float v[32];
                const int col0 = half * 128 + cc * 32;
                sm::tmem_ld32(tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TC + col0), v);
                if (P.mode == MODE_DEBUG) {
                    float* o = P.out_f + ((size_t)j * TQ + row) * TC + col0;
#pragma unroll
                    for (int i = 0; i < 32; ++i) o[i] = v[i];
                    continue;
                }
                // lane i holds the record of candidate col0 + i; broadcast by shuffles
                const long long brow = (long long)jb.ctile * TC + col0 + lane;
                const int my_cid = P.b_id[brow];
                float my_vn = 0.f, my_isp = 0.f, my_xm = 0.f;
                float my_x[kMaxD];
#pragma unroll
                for (int c = 0; c < kMaxD; ++c) my_x[c] = 0.f;
                if (my_cid >= 0) {
                    my_vn = P.vn[my_cid]; my_isp = P.isp[my_cid]; my_xm = P.xmax[my_cid];
#pragma unroll
                    for (int c = 0; c < kMaxD; ++c) if (c < P.d) my_x[c] = P.xs[(size_t)my_cid * P.d + c];
                }
#pragma unroll 2
                for (int i = 0; i < 32; ++i) {
                    const int cid = __shfl_sync(0xffffffffu, my_cid, i);
                    const float vnc = __shfl_sync(0xffffffffu, my_vn, i);
                    const float isc = __shfl_sync(0xffffffffu, my_isp, i);
                    const float xmc = __shfl_sync(0xffffffffu, my_xm, i);
                    float xc[kMaxD];
#pragma unroll
                    for (int c = 0; c < kMaxD; ++c) xc[c] = __shfl_sync(0xffffffffu, my_x[c], i);
                    if (qid < 0) continue;
                    const bool valid = cid >= 0 && (!P.predecessor || cid < qid);
                    float dl2 = 0.f, du2 = 0.f;
                    if (valid && cid != qid)
                        pair_bounds(v[i], xq, vnq, isq, xmq, xc, vnc, isc, xmc, P.d, P.var, P.kernel_type,
                                    P.err_coef, dl2, du2);
                    if (P.mode == MODE_WINDOW) {
                        P.out_f[(size_t)slot * P.out_stride + (size_t)jb.slot * TC + col0 + i] = valid ? du2 : 2.0f;
                    } else if (valid && dl2 <= tau2) {
                        int k = atomicAdd(&P.surv_cnt[slot], 1);
                        if (k < SURV_CAP) P.surv[(size_t)slot * SURV_CAP + k] = cid;
                    }
                }
            }
            sm::tc_fence_before();
            __syncwarp();
            if (lane == 0) sm::mbar_arrive(&acce[acc]);
        }
    }
    sm::tc_fence_before();
    __syncthreads();
    if (warp == 1) sm::tmem_dealloc(tmem_base, 512);
}

// -------------------------------------------------------------- operand prep
// hi/lo split of V rows into the blocked layout.  rowmap[r] = dataset row of
// blocked row r (or -1 for a zero row).  One thread per (row, 8-column group).
__global__ void split_blocked_kernel(const float* __restrict__ v, int m, const int* __restrict__ rowmap,
                                     long long rows_pad, bf16* __restrict__ hi, bf16* __restrict__ lo) {
    const long long groups = (long long)m / 8;
    const long long total = rows_pad * groups;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long r = t / groups;
        int cg = (int)(t - r * groups);
        int src = rowmap ? rowmap[r] : (int)r;
        __align__(16) bf16 h8[8];
        __align__(16) bf16 l8[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            float x = src >= 0 ? v[(size_t)src * m + cg * 8 + e] : 0.f;
            bf16 h = __float2bfloat16_rn(x);
            float rem = x - __bfloat162float(h);
            h8[e] = h;
            l8[e] = __float2bfloat16_rn(rem);
        }
        size_t off = blocked_offset(r, cg * 8, rows_pad / 8);
        *(uint4*)(hi + off) = *(const uint4*)h8;
        *(uint4*)(lo + off) = *(const uint4*)l8;
    }
}

// vn = ||v|| rounded up, isp = 1/sqrt(p), xmax = max |xs|.
__global__ void point_scalars_kernel(const float* __restrict__ v, const float* __restrict__ p,
                                     const float* __restrict__ xs, long long n, int m, int d, float* __restrict__ vn,
                                     float* __restrict__ isp, float* __restrict__ xmax) {
    long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= n) return;
    double s = 0.0;
    for (int c = 0; c < m; ++c) { double x = v[(size_t)r * m + c]; s += x * x; }
    vn[r] = __double2float_ru(sqrt(s) * (1.0 + 1e-12));
    isp[r] = (float)(1.0 / sqrt((double)p[r]));
    float mx = 0.f;
    for (int c = 0; c < d; ++c) mx = fmaxf(mx, fabsf(xs[(size_t)r * d + c]));
    xmax[r] = mx;
}

// ------------------------------------------------------------------ selection
// Bitonic sort of RBUF 64-bit keys held in shared memory by one warp.
__device__ void warp_bitonic_sort(unsigned long long* keys) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= RBUF; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < RBUF; i += 32) {
                int ixj = i ^ j;
                if (ixj > i) {
                    unsigned long long a = keys[i], b = keys[ixj];
                    bool up = (i & k) == 0;
                    if ((a > b) == up) { keys[i] = b; keys[ixj] = a; }
                }
            }
            __syncwarp();
        }
    }
}

__device__ __forceinline__ unsigned long long pack_key(float d, int id) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)id;
}

// tau2[slot] = k-th smallest certified upper bound in the slot's window row.
__global__ void window_tau_kernel(const float* __restrict__ win, int width, const int* __restrict__ a_slot,
                                  long long a_rows, int k, float* __restrict__ tau2) {
    extern __shared__ unsigned long long skeys[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned long long* keys = skeys + (size_t)warp * RBUF;
    long long row = (long long)blockIdx.x * (blockDim.x / 32) + warp;
    if (row >= a_rows) return;
    int slot = a_slot[row];
    if (slot < 0) return;
    for (int i = lane; i < RBUF; i += 32) {
        float v = i < width ? win[(size_t)slot * width + i] : 2.0f;
        keys[i] = pack_key(v, i);
    }
    __syncwarp();
    warp_bitonic_sort(keys);
    if (lane == 0) {
        float t = __uint_as_float((unsigned)(keys[k - 1] >> 32));
        tau2[slot] = t > 1.0f ? 1.0f : t;   // fewer than k valid: no pruning
    }
}

// ------------------------------------------------------------------ rescoring
struct RescoreParams {
    const float* v; int m;          // natural layout, dataset order
    const float* coords; int d;     // raw coordinates, dataset order
    const double* inv_ls;           // FP64 1 / lengthscale
    const float* p;
    double var; int kernel_type; int predecessor;
    long long n;
    const int* slot_id; long long nslots;
    const int* surv; const int* surv_cnt;
    const int* full_slots; int nfull;  // slots rescored against every valid candidate
    int k;
    long long* out_idx; float* out_dist;
    long long* evals;
};

// FP64-grade residual distance of (q, c): compensated FP32 dot (TwoProd via FMA,
// TwoSum), FP64 kernel value, normalisation and square root.  The warp holds
// the query row as vq[t] = v_q[32 t + lane] (m <= 1024).
__device__ __forceinline__ float exact_distance(const RescoreParams& P, int q, int c, const float (&vq)[32]) {
    const int lane = threadIdx.x & 31;
    float s = 0.f, comp = 0.f;
    const float* vc = P.v + (size_t)c * P.m;
#pragma unroll
    for (int t = 0; t < 32; ++t) {
        const int e = t * 32 + lane;
        if (e < P.m) {
            float a = vq[t], b = vc[e];
            float pr = a * b;
            float pe = fmaf(a, b, -pr);
            float ts = s + pr;
            float z = ts - s;
            float se = (s - (ts - z)) + (pr - z);
            s = ts;
            comp += se + pe;
        }
    }
    double dot = (double)s + (double)comp;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, off);
    if (q == c) return 0.f;
    double d2 = 0.0;
    for (int a = 0; a < P.d; ++a) {
        double t = ((double)P.coords[(size_t)q * P.d + a] - (double)P.coords[(size_t)c * P.d + a]) * P.inv_ls[a];
        d2 += t * t;
    }
    double kv;
    if (P.kernel_type == 0) {
        kv = P.var * exp(-0.5 * d2);
    } else {
        double a = sqrt(5.0) * sqrt(d2);
        kv = P.var * (1.0 + a + a * a / 3.0) * exp(-a);
    }
    double pp = (double)P.p[q] * (double)P.p[c];
    double denom = sqrt(pp > 1e-18 ? pp : 1e-18);
    double rho = (kv - dot) / denom;
    rho = rho < -1.0 ? -1.0 : (rho > 1.0 ? 1.0 : rho);
    double ds = 1.0 - fabs(rho);
    return (float)(ds > 0.0 ? sqrt(ds) : 0.0);
}

// One warp per query slot.  Candidates: the survivor list, or the full range
// [0, limit) for slots listed in full_slots.  Streaming top-k through a sorted
// shared buffer: entries [0, k) hold the current best, new candidates fill the
// rest, and a full buffer is re-sorted.
__global__ void rescore_kernel(RescoreParams P, int use_full) {
    extern __shared__ unsigned long long rkeys_all[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x / 32;
    unsigned long long* keys = rkeys_all + (size_t)warp * RBUF;
    long long w = (long long)blockIdx.x * wpb + warp;
    long long nwork = use_full ? P.nfull : P.nslots;
    if (w >= nwork) return;
    const int slot = use_full ? P.full_slots[w] : (int)w;
    if (!use_full && P.surv_cnt[slot] > SURV_CAP) return;  // handled by the full pass
    const int q = P.slot_id[slot];
    const int k = P.k;
    // query row slice held per lane
    float vql[32];
#pragma unroll
    for (int t = 0; t < 32; ++t) vql[t] = (t * 32 + lane < P.m) ? P.v[(size_t)q * P.m + t * 32 + lane] : 0.f;
    for (int i = lane; i < RBUF; i += 32) keys[i] = ~0ULL;
    __syncwarp();
    long long count = use_full ? (P.predecessor ? (long long)q : P.n) : (long long)P.surv_cnt[slot];
    int fill = k;  // next free position in the buffer
    long long evals = 0;
    for (long long base = 0; base < count; base += 32) {
        // each lane fetches one candidate id; the warp scores them one at a time
        long long ci = base + lane;
        int cid = -1;
        if (ci < count) cid = use_full ? (int)ci : P.surv[(size_t)slot * SURV_CAP + ci];
        float mydist = 0.f;
        const int nb = (int)((count - base) < 32 ? (count - base) : 32);
        for (int t = 0; t < nb; ++t) {
            int c = __shfl_sync(0xffffffffu, cid, t);
            float dist = exact_distance(P, q, c, vql);
            if (lane == t) mydist = dist;
        }
        evals += nb;
        // append to buffer
        bool has = ci < count;
        unsigned mask = __ballot_sync(0xffffffffu, has);
        int pos = fill + __popc(mask & ((1u << lane) - 1u));
        int added = __popc(mask);
        if (fill + added > RBUF) {
            // flush: sort and keep the best k, then append
            __syncwarp();
            warp_bitonic_sort(keys);
            for (int i = k + lane; i < RBUF; i += 32) keys[i] = ~0ULL;
            __syncwarp();
            fill = k;
            pos = fill + __popc(mask & ((1u << lane) - 1u));
        }
        if (has) keys[pos] = pack_key(mydist, cid);
        fill += added;
        __syncwarp();
    }
    warp_bitonic_sort(keys);
    for (int j = lane; j < k; j += 32) {
        unsigned long long key = keys[j];
        bool ok = key != ~0ULL;
        P.out_idx[(size_t)slot * k + j] = ok ? (long long)(unsigned)(key & 0xffffffffULL) : -1LL;
        P.out_dist[(size_t)slot * k + j] = ok ? __uint_as_float((unsigned)(key >> 32)) : CT_FLT_MAX;
    }
    if (lane == 0 && P.evals) atomicAdd((unsigned long long*)P.evals, (unsigned long long)evals);
}

__global__ void collect_overflow_kernel(const int* __restrict__ surv_cnt, long long nslots, int* __restrict__ list,
                                        int* __restrict__ nlist) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    if (surv_cnt[s] > SURV_CAP) list[atomicAdd(nlist, 1)] = (int)s;
}

__global__ void debug_jobs_kernel(Job* jobs, int njobs, int nqt, int nct) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    jobs[j].qtile = j / nct;
    jobs[j].ctile = j % nct;
    jobs[j].slot = 0;
    jobs[j].pad = 0;
}

}  // namespace screen
}  // namespace ct

// ======================================================================= host
namespace ct {
namespace screen {

struct State {
    long long n = 0, rows_pad = 0;        // candidate rows padded to TC
    int* hil_order = nullptr;             // sorted position -> dataset id
    int* hil_pos = nullptr;               // dataset id -> sorted position
    bf16 *ds_hi = nullptr, *ds_lo = nullptr;    // dataset order, blocked
    bf16 *hil_hi = nullptr, *hil_lo = nullptr;  // Hilbert order, blocked
    int* b_id_ds = nullptr;
    int* b_id_hil = nullptr;
    float *vn = nullptr, *isp = nullptr, *xmax = nullptr;
    double* inv_ls64 = nullptr;
    int* status = nullptr;
    std::vector<int> hil_order_host;
};

__global__ void iota_kernel(int* a, long long n, long long valid) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = i < valid ? (int)i : -1;
}
__global__ void gather_ids_kernel(const int* order, long long n, long long rows, int* out) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < rows) out[i] = i < n ? order[i] : -1;
}
__global__ void inverse_perm_kernel(const int* order, long long n, int* inv) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) inv[order[i]] = (int)i;
}
// slot ids from int64 query ids; out-of-range ids become -1
__global__ void slot_ids_kernel(const long long* q, long long nq, long long n, int* slot_id,
                                unsigned long long* key_ds, unsigned long long* key_hil, int* val_ds, int* val_hil,
                                const int* hil_pos) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nq) return;
    long long id = q[i];
    bool ok = id >= 0 && id < n;
    slot_id[i] = ok ? (int)id : -1;
    key_ds[i] = ok ? (unsigned long long)id : (unsigned long long)n;
    key_hil[i] = ok ? (unsigned long long)hil_pos[id] : (unsigned long long)n;
    val_ds[i] = (int)i;
    val_hil[i] = (int)i;
}
// rowmap (A row -> dataset row) and a_slot (A row -> slot) from a sorted slot list
__global__ void arows_kernel(const int* sorted_slots, long long nq, long long rows, const int* slot_id, int* a_slot,
                             int* rowmap) {
    long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    int s = r < nq ? sorted_slots[r] : -1;
    int id = s >= 0 ? slot_id[s] : -1;
    a_slot[r] = id >= 0 ? s : -1;
    rowmap[r] = id;
}

static inline unsigned grid_for(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

static float err_coef_for(int m) {
    const double u2 = 1.0 / 65536.0;
    return (float)(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * std::ldexp(1.0, -22));
}

static cudaError_t launch_mma(const MMAParams& P, cudaStream_t st) {
    const size_t smem = smem_layout().total;
    cudaError_t e = cudaFuncSetAttribute(screen_mma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int grid = P.njobs < sms ? P.njobs : sms;
    if (grid <= 0) return cudaSuccess;
    screen_mma_kernel<<<grid, kThreads, smem, st>>>(P);
    return cudaGetLastError();
}

}  // namespace screen
}  // namespace ct

using namespace ct::screen;

void ct_tree::release_screen() {
    State* S = (State*)screen;
    if (!S) return;
    cudaFree(S->hil_order); cudaFree(S->hil_pos); cudaFree(S->ds_hi); cudaFree(S->ds_lo);
    cudaFree(S->hil_hi); cudaFree(S->hil_lo); cudaFree(S->b_id_ds); cudaFree(S->b_id_hil);
    cudaFree(S->vn); cudaFree(S->isp); cudaFree(S->xmax); cudaFree(S->inv_ls64); cudaFree(S->status);
    delete S;
    screen = nullptr;
}

// Build the screened-form operands once per tree (lazily, on first use).
static int screen_prepare(ct_tree* T, cudaStream_t st) {
    if (T->screen) return CT_OK;
    State* S = new State();
    T->screen = S;
    const long long n = T->n;
    S->n = n;
    S->rows_pad = ((n + TC - 1) / TC) * TC;
    const int m = T->m;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 16); };
    A((void**)&S->hil_order, sizeof(int) * n);
    A((void**)&S->hil_pos, sizeof(int) * n);
    A((void**)&S->ds_hi, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->ds_lo, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->hil_hi, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->hil_lo, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->b_id_ds, sizeof(int) * S->rows_pad);
    A((void**)&S->b_id_hil, sizeof(int) * S->rows_pad);
    A((void**)&S->vn, sizeof(float) * n);
    A((void**)&S->isp, sizeof(float) * n);
    A((void**)&S->xmax, sizeof(float) * n);
    A((void**)&S->inv_ls64, sizeof(double) * 64);
    A((void**)&S->status, sizeof(int));
    if (e != cudaSuccess) return T->set_err(CT_ERR_NOMEM, "screen prep allocation: %s", cudaGetErrorString(e));
    e = ct::compute_order(T->coords_raw, n, T->d, 1, S->hil_order, st);
    if (e == cudaSuccess) {
        inverse_perm_kernel<<<grid_for(n), 256, 0, st>>>(S->hil_order, n, S->hil_pos);
        iota_kernel<<<grid_for(S->rows_pad), 256, 0, st>>>(S->b_id_ds, S->rows_pad, n);
        gather_ids_kernel<<<grid_for(S->rows_pad), 256, 0, st>>>(S->hil_order, n, S->rows_pad, S->b_id_hil);
        split_blocked_kernel<<<152 * 8, 256, 0, st>>>(T->vnat, m, S->b_id_ds, S->rows_pad, S->ds_hi, S->ds_lo);
        split_blocked_kernel<<<152 * 8, 256, 0, st>>>(T->vnat, m, S->b_id_hil, S->rows_pad, S->hil_hi, S->hil_lo);
        point_scalars_kernel<<<grid_for(n), 256, 0, st>>>(T->vnat, T->p, T->xs, n, m, T->d, S->vn, S->isp, S->xmax);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        double ils[64];
        for (int i = 0; i < T->d; ++i) ils[i] = T->inv_ls_host64[i];
        e = cudaMemcpyAsync(S->inv_ls64, ils, sizeof(double) * T->d, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(int), st);
        if (e == cudaSuccess) {
            S->hil_order_host.resize(n);
            e = cudaMemcpyAsync(S->hil_order_host.data(), S->hil_order, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    if (e != cudaSuccess) return T->set_err(CT_ERR_CUDA, "screen prep: %s", cudaGetErrorString(e));
    return CT_OK;
}

int ct_tree::knn_screened(const int64_t* q_ids, int64_t nq, int k, int predecessor, int64_t* out_idx, float* out_dist,
                          ct_stats* stats, cudaStream_t st) {
    if (d > kMaxD) return set_err(CT_ERR_UNSUPPORTED, "screened form supports d <= %d (got %d)", kMaxD, d);
    if (m % KC != 0 || m > 1024) return set_err(CT_ERR_UNSUPPORTED, "screened form needs m %% 32 == 0 and m <= 1024 (got %d)", m);
    if (k > 512) return set_err(CT_ERR_UNSUPPORTED, "screened form supports k <= 512");
    int rc = screen_prepare(this, st);
    if (rc != CT_OK) return rc;
    State* S = (State*)screen;
    const long long rows_q = ((nq + TQ - 1) / TQ) * TQ;
    const long long nqt = rows_q / TQ;
    const long long nct = S->rows_pad / TC;
    cudaError_t e = cudaSuccess;
    // ---- per-call buffers
    int *slot_id = nullptr, *val_ds = nullptr, *val_hil = nullptr, *vtmp = nullptr;
    unsigned long long *key_ds = nullptr, *key_hil = nullptr, *ktmp = nullptr;
    unsigned* hist = nullptr;
    int *a_slot_ds = nullptr, *a_slot_hil = nullptr, *rowmap_ds = nullptr, *rowmap_hil = nullptr;
    bf16 *aq_hi = nullptr, *aq_lo = nullptr, *ah_hi = nullptr, *ah_lo = nullptr;
    float *win = nullptr, *tau2 = nullptr;
    int *surv = nullptr, *surv_cnt = nullptr, *full_list = nullptr, *nfull_d = nullptr;
    long long* evals_d = nullptr;
    Job *jobs_a = nullptr, *jobs_b = nullptr;
    const int nbh = ct::radix_num_blocks(nq);
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMallocAsync(p, bytes ? bytes : 16, st); };
    A((void**)&slot_id, sizeof(int) * nq);
    A((void**)&val_ds, sizeof(int) * nq); A((void**)&val_hil, sizeof(int) * nq); A((void**)&vtmp, sizeof(int) * nq);
    A((void**)&key_ds, 8 * nq); A((void**)&key_hil, 8 * nq); A((void**)&ktmp, 8 * nq);
    A((void**)&hist, sizeof(unsigned) * 256 * (size_t)nbh);
    A((void**)&a_slot_ds, sizeof(int) * rows_q); A((void**)&a_slot_hil, sizeof(int) * rows_q);
    A((void**)&rowmap_ds, sizeof(int) * rows_q); A((void**)&rowmap_hil, sizeof(int) * rows_q);
    A((void**)&win, sizeof(float) * nq * WINDOW_TILES * TC);
    A((void**)&tau2, sizeof(float) * nq);
    A((void**)&surv, sizeof(int) * nq * SURV_CAP);
    A((void**)&surv_cnt, sizeof(int) * nq);
    A((void**)&full_list, sizeof(int) * nq);
    A((void**)&nfull_d, sizeof(int));
    A((void**)&evals_d, sizeof(long long));
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "screened form allocation: %s", cudaGetErrorString(e));

    slot_ids_kernel<<<grid_for(nq), 256, 0, st>>>((const long long*)q_ids, nq, n, slot_id, key_ds, key_hil, val_ds,
                                                 val_hil, S->hil_pos);
    bool in_tmp = false;
    int kb_ds = 0, kb_hil = 0;
    for (long long t = n; t > 0; t >>= 1) ++kb_ds;
    kb_hil = kb_ds;
    e = ct::radix_sort_pairs(key_ds, val_ds, ktmp, vtmp, nq, kb_ds, hist, nullptr, 0, st, &in_tmp);
    if (e == cudaSuccess && in_tmp) { e = cudaMemcpyAsync(val_ds, vtmp, sizeof(int) * nq, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(key_ds, ktmp, 8 * nq, cudaMemcpyDeviceToDevice, st); }
    if (e == cudaSuccess) e = ct::radix_sort_pairs(key_hil, val_hil, ktmp, vtmp, nq, kb_hil, hist, nullptr, 0, st, &in_tmp);
    if (e == cudaSuccess && in_tmp) { e = cudaMemcpyAsync(val_hil, vtmp, sizeof(int) * nq, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(key_hil, ktmp, 8 * nq, cudaMemcpyDeviceToDevice, st); }
    if (e == cudaSuccess) {
        arows_kernel<<<grid_for(rows_q), 256, 0, st>>>(val_ds, nq, rows_q, slot_id, a_slot_ds, rowmap_ds);
        arows_kernel<<<grid_for(rows_q), 256, 0, st>>>(val_hil, nq, rows_q, slot_id, a_slot_hil, rowmap_hil);
        e = cudaGetLastError();
    }
    // sorted keys to host to lay out the job lists
    std::vector<unsigned long long> hk_ds(nq), hk_hil(nq);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hk_ds.data(), key_ds, 8 * nq, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hk_hil.data(), key_hil, 8 * nq, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "screened form setup: %s", cudaGetErrorString(e));

    // ---- A operands: reuse the dataset blocks when the query set is 0..n-1
    bool all_ds = nq == n, all_hil = nq == n;
    for (long long i = 0; i < nq && all_ds; ++i) all_ds = hk_ds[i] == (unsigned long long)i;
    for (long long i = 0; i < nq && all_hil; ++i) all_hil = hk_hil[i] == (unsigned long long)i;
    const bf16 *Aq_hi = S->ds_hi, *Aq_lo = S->ds_lo, *Ah_hi = S->hil_hi, *Ah_lo = S->hil_lo;
    long long gq = S->rows_pad / 8, gh = S->rows_pad / 8;
    if (!all_ds) {
        A((void**)&aq_hi, sizeof(bf16) * rows_q * m); A((void**)&aq_lo, sizeof(bf16) * rows_q * m);
        if (e == cudaSuccess) split_blocked_kernel<<<152 * 8, 256, 0, st>>>(vnat, m, rowmap_ds, rows_q, aq_hi, aq_lo);
        Aq_hi = aq_hi; Aq_lo = aq_lo; gq = rows_q / 8;
    }
    if (!all_hil) {
        A((void**)&ah_hi, sizeof(bf16) * rows_q * m); A((void**)&ah_lo, sizeof(bf16) * rows_q * m);
        if (e == cudaSuccess) split_blocked_kernel<<<152 * 8, 256, 0, st>>>(vnat, m, rowmap_hil, rows_q, ah_hi, ah_lo);
        Ah_hi = ah_hi; Ah_lo = ah_lo; gh = rows_q / 8;
    }
    // ---- job lists
    std::vector<Job> ja, jbv;
    const int wt = nct < WINDOW_TILES ? (int)nct : WINDOW_TILES;
    for (long long t = 0; t < nqt; ++t) {
        long long r = t * TQ + TQ / 2;
        if (r >= nq) r = nq - 1;
        long long pos = (long long)hk_hil[r];
        if (pos >= n) pos = n - 1;
        long long c0 = pos / TC - (wt - 1) / 2;
        if (c0 < 0) c0 = 0;
        if (c0 + wt > nct) c0 = nct - wt;
        for (int w = 0; w < wt; ++w) ja.push_back(Job{(int)t, (int)(c0 + w), w, 0});
    }
    for (long long t = 0; t < nqt; ++t) {
        long long last = (t + 1) * TQ - 1;
        if (last >= nq) last = nq - 1;
        long long maxid = (long long)hk_ds[last];
        if (maxid >= n) {  // invalid ids sort last; use the last valid one
            long long r = last;
            while (r >= t * TQ && (long long)hk_ds[r] >= n) --r;
            maxid = r >= t * TQ ? (long long)hk_ds[r] : -1;
        }
        if (maxid < 0) continue;
        long long cend = predecessor ? (maxid + TC - 1) / TC : nct;  // candidates < maxid
        if (cend > nct) cend = nct;
        for (long long c = 0; c < cend; ++c) jbv.push_back(Job{(int)t, (int)c, 0, 0});
    }
    A((void**)&jobs_a, sizeof(Job) * (ja.size() + 1));
    A((void**)&jobs_b, sizeof(Job) * (jbv.size() + 1));
    if (e == cudaSuccess && !ja.empty()) e = cudaMemcpyAsync(jobs_a, ja.data(), sizeof(Job) * ja.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !jbv.empty()) e = cudaMemcpyAsync(jobs_b, jbv.data(), sizeof(Job) * jbv.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(surv_cnt, 0, sizeof(int) * nq, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(nfull_d, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(evals_d, 0, sizeof(long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(int), st);
    const int wwidth = WINDOW_TILES * TC;
    if (e == cudaSuccess) e = cudaMemsetAsync(win, 0x40, sizeof(float) * nq * wwidth, st);  // 0x40404040 ~ 3.0f: invalid
    // ---- Pass A
    MMAParams P{};
    P.b_hi = S->hil_hi; P.b_lo = S->hil_lo; P.b_groups = S->rows_pad / 8;
    P.a_hi = Ah_hi; P.a_lo = Ah_lo; P.a_groups = gh;
    P.m = m; P.jobs = jobs_a; P.njobs = (int)ja.size();
    P.a_slot = a_slot_hil; P.slot_id = slot_id; P.b_id = S->b_id_hil;
    P.xs = xs; P.d = d; P.vn = S->vn; P.isp = S->isp; P.xmax = S->xmax;
    P.var = var; P.kernel_type = kernel_type; P.predecessor = predecessor ? 1 : 0;
    P.err_coef = err_coef_for(m); P.mode = MODE_WINDOW; P.out_f = win; P.out_stride = wwidth;
    P.tau2 = tau2; P.surv = surv; P.surv_cnt = surv_cnt; P.status = S->status;
    if (e == cudaSuccess) e = launch_mma(P, st);
    if (e == cudaSuccess) {
        const int wpb = 4;
        window_tau_kernel<<<(unsigned)((rows_q + wpb - 1) / wpb), 32 * wpb, sizeof(unsigned long long) * RBUF * wpb, st>>>(
            win, wwidth, a_slot_hil, rows_q, k, tau2);
        e = cudaGetLastError();
    }
    // ---- Pass B
    P.b_hi = S->ds_hi; P.b_lo = S->ds_lo; P.b_groups = S->rows_pad / 8;
    P.a_hi = Aq_hi; P.a_lo = Aq_lo; P.a_groups = gq;
    P.jobs = jobs_b; P.njobs = (int)jbv.size(); P.a_slot = a_slot_ds; P.b_id = S->b_id_ds;
    P.mode = MODE_FILTER;
    if (e == cudaSuccess) e = launch_mma(P, st);
    // ---- rescoring
    RescoreParams R{};
    R.v = vnat; R.m = m; R.coords = coords_raw; R.d = d; R.inv_ls = S->inv_ls64; R.p = p;
    R.var = (double)var; R.kernel_type = kernel_type; R.predecessor = predecessor ? 1 : 0; R.n = n;
    R.slot_id = slot_id; R.nslots = nq; R.surv = surv; R.surv_cnt = surv_cnt; R.full_slots = full_list; R.nfull = 0;
    R.k = k; R.out_idx = (long long*)out_idx; R.out_dist = out_dist; R.evals = evals_d;
    const int rwpb = 8;
    const size_t rsmem = sizeof(unsigned long long) * RBUF * rwpb;
    if (e == cudaSuccess) e = cudaFuncSetAttribute(rescore_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem);
    if (e == cudaSuccess) {
        rescore_kernel<<<(unsigned)((nq + rwpb - 1) / rwpb), 32 * rwpb, rsmem, st>>>(R, 0);
        collect_overflow_kernel<<<grid_for(nq), 256, 0, st>>>(surv_cnt, nq, full_list, nfull_d);
        e = cudaGetLastError();
    }
    int nfull = 0, status = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nfull, nfull_d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, S->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && nfull > 0) {
        R.nfull = nfull;
        rescore_kernel<<<(unsigned)((nfull + rwpb - 1) / rwpb), 32 * rwpb, rsmem, st>>>(R, 1);
        e = cudaGetLastError();
    }
    long long evals = 0;
    if (e == cudaSuccess && stats) {
        e = cudaMemcpyAsync(&evals, evals_d, sizeof(long long), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFreeAsync(slot_id, st); cudaFreeAsync(val_ds, st); cudaFreeAsync(val_hil, st); cudaFreeAsync(vtmp, st);
    cudaFreeAsync(key_ds, st); cudaFreeAsync(key_hil, st); cudaFreeAsync(ktmp, st); cudaFreeAsync(hist, st);
    cudaFreeAsync(a_slot_ds, st); cudaFreeAsync(a_slot_hil, st); cudaFreeAsync(rowmap_ds, st); cudaFreeAsync(rowmap_hil, st);
    if (aq_hi) { cudaFreeAsync(aq_hi, st); cudaFreeAsync(aq_lo, st); }
    if (ah_hi) { cudaFreeAsync(ah_hi, st); cudaFreeAsync(ah_lo, st); }
    cudaFreeAsync(win, st); cudaFreeAsync(tau2, st); cudaFreeAsync(surv, st); cudaFreeAsync(surv_cnt, st);
    cudaFreeAsync(full_list, st); cudaFreeAsync(nfull_d, st); cudaFreeAsync(evals_d, st);
    cudaFreeAsync(jobs_a, st); cudaFreeAsync(jobs_b, st);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "screened form: %s", cudaGetErrorString(e));
    if (status != 0) return set_err(CT_ERR_TIMEOUT, "screened form: pipeline wait timed out (code %d)", status);
    if (stats) {
        stats->pairs_screened = (long long)(ja.size() + jbv.size()) * TQ * TC;
        stats->pairs_rescored = evals;
        stats->distance_evals = evals;
        stats->kernel_launches = 6 + (nfull > 0 ? 1 : 0);
    }
    return CT_OK;
}

// Diagnostic: raw screened dot products of 128 query rows x 256 candidate rows.
int ct_screen_debug_dots(ct_tree* T, const int* rows_a, const int* rows_b, float* out, cudaStream_t st) {
    if (T->m % KC != 0 || T->m > 1024) return T->set_err(CT_ERR_UNSUPPORTED, "%s", "m must be a multiple of 32, <= 1024");
    cudaError_t e = cudaSuccess;
    bf16 *ahi = nullptr, *alo = nullptr, *bhi = nullptr, *blo = nullptr;
    Job* job = nullptr;
    int* status = nullptr;
    const int m = T->m;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMallocAsync(p, bytes, st); };
    A((void**)&ahi, sizeof(bf16) * TQ * m); A((void**)&alo, sizeof(bf16) * TQ * m);
    A((void**)&bhi, sizeof(bf16) * TC * m); A((void**)&blo, sizeof(bf16) * TC * m);
    A((void**)&job, sizeof(Job)); A((void**)&status, sizeof(int));
    if (e != cudaSuccess) return T->set_err(CT_ERR_NOMEM, "debug dots allocation: %s", cudaGetErrorString(e));
    split_blocked_kernel<<<64, 256, 0, st>>>(T->vnat, m, rows_a, TQ, ahi, alo);
    split_blocked_kernel<<<64, 256, 0, st>>>(T->vnat, m, rows_b, TC, bhi, blo);
    Job hj{0, 0, 0, 0};
    int zero = 0;
    e = cudaMemcpyAsync(job, &hj, sizeof(Job), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(status, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
    MMAParams P{};
    P.a_hi = ahi; P.a_lo = alo; P.a_groups = TQ / 8; P.b_hi = bhi; P.b_lo = blo; P.b_groups = TC / 8;
    P.m = m; P.jobs = job; P.njobs = 1; P.mode = MODE_DEBUG; P.out_f = out; P.status = status;
    if (e == cudaSuccess) e = launch_mma(P, st);
    int hs = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(ahi, st); cudaFreeAsync(alo, st); cudaFreeAsync(bhi, st); cudaFreeAsync(blo, st);
    cudaFreeAsync(job, st); cudaFreeAsync(status, st);
    if (e != cudaSuccess) return T->set_err(CT_ERR_CUDA, "debug dots: %s", cudaGetErrorString(e));
    if (hs != 0) return T->set_err(CT_ERR_TIMEOUT, "debug dots: pipeline wait timed out (code %d)", hs);
    return CT_OK;
}
