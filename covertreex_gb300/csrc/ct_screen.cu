// ct_screen.cu — precision form: BF16 tcgen05 screening with certified bounds,
// then FP64-grade rescoring of the survivors.
//
// Pipeline of one ct_knn_residual(form = CT_FORM_SCREENED) call:
//   1. Operands.  V is split as v = hi + lo (hi = bf16(v), lo = bf16(v - hi)) and
//      stored in the UMMA "blocked" layout: for each K-chunk of 32 columns and
//      each group of 8 rows, one 512-byte block of four 8x8 core matrices.  A
//      K-chunk of a 128- or 256-row tile is one contiguous span that a single
//      1-D bulk copy (TMA) moves into shared memory.
//   2. Sweep.  A CTA owns a tile of 128 queries (sorted by Hilbert position
//      inside their "level": the dataset prefix [0, 2^j) with 2^j <= q in
//      predecessor mode, the whole dataset otherwise) and sweeps its candidate
//      tiles: a warm-up over the level's Hilbert tiles nearest-first (a spiral
//      around the queries), then the level's tiles (ascending in one-part calls,
//      the spiral in split calls) and (predecessor mode) the dataset tiles
//      [2^j, max q).  For every
//      query x candidate pair, s = hi.hi + hi.lo + lo.hi is accumulated in TMEM
//      by tcgen05.mma (kind::f16, M=128, N=256, K=16) and the epilogue turns it
//      into certified bounds [dl2, du2] of the squared residual distance.  Each
//      epilogue thread keeps the k smallest du2 of its row half in a heap; the
//      k-th is an upper bound tau^2 of the true k-th distance, and every
//      candidate with dl2 <= tau^2 (tau as it stands when the pair is seen) is
//      kept.  The nearest-first warm-up makes tau tight before any pair is kept.
//   3. Rescore.  Each survivor's distance is recomputed from the f32 inputs with
//      a compensated FP32 dot product (TwoProd/TwoSum) and an FP64 kernel value
//      and normalisation; the k best (distance, index) pairs are written out.
//      Queries whose survivor list overflowed are rescored exhaustively.
//
// Error bound of the screened dot (per pair), with u = 2^-8 (bf16) and
// v = hi + lo + r, |r| <= u^2 |v|:  |s - v_q.v_c| <= c_split ||v_q|| ||v_c|| with
// c_split = 3.1 u^2 + (3 m / 16 + 17) 2^-22, the second term covering FP32
// accumulation inside the tensor core (one rounding per MMA step plus the
// step's internal alignment), both relative to sum |v_qi v_ci| <= ||v_q|| ||v_c||.
#include <cuda_bf16.h>
#include <limits.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <tuple>
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
constexpr int STAGES = 3;  // maximum; the launch picks 3 or 2 to fit the heaps
constexpr int CHUNK_A = TQ * KC * 2;  // bytes
constexpr int CHUNK_B = TC * KC * 2;
constexpr int STAGE_BYTES = 2 * CHUNK_A + 2 * CHUNK_B;
constexpr int kEpiWarps = 8;
constexpr int kEpiThreads = 32 * kEpiWarps;
constexpr int kThreads = 96 + kEpiThreads;  // producer, MMA issuer, staging, epilogue
constexpr int kMaxD = 8;
constexpr int kMaxK = 64;                   // heap capacity per epilogue thread
constexpr int REC = 12;                     // floats per staged candidate record
// After a tile's candidate records: two half-tile boxes (lo[8], hi[8] of the scaled
// coordinates of candidates 0-127 and 128-255), then per group of 8 consecutive
// candidates its largest err_coef |v| and 1/sqrt(p).
constexpr int HBOX = 16;                    // floats per half-tile box
constexpr int GREC = 2;                     // floats per group of 8 candidates
constexpr int RT = TC * REC + 2 * HBOX + (TC / 8) * GREC;  // floats of one candidate tile's records
constexpr int kSurvCap = 1024;  // survivors per query slot (two column halves), at most RBUF
constexpr int RBUF = 1024;                  // rescoring sort buffer (power of two)
// Overflowed query slots with |v_q| / sqrt(p_q) up to this go to the filtered exhaustive
// pass (certified FP32 bounds first); above it the bounds exclude almost nothing.
constexpr float kFilterIsq = 256.f;
static_assert(kSurvCap <= RBUF, "a slot's survivors must fit the rescoring buffer");

enum Mode { MODE_DEBUG = 0, MODE_SWEEP = 1 };

// element offset of (row, col) in a blocked matrix with G = rows_pad / 8 row groups
__host__ __device__ inline size_t blocked_offset(long long row, int col, long long G) {
    int c = col >> 5, j = (col >> 3) & 3, e = col & 7;
    long long g = row >> 3;
    int rr = (int)(row & 7);
    return ((size_t)c * (size_t)G + (size_t)g) * 256 + (size_t)j * 64 + (size_t)rr * 8 + e;
}

// One job = one candidate tile for the CTA's current query tile.
struct Job {
    int qtile;  // query tile (rows qtile*128 .. of the A operand)
    int ctile;  // candidate tile in the B matrix selected by `which`
    int which;  // bit 0: 0 = level matrix (Hilbert order), 1 = dataset matrix;
                // bit 1: warm-up job (bounds feed the thresholds, nothing is kept);
                // bit 2: kept job whose tile already fed the thresholds in warm-up
    int first;  // 1 on the first job of a query tile
};

struct MMAParams {
    const bf16* a_hi; const bf16* a_lo; long long a_groups;
    const bf16* b_hi[2]; const bf16* b_lo[2]; long long b_groups[2];
    const int* b_id[2];  // B row -> dataset id (or -1)
    int m;
    const Job* jobs;
    const int* cta_job_begin;  // static schedule: per CTA [begin, end) into jobs (unit_jobs == nullptr)
    // dynamic schedule: units (query tile, part) as (first job, job count), largest first;
    // a CTA claims the next unit from unit_counter whenever it needs one
    const int2* unit_jobs;
    int nunits;
    int* unit_counter;
    const int* a_slot;   // A row -> query slot (or -1)
    const int* slot_id;  // query slot -> dataset id
    const float* xs; int d;
    const float* vn; const float* isp; const float* xmax;
    float var; int kernel_type; int predecessor;
    float err_coef;
    int k;
    int nstages;
    float* out_f;        // debug output
    int* surv; int* surv_cnt;
    float* survb;        // per survivor: the upper bound of |rho| / sqrt(p_q) that kept it
    int half_cap;        // survivor segment per (slot, column half)
    const float* rec[2]; // candidate records in tile order (levels, dataset), RT floats per tile
    const unsigned* xmax_max;  // bits of max |x_c| over the dataset rows
    int* status;
    unsigned* qtau;      // per query (slot / parts): the smallest part threshold, float bits
    int parts;           // candidate parts per query (slots s*parts .. s*parts+parts-1)
};

constexpr int kRing = 4;  // claimed units in flight per CTA (dynamic schedule)
struct SmemLayout {
    size_t stages, rec, heap, rowtau, bars, tmem_slot, ring, total;
};
__host__ __device__ inline SmemLayout smem_layout(int k, int nstages) {
    SmemLayout L;
    size_t off = 0;
    L.stages = off; off += (size_t)nstages * STAGE_BYTES;
    L.rec = off; off += (size_t)2 * RT * sizeof(float);
    L.heap = off; off += (size_t)kEpiThreads * (k > 0 ? k : 1) * sizeof(float);
    L.rowtau = off; off += (size_t)TQ * sizeof(unsigned long long);
    L.bars = off; off += (size_t)(2 * STAGES + 4 + 4 + 1 + 2 * kRing) * 8;
    L.tmem_slot = off; off += 16;
    L.ring = off; off += 16;
    L.total = off + 1024;  // alignment slack
    return L;
}

// Four-ary max-heap of floats stored strided (element i of thread t at h[i * kEpiThreads];
// children of i at 4i+1 .. 4i+4).  Three levels hold up to 85 elements, and the four child
// loads of a level are independent, so a sift costs about one shared-memory latency a level.
__device__ __forceinline__ void heap_sift_down(float* h, int n, float x) {
    int i = 0;
    for (;;) {
        const int c0 = 4 * i + 1;
        if (c0 >= n) break;
        const float ninf = __int_as_float(0xff800000);
        const float a0 = h[c0 * kEpiThreads];
        const float a1 = c0 + 1 < n ? h[(c0 + 1) * kEpiThreads] : ninf;
        const float a2 = c0 + 2 < n ? h[(c0 + 2) * kEpiThreads] : ninf;
        const float a3 = c0 + 3 < n ? h[(c0 + 3) * kEpiThreads] : ninf;
        const bool s01 = a1 > a0, s23 = a3 > a2;
        const float m01 = s01 ? a1 : a0, m23 = s23 ? a3 : a2;
        const int i01 = s01 ? c0 + 1 : c0, i23 = s23 ? c0 + 3 : c0 + 2;
        const bool hi = m23 > m01;
        const float mc = hi ? m23 : m01;
        const int c = hi ? i23 : i01;
        if (mc <= x) break;
        h[i * kEpiThreads] = mc;
        i = c;
    }
    h[i * kEpiThreads] = x;
}
__device__ __forceinline__ void heap_push(float* h, int n, float x) {
    int i = n;
    while (i > 0) {
        const int pnt = (i - 1) >> 2;
        const float pv = h[pnt * kEpiThreads];
        if (pv >= x) break;
        h[i * kEpiThreads] = pv;
        i = pnt;
    }
    h[i * kEpiThreads] = x;
}

// bit 2 of `which`: a kept job whose candidate tile already fed the heap during warm-up
__device__ __forceinline__ bool jb_warm_seen(const Job& jb) { return (jb.which & 4) != 0; }

// Squared scaled distance and kernel value of one query with two staged candidates
// (columns .x and .y of the record pair r4).  Matern also returns a = sqrt(5 d2) and e^-a
// for the error term.
template <int DP, int KT>
__device__ __forceinline__ void pair_kv2(const float4* r4, const float (&nxq)[kMaxD], float var, float2& d2,
                                         float2& kv, float2& a, float2& ea) {
    d2 = make_float2(0.f, 0.f);
    float2 t;
#pragma unroll
    for (int h = 0; h < DP / 2; ++h) {
        const float4 x = r4[h];
        t = __fadd2_rn(make_float2(x.x, x.y), make_float2(nxq[2 * h], nxq[2 * h]));
        d2 = __ffma2_rn(t, t, d2);
        t = __fadd2_rn(make_float2(x.z, x.w), make_float2(nxq[2 * h + 1], nxq[2 * h + 1]));
        d2 = __ffma2_rn(t, t, d2);
    }
    if (KT == 0) {
        const float2 h = __fmul2_rn(make_float2(-0.5f, -0.5f), d2);
        kv = __fmul2_rn(make_float2(var, var), make_float2(__expf(h.x), __expf(h.y)));
        a = ea = make_float2(0.f, 0.f);
    } else {
        a = __fmul2_rn(make_float2(2.2360679775f, 2.2360679775f), make_float2(sqrtf(d2.x), sqrtf(d2.y)));
        ea = make_float2(__expf(-a.x), __expf(-a.y));
        // var (1 + a + a^2 / 3) e^-a, each step rounded
        const float2 a2 = __fmul2_rn(__fmul2_rn(a, a), make_float2(0.33333334f, 0.33333334f));
        const float2 poly = __fadd2_rn(__fadd2_rn(make_float2(1.f, 1.f), a), a2);
        kv = __fmul2_rn(__fmul2_rn(make_float2(var, var), poly), ea);
    }
}

// DP: coordinates read per candidate (4 when D <= 4, else 8).  KT: kernel type (0 RBF,
// 1 Matern 5/2) as a template parameter, so each group of 8 pairs is one basic block.
template <int MODE, int DP, int KT>
__global__ void __launch_bounds__(kThreads, 1) screen_sweep_kernel(MMAParams P) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const SmemLayout L = smem_layout(P.k, P.nstages);
    const int NS = P.nstages;
    unsigned char* stage_base = smem + L.stages;
    float* recs = (float*)(smem + L.rec);
    float* heaps = (float*)(smem + L.heap);
    unsigned long long* rowtau = (unsigned long long*)(smem + L.rowtau);
    uint64_t* full = (uint64_t*)(smem + L.bars);
    uint64_t* empty = full + STAGES;  // barrier slots sized for the maximum stage count
    uint64_t* accf = empty + STAGES;
    uint64_t* acce = accf + 2;
    uint64_t* recf = acce + 2;
    uint64_t* rece = recf + 2;
    uint64_t* done = rece + 2;
    uint64_t* rfull = done + 1;        // unit ring: slot written by the producer
    uint64_t* rempty = rfull + kRing;  // slot released by every consumer
    uint32_t* tmem_slot = (uint32_t*)(smem + L.tmem_slot);
    int* ring = (int*)(smem + L.ring);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nchunks = P.m / KC;
    const uint32_t idesc = sm::idesc_bf16_f32(TQ, TC);
    const int jb0 = P.unit_jobs ? 0 : P.cta_job_begin[blockIdx.x];
    const int jb1 = P.unit_jobs ? 0 : P.cta_job_begin[blockIdx.x + 1];

    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) { sm::mbar_init(&full[s], 1); sm::mbar_init(&empty[s], 1); }
        for (int a = 0; a < 2; ++a) {
            sm::mbar_init(&accf[a], 1); sm::mbar_init(&acce[a], kEpiWarps);
            sm::mbar_init(&recf[a], 1); sm::mbar_init(&rece[a], kEpiWarps);
        }
        sm::mbar_init(done, 1);
        for (int r = 0; r < kRing; ++r) {
            sm::mbar_init(&rfull[r], 1);
            sm::mbar_init(&rempty[r], MODE == MODE_SWEEP ? 2 + kEpiWarps : 1 + kEpiWarps);
        }
        sm::fence_barrier_init();
    }
    for (int r = threadIdx.x; r < TQ; r += blockDim.x) rowtau[r] = 0ULL;
    if (warp == 1) {
        sm::tmem_alloc(tmem_slot, 512);
        sm::tmem_relinquish();
    }
    sm::tc_fence_before();
    __syncthreads();
    sm::tc_fence_after();
    const uint32_t tmem_base = *tmem_slot;

    // The job range of the CTA's ui-th unit.  Static schedule: one range, [jb0, jb1).
    // Dynamic schedule: the producer claims units into a ring of kRing slots; every other
    // role takes them from the ring in the same order and releases the slot when done.
    // A claimed index past the last unit ends every role.
    auto take_unit = [&](int ui, int& j0, int& j1) -> bool {
        if (!P.unit_jobs) {
            j0 = jb0; j1 = jb1;
            return ui == 0;
        }
        const int sl = ui % kRing;
        if (!sm::mbar_wait(&rfull[sl], (unsigned)((ui / kRing) & 1), P.status, 19)) return false;
        const int u = *(volatile int*)&ring[sl];
        if (u < 0) return false;
        const int2 r = P.unit_jobs[u];
        j0 = r.x; j1 = r.x + r.y;
        return true;
    };
    auto release_unit = [&](int ui) {
        if (P.unit_jobs) sm::mbar_arrive(&rempty[ui % kRing]);
    };

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        if (lane == 0) {
            long long it = 0;
            for (int ui = 0;; ++ui) {
            int j0u, j1u;
            if (P.unit_jobs) {
                const int sl = ui % kRing;
                if (!sm::mbar_wait(&rempty[sl], (unsigned)(((ui / kRing) & 1) ^ 1), P.status, 18)) break;
                const int u = atomicAdd(P.unit_counter, 1);
                ring[sl] = u < P.nunits ? u : -1;
                sm::mbar_arrive(&rfull[sl]);
                if (u >= P.nunits) break;
                const int2 r = P.unit_jobs[u];
                j0u = r.x; j1u = r.x + r.y;
            } else {
                if (ui > 0) break;
                j0u = jb0; j1u = jb1;
            }
            for (int j = j0u; j < j1u; ++j) {
                const Job jb = P.jobs[j];
                const bf16* bh = P.b_hi[jb.which & 1];
                const bf16* bl = P.b_lo[jb.which & 1];
                const long long bg = P.b_groups[jb.which & 1];
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int s = (int)(it % NS);
                    const unsigned ph = (unsigned)((it / NS) & 1);
                    if (!sm::mbar_wait(&empty[s], ph ^ 1u, P.status, 11)) goto producer_done;
                    unsigned char* dst = stage_base + (size_t)s * STAGE_BYTES;
                    sm::mbar_arrive_expect_tx(&full[s], STAGE_BYTES);
                    const size_t aoff = blocked_offset((long long)jb.qtile * TQ, c * KC, P.a_groups);
                    const size_t boff = blocked_offset((long long)jb.ctile * TC, c * KC, bg);
                    sm::bulk_g2s(dst, P.a_hi + aoff, CHUNK_A, &full[s]);
                    sm::bulk_g2s(dst + CHUNK_A, P.a_lo + aoff, CHUNK_A, &full[s]);
                    sm::bulk_g2s(dst + 2 * CHUNK_A, bh + boff, CHUNK_B, &full[s]);
                    sm::bulk_g2s(dst + 2 * CHUNK_A + CHUNK_B, bl + boff, CHUNK_B, &full[s]);
                }
            }
            }
        producer_done:;
        }
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            long long it = 0;
            int lt = 0;
            bool alive = true;
            for (int ui = 0; alive; ++ui) {
            int j0u, j1u;
            if (!take_unit(ui, j0u, j1u)) break;
            for (int j = j0u; j < j1u; ++j, ++lt) {
                const int acc = lt & 1;
                const unsigned aph = (unsigned)((lt >> 1) & 1);
                if (!sm::mbar_wait(&acce[acc], aph ^ 1u, P.status, 12)) { alive = false; break; }
                sm::tc_fence_after();
                const uint32_t dt = tmem_base + (uint32_t)(acc * TC);
                bool ok = true;
                for (int c = 0; c < nchunks; ++c, ++it) {
                    const int s = (int)(it % NS);
                    const unsigned ph = (unsigned)((it / NS) & 1);
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
                if (!ok) { alive = false; break; }
                sm::mma_commit(&accf[acc]);
            }
            release_unit(ui);
            }
            sm::mma_commit(done);
            sm::mbar_wait(done, 0, P.status, 14);
        }
    } else if (warp == 2) {
        // ------------------------------------------------------------ candidate records
        // One bulk copy per job brings the candidate tile's records (built once per tree
        // in tile order by build_records_kernel) into the free record buffer.
        if (MODE == MODE_SWEEP && lane == 0) {
            int lt = 0;
            bool alive = true;
            for (int ui = 0; alive; ++ui) {
                int j0u, j1u;
                if (!take_unit(ui, j0u, j1u)) break;
                for (int j = j0u; j < j1u; ++j, ++lt) {
                    const Job jb = P.jobs[j];
                    const int acc = lt & 1;
                    const unsigned aph = (unsigned)((lt >> 1) & 1);
                    if (!sm::mbar_wait(&rece[acc], aph ^ 1u, P.status, 16)) { alive = false; break; }
                    sm::mbar_arrive_expect_tx(&recf[acc], (unsigned)(RT * sizeof(float)));
                    sm::bulk_g2s(recs + (size_t)acc * RT, P.rec[jb.which & 1] + (size_t)jb.ctile * RT,
                                 (unsigned)(RT * sizeof(float)), &recf[acc]);
                }
                release_unit(ui);
            }
        }
    } else {
        // ------------------------------------------------------------ epilogue
        // Thread (row, half) owns the pairs of one query row with the 128 candidate
        // columns of its half: its own heap, threshold and survivor segment, so no
        // state is shared between warps.
        const int ew = warp - 3;
        const int quarter = warp & 3;        // TMEM lanes 32*quarter ..
        const int half = ew >> 2;            // columns half*128 ..
        const int row = quarter * 32 + lane;
        const int et = ew * 32 + lane;       // 0 .. kEpiThreads-1
        float* heap = heaps + et;
        int lt = 0;
        int slot = -1, qid = -1, hn = 0, cnt = 0;
        // A (row, half) whose survivor list overflowed is rescored exhaustively: it stops
        // keeping and heaping (thresholds +inf), so that a tiny-p row, whose wide bounds
        // pass nearly every pair, does not hold its warp in phase 2 for the rest of the sweep.
        bool ovf = false;
        unsigned gen = 0;  // query-tile generation, tags the shared row threshold
        float tau2 = 1.f;
        float nxq[kMaxD];  // negated query coordinates: x_c + (-x_q) is the rounded x_c - x_q
        float vnq = 0.f, isq = 0.f;
        int lim = 0;       // a candidate id is valid iff (unsigned)cid < (unsigned)lim
        // Kernel-value error bound of the query, linear in d2 (see phase 1): for RBF the
        // relative factor fk = alk d2 + bek, for Matern the d2 error ed2 = ale d2 + bee.
        float alk = 0.f, bek = 0.f, ale = 0.f, bee = 0.f;
        // Largest kernel-value error term ek of any pair of the query (the maxima over d2
        // of the expressions below: x e^-x/2 <= 2/e for RBF; for Matern 5/2 with
        // a = sqrt(5 d2): a (1 + a + a^2/3) e^-a <= 1.176, a^2 (1 + a) e^-a <= 1.814,
        // (1 + a) e^-a <= 1), used by the group test.
        float ekmax = 0.f;
        // keep the pair iff (R + e) * isc >= thr_keep; it may enter the heap iff
        // (R - e) * isc > thr_heap, i.e. its d^2 upper bound is below tau2 (both derived
        // from tau2: a pair at or above the row's threshold cannot lower it, since the
        // half's k-th bound could only fall to tau2)
        float thr_keep = 0.f, thr_heap = 0.f;
#pragma unroll
        for (int c = 0; c < kMaxD; ++c) nxq[c] = 0.f;
        const float dd = (float)P.d;
        const float ced2 = (dd + 2.f) * 5.97e-8f;
        bool alive = true;
        for (int ui = 0; alive; ++ui) {
        int j0u, j1u;
        if (!take_unit(ui, j0u, j1u)) break;
        for (int j = j0u; j < j1u; ++j, ++lt) {
            const Job jb = P.jobs[j];
            const int acc = lt & 1;
            const unsigned aph = (unsigned)((lt >> 1) & 1);
            if (MODE == MODE_SWEEP && jb.first) {
                if (slot >= 0) {
                    P.surv_cnt[2 * slot + half] = cnt;
                    // the final threshold, for the survivor pass (parts > 1 share it during the sweep)
                    if (P.parts == 1 && qid >= 0) atomicMin(&P.qtau[slot], __float_as_uint(tau2));
                }
                const long long arow = (long long)jb.qtile * TQ + row;
                slot = P.a_slot[arow];
                qid = slot >= 0 ? P.slot_id[slot] : -1;
                hn = 0; cnt = 0; tau2 = 1.f; ++gen; ovf = false;
                if (qid >= 0) {
                    vnq = P.vn[qid]; isq = P.isp[qid];
#pragma unroll
                    for (int c = 0; c < kMaxD; ++c) nxq[c] = c < P.d ? -P.xs[(size_t)qid * P.d + c] : 0.f;
                    // predecessor mode: 0 <= cid < qid; otherwise cid >= 0 (ids stay below INT_MAX)
                    lim = P.predecessor ? qid : 0x7fffffff;
                    // Error of d2 from the scaled coordinates: (D+2) 2^-24 d2 from the sum plus
                    // 2^-22 sum|dx| (|x_q| + |x_c|), sum|dx| <= sqrt(D d2) <= (D d2 + 1) / 2, with
                    // |x_c| bounded by the dataset's largest: ed2 <= ale d2 + bee.  The RBF value's
                    // relative error 6e-8 d2 + ed2 / 2 + 1e-6 <= alk d2 + bek.  The constants are
                    // rounded up by 1e-5 relative, far above their own rounding.
                    const float A = 2.4e-7f * (P.xmax[qid] + __uint_as_float(__ldg(P.xmax_max)));
                    ale = (ced2 + 0.5f * A * dd) * 1.00001f;
                    bee = 0.5f * A * 1.00001f;
                    alk = (6e-8f + 0.5f * ced2 + 0.25f * A * dd) * 1.00001f;
                    bek = (1e-6f + 0.25f * A) * 1.00001f;
                    ekmax = KT == 0 ? P.var * (0.7358f * alk + bek) * 1.01f
                                    : P.var * (1.283e-6f + 0.8334f * (0.3628f * ale + bee) + 1.82e-7f) * 1.01f;
                }
                thr_keep = 0.f;   // tau2 = 1: keep everything
                thr_heap = 0.f;   // and heap every pair whose |rho| bound is positive
            }
            if (MODE == MODE_SWEEP && !sm::mbar_wait(&recf[acc], aph, P.status, 17)) { alive = false; break; }
            if (!sm::mbar_wait(&accf[acc], aph, P.status, 15)) { alive = false; break; }
            sm::tc_fence_after();
            const float* rb = recs + (size_t)acc * RT;
            const float* gtab = rb + TC * REC + 2 * HBOX;  // group records of the tile
            // kmax: an upper bound of the kernel value phase 1 computes for this row and any
            // candidate of its half tile.  The half tile's box gives the smallest squared
            // scaled distance dmin; phase 1's f32 distance (rounded differences, FMA chain) is
            // at least dmin (1 - 1e-5), and its __expf / Matern polynomial stay within the
            // relative margins below.
            float kmax = 0.f;
            if (MODE == MODE_SWEEP && qid >= 0) {
                const float* hb = rb + TC * REC + half * HBOX;
                float dmin = 0.f;
#pragma unroll
                for (int c = 0; c < DP; ++c) {
                    const float a = hb[c] + nxq[c];      // lo_c - x_q,c
                    const float b = hb[8 + c] + nxq[c];  // hi_c - x_q,c
                    const float t = fmaxf(fmaxf(a, -b), 0.f);
                    dmin = fmaf(t, t, dmin);
                }
                dmin *= (1.f - 1e-5f);
                if (KT == 0) {
                    kmax = P.var * __expf(-0.5f * dmin) * (1.f + 1e-5f);
                } else {
                    const float a0 = 2.2360679775f * sqrtf(dmin);
                    kmax = P.var * (1.f + a0 + a0 * a0 * 0.33333334f) * __expf(-a0) * (1.f + 2e-5f);
                }
            }
            const bool keep_job = !(jb.which & 2);
            const bool feed_heap = !(jb.which & 4);
            const bool fast_ids = (jb.which & 8) != 0;
            if (MODE == MODE_SWEEP && qid >= 0 && !ovf) {
                // the other half's threshold, when it belongs to this query tile
                const unsigned long long w = *(volatile unsigned long long*)&rowtau[row];
                if ((unsigned)(w >> 32) == gen) {
                    const float t = __uint_as_float(~(unsigned)w);
                    if (t < tau2) {
                        tau2 = t;
                        thr_keep = (1.f - tau2) * (1.f - 2e-6f) / isq;
                        thr_heap = (1.f - tau2) * (1.f + 2e-6f) / isq;
                    }
                }
                // the other parts' thresholds of this query (any part's k-th upper
                // bound bounds the query's k-th distance)
                const float tg = __uint_as_float(__ldcg(&P.qtau[slot / P.parts]));
                if (tg < tau2) {
                    tau2 = tg;
                    thr_keep = (1.f - tau2) * (1.f - 2e-6f) / isq;
                    thr_heap = (1.f - tau2) * (1.f + 2e-6f) / isq;
                }
            }
            for (int cc = 0; cc < 16; ++cc) {
                float v[8];
                const int col0 = half * 128 + cc * 8;
                sm::tmem_ld8(tmem_base + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * TC + col0), v);
                if (MODE == MODE_DEBUG) {
                    float* o = P.out_f + ((size_t)(j - jb0) * TQ + row) * TC + col0;
#pragma unroll
                    for (int i = 0; i < 8; ++i) o[i] = v[i];
                    continue;
                }
                if (qid < 0) continue;
                // Group test: one certified bound for the group's 8 pairs.  kmax bounds the
                // kernel value phase 1 would compute for any candidate of the thread's half tile
                // (from the half tile's coordinate box, once per job), so |kv - s| <=
                // max(kmax - s, s) and phase 1's survivor bound of each pair is at most ghi (with
                // the group's largest error term and 1/sqrt(p)).  ghi < thr_keep (<= thr_heap)
                // means no pair of the group is kept or heaped: the group is done without phase
                // 1.  It skips the per-pair work where the kernel value is negligible (candidates
                // far from the query in coordinates); padding groups (NaN 1/sqrt(p)) always skip.
                {
                    const float* gr = gtab + (size_t)(col0 >> 3) * GREC;
                    float rmax = 0.f;
#pragma unroll
                    for (int i = 0; i < 8; ++i) rmax = fmaxf(rmax, fmaxf(kmax - v[i], v[i]));
                    const float ghi = (rmax * (1.f + 3e-7f) + vnq * gr[0] + ekmax + 1e-30f) * gr[1] * (1.f + 1e-6f);
                    if (!(ghi >= thr_keep)) continue;
                    // Second tier: each pair's kernel value, computed as phase 1 does, gives
                    // phase 1's R = |kv - s| up to the product kv being fused into the add in
                    // one tier and not the other (which moves kv - s by at most 2^-23 kv); with
                    // 2.4e-7 kv added, and the group's largest error term and 1/sqrt(p) as
                    // above, rc bounds phase 1's survivor bound of every pair.  Near
                    // candidates pass the box test (the box cannot see that s tracks kv) but
                    // rarely this one; it costs about half of phase 1.
                    float rc = 0.f;
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float4* r4 = (const float4*)(rb + ((col0 >> 1) + i) * (2 * REC));
                        float2 d2, kv, am, ea;
                        pair_kv2<DP, KT>(r4, nxq, P.var, d2, kv, am, ea);
                        const float2 dif = __fadd2_rn(kv, make_float2(-v[2 * i], -v[2 * i + 1]));
                        const float2 rr = __ffma2_rn(kv, make_float2(2.4e-7f, 2.4e-7f),
                                                     make_float2(fabsf(dif.x), fabsf(dif.y)));
                        rc = fmaxf(rc, fmaxf(rr.x, rr.y));
                    }
                    const float gc = (rc * (1.f + 3e-7f) + vnq * gr[0] + ekmax + 1e-30f) * gr[1] * (1.f + 1e-6f);
                    if (!(gc >= thr_keep)) continue;
                }
                // Phase 1, no stores: certified bounds of the group's 8 pairs, as
                //   blo = (R - e) * isc (heap test)  and  bhi = (R + e) * isc (survivor test),
                // +inf for the query itself, -inf for predecessor-violating pairs and NaN for
                // padding rows (their 1/sqrt(p) is NaN, so every test fails).  Jobs flagged 8
                // hold only candidate ids below every query id of the tile and skip the id
                // tests.  Free of stores, the pairs' loads and arithmetic overlap.
                float blo[8], bhi[8];
                int bid[8];
                auto phase1 = [&](auto check_ids) {
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        // columns col0 + 2i (.x) and col0 + 2i + 1 (.y)
                        const float4* r4 = (const float4*)(rb + ((col0 >> 1) + i) * (2 * REC));
                        const float4 m0 = r4[4];  // err_coef * |v_c|, 1/sqrt(p_c)
                        const float4 m1 = r4[5];  // 2.4e-7 max|x_c| (unused), id
                        const float2 err = make_float2(m0.x, m0.y), isc = make_float2(m0.z, m0.w);
                        float2 d2, kv, ek, am, ea;
                        pair_kv2<DP, KT>(r4, nxq, P.var, d2, kv, am, ea);
                        if (KT == 0) {
                            ek = __fmul2_rn(kv, __ffma2_rn(make_float2(alk, alk), d2, make_float2(bek, bek)));
                        } else {
                            const float2 ed2 = __ffma2_rn(make_float2(ale, ale), d2, make_float2(bee, bee));
                            const float aa = am.x, ab = am.y;
                            ek.x = kv.x * (1e-6f + 2.4e-7f * aa) + P.var * (0.8334f * ed2.x + 1e-7f * aa * aa) * (1.f + aa) * ea.x;
                            ek.y = kv.y * (1e-6f + 2.4e-7f * ab) + P.var * (0.8334f * ed2.y + 1e-7f * ab * ab) * (1.f + ab) * ea.y;
                        }
                        const float2 dif = __fadd2_rn(kv, make_float2(-v[2 * i], -v[2 * i + 1]));
                        const float2 R = make_float2(fabsf(dif.x), fabsf(dif.y));
                        const float2 e = __fadd2_rn(__ffma2_rn(make_float2(vnq, vnq), err, ek),
                                                    __ffma2_rn(R, make_float2(1.2e-7f, 1.2e-7f), make_float2(1e-30f, 1e-30f)));
                        const float2 lo = __fmul2_rn(__fadd2_rn(R, make_float2(-e.x, -e.y)), isc);
                        const float2 hi = __fmul2_rn(__fadd2_rn(R, e), isc);
                        const int ca = __float_as_int(m1.z), cb = __float_as_int(m1.w);
                        if constexpr (decltype(check_ids)::value) {
                            const bool va = (unsigned)ca < (unsigned)lim, vb = (unsigned)cb < (unsigned)lim;
                            const float inf = __int_as_float(0x7f800000);
                            blo[2 * i] = !va ? -inf : (ca == qid ? inf : lo.x);
                            bhi[2 * i] = !va ? -inf : (ca == qid ? inf : hi.x);
                            blo[2 * i + 1] = !vb ? -inf : (cb == qid ? inf : lo.y);
                            bhi[2 * i + 1] = !vb ? -inf : (cb == qid ? inf : hi.y);
                        } else {
                            blo[2 * i] = lo.x; bhi[2 * i] = hi.x;
                            blo[2 * i + 1] = lo.y; bhi[2 * i + 1] = hi.y;
                        }
                        bid[2 * i] = ca;
                        bid[2 * i + 1] = cb;
                    }
                };
                if (fast_ids) phase1(std::false_type{}); else phase1(std::true_type{});
                // Phase 2: survivors and heap against the thresholds as they stand at the
                // group's start.  Most groups have no pair to keep or heap; one test skips
                // them.  (The group's largest bounds decide: fmaxf skips the NaN of padding
                // rows.)  Keeping against the group's starting threshold keeps at least the
                // pairs that a threshold lowered within the group would; every kept pair
                // still satisfies dl2 <= tau^2 for a valid tau.
                float mh = bhi[0], ml = blo[0];
#pragma unroll
                for (int i = 1; i < 8; ++i) { mh = fmaxf(mh, bhi[i]); ml = fmaxf(ml, blo[i]); }
                const bool any = (keep_job & (mh >= thr_keep)) | (feed_heap & (ml > thr_heap));
                if (!any) continue;
                unsigned hmask = 0;  // pairs of the group that may lower the heap's top
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    if (keep_job && bhi[i] >= thr_keep) {
                        if (cnt < P.half_cap) {
                            P.surv[((size_t)slot * 2 + half) * P.half_cap + cnt] = bid[i];
                            P.survb[((size_t)slot * 2 + half) * P.half_cap + cnt] = bhi[i];
                        }
                        ++cnt;
                    }
                    if (feed_heap && blo[i] > thr_heap) hmask |= 1u << i;
                }
                if (cnt > P.half_cap) {
                    // overflowed: the row stops keeping and heaping
                    ovf = true;
                    thr_keep = __int_as_float(0x7f800000);
                    thr_heap = __int_as_float(0x7f800000);
                    hmask = 0;
                }
                // Heap updates one pending pair per iteration: the warp runs as many rounds as
                // its busiest lane has pairs, not one round per pair position that any lane
                // needs.  A pair whose bound no longer beats the top (lowered by an earlier
                // pair of the group) is dropped by the top test.
                while (hmask) {
                    const int pi = __ffs(hmask) - 1;
                    hmask &= hmask - 1u;
                    float b = blo[0];
#pragma unroll
                    for (int i = 1; i < 8; ++i) b = pi == i ? blo[i] : b;
                    {
                        // exact certified upper bound of d^2 for this pair (0 for the query itself)
                        const float du2 = 1.f - fminf(fmaxf(b, 0.f) * isq * (1.f - 1e-6f), 1.f);
                        bool changed = false;
                        if (hn < P.k) {
                            heap_push(heap, hn, du2);
                            ++hn;
                            changed = hn == P.k;
                        } else if (du2 < heap[0]) {
                            heap_sift_down(heap, hn, du2);
                            changed = true;
                        }
                        if (changed) {
                            const float top = heap[0];
                            if (top < tau2) {
                                tau2 = top;
                                thr_keep = (1.f - tau2) * (1.f - 2e-6f) / isq;
                                thr_heap = (1.f - tau2) * (1.f + 2e-6f) / isq;
                                atomicMax(&rowtau[row], ((unsigned long long)gen << 32) |
                                                            (unsigned long long)(~__float_as_uint(tau2)));
                                if (P.parts > 1) atomicMin(&P.qtau[slot / P.parts], __float_as_uint(tau2));
                            }
                        }
                    }
                }
            }
            sm::tc_fence_before();
            __syncwarp();
            if (lane == 0) {
                sm::mbar_arrive(&acce[acc]);
                if (MODE == MODE_SWEEP) sm::mbar_arrive(&rece[acc]);
            }
        }
        __syncwarp();
        if (lane == 0) release_unit(ui);
        }
        if (MODE == MODE_SWEEP && slot >= 0) {
            P.surv_cnt[2 * slot + half] = cnt;
            // the final threshold, for the survivor pass (parts > 1 share it during the sweep)
            if (P.parts == 1 && qid >= 0) atomicMin(&P.qtau[slot], __float_as_uint(tau2));
        }
    }
    sm::tc_fence_before();
    __syncthreads();
    if (warp == 1) sm::tmem_dealloc(tmem_base, 512);
}

// -------------------------------------------------------------- operand prep
// Candidate records of the sweep epilogue, in tile order (row r of a blocked operand
// = row r here), built once per tree.  Rows 2i and 2i+1 of a tile share 2 * REC
// floats with their fields interleaved (field f of row e at (e >> 1) * 2 * REC + 2f +
// (e & 1)) so that the epilogue bounds both pairs with one packed f32x2 instruction
// per step.  Fields: the scaled coordinates (padded to kMaxD), err_coef * |v|,
// 1/sqrt(p) (NaN for padding rows), 2.4e-7 max|x| and the id's bits (-1 for padding rows).
__global__ void build_records_kernel(const int* __restrict__ ids, long long rows, const float* __restrict__ xs, int d,
                                     const float* __restrict__ vn, const float* __restrict__ isp,
                                     const float* __restrict__ xmax, float err_coef, float* __restrict__ rec) {
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const long long tile = r / TC;
    const int e = (int)(r - tile * TC);
    float* o = rec + tile * RT + (e >> 1) * (2 * REC) + (e & 1);
    const int cid = ids[r];
    if (cid >= 0) {
#pragma unroll
        for (int c = 0; c < kMaxD; ++c) o[2 * c] = c < d ? xs[(size_t)cid * d + c] : 0.f;
        o[16] = err_coef * vn[cid];
        o[18] = isp[cid];
        o[20] = 2.4e-7f * xmax[cid];
        o[22] = __int_as_float(cid);
    } else {
#pragma unroll
        for (int c = 0; c < 11; ++c) o[2 * c] = 0.f;
        o[18] = __int_as_float(0x7fc00000);  // NaN 1/sqrt(p): every bound test of the row fails
        o[22] = __int_as_float(-1);
    }
}

// Half-tile boxes and group scalars of the sweep's group test (after a tile's candidate
// records): one thread per half tile writes the box of its 128 candidates' scaled
// coordinates (lo in floats 0-7, hi in 8-15; 0 past d; an empty box +inf / -inf when no
// row is valid) and, for each of its 16 groups of 8, the largest err_coef |v| and the
// largest 1/sqrt(p) (NaN when the group has no valid row).
__global__ void build_group_records_kernel(const int* __restrict__ ids, long long rows, const float* __restrict__ xs,
                                           int d, const float* __restrict__ vn, const float* __restrict__ isp,
                                           float err_coef, float* __restrict__ rec) {
    const long long hi_ = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (hi_ >= rows / (TC / 2)) return;
    const long long tile = hi_ / 2;
    const int h = (int)(hi_ - tile * 2);
    float lo[kMaxD], hi[kMaxD];
#pragma unroll
    for (int c = 0; c < kMaxD; ++c) { lo[c] = __int_as_float(0x7f800000); hi[c] = -__int_as_float(0x7f800000); }
    float* base = rec + tile * RT + TC * REC;
    for (int g = 0; g < TC / 16; ++g) {
        float emax = 0.f, imax = __int_as_float(0x7fc00000);
        bool any = false;
        for (int e = 0; e < 8; ++e) {
            const int cid = ids[tile * TC + h * (TC / 2) + 8 * g + e];
            if (cid < 0) continue;
#pragma unroll
            for (int c = 0; c < kMaxD; ++c) {
                const float x = c < d ? xs[(size_t)cid * d + c] : 0.f;
                lo[c] = fminf(lo[c], x);
                hi[c] = fmaxf(hi[c], x);
            }
            emax = fmaxf(emax, err_coef * vn[cid]);
            imax = any ? fmaxf(imax, isp[cid]) : isp[cid];
            any = true;
        }
        float* o = base + 2 * HBOX + (size_t)(h * (TC / 16) + g) * GREC;
        o[0] = emax;
        o[1] = imax;
    }
#pragma unroll
    for (int c = 0; c < kMaxD; ++c) { base[h * HBOX + c] = lo[c]; base[h * HBOX + 8 + c] = hi[c]; }
}

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
// Sorts keys[0, len) for a power of two len <= RBUF; callers keep every entry at or
// beyond their fill count at ~0 (the largest key), so sorting the smallest power of
// two that covers the fill orders the whole buffer.
__device__ void warp_bitonic_sort(unsigned long long* keys, int len = RBUF) {
    const int lane = threadIdx.x & 31;
    for (int k = 2; k <= len; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < len; i += 32) {
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

__device__ __forceinline__ int sort_len(int fill) {
    int len = 32;
    while (len < fill && len < RBUF) len <<= 1;
    return len;
}

__device__ __forceinline__ unsigned long long pack_key(float d, int id) {
    return ((unsigned long long)__float_as_uint(d) << 32) | (unsigned)id;
}

// ------------------------------------------------------------------ rescoring
struct RescoreParams {
    const float* v; int m;          // natural layout, dataset order
    const float* coords; int d;     // raw coordinates, dataset order
    const float* inv_ls_df;         // 1 / lengthscale as double-float pairs (hi, lo) per axis
    const float* p;
    float var; int kernel_type; int predecessor;
    long long n;
    const int* slot_id; long long nslots;
    const int* surv; const int* surv_cnt; int half_cap;
    const float* survb;  // the sweep's bound of each survivor (see MMAParams)
    const int* full_slots; int nfull;  // slots rescored against every valid candidate
    int k;
    long long* out_idx; float* out_dist;
    long long* evals;
    // visiting order of the survivor pass: query slots in the sweep's (Hilbert) order,
    // each followed by its candidate parts, so neighbouring warps gather overlapping rows
    const int* order; int parts;
    int chunk;  // candidates per item of the exhaustive pass (parts == 1)
    // certified FP32 filter of the survivor pass (see rescore_kernel)
    const float* xs;             // scaled coordinates x / l (f32, as the sweep uses them)
    const float* vn;             // |v| rounded up
    const float* isp;            // 1 / sqrt(p)
    const float* xmax;           // max |x / l| per row
    const unsigned* xmax_max;    // bits of the dataset's largest xmax
    const unsigned* isp_max;     // bits of the dataset's largest 1 / sqrt(p)
    const unsigned* qtau;        // per query (slot / parts): the sweep's smallest part threshold (d^2 bits)
};

// ---------------------------------------------------------- double-float
// A value is an unevaluated sum h + l of two floats with |l| <= ulp(h)/2 (about
// 48 significant bits).  TwoSum / TwoProd (Knuth, Dekker) give the exact rounding
// errors; products of pairs drop only l*l terms.  Used for the exact distance of a
// rescored pair: the FP64-grade result at FP32 issue rates.
struct df {
    float h, l;
};
__device__ __forceinline__ df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    return df{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z))};
}
__device__ __forceinline__ df df_fast(float a, float b) {  // |a| >= |b| or a == 0
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_add(df x, df y) {
    const df s = df_two_sum(x.h, y.h);
    return df_fast(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}
__device__ __forceinline__ df df_neg(df x) { return df{-x.h, -x.l}; }
__device__ __forceinline__ df df_mul(df x, df y) {
    const float p = __fmul_rn(x.h, y.h);
    float e = __fmaf_rn(x.h, y.h, -p);
    e = __fmaf_rn(x.h, y.l, e);
    e = __fmaf_rn(x.l, y.h, e);
    return df_fast(p, e);
}
__device__ __forceinline__ df df_mulf(df x, float f) {
    const float p = __fmul_rn(x.h, f);
    const float e = __fmaf_rn(x.l, f, __fmaf_rn(x.h, f, -p));
    return df_fast(p, e);
}
__device__ __forceinline__ df df_sqrt(df x) {  // one Newton step from sqrtf
    if (!(x.h > 0.f)) return df{0.f, 0.f};
    const float r = sqrtf(x.h);
    const float sq = __fmul_rn(r, r);
    const float res = __fadd_rn(__fsub_rn(__fsub_rn(x.h, sq), __fmaf_rn(r, r, -sq)), x.l);
    return df_fast(r, res / (2.f * r));
}
__device__ __forceinline__ df df_div(df a, df b) {  // two quotient digits
    const float q0 = a.h / b.h;
    const df r = df_add(a, df_neg(df_mulf(b, q0)));
    return df_fast(q0, r.h / b.h);
}
__device__ __forceinline__ bool df_gt(df a, df b) { return a.h > b.h || (a.h == b.h && a.l > b.l); }

// Double-float constants split from their double values at compile time.
#define CT_DF(x) df{(float)(x), (float)((x) - (double)(float)(x))}
// 1/i!, i = 0..12, as (hi, lo)
__constant__ float kInvFact[26] = {
#define CT_IF(f) (float)(1.0 / (f)), (float)(1.0 / (f) - (double)(float)(1.0 / (f)))
    CT_IF(1.0), CT_IF(1.0), CT_IF(2.0), CT_IF(6.0), CT_IF(24.0), CT_IF(120.0), CT_IF(720.0), CT_IF(5040.0),
    CT_IF(40320.0), CT_IF(362880.0), CT_IF(3628800.0), CT_IF(39916800.0), CT_IF(479001600.0)
#undef CT_IF
};

// e^x for x <= 0: x = n ln2 + r (|r| <= ln2/2, ln2 as a double-float pair), the
// Taylor series of e^r to degree 12 (truncation < 2e-16) in double-float Horner form,
// then the scaling by 2^n in two exact steps.
__device__ __forceinline__ df df_exp(df x) {
    if (x.h < -103.f) return df{0.f, 0.f};
    const float n = rintf(__fmul_rn(x.h, 1.44269504088896341f));
    const df ln2 = CT_DF(0.693147180559945309417);
    const df r = df_add(x, df_neg(df_mulf(ln2, n)));
    df p = df{kInvFact[24], kInvFact[25]};
#pragma unroll
    for (int i = 11; i >= 0; --i) p = df_add(df_mul(p, r), df{kInvFact[2 * i], kInvFact[2 * i + 1]});
    const int ni = (int)n;
    const int hh = ni / 2;
    const float s1 = __int_as_float((hh + 127) << 23), s2 = __int_as_float((ni - hh + 127) << 23);
    return df{__fmul_rn(__fmul_rn(p.h, s1), s2), __fmul_rn(__fmul_rn(p.l, s1), s2)};
}

// Compensated FP32 dot product pieces (TwoProd via FMA, TwoSum).  The warp
// splits a row of m <= 1024 floats into 32 lane slices of m/32 contiguous
// elements (4-float aligned when m % 128 == 0, else scalar); each lane keeps
// the query slice in registers and accumulates a (sum, compensation) pair.
// (explicitly rounded operations: no contraction, the same result at every call site)
__device__ __forceinline__ void two_sum_acc(float& s, float& comp, float a, float b) {
    const float pr = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -pr);
    const float ts = __fadd_rn(s, pr);
    const float z = __fsub_rn(ts, s);
    const float se = __fadd_rn(__fsub_rn(s, __fsub_rn(ts, z)), __fsub_rn(pr, z));
    s = ts;
    comp = __fadd_rn(comp, __fadd_rn(se, pe));
}

// Load the query slice: lane l holds elements [l*m/32, (l+1)*m/32).
__device__ __forceinline__ void load_query_slice(const float* row, int m, float (&vq)[32]) {
    const int lane = threadIdx.x & 31;
    const int per = m >> 5;
    const float* r = row + (size_t)lane * per;
#pragma unroll
    for (int t = 0; t < 32; ++t) vq[t] = t < per ? r[t] : 0.f;
}

// One step of the warp reduction of (sum, compensation) pairs: TwoSum of the sums, the
// compensations added.  Symmetric in its arguments, so both lanes of a butterfly pair
// end with the same value.
__device__ __forceinline__ void df_combine(float& hi, float& lo, float oh, float ol) {
    const float t = __fadd_rn(hi, oh);
    const float z = __fsub_rn(t, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, z)), __fsub_rn(oh, z));
    hi = t;
    lo = __fadd_rn(__fadd_rn(lo, ol), err);
}
// The same two steps on two independent sums at once (f32x2; each component rounds as the
// scalar __fadd_rn / __fmul_rn / __fmaf_rn do, and x - y is x + (-y) exactly).  Measured
// on GB300: an f32x2 multiply whose only use is an f32x2 add gives the bits of a fused
// multiply-add in about 5% of random cases, with or without -fmad=false; here the product
// pr has several uses, and the forced exhaustive tests check that these passes and the
// scalar warp reduction agree bit for bit.
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void two_sum_acc2(float2& s, float2& comp, float2 a, float2 b) {
    const float2 pr = __fmul2_rn(a, b);
    const float2 pe = __ffma2_rn(a, b, neg2(pr));
    const float2 ts = __fadd2_rn(s, pr);
    const float2 z = __fadd2_rn(ts, neg2(s));
    const float2 se = __fadd2_rn(__fadd2_rn(s, neg2(__fadd2_rn(ts, neg2(z)))), __fadd2_rn(pr, neg2(z)));
    s = ts;
    comp = __fadd2_rn(comp, __fadd2_rn(se, pe));
}
__device__ __forceinline__ void df_combine2(float2& hi, float2& lo, float2 oh, float2 ol) {
    const float2 t = __fadd2_rn(hi, oh);
    const float2 z = __fadd2_rn(t, neg2(hi));
    const float2 err = __fadd2_rn(__fadd2_rn(hi, neg2(__fadd2_rn(t, neg2(z)))), __fadd2_rn(oh, neg2(z)));
    hi = t;
    lo = __fadd2_rn(__fadd2_rn(lo, ol), err);
}

// Dots of the query slice with NC candidate rows at once (independent loads in flight).
// Lane L sums elements [L m/32, (L+1) m/32) in order; the lanes' pairs are combined by a
// butterfly over lane offsets 16, 8, 4, 2, 1.
template <int NC>
__device__ __forceinline__ void warp_dots(const float* __restrict__ V, int m, const int (&cid)[NC],
                                          const float (&vq)[32], df (&out)[NC]) {
    const int lane = threadIdx.x & 31;
    const int per = m >> 5;
    float s[NC], comp[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) { s[c] = 0.f; comp[c] = 0.f; }
    if ((per & 3) == 0) {
#pragma unroll
        for (int t4 = 0; t4 < 8; ++t4) {
            if (t4 * 4 < per) {
                float4 x[NC];
#pragma unroll
                for (int c = 0; c < NC; ++c)
                    x[c] = cid[c] >= 0 ? __ldg((const float4*)(V + (size_t)cid[c] * m + (size_t)lane * per) + t4)
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    two_sum_acc(s[c], comp[c], vq[4 * t4 + 0], x[c].x);
                    two_sum_acc(s[c], comp[c], vq[4 * t4 + 1], x[c].y);
                    two_sum_acc(s[c], comp[c], vq[4 * t4 + 2], x[c].z);
                    two_sum_acc(s[c], comp[c], vq[4 * t4 + 3], x[c].w);
                }
            }
        }
    } else {
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            if (t < per) {
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const float b = cid[c] >= 0 ? __ldg(V + (size_t)cid[c] * m + (size_t)lane * per + t) : 0.f;
                    two_sum_acc(s[c], comp[c], vq[t], b);
                }
            }
        }
    }
    // Warp reduction in double-float: a butterfly of TwoSum on the (sum, compensation)
    // pairs, so every lane ends with the same double-float value.
#pragma unroll
    for (int c = 0; c < NC; ++c) {
        float hi = s[c], lo = comp[c];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float oh = __shfl_xor_sync(0xffffffffu, hi, off);
            const float ol = __shfl_xor_sync(0xffffffffu, lo, off);
            df_combine(hi, lo, oh, ol);
        }
        out[c] = df_fast(hi, lo);
    }
}

// Exact residual distance of one pair from its double-float V dot product: the
// kernel value from the f32 coordinates, the normalisation and the square root, in
// double-float arithmetic (one lane per pair).
__device__ __forceinline__ float exact_from_dot(const RescoreParams& P, int q, int c, df dot) {
    if (q == c) return 0.f;
    df d2 = df{0.f, 0.f};
    for (int a = 0; a < P.d; ++a) {
        const df t = df_two_sum(P.coords[(size_t)q * P.d + a], -P.coords[(size_t)c * P.d + a]);  // exact
        const df u = df_mul(t, df{P.inv_ls_df[2 * a], P.inv_ls_df[2 * a + 1]});
        d2 = df_add(d2, df_mul(u, u));
    }
    df kv;
    if (P.kernel_type == 0) {
        kv = df_mulf(df_exp(df{-0.5f * d2.h, -0.5f * d2.l}), P.var);
    } else {
        const df a = df_mul(df_sqrt(d2), CT_DF(2.23606797749978969641));
        const df poly = df_add(df_add(df{1.f, 0.f}, a), df_mul(df_mul(a, a), CT_DF(1.0 / 3.0)));
        kv = df_mulf(df_mul(poly, df_exp(df_neg(a))), P.var);
    }
    const float pq = P.p[q], pc = P.p[c];
    const float ph = __fmul_rn(pq, pc);
    df pp = df_fast(ph, __fmaf_rn(pq, pc, -ph));  // exact product
    const df floor18 = CT_DF(1e-18);
    if (!df_gt(pp, floor18)) pp = floor18;
    df rho = df_div(df_add(kv, df_neg(dot)), df_sqrt(pp));
    if (rho.h < 0.f) rho = df_neg(rho);
    if (rho.h > 1.f || (rho.h == 1.f && rho.l > 0.f)) rho = df{1.f, 0.f};
    const df ds = df_add(df{1.f, 0.f}, df_neg(rho));
    if (!(ds.h > 0.f)) return 0.f;
    const df dist = df_sqrt(ds);
    return __fadd_rn(dist.h, dist.l);
}
#undef CT_DF

__device__ __forceinline__ void warp_topk_append(unsigned long long* keys, int& fill, int k, bool has,
                                                 unsigned long long key);

// Plain FP32 dots of the query slice with NC candidate rows (the split of warp_dots,
// one FMA per element, then a butterfly sum).  Each lane's chain has m/32 roundings
// and the butterfly 5 more, so |error| <= (m/32 + 7) 2^-24 |v_q| |v_c|.
template <int NC>
__device__ __forceinline__ void warp_dots_f32(const float* __restrict__ V, int m, const int (&cid)[NC],
                                              const float (&vq)[32], float (&out)[NC]) {
    const int lane = threadIdx.x & 31;
    const int per = m >> 5;
    float s[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) s[c] = 0.f;
    if ((per & 3) == 0) {
#pragma unroll
        for (int t4 = 0; t4 < 8; ++t4) {
            if (t4 * 4 < per) {
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const float4 x = cid[c] >= 0 ? __ldg((const float4*)(V + (size_t)cid[c] * m + (size_t)lane * per) + t4)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
                    s[c] = __fmaf_rn(vq[4 * t4 + 0], x.x, s[c]);
                    s[c] = __fmaf_rn(vq[4 * t4 + 1], x.y, s[c]);
                    s[c] = __fmaf_rn(vq[4 * t4 + 2], x.z, s[c]);
                    s[c] = __fmaf_rn(vq[4 * t4 + 3], x.w, s[c]);
                }
            }
        }
    } else {
#pragma unroll
        for (int t = 0; t < 32; ++t) {
            if (t < per) {
#pragma unroll
                for (int c = 0; c < NC; ++c) {
                    const float b = cid[c] >= 0 ? __ldg(V + (size_t)cid[c] * m + (size_t)lane * per + t) : 0.f;
                    s[c] = __fmaf_rn(vq[t], b, s[c]);
                }
            }
        }
    }
#pragma unroll
    for (int c = 0; c < NC; ++c) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s[c] = __fadd_rn(s[c], __shfl_xor_sync(0xffffffffu, s[c], off));
        out[c] = s[c];
    }
}

// Certified bounds [dl2, du2] of d^2 = 1 - |rho| for one pair from an FP32 dot with
// error <= ed: the kernel value from the scaled f32 coordinates with the sweep's error
// model (ale, bee, alk, bek as there), the normalisation 1 / sqrt(max(p_q p_c, 1e-18)).
// xq, xc: the pair's scaled coordinates (global or shared memory; the candidate's axes
// xc_stride apart); isc = 1 / sqrt(p_c).
__device__ __forceinline__ void pair_bounds_core(const RescoreParams& P, const float* xq, const float* xc, float isc,
                                                 float dot, float ed, float isq, float alk, float bek, float ale,
                                                 float bee, float& dl2, float& du2, int xc_stride = 1) {
    float d2 = 0.f;
    for (int a = 0; a < P.d; ++a) {
        const float t = __fsub_rn(xc[a * xc_stride], xq[a]);
        d2 = __fmaf_rn(t, t, d2);
    }
    float kv, ek;
    if (P.kernel_type == 0) {
        kv = __fmul_rn(P.var, __expf(__fmul_rn(-0.5f, d2)));
        ek = __fmul_rn(kv, __fmaf_rn(alk, d2, bek));
    } else {
        const float ed2 = __fmaf_rn(ale, d2, bee);
        const float a = 2.2360679775f * sqrtf(d2);
        const float ea = __expf(-a);
        kv = P.var * (1.f + a + a * a * 0.33333334f) * ea;
        ek = kv * (1e-6f + 2.4e-7f * a) + P.var * (0.8334f * ed2 + 1e-7f * a * a) * (1.f + a) * ea;
    }
    const float R = fabsf(__fsub_rn(kv, dot));
    const float e = __fadd_rn(__fadd_rn(ed, ek), __fmaf_rn(R, 1.2e-7f, 1e-30f));
    const float sc = fminf(__fmul_rn(isq, isc), 1e9f);
    const float rl = __fmul_rn(__fmul_rn(fmaxf(__fsub_rn(R, e), 0.f), sc), 1.f - 2e-6f);
    const float rh = __fmul_rn(__fmul_rn(__fadd_rn(R, e), sc), 1.f + 2e-6f);
    du2 = 1.f - fminf(rl, 1.f);
    dl2 = fmaxf(1.f - fminf(rh, 1.f), 0.f);
}
__device__ __forceinline__ void pair_bounds_f32(const RescoreParams& P, int q, int c, float dot, float ed, float isq,
                                                float alk, float bek, float ale, float bee, float& dl2, float& du2) {
    pair_bounds_core(P, P.xs + (size_t)q * P.d, P.xs + (size_t)c * P.d, P.isp[c], dot, ed, isq, alk, bek, ale, bee,
                     dl2, du2);
}

// Survivor rescoring, one warp per query slot, in two steps.
//  F: every survivor gets certified bounds [dl2, du2] of its d^2 from a plain FP32 dot
//     (error (m/32 + 7) 2^-24 |v_q| |v_c|, some fifty times tighter than the sweep's
//     BF16 bound) at one instruction per element.  tau = the k-th smallest du2, widened
//     by the double-float error of the exact distances, bounds the k-th distance.
//  E: only survivors with dl2 <= tau are rescored exactly (compensated FP32 dot,
//     double-float distance); the others cannot enter the top k.
// Streaming top-k of E through a sorted shared buffer: entries [0, k) hold the current
// best, new candidates fill the rest, and a full buffer is re-sorted.  Shared memory per
// warp: RBUF keys, then RBUF floats (du2, reused for the kept ids).
__global__ void rescore_kernel(RescoreParams P) {
    extern __shared__ unsigned long long rkeys_all[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x / 32;
    unsigned long long* keys = rkeys_all + (size_t)warp * RBUF;
    float* du2s = (float*)(rkeys_all + (size_t)wpb * RBUF) + (size_t)warp * RBUF;
    int* kept = (int*)du2s;
    const long long w = (long long)blockIdx.x * wpb + warp;
    if (w >= P.nslots) return;
    const int slot = P.order ? P.order[w / P.parts] * P.parts + (int)(w % P.parts) : (int)w;
    const int c0 = P.surv_cnt[2 * slot];
    const int c1 = P.surv_cnt[2 * slot + 1];
    if (c0 > P.half_cap || c1 > P.half_cap) return;  // handled by the exhaustive pass
    const int q = P.slot_id[slot];
    if (q < 0) {
        for (int j = lane; j < P.k; j += 32) { P.out_idx[(size_t)slot * P.k + j] = -1; P.out_dist[(size_t)slot * P.k + j] = CT_FLT_MAX; }
        return;
    }
    const int k = P.k;
    float vql[32];
    load_query_slice(P.v + (size_t)q * P.m, P.m, vql);
    // per-query constants of the bounds
    const float isq = P.isp[q];
    const float ed_q = (float)((P.m >> 5) + 7) * 5.97e-8f * P.vn[q];
    const float dd = (float)P.d, ced2 = (dd + 2.f) * 5.97e-8f;
    const float A = 2.4e-7f * (P.xmax[q] + __uint_as_float(__ldg(P.xmax_max)));
    const float ale = (ced2 + 0.5f * A * dd) * 1.00001f, bee = 0.5f * A * 1.00001f;
    const float alk = (6e-8f + 0.5f * ced2 + 0.25f * A * dd) * 1.00001f, bek = (1e-6f + 0.25f * A) * 1.00001f;
    // ---- survivors the query's final threshold excludes (the sweep's own keep test with
    // the threshold it ended with: any part's k-th upper bound) are dropped before any row
    // is read; the others are compacted into keys (ids in the low bits)
    int count = 0;
    const float tq = __uint_as_float(__ldcg(&P.qtau[slot / P.parts]));
    {
        const float thr = (1.f - tq) * (1.f - 2e-6f) / isq;
        for (int base = 0; base < c0 + c1; base += 32) {
            const int ci = base + lane;
            int cid = -1;
            bool keep = false;
            if (ci < c0 + c1) {
                const size_t o = ci < c0 ? (size_t)(2 * slot) * P.half_cap + ci : (size_t)(2 * slot + 1) * P.half_cap + (ci - c0);
                cid = P.surv[o];
                keep = P.survb[o] >= thr;
            }
            const unsigned mk = __ballot_sync(0xffffffffu, keep);
            if (keep) keys[count + __popc(mk & ((1u << lane) - 1u))] = (unsigned long long)(unsigned)cid;
            count += __popc(mk);
        }
        __syncwarp();
    }
    // ---- F: certified FP32 bounds of every remaining survivor
    for (int base = 0; base < count; base += 32) {
        const int ci = base + lane;
        const int cid = ci < count ? (int)(unsigned)(keys[ci] & 0xffffffffULL) : -1;
        const int nb = count - base < 32 ? count - base : 32;
        float mydot = 0.f;
        for (int t = 0; t < nb; t += 4) {
            int cc[4];
            float dots[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int src = __shfl_sync(0xffffffffu, cid, (t + u) & 31);
                cc[u] = (t + u) < nb ? src : -1;
            }
            warp_dots_f32<4>(P.v, P.m, cc, vql, dots);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (lane == t + u) mydot = dots[u];
        }
        if (ci < count) {
            float dl2 = 0.f, du2 = 0.f;  // the query itself: d = 0
            if (cid != q)
                pair_bounds_f32(P, q, cid, mydot, __fmul_rn(ed_q, P.vn[cid]), isq, alk, bek, ale, bee, dl2, du2);
            keys[ci] = ((unsigned long long)__float_as_uint(dl2) << 32) | (unsigned)cid;
            du2s[ci] = du2;
        }
    }
    __syncwarp();
    // tau: the k-th smallest du2 (bisection over the bit patterns of these non-negative
    // floats), plus the margin of the seeded thresholds; every survivor when fewer than k
    float tau = CT_FLT_MAX;
    if (count > k) {
        unsigned lo = 0, hi = 0x3f800000u;  // du2 <= 1
        while (lo < hi) {
            const unsigned mid = lo + ((hi - lo) >> 1);
            int c = 0;
            for (int i = lane; i < count; i += 32) c += __float_as_uint(du2s[i]) <= mid;
            c = __reduce_add_sync(0xffffffffu, c);
            if (c >= k) hi = mid; else lo = mid + 1;
        }
        const float margin = 4e-12f * fminf(isq * __uint_as_float(__ldg(P.isp_max)) * 1.01f, 1e9f) + 1e-12f;
        tau = __fadd_ru(__fmul_ru(__uint_as_float(lo), 1.000004f), margin);
    }
    // the query's final threshold bounds its k-th distance over all parts: a part slot
    // rescores only what can enter the query's top k, not its own k best
    tau = fminf(tau, tq);
    __syncwarp();
    // compaction of the survivors that can still be among the k nearest
    int nk = 0;
    for (int base = 0; base < count; base += 32) {
        const int ci = base + lane;
        unsigned long long key = ci < count ? keys[ci] : 0ULL;
        const bool keep = ci < count && __uint_as_float((unsigned)(key >> 32)) <= tau;
        const unsigned mask = __ballot_sync(0xffffffffu, keep);
        __syncwarp();  // every lane has read its key before the ids overwrite du2s
        if (keep) kept[nk + __popc(mask & ((1u << lane) - 1u))] = (int)(unsigned)(key & 0xffffffffULL);
        nk += __popc(mask);
    }
    for (int i = lane; i < RBUF; i += 32) keys[i] = ~0ULL;
    __syncwarp();
    // ---- E: exact rescoring of the kept survivors
    int fill = k;  // next free position in the buffer
    for (int base = 0; base < nk; base += 32) {
        const int ci = base + lane;
        const int cid = ci < nk ? kept[ci] : -1;
        df mydot = df{0.f, 0.f};
        const int nb = nk - base < 32 ? nk - base : 32;
        for (int t = 0; t < nb; t += 4) {
            int cc[4];
            df dots[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int src = __shfl_sync(0xffffffffu, cid, (t + u) & 31);
                cc[u] = (t + u) < nb ? src : -1;
            }
            warp_dots<4>(P.v, P.m, cc, vql, dots);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (lane == t + u) mydot = dots[u];
        }
        const float mydist = ci < nk ? exact_from_dot(P, q, cid, mydot) : 0.f;
        warp_topk_append(keys, fill, k, ci < nk, pack_key(mydist, cid));
    }
    warp_bitonic_sort(keys, sort_len(fill));
    for (int j = lane; j < k; j += 32) {
        unsigned long long key = keys[j];
        bool ok = key != ~0ULL;
        P.out_idx[(size_t)slot * k + j] = ok ? (long long)(unsigned)(key & 0xffffffffULL) : -1LL;
        P.out_dist[(size_t)slot * k + j] = ok ? __uint_as_float((unsigned)(key >> 32)) : CT_FLT_MAX;
    }
    if (lane == 0 && P.evals) atomicAdd((unsigned long long*)P.evals, (unsigned long long)nk);
}

__device__ __forceinline__ void warp_topk_append(unsigned long long* keys, int& fill, int k, bool has,
                                                 unsigned long long key) {
    const int lane = threadIdx.x & 31;
    unsigned mask = __ballot_sync(0xffffffffu, has);
    int added = __popc(mask);
    if (fill + added > RBUF) {
        __syncwarp();
        warp_bitonic_sort(keys);
        for (int i = k + lane; i < RBUF; i += 32) keys[i] = ~0ULL;
        __syncwarp();
        fill = k;
    }
    if (has) keys[fill + __popc(mask & ((1u << lane) - 1u))] = key;
    fill += added;
    __syncwarp();
}

// Merge the chunk results of each overflowed query into its output row.
__global__ void merge_chunks_kernel(RescoreParams P, const int* item_begin, const unsigned long long* partial) {
    extern __shared__ unsigned long long mkeys_all[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x / 32;
    unsigned long long* keys = mkeys_all + (size_t)warp * RBUF;
    const long long w = (long long)blockIdx.x * wpb + warp;
    if (w >= P.nfull) return;
    const int slot = P.full_slots[w];
    const int k = P.k;
    for (int i = lane; i < RBUF; i += 32) keys[i] = ~0ULL;
    __syncwarp();
    int fill = k;
    const long long e0 = (long long)item_begin[w] * k, e1 = (long long)item_begin[w + 1] * k;
    // 128 keys per round, loads issued together; chunk lists are mostly padding
    for (long long base = e0; base < e1; base += 128) {
        unsigned long long key[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const long long o = base + 32 * u + lane;
            key[u] = o < e1 ? __ldcs(partial + o) : ~0ULL;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (__any_sync(0xffffffffu, key[u] != ~0ULL)) warp_topk_append(keys, fill, k, key[u] != ~0ULL, key[u]);
    }
    warp_bitonic_sort(keys, sort_len(fill));
    for (int j = lane; j < k; j += 32) {
        const unsigned long long key = keys[j];
        const bool ok = key != ~0ULL;
        P.out_idx[(size_t)slot * k + j] = ok ? (long long)(unsigned)(key & 0xffffffffULL) : -1LL;
        P.out_dist[(size_t)slot * k + j] = ok ? __uint_as_float((unsigned)(key >> 32)) : CT_FLT_MAX;
    }
}

// Slots whose survivor lists overflowed; bit 31 marks those for the filtered pass.
__global__ void collect_overflow_kernel(const int* __restrict__ surv_cnt, long long nslots, int half_cap,
                                        const int* __restrict__ slot_id, const float* __restrict__ isp,
                                        const float* __restrict__ vn, int filter, int* __restrict__ list,
                                        int* __restrict__ nlist) {
    long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (s >= nslots) return;
    if (surv_cnt[2 * s] > half_cap || surv_cnt[2 * s + 1] > half_cap) {
        const int q = slot_id[s];
        const bool f = filter && q >= 0 && isp[q] * vn[q] <= kFilterIsq;
        list[atomicAdd(nlist, 1)] = (int)s | (f ? (int)0x80000000u : 0);
    }
}


}  // namespace screen
}  // namespace ct

// ======================================================================= host
namespace ct {
namespace screen {

// One "level" of the threshold pass: the points of a prefix [0, P) of the
// dataset (P = 2^j), or the whole dataset, in Hilbert order.  Predecessor-mode
// query q uses the largest prefix level with P <= q, so every candidate of its
// window is a valid predecessor.
struct Level {
    long long size = 0, row_off = 0, rows_pad = 0;
};

struct State {
    long long n = 0, rows_pad = 0;        // candidate rows padded to TC
    int* hil_order = nullptr;             // sorted position -> dataset id
    unsigned long long* hil_key = nullptr;  // Hilbert key by dataset id
    bf16 *ds_hi = nullptr, *ds_lo = nullptr;    // dataset order, blocked
    int* b_id_ds = nullptr;
    // threshold-pass levels, concatenated in one blocked matrix
    std::vector<Level> levels;
    long long lvl_rows = 0;
    bf16 *lvl_hi = nullptr, *lvl_lo = nullptr;
    int* lvl_id = nullptr;                  // row -> dataset id (-1 padding)
    unsigned long long* lvl_key = nullptr;  // row -> Hilbert key (UINT64_MAX padding)
    long long* lvl_meta = nullptr;          // [nlevels][3]: size, row_off, rows_pad
    float *vn = nullptr, *isp = nullptr, *xmax = nullptr;
    unsigned* isp_max = nullptr;            // bits of max 1/sqrt(p) over the dataset rows
    float *rec_lvl = nullptr, *rec_ds = nullptr;  // sweep candidate records, tile order
    unsigned* xmax_max = nullptr;                 // bits of max |x| over the dataset rows
    double* inv_ls64 = nullptr;
    float* inv_ls_df = nullptr;             // (hi, lo) float pairs of 1 / lengthscale
    int* status = nullptr;
    double* bounds = nullptr;               // Hilbert quantisation frame of the dataset (min/max per axis)
    // query slab: rows [n, n + slab_cap) of the query-side arrays hold new points
    long long slab_cap = 0;
    cudaEvent_t slab_done = nullptr;        // last call that read the slab
};

constexpr int kFirstPrefixLog2 = 10;  // prefixes below 1024 points: every predecessor is rescored

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
// slot ids from int64 query ids (out-of-range ids become -1) and the sweep sort
// key: high 32 bits = group (predecessor mode: level and one of kBands id bands
// of the level's query range), low 32 bits = row of the query's Hilbert
// position inside its level.  Queries without a level sort last.
constexpr int kBands = 16;
constexpr int kWarmTiles = 32;  // nearest candidate tiles that set the thresholds before any pair is kept (measured best of 8-64)

// A (query tile, part) unit of the sweep and the kernel that writes its jobs.
struct JobUnit {
    int qx;               // query tile of the A operand (t * parts + p)
    int p, parts;
    int cc, t0, ntl;      // level tiles [t0, t0 + ntl), spiral centre cc (ntl = 0: no level)
    int lo_tile;          // dataset tiles from lo_tile follow the level tiles
    int warm, count;      // warm-up jobs; all jobs
    long long off;        // first job in the flat list
    // Jobs whose candidate ids all lie below every query id of the tile need no
    // predecessor or self test (flag 8): level tiles when the level size is at most
    // the tile's smallest query id, dataset tiles below ds_fast_end.
    int fast_lvl, ds_fast_end;
    int lin;              // main sweep over the level tiles in ascending order (else the spiral)
};

// w-th tile of the spiral cc, cc+1, cc-1, cc+2, cc-2, ... clipped to [t0, t0 + ntl)
__device__ __forceinline__ int spiral_tile(const JobUnit& U, int w) {
    if (w == 0) return U.cc;
    const int left = U.cc - U.t0, right = U.t0 + U.ntl - 1 - U.cc;
    const int mm = left < right ? left : right;
    if (w <= 2 * mm) return (w & 1) ? U.cc + (w + 1) / 2 : U.cc - w / 2;
    return right > left ? U.cc + (w - mm) : U.cc - (w - mm);
}
// position of level tile t in that spiral (the inverse of spiral_tile)
__device__ __forceinline__ int spiral_index(const JobUnit& U, int t) {
    const int dd = t - U.cc;
    if (dd == 0) return 0;
    const int left = U.cc - U.t0, right = U.t0 + U.ntl - 1 - U.cc;
    const int mm = left < right ? left : right;
    const int ad = dd < 0 ? -dd : dd;
    if (ad <= mm) return dd > 0 ? 2 * dd - 1 : 2 * ad;
    return ad + mm;
}
// w-th level tile of the main sweep (w < ntl): ascending from t0, so that the units of a
// level in flight on different SMs read the same candidate tiles at about the same time
// and share them in L2; the warm-up has already taken the nearest tiles in spiral order.
__device__ __forceinline__ int main_tile(const JobUnit& U, int w) { return U.lin ? U.t0 + w : spiral_tile(U, w); }

// Exhaustive rescoring, tiled: a CTA takes a group of up to XQ overflowed query slots
// that share a candidate source (the main pass: the id range [0, cend); the part pass:
// the tiles of one (query tile, part) unit) and one chunk of that source.  Candidate
// rows are staged XC at a time in shared memory, transposed (element-major), so that
// every staged row serves all the group's queries: lane l of warp w forms the
// compensated dot products of candidate l with queries w and w + 8 (two interleaved
// TwoProd/TwoSum accumulators per pair, combined in double-float), then the exact
// distance and a streaming top-k per query.  Compared with one warp per (query,
// chunk), the L2 traffic of the candidate rows falls by the group size.  Each slot's
// partial top k of the chunk lands in its row of `partial`.
constexpr int XQ = 16;    // query slots per group (two per warp)
constexpr int XC = 32;    // candidates staged per block (one per lane)
constexpr int XKB = 128;  // key buffer per query (k <= 64)
struct ExhGroup {
    int g0, ng;       // slots full_slots[g0 .. g0 + ng)
    int unit;         // part pass: unit; main pass: -1
    int nchunks;
    long long cend;   // main pass: candidate ids [0, cend)
};
struct ExhItem {
    int group, chunk;
};
__host__ __device__ inline size_t tile_smem_bytes(int m) {
    return sizeof(float) * (size_t)m * XC + sizeof(float) * (size_t)XQ * m + sizeof(unsigned long long) * XQ * XKB;
}

__device__ __forceinline__ void keys_append(unsigned long long* keys, int& fill, int k, bool has,
                                            unsigned long long key) {
    const int lane = threadIdx.x & 31;
    const unsigned mask = __ballot_sync(0xffffffffu, has);
    const int added = __popc(mask);
    if (fill + added > XKB) {
        __syncwarp();
        warp_bitonic_sort(keys, XKB);
        for (int i = k + lane; i < XKB; i += 32) keys[i] = ~0ULL;
        __syncwarp();
        fill = k;
    }
    if (has) keys[fill + __popc(mask & ((1u << lane) - 1u))] = key;
    fill += added;
    __syncwarp();
}

template <int PER>  // m / 32 when fixed at compile time (8 or 16), else 0
__global__ void __launch_bounds__(256) rescore_tile_kernel(RescoreParams P, const ExhGroup* __restrict__ groups,
                                                           const ExhItem* __restrict__ items, const int* __restrict__ ibeg,
                                                           int cand_chunk, int tpc, const JobUnit* __restrict__ units,
                                                           const int* __restrict__ lvl_id, const int* __restrict__ ds_id,
                                                           unsigned long long* __restrict__ partial) {
    extern __shared__ __align__(16) unsigned char xs_raw[];
    const int m = P.m, k = P.k;
    float* cs = (float*)xs_raw;                                            // [m][XC]
    float* qs = cs + (size_t)m * XC;                                       // [XQ/2][m][2]
    unsigned long long* kb = (unsigned long long*)(qs + (size_t)XQ * m);  // [XQ][XKB]
    __shared__ int cid_s[XC];
    __shared__ int qid_s[XQ];
    const int per = PER > 0 ? PER : m >> 5;
    const ExhItem it = items[blockIdx.x];
    const ExhGroup G = groups[it.group];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x < XQ) qid_s[threadIdx.x] = threadIdx.x < G.ng ? P.slot_id[P.full_slots[G.g0 + threadIdx.x]] : -1;
    __syncthreads();
    // query rows interleaved by warp pair: element t of slots w and w + 8 side by side
    for (int e = threadIdx.x; e < XQ * m; e += blockDim.x) {
        const int g = e / m, t = e - g * m;
        const int q = qid_s[g];
        qs[((size_t)(g & 7) * m + t) * 2 + (g >> 3)] = q >= 0 ? P.v[(size_t)q * m + t] : 0.f;
    }
    for (int e = threadIdx.x; e < XQ * XKB; e += blockDim.x) kb[e] = ~0ULL;
    long long c_lo = 0, total = 0;
    int t_lo = 0;
    JobUnit U{};
    if (G.unit < 0) {
        c_lo = (long long)it.chunk * cand_chunk;
        const long long c_hi = G.cend < c_lo + cand_chunk ? G.cend : c_lo + cand_chunk;
        total = c_hi > c_lo ? c_hi - c_lo : 0;
    } else {
        U = units[G.unit];
        const int mine = U.count - U.warm;
        t_lo = it.chunk * tpc;
        const int t_hi = mine < t_lo + tpc ? mine : t_lo + tpc;
        total = t_hi > t_lo ? (long long)(t_hi - t_lo) * TC : 0;
    }
    const int ga = warp, gb = warp + 8;
    const int ida = qid_s[ga], idb = qid_s[gb];
    unsigned long long* ka = kb + (size_t)ga * XKB;
    unsigned long long* kbb = kb + (size_t)gb * XKB;
    const float* q2 = qs + (size_t)ga * m * 2;  // (slot ga, slot gb) pairs
    int fa = k, fb = k;
    long long evals = 0;
    __syncthreads();
    for (long long b0 = 0; b0 < total; b0 += XC) {
        if (threadIdx.x < XC) {
            const long long o = b0 + threadIdx.x;
            int cid = -1;
            if (o < total) {
                if (G.unit < 0) {
                    cid = (int)(c_lo + o);
                } else {
                    const int j = t_lo + (int)(o / TC);
                    const int wt = U.p + j * U.parts;
                    const int* ids = wt < U.ntl ? lvl_id + (size_t)main_tile(U, wt) * TC
                                                : ds_id + (size_t)(U.lo_tile + (wt - U.ntl)) * TC;
                    cid = ids[o % TC];
                }
            }
            cid_s[threadIdx.x] = cid;
        }
        __syncthreads();
        // stage: thread t moves float4 (t / XC) of row (t % XC); the transposed stores of a
        // warp fall in 32 different banks
        for (int t = threadIdx.x; t < XC * (m >> 2); t += blockDim.x) {
            const int r = t % XC, j = t / XC;
            const int cid = cid_s[r];
            const float4 x = cid >= 0 ? __ldg((const float4*)(P.v + (size_t)cid * m) + j) : make_float4(0.f, 0.f, 0.f, 0.f);
            cs[(4 * j + 0) * XC + r] = x.x;
            cs[(4 * j + 1) * XC + r] = x.y;
            cs[(4 * j + 2) * XC + r] = x.z;
            cs[(4 * j + 3) * XC + r] = x.w;
        }
        __syncthreads();
        const int cid = cid_s[lane];
        const bool va = ida >= 0 && cid >= 0 && (!P.predecessor || cid < ida);
        const bool vb = idb >= 0 && cid >= 0 && (!P.predecessor || cid < idb);
        // The dot in warp_dots' order, so that a pair's exact distance is the same whichever
        // pass scores it: 32 segments of m/32 elements, each summed in order, combined as
        // the butterfly does (lane offsets 16, 8, 4, 2, 1).  Taking segment rev5(c) at step
        // c turns that tree into a binary counter: pend[L] holds the finished subtree of
        // 2^L segments while bit L of c is set.
        float2 h2 = make_float2(0.f, 0.f), l2 = make_float2(0.f, 0.f);  // (slot ga, slot gb)
        float2 pend_h[5], pend_l[5];
#pragma unroll
        for (int L = 0; L < 5; ++L) pend_h[L] = pend_l[L] = make_float2(0.f, 0.f);
        for (int c = 0; c < 32; ++c) {
            const int seg = (int)(__brev((unsigned)c) >> 27);
            const float* q2s = q2 + seg * per * 2;
            const float* css = cs + (size_t)seg * per * XC + lane;
            h2 = make_float2(0.f, 0.f); l2 = make_float2(0.f, 0.f);
            if (PER > 0) {
#pragma unroll
                for (int t4 = 0; t4 < PER; t4 += 2) {
                    const float4 ab = *(const float4*)(q2s + 2 * t4);  // a[t4], b[t4], a[t4+1], b[t4+1]
                    const float x0 = css[(t4 + 0) * XC], x1 = css[(t4 + 1) * XC];
                    two_sum_acc2(h2, l2, make_float2(ab.x, ab.y), make_float2(x0, x0));
                    two_sum_acc2(h2, l2, make_float2(ab.z, ab.w), make_float2(x1, x1));
                }
            } else {
                for (int t = 0; t < per; ++t) {
                    const float x = css[t * XC];
                    const float2 ab = *(const float2*)(q2s + 2 * t);
                    two_sum_acc2(h2, l2, ab, make_float2(x, x));
                }
            }
            bool placed = false;
#pragma unroll
            for (int L = 0; L < 5; ++L) {
                if (!placed) {
                    if ((c >> L) & 1) {
                        df_combine2(h2, l2, pend_h[L], pend_l[L]);
                    } else {
                        pend_h[L] = h2; pend_l[L] = l2;
                        placed = true;
                    }
                }
            }
        }
        const float ha = h2.x, la = l2.x, hb = h2.y, lb = l2.y;
        const df da = df_fast(ha, la);
        const df db = df_fast(hb, lb);
        const float dista = va ? exact_from_dot(P, ida, cid, da) : 0.f;
        const float distb = vb ? exact_from_dot(P, idb, cid, db) : 0.f;
        evals += __popc(__ballot_sync(0xffffffffu, va)) + __popc(__ballot_sync(0xffffffffu, vb));
        keys_append(ka, fa, k, va, pack_key(dista, cid));
        keys_append(kbb, fb, k, vb, pack_key(distb, cid));
        __syncthreads();
    }
    warp_bitonic_sort(ka, XKB);
    warp_bitonic_sort(kbb, XKB);
    if (ga < G.ng)
        for (int j = lane; j < k; j += 32) partial[((size_t)ibeg[G.g0 + ga] + it.chunk) * k + j] = ka[j];
    if (gb < G.ng)
        for (int j = lane; j < k; j += 32) partial[((size_t)ibeg[G.g0 + gb] + it.chunk) * k + j] = kbb[j];
    if (lane == 0 && P.evals && evals) atomicAdd((unsigned long long*)P.evals, (unsigned long long)evals);
}

// Sparse plain slots: an overflowed slot of a tiny-p query whose candidate source no other
// such slot shares (a small call's part slots) gets whole warps instead of a 16-row group:
// warp per (slot, chunk) item, the survivor pass's warp dots on 32 candidates at a time,
// exact distances lane-parallel, a streaming top-k buffer per warp.
__global__ void __launch_bounds__(256) rescore_warp_kernel(RescoreParams P, const ExhGroup* __restrict__ groups,
                                                           const ExhItem* __restrict__ items, int nitems,
                                                           const int* __restrict__ ibeg, int cand_chunk, int tpc,
                                                           const JobUnit* __restrict__ units,
                                                           const int* __restrict__ lvl_id,
                                                           const int* __restrict__ ds_id,
                                                           unsigned long long* __restrict__ partial) {
    __shared__ unsigned long long wkeys[8][XKB];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * 8 + warp;
    if (w >= nitems) return;
    const ExhItem it = items[w];
    const ExhGroup G = groups[it.group];
    const int m = P.m, k = P.k;
    const int q = P.slot_id[P.full_slots[G.g0]];
    unsigned long long* keys = wkeys[warp];
    for (int i = lane; i < XKB; i += 32) keys[i] = ~0ULL;
    __syncwarp();
    long long c_lo = 0, total = 0;
    int t_lo = 0;
    JobUnit U{};
    if (G.unit < 0) {
        c_lo = (long long)it.chunk * cand_chunk;
        const long long c_hi = G.cend < c_lo + cand_chunk ? G.cend : c_lo + cand_chunk;
        total = c_hi > c_lo ? c_hi - c_lo : 0;
    } else {
        U = units[G.unit];
        const int mine = U.count - U.warm;
        t_lo = it.chunk * tpc;
        const int t_hi = mine < t_lo + tpc ? mine : t_lo + tpc;
        total = t_hi > t_lo ? (long long)(t_hi - t_lo) * TC : 0;
    }
    long long evals = 0;
    if (q >= 0) {
        float vql[32];
        load_query_slice(P.v + (size_t)q * m, m, vql);
        int fill = k;
        for (long long b0 = 0; b0 < total; b0 += 32) {
            const long long o = b0 + lane;
            int cid = -1;
            if (o < total) {
                if (G.unit < 0) {
                    cid = (int)(c_lo + o);
                } else {
                    const int wt = U.p + (t_lo + (int)(o / TC)) * U.parts;
                    const int* ids = wt < U.ntl ? lvl_id + (size_t)main_tile(U, wt) * TC
                                                : ds_id + (size_t)(U.lo_tile + (wt - U.ntl)) * TC;
                    cid = ids[o % TC];
                }
            }
            const bool has = cid >= 0 && !(P.predecessor && cid >= q);
            const unsigned hm = __ballot_sync(0xffffffffu, has);
            if (hm == 0u) continue;
            df mydot = df{0.f, 0.f};
            for (int t = 0; t < 32; t += 4) {
                if (((hm >> t) & 15u) == 0u) continue;
                int cc[4];
                df dd4[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int src = __shfl_sync(0xffffffffu, cid, t + u);
                    cc[u] = (hm >> (t + u)) & 1u ? src : -1;
                }
                warp_dots<4>(P.v, m, cc, vql, dd4);
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (lane == t + u) mydot = dd4[u];
            }
            const float dist = has ? exact_from_dot(P, q, cid, mydot) : 0.f;
            evals += __popc(hm);
            keys_append(keys, fill, k, has, pack_key(dist, cid));
        }
    }
    __syncwarp();
    warp_bitonic_sort(keys, XKB);
    for (int j = lane; j < k; j += 32) partial[((size_t)ibeg[G.g0] + it.chunk) * k + j] = keys[j];
    if (lane == 0 && P.evals && evals) atomicAdd((unsigned long long*)P.evals, (unsigned long long)evals);
}

// ---------------------------------------------------------- filtered exhaustive pass
// Overflowed slots whose residual variance is not tiny (|v_q| / sqrt(p_q) <= kFilterIsq)
// are rescored over their whole candidate source, block by block of FCB = 256
// candidates (one sweep tile), in two steps:
//  F: an FP32 GEMM of the group's FQ = 4 QPT query rows against the block.  A thread
//     holds QPT queries x 4 candidates; the block's rows are staged in K-chunks of 32 by
//     16-byte cp.async into a double buffer.  Each dot is a blocked sum: FMA chains of
//     FLB = 16 terms added into a running total, error <= (FLB + m / FLB + 1) 2^-24
//     |v_q| |v_c| (half the survivor pass's four interleaved chains at m = 256).  The dots
//     go to shared memory; the warp that owns a query row then bounds its 256 pairs
//     (pair_bounds_core) and keeps those whose dl2 reaches the query's threshold tau^2:
//     the query's shared threshold (seeded before the sweep, lowered by every part's
//     heap), then the k-th exact distance seen here plus the seeds' margin for the
//     double-float error.  A pair above tau^2 cannot enter the top k.
//  E: the same warp rescores its kept pairs exactly with the survivor pass's warp dots
//     (the same double-float value for a pair in either pass) into the query's streaming
//     top-k buffer.
// QPT = 8 serves groups of up to 32 slots, QPT = 4 groups of up to 16.
constexpr int FCB = 256;      // candidates per block
constexpr int FKC = 32;       // K-chunk per stage
constexpr int FKP = FKC + 4;  // padded staged row (floats): conflict-free 16-byte reads
constexpr int FLB = 16;       // FMA chain length per partial sum
constexpr int FDP = FCB + 4;  // padded row of the dot matrix (floats)
static_assert(FCB == TC, "a block of the filtered pass is one sweep tile");
__host__ __device__ inline size_t filter_smem_bytes(int m, int qpt) {
    const int fq = 4 * qpt, fqp = fq + 4;
    return sizeof(float) * (2 * FCB * FKP + (size_t)m * fqp) + sizeof(unsigned long long) * fq * XKB + fq * FCB +
           sizeof(float) * (FCB * 8 + 2 * FCB + fq * 16) + sizeof(int) * (FCB + 2 * fq);
}

__device__ __forceinline__ void cp_async16_zfill(void* smem_dst, const void* gsrc, int src_bytes) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gsrc), "r"(src_bytes) : "memory");
}

template <int QPT>
__global__ void __launch_bounds__(256, 1) filter_tile_kernel(RescoreParams P, const ExhGroup* __restrict__ groups,
                                                             const ExhItem* __restrict__ items,
                                                             const int* __restrict__ ibeg, int cand_chunk, int tpc,
                                                             const JobUnit* __restrict__ units,
                                                             const int* __restrict__ lvl_id,
                                                             const int* __restrict__ ds_id,
                                                             unsigned long long* __restrict__ partial) {
    constexpr int FQ = 4 * QPT, FQP = FQ + 4, RPW = FQ / 8;  // query rows, padded row, rows per warp
    static_assert(FQ * FDP <= 2 * FCB * FKP, "the dot matrix reuses the staging buffers");
    extern __shared__ __align__(16) unsigned char fsm[];
    const int m = P.m, k = P.k, d = P.d;
    float* cbuf = (float*)fsm;                                                     // [2][FCB][FKP]
    float* dots = cbuf;                                                            // [FQ][FDP] after the K loop
    float* qsT = cbuf + 2 * FCB * FKP;                                             // [m][FQP]
    unsigned long long* kb = (unsigned long long*)(qsT + (size_t)m * FQP);        // [FQ][XKB]
    unsigned char* plist = (unsigned char*)(kb + FQ * XKB);                       // [FQ][FCB]
    float* cx = (float*)(plist + FQ * FCB);                                        // [8][FCB] (axis-major)
    float* cisp = cx + FCB * 8;
    float* cvn = cisp + FCB;
    float* qc = cvn + FCB;        // [FQ][8]: isq, ed / |v_c|, alk, bek, ale, bee, margin, tau^2
    float* qx = qc + FQ * 8;      // [FQ][8]
    int* cid_s = (int*)(qx + FQ * 8);
    int* qid_s = cid_s + FCB;
    const ExhItem it = items[blockIdx.x];
    const ExhGroup G = groups[it.group];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < FQ) {
        const int q = tid < G.ng ? P.slot_id[P.full_slots[G.g0 + tid]] : -1;
        qid_s[tid] = q;
        float* c = qc + tid * 8;
        if (q >= 0) {
            const float dd = (float)d, ced2 = (dd + 2.f) * 5.97e-8f;
            const float isq = P.isp[q];
            const float A = 2.4e-7f * (P.xmax[q] + __uint_as_float(__ldg(P.xmax_max)));
            c[0] = isq;
            c[1] = (float)(FLB + m / FLB + 1) * 5.97e-8f * P.vn[q];
            c[2] = (6e-8f + 0.5f * ced2 + 0.25f * A * dd) * 1.00001f;
            c[3] = (1e-6f + 0.25f * A) * 1.00001f;
            c[4] = (ced2 + 0.5f * A * dd) * 1.00001f;
            c[5] = 0.5f * A * 1.00001f;
            c[6] = 4e-12f * fminf(isq * __uint_as_float(__ldg(P.isp_max)) * 1.01f, 1e9f) + 1e-12f;
            c[7] = fminf(1.f, __uint_as_float(P.qtau[P.full_slots[G.g0 + tid] / P.parts]));
            for (int a = 0; a < d; ++a) qx[tid * 8 + a] = P.xs[(size_t)q * d + a];
        } else {
            c[7] = -1.f;
        }
    }
    __syncthreads();
    for (int e = tid; e < FQ * m; e += blockDim.x) {
        const int g = e / m, kx = e - g * m;
        const int q = qid_s[g];
        qsT[(size_t)kx * FQP + g] = q >= 0 ? P.v[(size_t)q * m + kx] : 0.f;
    }
    for (int e = tid; e < FQ * XKB; e += blockDim.x) kb[e] = ~0ULL;
    // the item's candidate blocks
    long long c_lo = 0, total = 0;
    int t_lo = 0, nblocks = 0;
    JobUnit U{};
    if (G.unit < 0) {
        c_lo = (long long)it.chunk * cand_chunk;
        const long long c_hi = G.cend < c_lo + cand_chunk ? G.cend : c_lo + cand_chunk;
        total = c_hi > c_lo ? c_hi - c_lo : 0;
        nblocks = (int)((total + FCB - 1) / FCB);
    } else {
        U = units[G.unit];
        const int mine = U.count - U.warm;
        t_lo = it.chunk * tpc;
        const int t_hi = mine < t_lo + tpc ? mine : t_lo + tpc;
        nblocks = t_hi > t_lo ? t_hi - t_lo : 0;
    }
    const int tq = warp >> 1;                    // queries QPT tq .. QPT tq + QPT - 1
    const int tc = ((warp & 1) << 5) | lane;     // candidates tc + 64 j
    const int nk = m / FKC;
    int fill[RPW];
#pragma unroll
    for (int r = 0; r < RPW; ++r) fill[r] = k;
    long long evals = 0;
    for (int b = 0; b < nblocks; ++b) {
        __syncthreads();  // the previous block's ids, rows and dots are no longer read
        {
            int cid = -1;
            if (G.unit < 0) {
                const long long o = (long long)b * FCB + tid;
                if (o < total) cid = (int)(c_lo + o);
            } else {
                const int wt = U.p + (t_lo + b) * U.parts;
                const int* ids = wt < U.ntl ? lvl_id + (size_t)main_tile(U, wt) * TC
                                            : ds_id + (size_t)(U.lo_tile + (wt - U.ntl)) * TC;
                cid = ids[tid];
            }
            cid_s[tid] = cid;
            if (cid >= 0) {
                for (int a = 0; a < d; ++a) cx[a * FCB + tid] = P.xs[(size_t)cid * d + a];
                cisp[tid] = P.isp[cid];
                cvn[tid] = P.vn[cid];
            }
        }
        __syncthreads();
        auto stage = [&](int kc, int bf) {
            float* dst = cbuf + bf * FCB * FKP;
            const int piece = tid & 7;
#pragma unroll
            for (int i = 0; i < FCB / 32; ++i) {
                const int r = (tid >> 3) + 32 * i;
                const int cid = cid_s[r];
                const float* src = P.v + (size_t)(cid >= 0 ? cid : 0) * m + kc * FKC + piece * 4;
                cp_async16_zfill(dst + r * FKP + piece * 4, src, cid >= 0 ? 16 : 0);
            }
            asm volatile("cp.async.commit_group;\n" ::: "memory");
        };
        // running sums of queries (2i, 2i + 1) x candidate j as f32x2 (each component
        // rounds as __fmaf_rn / __fadd_rn do)
        float2 tot[QPT / 2][4];
#pragma unroll
        for (int i = 0; i < QPT / 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) tot[i][j] = make_float2(0.f, 0.f);
        stage(0, 0);
        for (int kc = 0; kc < nk; ++kc) {
            if (kc + 1 < nk) {
                stage(kc + 1, (kc + 1) & 1);
                asm volatile("cp.async.wait_group 1;\n" ::: "memory");
            } else {
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
            }
            __syncthreads();
            const float* cb = cbuf + (kc & 1) * FCB * FKP;
            const float* qb = qsT + (size_t)kc * FKC * FQP + QPT * tq;
#pragma unroll
            for (int h = 0; h < FKC / FLB; ++h) {
                float2 acc[QPT / 2][4];
#pragma unroll
                for (int i = 0; i < QPT / 2; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll
                for (int k4 = 0; k4 < FLB; k4 += 4) {
                    const int kk = h * FLB + k4;
                    float4 x[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) x[j] = *(const float4*)(cb + (tc + 64 * j) * FKP + kk);
#pragma unroll
                    for (int t = 0; t < 4; ++t) {
                        float2 qv[QPT / 2];
#pragma unroll
                        for (int i4 = 0; i4 < QPT; i4 += 4) {
                            const float4 qa = *(const float4*)(qb + (kk + t) * FQP + i4);
                            qv[i4 / 2] = make_float2(qa.x, qa.y); qv[i4 / 2 + 1] = make_float2(qa.z, qa.w);
                        }
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const float xv = t == 0 ? x[j].x : t == 1 ? x[j].y : t == 2 ? x[j].z : x[j].w;
                            const float2 x2 = make_float2(xv, xv);
#pragma unroll
                            for (int i = 0; i < QPT / 2; ++i) acc[i][j] = __ffma2_rn(qv[i], x2, acc[i][j]);
                        }
                    }
                }
#pragma unroll
                for (int i = 0; i < QPT / 2; ++i)
#pragma unroll
                    for (int j = 0; j < 4; ++j) tot[i][j] = __fadd2_rn(tot[i][j], acc[i][j]);
            }
            __syncthreads();  // buffer kc & 1 is free for chunk kc + 2 (and, at the end, for the dots)
        }
#pragma unroll
        for (int i = 0; i < QPT / 2; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                dots[(QPT * tq + 2 * i) * FDP + tc + 64 * j] = tot[i][j].x;
                dots[(QPT * tq + 2 * i + 1) * FDP + tc + 64 * j] = tot[i][j].y;
            }
        __syncthreads();
        // F bounds and E, warp w owns query rows w, w + 8, ...
        for (int r = 0; r < RPW; ++r) {
            const int ql = warp + 8 * r;
            const int q = qid_s[ql];
            if (q < 0) continue;
            const float* c = qc + ql * 8;
            const float tau2 = c[7];
            int nkept = 0;
            for (int c0 = 0; c0 < FCB; c0 += 32) {
                const int cl = c0 + lane;
                const int cid = cid_s[cl];
                bool keep = cid >= 0 && !(P.predecessor && cid >= q);
                if (keep && cid != q) {  // the query itself: d = 0
                    float dl2, du2;
                    pair_bounds_core(P, qx + ql * 8, cx + cl, cisp[cl], dots[ql * FDP + cl],
                                     __fmul_rn(c[1], cvn[cl]), c[0], c[2], c[3], c[4], c[5], dl2, du2, FCB);
                    keep = dl2 <= tau2;
                }
                const unsigned mk = __ballot_sync(0xffffffffu, keep);
                if (keep) plist[ql * FCB + nkept + __popc(mk & ((1u << lane) - 1u))] = (unsigned char)cl;
                nkept += __popc(mk);
            }
            if (nkept == 0) continue;
            __syncwarp();
            unsigned long long* keys = kb + (size_t)ql * XKB;
            float vql[32];
            load_query_slice(P.v + (size_t)q * m, m, vql);
            int fl = fill[0];
#pragma unroll
            for (int rr = 1; rr < RPW; ++rr)
                if (r == rr) fl = fill[rr];
            for (int base = 0; base < nkept; base += 32) {
                const int ci = base + lane;
                const bool has = ci < nkept;
                const int cid = has ? cid_s[plist[ql * FCB + ci]] : -1;
                const int nb = nkept - base < 32 ? nkept - base : 32;
                df mydot = df{0.f, 0.f};
                for (int t = 0; t < nb; t += 4) {
                    int cc[4];
                    df dd4[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const int src = __shfl_sync(0xffffffffu, cid, (t + u) & 31);
                        cc[u] = (t + u) < nb ? src : -1;
                    }
                    warp_dots<4>(P.v, m, cc, vql, dd4);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (lane == t + u) mydot = dd4[u];
                }
                const float dist = has ? exact_from_dot(P, q, cid, mydot) : 0.f;
                evals += nb;
                keys_append(keys, fl, k, has, pack_key(dist, cid));
            }
            // every 16 new entries: sort, keep the k best, tighten tau^2 by the k-th
            if (fl >= k + 16) {
                __syncwarp();
                warp_bitonic_sort(keys, XKB);
                for (int i = k + lane; i < XKB; i += 32) keys[i] = ~0ULL;
                fl = k;
                __syncwarp();
                const unsigned long long kk = keys[k - 1];
                if (kk != ~0ULL) {
                    const float dk = __uint_as_float((unsigned)(kk >> 32));
                    const float t2 = __fadd_ru(__fmul_ru(__fmul_ru(dk, dk), 1.000004f), c[6]);
                    __syncwarp();
                    if (lane == 0) qc[ql * 8 + 7] = fminf(tau2, t2);
                }
            }
#pragma unroll
            for (int rr = 0; rr < RPW; ++rr)
                if (r == rr) fill[rr] = fl;
        }
    }
    __syncthreads();
    for (int r = 0; r < RPW; ++r) {
        const int ql = warp + 8 * r;
        unsigned long long* keys = kb + (size_t)ql * XKB;
        warp_bitonic_sort(keys, XKB);
        if (ql < G.ng)
            for (int j = lane; j < k; j += 32) partial[((size_t)ibeg[G.g0 + ql] + it.chunk) * k + j] = keys[j];
    }
    if (lane == 0 && P.evals && evals) atomicAdd((unsigned long long*)P.evals, (unsigned long long)evals);
}

// Job i of a unit: i < warm: warm-up (heap only) over the part's i-th spiral tile;
// otherwise the part's (i - warm)-th tile, marked when its warm-up already fed its heap.
// The part's main tiles are entries p, p + parts, ... of the tile's list (the level's
// tiles in ascending order, then the dataset tiles).
__global__ void gen_jobs_kernel(const JobUnit* __restrict__ units, Job* __restrict__ jobs) {
    const JobUnit U = units[blockIdx.x];
    for (int i = threadIdx.x; i < U.count; i += blockDim.x) {
        const bool warmup = i < U.warm;
        const int j = warmup ? i : i - U.warm;
        const int w = U.p + j * U.parts;
        int which, ctile;
        if (w < U.ntl) {
            if (warmup) {
                ctile = spiral_tile(U, w);
                which = 2;
            } else {
                ctile = main_tile(U, w);
                // the part's own warm-up already fed this tile to its heaps
                bool warmed = j < U.warm;
                if (U.lin) {
                    const int sw = spiral_index(U, ctile);
                    warmed = sw >= U.p && (sw - U.p) % U.parts == 0 && (sw - U.p) / U.parts < U.warm;
                }
                which = warmed ? 4 : 0;
            }
            which |= U.fast_lvl ? 8 : 0;
        } else {
            ctile = U.lo_tile + (w - U.ntl);
            which = 1 | (ctile < U.ds_fast_end ? 8 : 0);
        }
        jobs[U.off + i] = Job{U.qx, ctile, which, i == 0 ? 1 : 0};
    }
}
__global__ void slot_ids_kernel(const long long* q, long long nq, long long n, int* slot_id,
                                unsigned long long* key_lvl, int* val_lvl, const unsigned long long* hil_key,
                                const unsigned long long* lvl_key, const long long* lvl_meta, int nlevels,
                                int predecessor) {
    long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nq) return;
    long long id = q[i];
    bool ok = id >= 0 && id < n;
    slot_id[i] = ok ? (int)id : -1;
    val_lvl[i] = (int)i;
    unsigned long long kl = 0xFFFFFFFFFFFFFFFFULL;
    if (ok) {
        int li = -1;
        if (!predecessor) {
            li = nlevels - 1;  // whole dataset
        } else {
            for (int l = 0; l < nlevels - 1; ++l)
                if (lvl_meta[3 * l] <= id) li = l;
        }
        if (li >= 0) {
            const long long off = lvl_meta[3 * li + 1], size = lvl_meta[3 * li];
            const unsigned long long key = hil_key[id];
            long long lo = 0, hi = size;  // first row with key >= query key
            while (lo < hi) {
                long long mid = (lo + hi) >> 1;
                if (lvl_key[off + mid] < key) lo = mid + 1; else hi = mid;
            }
            if (lo >= size) lo = size - 1;
            long long band = 0;
            if (predecessor) band = ((id - size) * kBands) / size;  // ids of this level lie in [size, 2 size)
            if (band < 0) band = 0;
            if (band >= kBands) band = kBands - 1;
            const unsigned long long group = (unsigned long long)(li * kBands + band);
            kl = (group << 32) | (unsigned long long)(off + lo);
        } else {
            kl = (0xFFFFFFFEULL << 32) | (unsigned long long)id;  // no level: by id
        }
    }
    key_lvl[i] = kl;
}

// Seeded thresholds.  Any k eligible candidates bound a query's k-th distance, so
// before the sweep each query (one warp) scores exactly the S rows of its level
// that surround its Hilbert position and starts its shared threshold qtau at the
// k-th smallest of those d^2 = 1 - |rho|, plus a margin for the double-float error
// of the exact distance (at most about 2e-12 / sqrt(p_q p_c) in rho).  Without it a
// query far from the centre of a scattered query tile keeps every pair until its
// own heap fills.  Level rows hold ids below the level size, which in predecessor
// mode is at most the query id, so every seed is an eligible candidate.
template <int S>
__global__ void seed_tau_kernel(RescoreParams R, const unsigned long long* __restrict__ key_sorted,
                                const int* __restrict__ val_sorted, long long nq, const int* __restrict__ lvl_id,
                                const long long* __restrict__ lvl_meta, const unsigned* __restrict__ isp_max,
                                unsigned* __restrict__ qtau) {
    const int lane = threadIdx.x & 31;
    const long long w = blockIdx.x * (long long)(blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= nq) return;
    const unsigned long long key = key_sorted[w];
    const unsigned group = (unsigned)(key >> 32);
    if (group >= 0xFFFFFFFEu) return;  // no level
    const int i = val_sorted[w];
    const int q = R.slot_id[i];
    if (q < 0) return;
    const int li = (int)(group / kBands);
    const long long size = lvl_meta[3 * li], off = lvl_meta[3 * li + 1];
    if (size < R.k) return;
    long long start = (long long)(key & 0xFFFFFFFFULL) - off - S / 2;
    if (start > size - S) start = size - S;
    if (start < 0) start = 0;
    const int cnt = size < S ? (int)size : S;
    float vql[32];
    load_query_slice(R.v + (size_t)q * R.m, R.m, vql);
    float dist[S / 32];
#pragma unroll
    for (int r = 0; r < S / 32; ++r) {
        const int cid = r * 32 + lane < cnt ? lvl_id[off + start + r * 32 + lane] : -1;
        df mydot = df{0.f, 0.f};
        for (int t = 0; t < 32; t += 4) {
            int cc[4];
            df dots[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) cc[u] = __shfl_sync(0xffffffffu, cid, t + u);
            warp_dots<4>(R.v, R.m, cc, vql, dots);
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (lane == t + u) mydot = dots[u];
        }
        dist[r] = cid >= 0 ? exact_from_dot(R, q, cid, mydot) : __int_as_float(0x7f800000);
    }
    // k-th smallest distance: bisection over the bit patterns (non-negative floats
    // order as unsigned integers)
    unsigned lo = 0, hi = 0x7f800000u;
    while (lo < hi) {
        const unsigned mid = lo + ((hi - lo) >> 1);
        int c = 0;
#pragma unroll
        for (int r = 0; r < S / 32; ++r) c += __popc(__ballot_sync(0xffffffffu, __float_as_uint(dist[r]) <= mid));
        if (c >= R.k) hi = mid; else lo = mid + 1;
    }
    if (lane == 0 && lo < 0x7f800000u) {
        const float dk = __uint_as_float(lo);
        const float isq = rsqrtf(fmaxf(R.p[q], 1e-30f)) * 1.01f;
        const float margin = 4e-12f * fminf(isq * __uint_as_float(*isp_max) * 1.01f, 1e9f) + 1e-12f;
        const float t2 = fminf(__fadd_ru(__fmul_ru(__fmul_ru(dk, dk), 1.000004f), margin), 1.f);
        atomicMin(&qtau[i], __float_as_uint(t2));
    }
}

__global__ void max_bits_kernel(const float* __restrict__ x, long long n, unsigned* __restrict__ out) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) atomicMax(out, __float_as_uint(fabsf(x[i])));
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

// Candidate parts: A row (t*parts + p)*TQ + r repeats A row t*TQ + r for part p,
// whose slot is s*parts + p.
__global__ void expand_parts_kernel(const int* a_slot, const int* rowmap, long long rows_q, int parts, int* a_slot_x,
                                    int* rowmap_x) {
    const long long r2 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r2 >= rows_q * parts) return;
    const long long t2 = r2 / TQ;
    const int r = (int)(r2 - t2 * TQ);
    const long long t = t2 / parts;
    const int pp = (int)(t2 - t * parts);
    const long long r1 = t * TQ + r;
    const int sl = a_slot[r1];
    a_slot_x[r2] = sl >= 0 ? sl * parts + pp : -1;
    rowmap_x[r2] = rowmap[r1];
}
__global__ void fill_u32_kernel(unsigned* a, long long n, unsigned v) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}
__global__ void expand_slots_kernel(const int* slot_id, long long nq, int parts, int* slot_id_x) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < nq * parts) slot_id_x[i] = slot_id[i / parts];
}
// One warp per query: the exact top-k over its parts.  The parts cover disjoint
// candidates (an overflowed part was rescored over its own candidates only), so
// their lists are k-way merged (lane p holds the head of part p).
__global__ void merge_parts_kernel(const long long* __restrict__ pidx, const float* __restrict__ pdist,
                                   long long nq, int parts, int k,
                                   long long* __restrict__ out_idx, float* __restrict__ out_dist) {
    const long long q = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (q >= nq) return;
    const float kInf = __int_as_float(0x7f800000);
    int pos = 0;
    float hd = kInf;
    long long hi = LLONG_MAX;
    auto load = [&]() {
        hd = kInf;
        hi = LLONG_MAX;
        if (lane < parts && pos < k) {
            const long long i = pidx[(q * parts + lane) * k + pos];
            if (i >= 0) { hi = i; hd = pdist[(q * parts + lane) * k + pos]; }
        }
    };
    load();
    for (int j = 0; j < k; ++j) {
        float bd = hd;
        long long bi = hi;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float od = __shfl_xor_sync(0xffffffffu, bd, o);
            const long long oi = __shfl_xor_sync(0xffffffffu, bi, o);
            if (od < bd || (od == bd && oi < bi)) { bd = od; bi = oi; }
        }
        if (lane == 0) {
            const bool pad = bi == LLONG_MAX;
            out_idx[q * k + j] = pad ? -1LL : bi;
            out_dist[q * k + j] = pad ? CT_FLT_MAX : bd;
        }
        if (bi != LLONG_MAX && hi == bi) { ++pos; load(); }
    }
}

static inline unsigned grid_for(long long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

static float err_coef_for(int m) {
    const double u2 = 1.0 / 65536.0;
    return (float)(3.1 * u2 + (3.0 * m / 16.0 + 17.0) * std::ldexp(1.0, -22));
}

static int pick_stages(int k) {
    for (int ns = STAGES; ns >= 2; --ns)
        if (smem_layout(k, ns).total <= 232448) return ns;
    return 0;
}

// ncta persistent CTAs: each claims units (dynamic schedule) or runs jobs
// [cta_job_begin[c], cta_job_begin[c+1]) (static schedule, the diagnostic launch).
static cudaError_t launch_sweep(const MMAParams& P, int mode, int ncta, cudaStream_t st) {
    if (ncta <= 0) return cudaSuccess;
    const size_t smem = smem_layout(P.k, P.nstages).total;
    cudaError_t e;
    if (mode == MODE_DEBUG) {
        e = cudaFuncSetAttribute(screen_sweep_kernel<MODE_DEBUG, 8, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        screen_sweep_kernel<MODE_DEBUG, 8, 0><<<ncta, kThreads, smem, st>>>(P);
        return cudaGetLastError();
    }
    void (*fn)(MMAParams) = P.d <= 4 ? (P.kernel_type == 0 ? screen_sweep_kernel<MODE_SWEEP, 4, 0> : screen_sweep_kernel<MODE_SWEEP, 4, 1>)
                                     : (P.kernel_type == 0 ? screen_sweep_kernel<MODE_SWEEP, 8, 0> : screen_sweep_kernel<MODE_SWEEP, 8, 1>);
    e = cudaFuncSetAttribute((const void*)fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    fn<<<ncta, kThreads, smem, st>>>(P);
    return cudaGetLastError();
}

}  // namespace screen
}  // namespace ct

using namespace ct::screen;

void ct_tree::release_screen() {
    State* S = (State*)screen;
    if (!S) return;
    cudaFree(S->hil_order); cudaFree(S->hil_key); cudaFree(S->ds_hi); cudaFree(S->ds_lo); cudaFree(S->b_id_ds);
    cudaFree(S->lvl_hi); cudaFree(S->lvl_lo); cudaFree(S->lvl_id); cudaFree(S->lvl_key); cudaFree(S->lvl_meta);
    cudaFree(S->vn); cudaFree(S->isp); cudaFree(S->xmax); cudaFree(S->inv_ls64); cudaFree(S->status);
    cudaFree(S->inv_ls_df); cudaFree(S->isp_max); cudaFree(S->rec_ds); cudaFree(S->rec_lvl); cudaFree(S->xmax_max);
    cudaFree(S->bounds);
    if (S->slab_done) cudaEventDestroy(S->slab_done);
    delete S;
    screen = nullptr;
}

// Build the screened-form operands once per tree (lazily, on first use):
// dataset-order blocked hi/lo V for the main sweep, the Hilbert order and keys,
// and the threshold levels (prefixes 2^10, 2^11, ... < n and the whole set),
// each in Hilbert order, concatenated into one blocked matrix.
static int screen_prepare(ct_tree* T, cudaStream_t st) {
    if (T->screen) return CT_OK;
    State* S = new State();
    T->screen = S;
    const long long n = T->n;
    S->n = n;
    S->rows_pad = ((n + TC - 1) / TC) * TC;
    const int m = T->m;
    for (int j = kFirstPrefixLog2; (1LL << j) < n; ++j) {
        Level L; L.size = 1LL << j; S->levels.push_back(L);
    }
    { Level L; L.size = n; S->levels.push_back(L); }
    long long off = 0;
    for (auto& L : S->levels) { L.row_off = off; L.rows_pad = ((L.size + TC - 1) / TC) * TC; off += L.rows_pad; }
    S->lvl_rows = off;
    cudaError_t e = cudaSuccess;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMalloc(p, bytes ? bytes : 16); };
    A((void**)&S->hil_order, sizeof(int) * n);
    A((void**)&S->hil_key, sizeof(unsigned long long) * (n + T->slab_rows));
    A((void**)&S->ds_hi, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->ds_lo, sizeof(bf16) * S->rows_pad * m);
    A((void**)&S->b_id_ds, sizeof(int) * S->rows_pad);
    A((void**)&S->lvl_hi, sizeof(bf16) * S->lvl_rows * m);
    A((void**)&S->lvl_lo, sizeof(bf16) * S->lvl_rows * m);
    A((void**)&S->lvl_id, sizeof(int) * S->lvl_rows);
    A((void**)&S->lvl_key, sizeof(unsigned long long) * S->lvl_rows);
    A((void**)&S->lvl_meta, sizeof(long long) * 3 * S->levels.size());
    const long long rows_q = n + T->slab_rows;  // per-row scalars cover the query slab
    A((void**)&S->vn, sizeof(float) * rows_q);
    A((void**)&S->isp, sizeof(float) * rows_q);
    A((void**)&S->xmax, sizeof(float) * rows_q);
    A((void**)&S->isp_max, sizeof(unsigned));
    A((void**)&S->xmax_max, sizeof(unsigned));
    A((void**)&S->rec_ds, sizeof(float) * RT * (S->rows_pad / TC));
    A((void**)&S->rec_lvl, sizeof(float) * RT * (S->lvl_rows / TC));
    A((void**)&S->inv_ls64, sizeof(double) * 64);
    A((void**)&S->inv_ls_df, sizeof(float) * 128);
    A((void**)&S->status, sizeof(int));
    A((void**)&S->bounds, sizeof(double) * 2 * 64);
    if (e == cudaSuccess && T->slab_rows > 0) {
        e = cudaEventCreateWithFlags(&S->slab_done, cudaEventDisableTiming);
        S->slab_cap = T->slab_rows;
    }
    if (e != cudaSuccess) return T->set_err(CT_ERR_NOMEM, "screen prep allocation: %s", cudaGetErrorString(e));
    e = ct::compute_order(T->coords_raw, n, T->d, 1, S->hil_order, st, S->hil_key, S->bounds);
    std::vector<int> order_h(n);
    std::vector<unsigned long long> key_h(n);
    if (e == cudaSuccess) {
        iota_kernel<<<grid_for(S->rows_pad), 256, 0, st>>>(S->b_id_ds, S->rows_pad, n);
        split_blocked_kernel<<<152 * 8, 256, 0, st>>>(T->vnat, m, S->b_id_ds, S->rows_pad, S->ds_hi, S->ds_lo);
        point_scalars_kernel<<<grid_for(n), 256, 0, st>>>(T->vnat, T->p, T->xs, n, m, T->d, S->vn, S->isp, S->xmax);
        e = cudaMemsetAsync(S->isp_max, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(S->xmax_max, 0, sizeof(unsigned), st);
        if (e == cudaSuccess) max_bits_kernel<<<grid_for(n), 256, 0, st>>>(S->isp, n, S->isp_max);
        if (e == cudaSuccess) max_bits_kernel<<<grid_for(n), 256, 0, st>>>(S->xmax, n, S->xmax_max);
        if (e == cudaSuccess) e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(order_h.data(), S->hil_order, sizeof(int) * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(key_h.data(), S->hil_key, 8 * n, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return T->set_err(CT_ERR_CUDA, "screen prep: %s", cudaGetErrorString(e));
    // level rows: the Hilbert order filtered to ids < size (stable, so still key-sorted)
    std::vector<int> lid(S->lvl_rows, -1);
    std::vector<unsigned long long> lkey(S->lvl_rows, ~0ULL);
    std::vector<long long> meta;
    for (const auto& L : S->levels) {
        long long r = L.row_off;
        for (long long i = 0; i < n; ++i) {
            int id = order_h[i];
            if (id < L.size) { lid[r] = id; lkey[r] = key_h[id]; ++r; }
        }
        meta.push_back(L.size); meta.push_back(L.row_off); meta.push_back(L.rows_pad);
    }
    e = cudaMemcpyAsync(S->lvl_id, lid.data(), sizeof(int) * S->lvl_rows, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S->lvl_key, lkey.data(), 8 * S->lvl_rows, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(S->lvl_meta, meta.data(), sizeof(long long) * meta.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        split_blocked_kernel<<<152 * 8, 256, 0, st>>>(T->vnat, m, S->lvl_id, S->lvl_rows, S->lvl_hi, S->lvl_lo);
        const float ec = err_coef_for(m);
        build_records_kernel<<<grid_for(S->rows_pad), 256, 0, st>>>(S->b_id_ds, S->rows_pad, T->xs, T->d, S->vn,
                                                                    S->isp, S->xmax, ec, S->rec_ds);
        build_records_kernel<<<grid_for(S->lvl_rows), 256, 0, st>>>(S->lvl_id, S->lvl_rows, T->xs, T->d, S->vn,
                                                                    S->isp, S->xmax, ec, S->rec_lvl);
        build_group_records_kernel<<<grid_for(S->rows_pad / (TC / 2)), 256, 0, st>>>(S->b_id_ds, S->rows_pad, T->xs,
                                                                                    T->d, S->vn, S->isp, ec, S->rec_ds);
        build_group_records_kernel<<<grid_for(S->lvl_rows / (TC / 2)), 256, 0, st>>>(S->lvl_id, S->lvl_rows, T->xs,
                                                                                     T->d, S->vn, S->isp, ec, S->rec_lvl);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        double ils[64];
        for (int i = 0; i < T->d; ++i) ils[i] = T->inv_ls_host64[i];
        e = cudaMemcpyAsync(S->inv_ls64, ils, sizeof(double) * T->d, cudaMemcpyHostToDevice, st);
        float ils_df[128];
        for (int i = 0; i < T->d; ++i) {
            ils_df[2 * i] = (float)ils[i];
            ils_df[2 * i + 1] = (float)(ils[i] - (double)ils_df[2 * i]);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(S->inv_ls_df, ils_df, sizeof(float) * 2 * T->d, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(int), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // host vectors above go out of scope
    }
    if (e != cudaSuccess) return T->set_err(CT_ERR_CUDA, "screen prep: %s", cudaGetErrorString(e));
    return CT_OK;
}

int ct_tree::knn_screened(const int64_t* q_ids, int64_t nq, int k, int predecessor, int64_t* out_idx, float* out_dist,
                          ct_stats* stats, cudaStream_t st, long long id_limit) {
    if (d > kMaxD) return set_err(CT_ERR_UNSUPPORTED, "screened form supports d <= %d (got %d)", kMaxD, d);
    if (m % KC != 0 || m > 1024) return set_err(CT_ERR_UNSUPPORTED, "screened form needs m %% 32 == 0 and m <= 1024 (got %d)", m);
    if (k > kMaxK) return set_err(CT_ERR_UNSUPPORTED, "screened form supports k <= %d (got %d)", kMaxK, k);
    const int nstages = pick_stages(k);
    if (nstages == 0) return set_err(CT_ERR_UNSUPPORTED, "screened form: k=%d does not fit shared memory", k);
    int rc = screen_prepare(this, st);
    if (rc != CT_OK) return rc;
    State* S = (State*)screen;
    const long long rows_q = ((nq + TQ - 1) / TQ) * TQ;
    const long long nqt = rows_q / TQ;
    const int nlev = (int)S->levels.size();
    cudaError_t e = cudaSuccess;
    const bool timing = ct::timing_enabled();
    cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (timing) {
        for (int i = 0; i < 6; ++i) cudaEventCreate(&ev[i]);
        cudaEventRecord(ev[0], st);
    }
    long long launches = 0;
    // ---- per-call buffers
    int *slot_id = nullptr, *val_lvl = nullptr, *vtmp = nullptr;
    unsigned long long *key_lvl = nullptr, *ktmp = nullptr;
    unsigned* hist = nullptr;
    int *a_slot_lvl = nullptr, *rowmap_lvl = nullptr;
    int *a_slot_x = nullptr, *rowmap_x = nullptr, *slot_id_x = nullptr;  // part-expanded (parts > 1)
    bf16 *al_hi = nullptr, *al_lo = nullptr;
    float* survb = nullptr;
    int *surv = nullptr, *surv_cnt = nullptr, *full_list = nullptr, *nfull_d = nullptr, *unit_counter = nullptr;
    int2* unit_jobs_d = nullptr;
    long long* part_idx = nullptr;
    float* part_dist = nullptr;
    long long* evals_d = nullptr;
    unsigned* qtau = nullptr;
    Job* jobs = nullptr;
    JobUnit* units_d = nullptr;
    const int nbh = ct::radix_num_blocks(nq);
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMallocAsync(p, bytes ? bytes : 16, st); };
    A((void**)&slot_id, sizeof(int) * nq);
    A((void**)&val_lvl, sizeof(int) * nq); A((void**)&vtmp, sizeof(int) * nq);
    A((void**)&key_lvl, 8 * nq); A((void**)&ktmp, 8 * nq);
    A((void**)&hist, sizeof(unsigned) * 256 * (size_t)nbh);
    A((void**)&a_slot_lvl, sizeof(int) * rows_q);
    A((void**)&rowmap_lvl, sizeof(int) * rows_q);
    A((void**)&nfull_d, sizeof(int));
    A((void**)&evals_d, sizeof(long long));
    A((void**)&qtau, sizeof(unsigned) * nq);
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "screened form allocation: %s", cudaGetErrorString(e));
    fill_u32_kernel<<<grid_for(nq), 256, 0, st>>>(qtau, nq, 0x3f800000u);  // tau^2 = 1
    ++launches;

    slot_ids_kernel<<<grid_for(nq), 256, 0, st>>>((const long long*)q_ids, nq, id_limit > 0 ? id_limit : n,
                                                 slot_id, key_lvl, val_lvl,
                                                 S->hil_key, S->lvl_key, S->lvl_meta, nlev, predecessor ? 1 : 0);
    ++launches;
    bool in_tmp = false;
    const int kb_lvl = 64;
    launches += ct::radix_sort_launches(nq, kb_lvl) + 2;
    e = ct::radix_sort_pairs(key_lvl, val_lvl, ktmp, vtmp, nq, kb_lvl, hist, nullptr, 0, st, &in_tmp);
    if (e == cudaSuccess && in_tmp) { e = cudaMemcpyAsync(val_lvl, vtmp, sizeof(int) * nq, cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(key_lvl, ktmp, 8 * nq, cudaMemcpyDeviceToDevice, st); }
    if (e == cudaSuccess) {
        arows_kernel<<<grid_for(rows_q), 256, 0, st>>>(val_lvl, nq, rows_q, slot_id, a_slot_lvl, rowmap_lvl);
        e = cudaGetLastError();
    }
    // seeded thresholds, when scoring S candidates per query costs less than the
    // exhaustive rescoring of a few overflowed queries would
    const int seed_s = k <= 32 ? 64 : 128;
    const bool seeded = (long long)seed_s * nq <= 16LL * n;
    if (e == cudaSuccess && seeded) {
        RescoreParams Rs{};
        Rs.v = vnat; Rs.m = m; Rs.coords = coords_raw; Rs.d = d; Rs.inv_ls_df = S->inv_ls_df; Rs.p = p;
        Rs.var = var; Rs.kernel_type = kernel_type; Rs.predecessor = predecessor ? 1 : 0; Rs.n = n;
        Rs.slot_id = slot_id; Rs.nslots = nq; Rs.k = k;
        const unsigned grid = (unsigned)((nq + 7) / 8);
        if (seed_s == 64)
            seed_tau_kernel<64><<<grid, 256, 0, st>>>(Rs, key_lvl, val_lvl, nq, S->lvl_id, S->lvl_meta, S->isp_max, qtau);
        else
            seed_tau_kernel<128><<<grid, 256, 0, st>>>(Rs, key_lvl, val_lvl, nq, S->lvl_id, S->lvl_meta, S->isp_max, qtau);
        e = cudaGetLastError();
        ++launches;
    }
    std::vector<unsigned long long> hk_lvl(nq);
    std::vector<int> hrow_id(rows_q);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hk_lvl.data(), key_lvl, 8 * nq, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hrow_id.data(), rowmap_lvl, sizeof(int) * rows_q, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "screened form setup: %s", cudaGetErrorString(e));

    // ---- per query tile: its candidate tiles nearest-first.  Tile t sweeps the
    // level's Hilbert tiles in a spiral around its queries' position (cc, then
    // cc+1, cc-1, cc+2, ... clipped to the level), then in predecessor mode the
    // dataset tiles [lo_tile, hi_tile) that hold ids beyond the level.
    struct TileSpec {
        int cc, t0, ntl, lo_tile, hi_tile;
        long long lvl_size, min_q;  // the spiral level's size; the tile's smallest query id
    };
    std::vector<TileSpec> spec(nqt, TileSpec{0, 0, 0, 0, 0, 0, 0});
    std::vector<char> busy(nqt, 0);
    const long long n_ds_tiles = S->rows_pad / TC;
    for (long long t = 0; t < nqt; ++t) {
        long long maxq = -1, minq = LLONG_MAX;
        for (long long r = t * TQ; r < (t + 1) * TQ; ++r) {
            maxq = std::max<long long>(maxq, hrow_id[r]);
            if (hrow_id[r] >= 0) minq = std::min<long long>(minq, hrow_id[r]);
        }
        if (maxq < 0) continue;  // no valid query in this tile
        long long r = std::min<long long>(t * TQ + TQ / 2, nq - 1);
        auto row_of = [&](long long rr) -> long long {
            unsigned long long key = hk_lvl[rr];
            if ((key >> 32) >= 0xFFFFFFFEULL) return -1;
            return (long long)(key & 0xFFFFFFFFULL);
        };
        long long row = row_of(r);
        if (row < 0) row = row_of(t * TQ);
        int li = -1;
        if (row >= 0)
            for (int l = 0; l < nlev; ++l)
                if (row >= S->levels[l].row_off && row < S->levels[l].row_off + S->levels[l].rows_pad) li = l;
        TileSpec& sp = spec[t];
        sp.min_q = minq;
        if (li >= 0) {
            const Level& L = S->levels[li];
            sp.t0 = (int)(L.row_off / TC);
            sp.ntl = (int)(L.rows_pad / TC);
            sp.cc = (int)std::min<long long>(std::max<long long>(row / TC, sp.t0), sp.t0 + sp.ntl - 1);
            sp.lvl_size = L.size;
        }
        if (predecessor) {
            // ids >= the level size are not in the level: sweep them in dataset order
            sp.lo_tile = (int)((li >= 0 && li < nlev - 1) ? S->levels[li].size / TC : (li == nlev - 1 ? n_ds_tiles : 0));
            sp.hi_tile = (int)std::min((maxq + TC - 1) / TC, n_ds_tiles);
            if (sp.hi_tile < sp.lo_tile) sp.hi_tile = sp.lo_tile;
        }
        busy[t] = (sp.ntl + sp.hi_tile - sp.lo_tile) > 0;
    }
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // Candidate parts: with fewer query tiles than SMs, each query tile's candidate
    // tiles are dealt round-robin into `parts` disjoint parts, each searched as its own
    // slot (own A rows, heap and survivor lists); the parts' exact top-k lists are
    // merged at the end.  A part's threshold bounds the k-th distance within the
    // part, so its survivors still contain the part's true top k.
    long long busy_tiles = 0, max_jobs = 0;
    for (long long t = 0; t < nqt; ++t)
        if (busy[t]) { ++busy_tiles; max_jobs = std::max<long long>(max_jobs, spec[t].ntl + spec[t].hi_tile - spec[t].lo_tile); }
    int parts = 1;
    if (busy_tiles > 0 && busy_tiles < sms) {
        parts = (int)std::min<long long>(32, sms / busy_tiles);
        parts = (int)std::max<long long>(1, std::min<long long>(parts, max_jobs / 8));
    }
    const long long nslots = nq * parts;
    // Survivor lists per slot: kSurvCap by default, at most RBUF (the survivor pass holds a
    // slot's survivors in shared memory); CT_SCREEN_SURVIVOR_CAP lowers it.  A slot that
    // overflows is rescored exhaustively.
    int half_cap = kSurvCap / 2;
    if (const char* env = std::getenv("CT_SCREEN_SURVIVOR_CAP")) {
        const long long want = std::atoll(env) / 2;
        half_cap = (int)std::max<long long>(32, std::min<long long>(want, RBUF / 2));
    }
    const long long rows_x = rows_q * parts;
    // Units (query tile, part): a heap-only warm-up over the part's first level tiles,
    // then every tile of the part (every parts-th of the tile's list) with survivors kept.
    std::vector<JobUnit> units;
    for (long long t = 0; t < nqt; ++t) {
        if (!busy[t]) continue;
        const TileSpec& sp = spec[t];
        const int nJ = sp.ntl + sp.hi_tile - sp.lo_tile;
        for (int pp = 0; pp < parts; ++pp) {
            const int mine = nJ > pp ? (nJ - pp + parts - 1) / parts : 0;
            if (mine == 0) continue;
            const int nlev_mine = sp.ntl > pp ? (sp.ntl - pp + parts - 1) / parts : 0;
            // seeded queries start from a tight threshold: two warm-up tiles fill the heaps
            const int warm_cap = seeded ? 2 : kWarmTiles;
            const int warm = std::min(parts > 1 ? std::max(1, std::min(warm_cap, nlev_mine / 4)) : warm_cap,
                                      nlev_mine);
            JobUnit u;
            u.qx = (int)(t * parts + pp); u.p = pp; u.parts = parts;
            u.cc = sp.cc; u.t0 = sp.t0; u.ntl = sp.ntl; u.lo_tile = sp.lo_tile;
            u.warm = warm; u.count = warm + mine; u.off = 0;
            u.fast_lvl = (sp.ntl > 0 && sp.lvl_size <= sp.min_q) ? 1 : 0;
            u.ds_fast_end = (int)std::min<long long>(sp.min_q / TC, (long long)INT_MAX);
            // one-part calls sweep the level in ascending order after the warm-up (units of a
            // level share its tiles in L2: 510 -> 422 GB of DRAM reads per sweep at N=262144);
            // split calls keep the spiral (their trees fit in L2 and nearest-first order keeps
            // their part thresholds tight)
            u.lin = parts == 1 ? 1 : 0;
            units.push_back(u);
        }
    }
    // Units are claimed dynamically by the persistent CTAs, largest first (a list
    // schedule in longest-processing-time order): a CTA whose units run fast takes more.
    std::vector<int> order(units.size());
    for (size_t i = 0; i < units.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return units[a].count > units[b].count; });
    const int ncta = (int)std::min<long long>((long long)sms, (long long)order.size());
    std::vector<JobUnit> flat_units;
    std::vector<int2> unit_jobs_h;
    long long njobs = 0;
    for (int u : order) {
        JobUnit x = units[u];
        x.off = njobs;
        unit_jobs_h.push_back(make_int2((int)njobs, x.count));
        njobs += x.count;
        flat_units.push_back(x);
    }
    const long long pairs_main = njobs * TQ * TC;  // every job runs its MMAs
    // part-expanded slots and A rows, the A operand, survivor lists
    const int* a_slot_use = a_slot_lvl;
    const int* rowmap_use = rowmap_lvl;
    const int* slot_id_use = slot_id;
    if (parts > 1) {
        A((void**)&a_slot_x, sizeof(int) * rows_x);
        A((void**)&rowmap_x, sizeof(int) * rows_x);
        A((void**)&slot_id_x, sizeof(int) * nslots);
        A((void**)&part_idx, sizeof(long long) * nslots * k);
        A((void**)&part_dist, sizeof(float) * nslots * k);
        if (e == cudaSuccess) {
            expand_parts_kernel<<<grid_for(rows_x), 256, 0, st>>>(a_slot_lvl, rowmap_lvl, rows_q, parts, a_slot_x, rowmap_x);
            expand_slots_kernel<<<grid_for(nslots), 256, 0, st>>>(slot_id, nq, parts, slot_id_x);
            e = cudaGetLastError();
            launches += 2;
        }
        a_slot_use = a_slot_x; rowmap_use = rowmap_x; slot_id_use = slot_id_x;
    }
    A((void**)&al_hi, sizeof(bf16) * rows_x * m); A((void**)&al_lo, sizeof(bf16) * rows_x * m);
    A((void**)&surv, sizeof(int) * nslots * 2 * (size_t)half_cap);
    A((void**)&survb, sizeof(float) * nslots * 2 * (size_t)half_cap);
    A((void**)&surv_cnt, sizeof(int) * 2 * nslots);
    A((void**)&full_list, sizeof(int) * nslots);
    A((void**)&jobs, sizeof(Job) * (njobs + 1));
    A((void**)&units_d, sizeof(JobUnit) * (flat_units.size() + 1));
    A((void**)&unit_jobs_d, sizeof(int2) * (unit_jobs_h.size() + 1));
    A((void**)&unit_counter, sizeof(int));
    if (e != cudaSuccess) return set_err(CT_ERR_NOMEM, "screened form allocation: %s", cudaGetErrorString(e));
    split_blocked_kernel<<<152 * 8, 256, 0, st>>>(vnat, m, rowmap_use, rows_x, al_hi, al_lo);
    ++launches;
    if (e == cudaSuccess && !flat_units.empty()) {
        e = cudaMemcpyAsync(units_d, flat_units.data(), sizeof(JobUnit) * flat_units.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) {
            gen_jobs_kernel<<<(unsigned)flat_units.size(), 128, 0, st>>>(units_d, jobs);
            e = cudaGetLastError();
            ++launches;
        }
    }
    if (e == cudaSuccess && !unit_jobs_h.empty())
        e = cudaMemcpyAsync(unit_jobs_d, unit_jobs_h.data(), sizeof(int2) * unit_jobs_h.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(unit_counter, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(surv_cnt, 0, sizeof(int) * 2 * nslots, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(nfull_d, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(evals_d, 0, sizeof(long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(S->status, 0, sizeof(int), st);
    // ---- sweep
    if (timing) cudaEventRecord(ev[1], st);
    if (timing) cudaEventRecord(ev[2], st);
    MMAParams P{};
    P.a_hi = al_hi; P.a_lo = al_lo; P.a_groups = rows_x / 8;
    P.b_hi[0] = S->lvl_hi; P.b_lo[0] = S->lvl_lo; P.b_groups[0] = S->lvl_rows / 8; P.b_id[0] = S->lvl_id;
    P.b_hi[1] = S->ds_hi; P.b_lo[1] = S->ds_lo; P.b_groups[1] = S->rows_pad / 8; P.b_id[1] = S->b_id_ds;
    P.m = m; P.jobs = jobs; P.cta_job_begin = nullptr;
    P.unit_jobs = unit_jobs_d; P.nunits = (int)unit_jobs_h.size(); P.unit_counter = unit_counter;
    P.a_slot = a_slot_use; P.slot_id = slot_id_use;
    P.xs = xs; P.d = d; P.vn = S->vn; P.isp = S->isp; P.xmax = S->xmax;
    P.var = var; P.kernel_type = kernel_type; P.predecessor = predecessor ? 1 : 0;
    P.err_coef = err_coef_for(m); P.k = k; P.nstages = nstages;
    P.surv = surv; P.surv_cnt = surv_cnt; P.half_cap = half_cap; P.status = S->status; P.survb = survb;
    P.qtau = qtau; P.parts = parts;
    P.rec[0] = S->rec_lvl; P.rec[1] = S->rec_ds; P.xmax_max = S->xmax_max;
    if (e == cudaSuccess) { e = launch_sweep(P, MODE_SWEEP, ncta, st); ++launches; }
    if (timing) cudaEventRecord(ev[3], st);
    // ---- rescoring (into the part lists when parts > 1)
    RescoreParams R{};
    R.v = vnat; R.m = m; R.coords = coords_raw; R.d = d; R.inv_ls_df = S->inv_ls_df; R.p = p;
    R.var = var; R.kernel_type = kernel_type; R.predecessor = predecessor ? 1 : 0; R.n = n;
    R.slot_id = slot_id_use; R.nslots = nslots; R.surv = surv; R.surv_cnt = surv_cnt; R.half_cap = half_cap;
    R.survb = survb;
    R.full_slots = full_list;
    R.nfull = 0; R.chunk = 4096;
    R.k = k; R.evals = evals_d;
    R.order = val_lvl; R.parts = parts;
    R.xs = xs; R.vn = S->vn; R.isp = S->isp; R.xmax = S->xmax; R.xmax_max = S->xmax_max; R.isp_max = S->isp_max;
    R.qtau = qtau;
    R.out_idx = parts > 1 ? part_idx : (long long*)out_idx;
    R.out_dist = parts > 1 ? part_dist : out_dist;
    const int rwpb = 8;
    const size_t rsmem = sizeof(unsigned long long) * RBUF * rwpb;
    int smem_optin = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    const size_t fsmem8 = filter_smem_bytes(m, 8), fsmem4 = filter_smem_bytes(m, 4);
    const bool can_filter = m <= 1024 && fsmem8 <= (size_t)smem_optin;
    const size_t ssmem = (sizeof(unsigned long long) + sizeof(float)) * RBUF * rwpb;  // survivor pass
    if (e == cudaSuccess) e = cudaFuncSetAttribute(rescore_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ssmem);
    // The overflow list first: the exhaustive pass is planned on the host and runs on side
    // streams while the survivor pass runs on the call's stream.
    int nfull = 0, status = 0;
    long long exh_pairs = 0;  // candidates of the exhaustive pass (part tiles count whole tiles)
    cudaEvent_t ev_ovf = nullptr;
    if (e == cudaSuccess) {
        collect_overflow_kernel<<<grid_for(nslots), 256, 0, st>>>(surv_cnt, nslots, half_cap, slot_id_use, S->isp, S->vn,
                                                                    can_filter ? 1 : 0, full_list, nfull_d);
        e = cudaGetLastError();
        ++launches;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nfull, nfull_d, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&status, S->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_ovf, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(ev_ovf, st);
    if (e == cudaSuccess) {
        rescore_kernel<<<(unsigned)((nslots + rwpb - 1) / rwpb), 32 * rwpb, ssmem, st>>>(R);
        e = cudaGetLastError();
        ++launches;
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(ev_ovf);
    ExhGroup* groups_d = nullptr;
    ExhItem* xitems_d = nullptr;
    int* item_begin_d = nullptr;
    unsigned long long* partial = nullptr;
    cudaStream_t aux[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaEvent_t ev_aux[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    if (e == cudaSuccess && nfull > 0) {
        int prio = 0;
        cudaStreamGetPriority(st, &prio);
        for (auto& a : aux)
            if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&a, cudaStreamNonBlocking, prio);
        for (auto& v : ev_aux)
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
        cudaStream_t x0 = aux[0];
        if (e == cudaSuccess) e = cudaStreamWaitEvent(x0, ev_ovf, 0);
        auto AX = [&](void** ptr, size_t bytes) { if (e == cudaSuccess) e = cudaMallocAsync(ptr, bytes ? bytes : 16, x0); };
        // Group the overflowed slots that share a candidate source and split each group's
        // source into chunks.  Four kinds: plain (tiny p; 5..XQ slots per group), filtered
        // groups of 17..32 slots (QPT = 8) and of up to 16 (QPT = 4), and plain slots in
        // groups of up to 4, split into one warp item per slot and chunk.
        const long long target_items = (long long)sms * 4;
        std::vector<int> fl(nfull), sid(nslots);
        if (e == cudaSuccess) e = cudaMemcpyAsync(fl.data(), full_list, sizeof(int) * nfull, cudaMemcpyDeviceToHost, x0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(sid.data(), slot_id_use, sizeof(int) * nslots, cudaMemcpyDeviceToHost, x0);
        std::vector<int> sorted_q;
        if (parts > 1) {
            sorted_q.resize(nq);
            if (e == cudaSuccess) e = cudaMemcpyAsync(sorted_q.data(), val_lvl, sizeof(int) * nq, cudaMemcpyDeviceToHost, x0);
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(x0);
        // fl entries carry bit 31 for slots of the filtered pass until they are grouped
        auto slot_of = [](int v) { return v & 0x7fffffff; };
        auto filt_of = [](int v) { return v < 0 ? 1 : 0; };
        std::vector<ExhGroup> groups;
        std::vector<int> gkind;
        auto kind_of = [](int f, int ng) { return f ? (ng > 16 ? 1 : 2) : (ng > 4 ? 0 : 3); };
        auto add_group = [&](ExhGroup g, int kd) {  // a sparse plain group becomes one group per slot
            if (kd == 3) {
                for (int t = 0; t < g.ng; ++t) {
                    groups.push_back(ExhGroup{g.g0 + t, 1, g.unit, 0, g.cend});
                    gkind.push_back(3);
                }
            } else {
                groups.push_back(g);
                gkind.push_back(kd);
            }
        };
        if (parts > 1) {
            // slot s*parts + pp of query s: its A tile, then the unit (tile, part)
            std::vector<int> tile_of(nq, -1), unit_of(nqt * parts, -1);
            for (long long r = 0; r < nq; ++r) tile_of[sorted_q[r]] = (int)(r / TQ);
            for (size_t u = 0; u < flat_units.size(); ++u) unit_of[flat_units[u].qx] = (int)u;
            std::vector<std::tuple<int, int, int>> su(nfull);  // (unit, filtered, slot)
            for (int i = 0; i < nfull; ++i) {
                const int sl = slot_of(fl[i]);
                const int qi = sl / parts, pp = sl % parts;
                su[i] = std::make_tuple(unit_of[(long long)tile_of[qi] * parts + pp], filt_of(fl[i]), sl);
            }
            std::sort(su.begin(), su.end());
            for (int i = 0; i < nfull; ++i) fl[i] = std::get<2>(su[i]);
            for (int i = 0; i < nfull;) {
                const int u = std::get<0>(su[i]), f = std::get<1>(su[i]);
                const int cap = f ? 32 : XQ;
                int j = i;
                while (j < nfull && j - i < cap && std::get<0>(su[j]) == u && std::get<1>(su[j]) == f) ++j;
                const int mine = u >= 0 ? flat_units[u].count - flat_units[u].warm : 0;
                add_group(ExhGroup{i, j - i, u, 0, mine}, kind_of(f, j - i));  // cend: the source's tiles (for chunking)
                if (u >= 0) exh_pairs += (long long)mine * TC * (j - i);
                i = j;
            }
        } else {
            std::sort(fl.begin(), fl.end(), [&](int a, int b) {
                const int fa = filt_of(a), fb = filt_of(b), sa = slot_of(a), sb = slot_of(b);
                if (fa != fb) return fa < fb;
                return sid[sa] < sid[sb] || (sid[sa] == sid[sb] && sa < sb);
            });
            for (int i = 0; i < nfull;) {
                const int f = filt_of(fl[i]);
                const int cap = f ? 32 : XQ;
                int j = i;
                while (j < nfull && j - i < cap && filt_of(fl[j]) == f) ++j;
                const long long cend = predecessor ? (long long)sid[slot_of(fl[j - 1])] : n;
                add_group(ExhGroup{i, j - i, -1, 0, cend}, kind_of(f, j - i));
                for (int t = i; t < j; ++t) exh_pairs += predecessor ? (long long)sid[slot_of(fl[t])] : n;
                i = j;
            }
            for (int i = 0; i < nfull; ++i) fl[i] = slot_of(fl[i]);
        }
        // chunking per kind: about target_items CTAs each (warps for the warp items)
        int ktpc[4] = {1, 1, 1, 1}, kchunk[4] = {4096, 4096, 4096, 4096};
        for (int kd = 0; kd < 4; ++kd) {
            long long work = 0;
            for (size_t gi = 0; gi < groups.size(); ++gi)
                if (gkind[gi] == kd) work += groups[gi].cend;
            const long long target = kd == 3 ? target_items * 8 : target_items;
            if (parts > 1)
                ktpc[kd] = (int)std::min<long long>(16, std::max<long long>(1, (work + target - 1) / target));
            else
                kchunk[kd] = (int)std::min<long long>(
                    16384, std::max<long long>(1024, ((work + target - 1) / target + 255) / 256 * 256));
        }
        for (size_t gi = 0; gi < groups.size(); ++gi) {
            ExhGroup& g = groups[gi];
            const int kd = gkind[gi];
            if (parts > 1) {
                g.nchunks = (int)((g.cend + ktpc[kd] - 1) / ktpc[kd]);
                g.cend = 0;
            } else {
                g.nchunks = (int)((g.cend + kchunk[kd] - 1) / kchunk[kd]);
            }
        }
        std::vector<int> ibeg(nfull + 1, 0);
        int rows = 0;
        std::vector<ExhItem> kitems[4];
        for (size_t gi = 0; gi < groups.size(); ++gi) {
            const ExhGroup& g = groups[gi];
            for (int t = g.g0; t < g.g0 + g.ng; ++t) { ibeg[t] = rows; rows += g.nchunks; }
            for (int c = 0; c < g.nchunks; ++c) kitems[gkind[gi]].push_back(ExhItem{(int)gi, c});
        }
        ibeg[nfull] = rows;
        // chunk-major within each kind: CTAs in flight read the same candidate rows
        std::vector<ExhItem> xitems;
        int koff[5] = {0, 0, 0, 0, 0};
        for (int kd = 0; kd < 4; ++kd) {
            std::stable_sort(kitems[kd].begin(), kitems[kd].end(),
                             [](const ExhItem& a, const ExhItem& b) { return a.chunk < b.chunk; });
            koff[kd] = (int)xitems.size();
            xitems.insert(xitems.end(), kitems[kd].begin(), kitems[kd].end());
        }
        koff[4] = (int)xitems.size();
        const int nitems = koff[4];
        AX((void**)&item_begin_d, sizeof(int) * (nfull + 1));
        AX((void**)&partial, sizeof(unsigned long long) * ((size_t)rows * k + 1));
        AX((void**)&groups_d, sizeof(ExhGroup) * (groups.size() + 1));
        AX((void**)&xitems_d, sizeof(ExhItem) * (nitems + 1));
        if (e == cudaSuccess && !groups.empty())
            e = cudaMemcpyAsync(groups_d, groups.data(), sizeof(ExhGroup) * groups.size(), cudaMemcpyHostToDevice, x0);
        if (e == cudaSuccess && nitems > 0)
            e = cudaMemcpyAsync(xitems_d, xitems.data(), sizeof(ExhItem) * nitems, cudaMemcpyHostToDevice, x0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(full_list, fl.data(), sizeof(int) * nfull, cudaMemcpyHostToDevice, x0);
        if (e == cudaSuccess) e = cudaMemcpyAsync(item_begin_d, ibeg.data(), sizeof(int) * (nfull + 1), cudaMemcpyHostToDevice, x0);
        if (e == cudaSuccess) e = cudaStreamSynchronize(x0);  // the host vectors may go
        R.nfull = nfull;
        const size_t tsmem = tile_smem_bytes(m);
        auto tile_fn = m == 512 ? rescore_tile_kernel<16> : m == 256 ? rescore_tile_kernel<8> : rescore_tile_kernel<0>;
        if (e == cudaSuccess) e = cudaFuncSetAttribute(tile_fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tsmem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(merge_chunks_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rsmem);
        if (e == cudaSuccess && koff[2] > koff[1])
            e = cudaFuncSetAttribute(filter_tile_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem8);
        if (e == cudaSuccess && koff[3] > koff[2])
            e = cudaFuncSetAttribute(filter_tile_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsmem4);
        if (e == cudaSuccess && nitems > 0) {
            // the kinds run side by side; merge_chunks waits for all three
            if (koff[1] > koff[0]) {
                tile_fn<<<(unsigned)(koff[1] - koff[0]), 256, tsmem, x0>>>(
                    R, groups_d, xitems_d + koff[0], item_begin_d, kchunk[0], ktpc[0], units_d, S->lvl_id, S->b_id_ds,
                    partial);
                ++launches;
            }
            if (koff[2] > koff[1]) {
                filter_tile_kernel<8><<<(unsigned)(koff[2] - koff[1]), 256, fsmem8, aux[1]>>>(
                    R, groups_d, xitems_d + koff[1], item_begin_d, kchunk[1], ktpc[1], units_d, S->lvl_id, S->b_id_ds,
                    partial);
                ++launches;
            }
            if (koff[3] > koff[2]) {
                filter_tile_kernel<4><<<(unsigned)(koff[3] - koff[2]), 256, fsmem4, aux[2]>>>(
                    R, groups_d, xitems_d + koff[2], item_begin_d, kchunk[2], ktpc[2], units_d, S->lvl_id, S->b_id_ds,
                    partial);
                ++launches;
            }
            if (koff[4] > koff[3]) {
                const int nw = koff[4] - koff[3];
                rescore_warp_kernel<<<(unsigned)((nw + 7) / 8), 256, 0, aux[3]>>>(
                    R, groups_d, xitems_d + koff[3], nw, item_begin_d, kchunk[3], ktpc[3], units_d, S->lvl_id,
                    S->b_id_ds, partial);
                ++launches;
            }
            e = cudaGetLastError();
            for (int a = 1; a < 4; ++a) {
                if (e == cudaSuccess) e = cudaEventRecord(ev_aux[a], aux[a]);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(x0, ev_aux[a], 0);
            }
            if (e == cudaSuccess) {
                merge_chunks_kernel<<<(unsigned)((nfull + rwpb - 1) / rwpb), 32 * rwpb, rsmem, x0>>>(R, item_begin_d, partial);
                e = cudaGetLastError();
                ++launches;
            }
        }
        if (e == cudaSuccess) e = cudaEventRecord(ev_aux[4], x0);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_aux[4], 0);
        if (e != cudaSuccess)  // nothing of the side streams may outlive the buffers freed below
            for (auto& a : aux)
                if (a) cudaStreamSynchronize(a);
    }
    for (auto& a : aux)
        if (a) cudaStreamDestroy(a);
    for (auto& v : ev_aux)
        if (v) cudaEventDestroy(v);
    if (ev_ovf) cudaEventDestroy(ev_ovf);
    if (e == cudaSuccess && parts > 1) {
        merge_parts_kernel<<<(unsigned)((nq + 7) / 8), 256, 0, st>>>(part_idx, part_dist, nq, parts, k,
                                                                     (long long*)out_idx, out_dist);
        e = cudaGetLastError();
        ++launches;
    }
    float ms_total = 0.f, ms_a = 0.f, ms_b = 0.f, ms_r = 0.f;
    if (timing && e == cudaSuccess) {
        cudaEventRecord(ev[4], st);
        e = cudaEventSynchronize(ev[4]);
        if (e == cudaSuccess) {
            cudaEventElapsedTime(&ms_total, ev[0], ev[4]);
            cudaEventElapsedTime(&ms_a, ev[0], ev[2]);
            cudaEventElapsedTime(&ms_b, ev[2], ev[3]);
            cudaEventElapsedTime(&ms_r, ev[3], ev[4]);
        }
    }
    if (timing) for (int i = 0; i < 6; ++i) cudaEventDestroy(ev[i]);
    long long evals = 0;
    if (e == cudaSuccess && stats) {
        e = cudaMemcpyAsync(&evals, evals_d, sizeof(long long), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
    cudaFreeAsync(slot_id, st); cudaFreeAsync(val_lvl, st); cudaFreeAsync(vtmp, st);
    cudaFreeAsync(key_lvl, st); cudaFreeAsync(ktmp, st); cudaFreeAsync(hist, st);
    cudaFreeAsync(a_slot_lvl, st); cudaFreeAsync(rowmap_lvl, st);
    cudaFreeAsync(al_hi, st); cudaFreeAsync(al_lo, st);
    cudaFreeAsync(surv, st); cudaFreeAsync(surv_cnt, st); cudaFreeAsync(survb, st);
    cudaFreeAsync(full_list, st); cudaFreeAsync(nfull_d, st); cudaFreeAsync(evals_d, st);
    cudaFreeAsync(jobs, st); cudaFreeAsync(unit_jobs_d, st); cudaFreeAsync(unit_counter, st); cudaFreeAsync(qtau, st);
    if (units_d) cudaFreeAsync(units_d, st);
    if (a_slot_x) cudaFreeAsync(a_slot_x, st);
    if (rowmap_x) cudaFreeAsync(rowmap_x, st);
    if (slot_id_x) cudaFreeAsync(slot_id_x, st);
    if (part_idx) cudaFreeAsync(part_idx, st);
    if (part_dist) cudaFreeAsync(part_dist, st);
    if (groups_d) cudaFreeAsync(groups_d, st);
    if (xitems_d) cudaFreeAsync(xitems_d, st);
    if (item_begin_d) cudaFreeAsync(item_begin_d, st);
    if (partial) cudaFreeAsync(partial, st);
    if (e != cudaSuccess) return set_err(CT_ERR_CUDA, "screened form: %s", cudaGetErrorString(e));
    if (status != 0) return set_err(CT_ERR_TIMEOUT, "screened form: pipeline wait timed out (code %d)", status);
    if (stats) {
        stats->pairs_screened = pairs_main;
        stats->pairs_rescored = evals;
        stats->distance_evals = evals;
        stats->kernel_launches = launches;
        stats->device_ms = ms_total;
        stats->threshold_ms = ms_a;
        stats->screen_ms = ms_b;
        stats->rescore_ms = ms_r;
        stats->screen_pairs_main = pairs_main;
        stats->overflow_queries = nfull;
        stats->pairs_exhaustive = exh_pairs;
    }
    return CT_OK;
}

// Device bytes of the metric arrays, the cover tree and the screened operands.
long long ct_tree::device_bytes() const {
    const long long rows = n + std::max<long long>(slab_rows, screen ? ((const State*)screen)->slab_cap : 0);
    long long b = (long long)n * m * 4 + n * (long long)d * 4 + n * 8 + 64 * 4;  // vperm, xs (dataset part), norms, p
    b += rows * (long long)m * 4 + rows * (long long)d * 8 + rows * 4;           // vnat, coords_raw + slab xs, slab p
    if (has_tree) b += n * (8 * 7 + 4 * 6) + (long long)n * (m + d + 2) * 4;
    if (screen) {
        const State* S = (const State*)screen;
        b += S->rows_pad * (long long)m * 4 + S->lvl_rows * (long long)m * 4;   // hi + lo BF16 operands
        b += S->rows_pad * 4 + S->lvl_rows * 12 + n * 12 + rows * 20 + 1024;
        b += (S->rows_pad + S->lvl_rows) / TC * (long long)RT * 4;                  // sweep records
    }
    return b;
}

// ---------------------------------------------------------------- new points
namespace {

__global__ void scale_rows_kernel(const float* __restrict__ coords, long long n, int d,
                                  const float* __restrict__ inv_ls, float* __restrict__ xs) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n * d) return;
    xs[e] = __fmul_rn(coords[e], inv_ls[e % d]);
}

__global__ void iota64_kernel(long long* a, long long n, long long base) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) a[i] = base + i;
}

// Grow the query-side arrays (V, scaled and raw coordinates, p, and the screened
// form's per-row scalars and Hilbert keys) to n + rows rows.  Rows < n are copied;
// the device is synchronised first because in-flight work may read the old arrays.
int ensure_slab(ct_tree* T, State* S, long long rows) {
    if (rows <= S->slab_cap) return CT_OK;
    long long cap = std::max<long long>(rows, std::min<long long>(2 * S->slab_cap, 1LL << 20));
    cap = std::max<long long>(cap, 4096);
    if (T->n + cap >= (1LL << 31)) return T->set_err(CT_ERR_UNSUPPORTED, "%s", "query slab beyond 2^31 rows");
    cudaError_t e = cudaDeviceSynchronize();
    const size_t n = (size_t)T->n, tot = (size_t)(T->n + cap);
    auto grow = [&](void** ptr, size_t row_bytes) {
        void* np = nullptr;
        if (e == cudaSuccess) e = cudaMalloc(&np, row_bytes * tot);
        if (e == cudaSuccess) e = cudaMemcpy(np, *ptr, row_bytes * n, cudaMemcpyDeviceToDevice);
        if (e == cudaSuccess) { cudaFree(*ptr); *ptr = np; }
        else if (np) cudaFree(np);
    };
    grow((void**)&T->vnat, sizeof(float) * T->m);
    grow((void**)&T->xs, sizeof(float) * T->d);
    grow((void**)&T->coords_raw, sizeof(float) * T->d);
    grow((void**)&T->p, sizeof(float));
    grow((void**)&S->vn, sizeof(float));
    grow((void**)&S->isp, sizeof(float));
    grow((void**)&S->xmax, sizeof(float));
    grow((void**)&S->hil_key, sizeof(unsigned long long));
    if (e == cudaSuccess && !S->slab_done) e = cudaEventCreateWithFlags(&S->slab_done, cudaEventDisableTiming);
    if (e != cudaSuccess) return T->set_err(CT_ERR_NOMEM, "query slab of %lld rows: %s", cap, cudaGetErrorString(e));
    S->slab_cap = cap;
    return CT_OK;
}

}  // namespace

// Build the screened operands ahead of the first query (the query slab, if the tree
// was built with CT_BUILD_QUERY_SLAB, is already allocated).
int ct_tree::prepare_screened(cudaStream_t st) {
    if (m % KC != 0 || m > 1024) return set_err(CT_ERR_UNSUPPORTED, "screened form needs m %% 32 == 0 and m <= 1024 (got %d)", m);
    if (d > kMaxD) return set_err(CT_ERR_UNSUPPORTED, "screened form supports d <= %d (got %d)", kMaxD, d);
    return screen_prepare(this, st);
}

// kNN of new points with the screened form: the points are written to the query
// slab (rows n .. n+nq-1, with the dataset's own scaling, scalars and Hilbert
// frame) and searched as query ids n + i against the n dataset rows.  Calls on one
// tree take turns on the slab through an event.
int ct_tree::knn_screened_points(const float* qv, const float* qp, const float* qcoords, int64_t nq, int k,
                                 int64_t* out_idx, float* out_dist, ct_stats* stats, cudaStream_t st) {
    if (stats) memset(stats, 0, sizeof(*stats));
    if (nq <= 0) return CT_OK;
    if (d > kMaxD) return set_err(CT_ERR_UNSUPPORTED, "screened form supports d <= %d (got %d)", kMaxD, d);
    int rc = screen_prepare(this, st);
    if (rc != CT_OK) return rc;
    State* S = (State*)screen;
    rc = ensure_slab(this, S, nq);
    if (rc != CT_OK) return rc;
    cudaError_t e = cudaStreamWaitEvent(st, S->slab_done, 0);
    const size_t n0 = (size_t)n;
    long long* ids = nullptr;
    int* scratch = nullptr;
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&ids, sizeof(long long) * nq, st);
    if (e == cudaSuccess) e = cudaMallocAsync((void**)&scratch, sizeof(int) * nq, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(vnat + n0 * m, qv, sizeof(float) * nq * m, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(coords_raw + n0 * d, qcoords, sizeof(float) * nq * d, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(p + n0, qp, sizeof(float) * nq, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) {
        scale_rows_kernel<<<grid_for(nq * d), 256, 0, st>>>(qcoords, nq, d, inv_ls, xs + n0 * d);
        point_scalars_kernel<<<grid_for(nq), 256, 0, st>>>(vnat + n0 * m, p + n0, xs + n0 * d, nq, m, d,
                                                         S->vn + n0, S->isp + n0, S->xmax + n0);
        iota64_kernel<<<grid_for(nq), 256, 0, st>>>(ids, nq, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = ct::hilbert_keys_bounded(qcoords, nq, d, S->bounds, S->hil_key + n0, scratch, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(ids, st); cudaFreeAsync(scratch, st);
        return set_err(CT_ERR_CUDA, "screened points: slab fill: %s", cudaGetErrorString(e));
    }
    rc = knn_screened((const int64_t*)ids, nq, k, 0, out_idx, out_dist, stats, st, n + nq);
    cudaFreeAsync(ids, st);
    cudaFreeAsync(scratch, st);
    cudaEventRecord(S->slab_done, st);
    if (stats && rc == CT_OK) stats->kernel_launches += 4;
    return rc;
}

// Diagnostic: raw screened dot products of 128 query rows x 256 candidate rows.
int ct_screen_debug_dots(ct_tree* T, const int* rows_a, const int* rows_b, float* out, cudaStream_t st) {
    if (T->m % KC != 0 || T->m > 1024) return T->set_err(CT_ERR_UNSUPPORTED, "%s", "m must be a multiple of 32, <= 1024");
    cudaError_t e = cudaSuccess;
    bf16 *ahi = nullptr, *alo = nullptr, *bhi = nullptr, *blo = nullptr;
    Job* job = nullptr;
    int *status = nullptr, *begin = nullptr;
    const int m = T->m;
    auto A = [&](void** p, size_t bytes) { if (e == cudaSuccess) e = cudaMallocAsync(p, bytes, st); };
    A((void**)&ahi, sizeof(bf16) * TQ * m); A((void**)&alo, sizeof(bf16) * TQ * m);
    A((void**)&bhi, sizeof(bf16) * TC * m); A((void**)&blo, sizeof(bf16) * TC * m);
    A((void**)&job, sizeof(Job)); A((void**)&status, sizeof(int)); A((void**)&begin, 2 * sizeof(int));
    if (e != cudaSuccess) return T->set_err(CT_ERR_NOMEM, "debug dots allocation: %s", cudaGetErrorString(e));
    split_blocked_kernel<<<64, 256, 0, st>>>(T->vnat, m, rows_a, TQ, ahi, alo);
    split_blocked_kernel<<<64, 256, 0, st>>>(T->vnat, m, rows_b, TC, bhi, blo);
    Job hj{0, 0, 0, 1};
    int hb[2] = {0, 1};
    int zero = 0;
    e = cudaMemcpyAsync(job, &hj, sizeof(Job), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(begin, hb, sizeof(hb), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(status, &zero, sizeof(int), cudaMemcpyHostToDevice, st);
    MMAParams P{};
    P.a_hi = ahi; P.a_lo = alo; P.a_groups = TQ / 8;
    P.b_hi[0] = bhi; P.b_lo[0] = blo; P.b_groups[0] = TC / 8;
    P.b_hi[1] = bhi; P.b_lo[1] = blo; P.b_groups[1] = TC / 8;
    P.m = m; P.jobs = job; P.cta_job_begin = begin; P.k = 1; P.nstages = STAGES; P.out_f = out; P.status = status;
    if (e == cudaSuccess) e = launch_sweep(P, MODE_DEBUG, 1, st);
    int hs = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(ahi, st); cudaFreeAsync(alo, st); cudaFreeAsync(bhi, st); cudaFreeAsync(blo, st);
    cudaFreeAsync(job, st); cudaFreeAsync(status, st); cudaFreeAsync(begin, st);
    if (e != cudaSuccess) return T->set_err(CT_ERR_CUDA, "debug dots: %s", cudaGetErrorString(e));
    if (hs != 0) return T->set_err(CT_ERR_TIMEOUT, "debug dots: pipeline wait timed out (code %d)", hs);
    return CT_OK;
}
