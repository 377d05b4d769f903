// (b) precision form of the cosine search: a dense Q x R^T contraction on the
// sm_103a tensor cores (tcgen05.mma kind::f16, fp32 accumulators in TMEM,
// operands staged by TMA), exact in every dot product.
//
// Exactness.  fp16 holds every integer of magnitude <= 2048 exactly, and an
// fp32 accumulator holds every integer of magnitude <= 2^24 exactly, so
//   * queries are +1/-1 (the bipolar read hypervectors) or small integers,
//   * every reference count v is split into balanced base-2048 limbs
//     v = sum_l 2048^l * limb_l with limb_l in [-1024, 1023] (the top limb in
//     [-2048, 2048]), each an exact fp16,
//   * each limb gets its own accumulator, and the host checks
//     dim * max|q| * max|limb_l| <= 2^24 so that no partial sum can round;
//   * the epilogue recombines dot = sum_l 2048^l * acc_l in int64.
// GB300's dense fp16/bf16 tensor rate is far above its INT8 rate, so integer
// limbs on fp16 tensor cores are the fast exact path here.
//
// Kernel shape (one CTA per SM, persistent): M = 128 queries x N = 128
// references per tile, K in blocks of 64 dims (one 128-byte swizzled row per
// operand row), a multi-stage TMA ring, one MMA-issuing thread, and four
// epilogue warps that read the accumulators with tcgen05.ld.  Each epilogue
// thread owns one query (one TMEM lane) and keeps that query's running top-k
// in registers/local memory: an fp32 estimate of every score filters
// candidates, and only those near the current k-th best get the exact FP64
// score of the reference CPU cosine (src/HV.cpp:219-242).
//
// Schedule.  With D in the thousands neither operand tile fits in shared
// memory for the whole K loop, so both are streamed from L2 for every
// (query tile, reference tile) pair.  The persistent grid is G x S CTAs:
// for each group of G query tiles, CTA (g, j) takes query tile g and the
// reference tiles j, j+S, j+2S, ...  All CTAs advance in lockstep, so at any
// moment G query tiles are each read by S CTAs and S reference tiles are each
// read by G CTAs; query tiles are loaded with an L2 evict-last policy and
// reference tiles with evict-first, so DRAM sees each reference tile about
// once per group instead of each query tile once per pair.
#include <cuda.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "hdc_internal.cuh"
#include "tc_ptx.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kBM = 128;  // queries per tile (TMEM lanes)
constexpr int kRowPad = 256;    // database rows are padded to a multiple of the largest N
constexpr int kThreadsTC = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int kMaxLimbs = 4;
constexpr int kMaxKTC = 32;

// Tile shapes: N references per tile and K blocks of BK dims: BK = 64 gives
// 128-byte rows (128-byte swizzle), BK = 32 64-byte rows (64-byte swizzle),
// half the bytes per stage for a deeper ring (N = 256 always uses 32).
// Swizzle atoms are 8 rows, so the descriptor stride between 8-row groups is
// 8 * row bytes.
template <int N, int BKX = (N == 256 ? 32 : 64)>
struct Tile {
    static constexpr int BK = BKX;
    static constexpr int ROWB = BK * 2;
    static constexpr int A_BYTES = kBM * ROWB;
    static constexpr int B_BYTES = N * ROWB;  // per limb
    static constexpr uint32_t SBO = 8 * ROWB;
    static constexpr uint32_t LAYOUT = BK == 32 ? 4u : 2u;  // descriptor swizzle code: 64B : 128B
};

// A stage holds MB query tiles (M-blocks of 128 rows) and L reference-limb tiles; the ring
// gets as many stages as fit in 216 KB (at most 12).
constexpr int kRingBytes = 216 * 1024;
template <int N, int BK = Tile<N>::BK>
__host__ __device__ constexpr int tc_stage_bytes(int L, int MB) {
    return MB * Tile<N, BK>::A_BYTES + L * Tile<N, BK>::B_BYTES;
}
template <int N, int BK = Tile<N>::BK>
__host__ __device__ constexpr int tc_stages(int L, int MB) {
    return kRingBytes / tc_stage_bytes<N, BK>(L, MB) < 12 ? kRingBytes / tc_stage_bytes<N, BK>(L, MB) : 12;
}
// accumulator sets (TMEM columns MB * L * N each): two when they fit in 256 columns
__host__ __device__ constexpr int tc_acc_bufs(int L, int N, int MB) { return MB * L * N <= 256 ? 2 : 1; }
__host__ __device__ constexpr int tc_tmem_cols(int L, int N, int MB) {
    return tc_acc_bufs(L, N, MB) * MB * L * N <= 256 ? 256 : 512;
}

struct TcArgs {
    int64_t nq, nr;
    int dim, k, mode, n_kblocks;
    int64_t r_pad;        // rows per limb in the B tensor
    int n_qtiles, n_rtiles;
    int G, S, n_groups;   // query tiles per group, reference lanes, groups
    int policy;           // 0: no L2 hint, 1: queries evict-last, 2: + references evict-first
    int prefetch;         // K blocks of the same tile pair prefetched into L2 ahead of the ring (0: none)
    int t_stride;         // reference tiles are visited in the order (t * t_stride) mod n_rtiles
    const int64_t* qn;    // [nq] squared norms of the queries
    const float* rr;      // [nr] fp32 1/sqrt(norm)
    uint64_t* ws_key;     // [S][nq][k]
    int64_t* ws_dot;
    int* status;          // device status word (0 = ok)
    const double* rs;     // [nr] sqrt(norm2) of the references
    const double* ri;     // [nr] their rounded reciprocals (0 for a zero norm)
    // [S][nq] the orderable k-th best score of each reference lane's list (0: not full),
    // zeroed before the launch; null when the lanes do not exchange them
    uint32_t* lane_kth;
    int slist;  // 1: the top-k lists live in shared memory after the tile ring, else in local memory
    int limb_bits;     // the database's limbs are base-2^limb_bits digits
    float limb_base;   // 2^limb_bits
    long long wait_cycles;  // limit of the pipeline's bounded waits (SM cycles)
    int withhold;           // test hook: the producer issues no loads, so the waits run out
};

// Insert (key, dot) into a descending list of length k whose entry i is at keys[i * st].
__device__ __forceinline__ void list_insert_strided(uint64_t* keys, int64_t* dots, int st, int k, uint64_t key,
                                                    int64_t dot) {
    int pos = k - 1;
    while (pos > 0 && keys[(pos - 1) * st] < key) {
        keys[pos * st] = keys[(pos - 1) * st];
        dots[pos * st] = dots[(pos - 1) * st];
        --pos;
    }
    keys[pos * st] = key;
    dots[pos * st] = dot;
}

// Filter threshold below a k-th best score sk: the fp32 estimate of any score
// that can still beat sk is at least this (DOT estimates are within a
// relative 4e-6 plus one unit).
// Insert (key, dot) into a descending list of k <= KR keys held in registers
// (keys[i] for i < k, 0 = empty), dropping the last entry, and return the new
// last key.  The dots live in k slots at dots[slot * st]: nibble i of `slots` is
// the slot of entry i, and the entry that drops out hands its slot to the new
// dot.  Every index is a compile-time constant after unrolling, so the keys stay
// in registers and an insertion costs one shared-memory store.
template <int KR>
__device__ __forceinline__ uint64_t reg_insert(uint64_t (&keys)[KR], uint64_t& slots, int k, uint64_t key, int64_t dot,
                                               int64_t* dots, int st) {
    static_assert(KR <= 16, "slots are nibbles of one word");
    int pos = 0;
#pragma unroll
    for (int i = 0; i < KR - 1; ++i) pos += (i < k - 1 && keys[i] > key) ? 1 : 0;
    // shift entries pos..k-2 down one place and put the key at pos, as masked selects
    // (a plain "if (i == pos)" is folded back into a dynamic index, which would move
    // the array to local memory)
#pragma unroll
    for (int i = KR - 1; i >= 0; --i) {
        const uint64_t prev = i > 0 ? keys[i > 0 ? i - 1 : 0] : 0;
        const uint64_t sh = 0ull - (uint64_t)(i > pos && i < k);
        const uint64_t at = 0ull - (uint64_t)(i == pos);
        keys[i] = (keys[i] & ~(sh | at)) | (prev & sh) | (key & at);
    }
    const uint64_t freed = (slots >> (4 * (k - 1))) & 15u;
    const uint64_t below = (1ull << (4 * pos)) - 1;                        // nibbles 0..pos-1
    const uint64_t thru = pos >= 15 ? ~0ull : (1ull << (4 * pos + 4)) - 1;  // nibbles 0..pos
    const uint64_t upto = k >= 16 ? ~0ull : (1ull << (4 * k)) - 1;         // nibbles 0..k-1
    slots = (slots & below) | (freed << (4 * pos)) | ((slots << 4) & upto & ~thru) | (slots & ~upto);
    dots[(int)freed * st] = dot;
    uint64_t last = 0;
#pragma unroll
    for (int i = 0; i < KR; ++i) last |= keys[i] & (0ull - (uint64_t)(i == k - 1));
    return last;
}

__device__ __forceinline__ float filter_below(float sk, int mode) {
    return mode == HDC_SCORE_DOT ? sk - (fabsf(sk) * 4e-6f + 1.0f) : sk - kFilterMargin;
}

__device__ __forceinline__ float approx_tc(float af, float rq, float rr, int mode) {
    if (mode == HDC_SCORE_DOT) return af;
    const float c = af * rq * rr;
    return mode == HDC_SCORE_NORM ? fmaf(2.0f, c, -1.0f) : c;
}

// PAIR_MMA: the CTA pair is one M = 256 MMA (cta_group::2) over its two query
// tiles; with two limbs the even CTA stages limb 0 of the reference tile and the
// odd CTA limb 1, and one 256 x 256 x 16 MMA covers both (each CTA's TMEM gets
// its own 128 queries x both limbs, the layout of the single-CTA form), so each
// SM holds half the reference bytes per stage.  With CL = 4 two such pairs run
// the same two query tiles on two neighbouring reference lanes: each query block
// is loaded once, half by each pair, and multicast into both, which also keeps
// the two lanes in step (a lane with fewer tiles runs empty ones at the end).
template <int L, int kBN, int MB, int CL, bool SHARE_A, int BKT, bool PAIR_MMA, int KR>
__global__ void __launch_bounds__(kThreadsTC, 1)
    tc_search_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, const TcArgs a) {
    using T = Tile<kBN, BKT>;
    constexpr int kBK = T::BK;
    static_assert(!PAIR_MMA || (L == 2 && kBN == 128 && MB == 1 && (CL == 2 || CL == 4) && !SHARE_A),
                  "pair MMA shape");
    static_assert(CL <= 2 || PAIR_MMA, "clusters of 4 pair the MMA");
    static_assert(KR == 0 || (KR == 16 && MB == 1), "register lists: one M-block, k <= 16");
    constexpr bool QUAD = PAIR_MMA && CL == 4;
    constexpr int LS = PAIR_MMA ? 1 : L;  // limb blocks this CTA stages
    constexpr int STAGES = tc_stages<kBN, BKT>(LS, MB);
    constexpr int ACC = tc_acc_bufs(L, kBN, MB);
    constexpr int TCOLS = tc_tmem_cols(L, kBN, MB);
    constexpr int QT = MB * kBM;  // queries per query tile
    constexpr uint32_t kStageBytes = (uint32_t)tc_stage_bytes<kBN, BKT>(LS, MB);
    constexpr uint32_t kAccCols = (uint32_t)(MB * L * kBN);
    constexpr uint32_t IDESC = tc::idesc_f16_f32(kBM, kBN);
    constexpr bool kPairLimbs = kBN == 128 && L >= 2 && !PAIR_MMA;  // limb pairs as one N = 256 MMA
    constexpr uint32_t IDESC2 = kPairLimbs ? tc::idesc_f16_f32(kBM, 2 * kBN) : IDESC;
    constexpr uint32_t IDESC_PAIR = tc::idesc_f16_f32(2 * kBM, 2 * kBN);
    static_assert(MB * L * kBN <= 512, "accumulators exceed TMEM");

    extern __shared__ uint8_t smem_raw[];
    // 1024-byte aligned tile ring (required by the 128-byte swizzle atoms)
    const uint32_t raw_addr = tc::smem_u32(smem_raw);
    uint8_t* ring = smem_raw + ((1024 - (raw_addr & 1023)) & 1023);
    __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES], accf_bar[ACC], acce_bar[ACC];
    __shared__ uint32_t tmem_base_s;
    __shared__ volatile int err_s;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        err_s = 0;
        for (int s = 0; s < STAGES; ++s) {
            tc::mbar_init(&full_bar[s], 1);
            // one commit from each CTA that reads the stage's multicast (with pair MMAs: from the
            // even CTA of each pair that reads it)
            tc::mbar_init(&empty_bar[s], PAIR_MMA ? CL / 2 : CL);
        }
        for (int b = 0; b < ACC; ++b) {
            tc::mbar_init(&accf_bar[b], 1);
            tc::mbar_init(&acce_bar[b], PAIR_MMA ? 8 : 128);  // pair MMAs: each epilogue warp of both CTAs
        }
        tc::fence_mbar_init();
        tc::prefetch_tmap(&tmA);
        tc::prefetch_tmap(&tmB);
    }
    if (warp == 1) {
        if constexpr (PAIR_MMA) {
            tc::tmem_alloc_pair(&tmem_base_s, TCOLS);
            tc::tmem_relinquish_pair();
        } else {
            tc::tmem_alloc(&tmem_base_s, TCOLS);
            tc::tmem_relinquish();
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if constexpr (CL > 1) tc::cluster_sync();  // the peer's barriers exist before anything targets them
    const uint32_t tmem = tmem_base_s;
    // CTA pairs (CL = 2) share one operand by multicast.  Sharing references: the pair
    // runs the same reference tiles for two neighbouring query tiles, and takes part in a
    // group when its first CTA has a query tile (a CTA without one loads the last tile
    // again and writes nothing).  Sharing queries (SHARE_A): the pair runs one query
    // tile on two neighbouring reference lanes, tile by tile in step (the tile count is
    // even, so both CTAs of a pair have a tile in every step; the clamp below only guards).
    // clusters of 4: CTA 2p + r runs query tile r of the cluster's two on reference lane p of its two
    const int quad = (int)(blockIdx.x / 4), qr = (int)(blockIdx.x % 4);
    const int gslot = QUAD      ? 2 * (quad % (a.G / 2)) + (qr & 1)
                      : SHARE_A ? (int)((blockIdx.x / CL) % a.G)
                                : (int)(blockIdx.x % a.G);
    const int lane_j = QUAD      ? 2 * (quad / (a.G / 2)) + (qr >> 1)
                       : SHARE_A ? CL * (int)((blockIdx.x / CL) / a.G) + (int)(blockIdx.x % CL)
                                 : (int)(blockIdx.x / a.G);
    const int lead_slot = SHARE_A ? gslot : gslot & ~(QUAD ? 1 : CL - 1);
    // every lane of a cluster of 4 steps through the same number of tiles
    const int t_end = QUAD ? (a.n_rtiles + a.S - 1) / a.S * a.S : a.n_rtiles;
    const int pair_rank = CL > 1 ? (int)(blockIdx.x % CL) : 0;
    const int t_first = SHARE_A ? lane_j - pair_rank : lane_j;  // both CTAs of a pair step through the same t0
    const int t_off = SHARE_A ? pair_rank : 0;
    const int crank = CL > 1 ? (int)tc::cluster_ctarank() : 0;

    if (warp == 0) {
        // ------------------------------------------------ TMA producer
        if (lane == 0) {
            int stage = 0;
            uint32_t phase = 0;
            int64_t issued = 0;
            bool ok = true;
            const uint64_t pol_q = tc::make_policy_evict_last(), pol_r = tc::make_policy_evict_first();
            const bool hint_q = a.policy >= 1, hint_r = a.policy >= 2;
            const int rank = crank;
            // a.withhold (tests of the bounded waits): no load is issued, so the MMA issuer's and the
            // epilogue's waits run out with nothing in flight
            for (int grp = 0; ok && !a.withhold && grp < a.n_groups; ++grp) {
                if (grp * a.G + lead_slot >= a.n_qtiles) continue;
                const int qt = min(grp * a.G + gslot, a.n_qtiles - 1);
                for (int t0 = t_first; ok && t0 < t_end; t0 += a.S) {
                    const int t = (int)((int64_t)min(t0 + t_off, a.n_rtiles - 1) * a.t_stride % a.n_rtiles);
                    for (int kb = 0; kb < a.n_kblocks; ++kb) {
                        if (!tc::mbar_wait(&empty_bar[stage], phase ^ 1, &err_s, 1, a.wait_cycles)) {
                            ok = false;
                            break;
                        }
                        uint8_t* st = ring + (size_t)stage * kStageBytes;
                        if constexpr (PAIR_MMA) {
                            // this CTA's query block and its limb's reference block; the bytes of
                            // both CTAs complete on the even CTA's full barrier, where its MMA waits
                            const int pr = rank & 1;  // rank in the pair: limb and query tile
                            if (pr == 0) tc::mbar_arrive_expect_tx(&full_bar[stage], 2 * kStageBytes);
                            const uint32_t fb = tc::cluster_addr(&full_bar[stage], (uint32_t)(rank & ~1));
                            const int yb = (int)(pr * a.r_pad + (int64_t)t * kBN);
                            if constexpr (QUAD) {
                                // half of the query block (pair p loads rows 64p..64p+63), into this
                                // CTA and the CTA of the other pair that runs the same query tile
                                const int pp = rank >> 1;
                                tc::tma_load_2d_pair_mc(st + pp * (T::A_BYTES / 2), &tmA, fb, kb * kBK,
                                                        qt * QT + pp * (kBM / 2), (uint16_t)((1u << pr) | (4u << pr)));
                            } else if (hint_q) {
                                tc::tma_load_2d_pair_hint(st, &tmA, fb, kb * kBK, qt * QT, pol_q);
                            } else {
                                tc::tma_load_2d_pair(st, &tmA, fb, kb * kBK, qt * QT);
                            }
                            if (hint_r)
                                tc::tma_load_2d_pair_hint(st + T::A_BYTES, &tmB, fb, kb * kBK, yb, pol_r);
                            else
                                tc::tma_load_2d_pair(st + T::A_BYTES, &tmB, fb, kb * kBK, yb);
                            ++issued;
                            if (++stage == STAGES) {
                                stage = 0;
                                phase ^= 1;
                            }
                            continue;
                        }
                        tc::mbar_arrive_expect_tx(&full_bar[stage], kStageBytes);
#pragma unroll
                        for (int m = 0; m < MB; ++m) {
                            if constexpr (SHARE_A) {
                                // this CTA's 1/CL of the query block's rows, into every CTA of the pair
                                void* dst = st + (size_t)T::A_BYTES * m + (size_t)rank * (T::A_BYTES / CL);
                                tc::tma_load_2d_mc(dst, &tmA, &full_bar[stage], kb * kBK,
                                                   qt * QT + m * kBM + rank * (kBM / CL), (uint16_t)((1u << CL) - 1));
                                continue;
                            }
                            void* dst = st + (size_t)T::A_BYTES * m;
                            if (hint_q)
                                tc::tma_load_2d_hint(dst, &tmA, &full_bar[stage], kb * kBK, qt * QT + m * kBM, pol_q);
                            else
                                tc::tma_load_2d(dst, &tmA, &full_bar[stage], kb * kBK, qt * QT + m * kBM);
                        }
#pragma unroll
                        for (int l = 0; l < L; ++l) {
                            if constexpr (CL > 1 && !SHARE_A) {
                                // this CTA's 1/CL of the block's rows, into every CTA of the pair
                                void* dst = st + (size_t)T::A_BYTES * MB + (size_t)T::B_BYTES * l +
                                            (size_t)rank * (T::B_BYTES / CL);
                                const int y = (int)(l * a.r_pad + (int64_t)t * kBN) + rank * (kBN / CL);
                                tc::tma_load_2d_mc(dst, &tmB, &full_bar[stage], kb * kBK, y, (uint16_t)((1u << CL) - 1));
                                continue;
                            }
                            void* dst = st + (size_t)T::A_BYTES * MB + (size_t)T::B_BYTES * l;
                            const int y = (int)(l * a.r_pad + (int64_t)t * kBN);
                            if (hint_r)
                                tc::tma_load_2d_hint(dst, &tmB, &full_bar[stage], kb * kBK, y, pol_r);
                            else
                                tc::tma_load_2d(dst, &tmB, &full_bar[stage], kb * kBK, y);
                        }
                        if (CL == 1 && a.prefetch > 0 && kb + a.prefetch < a.n_kblocks) {
                            // the ring holds STAGES blocks in flight; start the one `prefetch` blocks
                            // ahead toward L2 now, so its load later finds it there
                            const int xk = (kb + a.prefetch) * kBK;
#pragma unroll
                            for (int m = 0; m < MB; ++m) tc::tma_prefetch_2d(&tmA, xk, qt * QT + m * kBM);
#pragma unroll
                            for (int l = 0; l < L; ++l)
                                tc::tma_prefetch_2d(&tmB, xk, (int)(l * a.r_pad + (int64_t)t * kBN));
                        }
                        ++issued;
                        if (++stage == STAGES) {
                            stage = 0;
                            phase ^= 1;
                        }
                    }
                }
            }
            // before leaving, let the last loads land (bounded); with pair MMAs they land on the
            // even CTA's barriers, so wait until the commits that free them reach this CTA
            int s = stage;
            uint32_t ph = phase;
            for (int64_t i = 0; i < (issued < STAGES ? issued : (int64_t)STAGES); ++i) {
                if (--s < 0) {
                    s = STAGES - 1;
                    ph ^= 1;
                }
                uint64_t* bar = PAIR_MMA ? &empty_bar[s] : &full_bar[s];
                const long long c0 = clock64();
                while (!tc::mbar_try_wait(tc::smem_u32(bar), ph) && clock64() - c0 < tc::kWaitCycles) {
                }
            }
        }
    } else if (warp == 1) {
        // ------------------------------------------------ MMA issuer (the even CTA's, with pair MMAs)
        if (lane == 0 && (!PAIR_MMA || (crank & 1) == 0)) {
            int stage = 0, acc = 0;
            uint32_t phase = 0, acc_phase = 0;
            bool ok = true;
            int64_t consumed = 0, tiles = 0;
            for (int grp = 0; ok && grp < a.n_groups; ++grp) {
                if (grp * a.G + lead_slot >= a.n_qtiles) continue;
                for (int t0 = t_first; ok && t0 < t_end; t0 += a.S) {
                    if (!(PAIR_MMA ? tc::mbar_wait_cluster(&acce_bar[acc], acc_phase ^ 1, &err_s, 2, a.wait_cycles)
                                   : tc::mbar_wait(&acce_bar[acc], acc_phase ^ 1, &err_s, 2, a.wait_cycles))) {
                        ok = false;
                        break;
                    }
                    tc::fence_after();
                    const uint32_t d0 = tmem + (uint32_t)acc * kAccCols;
                    for (int kb = 0; kb < a.n_kblocks; ++kb) {
                        if (!tc::mbar_wait(&full_bar[stage], phase, &err_s, 3, a.wait_cycles)) {
                            ok = false;
                            break;
                        }
                        tc::fence_after();
                        const uint32_t sa = tc::smem_u32(ring + (size_t)stage * kStageBytes);
                        if constexpr (PAIR_MMA) {
                            const uint64_t adesc = tc::kmajor_desc(sa, T::SBO, T::LAYOUT);
                            const uint64_t bdesc = tc::kmajor_desc(sa + (uint32_t)T::A_BYTES, T::SBO, T::LAYOUT);
#pragma unroll
                            for (int kk = 0; kk < kBK / 16; ++kk)
                                tc::mma_f16_pair(d0, adesc + 2 * kk, bdesc + 2 * kk, IDESC_PAIR, (kb | kk) != 0 ? 1u : 0u);
                            // frees the stage in the pair (and, in a cluster of 4, in the other pair,
                            // whose query-block half landed there too)
                            tc::mma_commit_pair_mc(&empty_bar[stage], QUAD ? 0xF : 3);
                        } else {
#pragma unroll
                            for (int l = 0; l < L; ++l) {
                                // With 128-row tiles two neighbouring limbs' blocks are 256 consecutive
                                // rows, and their accumulators 256 consecutive columns: one N = 256 MMA
                                // covers both, reading each query slice from shared memory once.
                                if (kPairLimbs && (l & 1)) continue;
                                const bool wide = kPairLimbs && l + 1 < L;
                                const uint64_t bdesc = tc::kmajor_desc(
                                    sa + (uint32_t)T::A_BYTES * MB + (uint32_t)T::B_BYTES * l, T::SBO, T::LAYOUT);
#pragma unroll
                                for (int m = 0; m < MB; ++m) {
                                    const uint64_t adesc = tc::kmajor_desc(sa + (uint32_t)T::A_BYTES * m, T::SBO, T::LAYOUT);
#pragma unroll
                                    for (int kk = 0; kk < kBK / 16; ++kk)  // K = 16 fp16 per MMA = 32 bytes
                                        tc::mma_f16(d0 + (uint32_t)((m * L + l) * kBN), adesc + 2 * kk, bdesc + 2 * kk,
                                                    wide ? IDESC2 : IDESC, (kb | kk) != 0 ? 1u : 0u);
                                }
                            }
                            // frees the stage (in every CTA of the pair) when these MMAs finish
                            if constexpr (CL > 1)
                                tc::mma_commit_mc(&empty_bar[stage], (uint16_t)((1u << CL) - 1));
                            else
                                tc::mma_commit(&empty_bar[stage]);
                        }
                        ++consumed;
                        if (++stage == STAGES) {
                            stage = 0;
                            phase ^= 1;
                        }
                    }
                    if (!ok) break;
                    // accumulators of this tile are complete
                    if constexpr (PAIR_MMA)
                        tc::mma_commit_pair_mc(&accf_bar[acc], (uint16_t)(3u << (crank & 2)));
                    else
                        tc::mma_commit(&accf_bar[acc]);
                    ++tiles;
                    if (++acc == ACC) {
                        acc = 0;
                        acc_phase ^= 1;
                    }
                }
            }
            if constexpr (PAIR_MMA) {
                // the odd CTA's epilogue warps arrive on this CTA's barriers: let the arrivals
                // for the last tiles land before the CTA can leave (bounded)
                for (int64_t i = 0; i < (tiles < ACC ? tiles : (int64_t)ACC); ++i) {
                    const long long c0 = clock64();
                    while (!tc::mbar_try_wait_cluster(tc::smem_u32(&acce_bar[acc]), acc_phase ^ 1) &&
                           clock64() - c0 < tc::kWaitCycles) {
                    }
                    if (++acc == ACC) {
                        acc = 0;
                        acc_phase ^= 1;
                    }
                }
            } else if constexpr (CL > 1) {
                // the peer's commits for the last stages arrive on this CTA's barriers: let them
                // land before the CTA can leave (bounded)
                int s_ = stage;
                uint32_t ph = phase;
                for (int64_t i = 0; i < (consumed < STAGES ? consumed : (int64_t)STAGES); ++i) {
                    if (--s_ < 0) {
                        s_ = STAGES - 1;
                        ph ^= 1;
                    }
                    const long long c0 = clock64();
                    while (!tc::mbar_try_wait(tc::smem_u32(&empty_bar[s_]), ph) && clock64() - c0 < tc::kWaitCycles) {
                    }
                }
            }
        }
    } else {
        // ------------------------------------------------ epilogue: warps 2..5
        const int quarter = warp & 3;  // TMEM lane quarter this warp may access
        const int row = quarter * 32 + lane;
        const uint32_t lane_addr = (uint32_t)(quarter * 32) << 16;
        const int k = a.k;
        int acc = 0;
        uint32_t acc_phase = 0;
        bool ok = true;
        // this thread's top-k list of each M-block: entry i at lk[m][i * ls] / ld[m][i * ls], in
        // shared memory after the ring (one column per TMEM lane) when it fits, else local memory
        uint64_t keys_local[MB][kMaxKTC];
        int64_t dots_local[MB][kMaxKTC];
        uint64_t* lk[MB];
        int64_t* ld[MB];
        const int ls = a.slist ? kBM : 1;
#pragma unroll
        for (int m = 0; m < MB; ++m) {
            if (a.slist) {
                uint64_t* sk = reinterpret_cast<uint64_t*>(ring + (size_t)STAGES * kStageBytes);
                lk[m] = sk + (size_t)m * k * kBM + row;
                ld[m] = reinterpret_cast<int64_t*>(sk + (size_t)MB * k * kBM) + (size_t)m * k * kBM + row;
            } else {
                lk[m] = keys_local[m];
                ld[m] = dots_local[m];
            }
        }
        uint64_t kth[MB];  // each list's k-th key (0 while it has fewer than k entries)
        // KR > 0: the keys of the (single) list in registers, its dots in slots of ld[0]
        uint64_t rkeys[KR > 0 ? KR : 1];
        uint64_t rslots = 0;
        for (int grp = 0; ok && grp < a.n_groups; ++grp) {
            if (grp * a.G + lead_slot >= a.n_qtiles) continue;
            const int qt = grp * a.G + gslot;  // past the last tile for a CTA without one: no live rows
            // this thread owns query row `row` of each M-block
            int64_t gq[MB];
            double my_sq[MB], my_iq[MB];
            float my_rq[MB], thr[MB];
            uint32_t other_kth[MB], told[MB];  // best k-th of the other lanes; the value this lane last told
            bool live[MB];
#pragma unroll
            for (int m = 0; m < MB; ++m) {
                gq[m] = (int64_t)qt * QT + m * kBM + row;
                live[m] = gq[m] < a.nq;
                const int64_t qn = live[m] ? a.qn[gq[m]] : 0;
                my_rq[m] = rsqrt_norm(qn);
                my_sq[m] = __dsqrt_rn((double)qn);
                my_iq[m] = qn ? __drcp_rn(my_sq[m]) : 0.0;
                thr[m] = -INFINITY;
                other_kth[m] = 0;
                told[m] = 0;
                if constexpr (KR > 0) {
#pragma unroll
                    for (int i = 0; i < KR; ++i) rkeys[i] = 0;
                    rslots = 0xfedcba9876543210ull;  // entry i in slot i
                } else {
                    for (int i = 0; i < k; ++i) {
                        lk[m][i * ls] = 0;
                        ld[m][i * ls] = 0;
                    }
                }
                kth[m] = 0;
            }
            for (int t0 = t_first; t0 < t_end; t0 += a.S) {
                // the tile the producer loaded (a step past the last tile keeps its columns past nr)
                const int t = t0 + t_off < a.n_rtiles ? (int)((int64_t)(t0 + t_off) * a.t_stride % a.n_rtiles)
                                                      : t0 + t_off;
                if (!tc::mbar_wait(&accf_bar[acc], acc_phase, &err_s, 4, a.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc::fence_after();
                const uint32_t d0 = tmem + lane_addr + (uint32_t)acc * kAccCols;
#pragma unroll
                for (int m = 0; m < MB; ++m) {
                    for (int c0 = 0; c0 < kBN; c0 += 32) {
                        uint32_t v[L][32];
#pragma unroll
                        for (int l = 0; l < L; ++l) tc::tmem_ld32(d0 + (uint32_t)((m * L + l) * kBN + c0), v[l]);
                        tc::tmem_ld_wait();
                        const int64_t rbase = (int64_t)t * kBN + c0;
                        // the chunk's 32 reference norms, one per lane (coalesced), for the rare
                        // candidates that pass the fp32 filter
                        const bool in_lane = rbase + lane < a.nr;
                        const float rr_lane = in_lane ? __ldg(a.rr + rbase + lane) : 0.0f;
                        const double rs_lane = in_lane ? __ldg(a.rs + rbase + lane) : 0.0;
                        const double ri_lane = in_lane ? __ldg(a.ri + rbase + lane) : 0.0;
                        // the fp32 filter over the chunk's 32 columns (unrolled, no slow path in
                        // between, so the loop stays small in the instruction cache) ...
                        uint32_t pm = 0;  // this lane's columns that pass
#pragma unroll
                        for (int c = 0; c < 32; ++c) {
                            const float rrc = __shfl_sync(0xffffffffu, rr_lane, c);
                            float af = __uint_as_float(v[0][c]);
                            float scale = 1.0f;
#pragma unroll
                            for (int l = 1; l < L; ++l) {
                                scale *= a.limb_base;
                                af = fmaf(__uint_as_float(v[l][c]), scale, af);
                            }
                            const float ap = approx_tc(af, my_rq[m], rrc, a.mode);
                            pm |= (uint32_t)(ap >= thr[m] && live[m] && rbase + c < a.nr) << c;
                        }
                        // ... then one copy of the exact path for each column any lane passed, its
                        // limb sums read again from TMEM (the accumulator is held until the arrival
                        // below).  The threshold of the chunk's later columns is the one of its
                        // start: a few more candidates, all decided by the exact key.
                        uint32_t wm = __reduce_or_sync(0xffffffffu, pm);
                        while (wm) {
                            const int c = __ffs(wm) - 1;
                            wm &= wm - 1;
                            uint32_t vc[L];
#pragma unroll
                            for (int l = 0; l < L; ++l) vc[l] = tc::tmem_ld1(d0 + (uint32_t)((m * L + l) * kBN + c0 + c));
                            tc::tmem_ld_wait();
                            const double rsc = __shfl_sync(0xffffffffu, rs_lane, c);
                            const double ric = __shfl_sync(0xffffffffu, ri_lane, c);
                            if ((pm >> c) & 1u) {
                                // each limb sum is an integer of magnitude <= 2^24: a 32-bit
                                // conversion is exact and stays off the FP64 pipe
                                int64_t dot = 0;
#pragma unroll
                                for (int l = 0; l < L; ++l)
                                    dot += (int64_t)__float2int_rn(__uint_as_float(vc[l])) * ((int64_t)1 << (a.limb_bits * l));
                                const int64_t gr = rbase + c;
                                const float s = exact_score_recip(dot, my_sq[m], rsc, my_iq[m], ric, a.mode);
                                const uint64_t key = make_key(s, (uint32_t)gr);
                                // below another lane's k-th best: k better references already exist
                                if (key > kth[m] && (uint32_t)(key >> 32) >= other_kth[m]) {
                                    if constexpr (KR > 0) {
                                        kth[m] = reg_insert<KR>(rkeys, rslots, k, key, dot, ld[m], ls);
                                    } else {
                                        list_insert_strided(lk[m], ld[m], ls, k, key, dot);
                                        kth[m] = lk[m][(k - 1) * ls];
                                    }
                                    if (kth[m] != 0) thr[m] = fmaxf(thr[m], filter_below(key_score(kth[m]), a.mode));
                                }
                            }
                            __syncwarp();  // converged for the next column's warp-wide TMEM load
                        }
                    }
                }
                if (a.lane_kth) {
                    // tell the other reference lanes this lane's k-th best of each query, and
                    // filter by theirs (stale values are lower, so only less selective)
#pragma unroll
                    for (int m = 0; m < MB; ++m) {
                        if (!live[m]) continue;
                        const uint32_t mine = (uint32_t)(kth[m] >> 32);  // 0 while the list is not full
                        if (mine != told[m]) {
                            tc::st_relaxed_u32(a.lane_kth + (int64_t)lane_j * a.nq + gq[m], mine);
                            told[m] = mine;
                        }
                        uint32_t best = other_kth[m];
                        for (int j = 0; j < a.S; ++j)
                            if (j != lane_j) best = max(best, tc::ld_relaxed_u32(a.lane_kth + (int64_t)j * a.nq + gq[m]));
                        if (best > other_kth[m]) {
                            other_kth[m] = best;
                            thr[m] = fmaxf(thr[m], filter_below(unord_float(best), a.mode));
                        }
                    }
                }
                tc::fence_before();
                if constexpr (PAIR_MMA) {
                    // one arrival per warp, on the even CTA's barrier (its MMAs write both TMEMs)
                    __syncwarp();
                    if (lane == 0) {
                        if ((crank & 1) == 0)
                            tc::mbar_arrive(&acce_bar[acc]);
                        else
                            tc::mbar_arrive_cluster(tc::cluster_addr(&acce_bar[acc], (uint32_t)(crank & ~1)));
                    }
                } else {
                    tc::mbar_arrive(&acce_bar[acc]);
                }
                if (++acc == ACC) {
                    acc = 0;
                    acc_phase ^= 1;
                }
            }
            if (!ok) break;
#pragma unroll
            for (int m = 0; m < MB; ++m) {
                if (!live[m]) continue;
                uint64_t* ok_ = a.ws_key + ((int64_t)lane_j * a.nq + gq[m]) * k;
                int64_t* od = a.ws_dot + ((int64_t)lane_j * a.nq + gq[m]) * k;
                if constexpr (KR > 0) {
#pragma unroll
                    for (int i = 0; i < KR; ++i)
                        if (i < k) {
                            ok_[i] = rkeys[i];
                            od[i] = rkeys[i] ? ld[m][(int)((rslots >> (4 * i)) & 15u) * ls] : 0;
                        }
                } else {
                    for (int i = 0; i < k; ++i) {
                        ok_[i] = lk[m][i * ls];
                        od[i] = ld[m][i * ls];
                    }
                }
            }
        }
    }

    tc::fence_before();
    __syncthreads();
    // pair MMAs: the even CTA's MMAs into this CTA's TMEM are complete (its epilogue waited for
    // every tile) and both CTAs free the columns together
    if constexpr (PAIR_MMA) tc::cluster_sync();
    if (warp == 1) {
        tc::fence_after();
        if constexpr (PAIR_MMA)
            tc::tmem_dealloc_pair(tmem, TCOLS);
        else
            tc::tmem_dealloc(tmem, TCOLS);
    }
    if (threadIdx.x == 0 && err_s) atomicCAS(a.status, 0, 100 + err_s);
    if constexpr (CL > 1) tc::cluster_sync();  // no CTA leaves while its peer may still write into it
}

// ---------------------------------------------------------------- database build
// limbs[l][r][d] (fp16) of ref[r][d]; rows r >= nr of each limb are zero.
template <typename T>
__global__ void limbs_kernel(const T* __restrict__ ref, int64_t nr, int dim, int L, int bits, int64_t r_pad,
                             __half* __restrict__ limbs, int32_t* __restrict__ limb_max) {
    const int64_t base = (int64_t)1 << bits, half = base >> 1;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = r_pad * dim;
    int32_t mx[kMaxLimbs] = {0, 0, 0, 0};
    if (i < total) {
        const int64_t r = i / dim;
        int64_t v = r < nr ? (int64_t)ref[i] : 0;
        for (int l = 0; l < L; ++l) {
            int64_t digit;
            if (l == L - 1) {
                digit = v;
            } else {
                digit = ((v + half) & (base - 1)) - half;
                v = (v - digit) / base;
            }
            limbs[(int64_t)l * total + i] = __int2half_rn((int)digit);
            mx[l] = (int32_t)(digit < 0 ? -digit : digit);
        }
    }
    for (int l = 0; l < L; ++l) {
        int32_t m = mx[l];
        for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && m) atomicMax(limb_max + l, m);
    }
}

__global__ void rsqrt_kernel(const int64_t* __restrict__ n2, int64_t n, float* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = rsqrt_norm(n2[i]);
}

__global__ void sqrt_kernel(const int64_t* __restrict__ n2, int64_t n, double* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        const double s = __dsqrt_rn((double)n2[i]);
        out[i] = s;
        out[n + i] = n2[i] ? __drcp_rn(s) : 0.0;
    }
}

// cuTensorMapEncodeTiled resolved through the runtime, so the library does not
// link libcuda (it must load on hosts without a driver).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled_fn() {
    static EncodeTiledFn fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    }
    return fn;
}

// Tensor map of a row-major [rows][dim] fp16 matrix read in boxes of
// box_rows x bk elements with the swizzle matching the row bytes (bk * 2).
bool make_tmap(CUtensorMap* map, const void* base, int64_t rows, int dim, int bk, int box_rows) {
    EncodeTiledFn encode = encode_tiled_fn();
    if (!encode) return false;
    cuuint64_t gdim[2] = {(cuuint64_t)dim, (cuuint64_t)rows};
    cuuint64_t gstride[1] = {(cuuint64_t)dim * 2};
    cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), gdim, gstride, box, estr,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace

int refdb_create(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                 int32_t max_query_abs, hdc_refdb** out, cudaStream_t stream) {
    *out = nullptr;
    const int dim = ctx->dim;
    if (dim % 8 != 0) return fail(HDC_ERR_INVALID, "refdb: dim must be a multiple of 8 (TMA row stride)");
    if (nr < 1) return fail(HDC_ERR_INVALID, "refdb: empty reference set");
    // Limb magnitude cap T: every limb is an exact fp16 (<= 2048), and with queries up to
    // max_query_abs every fp32 partial sum stays an exact integer (dim * max|q| * T <= 2^24).
    // The base is the largest power of two whose balanced digits stay within T.
    int bits = 11;
    int64_t cap = 2048;
    if (max_query_abs > 0) {
        cap = std::min<int64_t>(2048, ((int64_t)1 << 24) / ((int64_t)dim * max_query_abs));
        if (cap < 1) return fail(HDC_ERR_RANGE, "refdb: dim * max query magnitude exceeds 2^24 (fp32 inexact)");
        bits = 1;
        while (bits < 11 && ((int64_t)1 << bits) <= cap) ++bits;  // 2^(bits-1) <= cap
    }
    // limbs needed for |v| <= max_abs: L-1 balanced base-2^bits digits, then a top digit
    // within the cap (cover_L = cover_{L-1} * base + base/2 - 1 bounds every digit by the cap)
    int L = 1;
    int64_t cover = cap;
    while ((int64_t)max_abs > cover) {
        ++L;
        cover = cover * ((int64_t)1 << bits) + ((int64_t)1 << (bits - 1)) - 1;
        if (L > kMaxLimbs) return fail(HDC_ERR_RANGE, "refdb: values need more than 4 limbs");
    }
    auto* db = new hdc_refdb();
    db->nr = nr;
    db->dim = dim;
    db->L = L;
    db->limb_bits = bits;
    db->max_abs = max_abs;
    db->r_pad = (nr + kRowPad - 1) / kRowPad * kRowPad;
    const size_t nl = (size_t)L * db->r_pad * dim;
    cudaError_t e = cudaMalloc(&db->d_limbs, nl * sizeof(__half));
    if (e == cudaSuccess) e = cudaMalloc(&db->d_norm2, nr * sizeof(int64_t));
    if (e == cudaSuccess) e = cudaMalloc(&db->d_rsq, nr * sizeof(float));
    int32_t* d_lmax = nullptr;
    if (e == cudaSuccess) e = cudaMalloc(&d_lmax, sizeof(int32_t) * kMaxLimbs);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_lmax, 0, sizeof(int32_t) * kMaxLimbs, stream);
    if (e != cudaSuccess) {
        cudaFree(db->d_limbs);
        cudaFree(db->d_norm2);
        cudaFree(db->d_rsq);
        cudaFree(d_lmax);
        delete db;
        return cuda_fail(e, "refdb: allocation");
    }
    const int64_t total = db->r_pad * dim;
    const unsigned grid = (unsigned)((total + 255) / 256);
    if (elem_bytes == 2)
        limbs_kernel<int16_t><<<grid, 256, 0, stream>>>(static_cast<const int16_t*>(d_ref), nr, dim, L, bits, db->r_pad,
                                                        db->d_limbs, d_lmax);
    else
        limbs_kernel<int32_t><<<grid, 256, 0, stream>>>(static_cast<const int32_t*>(d_ref), nr, dim, L, bits, db->r_pad,
                                                        db->d_limbs, d_lmax);
    int st = launch_norms(ctx, d_ref, elem_bytes, nr, db->d_norm2, nullptr, stream);
    if (st == HDC_OK) {
        rsqrt_kernel<<<(unsigned)((nr + 255) / 256), 256, 0, stream>>>(db->d_norm2, nr, db->d_rsq);
        e = cudaGetLastError();
        if (e == cudaSuccess && refdb_sqrt_table(db, stream) != HDC_OK) e = cudaErrorMemoryAllocation;
        if (e == cudaSuccess) e = cudaMemcpyAsync(db->limb_max, d_lmax, sizeof(int32_t) * kMaxLimbs,
                                                  cudaMemcpyDeviceToHost, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
        if (e != cudaSuccess) st = cuda_fail(e, "refdb: build");
    }
    cudaFree(d_lmax);
    if (st != HDC_OK) {
        refdb_destroy(db);
        return st;
    }
    *out = db;
    return HDC_OK;
}

void refdb_destroy(hdc_refdb* db) {
    if (!db) return;
    cudaFree(db->d_limbs);
    cudaFree(db->d_norm2);
    cudaFree(db->d_rsq);
    cudaFree(db->d_sqrt);
    delete db;
}

int refdb_sqrt_table(hdc_refdb* db, cudaStream_t stream) {
    cudaError_t e = cudaMalloc(&db->d_sqrt, 2 * (size_t)db->nr * sizeof(double));
    if (e != cudaSuccess) return cuda_fail(e, "refdb: allocation");
    sqrt_kernel<<<(unsigned)((db->nr + 255) / 256), 256, 0, stream>>>(db->d_norm2, db->nr, db->d_sqrt);
    e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "refdb: norms");
}

int tc_default_group() { return 1 << 30; }  // every SM on its own query tile, references shared
int tc_default_policy() { return 0; }
int tc_default_prefetch() { return 0; }
int tc_default_cluster() { return 4; }
int tc_default_share() { return 0; }
int tc_default_scatter() { return 1; }
int tc_default_kblock() { return 64; }
int tc_default_pair_mma() { return 1; }

// A stride coprime to n near n / golden ratio: consecutive steps visit reference tiles
// far apart, so a query's scores do not rise tile after tile as the scan approaches its
// own part of a tree-ordered database (every new best costs an exact score and an insert).
static int tile_stride(int n) {
    if (n <= 2) return 1;
    int s = (int)(0.6180339887 * n);
    if (s < 1) s = 1;
    while (std::gcd(s, n) != 1) ++s;
    return s % n ? s : 1;
}
int tc_default_tile_n() { return 128; }
int tc_default_m_blocks() { return 1; }

// G query tiles per group (fewer for small batches) and S = SMs / G lanes.
// N = 256 needs L * 256 TMEM columns for one accumulator set: 3 and 4 limbs use N = 128.
static int tc_tile_n(const hdc_context* ctx, const hdc_refdb* db) {
    const int n = ctx->tc_tile_n > 0 ? ctx->tc_tile_n : tc_default_tile_n();
    return db->L > 2 ? 128 : n;
}

// Two M-blocks per CTA need MB * L * N <= 512 TMEM columns: N = 128 and at most 2 limbs.
static int tc_m_blocks(const hdc_context* ctx, const hdc_refdb* db) {
    const int mb = ctx->tc_m_blocks > 0 ? ctx->tc_m_blocks : tc_default_m_blocks();
    return (mb == 2 && db->L <= 2 && tc_tile_n(ctx, db) == 128) ? 2 : 1;
}

// CTA pairs sharing reference blocks by multicast: N = 128, one M-block, and an
// even number of query tiles per group (a pair must not straddle two lanes).
static int tc_cluster(const hdc_context* ctx, const hdc_refdb* db) {
    const int c = ctx->tc_cluster > 0 ? ctx->tc_cluster : tc_default_cluster();
    return (c >= 2 && tc_tile_n(ctx, db) == 128 && tc_m_blocks(ctx, db) == 1) ? 2 : 1;
}

// 32-dim K blocks (deeper ring) on the paired reference-sharing path, when chosen.
static bool tc_kb32(const hdc_context* ctx, const hdc_refdb* db) {
    return tc_tile_n(ctx, db) == 128 && tc_m_blocks(ctx, db) == 1 && tc_cluster(ctx, db) == 2 &&
           (ctx->tc_share >= 0 ? ctx->tc_share : tc_default_share()) == 0 &&
           (ctx->tc_kblock > 0 ? ctx->tc_kblock : tc_default_kblock()) == 32;
}

// The reference-sharing pair as one M = 256 MMA: two limbs, 64-dim K blocks.
static bool tc_pair_mma(const hdc_context* ctx, const hdc_refdb* db) {
    return db->L == 2 && tc_tile_n(ctx, db) == 128 && tc_m_blocks(ctx, db) == 1 && tc_cluster(ctx, db) == 2 &&
           (ctx->tc_share >= 0 ? ctx->tc_share : tc_default_share()) == 0 && !tc_kb32(ctx, db) &&
           (ctx->tc_pair_mma >= 0 ? ctx->tc_pair_mma : tc_default_pair_mma()) != 0;
}

// Reference lanes of one query tile exchange their k-th best scores when there
// are 2 to 16 of them (each reads the others' after every tile).
static size_t tc_lane_kth_bytes(int S, int64_t nq) {
    return (S >= 2 && S <= 16) ? ((size_t)S * nq * sizeof(uint32_t) + 15) / 16 * 16 : 0;
}

// share = 0: a pair shares reference blocks (neighbouring query tiles, G even);
// share = 1: a pair shares query blocks (neighbouring reference lanes, S even).
// Pair MMAs default to two reference lanes (G = SMs / 2): the two CTAs on a query
// tile read its blocks at about the same time, so half of the query re-reads hit L2.
struct TcShape {
    int n_qtiles = 0, n_rtiles = 0, G = 1, S = 1, n_groups = 0, CL = 1, share = 0;
};

// group / lanes > 0 override the group size and cap the lanes; no_quad keeps pairs.
static TcShape tc_plan(const hdc_context* ctx, int64_t nq, const hdc_refdb* db, int group = 0, int lanes = 0,
                       bool no_quad = false) {
    TcShape p;
    const int qt_rows = kBM * tc_m_blocks(ctx, db);
    p.n_qtiles = (int)((nq + qt_rows - 1) / qt_rows);
    p.n_rtiles = (int)(db->r_pad / tc_tile_n(ctx, db));
    p.CL = tc_cluster(ctx, db);
    p.share = p.CL == 2 ? (ctx->tc_share >= 0 ? ctx->tc_share : tc_default_share()) : 0;
    const int want = group > 0            ? group
                     : ctx->tc_group > 0 ? ctx->tc_group
                     : (p.share || (p.CL == 2 && tc_pair_mma(ctx, db))) ? ctx->num_sms / 2
                                                                          : tc_default_group();
    p.G = std::max(1, std::min(std::min(want, ctx->num_sms), p.n_qtiles));
    if (p.CL == 2 && !p.share) {
        if (p.G >= 2 && (p.G & 1)) --p.G;
        if (p.G < 2) p.CL = 1;
    }
    p.S = std::max(1, ctx->num_sms / p.G);
    if (ctx->tc_lanes > 0) p.S = std::min(p.S, ctx->tc_lanes);
    if (lanes > 0) p.S = std::min(p.S, lanes);
    p.S = std::min(p.S, p.n_rtiles);
    // clusters of 4 (pair MMAs on two reference lanes): G and S even
    if (!no_quad && p.CL == 2 && !p.share && p.G >= 2 && p.S >= 2 && tc_pair_mma(ctx, db) &&
        (ctx->tc_cluster > 0 ? ctx->tc_cluster : tc_default_cluster()) == 4) {
        p.CL = 4;
        p.S &= ~1;
    }
    if (p.CL == 2 && p.share) {
        p.S &= ~1;
        if (p.S < 2) {
            p.CL = 1;
            p.share = 0;
            p.S = std::max(1, std::min(ctx->num_sms / p.G, p.n_rtiles));
        }
    }
    p.n_groups = (p.n_qtiles + p.G - 1) / p.G;
    return p;
}

// Workspace of one launch: S partial lists per query, then the lanes' k-th scores.
static size_t tc_part_bytes(const TcShape& p, int64_t nq, int k) {
    return (size_t)p.S * nq * k * (sizeof(uint64_t) + sizeof(int64_t)) + tc_lane_kth_bytes(p.S, nq);
}

static int quad_clusters_fit(const hdc_context* ctx);

// Clusters of 4 may fit on fewer SMs than the grid of the plan (on GB300, 36
// clusters of 4 = 144 of the 152 SMs).  Then the leading whole groups of the
// largest even size that fits run as clusters of 4 and the remaining queries as
// pairs on every SM.  Returns the number of leading queries for clusters of 4
// (nq: all of them, 0: none) and their group size and lanes.
// With the cluster size left automatic, clusters of 4 are used up to k = 16: past that the
// epilogue's exact scores bound the kernel, and clusters of 4, which hold two pairs' MMAs in
// step, pass each pair's epilogue stalls on to the other (k = 32: 4 % slower than pairs).
constexpr int kQuadMaxK = 16;

static int64_t tc_quad_queries(const hdc_context* ctx, int64_t nq, const hdc_refdb* db, int k, int& G4, int& S4) {
    const TcShape p = tc_plan(ctx, nq, db);
    G4 = p.G;
    S4 = p.S;
    if (p.CL != 4 || (ctx->tc_cluster <= 0 && k > kQuadMaxK)) return 0;
    const int fit = quad_clusters_fit(ctx);
    if (fit * 4 >= p.G * p.S) return nq;
    G4 = 2 * (fit / (p.S / 2));
    if (G4 < 2) return 0;
    const int64_t rows = (int64_t)G4 * kBM;
    return nq / rows * rows;
}

size_t tc_workspace_bytes(const hdc_context* ctx, int64_t nq, const hdc_refdb* db, int k) {
    k = std::max(1, (int)std::min<int64_t>(k, db->nr));
    int G4, S4;
    const int64_t n4 = tc_quad_queries(ctx, nq, db, k, G4, S4);
    if (n4 == nq) return tc_part_bytes(tc_plan(ctx, nq, db), nq, k);
    if (n4 == 0) return tc_part_bytes(tc_plan(ctx, nq, db, 0, 0, true), nq, k);
    return tc_part_bytes(tc_plan(ctx, n4, db, G4, S4), n4, k) +
           tc_part_bytes(tc_plan(ctx, nq - n4, db, 0, 0, true), nq - n4, k);
}

constexpr int kNoClusterFit = -1;  // launch_tc_t: the clusters cannot all be resident
// dynamic shared memory a CTA may opt into (227 KB), less 1 KB for the kernel's static
// shared memory (its mbarriers and flags)
constexpr size_t kMaxDynSmem = 226 * 1024;

template <int L, int N, int MB, int CL, bool SHARE_A = false, int BKT = Tile<N>::BK, bool PAIR_MMA = false,
          int KR = 0>
static int launch_tc_t(const __half* d_q, const hdc_refdb* db, const TcArgs& a, int grid, cudaStream_t stream) {
    CUtensorMap tmA, tmB;
    // with CL CTAs sharing a block by multicast, each loads 1 / CL of its rows; with pair
    // MMAs each CTA loads whole blocks of its own
    constexpr bool QUAD = PAIR_MMA && CL == 4;  // query blocks loaded in halves, one by each pair
    if (!make_tmap(&tmA, d_q, a.nq, a.dim, BKT, SHARE_A ? kBM / CL : QUAD ? kBM / 2 : kBM) ||
        !make_tmap(&tmB, db->d_limbs, (int64_t)db->L * db->r_pad, a.dim, BKT, (SHARE_A || PAIR_MMA) ? N : N / CL))
        return fail(HDC_ERR_CUDA, "tc search: cuTensorMapEncodeTiled failed");
    constexpr int LS = PAIR_MMA ? 1 : L;
    const size_t ring = (size_t)tc_stages<N, BKT>(LS, MB) * tc_stage_bytes<N, BKT>(LS, MB) + 1024;
    // the top-k lists (k keys + k dots per query row) go into shared memory when they fit
    const size_t lists = (size_t)MB * a.k * kBM * (sizeof(uint64_t) + sizeof(int64_t));
    TcArgs args = a;
    args.slist = ring + lists <= kMaxDynSmem ? 1 : 0;
    const size_t smem = ring + (args.slist ? lists : 0);
    auto kern = tc_search_kernel<L, N, MB, CL, SHARE_A, BKT, PAIR_MMA, KR>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "tc search: cudaFuncSetAttribute");
    if constexpr (CL == 1) {
        kern<<<grid, kThreadsTC, smem, stream>>>(tmA, tmB, args);
    } else {
        if (grid % CL) return fail(HDC_ERR_INVALID, "tc search: grid is not a whole number of clusters");
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)grid, 1, 1);
        cfg.blockDim = dim3(kThreadsTC, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if constexpr (CL > 2) {
            // the persistent grid needs every cluster resident at once: otherwise run pairs
            int fit = 0;
            e = cudaOccupancyMaxActiveClusters(&fit, kern, &cfg);
            if (e != cudaSuccess || fit * CL < grid) {
                cudaGetLastError();
                return kNoClusterFit;
            }
        }
        e = cudaLaunchKernelEx(&cfg, kern, tmA, tmB, args);
        if (e != cudaSuccess) return cuda_fail(e, "tc search: cluster launch");
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "tc search: launch");
}

// One launch of the search over queries [0, nq) of d_q with the schedule p.
static int search_part(hdc_context* ctx, const hdc_refdb* db, const __half* d_q, const int64_t* d_qn, int64_t nq, int k,
                       int mode, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot, void* d_work,
                       size_t work_bytes, int* d_status, cudaStream_t stream, const TcShape& p, bool record) {
    const int N = tc_tile_n(ctx, db);
    TcArgs a{};
    a.nq = nq;
    a.nr = db->nr;
    a.dim = ctx->dim;
    a.k = k;
    a.mode = mode;
    const bool kb32 = tc_kb32(ctx, db);
    const int bk = (N == 256 || kb32) ? 32 : 64;
    a.n_kblocks = (ctx->dim + bk - 1) / bk;
    a.r_pad = db->r_pad;
    int CL = p.CL;
    const int share = p.share;
    a.n_qtiles = p.n_qtiles;
    a.n_rtiles = p.n_rtiles;
    a.G = p.G;
    a.S = p.S;
    a.n_groups = p.n_groups;
    a.qn = d_qn;
    a.rr = db->d_rsq;
    const size_t lists = (size_t)a.S * nq * k * (sizeof(uint64_t) + sizeof(int64_t));
    const size_t kth_bytes = tc_lane_kth_bytes(a.S, nq);
    if (!d_work || work_bytes < lists + kth_bytes) return fail(HDC_ERR_INVALID, "tc search: workspace too small");
    a.ws_key = static_cast<uint64_t*>(d_work);
    a.ws_dot = reinterpret_cast<int64_t*>(a.ws_key + (size_t)a.S * nq * k);
    a.lane_kth = kth_bytes ? reinterpret_cast<uint32_t*>(static_cast<uint8_t*>(d_work) + lists) : nullptr;
    if (a.lane_kth) {
        cudaError_t e = cudaMemsetAsync(a.lane_kth, 0, kth_bytes, stream);
        if (e != cudaSuccess) return cuda_fail(e, "tc search: clear lane thresholds");
    }
    a.rs = db->d_sqrt;
    a.ri = db->d_sqrt + db->nr;
    a.limb_bits = db->limb_bits;
    a.limb_base = (float)(1 << db->limb_bits);
    a.status = d_status;
    a.wait_cycles = ctx->wait_cycles > 0 ? ctx->wait_cycles : tc::kWaitCycles;
    a.withhold = ctx->test_withhold_loads;
    a.policy = ctx->tc_policy >= 0 ? ctx->tc_policy : tc_default_policy();
    a.prefetch = ctx->tc_prefetch >= 0 ? ctx->tc_prefetch : tc_default_prefetch();
    a.t_stride = (ctx->tc_scatter >= 0 ? ctx->tc_scatter : tc_default_scatter()) ? tile_stride(a.n_rtiles) : 1;
    const int grid = a.G * a.S;
    int st;
    const int MB = tc_m_blocks(ctx, db);
    const bool pair_mma = CL == 2 && !share && tc_pair_mma(ctx, db);
    // register-resident lists for 8 < k <= 16 (measured on 200,000 references of
    // D = 10,240: top-10 194.9K -> 200.6K reads/s, top-5 219.2K -> 215.1K, so
    // k <= 8 keeps the shared-memory lists)
    const bool kreg = k > 8 && k <= 16;
    if (N == 256) {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 256, 1, 1>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<2, 256, 1, 1>(d_q, db, a, grid, stream); break;
        }
    } else if (MB == 2) {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 128, 2, 1>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<2, 128, 2, 1>(d_q, db, a, grid, stream); break;
        }
    } else if (CL == 2 && share) {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 128, 1, 2, true>(d_q, db, a, grid, stream); break;
            case 2: st = launch_tc_t<2, 128, 1, 2, true>(d_q, db, a, grid, stream); break;
            case 3: st = launch_tc_t<3, 128, 1, 2, true>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<4, 128, 1, 2, true>(d_q, db, a, grid, stream); break;
        }
    } else if (CL == 4) {
        st = kreg ? launch_tc_t<2, 128, 1, 4, false, 64, true, 16>(d_q, db, a, grid, stream)
                     : launch_tc_t<2, 128, 1, 4, false, 64, true>(d_q, db, a, grid, stream);
        if (st == kNoClusterFit) {
            CL = 2;
            st = kreg ? launch_tc_t<2, 128, 1, 2, false, 64, true, 16>(d_q, db, a, grid, stream)
                         : launch_tc_t<2, 128, 1, 2, false, 64, true>(d_q, db, a, grid, stream);
        }
    } else if (CL == 2 && pair_mma) {
        st = kreg ? launch_tc_t<2, 128, 1, 2, false, 64, true, 16>(d_q, db, a, grid, stream)
                     : launch_tc_t<2, 128, 1, 2, false, 64, true>(d_q, db, a, grid, stream);
    } else if (CL == 2 && kb32) {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 128, 1, 2, false, 32>(d_q, db, a, grid, stream); break;
            case 2: st = launch_tc_t<2, 128, 1, 2, false, 32>(d_q, db, a, grid, stream); break;
            case 3: st = launch_tc_t<3, 128, 1, 2, false, 32>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<4, 128, 1, 2, false, 32>(d_q, db, a, grid, stream); break;
        }
    } else if (CL == 2) {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 128, 1, 2>(d_q, db, a, grid, stream); break;
            case 2: st = launch_tc_t<2, 128, 1, 2>(d_q, db, a, grid, stream); break;
            case 3: st = launch_tc_t<3, 128, 1, 2>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<4, 128, 1, 2>(d_q, db, a, grid, stream); break;
        }
    } else {
        switch (db->L) {
            case 1: st = launch_tc_t<1, 128, 1, 1>(d_q, db, a, grid, stream); break;
            case 2: st = launch_tc_t<2, 128, 1, 1>(d_q, db, a, grid, stream); break;
            case 3: st = launch_tc_t<3, 128, 1, 1>(d_q, db, a, grid, stream); break;
            default: st = launch_tc_t<4, 128, 1, 1>(d_q, db, a, grid, stream); break;
        }
    }
    if (st != HDC_OK) return st;
    if (record) {
        ctx->tc_last_shape[0] = CL;
        ctx->tc_last_shape[1] = a.G;
        ctx->tc_last_shape[2] = a.S;
        ctx->tc_last_shape[3] = (CL == 4 || pair_mma || (CL == 2 && tc_pair_mma(ctx, db) && !share)) ? 1 : 0;
        ctx->tc_last_shape[4] = 0;
    }
    ctx->tc_last_shape[4] += 2;  // the search kernel and its merge
    return launch_merge(a.ws_key, a.ws_dot, a.S, nq, k, d_qn, db->d_norm2, db->nr, d_score, d_idx, d_cos, d_dot,
                        stream);
}


static int quad_clusters_fit(const hdc_context* ctx) {
    if (ctx->tc_quad_fit >= 0) return ctx->tc_quad_fit;
    auto kern = tc_search_kernel<2, 128, 1, 4, false, 64, true, 0>;
    const size_t smem = (size_t)tc_stages<128, 64>(1, 1) * tc_stage_bytes<128, 64>(1, 1) + 1024;
    int fit = 0;
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) == cudaSuccess) {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(4 * (unsigned)ctx->num_sms, 1, 1);
        cfg.blockDim = dim3(kThreadsTC, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 4;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        if (cudaOccupancyMaxActiveClusters(&fit, kern, &cfg) != cudaSuccess) fit = 0;
    }
    cudaGetLastError();
    ctx->tc_quad_fit = fit;  // a cache of a device property
    return fit;
}

int launch_search_tc(hdc_context* ctx, const hdc_refdb* db, const __half* d_q, const int64_t* d_qn, int64_t nq,
                     int32_t maxq, int k, int mode, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot,
                     void* d_work, size_t work_bytes, int* d_status, cudaStream_t stream) {
    if (nq == 0) return HDC_OK;
    if (db->dim != ctx->dim) return fail(HDC_ERR_INVALID, "tc search: database and context dims differ");
    if (k > db->nr) k = (int)db->nr;
    if (k < 1 || k > kMaxKTC) return fail(HDC_ERR_INVALID, "tc search: k must be in 1..32");
    if (maxq < 0 || maxq > 2048) return fail(HDC_ERR_RANGE, "tc search: queries must be integers with |q| <= 2048");
    for (int l = 0; l < db->L; ++l) {
        const double bound = (double)ctx->dim * std::max(maxq, 1) * std::max(db->limb_max[l], 1);
        if (bound > 16777216.0)
            return fail(HDC_ERR_RANGE, "tc search: dim * max|q| * max|limb| exceeds 2^24 (fp32 accumulators inexact)");
    }
    if ((reinterpret_cast<uintptr_t>(d_q) & 15) != 0) return fail(HDC_ERR_INVALID, "tc search: queries not 16B aligned");
    int G4, S4;
    const int64_t n4 = tc_quad_queries(ctx, nq, db, k, G4, S4);
    if (n4 == nq)
        return search_part(ctx, db, d_q, d_qn, nq, k, mode, d_score, d_idx, d_cos, d_dot, d_work, work_bytes, d_status,
                           stream, tc_plan(ctx, nq, db), true);
    const TcShape rest = tc_plan(ctx, nq - n4, db, 0, 0, true);
    if (n4 == 0)
        return search_part(ctx, db, d_q, d_qn, nq, k, mode, d_score, d_idx, d_cos, d_dot, d_work, work_bytes, d_status,
                           stream, rest, true);
    // leading whole groups as clusters of 4, the remaining queries as pairs
    const TcShape lead = tc_plan(ctx, n4, db, G4, S4);
    const size_t w4 = tc_part_bytes(lead, n4, k);
    if (!d_work || work_bytes < w4 + tc_part_bytes(rest, nq - n4, k))
        return fail(HDC_ERR_INVALID, "tc search: workspace too small");
    int st = search_part(ctx, db, d_q, d_qn, n4, k, mode, d_score, d_idx, d_cos, d_dot, d_work, w4, d_status, stream,
                         lead, true);
    if (st != HDC_OK) return st;
    const int64_t o = n4;  // outputs the caller does not want stay null
    return search_part(ctx, db, d_q + o * ctx->dim, d_qn + o, nq - n4, k, mode, d_score ? d_score + o * k : nullptr,
                       d_idx ? d_idx + o * k : nullptr, d_cos ? d_cos + o * k : nullptr,
                       d_dot ? d_dot + o * k : nullptr, static_cast<uint8_t*>(d_work) + w4, work_bytes - w4, d_status,
                       stream, rest, false);
}

}  // namespace hdc
