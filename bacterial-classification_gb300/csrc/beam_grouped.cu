// Hierarchical descent with the reads of a batch grouped by candidate node.
//
// Same semantics as the one-warp-per-read descent (beam.cu, the level loop of
// targets/identify.cpp:89-202 with one prototype per node), computed level by
// level for the whole batch:
//   1. count + expand: every live read lists its candidates (level 0: the
//      roots; later: the children of its beam entries, a node without
//      children itself), one (read, node, beam slot) pair each;
//   2. the pairs are counting-sorted by node;
//   3. score: one warp per pair, the warps walking the pairs in node order so
//      the pairs of a node meet its prototype row in L1/L2, each computing the
//      read's exact int64 dot from its packed +1/-1 bits (each element adds +p
//      or -p);
//   4. select: per read, the `beam` best candidates by make_key(score, node)
//      (ties to the lower node index), the threshold stop and the new beam
//      rows, exactly as the per-read kernel.
// A prototype row is then read from memory once per level for the batch
// instead of once per read that needs it, and a read costs 2 KB of bits
// (D = 16,384) instead of a 64 KB row per candidate.
#include "hdc_internal.cuh"
#include "tc_ptx.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kMaxBeamG = 8;
constexpr int kMaxLevelsG = 8;
constexpr int kScoreThreads = 256;          // 8 warps, one pair each at a time
constexpr int kScoreBlocks = 8;             // resident per SM; the grid is one wave
constexpr int kScoreBlocks16 = 5;           // the same with int16 rows (48 registers a thread)
constexpr int kScanItems = 16;              // elements per thread of the scan
constexpr int kScanBlock = 256 * kScanItems;

// ---------------------------------------------------------------- exclusive scan (int32)
// out[i] = sum(in[0..i)) for i <= n; block sums go through `sums` (ceil(n / 4096) entries).
__device__ __forceinline__ int32_t block_scan_excl(int32_t v, int32_t* sh, int32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int32_t w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    const int32_t before = (warp ? sh[warp - 1] : 0) + x - v;
    if (total) *total = sh[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before;
}

__global__ void scan_block_sums(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int32_t sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int32_t v = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) v += in[base + i];
    int32_t total;
    block_scan_excl(v, sh, &total);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_sums(int32_t* __restrict__ sums, int64_t nb) {  // one block, nb <= kScanBlock
    __shared__ int32_t sh[32];
    const int64_t base = (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < nb ? sums[base + i] : 0;
        s += v[i];
    }
    int32_t run = block_scan_excl(s, sh, nullptr);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < nb) {
            sums[base + i] = run;
            run += v[i];
        }
}

__global__ void scan_apply(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ sums,
                           int32_t* __restrict__ out) {
    __shared__ int32_t sh[32];
    const int64_t base = (int64_t)blockIdx.x * kScanBlock + (int64_t)threadIdx.x * kScanItems;
    int32_t v[kScanItems], s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        v[i] = base + i < n ? in[base + i] : 0;
        s += v[i];
    }
    int32_t total;
    int32_t run = sums[blockIdx.x] + block_scan_excl(s, sh, &total);
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) {
            out[base + i] = run;
            run += v[i];
        }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) out[n] = sums[blockIdx.x] + total;
}

int scan_blocks_needed(int64_t n) { return (int)((n + kScanBlock - 1) / kScanBlock); }

// out has n + 1 entries; sums has scan_blocks_needed(n) entries (n <= 4096 * 4096)
void exclusive_scan(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, cudaStream_t stream) {
    const int nb = scan_blocks_needed(n);
    scan_block_sums<<<nb, 256, 0, stream>>>(in, n, sums);
    scan_sums<<<1, 256, 0, stream>>>(sums, nb);
    scan_apply<<<nb, 256, 0, stream>>>(in, n, sums, out);
}

// ---------------------------------------------------------------- reads as bits
// bit b of word w of read r: q[r][32 w + b] > 0
__global__ void pack_bits_kernel(const int8_t* __restrict__ q, int64_t nq, int dim, uint32_t* __restrict__ bits) {
    const int words = dim / 32;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq * words) return;
    const int8_t* p = q + (i / words) * dim + (i % words) * 32;
    const int4 a = *reinterpret_cast<const int4*>(p), b = *reinterpret_cast<const int4*>(p + 16);
    const uint32_t w8[8] = {(uint32_t)a.x, (uint32_t)a.y, (uint32_t)a.z, (uint32_t)a.w,
                            (uint32_t)b.x, (uint32_t)b.y, (uint32_t)b.z, (uint32_t)b.w};
    uint32_t m = 0;
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int8_t v = (int8_t)(w8[j >> 2] >> (8 * (j & 3)));
        m |= (v > 0 ? 1u : 0u) << j;
    }
    bits[i] = m;
}

__global__ void max_children_kernel(const int64_t* __restrict__ child_ptr, int64_t n_nodes, int32_t* __restrict__ out) {
    int32_t m = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (int32_t)(child_ptr[i + 1] - child_ptr[i]));
    for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// ---------------------------------------------------------------- descent state
struct GArgs {
    int64_t nq;
    int dim, words, steps, levels, beam, mode, n_roots;
    int64_t n_nodes;
    double threshold;
    const uint32_t* bits;     // [nq][words]
    const int64_t* qn;        // [nq]
    const int32_t* proto;     // [n32][dim] int32 rows of nodes < n32
    const int16_t* proto16;   // [n_nodes - n32][dim] int16 rows of nodes >= n32 (row node - n32)
    int64_t n32;
    const int64_t* pn;        // [n_nodes]
    const int64_t* child_ptr;
    const int32_t* child_idx;
    const int32_t* roots;
    int32_t* paths;           // [nq][kMaxBeamG][kMaxLevelsG] node of beam row b at level l
    float* scores;            // same shape
    int32_t* nbeam;           // [nq]
    int32_t* done;            // [nq] 1 once the read stopped or ran every level
    int32_t* out_depth;       // [nq]
    int32_t* cnt;             // [nq] candidates of this level
    int32_t* off;             // [nq + 1] their offsets (exclusive scan of cnt)
    int32_t* node_cnt;        // [n_nodes]
    int32_t* node_off;        // [n_nodes + 1]
    int32_t* cursor;          // [n_nodes]
    int32_t* pair_read;       // [P]
    int32_t* pair_node;       // [P]
    int32_t* pair_slot;       // [P] beam row the candidate expands
    uint64_t* pair_key;       // [P]
    int32_t* sorted;          // [P] pair indices ordered by node
    int64_t* part;            // [kQuarters][pstride] partial dots of a streamed level (one-launch form)
    int64_t pstride;
    long long wait_cycles;    // limit of the descent's bounded waits (SM cycles)
};

// A caller-given largest child count below the tree's sizes the pair arrays too small: every
// read is marked done before level 0 (no candidates, depth 0) and the context status records
// kStatusChildCount.
constexpr int kStatusChildCount = 200;
__global__ void check_children_kernel(const GArgs a, const int32_t* __restrict__ maxc, int32_t given, int* status) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (*maxc <= given || r >= a.nq) return;
    a.done[r] = 1;
    if (r == 0) atomicCAS(status, 0, kStatusChildCount);
}

__device__ __forceinline__ int64_t state_at(int64_t r, int b, int l) {
    return (r * kMaxBeamG + b) * kMaxLevelsG + l;
}

// candidates of read r at level L (0 once it is done)
__device__ __forceinline__ int32_t count_one(const GArgs& a, int L, int64_t r) {
    int32_t c = 0;
    if (!a.done[r]) {
        if (L == 0) {
            c = a.n_roots;
        } else {
            for (int b = 0; b < a.nbeam[r]; ++b) {
                const int32_t node = a.paths[state_at(r, b, L - 1)];
                const int64_t k = a.child_ptr[node + 1] - a.child_ptr[node];
                c += k ? (int32_t)k : 1;  // a node without children scores itself again
            }
        }
    }
    return c;
}

__global__ void count_kernel(const GArgs a, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
    a.cnt[r] = count_one(a, L, r);
}

// atomicAdd(ctr + node, 1) for the calling lanes, one atomic per distinct node of the warp
// (the levels near the root have few nodes, each counted by most reads: the atomics on one
// address serialise); returns the old value plus the lane's rank among its node's lanes.
__device__ __forceinline__ int32_t warp_count(int32_t* ctr, int32_t node) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, node);
    const int lane = threadIdx.x & 31, leader = __ffs(peers) - 1;
    int32_t base = 0;
    if (lane == leader) base = atomicAdd(ctr + node, __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + __popc(peers & ((1u << lane) - 1u));
}

// count_nodes: the level is scored from node-sorted pairs (score_kernel), which need the
// pairs per node; a tensor-core level groups the entries by parent instead
__device__ __forceinline__ void put_pair(const GArgs& a, int32_t p, int64_t r, int32_t node, int slot,
                                         bool count_nodes) {
    a.pair_read[p] = (int32_t)r;
    a.pair_node[p] = node;
    a.pair_slot[p] = slot;
    if (count_nodes) atomicAdd(a.node_cnt + node, 1);
}

// The pairs of beam entry b of read r (level 0: b = 0 writes the roots), at a.off[r] plus the
// candidates of the entries before it: one thread per (read, entry), so the entries' dependent
// loads (path, child range, children) run side by side.  With par_cnt set (a tensor-core level
// above 0), the entry also counts itself to its parent.
__device__ __forceinline__ void expand_entry(const GArgs& a, int L, int64_t r, int b, bool count_nodes,
                                             int32_t* par_cnt) {
    if (a.done[r]) return;
    if (L == 0) {
        if (b == 0) {
            int32_t p = a.off[r];
            for (int i = 0; i < a.n_roots; ++i) put_pair(a, p++, r, a.roots[i], 0, count_nodes);
        }
        return;
    }
    const int nb = a.nbeam[r];
    if (b >= nb) return;
    int32_t p = a.off[r];
    for (int e = 0; e < b; ++e) {
        const int32_t prev = a.paths[state_at(r, e, L - 1)];
        const int64_t k = a.child_ptr[prev + 1] - a.child_ptr[prev];
        p += k ? (int32_t)k : 1;
    }
    const int32_t node = a.paths[state_at(r, b, L - 1)];
    if (par_cnt) warp_count(par_cnt, node);
    const int64_t c0 = a.child_ptr[node], c1 = a.child_ptr[node + 1];
    if (c0 == c1) {
        put_pair(a, p, r, node, b, count_nodes);
    } else {
        for (int64_t c = c0; c < c1; ++c) put_pair(a, p++, r, a.child_idx[c], b, count_nodes);
    }
}

__global__ void expand_kernel(const GArgs a, int L, bool count_nodes) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nq * a.beam) return;
    expand_entry(a, L, i / a.beam, (int)(i % a.beam), count_nodes, nullptr);
}

// pairs p = first, first + stride, ... to their node-ordered slots
__device__ __forceinline__ void scatter_range(const GArgs& a, int64_t first, int64_t stride) {
    const int32_t total = a.off[a.nq];
    for (int64_t p = first; p < total; p += stride) {
        const int32_t pos = atomicAdd(a.cursor + a.pair_node[p], 1);
        a.sorted[pos] = (int32_t)p;
    }
}

__global__ void scatter_kernel(const GArgs a) {
    scatter_range(a, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// One warp per pair, the warps walking the pairs in node order: the pairs of a node are
// scored by neighbouring warps at about the same time, so its prototype row comes from
// DRAM once and from L1/L2 for the others.  Four 16-byte prototype loads are in flight per
// lane, and the read is its packed bits.  With int16 rows (about twice the pairs per second)
// the FP64 scores are computed 32 pairs at a time, one per lane: the warp keeps pair i's dot
// in lane i mod 32.
// -x in 32 bits, with wrap-around defined (exact for every prototype element but INT32_MIN,
// which hdc_beam_search excludes; widening before negating costs ~40 % of the kernel)
__device__ __forceinline__ int32_t neg32(int32_t x) { return (int32_t)(0u - (uint32_t)x); }

// Lane l's share of the dot of an int32 row: dims 128 j + 4 l .. + 3.
constexpr int kRowPrefetch = 2;  // blocks of a row prefetched into L2 ahead of its loads

__device__ __forceinline__ int64_t lane_dot32(const GArgs& a, int lane, int32_t node, int64_t r) {
    const int nsteps = a.dim / 128;  // a multiple of 8 (dim % 1024 == 0)
    const int sh = (lane & 7) * 4;
    const int32_t* row0 = a.proto + (int64_t)node * a.dim;
    const int32_t* row = row0 + 4 * lane;
    const uint32_t* qb = a.bits + r * a.words + (lane >> 3);
    // lane 0 prefetches the row into L2 kRowPrefetch blocks of 4 steps (2 KB) ahead
    const int nblk = nsteps / 4;
    auto prefetch = [&](int q) {
        if (lane == 0 && q < nblk) tc::prefetch_l2(row0 + (size_t)q * 512, 2048);
    };
    for (int q = 0; q < kRowPrefetch; ++q) prefetch(q);
    if (a.pn[node] < ((int64_t)1 << 44)) {
        // every |p| < 2^22, so a lane's (at most 512) terms sum below 2^31: int32 throughout
        int32_t acc32 = 0;
        for (int j = 0; j < nsteps; j += 4) {
            prefetch(j / 4 + kRowPrefetch);
            int4 x[4];
            uint32_t w[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                x[u] = __ldg(reinterpret_cast<const int4*>(row + 128 * (j + u)));
                w[u] = __ldg(qb + 4 * (j + u));
            }
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t nib = w[u] >> sh;
                acc32 += ((nib & 1u) ? x[u].x : -x[u].x) + ((nib & 2u) ? x[u].y : -x[u].y) +
                         ((nib & 4u) ? x[u].z : -x[u].z) + ((nib & 8u) ? x[u].w : -x[u].w);
            }
        }
        return acc32;
    }
    int64_t acc = 0;
    for (int j = 0; j < nsteps; j += 4) {
        prefetch(j / 4 + kRowPrefetch);
        int4 x[4];
        uint32_t w[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            x[u] = __ldg(reinterpret_cast<const int4*>(row + 128 * (j + u)));
            w[u] = __ldg(qb + 4 * (j + u));
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const uint32_t nib = w[u] >> sh;
            acc += (int64_t)((nib & 1u) ? x[u].x : neg32(x[u].x)) + (int64_t)((nib & 2u) ? x[u].y : neg32(x[u].y)) +
                   (int64_t)((nib & 4u) ? x[u].z : neg32(x[u].z)) + (int64_t)((nib & 8u) ? x[u].w : neg32(x[u].w));
        }
    }
    return acc;
}

// Four sign bits (bit i set: +1) as four signed bytes +1 / -1: the bits spread to the low bit
// of each byte (the four shifted copies of the nibble do not overlap), then 1 -> 0x01 and
// 0 -> 0xFF by ~(b * 0xFE) per byte.
__device__ __forceinline__ int signs4_bytes(uint32_t nib) {
    return (int)~(((nib * 0x00204081u) & 0x01010101u) * 0xFEu);
}

// Lane l's share of the dot of an int16 row: dims 256 j + 8 l .. + 7 (one 16-byte load, one
// byte of the read's bits), U loads in flight, and lane 0 prefetching the row into L2
// kRowPrefetch blocks of U steps ahead (the loads of a block then find it there: 3.9 -> 3.55
// ms for the c5 leaf level; 4 blocks ahead was slower).  Each word holds two int16 values (the lower
// dim in the low half); dp2a multiplies them by two of the signed sign bytes and accumulates,
// exactly.  |p| <= 2^15 and at most 512 terms a lane: int32 throughout.
template <int U>
__device__ __forceinline__ int64_t lane_dot16_u(const GArgs& a, int lane, int32_t node, int64_t r) {
    const int nsteps = a.dim / 256;  // a multiple of U
    const int sh = (lane & 3) * 8;
    const int16_t* row16 = a.proto16 + (node - a.n32) * a.dim;
    const int4* row = reinterpret_cast<const int4*>(row16) + lane;
    const uint32_t* qb = a.bits + r * a.words + (lane >> 2);
    constexpr uint32_t kBlk = U * 512;  // the warp's row bytes of one block of U steps
    const int nblk = nsteps / U;
    if (lane == 0)
        for (int q = 0; q < kRowPrefetch && q < nblk; ++q) tc::prefetch_l2(row16 + (size_t)q * kBlk / 2, kBlk);
    int acc = 0;
    for (int j = 0; j < nsteps; j += U) {
        if (lane == 0 && j / U + kRowPrefetch < nblk) tc::prefetch_l2(row16 + (size_t)(j / U + kRowPrefetch) * kBlk / 2, kBlk);
        int4 x[U];
        uint32_t w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            x[u] = __ldg(row + 32 * (j + u));
            w[u] = __ldg(qb + 8 * (j + u));
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t byte = w[u] >> sh;
            const int s0 = signs4_bytes(byte & 15u), s1 = signs4_bytes((byte >> 4) & 15u);
            acc = __dp2a_lo(x[u].x, s0, acc);  // dims 0, 1
            acc = __dp2a_hi(x[u].y, s0, acc);  // dims 2, 3
            acc = __dp2a_lo(x[u].z, s1, acc);  // dims 4, 5
            acc = __dp2a_hi(x[u].w, s1, acc);  // dims 6, 7
        }
    }
    return acc;
}

// eight loads in flight where the row has a multiple of 8 steps (dim % 2048 == 0), else four
// (dim % 1024 == 0 gives a multiple of 4)
__device__ __forceinline__ int64_t lane_dot16(const GArgs& a, int lane, int32_t node, int64_t r) {
    return (a.dim / 256) % 8 == 0 ? lane_dot16_u<8>(a, lane, node, r) : lane_dot16_u<4>(a, lane, node, r);
}

// ROWS16: some nodes have int16 rows (hdc_beam_search_split); without, the kernel is the
// int32 one alone (fewer registers, every warp slot of the SM resident)
// Warp w of nw scores the node-ordered pairs w, w + nw, ...
template <bool ROWS16>
__device__ __forceinline__ void score_pairs(const GArgs& a, int64_t w, int64_t nw) {
    const int lane = threadIdx.x & 31;
    const int32_t total = a.off[a.nq];
    int32_t my_pi = -1, my_node = 0;
    int64_t my_r = 0, my_dot = 0;
    int i = 0;
    for (int64_t s = w; s < total; s += nw, ++i) {
        const int32_t pi = a.sorted[s];
        const int32_t node = a.pair_node[pi];
        const int64_t r = a.pair_read[pi];
        int64_t acc = ROWS16 && node >= a.n32 ? lane_dot16(a, lane, node, r) : lane_dot32(a, lane, node, r);
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (!ROWS16) {  // the int32 kernel scores on lane 0 (holding 32 pairs would spill at 32 registers)
            if (lane == 0) a.pair_key[pi] = make_key(exact_score(acc, a.qn[r], a.pn[node], a.mode), (uint32_t)node);
            continue;
        }
        if (lane == (i & 31)) {
            my_pi = pi;
            my_node = node;
            my_r = r;
            my_dot = acc;
        }
        if ((i & 31) == 31 && my_pi >= 0) {
            a.pair_key[my_pi] = make_key(exact_score(my_dot, a.qn[my_r], a.pn[my_node], a.mode), (uint32_t)my_node);
            my_pi = -1;
        }
    }
    if (my_pi >= 0)
        a.pair_key[my_pi] = make_key(exact_score(my_dot, a.qn[my_r], a.pn[my_node], a.mode), (uint32_t)my_node);
}

template <bool ROWS16>
__global__ void __launch_bounds__(kScoreThreads, ROWS16 ? kScoreBlocks16 : kScoreBlocks) score_kernel(const GArgs a) {
    score_pairs<ROWS16>(a, (((int64_t)blockIdx.x * blockDim.x) >> 5) + (threadIdx.x >> 5),
                        ((int64_t)gridDim.x * blockDim.x) >> 5);
}

// Per read: the best `beam` candidates, then the rule of the per-read kernel (stop below
// the threshold with the best path, else keep the entries >= threshold, at most `beam`).
// A group of G lanes per read (G = 8: four reads a warp at once, their dependent loads
// overlapping), every lane of the group calling with the same r.  The candidates are ordered
// by key (descending), ties to the lower pair index (the order an insertion in pair order
// keeps); round t takes the group-wide first of those after round t - 1's pick, lane t keeps
// it.  The keys of the first 8 G pairs stay in registers (8 a lane), later ones are re-read
// each round.  The kept entries' paths are then copied lane-parallel: every old value is read
// before any is written (a new entry's path comes from its parent's slot, possibly another
// entry's).
constexpr int kSelCache = 8;

__device__ __forceinline__ bool key_before(uint64_t k, int32_t p, uint64_t bk, int32_t bp) {
    return k > bk || (k == bk && p < bp);
}

// lane: 0 .. G-1 within the group; gmask: the group's lanes in the warp
template <int G>
__device__ void select_group(const GArgs& a, int L, int64_t r, int lane, uint32_t gmask) {
    static_assert(G >= kMaxBeamG && (G & (G - 1)) == 0 && G <= 32, "a lane per kept entry");
    if (a.done[r]) return;
    const int32_t p0 = a.off[r], p1 = a.off[r + 1];
    uint64_t ck[kSelCache];
#pragma unroll
    for (int i = 0; i < kSelCache; ++i) {
        const int32_t p = p0 + lane + G * i;
        ck[i] = p < p1 ? __ldcg(a.pair_key + p) : 0;  // from L2: written by other SMs in this kernel
    }
    const bool more = p1 - p0 > G * kSelCache;
    uint64_t prev_k = 0, my_k = 0;
    int32_t prev_p = -1, my_p = -1;
    int n = 0;
    for (int t = 0; t < a.beam; ++t) {
        uint64_t bk = 0;
        int32_t bp = INT32_MAX;  // nothing found: loses to every candidate
        auto consider = [&](uint64_t k, int32_t p) {
            if ((t == 0 || key_before(prev_k, prev_p, k, p)) && key_before(k, p, bk, bp)) {
                bk = k;
                bp = p;
            }
        };
#pragma unroll
        for (int i = 0; i < kSelCache; ++i)
            if (p0 + lane + G * i < p1) consider(ck[i], p0 + lane + G * i);
        if (more)
            for (int32_t p = p0 + lane + G * kSelCache; p < p1; p += G) consider(__ldcg(a.pair_key + p), p);
#pragma unroll
        for (int o = G / 2; o; o >>= 1) {
            const uint64_t ok = __shfl_xor_sync(gmask, bk, o, G);
            const int32_t op = __shfl_xor_sync(gmask, bp, o, G);
            if (key_before(ok, op, bk, bp)) {
                bk = ok;
                bp = op;
            }
        }
        if (bp == INT32_MAX) break;  // no candidate left (the same on every lane of the group)
        if (lane == t) {
            my_k = bk;
            my_p = bp;
        }
        prev_k = bk;
        prev_p = bp;
        ++n;
    }
    const float my_s = key_score(my_k);
    int32_t my_node = 0, my_slot = 0;
    if (lane < n) {
        my_node = a.pair_node[my_p];
        my_slot = a.pair_slot[my_p];
    }
    const bool stop = n == 0 || (double)__shfl_sync(gmask, my_s, 0, G) < a.threshold;
    int keep;
    if (stop) {
        keep = n ? 1 : 0;  // the best candidate's path is the answer
    } else {
        const uint32_t base = __ffs(gmask) - 1;
        const uint32_t ok = (__ballot_sync(gmask, lane < n && (double)my_s >= a.threshold) & gmask) >> base;
        keep = __ffs(~ok) - 1;  // the leading entries >= threshold (n <= 8 < G + 1: ~ok has a set bit)
    }
    if (lane == 0) {
        if (stop) {
            a.out_depth[r] = n ? L + 1 : L;
            a.done[r] = 1;
        } else {
            a.nbeam[r] = keep;
            if (L == a.levels - 1) {
                a.out_depth[r] = a.levels;
                a.done[r] = 1;
            }
        }
    }
    // entry t's levels 0..L: lanes i, i + G, ... of the keep x (L + 1) values
    constexpr int H = kMaxBeamG * kMaxLevelsG / G;
    int32_t vp[H];
    float vs[H];
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int i = lane + G * h, t = i / (L + 1), l = i - t * (L + 1);
        const int src = t < kMaxBeamG ? t : 0;
        const int32_t slot = __shfl_sync(gmask, my_slot, src, G);
        const int32_t node = __shfl_sync(gmask, my_node, src, G);
        const float sc = __shfl_sync(gmask, my_s, src, G);
        vp[h] = node;
        vs[h] = sc;
        if (t < keep && l < L) {
            vp[h] = a.paths[state_at(r, slot, l)];
            vs[h] = a.scores[state_at(r, slot, l)];
        }
    }
    __syncwarp(gmask);
#pragma unroll
    for (int h = 0; h < H; ++h) {
        const int i = lane + G * h, t = i / (L + 1), l = i - t * (L + 1);
        if (t < keep) {
            a.paths[state_at(r, t, l)] = vp[h];
            a.scores[state_at(r, t, l)] = vs[h];
        }
    }
}

constexpr int kSelLanes = 8;  // lanes per read in every select

// The reads first, first + stride, ... of a warp's share: each group of kSelLanes lanes takes
// every (32 / kSelLanes)-th of them.  `fin` (optional) runs on the group's lane 0 after a read's
// beam is taken.
template <int G = kSelLanes, class Fin>
__device__ __forceinline__ void select_reads(const GArgs& a, int L, int64_t first, int64_t end, int64_t stride,
                                             Fin fin) {
    constexpr int kGroups = 32 / G;
    const int lane = threadIdx.x & 31, grp = lane / G, gl = lane % G;
    const uint32_t gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << (grp * G);
    for (int64_t r = first + grp * stride; r < end; r += kGroups * stride) {
        select_group<G>(a, L, r, gl, gmask);
        __syncwarp(gmask);
        if (gl == 0) fin(r);
    }
}

// a group of kSelLanes lanes per read
__global__ void select_kernel(const GArgs a, int L) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    select_reads(a, L, w, a.nq, ((int64_t)gridDim.x * blockDim.x) >> 5, [](int64_t) {});
}

__device__ __forceinline__ void output_one(const GArgs& a, int64_t r, int32_t* path, float* path_score,
                                           int32_t* depth) {
    const int d = a.out_depth[r];
    for (int l = 0; l < a.levels; ++l) {
        path[r * a.levels + l] = l < d ? a.paths[state_at(r, 0, l)] : -1;
        path_score[r * a.levels + l] = l < d ? a.scores[state_at(r, 0, l)] : 0.0f;
    }
    depth[r] = d;
}

__global__ void output_kernel(const GArgs a, int32_t* __restrict__ path, float* __restrict__ path_score,
                              int32_t* __restrict__ depth) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
    output_one(a, r, path, path_score, depth);
}

// ---------------------------------------------------------------- tensor-core scoring
// Levels above the leaves score on the tensor cores, grouped by parent: the entries (read,
// beam slot) whose beam row is node P are scored against P's children (a childless P
// against itself) as one dense [entries] x [children] product.  A work item is up to 128
// entries x 32 children of one parent.  Producer warps, in groups of four taking every G-th K
// block (TcLayout: three groups in the level kernel, two in the one-launch kernel), write the
// entries' +1/-1 signs (from the packed bits) as fp16 straight into TMEM with tcgen05.st (the
// A operand: lane = entry, two signs a column), and the children's int32
// prototype rows, split into three balanced base-2048 fp16 limbs, into 128-byte-swizzled
// shared memory (the B operand); one thread issues M128 x N96 x K16 tcgen05 MMAs with A from
// TMEM, the three limb tiles side by side, into one fp32 TMEM accumulator of 32 columns per
// limb.  An item whose children all have |v| <= 2^21 (known from their squared norms) takes
// two limbs and N64 MMAs: a third less of the producers' conversions and stores.  A in TMEM
// takes the signs' shared-memory stores and the MMAs' shared-memory reads of A (32 KB of the
// ~60 KB of shared-memory traffic of a K block) off the shared memory.  Four epilogue warps
// recombine the exact int64 dots and write the pair keys the select kernel reads.
// Exact: a limb is at most 1024 in magnitude (the top one of three 512), so every partial sum
// is an integer of magnitude <= dim * 1024 <= 2^24.  Level 0 is one parent (-1) whose children
// are the roots and whose entries are all reads.
constexpr int kTcE = 128;                                         // entries per item (TMEM lanes)
constexpr int kTcC = 32;                                          // children per item (MMA N)
constexpr int kTcLimbs = 3;
// Each producer thread streams its own slice of a K block (16 prototype values, 64 bits of
// its entry's read) with cp.async this many of its blocks ahead, into a private staging
// area of shared memory ([slot][16-byte part][thread]: conflict-free), and converts it when
// its copy group has landed.
constexpr int kTcDepth = 4;
constexpr int kTcAccCols = kTcLimbs * kTcC;                       // one accumulator set
constexpr int kTcTmemCols = 512;                                  // two sets, then the A stages
constexpr int kTcACol = 256;                                      // A of stage s: columns kTcACol + 32 s
constexpr int kTcBBytes = kTcC * 128;                             // per limb
constexpr int kTcStageBytes = kTcLimbs * kTcBBytes;              // 12 KB of B (A is in TMEM)
constexpr int kTcMaxStages = 6;

// The CTA of a tensor-core level with G producer groups of four warps (group g takes K blocks
// g, g + G, ...): warps 0 .. 4G-1 produce, 4G .. 4G+3 run the epilogue, lane 0 of warp 4G+4
// issues the MMAs.  A warp's registers come from its SM sub-partition's quarter of the file,
// so 17 warps (G = 3: five on one sub-partition) get 96 registers a thread, 13 warps (G = 2)
// 128: the level kernel takes three groups, the one-launch kernel, whose other phases need the
// registers, two.
template <int G>
struct TcLayout {
    static constexpr int kGroups = G;
    static constexpr int kStages = 2 * G;  // two stages in flight per group
    static constexpr int kProducers = 128 * G;
    static constexpr size_t kStageArea = (size_t)kTcDepth * 5 * kProducers * 16;  // 4 x 16 B values + 16 B bits
    static constexpr int kEpiWarp = 4 * G;
    static constexpr int kMmaWarp = kEpiWarp + 4;
    static constexpr int kThreads = 32 * (kMmaWarp + 1);
    static constexpr size_t kSmem = (size_t)kStages * kTcStageBytes + kStageArea + 1024;
    static_assert(kStages <= kTcMaxStages, "the barrier arrays hold every stage");
    static_assert(kTcACol + 32 * kStages <= kTcTmemCols, "the A stages fit the TMEM allocation");
};
using TcLevel = TcLayout<3>;  // descent_tc_kernel: 544 threads
using TcOne = TcLayout<2>;    // descent_one_kernel: 416 threads

struct TcItems {
    int32_t* ent_read;    // [entries] grouped by parent
    int32_t* ent_p0;      // first pair index of the entry's candidates
    int32_t* par_cnt;     // [n_nodes] entries per parent
    int32_t* par_off;     // [n_nodes + 1]
    int32_t* par_cursor;  // [n_nodes]
    int32_t* item_cnt;    // [n_nodes] items of a parent of its own
    int32_t* item_off;    // [n_nodes + 1]; item_off[n_nodes] = number of such items of the level
    int32_t* small;       // [n_nodes] 1: the parent shares an item (<= 64 entries, <= 16 children)
    int32_t* small_off;   // [n_nodes + 1]; small_off[n_nodes] = number of such parents
    int32_t* fit2;        // [n_nodes] 1: every child of the parent fits two limbs (|v| <= 2^21)
    // item i: parent, first entry, first child (-1 parent: level 0); an item shared by two
    // parents (after the others) has item_e0 = -1, parent item_par and second parent item_j0 (or -1)
    int32_t* item_par;
    int32_t* item_e0;
    int32_t* item_j0;
    int* status;          // context status word: 100 + code of a wait that gave up
};

__device__ __forceinline__ int32_t n_children(const GArgs& a, int32_t P) {
    if (P < 0) return a.n_roots;
    const int32_t c = (int32_t)(a.child_ptr[P + 1] - a.child_ptr[P]);
    return c ? c : 1;
}

__device__ __forceinline__ int32_t child_at(const GArgs& a, int32_t P, int32_t j) {
    if (P < 0) return a.roots[j];
    const int64_t c0 = a.child_ptr[P];
    return c0 == a.child_ptr[P + 1] ? P : a.child_idx[c0 + j];
}

// entries (read, beam slot) per parent, then their slots in parent order
__device__ __forceinline__ void par_count_one(const GArgs& a, const TcItems& t, int L, int64_t r) {
    if (a.done[r]) return;
    for (int b = 0; b < a.nbeam[r]; ++b) atomicAdd(t.par_cnt + a.paths[state_at(r, b, L - 1)], 1);
}

__global__ void par_count_kernel(const GArgs a, TcItems t, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
    par_count_one(a, t, L, r);
}

__device__ __forceinline__ void par_scatter_one(const GArgs& a, const TcItems& t, int L, int64_t r) {
    if (a.done[r]) return;
    int32_t p = a.off[r];  // the candidates of beam slot b follow those of slots < b (expand_kernel)
    for (int b = 0; b < a.nbeam[r]; ++b) {
        const int32_t P = a.paths[state_at(r, b, L - 1)];
        const int32_t pos = warp_count(t.par_cursor, P);
        t.ent_read[pos] = (int32_t)r;
        t.ent_p0[pos] = p;
        p += n_children(a, P);
    }
}

__global__ void par_scatter_kernel(const GArgs a, TcItems t, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
    par_scatter_one(a, t, L, r);
}

// A parent with at most 64 entries and 16 children shares an item with another such parent
// (entries in rows 0-63 / 64-127, children in slots 0-15 / 16-31): the K loop of an item costs
// the same whatever its fill, and most parents of the lower levels are that small.
constexpr int kTcHalfE = kTcE / 2, kTcHalfC = kTcC / 2;

// A row fits two limbs when every element has |v| <= 2^21, and |v| <= sqrt(squared norm) for
// each element: int16 rows always, int32 rows whose squared norm is at most 2^42.
__device__ __forceinline__ bool row_fits2(const GArgs& a, int32_t c) {
    return c >= a.n32 || a.pn[c] <= (int64_t(1) << 42);
}

__device__ __forceinline__ void item_count_one(const GArgs& a, const TcItems& t, int64_t P) {
    const int32_t m = t.par_cnt[P], nch = n_children(a, (int32_t)P);
    const bool small = m > 0 && m <= kTcHalfE && nch <= kTcHalfC;
    t.small[P] = small ? 1 : 0;
    t.item_cnt[P] = m && !small ? ((m + kTcE - 1) / kTcE) * ((nch + kTcC - 1) / kTcC) : 0;
    if (m) {  // the children's norms loaded independently (no early exit), four at a time
        const int64_t c0 = a.child_ptr[P], c1 = a.child_ptr[P + 1];
        bool two = c0 < c1 || row_fits2(a, (int32_t)P);
#pragma unroll 4
        for (int64_t c = c0; c < c1; ++c) two &= row_fits2(a, a.child_idx[c]);
        t.fit2[P] = two ? 1 : 0;
    }
}

__global__ void item_count_kernel(const GArgs a, TcItems t) {
    const int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= a.n_nodes) return;
    item_count_one(a, t, P);
}

__device__ void item_write_one(const GArgs& a, const TcItems& t, int64_t P) {
    if (t.small[P]) {
        const int32_t slot = t.small_off[P], x = t.item_off[a.n_nodes] + slot / 2;
        if (slot & 1) {
            t.item_j0[x] = (int32_t)P;
        } else {
            t.item_par[x] = (int32_t)P;
            t.item_e0[x] = -1;
            if (slot + 1 == t.small_off[a.n_nodes]) t.item_j0[x] = -1;  // an odd one out
        }
        return;
    }
    const int32_t n = t.item_cnt[P];
    const int32_t nj = (n_children(a, (int32_t)P) + kTcC - 1) / kTcC;
    for (int32_t i = 0; i < n; ++i) {
        const int32_t x = t.item_off[P] + i;
        t.item_par[x] = (int32_t)P;
        t.item_e0[x] = (i / nj) * kTcE;
        t.item_j0[x] = (i % nj) * kTcC;
    }
}

__global__ void item_write_kernel(const GArgs a, TcItems t) {
    const int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (P >= a.n_nodes) return;
    item_write_one(a, t, P);
}

// What row `row` (an entry) and child slot `js` of item `it` are.
struct ItemRow {
    int64_t r = -1;       // the entry's read (-1: an unused row)
    int32_t p0 = 0;       // its first pair index
    int32_t P = -1;       // the parent its columns belong to (-1 with level 0's roots too)
    int32_t cbase = 0;    // first column of that parent in the item
    int32_t cfirst = 0;   // the child index of column cbase
    int32_t ncols = 0;    // columns of that parent in the item
};

__device__ __forceinline__ ItemRow item_row(const GArgs& a, const TcItems& t, int32_t it, int row) {
    ItemRow x;
    const int32_t p = t.item_par[it], e0 = t.item_e0[it], j0 = t.item_j0[it];
    int32_t e;
    if (e0 < 0) {  // shared: rows 0-63 the first parent, 64-127 the second
        const int seg = row / kTcHalfE;
        x.P = seg ? j0 : p;
        if (x.P < 0) return x;
        e = row % kTcHalfE;
        x.cbase = seg * kTcHalfC;
        x.ncols = n_children(a, x.P);
    } else {
        x.P = p;
        e = e0 + row;
        x.cfirst = j0;
        x.ncols = min(kTcC, n_children(a, p) - j0);
    }
    if (x.P < 0 && e0 >= 0) {  // level 0: entry e is read e
        if (e < a.nq) {
            x.r = e;
            x.p0 = a.off[e];
        }
    } else if (e < t.par_cnt[x.P]) {
        x.r = t.ent_read[t.par_off[x.P] + e];
        x.p0 = t.ent_p0[t.par_off[x.P] + e];
    }
    return x;
}

// Whether item `it` runs with two limbs (every child of its parents fits them; level 0's
// roots always take three).
__device__ __forceinline__ bool item_two(const TcItems& t, int32_t it) {
    const int32_t p = t.item_par[it], e0 = t.item_e0[it], j0 = t.item_j0[it];
    if (p < 0) return false;
    return t.fit2[p] != 0 && (e0 >= 0 || j0 < 0 || t.fit2[j0] != 0);
}

__device__ __forceinline__ int32_t item_child(const GArgs& a, const TcItems& t, int32_t it, int js) {
    const int32_t p = t.item_par[it], e0 = t.item_e0[it], j0 = t.item_j0[it];
    if (e0 < 0) {
        const int seg = js / kTcHalfC, c = js % kTcHalfC;
        const int32_t P = seg ? j0 : p;
        return P >= 0 && c < n_children(a, P) ? child_at(a, P, c) : -1;
    }
    return j0 + js < n_children(a, p) ? child_at(a, p, j0 + js) : -1;
}

// level 0: every read against the roots; items i = first, first + stride, ...
__device__ __forceinline__ void items_level0_range(const GArgs& a, const TcItems& t, int64_t first, int64_t stride) {
    const int32_t ne = (int32_t)((a.nq + kTcE - 1) / kTcE), nj = (a.n_roots + kTcC - 1) / kTcC;
    if (first == 0) {
        t.item_off[a.n_nodes] = ne * nj;
        t.small_off[a.n_nodes] = 0;
    }
    for (int64_t i = first; i < (int64_t)ne * nj; i += stride) {
        t.item_par[i] = -1;
        t.item_e0[i] = (int32_t)(i / nj) * kTcE;
        t.item_j0[i] = (int32_t)(i % nj) * kTcC;
    }
}

__global__ void items_level0_kernel(const GArgs a, TcItems t) {
    items_level0_range(a, t, (int64_t)blockIdx.x * blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

// v = l0 + 2048 l1 with l0 in [-1024, 1023] and |l1| <= 1024, for |v| <= 2^21
__device__ __forceinline__ void limbs2(int32_t v, int32_t& l0, int32_t& l1) {
    l1 = (v >> 11) + (((v & 2047) + 1024) >> 11);  // floor((v + 1024) / 2048)
    l0 = (int32_t)((uint32_t)v - ((uint32_t)l1 << 11));
}

// v = l0 + 2048 l1 + 2048^2 l2 with l0, l1 in [-1024, 1023] and |l2| <= 512, for every int32 v
__device__ __forceinline__ void limbs3(int32_t v, int32_t& l0, int32_t& l1, int32_t& l2) {
    const int32_t q1 = (v >> 11) + (((v & 2047) + 1024) >> 11);  // floor((v + 1024) / 2048)
    l0 = (int32_t)((uint32_t)v - ((uint32_t)q1 << 11));
    const int32_t q2 = (q1 >> 11) + (((q1 & 2047) + 1024) >> 11);
    l1 = q1 - q2 * 2048;
    l2 = q2;
}

// Two small integers (|x| <= 2048) as an fp16 pair: each becomes an fp32 by the magic
// number 1.5 * 2^23 (exact for |x| < 2^22: one integer and one float add, no conversion
// unit), and the pair is packed with one cvt.rn.f16x2.f32 (exact: both fit 11 bits).
__device__ __forceinline__ uint32_t half2_bits(int32_t x, int32_t y) {
    const float fx = __int_as_float(0x4B400000 + x) - 12582912.0f;
    const float fy = __int_as_float(0x4B400000 + y) - 12582912.0f;
    const __half2 h = __floats2half2_rn(fx, fy);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// cp.async of 16 / 8 bytes global -> shared; with src_bytes 0 nothing is read and zeros land
__device__ __forceinline__ void cp_async16(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(tc::smem_u32(dst)), "l"(src), "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 16-byte chunk c of row r of a 128-byte-row tile in the 128-byte swizzle layout
__device__ __forceinline__ uint8_t* swz(uint8_t* tile, int r, int c) { return tile + r * 128 + ((c ^ (r & 7)) << 4); }

// A streamed level's rows are staged in dim quarters, one ring of at most kRowSlots slots per
// quarter; warps 1-12 score (three groups of four, warp 1 + 4 g + q takes quarter q of group g's
// pairs) and warp 0 stages.
constexpr int kRowSlots = 8;
constexpr int kRowConsumers = 12;
constexpr int kQuarters = 4;
constexpr int kRowGroups = kRowConsumers / kQuarters;

// Shared-memory state of the tensor-core scoring (one CTA per SM).
struct TcShared {
    uint64_t full_bar[kTcMaxStages], empty_bar[kTcMaxStages], accf_bar[2], acce_bar[2];
    uint64_t drain_bar;  // the MMA issuer's last commit before TMEM is freed
    uint64_t row_full[kQuarters * kRowSlots], row_empty[kQuarters * kRowSlots];  // quarter q's ring: [q * kRowSlots, ..)
    uint32_t tmem_base;
    int err;             // code of a wait that gave up (0: none)
};

// Ring positions of the roles, carried from one scoring phase to the next when one
// launch scores several levels (each role keeps its own copy in its threads).
struct TcRun {
    int64_t nbase = 0;          // producers: K blocks of the items this CTA has staged
    int stage = 0, acc = 0;     // MMA issuer: next stage and accumulator set; epilogue: next set
    uint32_t phase = 0, acc_phase = 0;
    int64_t row_ord = 0;        // streamed levels: rows this CTA has staged (producer) or scored (consumers)
};

// Barriers and the TMEM columns of the CTA (every thread calls it).
template <class Lay>
__device__ void tc_setup(TcShared& sm) {
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        sm.err = 0;
        for (int s = 0; s < Lay::kStages; ++s) {
            tc::mbar_init(&sm.full_bar[s], 4);  // one arrival per warp of the producer group
            tc::mbar_init(&sm.empty_bar[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&sm.accf_bar[b], 1);
            tc::mbar_init(&sm.acce_bar[b], 4);  // one arrival per epilogue warp
        }
        tc::mbar_init(&sm.drain_bar, 1);
        for (int i = 0; i < kQuarters * kRowSlots; ++i) {
            tc::mbar_init(&sm.row_full[i], 1);
            tc::mbar_init(&sm.row_empty[i], kRowGroups);  // one warp per group reads a quarter
        }
        tc::fence_mbar_init();
    }
    if (warp == Lay::kMmaWarp) {
        tc::tmem_alloc(&sm.tmem_base, kTcTmemCols);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
}

// Scores the items of one level: warps 0-11 produce, 12-15 run the epilogue, lane 0 of warp 16
// issues the MMAs.  Every thread of the CTA calls it; the items are blockIdx.x, + gridDim.x, ...
template <class Lay>
__device__ void tc_phase(const GArgs& a, const TcItems& t, TcShared& sm, TcRun& run, uint8_t* ring, uint4* staging) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tmem = sm.tmem_base;
    const int32_t n_items = t.item_off[a.n_nodes] + (t.small_off[a.n_nodes] + 1) / 2;
    const int kblocks = a.dim / 64;

    if (warp < Lay::kEpiWarp) {
        // ------------------------------------------------ producers: group g takes K blocks g, g + 3, ...
        // Row tid of A is this thread's entry.  The valid children's values of a K block are
        // groups of 4 (group 16 v + u: the item's v-th valid child, dims 4u..4u+3); group x
        // goes to the thread with tb = x mod 128, so the limb split is spread over the whole
        // group.  tb is tid rotated so that the groups past the first 128 (a warp that has any
        // takes a second pass) fall to warp 1, 6 or 11, not to the warps that share their SM
        // sub-partition with the MMA issuer.  Nothing
        // is written for an unused row or child slot: an accumulator row or column depends only
        // on its own A row or B row, and the epilogue never reads those of unused ones.
        const int g = warp >> 2;
        const int tid = threadIdx.x & 127;
        const int tb = (tid + 96 - 32 * g) & 127;
        const int ptid = threadIdx.x;  // this thread's staging column
        int64_t& nbase = run.nbase;    // K blocks of the items before this one (the ring position)
        bool ok = true;
        for (int32_t it = blockIdx.x; ok && it < n_items; it += gridDim.x, nbase += kblocks) {
            const int64_t rrow = item_row(a, t, it, tid).r;
            const bool two = item_two(t, it);
            const uint2* bits_row = reinterpret_cast<const uint2*>(a.bits + (rrow >= 0 ? rrow : 0) * a.words);
            // the valid child slots: 0..n0-1 and, in a shared item, 16..16+n1-1
            const int32_t ip = t.item_par[it], ie0 = t.item_e0[it], ij0 = t.item_j0[it];
            int n0, n1 = 0;
            if (ie0 < 0) {
                n0 = n_children(a, ip);
                n1 = ij0 >= 0 ? n_children(a, ij0) : 0;
            } else {
                n0 = min(kTcC, n_children(a, ip) - ij0);
            }
            const int ngroups = (n0 + n1) * 16;
            const char* gsrc[4];  // this group's 4 values in K block 0: 16 bytes of an int32 row or 8 of an int16 row
            int gdst[4];          // child slot * 16 + u
            bool g16[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int x = tb + kTcE * i;
                gsrc[i] = reinterpret_cast<const char*>(a.proto);
                gdst[i] = 0;
                g16[i] = false;
                if (x < ngroups) {
                    const int v = x >> 4, u = x & 15;
                    const int js = v < n0 ? v : kTcHalfC + (v - n0);
                    const int64_t c = item_child(a, t, it, js);
                    g16[i] = c >= a.n32;
                    gsrc[i] = g16[i] ? reinterpret_cast<const char*>(a.proto16 + (c - a.n32) * a.dim + 4 * u)
                                     : reinterpret_cast<const char*>(a.proto + c * a.dim + 4 * u);
                    gdst[i] = js * 16 + u;
                }
            }
            // a warp whose groups are all int32 rows runs the int32-only body
            bool my16 = false;
#pragma unroll
            for (int i = 0; i < 4; ++i) my16 |= g16[i];
            auto body = [&](auto rows16) {
                constexpr bool R16 = decltype(rows16)::value;
                auto issue = [&](int kb, int slot) {  // this thread's slices of K block kb, into staging slot `slot`
                    if (kb < kblocks) {
                        uint4* sb = staging + (size_t)slot * 5 * Lay::kProducers;
#pragma unroll
                        for (int i = 0; i < 4; ++i)
                            if (tb + kTcE * i < ngroups) {
                                if (R16 && g16[i])
                                    cp_async8(sb + i * Lay::kProducers + ptid, gsrc[i] + kb * 128, 8);
                                else
                                    cp_async16(sb + i * Lay::kProducers + ptid, gsrc[i] + kb * 256, 16);
                            }
                        if (rrow >= 0) cp_async8(sb + 4 * Lay::kProducers + ptid, bits_row + kb, 8);
                    }
                    cp_async_commit();  // one group per call (possibly empty), so the wait below counts blocks
                };
#pragma unroll
                for (int i = 0; i < kTcDepth; ++i) issue(g + Lay::kGroups * i, i);
                for (int kb = g, i = 0; kb < kblocks; kb += Lay::kGroups, ++i) {
                    cp_async_wait<kTcDepth - 1>();  // this thread's copies of block kb have landed
                    const int slot = i % kTcDepth;
                    const uint4* sb = staging + (size_t)slot * 5 * Lay::kProducers;
                    uint4 pv[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) pv[j] = tb + kTcE * j < ngroups ? sb[j * Lay::kProducers + ptid] : make_uint4(0, 0, 0, 0);
                    const uint2 w = rrow >= 0 ? *reinterpret_cast<const uint2*>(sb + 4 * Lay::kProducers + ptid) : make_uint2(0, 0);
                    issue(kb + Lay::kGroups * kTcDepth, slot);  // the slot is free again: refill it kTcDepth blocks ahead
                    const int64_t n = nbase + kb;
                    const int stage = (int)(n % Lay::kStages);
                    const uint32_t phase = (uint32_t)((n / Lay::kStages) & 1);
                    const bool got = tc::mbar_wait(&sm.empty_bar[stage], phase ^ 1, &sm.err, 11, a.wait_cycles);
                    if (__any_sync(0xffffffffu, !got)) {
                        ok = false;
                        break;
                    }
                    uint8_t* st = ring + (size_t)stage * kTcStageBytes;
                    // A: this entry's 64 signs, two fp16 to a column, into TMEM lane tid (an unused
                    // row's garbage only reaches its own accumulator row, which is never read)
                    {
                        uint32_t col[32];
#pragma unroll
                        for (int j = 0; j < 32; ++j) {
                            const uint32_t t = (j < 16 ? w.x : w.y) >> (2 * (j & 15));
                            col[j] = 0xBC00BC00u ^ ((t & 1u) << 15) ^ ((t & 2u) << 30);
                        }
                        tc::tmem_st32(tmem + ((uint32_t)(warp & 3) << 21) + (uint32_t)(kTcACol + 32 * stage), col);
                    }
                    // B: this thread's groups of 4 prototype values, each in two or three limbs (8
                    // bytes per limb)
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        if (tb + kTcE * j >= ngroups) break;
                        int32_t l0[4], l1[4], l2[4];
                        int32_t x[4] = {(int32_t)pv[j].x, (int32_t)pv[j].y, (int32_t)pv[j].z, (int32_t)pv[j].w};
                        if (R16 && g16[j]) {  // four int16 values in the first 8 bytes
                            x[0] = (int32_t)(pv[j].x << 16) >> 16;
                            x[1] = (int32_t)pv[j].x >> 16;
                            x[2] = (int32_t)(pv[j].y << 16) >> 16;
                            x[3] = (int32_t)pv[j].y >> 16;
                        }
                        const int js = gdst[j] >> 4, u = gdst[j] & 15;
                        const int off = (u & 1) * 8;
                        if (two) {
#pragma unroll
                            for (int e = 0; e < 4; ++e) limbs2(x[e], l0[e], l1[e]);
                        } else {
#pragma unroll
                            for (int e = 0; e < 4; ++e) limbs3(x[e], l0[e], l1[e], l2[e]);
                            *reinterpret_cast<uint2*>(swz(st + 2 * kTcBBytes, js, u >> 1) + off) =
                                make_uint2(half2_bits(l2[0], l2[1]), half2_bits(l2[2], l2[3]));
                        }
                        *reinterpret_cast<uint2*>(swz(st, js, u >> 1) + off) =
                            make_uint2(half2_bits(l0[0], l0[1]), half2_bits(l0[2], l0[3]));
                        *reinterpret_cast<uint2*>(swz(st + kTcBBytes, js, u >> 1) + off) =
                            make_uint2(half2_bits(l1[0], l1[1]), half2_bits(l1[2], l1[3]));
                    }
                    tc::tmem_st_wait();       // the A columns are written
                    tc::fence_before();       // ... before the arrive below (tcgen05 ordering)
                    tc::fence_proxy_async();  // the B writes above are read by the tensor cores
                    __syncwarp();
                    if (lane == 0) tc::mbar_arrive(&sm.full_bar[stage]);
                }
            };
            if (__any_sync(0xffffffffu, my16))
                body(std::true_type{});
            else
                body(std::false_type{});
        }
        cp_async_wait<0>();  // no copy may still be landing when the CTA leaves
    } else if (warp < Lay::kMmaWarp) {
        // ------------------------------------------------ epilogue
        const int quarter = warp & 3, row = quarter * 32 + lane;
        int& acc = run.acc;
        uint32_t& acc_phase = run.acc_phase;
        for (int32_t it = blockIdx.x; it < n_items; it += gridDim.x) {
            // this row's entry and its parent's columns (the same for the warp's 32 rows: a shared
            // item's halves are 64 rows)
            const ItemRow x = item_row(a, t, it, row);
            const bool two = item_two(t, it);
            if (!tc::mbar_wait(&sm.accf_bar[acc], acc_phase, &sm.err, 12, a.wait_cycles)) break;
            tc::fence_after();
            const uint32_t d = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(acc * kTcAccCols);
            const int64_t qn = x.r >= 0 ? a.qn[x.r] : 0;
            // the exact dots of 16 columns at a time (limb l of column j is TMEM column 32 l + j)
            for (int h = x.cbase; h < x.cbase + x.ncols; h += 16) {
                uint32_t v0[16], v1[16], v2[16];
                tc::tmem_ld16(d + h, v0);
                tc::tmem_ld16(d + kTcC + h, v1);
                if (two) {
#pragma unroll
                    for (int j = 0; j < 16; ++j) v2[j] = 0;
                } else {
                    tc::tmem_ld16(d + 2 * kTcC + h, v2);
                }
                tc::tmem_ld_wait();
                if (x.r < 0) continue;
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    if (h + j >= x.cbase + x.ncols) break;
                    const int32_t ci = x.cfirst + h + j - x.cbase;  // child index within the parent
                    const int32_t c = child_at(a, x.P, ci);
                    const int64_t dot = (int64_t)__float2ll_rn(__uint_as_float(v0[j])) +
                                        (int64_t)__float2ll_rn(__uint_as_float(v1[j])) * 2048 +
                                        (int64_t)__float2ll_rn(__uint_as_float(v2[j])) * (2048 * 2048);
                    a.pair_key[x.p0 + ci] = make_key(exact_score(dot, qn, a.pn[c], a.mode), (uint32_t)c);
                }
            }
            tc::fence_before();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&sm.acce_bar[acc]);  // the accumulators may be reused
            if (++acc == 2) {
                acc = 0;
                acc_phase ^= 1;
            }
        }
    } else if (lane == 0) {
        // ------------------------------------------------ MMA issuer
        // the limb tiles of B are 64 or 96 consecutive rows of shared memory and their
        // accumulators as many consecutive columns: one N = 64 or 96 MMA covers them all
        constexpr uint32_t IDESC3 = tc::idesc_f16_f32(kTcE, kTcLimbs * kTcC);
        constexpr uint32_t IDESC2 = tc::idesc_f16_f32(kTcE, 2 * kTcC);
        int& stage = run.stage;
        int& acc = run.acc;
        uint32_t& phase = run.phase;
        uint32_t& acc_phase = run.acc_phase;
        bool ok = true;
        for (int32_t it = blockIdx.x; ok && it < n_items; it += gridDim.x) {
            if (!tc::mbar_wait(&sm.acce_bar[acc], acc_phase ^ 1, &sm.err, 13, a.wait_cycles)) break;
            tc::fence_after();
            const uint32_t d = tmem + (uint32_t)(acc * kTcAccCols);
            const uint32_t IDESC = item_two(t, it) ? IDESC2 : IDESC3;
            for (int kb = 0; kb < kblocks; ++kb) {
                if (!tc::mbar_wait(&sm.full_bar[stage], phase, &sm.err, 14, a.wait_cycles)) {
                    ok = false;
                    break;
                }
                tc::fence_after();
                const uint32_t sa = tc::smem_u32(ring + (size_t)stage * kTcStageBytes);
                const uint64_t bdesc = tc::kmajor_desc(sa, 1024, 2);
                const uint32_t a_tm = tmem + (uint32_t)(kTcACol + 32 * stage);  // 8 columns per K = 16
#pragma unroll
                for (int kk = 0; kk < 4; ++kk)
                    tc::mma_f16_ta(d, a_tm + 8 * kk, bdesc + 2 * kk, IDESC, (kb | kk) != 0 ? 1u : 0u);
                tc::mma_commit(&sm.empty_bar[stage]);
                if (++stage == Lay::kStages) {
                    stage = 0;
                    phase ^= 1;
                }
            }
            if (!ok) break;
            tc::mma_commit(&sm.accf_bar[acc]);
            if (++acc == 2) {
                acc = 0;
                acc_phase ^= 1;
            }
        }
    }
}

// After the last scoring phase: wait (bounded) until every MMA this CTA issued has
// completed, then free the TMEM columns and record a wait that gave up.
template <class Lay>
__device__ void tc_teardown(TcShared& sm, int* status) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == Lay::kMmaWarp && lane == 0) {
        tc::mma_commit(&sm.drain_bar);
        const long long c0 = clock64();
        while (!tc::mbar_try_wait(tc::smem_u32(&sm.drain_bar), 0) && clock64() - c0 < tc::kWaitCycles) {
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == Lay::kMmaWarp) {
        tc::fence_after();
        tc::tmem_dealloc(sm.tmem_base, kTcTmemCols);
    }
    if (threadIdx.x == 0 && sm.err) atomicCAS(status, 0, 100 + sm.err);
}

__device__ __forceinline__ uint8_t* tc_ring(uint8_t* smem_raw) {
    const uint32_t raw_addr = tc::smem_u32(smem_raw);
    return smem_raw + ((1024 - (raw_addr & 1023)) & 1023);
}

__global__ void __launch_bounds__(TcLevel::kThreads, 1) descent_tc_kernel(const GArgs a, const TcItems t) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ TcShared sm;
    uint8_t* ring = tc_ring(smem_raw);
    uint4* staging = reinterpret_cast<uint4*>(ring + (size_t)TcLevel::kStages * kTcStageBytes);
    tc_setup<TcLevel>(sm);
    TcRun run;
    tc_phase<TcLevel>(a, t, sm, run, ring, staging);
    tc_teardown<TcLevel>(sm, t.status);
}

// ---------------------------------------------------------------- the whole descent in one launch
// descent_one_kernel runs every level of the grouped descent in one cooperative launch (one
// CTA per SM, all resident): the phases the multi-launch form runs as separate kernels are
// separated here by a grid-wide barrier, and each CTA owns a fixed chunk of the reads (count,
// expand, select and output of a read run in the CTA that owns it, so those phases need no
// barrier between them) and a fixed chunk of the nodes (the per-node scans).  The tensor-core
// scoring keeps its TMEM columns and mbarrier ring positions from one level to the next.

constexpr int kCodeGridBarrier = 20;  // status 100 + this: a grid barrier gave up
// Dynamic shared memory of the one-launch kernel: the tensor-core levels use the first TcOne::kSmem
// bytes; the streamed leaf level uses all of it (row slots + the consumers' bit buffers).
constexpr size_t kOneSmem = 225 * 1024;
static_assert(kOneSmem >= TcOne::kSmem, "the one-launch kernel also runs the tensor-core levels");
constexpr int kMaxPhaseTs = 64;       // phase timestamps kept of a launch (hdc_beam_phase_times)

struct OneArgs {
    unsigned* bar_count;  // arrivals at the current grid barrier
    unsigned* bar_gen;    // barriers passed
    int* abort;           // 1 once a CTA gave up: every CTA then leaves at its next barrier
    int32_t* blk;         // [3][gridDim.x] per-CTA partial sums of the scans
    int32_t* maxc;        // the tree's largest child count, computed in the launch (null: not checked)
    int32_t given;        // the caller's largest child count
    int* status;
    int use_tc;
    int32_t* out_path;
    float* out_score;
    int32_t* out_depth;
    unsigned long long* phase_ts;  // [kMaxPhaseTs] CTA 0's clock at the start and after every barrier
    int leaf_apart;                // 1: stop at the last level's node-ordered pairs (scored by leaf_kernel)
    long long wait_cycles;         // limit of every bounded wait (SM cycles)
    int late_cta;                  // test hook: CTA 0 reaches its first grid barrier 4 limits late
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_volatile(const int* p) { return *reinterpret_cast<const volatile int*>(p); }

// Grid-wide barrier of a cooperative launch (every CTA is resident).  The wait is bounded: a
// barrier that runs out of time, or a CTA whose scoring gave up, raises o.abort, and every
// CTA then returns false here and leaves.  Writes before the barrier are visible after it.
__device__ bool grid_barrier(const OneArgs& o, const TcShared& sm, int* ok_s, int* n_ts) {
    __syncthreads();
    if (threadIdx.x == 0) {
        if (sm.err) atomicExch(o.abort, 1);
        __threadfence();
        const unsigned g = ld_acquire_gpu(o.bar_gen);
        if (atomicAdd(o.bar_count, 1u) == gridDim.x - 1) {
            atomicExch(o.bar_count, 0u);
            __threadfence();
            st_release_gpu(o.bar_gen, g + 1);
        } else {
            const long long t0 = clock64();
            while (ld_acquire_gpu(o.bar_gen) == g) {
                if (ld_volatile(o.abort)) break;
                if (clock64() - t0 > o.wait_cycles) {
                    if (atomicExch(o.abort, 1) == 0) atomicCAS(o.status, 0, 100 + kCodeGridBarrier);
                    break;
                }
                __nanosleep(64);
            }
        }
        *ok_s = ld_volatile(o.abort) == 0;
        if (blockIdx.x == 0 && *n_ts < kMaxPhaseTs) o.phase_ts[(*n_ts)++] = global_ns();
    }
    __syncthreads();
    return *ok_s != 0;
}

// sum over in[lo, hi) (every thread of the CTA gets it)
__device__ int32_t cta_sum(const int32_t* in, int64_t lo, int64_t hi, int32_t* sh) {
    int32_t v = 0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) v += in[i];
    int32_t total;
    block_scan_excl(v, sh, &total);
    return total;
}

// out[i] (and out2[i]) = base + sum(in[lo .. i)) for i in [lo, hi); returns base + sum(in[lo, hi))
__device__ int32_t cta_scan(const int32_t* in, int32_t* out, int32_t* out2, int64_t lo, int64_t hi, int32_t base,
                            int32_t* sh) {
    const int64_t per = (hi - lo + blockDim.x - 1) / blockDim.x;
    const int64_t a0 = min(hi, lo + (int64_t)threadIdx.x * per), a1 = min(hi, a0 + per);
    int32_t v = 0;
    for (int64_t i = a0; i < a1; ++i) v += in[i];
    int32_t total;
    int32_t run = base + block_scan_excl(v, sh, &total);
    for (int64_t i = a0; i < a1; ++i) {
        const int32_t x = in[i];
        out[i] = run;
        if (out2) out2[i] = run;
        run += x;
    }
    return base + total;
}

// sum of the first b entries of a per-CTA array (every thread of the CTA gets it)
__device__ int32_t cta_prefix(const int32_t* blk, int b, int32_t* sh) {
    int32_t v = 0;
    for (int j = threadIdx.x; j < b; j += blockDim.x) v += blk[j];
    int32_t total;
    block_scan_excl(v, sh, &total);
    return total;
}

// A streamed CUDA-core level (the leaves of the one-launch descent): the pairs are in node
// order, so each candidate node's prototype row is copied once from HBM into shared memory by
// 1-D bulk copies (warp 0, evict-first in L2: a row is read once per call) and its pairs are
// scored from there.  A row travels as four quarters of its dims, each through its own ring;
// warp 1 + 4 g + q sums quarter q of the pairs of group g (the pairs at positions P0 + g,
// P0 + g + 3, ... of the CTA's share of the node-ordered list) and writes that partial dot,
// so a pair is scored by four warps at once and a quarter row is held only while three warps
// use it: more of the shared memory holds rows in flight.  The bits of a warp's next pair (its
// quarter) are copied into a private buffer (cp.async) while it scores the current one.  The
// partial dots are summed, and the FP64 scores computed, by the CTA that owns the read, after
// the next grid barrier (keys_from_parts).  CTA b owns the nodes whose first pair falls in its
// share of the pair list.
constexpr int kBitsBufs = 4;  // per consumer warp: the bits of the pairs being scored and of the next ones

// Lane l's share of a quarter of int16 row dims: steps j of 256 dims, 8 dims a lane (one
// 16-byte word of the row, one byte of the read's bits)
__device__ __forceinline__ int smem_dot16(const int4* rowv, const uint32_t* bits, int lane, int nsteps) {
    constexpr int U = 8;
    const int sh = (lane & 3) * 8;
    const uint32_t* qb = bits + (lane >> 2);
    int acc0 = 0, acc1 = 0, acc2 = 0, acc3 = 0;  // four independent dp2a chains
    for (int j = 0; j < nsteps; j += U) {
        int4 x[U];
        uint32_t w[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool in = j + u < nsteps;
            x[u] = in ? rowv[32 * (j + u)] : make_int4(0, 0, 0, 0);
            w[u] = in ? qb[8 * (j + u)] : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t byte = w[u] >> sh;
            const int s0 = signs4_bytes(byte & 15u), s1 = signs4_bytes((byte >> 4) & 15u);
            acc0 = __dp2a_lo(x[u].x, s0, acc0);
            acc1 = __dp2a_hi(x[u].y, s0, acc1);
            acc2 = __dp2a_lo(x[u].z, s1, acc2);
            acc3 = __dp2a_hi(x[u].w, s1, acc3);
        }
    }
    return acc0 + acc1 + acc2 + acc3;  // |sum| <= 4,096 x 32,767 a lane at D = 16,384: int32
}

// The same for two pairs of one row (one shared-memory read of the row for both).
__device__ __forceinline__ int2 smem_dot16x2(const int4* rowv, const uint32_t* bits0, const uint32_t* bits1, int lane,
                                             int nsteps) {
    constexpr int U = 8;
    const int sh = (lane & 3) * 8;
    const uint32_t* qb0 = bits0 + (lane >> 2);
    const uint32_t* qb1 = bits1 + (lane >> 2);
    int a0 = 0, a1 = 0, c0 = 0, c1 = 0;
    for (int j = 0; j < nsteps; j += U) {
        int4 x[U];
        uint32_t w[U], v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool in = j + u < nsteps;
            x[u] = in ? rowv[32 * (j + u)] : make_int4(0, 0, 0, 0);
            w[u] = in ? qb0[8 * (j + u)] : 0u;
            v[u] = in ? qb1[8 * (j + u)] : 0u;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const uint32_t bw = w[u] >> sh, bv = v[u] >> sh;
            const int s0 = signs4_bytes(bw & 15u), s1 = signs4_bytes((bw >> 4) & 15u);
            const int t0 = signs4_bytes(bv & 15u), t1 = signs4_bytes((bv >> 4) & 15u);
            a0 = __dp2a_lo(x[u].x, s0, a0);
            a1 = __dp2a_hi(x[u].y, s0, a1);
            a0 = __dp2a_lo(x[u].z, s1, a0);
            a1 = __dp2a_hi(x[u].w, s1, a1);
            c0 = __dp2a_lo(x[u].x, t0, c0);
            c1 = __dp2a_hi(x[u].y, t0, c1);
            c0 = __dp2a_lo(x[u].z, t1, c0);
            c1 = __dp2a_hi(x[u].w, t1, c1);
        }
    }
    return make_int2(a0 + a1, c0 + c1);
}

// the same for int32 rows: steps of 128 dims, 4 dims a lane
__device__ __forceinline__ int64_t smem_dot32(const int4* rowv, const uint32_t* bits, int lane, int nsteps) {
    const int sh = (lane & 7) * 4;
    const uint32_t* qb = bits + (lane >> 3);
    int64_t acc = 0;
    for (int j = 0; j < nsteps; ++j) {
        const int4 x = rowv[32 * j];
        const uint32_t nib = qb[4 * j] >> sh;
        acc += (int64_t)((nib & 1u) ? x.x : neg32(x.x)) + (int64_t)((nib & 2u) ? x.y : neg32(x.y)) +
               (int64_t)((nib & 4u) ? x.z : neg32(x.z)) + (int64_t)((nib & 8u) ? x.w : neg32(x.w));
    }
    return acc;
}

// first n in [0, n_nodes] with node_off[n] >= x
__device__ __forceinline__ int64_t first_node_at(const GArgs& a, int64_t x) {
    int64_t lo = 0, hi = a.n_nodes;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a.node_off[mid] >= x)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// first n in [lo, hi) with node_off[n + 1] > y (hi if none): skips the nodes without pairs
// before position y
__device__ __forceinline__ int64_t first_node_after(const GArgs& a, int64_t lo, int64_t hi, int64_t y) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a.node_off[mid + 1] > y)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

// `area` bytes of shared memory from `ring` on: the four rings' slots, then the consumers'
// bit buffers
__device__ void stream_phase(const GArgs& a, TcShared& sm, TcRun& run, uint8_t* ring, size_t area) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t total = a.off[a.nq];
    const int64_t pc = (total + gridDim.x - 1) / gridDim.x;
    const int64_t n_hi = blockIdx.x + 1 == gridDim.x ? a.n_nodes : first_node_at(a, (int64_t)(blockIdx.x + 1) * pc);
    int64_t n_lo = first_node_at(a, (int64_t)blockIdx.x * pc);
    // the range starts at its first node with pairs (CTA 0's would start at node 0, and every
    // node of the ranks above the level has none)
    n_lo = first_node_after(a, n_lo, n_hi, a.node_off[n_lo]);
    const int qdim = a.dim / kQuarters;  // a multiple of 256
    const uint32_t item_bytes = (uint32_t)qdim * (n_lo < a.n32 ? 4u : 2u);  // a slot holds any quarter of the range
    const uint32_t qbits_bytes = (uint32_t)qdim / 8u;                       // a quarter of a read's bits
    const size_t bits_area = (size_t)kRowConsumers * kBitsBufs * qbits_bytes;
    // >= 3 for every dim <= 16384
    const int S = min(kRowSlots, (int)((area - bits_area) / ((size_t)kQuarters * item_bytes)));
    uint8_t* bits_sm = ring + (size_t)kQuarters * S * item_bytes;
    const int64_t ord0 = run.row_ord;  // this phase's first row ordinal (every role's copy agrees)
    if (warp == 0) {
        // the warp walks the nodes (their offsets loaded 31 at a time, lane j holding
        // node_off[nb + j]); lane 0 waits for the slots and issues the copies
        tc::fence_proxy_async();  // the ring's earlier generic-proxy writes come before the bulk copies
        const uint64_t once = tc::make_policy_evict_first();
        int64_t issued[kQuarters] = {0, 0, 0, 0};  // rows whose quarter q is on its way (lane 0)
        bool ok = true;
        int64_t i = run.row_ord;
        int slot = (int)(i % S);  // i % S and (i / S) & 1, kept incrementally
        uint32_t parity = (uint32_t)((i / S) & 1);
        for (int64_t nb = n_lo; ok && nb < n_hi; nb += 31) {
            const int32_t offv = nb + lane <= a.n_nodes ? a.node_off[nb + lane] : 0;
            const int cnt = (int)min((int64_t)31, n_hi - nb);
            for (int j = 0; ok && j < cnt; ++j) {
                const int32_t ps = __shfl_sync(0xffffffffu, offv, j), pe = __shfl_sync(0xffffffffu, offv, j + 1);
                if (ps == pe) continue;
                const int64_t n = nb + j;
                if (lane == 0) {
                    const bool w16 = n >= a.n32;
                    const uint32_t bytes = (uint32_t)qdim * (w16 ? 2u : 4u);
                    const char* src = w16 ? reinterpret_cast<const char*>(a.proto16 + (n - a.n32) * a.dim)
                                          : reinterpret_cast<const char*>(a.proto + n * a.dim);
                    for (int q = 0; q < kQuarters; ++q) {
                        const int b = q * kRowSlots + slot;
                        if (!tc::mbar_wait(&sm.row_empty[b], parity ^ 1u, &sm.err, 15, a.wait_cycles)) {
                            ok = false;
                            break;
                        }
                        tc::mbar_arrive_expect_tx(&sm.row_full[b], bytes);
                        tc::bulk_load_1d_hint(ring + ((size_t)q * S + slot) * item_bytes, src + (size_t)q * bytes,
                                              bytes, &sm.row_full[b], once);
                        ++issued[q];
                    }
                }
                ok = __shfl_sync(0xffffffffu, ok, 0);
                ++i;
                if (++slot == S) {
                    slot = 0;
                    parity ^= 1u;
                }
            }
        }
        run.row_ord = i;
        // copies still landing when the consumers gave up early: let them finish (bounded)
        if (lane == 0)
            for (int q = 0; q < kQuarters; ++q)
                for (int64_t k = ord0 + issued[q] - min(issued[q], (int64_t)S); k < ord0 + issued[q]; ++k) {
                    const long long c0 = clock64();
                    while (!tc::mbar_try_wait(tc::smem_u32(&sm.row_full[q * kRowSlots + (int)(k % S)]),
                                              (uint32_t)((k / S) & 1)) &&
                           clock64() - c0 < tc::kWaitCycles) {
                    }
                }
        __syncwarp();
        return;
    }
    // consumers: warp c = 4 g + q scores quarter q of group g's pairs.  The CTA's pair list is cut
    // into chunks of two consecutive pairs, chunk t going to group t % 3, so group g's k-th pair
    // is at position P0 + 2 g + 6 (k / 2) + k % 2; the two pairs of a chunk inside one node are
    // scored together from one read of the row.
    if (warp > kRowConsumers) return;  // the CTA's warps past the consumers have no part here
    const int c = warp - 1, q = c % kQuarters, g = c / kQuarters;
    const int64_t P0 = a.node_off[n_lo], P1 = a.node_off[n_hi];
    const int64_t g0 = P0 + 2 * g;
    const int64_t span = P1 - g0;
    const int64_t nk = span > 0 ? 2 * (span / 6) + min((int64_t)2, span % 6) : 0;
    auto pos = [&](int64_t k) { return g0 + 6 * (k >> 1) + (k & 1); };
    uint8_t* wbits = bits_sm + (size_t)c * kBitsBufs * qbits_bytes;
    int64_t* part = a.part + (size_t)q * a.pstride;
    // lane j holds the pair index and read of the group's pair 32 b + j, for the current batch
    // b and the next one
    int64_t batch = 0;
    int32_t pi_cur = -1, r_cur = 0, pi_nxt = -1, r_nxt = 0;
    auto load_batch = [&](int64_t b, int32_t& pi, int32_t& r) {
        const int64_t k = 32 * b + lane;
        pi = -1;
        r = 0;
        if (k < nk) {
            pi = a.sorted[pos(k)];
            r = a.pair_read[pi];
        }
    };
    load_batch(0, pi_cur, r_cur);
    load_batch(1, pi_nxt, r_nxt);
    // quarter q of the bits of pair k (in the current or the next batch) into buffer
    // k % kBitsBufs; one cp.async group per pair, possibly empty, so the waits below count pairs
    int64_t issued = 0;
    auto prefetch_to = [&](int64_t last) {
        for (; issued <= last; ++issued) {
            const int64_t k = issued;
            if (k < nk) {
                // k is the same in every lane; the next batch's indices are only read once needed
                const int64_t r = (k >> 5) == batch ? __shfl_sync(0xffffffffu, r_cur, (int)(k & 31))
                                                    : __shfl_sync(0xffffffffu, r_nxt, (int)(k & 31));
                const char* src = reinterpret_cast<const char*>(a.bits + r * a.words) + (size_t)q * qbits_bytes;
                uint8_t* dst = wbits + (size_t)(k % kBitsBufs) * qbits_bytes;
                for (uint32_t o = 16u * lane; o < qbits_bytes; o += 512u) cp_async16(dst + o, src + o, 16);
            }
            cp_async_commit();
        }
    };
    auto qbits = [&](int64_t k) {
        return reinterpret_cast<const uint32_t*>(wbits + (size_t)(k % kBitsBufs) * qbits_bytes);
    };
    int64_t k = 0;
    int64_t s = nk > 0 ? pos(0) : P1;  // the group's next pair position
    int64_t i = run.row_ord;
    int slot = (int)(i % S);  // i % S and (i / S) & 1, kept incrementally
    uint32_t parity = (uint32_t)((i / S) & 1);
    bool ok = true;
    // the node offsets 31 nodes at a time (lane j holds node_off[nb + j]), the next batch's
    // loaded while this one is walked
    int32_t offn = n_lo + lane <= a.n_nodes ? a.node_off[n_lo + lane] : 0;
    for (int64_t nb = n_lo; ok && nb < n_hi; nb += 31) {
        const int32_t offv = offn;
        offn = nb + 31 + lane <= a.n_nodes ? a.node_off[nb + 31 + lane] : 0;
        const int cnt = (int)min((int64_t)31, n_hi - nb);
        for (int j = 0; j < cnt; ++j) {
            const int32_t ps = __shfl_sync(0xffffffffu, offv, j), pe = __shfl_sync(0xffffffffu, offv, j + 1);
            if (ps == pe) continue;
            const int64_t n = nb + j;
            const int b = q * kRowSlots + slot;
            if (!tc::mbar_wait(&sm.row_full[b], parity, &sm.err, 16, a.wait_cycles)) {
                ok = false;
                break;
            }
            ++i;
            const int4* rowv = reinterpret_cast<const int4*>(ring + ((size_t)q * S + slot) * item_bytes) + lane;
            const bool w16 = n >= a.n32;
            while (s < pe) {
                while ((k >> 5) > batch) {  // a new batch: its indices move up
                    ++batch;
                    pi_cur = pi_nxt;
                    r_cur = r_nxt;
                    load_batch(batch + 1, pi_nxt, r_nxt);
                }
                const int u = w16 && (k & 1) == 0 && s + 1 < pe ? 2 : 1;  // both pairs of the chunk in this node
                prefetch_to(k + u + 1);  // the bits of the next pairs are on their way while these are scored
                cp_async_wait<2>();      // this lane's copies of pairs k .. k + u - 1 have landed
                __syncwarp();            // and every lane's
                if (u == 2) {  // quarters of an int16 row: |dot| <= 4,096 x 32,767 each, summed in int32
                    int2 d = smem_dot16x2(rowv, qbits(k), qbits(k + 1), lane, qdim / 256);
                    for (int o = 16; o; o >>= 1) {
                        d.x += __shfl_xor_sync(0xffffffffu, d.x, o);
                        d.y += __shfl_xor_sync(0xffffffffu, d.y, o);
                    }
                    if (lane == (int)(k & 31)) part[pi_cur] = d.x;
                    if (lane == (int)((k + 1) & 31)) part[pi_cur] = d.y;
                } else {
                    int64_t acc;
                    if (w16) {
                        int a32 = smem_dot16(rowv, qbits(k), lane, qdim / 256);
                        for (int o = 16; o; o >>= 1) a32 += __shfl_xor_sync(0xffffffffu, a32, o);
                        acc = a32;
                    } else {
                        acc = smem_dot32(rowv, qbits(k), lane, qdim / 128);
                        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
                    }
                    if (lane == (int)(k & 31)) part[pi_cur] = acc;
                }
                __syncwarp();  // these buffers are refilled by the prefetches of the next pairs
                k += u;
                s = k < nk ? pos(k) : P1;
            }
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&sm.row_empty[b]);
            if (++slot == S) {
                slot = 0;
                parity ^= 1u;
            }
        }
    }
    run.row_ord = i;
    cp_async_wait<0>();  // no copy may still be landing when the phase ends
}

// The keys of the pairs of reads [r0, r1) from a streamed level's partial dots (every thread of
// the CTA, the pairs spread over its threads).
__device__ void keys_from_parts(const GArgs& a, int64_t r0, int64_t r1) {
    for (int64_t p = a.off[r0] + threadIdx.x; p < a.off[r1]; p += blockDim.x) {
        int64_t dot = 0;
#pragma unroll
        for (int q = 0; q < kQuarters; ++q) dot += a.part[(size_t)q * a.pstride + p];
        const int32_t node = a.pair_node[p];
        a.pair_key[p] = make_key(exact_score(dot, a.qn[a.pair_read[p]], a.pn[node], a.mode), (uint32_t)node);
    }
}

// The last level scored apart from the one-launch descent, which stops once that level's
// pairs are in node order (HDC_BEAM_ONE_LAUNCH 2): one more cooperative launch of score_kernel's
// shape (more warps per SM than the descent's CTA holds) scores them, then, past a bounded grid
// barrier, takes each read's final beam (one warp per read) and writes its output.  Selecting a
// read's beam in the scoring phase, by whichever warp retired its last pair, cost 1.9 ms of a
// 15 ms step (the count's atomics and the selects' dependent loads wait behind the level's row
// traffic).  Nothing runs when the descent gave up (abort raised): its pair arrays are then
// incomplete; a barrier that runs out of time raises it and reports status 120.
struct LeafArgs {
    int L;
    int32_t* path;
    float* path_score;
    int32_t* depth;
    unsigned* bar_count;  // the descent's grid barrier words, reused (both zero-based at rest)
    unsigned* bar_gen;
    int* abort;
    int* status;
};

// with int32 rows alone one CTA fewer per SM than score_kernel<false>: the select's registers
constexpr int kLeafBlocks32 = kScoreBlocks - 2;

template <bool ROWS16>
__global__ void __launch_bounds__(kScoreThreads, ROWS16 ? kScoreBlocks16 : kLeafBlocks32)
    leaf_kernel(const GArgs a, const LeafArgs l) {
    __shared__ int ok_s;
    if (ld_volatile(l.abort)) return;  // the same for every CTA: the descent finished before this launch
    const int64_t w = (((int64_t)blockIdx.x * blockDim.x) >> 5) + (threadIdx.x >> 5);
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    score_pairs<ROWS16>(a, w, nw);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned g = ld_acquire_gpu(l.bar_gen);
        if (atomicAdd(l.bar_count, 1u) == gridDim.x - 1) {
            atomicExch(l.bar_count, 0u);
            __threadfence();
            st_release_gpu(l.bar_gen, g + 1);
        } else {
            const long long t0 = clock64();
            while (ld_acquire_gpu(l.bar_gen) == g) {
                if (ld_volatile(l.abort)) break;
                if (clock64() - t0 > a.wait_cycles) {
                    if (atomicExch(l.abort, 1) == 0) atomicCAS(l.status, 0, 100 + kCodeGridBarrier);
                    break;
                }
                __nanosleep(64);
            }
        }
        ok_s = ld_volatile(l.abort) == 0;
    }
    __syncthreads();
    if (!ok_s) return;
    // 16 lanes a read here: the scoring phase's registers leave no room for 8 keys a lane
    select_reads<16>(a, l.L, w, a.nq, nw, [&](int64_t r) { output_one(a, r, l.path, l.path_score, l.depth); });
}

__global__ void __launch_bounds__(TcOne::kThreads, 1) descent_one_kernel(const GArgs a, const TcItems t, const OneArgs o) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ TcShared sm;
    __shared__ int32_t sh[32];
    __shared__ int ok_s;
    __shared__ int n_ts;
    uint8_t* ring = tc_ring(smem_raw);
    if (threadIdx.x == 0) {
        n_ts = 0;
        if (blockIdx.x == 0) o.phase_ts[n_ts++] = global_ns();
    }
    uint4* staging = reinterpret_cast<uint4*>(ring + (size_t)TcOne::kStages * kTcStageBytes);
    if (o.use_tc) {
        tc_setup<TcOne>(sm);
    } else {
        if (threadIdx.x == 0) sm.err = 0;
        __syncthreads();
    }
    TcRun run;
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    // this CTA's reads [r0, r1) and nodes [n0, n1)
    const int64_t rc = (a.nq + G - 1) / G, r0 = min(a.nq, (int64_t)b * rc), r1 = min(a.nq, r0 + rc);
    const int64_t ncn = (a.n_nodes + G - 1) / G, n0 = min(a.n_nodes, (int64_t)b * ncn), n1 = min(a.n_nodes, n0 + ncn);
    const bool last_reads = r0 < r1 && r1 == a.nq, last_nodes = n0 < n1 && n1 == a.n_nodes;
    const int64_t gtid = (int64_t)b * nt + tid, gstride = (int64_t)G * nt;
    int32_t* blk0 = o.blk;
    int32_t* blk1 = o.blk + G;
    int32_t* blk2 = o.blk + 2 * G;
    const bool rows16 = a.n32 < a.n_nodes;

    for (int64_t r = r0 + tid; r < r1; r += nt) {
        a.nbeam[r] = 0;
        a.done[r] = 0;
        a.out_depth[r] = 0;
    }
    if (o.maxc) {  // the caller's largest child count is checked against the tree's
        int32_t m = 0;
        for (int64_t i = gtid; i < a.n_nodes; i += gstride) m = max(m, (int32_t)(a.child_ptr[i + 1] - a.child_ptr[i]));
        for (int off = 16; off; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
        if ((tid & 31) == 0 && m) atomicMax(o.maxc, m);
    }
    if (o.late_cta && b == 0 && tid == 0) {  // test hook: the other CTAs' first wait runs out
        const long long t0 = clock64();
        while (clock64() - t0 < 4 * o.wait_cycles) __nanosleep(256);
    }
    bool ok = grid_barrier(o, sm, &ok_s, &n_ts);
    if (ok && o.maxc && ld_volatile(o.maxc) > o.given) {
        // too small: the pair arrays could overflow, so every read stops at depth 0
        for (int64_t r = r0 + tid; r < r1; r += nt) a.done[r] = 1;
        if (b == 0 && tid == 0) atomicCAS(o.status, 0, kStatusChildCount);
    }
    __syncthreads();
    bool apart_done = false;
    for (int L = 0; ok && L < a.levels; ++L) {
        const bool tcl = o.use_tc && L < a.levels - 1;
        // A: candidate counts of this CTA's reads and their sum; zero this level's node counters
        for (int64_t r = r0 + tid; r < r1; r += nt) a.cnt[r] = count_one(a, L, r);
        int32_t* node_counter = tcl ? (L > 0 ? t.par_cnt : nullptr) : a.node_cnt;
        if (node_counter)
            for (int64_t i = gtid; i < a.n_nodes; i += gstride) node_counter[i] = 0;
        __syncthreads();
        int32_t sum = cta_sum(a.cnt, r0, r1, sh);
        if (tid == 0) blk0[b] = sum;
        if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
        // B: pair offsets of this CTA's reads, their pairs and (tensor-core levels) the entries per parent
        int32_t base = cta_prefix(blk0, b, sh);
        int32_t total = cta_scan(a.cnt, a.off, nullptr, r0, r1, base, sh);
        if (last_reads && tid == 0) a.off[a.nq] = total;
        __syncthreads();
        for (int64_t i = r0 * a.beam + tid; i < r1 * a.beam; i += nt)
            expand_entry(a, L, i / a.beam, (int)(i % a.beam), !tcl, tcl && L > 0 ? t.par_cnt : nullptr);
        if (tcl && L == 0) items_level0_range(a, t, gtid, gstride);
        if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
        if (tcl) {
            if (L > 0) {
                // C: entries per parent, summed per CTA
                sum = cta_sum(t.par_cnt, n0, n1, sh);
                if (tid == 0) blk0[b] = sum;
                if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
                // D: parent offsets and cursors; items per parent and the small parents, summed per CTA
                base = cta_prefix(blk0, b, sh);
                total = cta_scan(t.par_cnt, t.par_off, t.par_cursor, n0, n1, base, sh);
                if (last_nodes && tid == 0) t.par_off[a.n_nodes] = total;
                for (int64_t P = n0 + tid; P < n1; P += nt) item_count_one(a, t, P);
                __syncthreads();
                sum = cta_sum(t.item_cnt, n0, n1, sh);
                const int32_t sum2 = cta_sum(t.small, n0, n1, sh);
                if (tid == 0) {
                    blk1[b] = sum;
                    blk2[b] = sum2;
                }
                if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
                // E: entries to their parents' slots; item and small-parent offsets
                for (int64_t r = r0 + tid; r < r1; r += nt) par_scatter_one(a, t, L, r);
                base = cta_prefix(blk1, b, sh);
                total = cta_scan(t.item_cnt, t.item_off, nullptr, n0, n1, base, sh);
                if (last_nodes && tid == 0) t.item_off[a.n_nodes] = total;
                base = cta_prefix(blk2, b, sh);
                total = cta_scan(t.small, t.small_off, nullptr, n0, n1, base, sh);
                if (last_nodes && tid == 0) t.small_off[a.n_nodes] = total;
                if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
                // F: the items
                for (int64_t P = n0 + tid; P < n1; P += nt) item_write_one(a, t, P);
                if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
            }
            // G: the level's pairs scored on the tensor cores
            tc_phase<TcOne>(a, t, sm, run, ring, staging);
        } else {
            // C: pairs per node, summed per CTA
            sum = cta_sum(a.node_cnt, n0, n1, sh);
            if (tid == 0) blk0[b] = sum;
            if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
            // D: node offsets and cursors
            base = cta_prefix(blk0, b, sh);
            total = cta_scan(a.node_cnt, a.node_off, a.cursor, n0, n1, base, sh);
            if (last_nodes && tid == 0) a.node_off[a.n_nodes] = total;
            if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
            // E: the pairs in node order
            scatter_range(a, gtid, gstride);
            if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
            if (o.leaf_apart && L == a.levels - 1) {
                // the last level is scored and selected by leaf_kernel
                apart_done = true;
                break;
            }
            // F: the pairs scored on the CUDA cores: the leaf level's rows streamed through shared
            // memory, other levels (every level without the tensor cores) one warp per pair
            if (o.use_tc)
                stream_phase(a, sm, run, ring, kOneSmem - 1024);
            else if (rows16)
                score_pairs<true>(a, gtid >> 5, gstride >> 5);
            else
                score_pairs<false>(a, gtid >> 5, gstride >> 5);
        }
        if (!(ok = grid_barrier(o, sm, &ok_s, &n_ts))) break;
        // H: the beams of this CTA's reads (after a streamed level, their pairs' keys first)
        if (o.use_tc && !tcl && r0 < r1) {
            keys_from_parts(a, r0, r1);
            __syncthreads();
        }
        select_reads(a, L, r0 + (tid >> 5), r1, nt >> 5, [](int64_t) {});
        __syncthreads();
    }
    if (ok && !apart_done)
        for (int64_t r = r0 + tid; r < r1; r += nt) output_one(a, r, o.out_path, o.out_score, o.out_depth);
    if (b == 0 && tid == 0) {
        if (n_ts < kMaxPhaseTs) o.phase_ts[n_ts++] = global_ns();
        for (int i = n_ts; i < kMaxPhaseTs; ++i) o.phase_ts[i] = 0;
    }
    if (o.use_tc) {
        tc_teardown<TcOne>(sm, o.status);
    } else if (tid == 0 && sm.err) {
        atomicCAS(o.status, 0, 100 + sm.err);
    }
}

// The one-launch descent needs every CTA (one per SM) resident at once; checked once per
// context, with the kernel's shared memory set.
bool one_launch_fits(hdc_context* ctx) {
    if (ctx->beam_one == 0) return false;
    if (ctx->beam_one_fit < 0) {
        int per_sm = 0;
        cudaError_t e = cudaFuncSetAttribute(descent_one_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kOneSmem);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, descent_one_kernel, TcOne::kThreads, kOneSmem);
        int coop = 0;
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
        cudaGetLastError();
        ctx->beam_one_fit = e == cudaSuccess && per_sm >= 1 && coop ? 1 : 0;
    }
    return ctx->beam_one_fit == 1;
}

template <typename T>
T* carve(uint8_t*& cur, int64_t n) {
    T* p = reinterpret_cast<T*>(cur);
    cur += ((size_t)std::max<int64_t>(n, 1) * sizeof(T) + 255) & ~(size_t)255;
    return p;
}

}  // namespace

int launch_beam_grouped(hdc_context* ctx, const int8_t* d_q, const uint32_t* d_qbits, const int64_t* d_qn, int64_t nq,
                        const int32_t* d_proto,
                        int64_t n32, const int16_t* d_proto16, const int64_t* d_pn, int64_t n_nodes, const int64_t* d_child_ptr, const int32_t* d_child_idx,
                        const int32_t* d_roots, int n_roots, int max_children, int levels, int beam,
                        double threshold, int mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                        cudaStream_t stream) {
    if ((int64_t)n_nodes > (int64_t)kScanBlock * kScanBlock || nq > (int64_t)kScanBlock * kScanBlock)
        return fail(HDC_ERR_INVALID, "beam: too many reads or nodes for one grouped launch");
    cudaError_t e;
    // the largest child count bounds a read's candidates, hence the pair arrays: the caller's
    // value (checked on the device below), or read back from the device
    const unsigned mc_grid = (unsigned)std::max(1, std::min(ctx->num_sms * 4, (int)((n_nodes + 255) / 256)));
    int32_t maxc = max_children;
    if (maxc <= 0) {
        int32_t* d_maxc = nullptr;
        if ((e = cudaMallocAsync(&d_maxc, sizeof(int32_t), stream)) != cudaSuccess)
            return cuda_fail(e, "beam: workspace");
        cudaMemsetAsync(d_maxc, 0, sizeof(int32_t), stream);
        max_children_kernel<<<mc_grid, 256, 0, stream>>>(d_child_ptr, n_nodes, d_maxc);
        cudaMemcpyAsync(&maxc, d_maxc, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
        cudaFreeAsync(d_maxc, stream);
        if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_fail(e, "beam: child count");
    }
    const int64_t per_read = std::max<int64_t>(n_roots, (int64_t)beam * std::max(maxc, 1));
    const int64_t P = nq * per_read;
    if (P > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "beam: too many candidate pairs for one grouped launch");

    GArgs a{};
    a.nq = nq;
    a.dim = ctx->dim;
    a.words = ctx->dim / 32;
    a.steps = ctx->dim / 1024;
    a.levels = levels;
    a.beam = beam;
    a.mode = mode;
    a.n_roots = n_roots;
    a.n_nodes = n_nodes;
    a.threshold = threshold;
    a.qn = d_qn;
    a.proto = d_proto;
    a.proto16 = d_proto16;
    a.n32 = n32;
    a.pn = d_pn;
    a.child_ptr = d_child_ptr;
    a.child_idx = d_child_idx;
    a.roots = d_roots;
    a.wait_cycles = ctx->wait_cycles > 0 ? ctx->wait_cycles : tc::kWaitCycles;
    const int64_t sums = std::max(scan_blocks_needed(nq), scan_blocks_needed(n_nodes));
    int32_t* d_sums = nullptr;
    int32_t* d_maxc_dev = nullptr;
    uint32_t* bits = nullptr;
    uint32_t* one_state = nullptr;
    int32_t* one_blk = nullptr;
    // every level but the last on the tensor cores (HDC_BEAM_GROUPED 2 or automatic)
    const bool use_tc = (ctx->beam_grouped == 2 || ctx->beam_grouped < 0) && a.dim % 64 == 0 && a.dim <= 16384;
    TcItems t{};
    t.status = ctx->d_status;
    const int64_t cchunks = (std::max<int64_t>(std::max(maxc, n_roots), 1) + kTcC - 1) / kTcC;
    const int64_t max_items = (nq * beam + 2) * cchunks + ((nq + kTcE - 1) / kTcE) * ((n_roots + kTcC - 1) / kTcC);
    const bool one = one_launch_fits(ctx);
    // carve the workspace: once from address 0 to measure it, then from the allocation
    auto carve_all = [&](uint8_t* base) {
        uint8_t* cur = base;
        if (!d_qbits) bits = carve<uint32_t>(cur, nq * a.words);
        a.paths = carve<int32_t>(cur, nq * kMaxBeamG * kMaxLevelsG);
        a.scores = carve<float>(cur, nq * kMaxBeamG * kMaxLevelsG);
        a.nbeam = carve<int32_t>(cur, nq);
        a.done = carve<int32_t>(cur, nq);
        a.out_depth = carve<int32_t>(cur, nq);
        a.cnt = carve<int32_t>(cur, nq);
        a.off = carve<int32_t>(cur, nq + 1);
        a.node_cnt = carve<int32_t>(cur, n_nodes);
        a.node_off = carve<int32_t>(cur, n_nodes + 1);
        a.cursor = carve<int32_t>(cur, n_nodes);
        a.pair_read = carve<int32_t>(cur, P);
        a.pair_node = carve<int32_t>(cur, P);
        a.pair_slot = carve<int32_t>(cur, P);
        a.sorted = carve<int32_t>(cur, P);
        a.pair_key = carve<uint64_t>(cur, P);
        if (one && use_tc) {
            a.part = carve<int64_t>(cur, (int64_t)kQuarters * P);
            a.pstride = P;
        }
        d_sums = carve<int32_t>(cur, sums);
        d_maxc_dev = carve<int32_t>(cur, 1);
        one_state = carve<uint32_t>(cur, 4);  // barrier count, barrier generation, abort, child count
        one_blk = carve<int32_t>(cur, 3 * (int64_t)ctx->num_sms);
        if (use_tc) {
            t.ent_read = carve<int32_t>(cur, nq * beam);
            t.ent_p0 = carve<int32_t>(cur, nq * beam);
            t.par_cnt = carve<int32_t>(cur, n_nodes);
            t.par_off = carve<int32_t>(cur, n_nodes + 1);
            t.par_cursor = carve<int32_t>(cur, n_nodes);
            t.item_cnt = carve<int32_t>(cur, n_nodes);
            t.item_off = carve<int32_t>(cur, n_nodes + 1);
            t.small = carve<int32_t>(cur, n_nodes);
            t.small_off = carve<int32_t>(cur, n_nodes + 1);
            t.fit2 = carve<int32_t>(cur, n_nodes);
            t.item_par = carve<int32_t>(cur, max_items);
            t.item_e0 = carve<int32_t>(cur, max_items);
            t.item_j0 = carve<int32_t>(cur, max_items);
        }
        return (size_t)(cur - base);
    };
    const size_t bytes = carve_all(nullptr);
    uint8_t* ws = nullptr;
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, stream)) != cudaSuccess)
        return cuda_fail(e, "beam: workspace");
    carve_all(ws);
    a.bits = d_qbits ? d_qbits : bits;

    const unsigned rb = (unsigned)((nq + 255) / 256);
    if (!d_qbits) pack_bits_kernel<<<(unsigned)((nq * a.words + 255) / 256), 256, 0, stream>>>(d_q, nq, a.dim, bits);
    if (one) {
        // every level in one cooperative launch (descent_one_kernel)
        OneArgs o{};
        o.bar_count = one_state;
        o.bar_gen = one_state + 1;
        o.abort = reinterpret_cast<int*>(one_state + 2);
        o.maxc = max_children > 0 ? reinterpret_cast<int32_t*>(one_state + 3) : nullptr;
        o.given = max_children;
        o.blk = one_blk;
        o.status = ctx->d_status;
        o.use_tc = use_tc ? 1 : 0;
        o.out_path = d_path;
        o.out_score = d_path_score;
        o.out_depth = d_depth;
        if (!ctx->d_phase_ts) {
            e = cudaMalloc(&ctx->d_phase_ts, kMaxPhaseTs * sizeof(unsigned long long));
            if (e == cudaSuccess) e = cudaMemset(ctx->d_phase_ts, 0, kMaxPhaseTs * sizeof(unsigned long long));
            if (e != cudaSuccess) {
                cudaFreeAsync(ws, stream);
                return cuda_fail(e, "beam: phase clock buffer");
            }
        }
        o.phase_ts = ctx->d_phase_ts;
        o.wait_cycles = a.wait_cycles;
        o.late_cta = ctx->test_withhold_loads == 2 ? 1 : 0;
        o.leaf_apart = ctx->beam_one != 1 ? 1 : 0;  // automatic: the last level in a launch of its own
        e = cudaMemsetAsync(one_state, 0, 4 * sizeof(uint32_t), stream);
        void* args[] = {(void*)&a, (void*)&t, (void*)&o};
        if (e == cudaSuccess)
            e = cudaLaunchCooperativeKernel((const void*)descent_one_kernel, dim3((unsigned)ctx->num_sms),
                                            dim3(TcOne::kThreads), args, kOneSmem, stream);
        if (e == cudaSuccess && o.leaf_apart) {
            LeafArgs l{levels - 1, d_path, d_path_score, d_depth, o.bar_count, o.bar_gen, o.abort, o.status};
            void* largs[] = {(void*)&a, (void*)&l};
            const bool r16 = n32 < n_nodes;
            const void* kern = r16 ? (const void*)leaf_kernel<true> : (const void*)leaf_kernel<false>;
            int per_sm = 0;
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kScoreThreads, 0);
            if (e == cudaSuccess) {
                per_sm = std::min(per_sm, r16 ? kScoreBlocks16 : kLeafBlocks32);
                e = per_sm < 1 ? cudaErrorCooperativeLaunchTooLarge
                               : cudaLaunchCooperativeKernel(kern, dim3((unsigned)(ctx->num_sms * per_sm)),
                                                             dim3(kScoreThreads), largs, 0, stream);
            }
        }
        cudaFreeAsync(ws, stream);
        return e == cudaSuccess ? HDC_OK : cuda_fail(e, "beam: one-launch descent");
    }
    cudaMemsetAsync(a.nbeam, 0, nq * 4, stream);
    cudaMemsetAsync(a.done, 0, nq * 4, stream);
    cudaMemsetAsync(a.out_depth, 0, nq * 4, stream);
    if (max_children > 0) {  // a count below the tree's: every read stops at depth 0 (no pair is written)
        cudaMemsetAsync(d_maxc_dev, 0, sizeof(int32_t), stream);
        max_children_kernel<<<mc_grid, 256, 0, stream>>>(d_child_ptr, n_nodes, d_maxc_dev);
        check_children_kernel<<<rb, 256, 0, stream>>>(a, d_maxc_dev, max_children, ctx->d_status);
    }
    const int work_grid = ctx->num_sms * 8;
    const unsigned nb = (unsigned)((n_nodes + 255) / 256);
    if (use_tc && (e = cudaFuncSetAttribute(descent_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            (int)TcLevel::kSmem)) != cudaSuccess) {
        cudaFreeAsync(ws, stream);
        return cuda_fail(e, "beam: tensor-core scoring setup");
    }
    for (int L = 0; L < levels; ++L) {
        const bool tc_level = use_tc && L < levels - 1;
        count_kernel<<<rb, 256, 0, stream>>>(a, L);
        exclusive_scan(a.cnt, a.off, nq, d_sums, stream);
        if (!tc_level) cudaMemsetAsync(a.node_cnt, 0, (size_t)n_nodes * 4, stream);
        expand_kernel<<<(unsigned)((nq * beam + 255) / 256), 256, 0, stream>>>(a, L, !tc_level);
        if (tc_level) {
            // entries grouped by parent, then items of up to 128 entries x 32 children
            if (L == 0) {
                const int64_t n0 = ((nq + kTcE - 1) / kTcE) * ((n_roots + kTcC - 1) / kTcC);
                items_level0_kernel<<<(unsigned)((n0 + 255) / 256), 256, 0, stream>>>(a, t);
            } else {
                cudaMemsetAsync(t.par_cnt, 0, (size_t)n_nodes * 4, stream);
                par_count_kernel<<<rb, 256, 0, stream>>>(a, t, L);
                exclusive_scan(t.par_cnt, t.par_off, n_nodes, d_sums, stream);
                cudaMemcpyAsync(t.par_cursor, t.par_off, (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, stream);
                par_scatter_kernel<<<rb, 256, 0, stream>>>(a, t, L);
                item_count_kernel<<<nb, 256, 0, stream>>>(a, t);
                exclusive_scan(t.item_cnt, t.item_off, n_nodes, d_sums, stream);
                exclusive_scan(t.small, t.small_off, n_nodes, d_sums, stream);
                item_write_kernel<<<nb, 256, 0, stream>>>(a, t);
            }
            descent_tc_kernel<<<ctx->num_sms, TcLevel::kThreads, TcLevel::kSmem, stream>>>(a, t);
        } else {
            exclusive_scan(a.node_cnt, a.node_off, n_nodes, d_sums, stream);
            cudaMemcpyAsync(a.cursor, a.node_off, (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, stream);
            scatter_kernel<<<work_grid, 256, 0, stream>>>(a);
            if (n32 < n_nodes)
                score_kernel<true><<<ctx->num_sms * kScoreBlocks16, kScoreThreads, 0, stream>>>(a);
            else
                score_kernel<false><<<ctx->num_sms * kScoreBlocks, kScoreThreads, 0, stream>>>(a);
        }
        select_kernel<<<(unsigned)((nq * kSelLanes + 255) / 256), 256, 0, stream>>>(a, L);
    }
    output_kernel<<<rb, 256, 0, stream>>>(a, d_path, d_path_score, d_depth);
    e = cudaGetLastError();
    cudaFreeAsync(ws, stream);
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "beam: grouped launch");
}

int beam_phase_times(const hdc_context* ctx, int64_t* out_ns, int max_n) {
    std::fill(out_ns, out_ns + max_n, 0);
    if (!ctx->d_phase_ts) return 0;
    unsigned long long ts[kMaxPhaseTs];
    cudaError_t e = cudaMemcpy(ts, ctx->d_phase_ts, sizeof ts, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return -1;
    int n = 0;
    while (n < kMaxPhaseTs && ts[n]) ++n;
    for (int i = 1; i < n && i - 1 < max_n; ++i) out_ns[i - 1] = (int64_t)(ts[i] - ts[i - 1]);
    return n > 0 ? n - 1 : 0;
}

}  // namespace hdc
