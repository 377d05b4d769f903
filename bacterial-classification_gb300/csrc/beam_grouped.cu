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
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kMaxBeamG = 8;
constexpr int kMaxLevelsG = 8;
constexpr int kScoreThreads = 256;          // 8 warps, one pair each at a time
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
    const int32_t* proto;     // [n_nodes][dim]
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
};

__device__ __forceinline__ int64_t state_at(int64_t r, int b, int l) {
    return (r * kMaxBeamG + b) * kMaxLevelsG + l;
}

__global__ void count_kernel(const GArgs a, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
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
    a.cnt[r] = c;
}

__device__ __forceinline__ void put_pair(const GArgs& a, int32_t p, int64_t r, int32_t node, int slot) {
    a.pair_read[p] = (int32_t)r;
    a.pair_node[p] = node;
    a.pair_slot[p] = slot;
    atomicAdd(a.node_cnt + node, 1);
}

__global__ void expand_kernel(const GArgs a, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq || a.done[r]) return;
    int32_t p = a.off[r];
    if (L == 0) {
        for (int i = 0; i < a.n_roots; ++i) put_pair(a, p++, r, a.roots[i], 0);
        return;
    }
    for (int b = 0; b < a.nbeam[r]; ++b) {
        const int32_t node = a.paths[state_at(r, b, L - 1)];
        const int64_t c0 = a.child_ptr[node], c1 = a.child_ptr[node + 1];
        if (c0 == c1) {
            put_pair(a, p++, r, node, b);
        } else {
            for (int64_t c = c0; c < c1; ++c) put_pair(a, p++, r, a.child_idx[c], b);
        }
    }
}

__global__ void scatter_kernel(const GArgs a) {
    const int32_t total = a.off[a.nq];
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x) {
        const int32_t pos = atomicAdd(a.cursor + a.pair_node[p], 1);
        a.sorted[pos] = (int32_t)p;
    }
}

// One warp per pair, the warps walking the pairs in node order: the pairs of a node are
// scored by neighbouring warps at about the same time, so its prototype row comes from
// DRAM once and from L1/L2 for the others.  Lane l covers dims 128 j + 4 l .. + 3; four
// 16-byte prototype loads are in flight per lane, and the read is its packed bits.
// -x in 32 bits, with wrap-around defined (exact for every prototype element but INT32_MIN,
// which hdc_beam_search excludes; widening before negating costs ~40 % of the kernel)
__device__ __forceinline__ int32_t neg32(int32_t x) { return (int32_t)(0u - (uint32_t)x); }

__global__ void __launch_bounds__(kScoreThreads) score_kernel(const GArgs a) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int32_t total = a.off[a.nq];
    const int nsteps = a.dim / 128;  // a multiple of 8 (dim % 1024 == 0)
    const int sh = (lane & 7) * 4;
    for (int64_t s = (((int64_t)blockIdx.x * blockDim.x) >> 5) + (threadIdx.x >> 5); s < total; s += nw) {
        const int32_t pi = a.sorted[s];
        const int32_t node = a.pair_node[pi];
        const int64_t r = a.pair_read[pi];
        const int32_t* row = a.proto + (int64_t)node * a.dim + 4 * lane;
        const uint32_t* qb = a.bits + r * a.words + (lane >> 3);
        int64_t acc = 0;
        for (int j = 0; j < nsteps; j += 4) {
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
        for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) a.pair_key[pi] = make_key(exact_score(acc, a.qn[r], a.pn[node], a.mode), (uint32_t)node);
    }
}

// Per read: the best `beam` candidates, then the rule of the per-read kernel (stop below
// the threshold with the best path, else keep the entries >= threshold, at most `beam`).
__global__ void select_kernel(const GArgs a, int L) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq || a.done[r]) return;
    uint64_t key[kMaxBeamG];
    int32_t node[kMaxBeamG], slot[kMaxBeamG];
    int n = 0;
    for (int32_t p = a.off[r]; p < a.off[r + 1]; ++p) {
        const uint64_t k = a.pair_key[p];
        if (n < a.beam || k > key[n - 1]) {
            int pos = n < a.beam ? n++ : a.beam - 1;
            while (pos > 0 && key[pos - 1] < k) {
                key[pos] = key[pos - 1];
                node[pos] = node[pos - 1];
                slot[pos] = slot[pos - 1];
                --pos;
            }
            key[pos] = k;
            node[pos] = a.pair_node[p];
            slot[pos] = a.pair_slot[p];
        }
    }
    int32_t np[kMaxBeamG][kMaxLevelsG];
    float ns[kMaxBeamG][kMaxLevelsG];
    for (int t = 0; t < n; ++t) {  // new beam rows from their parents' rows
        for (int l = 0; l < L; ++l) {
            np[t][l] = a.paths[state_at(r, slot[t], l)];
            ns[t][l] = a.scores[state_at(r, slot[t], l)];
        }
        np[t][L] = node[t];
        ns[t][L] = key_score(key[t]);
    }
    const bool stop = n == 0 || (double)key_score(key[0]) < a.threshold;
    int keep = 0;
    if (stop) {
        a.out_depth[r] = n ? L + 1 : L;
        keep = n ? 1 : 0;  // the best candidate's path is the answer
        a.done[r] = 1;
    } else {
        while (keep < n && keep < a.beam && (double)key_score(key[keep]) >= a.threshold) ++keep;
        a.nbeam[r] = keep;
        if (L == a.levels - 1) {
            a.out_depth[r] = a.levels;
            a.done[r] = 1;
        }
    }
    for (int t = 0; t < keep; ++t)
        for (int l = 0; l <= L; ++l) {
            a.paths[state_at(r, t, l)] = np[t][l];
            a.scores[state_at(r, t, l)] = ns[t][l];
        }
}

__global__ void output_kernel(const GArgs a, int32_t* __restrict__ path, float* __restrict__ path_score,
                              int32_t* __restrict__ depth) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= a.nq) return;
    const int d = a.out_depth[r];
    for (int l = 0; l < a.levels; ++l) {
        path[r * a.levels + l] = l < d ? a.paths[state_at(r, 0, l)] : -1;
        path_score[r * a.levels + l] = l < d ? a.scores[state_at(r, 0, l)] : 0.0f;
    }
    depth[r] = d;
}

template <typename T>
T* carve(uint8_t*& cur, int64_t n) {
    T* p = reinterpret_cast<T*>(cur);
    cur += ((size_t)std::max<int64_t>(n, 1) * sizeof(T) + 255) & ~(size_t)255;
    return p;
}

}  // namespace

int launch_beam_grouped(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qn, int64_t nq, const int32_t* d_proto,
                        const int64_t* d_pn, int64_t n_nodes, const int64_t* d_child_ptr, const int32_t* d_child_idx,
                        const int32_t* d_roots, int n_roots, int levels, int beam, double threshold, int mode,
                        int32_t* d_path, float* d_path_score, int32_t* d_depth, cudaStream_t stream) {
    if ((int64_t)n_nodes > (int64_t)kScanBlock * kScanBlock || nq > (int64_t)kScanBlock * kScanBlock)
        return fail(HDC_ERR_INVALID, "beam: too many reads or nodes for one grouped launch");
    cudaError_t e;
    // the largest child count bounds a read's candidates, hence the pair arrays
    int32_t* d_maxc = nullptr;
    if ((e = cudaMallocAsync(&d_maxc, sizeof(int32_t), stream)) != cudaSuccess) return cuda_fail(e, "beam: workspace");
    cudaMemsetAsync(d_maxc, 0, sizeof(int32_t), stream);
    max_children_kernel<<<std::max(1, std::min(ctx->num_sms * 4, (int)((n_nodes + 255) / 256))), 256, 0, stream>>>(
        d_child_ptr, n_nodes, d_maxc);
    int32_t maxc = 0;
    cudaMemcpyAsync(&maxc, d_maxc, sizeof(int32_t), cudaMemcpyDeviceToHost, stream);
    cudaFreeAsync(d_maxc, stream);
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_fail(e, "beam: child count");
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
    a.pn = d_pn;
    a.child_ptr = d_child_ptr;
    a.child_idx = d_child_idx;
    a.roots = d_roots;
    const int64_t sums = std::max(scan_blocks_needed(nq), scan_blocks_needed(n_nodes));
    int32_t* d_sums = nullptr;
    uint32_t* bits = nullptr;
    // carve the workspace: once from address 0 to measure it, then from the allocation
    auto carve_all = [&](uint8_t* base) {
        uint8_t* cur = base;
        bits = carve<uint32_t>(cur, nq * a.words);
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
        d_sums = carve<int32_t>(cur, sums);
        return (size_t)(cur - base);
    };
    const size_t bytes = carve_all(nullptr);
    uint8_t* ws = nullptr;
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&ws), bytes, stream)) != cudaSuccess)
        return cuda_fail(e, "beam: workspace");
    carve_all(ws);
    a.bits = bits;

    const unsigned rb = (unsigned)((nq + 255) / 256);
    cudaMemsetAsync(a.nbeam, 0, nq * 4, stream);
    cudaMemsetAsync(a.done, 0, nq * 4, stream);
    cudaMemsetAsync(a.out_depth, 0, nq * 4, stream);
    pack_bits_kernel<<<(unsigned)((nq * a.words + 255) / 256), 256, 0, stream>>>(d_q, nq, a.dim, bits);
    const int work_grid = ctx->num_sms * 8;
    for (int L = 0; L < levels; ++L) {
        count_kernel<<<rb, 256, 0, stream>>>(a, L);
        exclusive_scan(a.cnt, a.off, nq, d_sums, stream);
        cudaMemsetAsync(a.node_cnt, 0, (size_t)n_nodes * 4, stream);
        expand_kernel<<<rb, 256, 0, stream>>>(a, L);
        exclusive_scan(a.node_cnt, a.node_off, n_nodes, d_sums, stream);
        cudaMemcpyAsync(a.cursor, a.node_off, (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, stream);
        scatter_kernel<<<work_grid, 256, 0, stream>>>(a);
        score_kernel<<<work_grid, kScoreThreads, 0, stream>>>(a);
        select_kernel<<<rb, 256, 0, stream>>>(a, L);
    }
    output_kernel<<<rb, 256, 0, stream>>>(a, d_path, d_path_score, d_depth);
    e = cudaGetLastError();
    cudaFreeAsync(ws, stream);
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "beam: grouped launch");
}

}  // namespace hdc
