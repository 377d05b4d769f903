// (c) propagate-children: greedy representative selection of taxonomy nodes.
//
// Reference semantics (targets/propogate-children.cpp:60-73): for one parent,
// visit its descendant sequences in order; for candidate x,
//     best = max(0, max over s in parent_seqs and added of cosine(x, s))
// with the NORM_COSINE score of src/HV.cpp:219-242 (float), and append x to
// the parent (and to `added`) when best < threshold (0.75).  The decision of
// a candidate depends on every earlier decision, so candidates are visited in
// order; the work inside one visit -- one exact dot product per current
// representative -- is spread over the CTA, and every parent of a rank runs
// in its own CTA at the same time.
//
// Hypervectors are whole-sequence int16 encodings (HVCache::get in the
// reference).  Dots are exact int64; the float score is the reference's
// double expression rounded to float, so the threshold decisions match the
// reference bit for bit.
//
// Two forms.  The scored form (dim % 8 == 0, the default) first computes, in
// bulk, every score a decision can need, then runs only the decisions in
// order: a parent's candidates are taken in blocks of kGB; for a block,
//   * fixed_kernel: each candidate against the parent's existing sequences
//     and the candidates appended in earlier blocks, keeping the largest
//     score per candidate (tiles of 32 x 32 dot products);
//   * tri_kernel: each candidate against every earlier candidate of the
//     block (the lower triangle, stored column by column);
//   * scan_kernel: one CTA per parent decides the block's candidates in order
//     from a running best per candidate, raised by the column of every
//     candidate it appends (the reference's max over the parent's sequences
//     is order-free, so the running maximum gives the same float).
// The sequential form (greedy_kernel: one CTA per parent, each decision one
// exact dot per current representative) serves the other dims.
#include <algorithm>
#include <vector>

#include "hdc_internal.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kThreadsG = 256;
constexpr int kWarpsG = kThreadsG / 32;

// exact dot of two int16 rows of length dim, computed by one warp
__device__ __forceinline__ int64_t warp_dot(const int16_t* __restrict__ a, const int16_t* __restrict__ b, int dim,
                                            bool vec) {
    const int lane = threadIdx.x & 31;
    int64_t acc = 0;
    if (vec) {
        const uint4* a4 = reinterpret_cast<const uint4*>(a);
        const uint4* b4 = reinterpret_cast<const uint4*>(b);
        for (int i = lane; i < dim / 8; i += 32) {
            const uint4 x = __ldg(a4 + i), y = __ldg(b4 + i);
            const uint32_t xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int32_t p0 = (int32_t)(int16_t)(xs[u] & 0xffff) * (int32_t)(int16_t)(ys[u] & 0xffff);
                const int32_t p1 = (int32_t)(int16_t)(xs[u] >> 16) * (int32_t)(int16_t)(ys[u] >> 16);
                acc += (int64_t)p0 + (int64_t)p1;  // each product fits int32
            }
        }
    } else {
        for (int i = lane; i < dim; i += 32) acc += (int64_t)a[i] * (int64_t)b[i];
    }
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

struct GreedyArgs {
    const int16_t* hv;      // [n_hv][dim] whole-sequence hypervectors
    const int64_t* norm2;   // [n_hv]
    int dim;
    const int64_t* cand_ptr;  // [n_parents+1] into cand_idx
    const int32_t* cand_idx;  // candidate hypervector indices, in visiting order
    const int64_t* rep_ptr;   // [n_parents+1] into rep_idx
    const int32_t* rep_idx;   // the parent's existing sequences
    double threshold;
    int mode;
    uint8_t* selected;        // [cand_ptr[n]] 1 when the candidate is appended
    float* best_out;          // [cand_ptr[n]] best score seen by the candidate
    int32_t* added;           // [cand_ptr[n]] scratch: the appended candidates of each parent
};

__global__ void __launch_bounds__(kThreadsG) greedy_kernel(const GreedyArgs a) {
    const int64_t p = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t c0 = a.cand_ptr[p], c1 = a.cand_ptr[p + 1];
    const int64_t r0 = a.rep_ptr[p], r1 = a.rep_ptr[p + 1];
    const bool vec = (a.dim % 8) == 0;
    __shared__ float warp_best[kWarpsG];
    __shared__ int n_added_s;
    if (threadIdx.x == 0) n_added_s = 0;
    __syncthreads();
    int32_t* added = a.added + c0;
    for (int64_t c = c0; c < c1; ++c) {
        const int32_t x = a.cand_idx[c];
        const int16_t* xv = a.hv + (int64_t)x * a.dim;
        const int64_t xn = a.norm2[x];
        const int n_added = n_added_s;
        const int64_t n_reps = (r1 - r0) + n_added;
        float best = 0.0f;  // the reference starts from 0 (targets/propogate-children.cpp:63)
        for (int64_t j = warp; j < n_reps; j += kWarpsG) {
            const int32_t s = j < (r1 - r0) ? a.rep_idx[r0 + j] : added[j - (r1 - r0)];
            const int64_t dot = warp_dot(xv, a.hv + (int64_t)s * a.dim, a.dim, vec);
            const float sc = exact_score(dot, xn, a.norm2[s], a.mode);
            best = fmaxf(best, sc);  // std::max(best, score); scores are never NaN
        }
        if (lane == 0) warp_best[warp] = best;
        __syncthreads();
        if (threadIdx.x == 0) {
            float b = 0.0f;
            for (int w = 0; w < kWarpsG; ++w) b = fmaxf(b, warp_best[w]);
            const bool take = (double)b < a.threshold;
            a.selected[c] = take ? 1 : 0;
            if (a.best_out) a.best_out[c] = b;
            if (take) added[n_added_s++] = x;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- scored form
constexpr int kGB = 1024;        // candidates per block of a parent
constexpr int kTileT = 256;      // threads of a tile CTA: 32 x 32 dot products, 4 per thread

// A tile of 32 rows (candidates of a block) x 32 columns.
struct GTile {
    int64_t rows_at;   // cand_idx offset of the block's first candidate
    int64_t tri_off;   // tri tiles: the block's triangle in the score buffer
    int32_t n;         // candidates in the block
    int32_t ib, jb;    // row / column tile
    int32_t parent;    // fixed tiles: the parent (its column list)
    int32_t ncols;     // fixed tiles: existing sequences + candidates appended so far
};

struct GScoredArgs {
    const int16_t* hv;
    const int64_t* norm2;
    int dim, mode;
    const int64_t* cand_ptr;
    const int32_t* cand_idx;
    const int64_t* rep_ptr;
    const int32_t* rep_idx;
    const int32_t* added;       // [cand_ptr[n]] the appended candidates of each parent, from cand_ptr[p] on
    const int32_t* n_added;     // [n_parents]
    uint32_t* prevmax;          // [cand_ptr[n]] ord_float of the largest fixed-column score of each candidate
    float* tri;                 // triangles of the current block
};

// Column j of a triangle over n rows holds rows j + 1 .. n - 1.
__device__ __forceinline__ int64_t tri_col(int64_t j, int64_t n) { return j * n - j * (j + 1) / 2; }

// The 4 exact dots of thread t (row t >> 3, columns (t & 7) + 8 u) of a 32 x 32 tile: rows and
// columns are hypervector indices (-1: none) in shared memory, the vectors staged 64 dims at a
// time as int16 pairs (rows of 33 words: conflict-free).
__device__ void tile_dots(const GScoredArgs& a, const int32_t* rid, const int32_t* cid, uint32_t (*rs)[33],
                          uint32_t (*cs)[33], int64_t (&acc)[4]) {
    const int t = threadIdx.x, r = t >> 3, c0 = t & 7;
    const int vr = t >> 3, part = t & 7;  // staging: vector vr, 16 bytes `part` of the chunk
#pragma unroll
    for (int u = 0; u < 4; ++u) acc[u] = 0;
    for (int d0 = 0; d0 < a.dim; d0 += 64) {
        const bool in = d0 + 8 * part < a.dim;
        uint4 x = make_uint4(0, 0, 0, 0), y = make_uint4(0, 0, 0, 0);
        if (in && rid[vr] >= 0) x = __ldg(reinterpret_cast<const uint4*>(a.hv + (int64_t)rid[vr] * a.dim + d0) + part);
        if (in && cid[vr] >= 0) y = __ldg(reinterpret_cast<const uint4*>(a.hv + (int64_t)cid[vr] * a.dim + d0) + part);
        rs[vr][4 * part] = x.x;
        rs[vr][4 * part + 1] = x.y;
        rs[vr][4 * part + 2] = x.z;
        rs[vr][4 * part + 3] = x.w;
        cs[vr][4 * part] = y.x;
        cs[vr][4 * part + 1] = y.y;
        cs[vr][4 * part + 2] = y.z;
        cs[vr][4 * part + 3] = y.w;
        __syncthreads();
#pragma unroll 4
        for (int w = 0; w < 32; ++w) {
            const uint32_t xv = rs[r][w];
            const int32_t xl = (int32_t)(int16_t)(xv & 0xffffu), xh = (int32_t)xv >> 16;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const uint32_t yv = cs[c0 + 8 * u][w];
                // each product fits int32 (|int16| <= 2^15); their sum may not
                acc[u] += (int64_t)(xl * (int32_t)(int16_t)(yv & 0xffffu)) + (int64_t)(xh * ((int32_t)yv >> 16));
            }
        }
        __syncthreads();
    }
}

// Each candidate of a block against the parent's fixed columns; the largest score per candidate.
__global__ void __launch_bounds__(kTileT) fixed_kernel(const GScoredArgs a, const GTile* __restrict__ tiles) {
    const GTile tl = tiles[blockIdx.x];
    __shared__ int32_t rid[32], cid[32];
    __shared__ uint32_t rs[32][33], cs[32][33];
    const int t = threadIdx.x;
    if (t < 32) {
        const int i = tl.ib * 32 + t;
        rid[t] = i < tl.n ? a.cand_idx[tl.rows_at + i] : -1;
        const int j = tl.jb * 32 + t;
        const int64_t r0 = a.rep_ptr[tl.parent], nr = a.rep_ptr[tl.parent + 1] - r0;
        cid[t] = j >= tl.ncols ? -1 : j < nr ? a.rep_idx[r0 + j] : a.added[a.cand_ptr[tl.parent] + (j - nr)];
    }
    __syncthreads();
    int64_t acc[4];
    tile_dots(a, rid, cid, rs, cs, acc);
    const int r = t >> 3, c0 = t & 7;
    float best = -INFINITY;
    if (rid[r] >= 0) {
        const int64_t xn = a.norm2[rid[r]];
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (cid[c0 + 8 * u] >= 0) best = fmaxf(best, exact_score(acc[u], xn, a.norm2[cid[c0 + 8 * u]], a.mode));
    }
    // the row's 8 threads are lanes 8 (r % 4) .. + 7 of one warp (every lane takes part)
    for (int o = 4; o; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
    if (c0 == 0 && rid[r] >= 0 && best > -INFINITY) atomicMax(a.prevmax + tl.rows_at + tl.ib * 32 + r, ord_float(best));
}

// Each candidate of a block against every earlier one: the lower triangle, column by column.
__global__ void __launch_bounds__(kTileT) tri_kernel(const GScoredArgs a, const GTile* __restrict__ tiles) {
    const GTile tl = tiles[blockIdx.x];
    __shared__ int32_t rid[32], cid[32];
    __shared__ uint32_t rs[32][33], cs[32][33];
    const int t = threadIdx.x;
    if (t < 32) {
        const int i = tl.ib * 32 + t, j = tl.jb * 32 + t;
        rid[t] = i < tl.n ? a.cand_idx[tl.rows_at + i] : -1;
        cid[t] = j < tl.n ? a.cand_idx[tl.rows_at + j] : -1;
    }
    __syncthreads();
    int64_t acc[4];
    tile_dots(a, rid, cid, rs, cs, acc);
    const int r = t >> 3, c0 = t & 7;
    const int i = tl.ib * 32 + r;
    if (rid[r] < 0) return;
    const int64_t xn = a.norm2[rid[r]];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int j = tl.jb * 32 + c0 + 8 * u;
        if (j < i && cid[c0 + 8 * u] >= 0)  // candidate i (later) against candidate j, the reference's argument order
            a.tri[tl.tri_off + tri_col(j, tl.n) + (i - j - 1)] =
                exact_score(acc[u], xn, a.norm2[cid[c0 + 8 * u]], a.mode);
    }
}

struct GScanArgs {
    const int64_t* cand_ptr;
    const int32_t* cand_idx;
    const uint32_t* prevmax;
    const float* tri;
    const int32_t* parents;   // [active] parents with candidates in this block
    const int64_t* tri_off;   // [active]
    int block;                // the block index
    double threshold;
    uint8_t* selected;
    float* best_out;
    int32_t* added;
    int32_t* n_added;
};

// One CTA per parent: the block's decisions in order.  best[i] starts at max(0, fixed-column
// maximum) and is raised by the triangle column of every candidate appended before i.
__global__ void __launch_bounds__(256) scan_kernel(const GScanArgs s) {
    __shared__ float m[kGB];
    __shared__ int take_s;
    const int P = s.parents[blockIdx.x];
    const int64_t c0 = s.cand_ptr[P] + (int64_t)s.block * kGB;
    const int n = (int)min((int64_t)kGB, s.cand_ptr[P + 1] - c0);
    const float* tri = s.tri + s.tri_off[blockIdx.x];
    for (int i = threadIdx.x; i < n; i += blockDim.x) m[i] = fmaxf(0.0f, unord_float(s.prevmax[c0 + i]));
    int na = s.n_added[P];
    __syncthreads();
    for (int i = 0; i < n; ++i) {
        if (threadIdx.x == 0) {
            const float b = m[i];
            const bool take = (double)b < s.threshold;
            s.selected[c0 + i] = take ? 1 : 0;
            if (s.best_out) s.best_out[c0 + i] = b;
            if (take) s.added[s.cand_ptr[P] + na] = s.cand_idx[c0 + i];
            take_s = take;
        }
        __syncthreads();
        if (take_s) {
            ++na;
            const float* col = tri + tri_col(i, n);
            for (int k = i + 1 + threadIdx.x; k < n; k += blockDim.x) m[k] = fmaxf(m[k], col[k - i - 1]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) s.n_added[P] = na;
}

__global__ void fill_u32(uint32_t* p, int64_t n, uint32_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

int propagate_scored(hdc_context* ctx, const int16_t* d_hv, const int64_t* d_norm2, const int64_t* d_cand_ptr,
                     const int32_t* d_cand_idx, const int64_t* d_rep_ptr, const int32_t* d_rep_idx, int64_t n_parents,
                     double threshold, int mode, uint8_t* d_selected, float* d_best, int32_t* d_added,
                     cudaStream_t stream) {
    std::vector<int64_t> cp(n_parents + 1), rp(n_parents + 1);
    cudaError_t e = cudaMemcpyAsync(cp.data(), d_cand_ptr, (n_parents + 1) * 8, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(rp.data(), d_rep_ptr, (n_parents + 1) * 8, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) return cuda_fail(e, "propagate: candidate counts");
    const int64_t n_cand = cp[n_parents] - cp[0];
    if (n_cand <= 0) return HDC_OK;
    int64_t max_blocks = 0, max_tri = 0;
    for (int64_t p = 0; p < n_parents; ++p) {
        if (cp[p + 1] < cp[p] || rp[p + 1] < rp[p]) return fail(HDC_ERR_INVALID, "propagate: offsets decrease");
        max_blocks = std::max(max_blocks, (cp[p + 1] - cp[p] + kGB - 1) / kGB);
    }
    // the triangles of one block of every parent at once
    for (int64_t b = 0; b < max_blocks; ++b) {
        int64_t tot = 0;
        for (int64_t p = 0; p < n_parents; ++p) {
            const int64_t n = std::min<int64_t>(kGB, cp[p + 1] - cp[p] - b * kGB);
            if (n > 1) tot += n * (n - 1) / 2;
        }
        max_tri = std::max(max_tri, tot);
    }
    const int64_t n_slots = cp[n_parents];
    uint8_t* ws = nullptr;
    auto align = [](size_t x) { return (x + 255) & ~(size_t)255; };
    const size_t b_prev = align((size_t)n_slots * 4), b_tri = align((size_t)std::max<int64_t>(max_tri, 1) * 4),
                 b_na = align((size_t)n_parents * 4);
    if ((e = cudaMallocAsync(reinterpret_cast<void**>(&ws), b_prev + b_tri + b_na, stream)) != cudaSuccess)
        return cuda_fail(e, "propagate: workspace");
    GScoredArgs a{};
    a.hv = d_hv;
    a.norm2 = d_norm2;
    a.dim = ctx->dim;
    a.mode = mode;
    a.cand_ptr = d_cand_ptr;
    a.cand_idx = d_cand_idx;
    a.rep_ptr = d_rep_ptr;
    a.rep_idx = d_rep_idx;
    a.added = d_added;
    a.prevmax = reinterpret_cast<uint32_t*>(ws);
    a.tri = reinterpret_cast<float*>(ws + b_prev);
    int32_t* d_na = reinterpret_cast<int32_t*>(ws + b_prev + b_tri);
    a.n_added = d_na;
    fill_u32<<<(unsigned)((n_slots + 255) / 256), 256, 0, stream>>>(a.prevmax, n_slots, ord_float(-INFINITY));
    cudaMemsetAsync(d_na, 0, n_parents * 4, stream);
    std::vector<int32_t> na(n_parents, 0);
    std::vector<GTile> ft, tt;
    std::vector<int32_t> parents;
    std::vector<int64_t> toff;
    GTile* d_tiles = nullptr;
    int32_t* d_par = nullptr;
    int64_t* d_toff = nullptr;
    int st = HDC_OK;
    for (int64_t b = 0; b < max_blocks && st == HDC_OK; ++b) {
        ft.clear();
        tt.clear();
        parents.clear();
        toff.clear();
        int64_t off = 0;
        for (int64_t p = 0; p < n_parents; ++p) {
            const int64_t n64 = std::min<int64_t>(kGB, cp[p + 1] - cp[p] - b * kGB);
            if (n64 <= 0) continue;
            const int n = (int)n64;
            const int64_t at = cp[p] + b * kGB;
            const int ncols = (int)(rp[p + 1] - rp[p]) + na[p];
            const int nt = (n + 31) / 32;
            for (int ib = 0; ib < nt; ++ib) {
                for (int jb = 0; jb * 32 < ncols; ++jb) ft.push_back(GTile{at, 0, n, ib, jb, (int32_t)p, ncols});
                for (int jb = 0; jb <= ib && n > 1; ++jb) tt.push_back(GTile{at, off, n, ib, jb, (int32_t)p, 0});
            }
            parents.push_back((int32_t)p);
            toff.push_back(off);
            off += n > 1 ? n64 * (n64 - 1) / 2 : 0;
        }
        const size_t bytes = (ft.size() + tt.size()) * sizeof(GTile) + parents.size() * 4 + toff.size() * 8 + 64;
        uint8_t* tb = nullptr;
        if ((e = cudaMallocAsync(reinterpret_cast<void**>(&tb), bytes, stream)) != cudaSuccess) {
            st = cuda_fail(e, "propagate: tile list");
            break;
        }
        d_tiles = reinterpret_cast<GTile*>(tb);
        d_toff = reinterpret_cast<int64_t*>(tb + (ft.size() + tt.size()) * sizeof(GTile));
        d_par = reinterpret_cast<int32_t*>(d_toff + toff.size());
        if (!ft.empty()) cudaMemcpyAsync(d_tiles, ft.data(), ft.size() * sizeof(GTile), cudaMemcpyHostToDevice, stream);
        if (!tt.empty())
            cudaMemcpyAsync(d_tiles + ft.size(), tt.data(), tt.size() * sizeof(GTile), cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_toff, toff.data(), toff.size() * 8, cudaMemcpyHostToDevice, stream);
        cudaMemcpyAsync(d_par, parents.data(), parents.size() * 4, cudaMemcpyHostToDevice, stream);
        if (!ft.empty()) fixed_kernel<<<(unsigned)ft.size(), kTileT, 0, stream>>>(a, d_tiles);
        if (!tt.empty()) tri_kernel<<<(unsigned)tt.size(), kTileT, 0, stream>>>(a, d_tiles + ft.size());
        GScanArgs sa{d_cand_ptr, d_cand_idx, a.prevmax, a.tri, d_par, d_toff, (int)b, threshold,
                     d_selected, d_best, d_added, d_na};
        scan_kernel<<<(unsigned)parents.size(), 256, 0, stream>>>(sa);
        if ((e = cudaGetLastError()) != cudaSuccess) st = cuda_fail(e, "propagate: launch");
        // the host copies of the tile lists must outlive their copies
        if (st == HDC_OK && (e = cudaStreamSynchronize(stream)) != cudaSuccess) st = cuda_fail(e, "propagate: block");
        if (st == HDC_OK && b + 1 < max_blocks) {  // the next block's fixed columns include these appends
            e = cudaMemcpyAsync(na.data(), d_na, n_parents * 4, cudaMemcpyDeviceToHost, stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
            if (e != cudaSuccess) st = cuda_fail(e, "propagate: appended counts");
        }
        cudaFreeAsync(tb, stream);
    }
    cudaFreeAsync(ws, stream);
    return st;
}

}  // namespace

int launch_propagate_greedy(hdc_context* ctx, const int16_t* d_hv, const int64_t* d_norm2,
                            const int64_t* d_cand_ptr, const int32_t* d_cand_idx, const int64_t* d_rep_ptr,
                            const int32_t* d_rep_idx, int64_t n_parents, double threshold, int mode,
                            uint8_t* d_selected, float* d_best, int32_t* d_scratch, cudaStream_t stream) {
    if (n_parents == 0) return HDC_OK;
    if (n_parents > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "propagate: too many parents");
    GreedyArgs a{d_hv, d_norm2, ctx->dim, d_cand_ptr, d_cand_idx, d_rep_ptr, d_rep_idx, threshold, mode,
                 d_selected, d_best, d_scratch};
    if (ctx->dim % 8 == 0 && (reinterpret_cast<uintptr_t>(d_hv) & 15) != 0)
        return fail(HDC_ERR_INVALID, "propagate: hypervectors not 16-byte aligned");
    if (ctx->dim % 8 == 0 && ctx->greedy_form != 0)
        return propagate_scored(ctx, d_hv, d_norm2, d_cand_ptr, d_cand_idx, d_rep_ptr, d_rep_idx, n_parents, threshold,
                                mode, d_selected, d_best, d_scratch, stream);
    greedy_kernel<<<(unsigned)n_parents, kThreadsG, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "propagate: launch");
}

}  // namespace hdc
