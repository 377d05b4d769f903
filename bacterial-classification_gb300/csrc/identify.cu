// Windowed reference similarity and the identify descent over it.
//
// HVCache::similarity (src/encoder.cpp:198-215) scores a query against a
// reference sequence as the best NORM cosine over the reference's windows
// x = 0, step, 2*step, ... while x + L < len (strict), starting from -1 and
// keeping the first window that beats the running best; a reference no longer
// than one window (len <= L) is scored as one whole-sequence hypervector.
// Every "similarity row" below is one such window (or whole sequence), an
// int16 hypervector of compute semantics (src/encoder.cpp:106-132).
//
// identify (targets/identify.cpp:89-202) scores a taxonomy node for a read as
// max(-1, similarity over every sequence of the node) (:138-159), so with the
// node's rows in CSR (node -> rows of all its sequences) a node's score is
// max(-1, max over its rows).  The level loop is the one of the prototype
// descent in beam.cu: level 0 scores the get_order("p__") nodes, each beam
// entry expands to its children (a node without children to itself, :28-33),
// candidates are ranked by score with ties to the lower node index (the
// reference's std::sort leaves tie order unspecified), the read stops with the
// best path when the best score is below the threshold (:174-189), and
// otherwise keeps the entries scoring >= threshold, at most `beam`
// (:191-199).
//
// One CTA per read: the read's int16 hypervector is staged in shared memory
// once, and the CTA's warps split each candidate node's rows (coalesced
// 16-byte loads of a row per warp step); dots are exact int64.
#include "hdc_internal.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kMaxBeam = 8;
constexpr int kMaxLevels = 8;
constexpr int kIdWarps = 8;
constexpr int kSimWarps = 8;

// exact dot of an int16 row (global) with an int16 vector (shared or global),
// one warp; dim % 8 == 0 and both 16-byte aligned.  NARROW: every partial sum
// fits int32, so the products are accumulated in int32 (two multiply-adds a
// word instead of 64-bit additions).
template <bool NARROW>
__device__ __forceinline__ int64_t warp_dot_i16_t(const int16_t* __restrict__ q, const int16_t* __restrict__ v,
                                                  int dim) {
    const int lane = threadIdx.x & 31;
    const uint4* q4 = reinterpret_cast<const uint4*>(q);
    const uint4* v4 = reinterpret_cast<const uint4*>(v);
    int64_t acc = 0;
    int32_t acc32 = 0;
    for (int i = lane; i < dim / 8; i += 32) {
        const uint4 x = q4[i], y = __ldg(v4 + i);
        const uint32_t xs[4] = {x.x, x.y, x.z, x.w}, ys[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int32_t xl = (int32_t)(xs[u] << 16) >> 16, xh = (int32_t)xs[u] >> 16;
            const int32_t yl = (int32_t)(ys[u] << 16) >> 16, yh = (int32_t)ys[u] >> 16;
            if (NARROW) {
                acc32 += xl * yl + xh * yh;
            } else {
                acc += (int64_t)(xl * yl) + (int64_t)(xh * yh);  // each product fits int32, their sum may not
            }
        }
    }
    if (NARROW) acc = acc32;
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// Cauchy-Schwarz bounds every partial sum of a dot (any subset of its products) by
// sqrt(|q|^2 |r|^2): below 2^62 for the product of the squared norms, int32 never overflows.
__device__ __forceinline__ bool dot_fits_i32(int64_t nq, int64_t nr) {
    return nq <= 0 || nr <= 0 || nr < ((int64_t)1 << 62) / nq;
}

__device__ __forceinline__ int64_t warp_dot_i16(const int16_t* __restrict__ q, const int16_t* __restrict__ v, int dim,
                                                int64_t nq, int64_t nr) {
    return dot_fits_i32(nq, nr) ? warp_dot_i16_t<true>(q, v, dim) : warp_dot_i16_t<false>(q, v, dim);
}

struct Entry {
    uint64_t key;  // make_key(score, node): larger ranks first
    int32_t node;
    int32_t parent_slot;
};

struct IdentifyArgs {
    const int16_t* q;         // [nq][dim] whole-read hypervectors
    const int64_t* qn;        // [nq]
    const int16_t* rows;      // [n_rows][dim] similarity rows
    const int64_t* rn;        // [n_rows]
    const int64_t* node_rows; // [n_nodes+1] CSR: node -> its rows
    const int64_t* child_ptr;
    const int32_t* child_idx;
    const int32_t* roots;
    int n_roots;
    int dim, levels, beam, mode;
    double threshold;
    int32_t* path;            // [nq][levels]
    float* path_score;        // [nq][levels]
    int32_t* depth;           // [nq]
    int32_t* stop_level;      // [nq] level of an early stop, -1 when all levels ran (may be null)
};

__global__ void __launch_bounds__(32 * kIdWarps) identify_kernel(const IdentifyArgs a) {
    extern __shared__ __align__(16) int16_t qs[];
    __shared__ int32_t paths[kMaxBeam][kMaxLevels];
    __shared__ float scores[kMaxBeam][kMaxLevels];
    __shared__ Entry top[kMaxBeam];
    __shared__ float wbest[2][kIdWarps];
    __shared__ int n_beam_s, done_s;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t r = blockIdx.x;
    {
        const uint4* src = reinterpret_cast<const uint4*>(a.q + r * a.dim);
        uint4* dst = reinterpret_cast<uint4*>(qs);
        for (int i = threadIdx.x; i < a.dim / 8; i += blockDim.x) dst[i] = src[i];
    }
    const int64_t qn = a.qn[r];
    // thread 0 owns the ranking state; the others follow the beam through shared memory
    int n_top = 0;
    int out_depth = 0, stop_at = -1;
    int32_t out_path[kMaxLevels];
    float out_score[kMaxLevels];
    if (threadIdx.x == 0) {
        n_beam_s = 0;
        done_s = 0;
    }
    __syncthreads();
    int parity = 0;
    for (int L = 0; L < a.levels; ++L) {
        n_top = 0;
        const int n_src = L == 0 ? 1 : n_beam_s;
        for (int b = 0; b < n_src; ++b) {
            int64_t c0, c1;
            const int32_t* list;
            int32_t self = -1;
            if (L == 0) {
                list = a.roots;
                c0 = 0;
                c1 = a.n_roots;
            } else {
                const int32_t node = paths[b][L - 1];
                c0 = a.child_ptr[node];
                c1 = a.child_ptr[node + 1];
                list = a.child_idx;
                if (c0 == c1) self = node;
            }
            const int64_t cnt = self >= 0 ? 1 : c1 - c0;
            for (int64_t c = 0; c < cnt; ++c) {
                const int32_t node = self >= 0 ? self : list[c0 + c];
                const int64_t r0 = a.node_rows[node], r1 = a.node_rows[node + 1];
                float best = -1.0f;  // identify starts every candidate at -1 (:127)
                for (int64_t j = r0 + warp; j < r1; j += kIdWarps) {
                    const int64_t rn = a.rn[j];
                    const int64_t dot = warp_dot_i16(qs, a.rows + j * a.dim, a.dim, qn, rn);
                    best = fmaxf(best, exact_score(dot, qn, rn, a.mode));
                }
                if (lane == 0) wbest[parity][warp] = best;
                __syncthreads();
                if (threadIdx.x == 0) {
                    float s = -1.0f;
                    for (int w = 0; w < kIdWarps; ++w) s = fmaxf(s, wbest[parity][w]);
                    const uint64_t key = make_key(s, (uint32_t)node);
                    if (n_top < a.beam || key > top[n_top - 1].key) {
                        int pos = n_top < a.beam ? n_top++ : a.beam - 1;
                        while (pos > 0 && top[pos - 1].key < key) {
                            top[pos] = top[pos - 1];
                            --pos;
                        }
                        top[pos] = Entry{key, node, b};
                    }
                }
                parity ^= 1;  // the next candidate writes the other buffer: one barrier per candidate
            }
        }
        if (threadIdx.x == 0) {
            int32_t np[kMaxBeam][kMaxLevels];
            float ns[kMaxBeam][kMaxLevels];
            for (int t = 0; t < n_top; ++t) {
                for (int l = 0; l < L; ++l) {
                    np[t][l] = paths[top[t].parent_slot][l];
                    ns[t][l] = scores[top[t].parent_slot][l];
                }
                np[t][L] = top[t].node;
                ns[t][L] = key_score(top[t].key);
            }
            const bool stop = n_top == 0 || (double)key_score(top[0].key) < a.threshold;
            if (stop) {
                out_depth = n_top ? L + 1 : L;
                stop_at = L;
                for (int l = 0; l < out_depth; ++l) {
                    out_path[l] = n_top ? np[0][l] : paths[0][l];
                    out_score[l] = n_top ? ns[0][l] : scores[0][l];
                }
                done_s = 1;
            } else {
                int keep = 0;
                while (keep < n_top && keep < a.beam && (double)key_score(top[keep].key) >= a.threshold) ++keep;
                n_beam_s = keep;
                for (int t = 0; t < keep; ++t)
                    for (int l = 0; l <= L; ++l) {
                        paths[t][l] = np[t][l];
                        scores[t][l] = ns[t][l];
                    }
                if (L == a.levels - 1) {
                    out_depth = a.levels;
                    for (int l = 0; l < a.levels; ++l) {
                        out_path[l] = paths[0][l];
                        out_score[l] = scores[0][l];
                    }
                }
            }
        }
        __syncthreads();
        if (done_s) break;
    }
    if (threadIdx.x == 0) {
        a.depth[r] = out_depth;
        if (a.stop_level) a.stop_level[r] = stop_at;
        for (int l = 0; l < a.levels; ++l) {
            a.path[r * a.levels + l] = l < out_depth ? out_path[l] : -1;
            a.path_score[r * a.levels + l] = l < out_depth ? out_score[l] : 0.0f;
        }
    }
}

struct SimilarityArgs {
    const int16_t* q;
    const int64_t* qn;
    const int16_t* rows;
    const int64_t* rn;
    const int64_t* ref_rows;  // [n_refs+1] CSR: reference sequence -> its rows, in window order
    const uint8_t* ref_whole; // [n_refs] 1: one whole-sequence row, scored as is (may be null: none)
    const int32_t* pair_q;
    const int32_t* pair_ref;
    int64_t n_pairs;
    int dim, mode;
    float* score;             // [n_pairs]
    int32_t* window;          // [n_pairs] first best row within the reference, -1 if none beat -1
};

// one warp per (query, reference) pair, the reference's windows in order
__global__ void __launch_bounds__(32 * kSimWarps) similarity_kernel(const SimilarityArgs a) {
    const int64_t p = (int64_t)blockIdx.x * kSimWarps + (threadIdx.x >> 5);
    if (p >= a.n_pairs) return;
    const int32_t qi = a.pair_q[p], ri = a.pair_ref[p];
    const int16_t* q = a.q + (int64_t)qi * a.dim;
    const int64_t qn = a.qn[qi];
    const int64_t r0 = a.ref_rows[ri];
    int64_t r1 = a.ref_rows[ri + 1];
    float best = -1.0f;
    int32_t win = -1;
    if (a.ref_whole && a.ref_whole[ri] && r1 > r0) {
        // len <= L: the cosine of the two whole-sequence vectors, unclamped (:200-203)
        best = exact_score(warp_dot_i16(q, a.rows + r0 * a.dim, a.dim, qn, a.rn[r0]), qn, a.rn[r0], a.mode);
        win = 0;
        r1 = r0;
    }
    for (int64_t j = r0; j < r1; ++j) {
        const int64_t rn = a.rn[j];
        const int64_t dot = warp_dot_i16(q, a.rows + j * a.dim, a.dim, qn, rn);
        const float s = exact_score(dot, qn, rn, a.mode);
        if (s > best) {  // strict: the first window reaching the maximum wins (:208-212)
            best = s;
            win = (int32_t)(j - r0);
        }
    }
    if ((threadIdx.x & 31) == 0) {
        a.score[p] = best;
        a.window[p] = win;
    }
}

bool rows_ok(const hdc_context* ctx, const void* q, const void* rows) {
    return ctx->dim % 8 == 0 && !(reinterpret_cast<uintptr_t>(q) & 15) && !(reinterpret_cast<uintptr_t>(rows) & 15);
}

}  // namespace

int launch_identify(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, int64_t nq, const int16_t* d_rows,
                    const int64_t* d_rn, const int64_t* d_node_rows, const int64_t* d_child_ptr,
                    const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int levels, int beam,
                    double threshold, int mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                    int32_t* d_stop_level, cudaStream_t stream) {
    if (nq == 0) return HDC_OK;
    if (nq > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "identify: too many reads for one launch");
    if (levels < 1 || levels > kMaxLevels) return fail(HDC_ERR_INVALID, "identify: levels must be in 1..8");
    if (beam < 1 || beam > kMaxBeam) return fail(HDC_ERR_INVALID, "identify: beam width must be in 1..8");
    if (n_roots < 0) return fail(HDC_ERR_INVALID, "identify: negative root count");
    if (!rows_ok(ctx, d_q, d_rows))
        return fail(HDC_ERR_INVALID, "identify: dim must be a multiple of 8 and rows 16-byte aligned");
    const size_t smem = (size_t)ctx->dim * sizeof(int16_t);
    if (smem > 200 * 1024) return fail(HDC_ERR_INVALID, "identify: dim too large for a shared-memory query");
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(identify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_fail(e, "identify: shared memory attribute");
    }
    IdentifyArgs a{d_q, d_qn, d_rows, d_rn, d_node_rows, d_child_ptr, d_child_idx, d_roots, n_roots, ctx->dim,
                   levels, beam, mode, threshold, d_path, d_path_score, d_depth, d_stop_level};
    identify_kernel<<<(unsigned)nq, 32 * kIdWarps, smem, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "identify: launch");
}

int launch_similarity(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, const int16_t* d_rows,
                      const int64_t* d_rn, const int64_t* d_ref_rows, const uint8_t* d_ref_whole,
                      const int32_t* d_pair_q,
                      const int32_t* d_pair_ref, int64_t n_pairs, int mode, float* d_score, int32_t* d_window,
                      cudaStream_t stream) {
    if (n_pairs == 0) return HDC_OK;
    if (!rows_ok(ctx, d_q, d_rows))
        return fail(HDC_ERR_INVALID, "similarity: dim must be a multiple of 8 and rows 16-byte aligned");
    const int64_t blocks = (n_pairs + kSimWarps - 1) / kSimWarps;
    if (blocks > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "similarity: too many pairs for one launch");
    SimilarityArgs a{d_q, d_qn, d_rows, d_rn, d_ref_rows, d_ref_whole, d_pair_q, d_pair_ref, n_pairs, ctx->dim, mode, d_score,
                     d_window};
    similarity_kernel<<<(unsigned)blocks, 32 * kSimWarps, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "similarity: launch");
}

}  // namespace hdc
