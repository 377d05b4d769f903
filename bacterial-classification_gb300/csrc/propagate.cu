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
#include <algorithm>

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
    greedy_kernel<<<(unsigned)n_parents, kThreadsG, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "propagate: launch");
}

}  // namespace hdc
