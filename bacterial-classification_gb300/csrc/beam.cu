// Hierarchical descent (config 5): beam search of reads down a taxonomy
// whose nodes carry prototype hypervectors (leaves: their encoding; internal
// nodes: the bundle of their children, hdc_bundle).
//
// Semantics follow the level loop of targets/identify.cpp:89-202 with one
// prototype per node in place of the node's representative sequences:
//   level 0 candidates are the children of the root (the reference's
//   get_order("p__")); at every level each beam entry expands to its
//   children (a node without children expands to itself,
//   targets/identify.cpp:28-33), every candidate is scored with the cosine
//   score of src/HV.cpp:219-242 against the read, candidates are ranked by
//   score (ties to the lower node index, where the reference's std::sort
//   leaves the order unspecified), and when the best score is below the
//   threshold the read stops with that best path (targets/identify.cpp:
//   174-189); otherwise the entries with score >= threshold, at most `beam`
//   of them, go on (:191-199).  After `levels` levels the best entry's path is returned.
//
// One warp per read: the read's +1/-1 hypervector stays in L1 while the warp
// streams each candidate prototype with coalesced 16-byte loads, several in
// flight per lane; dots are exact int64 (the prototypes of internal nodes
// exceed int16).  The beam bookkeeping lives in shared memory, written by
// lane 0, so the registers go to loads in flight.
#include "hdc_internal.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kMaxBeam = 8;
constexpr int kMaxLevels = 8;
constexpr int kBeamWarps = 8;
constexpr int kDotUnroll = 4;  // 16-byte prototype loads in flight per lane

struct BeamArgs {
    const int8_t* q;        // [nq][dim] +1/-1
    const int64_t* qn;      // [nq]
    int64_t nq;
    const int32_t* proto;   // [n_nodes][dim]
    const int64_t* pn;      // [n_nodes]
    const int64_t* child_ptr;
    const int32_t* child_idx;
    const int32_t* roots;   // level-0 candidates
    int n_roots;
    int dim, levels, beam, mode;
    double threshold;
    int32_t* path;          // [nq][levels]
    float* path_score;      // [nq][levels]
    int32_t* depth;         // [nq] levels on the returned path
};

// exact dot of a +1/-1 int8 read with an int32 prototype row, one warp:
// lane l covers dims 4l..4l+3 of every 128-dim block; kDotUnroll blocks are
// loaded before any is used, so each lane keeps that many 16-byte loads in
// flight (the kernel is bound by gathering rows, not by arithmetic)
__device__ __forceinline__ int64_t warp_dot_i8_i32(const int8_t* __restrict__ q, const int32_t* __restrict__ v, int dim) {
    const int lane = threadIdx.x & 31;
    int64_t acc = 0;
    const int full = dim / (128 * kDotUnroll);
    for (int blk = 0; blk < full; ++blk) {
        const int d0 = blk * 128 * kDotUnroll + 4 * lane;
        int4 x[kDotUnroll];
        char4 s[kDotUnroll];
#pragma unroll
        for (int u = 0; u < kDotUnroll; ++u) {
            x[u] = __ldg(reinterpret_cast<const int4*>(v + d0 + 128 * u));
            s[u] = *reinterpret_cast<const char4*>(q + d0 + 128 * u);
        }
#pragma unroll
        for (int u = 0; u < kDotUnroll; ++u)
            acc += (int64_t)s[u].x * x[u].x + (int64_t)s[u].y * x[u].y + (int64_t)s[u].z * x[u].z +
                   (int64_t)s[u].w * x[u].w;
    }
    for (int d = full * 128 * kDotUnroll + 4 * lane; d + 3 < dim; d += 128) {
        const char4 s = *reinterpret_cast<const char4*>(q + d);
        const int4 x = __ldg(reinterpret_cast<const int4*>(v + d));
        acc += (int64_t)s.x * x.x + (int64_t)s.y * x.y + (int64_t)s.z * x.z + (int64_t)s.w * x.w;
    }
    for (int d = (dim & ~3) + lane; d < dim; d += 32) acc += (int64_t)q[d] * v[d];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

// one warp's descent state, in shared memory (lane 0 writes, the warp reads)
struct WarpBeam {
    int32_t paths[kMaxBeam][kMaxLevels];
    float scores[kMaxBeam][kMaxLevels];
    int32_t np[kMaxBeam][kMaxLevels];
    float ns[kMaxBeam][kMaxLevels];
    uint64_t key[kMaxBeam];   // make_key(score, node): larger ranks first
    int32_t node[kMaxBeam];
    int32_t slot[kMaxBeam];   // beam row the candidate expanded
    int n_beam, n_top, done, out_depth;
};

__global__ void __launch_bounds__(32 * kBeamWarps) beam_kernel(const BeamArgs a) {
    __shared__ WarpBeam st_all[kBeamWarps];
    const int lane = threadIdx.x & 31;
    WarpBeam& st = st_all[threadIdx.x >> 5];
    const int64_t r = (int64_t)blockIdx.x * kBeamWarps + (threadIdx.x >> 5);
    if (r >= a.nq) return;  // whole warps leave; no block-wide barrier below
    const int8_t* q = a.q + r * a.dim;
    const int64_t qn = a.qn[r];
    if (lane == 0) {
        st.n_beam = 0;
        st.done = 0;
        st.out_depth = 0;
    }
    __syncwarp();
    for (int L = 0; L < a.levels && !st.done; ++L) {
        if (lane == 0) st.n_top = 0;
        const int n_src = L == 0 ? 1 : st.n_beam;
        for (int b = 0; b < n_src; ++b) {
            int64_t c0, c1;
            const int32_t* list;
            int32_t self = -1;
            if (L == 0) {
                list = a.roots;
                c0 = 0;
                c1 = a.n_roots;
            } else {
                const int32_t node = st.paths[b][L - 1];
                c0 = a.child_ptr[node];
                c1 = a.child_ptr[node + 1];
                list = a.child_idx;
                if (c0 == c1) self = node;  // a node without children scores itself again
            }
            const int64_t cnt = self >= 0 ? 1 : c1 - c0;
            for (int64_t c = 0; c < cnt; ++c) {
                const int32_t node = self >= 0 ? self : list[c0 + c];
                const int64_t dot = warp_dot_i8_i32(q, a.proto + (int64_t)node * a.dim, a.dim);
                if (lane == 0) {  // keep the best `beam` candidates
                    const uint64_t key = make_key(exact_score(dot, qn, a.pn[node], a.mode), (uint32_t)node);
                    int n = st.n_top;
                    if (n < a.beam || key > st.key[n - 1]) {
                        int pos = n < a.beam ? n++ : a.beam - 1;
                        while (pos > 0 && st.key[pos - 1] < key) {
                            st.key[pos] = st.key[pos - 1];
                            st.node[pos] = st.node[pos - 1];
                            st.slot[pos] = st.slot[pos - 1];
                            --pos;
                        }
                        st.key[pos] = key;
                        st.node[pos] = node;
                        st.slot[pos] = b;
                        st.n_top = n;
                    }
                }
            }
        }
        if (lane == 0) {
            const int n_top = st.n_top;
            for (int t = 0; t < n_top; ++t) {  // new beam rows from their parents' rows
                for (int l = 0; l < L; ++l) {
                    st.np[t][l] = st.paths[st.slot[t]][l];
                    st.ns[t][l] = st.scores[st.slot[t]][l];
                }
                st.np[t][L] = st.node[t];
                st.ns[t][L] = key_score(st.key[t]);
            }
            const bool stop = n_top == 0 || (double)key_score(st.key[0]) < a.threshold;
            if (stop) {
                st.out_depth = n_top ? L + 1 : L;
                if (n_top)
                    for (int l = 0; l <= L; ++l) {
                        st.paths[0][l] = st.np[0][l];
                        st.scores[0][l] = st.ns[0][l];
                    }
                st.done = 1;
            } else {
                int keep = 0;
                while (keep < n_top && keep < a.beam && (double)key_score(st.key[keep]) >= a.threshold) ++keep;
                st.n_beam = keep;
                for (int t = 0; t < keep; ++t)
                    for (int l = 0; l <= L; ++l) {
                        st.paths[t][l] = st.np[t][l];
                        st.scores[t][l] = st.ns[t][l];
                    }
                if (L == a.levels - 1) st.out_depth = a.levels;
            }
        }
        __syncwarp();
    }
    // the returned path is beam row 0
    for (int l = lane; l < a.levels; l += 32) {
        const bool in = l < st.out_depth;
        a.path[r * a.levels + l] = in ? st.paths[0][l] : -1;
        a.path_score[r * a.levels + l] = in ? st.scores[0][l] : 0.0f;
    }
    if (lane == 0) a.depth[r] = st.out_depth;
}

}  // namespace

int launch_beam_search(hdc_context* ctx, const int8_t* d_q, const uint32_t* d_qbits, const int64_t* d_qn, int64_t nq,
                       const int32_t* d_proto,
                       int64_t n32, const int16_t* d_proto16, const int64_t* d_pn, int64_t n_nodes,
                       const int64_t* d_child_ptr, const int32_t* d_child_idx, const int32_t* d_roots, int n_roots,
                       int max_children, int levels, int beam, double threshold, int mode, int32_t* d_path,
                       float* d_path_score, int32_t* d_depth, cudaStream_t stream) {
    if (nq == 0) return HDC_OK;
    if (levels < 1 || levels > kMaxLevels) return fail(HDC_ERR_INVALID, "beam: levels must be in 1..8");
    if (beam < 1 || beam > kMaxBeam) return fail(HDC_ERR_INVALID, "beam: beam width must be in 1..8");
    if (n_roots < 1) return fail(HDC_ERR_INVALID, "beam: no level-0 candidates");
    const bool grouped_ok = ctx->dim % 1024 == 0 && ctx->dim <= 16384 && (reinterpret_cast<uintptr_t>(d_proto) & 15) == 0 &&
                            (reinterpret_cast<uintptr_t>(d_proto16) & 15) == 0 && (reinterpret_cast<uintptr_t>(d_q) & 15) == 0 &&
                            (reinterpret_cast<uintptr_t>(d_qbits) & 15) == 0;
    if (ctx->beam_grouped != 0 && grouped_ok)
        return launch_beam_grouped(ctx, d_q, d_qbits, d_qn, nq, d_proto, n32, d_proto16, d_pn, n_nodes, d_child_ptr,
                                   d_child_idx, d_roots, n_roots, max_children, levels, beam, threshold, mode, d_path,
                                   d_path_score, d_depth, stream);
    if (n32 < n_nodes || d_qbits)
        return fail(HDC_ERR_INVALID, "beam: int16 rows and bit reads need the grouped descent (dim % 1024 == 0, "
                                     "dim <= 16384, 16-byte aligned rows and reads, HDC_BEAM_GROUPED != 0)");
    if (ctx->dim % 4 != 0 || (reinterpret_cast<uintptr_t>(d_proto) & 15) || (reinterpret_cast<uintptr_t>(d_q) & 3))
        return fail(HDC_ERR_INVALID, "beam: dim must be a multiple of 4 and rows aligned");
    BeamArgs a{d_q, d_qn, nq, d_proto, d_pn, d_child_ptr, d_child_idx, d_roots, n_roots, ctx->dim, levels, beam,
               mode, threshold, d_path, d_path_score, d_depth};
    const int64_t blocks = (nq + kBeamWarps - 1) / kBeamWarps;
    beam_kernel<<<(unsigned)blocks, 32 * kBeamWarps, 0, stream>>>(a);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "beam: launch");
}

}  // namespace hdc
