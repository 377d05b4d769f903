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
// streams each candidate prototype with coalesced 16-byte loads; dots are
// exact int64 (the prototypes of internal nodes exceed int16).
#include "hdc_internal.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kMaxBeam = 8;
constexpr int kMaxLevels = 8;
constexpr int kBeamWarps = 4;

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

__device__ __forceinline__ int64_t warp_dot_i8_i32(const int8_t* __restrict__ q, const int32_t* __restrict__ v, int dim) {
    const int lane = threadIdx.x & 31;
    int64_t acc = 0;
    // 4 dims per lane per step: char4 of the query, int4 of the prototype
    for (int d = 4 * lane; d + 3 < dim; d += 128) {
        const char4 s = *reinterpret_cast<const char4*>(q + d);
        const int4 x = __ldg(reinterpret_cast<const int4*>(v + d));
        acc += (int64_t)s.x * x.x + (int64_t)s.y * x.y + (int64_t)s.z * x.z + (int64_t)s.w * x.w;
    }
    for (int d = (dim & ~3) + lane; d < dim; d += 32) acc += (int64_t)q[d] * v[d];
    for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    return acc;
}

struct Entry {
    uint64_t key;  // make_key(score, node): larger ranks first
    int32_t node;
    int32_t parent_slot;
};

__global__ void __launch_bounds__(32 * kBeamWarps) beam_kernel(const BeamArgs a) {
    const int64_t r = (int64_t)blockIdx.x * kBeamWarps + (threadIdx.x >> 5);
    if (r >= a.nq) return;
    const int8_t* q = a.q + r * a.dim;
    const int64_t qn = a.qn[r];
    // beam paths, one row per slot
    int32_t paths[kMaxBeam][kMaxLevels];
    float scores[kMaxBeam][kMaxLevels];
    int n_beam = 0;
    int out_depth = 0;
    int32_t out_path[kMaxLevels];
    float out_score[kMaxLevels];
    for (int L = 0; L < a.levels; ++L) {
        Entry top[kMaxBeam];
        int n_top = 0;
        const int n_src = L == 0 ? 1 : n_beam;
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
                if (c0 == c1) self = node;  // a node without children scores itself again
            }
            const int64_t cnt = self >= 0 ? 1 : c1 - c0;
            for (int64_t c = 0; c < cnt; ++c) {
                const int32_t node = self >= 0 ? self : list[c0 + c];
                const int64_t dot = warp_dot_i8_i32(q, a.proto + (int64_t)node * a.dim, a.dim);
                const float s = exact_score(dot, qn, a.pn[node], a.mode);
                const uint64_t key = make_key(s, (uint32_t)node);
                // keep the best `beam` candidates (uniform across the warp)
                if (n_top < a.beam || key > top[n_top - 1].key) {
                    int pos = n_top < a.beam ? n_top++ : a.beam - 1;
                    while (pos > 0 && top[pos - 1].key < key) {
                        top[pos] = top[pos - 1];
                        --pos;
                    }
                    top[pos] = Entry{key, node, b};
                }
            }
        }
        // new beam rows from their parents' rows
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
        int keep = 0;
        while (keep < n_top && keep < a.beam && (double)key_score(top[keep].key) >= a.threshold) ++keep;
        if (stop) {
            out_depth = n_top ? L + 1 : L;
            for (int l = 0; l < out_depth; ++l) {
                out_path[l] = n_top ? np[0][l] : paths[0][l];
                out_score[l] = n_top ? ns[0][l] : scores[0][l];
            }
            break;
        }
        n_beam = keep;
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
    if ((threadIdx.x & 31) == 0) {
        a.depth[r] = out_depth;
        for (int l = 0; l < a.levels; ++l) {
            a.path[r * a.levels + l] = l < out_depth ? out_path[l] : -1;
            a.path_score[r * a.levels + l] = l < out_depth ? out_score[l] : 0.0f;
        }
    }
}

}  // namespace

int launch_beam_search(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qn, int64_t nq, const int32_t* d_proto,
                       const int64_t* d_pn, const int64_t* d_child_ptr, const int32_t* d_child_idx,
                       const int32_t* d_roots, int n_roots, int levels, int beam, double threshold, int mode,
                       int32_t* d_path, float* d_path_score, int32_t* d_depth, cudaStream_t stream) {
    if (nq == 0) return HDC_OK;
    if (levels < 1 || levels > kMaxLevels) return fail(HDC_ERR_INVALID, "beam: levels must be in 1..8");
    if (beam < 1 || beam > kMaxBeam) return fail(HDC_ERR_INVALID, "beam: beam width must be in 1..8");
    if (n_roots < 1) return fail(HDC_ERR_INVALID, "beam: no level-0 candidates");
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
