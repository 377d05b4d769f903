// (b) plain form of the query x reference cosine search on CUDA cores, plus
// the norm, merge and bundling kernels.
//
// Replaces compute_inv_norms_kernel, cosine_score_matrix_kernel and the
// bitonic / k-pass top-k kernels of src/cosine.cu:35-496.  Differences that
// matter for the result:
//   * every dot product is exact (the reference accumulates int32 partials,
//     src/cosine.cu:59-83) and the float score is the reference CPU score
//     computed from the exact dot and norms in FP64 (src/HV.cpp:219-242);
//   * no [Q][R] score matrix is written: each CTA keeps a running top-k per
//     query for its share of the references and a merge kernel combines the
//     shares (the reference writes Q*R floats and re-reads them k times);
//   * ties rank the lower reference index first for every R (the reference
//     bitonic path is wrong for non-power-of-two R, src/cosine.cu:302-316).
//
// Exact integer arithmetic on the FP32 pipe: int16 values are exact in fp32;
// while every partial sum stays below 2^22 in magnitude an FFMA chain is
// exact, so the K loop accumulates fp32 for `chunk` dims (chunk * max|q| *
// max|r| < 2^22) and then folds the accumulator into an integer with the
// 1.5*2^23 magic-number trick (one FADD + one IADD).  The integer
// accumulator is int32 when max|q|*max|r|*dim < 2^31, else int64.
#include <cuda_bf16.h>

#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>

#include "hdc_internal.cuh"
#include "topk.cuh"

namespace hdc {
namespace {

constexpr int kKT = 32;        // dims per K tile
constexpr int kThreadsP = 256;  // 16 x 16 threads
constexpr int kBR = 128;        // references per CTA tile
constexpr int kMaxK = 32;       // largest top-k
// int32 form: 4 x 8 register tiles where the fp32 partials are folded at least every 256 dims
// (count-valued queries) and there are at least this many references
constexpr int64_t kPlainWideTileRefs = 16384;
constexpr int kPlainFoldTile = 64;

// ---------------------------------------------------------------- norms
__device__ __forceinline__ int64_t as_i64(int8_t x) { return x; }
__device__ __forceinline__ int64_t as_i64(int16_t x) { return x; }
__device__ __forceinline__ int64_t as_i64(int32_t x) { return x; }
__device__ __forceinline__ int64_t as_i64(__half x) { return (int64_t)__half2int_rn(x); }  // integer-valued fp16

template <typename T>
__global__ void norms_kernel(const T* __restrict__ v, int64_t n, int dim, int64_t* __restrict__ norm2,
                             int32_t* __restrict__ maxabs) {
    const int lane = threadIdx.x & 31;
    const int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= n) return;
    const T* p = v + row * dim;
    int64_t s = 0;
    int32_t m = 0;
    for (int d = lane; d < dim; d += 32) {
        const int64_t x = as_i64(p[d]);
        s += x * x;
        m = max(m, (int32_t)(x < 0 ? -x : x));
    }
    for (int o = 16; o; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    }
    if (lane == 0) {
        norm2[row] = s;
        if (maxabs) atomicMax(maxabs, m);
    }
}

// ---------------------------------------------------------------- plain top-k
struct PlainArgs {
    const int16_t* q;
    const int64_t* qn;
    int64_t nq;
    const int16_t* r;
    const int64_t* rn;
    int64_t nr;
    int dim, k, mode;
    int fold_groups;   // 4-dim groups per exact fp32 chunk (>= 1)
    int n_splits;      // reference ranges per query tile
    int64_t split_len;  // references per range (multiple of kBR)
    uint64_t* ws_key;   // [n_splits][nq][k]
    int64_t* ws_dot;    // [n_splits][nq][k]
};

__device__ __forceinline__ int32_t fold_bits(float acc) { return __float_as_int(acc + 12582912.0f); }
constexpr int32_t kMagicBits = 0x4B400000;

template <int TQ, bool WIDE, bool VEC>
// Two CTAs per SM for the int32 accumulators with 4 queries x 8 references a thread (127
// registers): more warps to hide the shared-memory loads than one CTA of 8 x 8 tiles at 248
// registers, when the fp32 partials are folded often (c2, count-valued reads against 50,000
// references: 47,850 -> 49,543 reads/s).  Otherwise the 8 x 8 tiles stay faster: with few
// references (c1, 2,000: 841,788 against 584,322 reads/s) four threads per query keep top-k
// lists whose inserts and merge weigh more than the dots, and with rare folds (c3's bipolar
// queries: 8,497 against 6,760) the larger tiles' fewer shared-memory loads per FMA win.
// The int64 form keeps one CTA (it would spill).
__global__ void __launch_bounds__(kThreadsP, (TQ == 4 && !WIDE) ? 2 : 1) plain_kernel(const PlainArgs a) {
    constexpr int BQ = TQ * 16;          // queries per CTA tile
    constexpr int QLD = BQ + 4, RLD = kBR + 4;
    using Mid = typename std::conditional<WIDE, int64_t, int32_t>::type;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* qs = reinterpret_cast<float*>(smem_raw);       // [2][kKT][QLD]
    float* rs = qs + 2 * kKT * QLD;                        // [2][kKT][RLD]
    Mid* dtile = reinterpret_cast<Mid*>(smem_raw);         // [BQ][kBR+1] after the K loop
    __shared__ float rr_s[kBR];
    __shared__ int64_t rn_s[kBR];
    // lists exchanged by the final merge (aliases the tiles, used after the loop)
    uint64_t* xkeys = reinterpret_cast<uint64_t*>(smem_raw);          // [BQ][kMaxK]
    int64_t* xdots = reinterpret_cast<int64_t*>(xkeys + BQ * kMaxK);  // [BQ][kMaxK]

    const int t = threadIdx.x, tx = t & 15, ty = t >> 4;
    const int64_t q0 = (int64_t)blockIdx.x * BQ;
    const int split = blockIdx.y;
    const int64_t rbeg = (int64_t)split * a.split_len;
    const int64_t rend = min(a.nr, rbeg + a.split_len);
    const int dim = a.dim, k = a.k;
    const int nkt = (dim + kKT - 1) / kKT;

    // scan role: query qi (local), reference half h of each tile
    const int qi = t % BQ, hh = t / BQ, nh = kThreadsP / BQ;  // nh halves/quarters
    const int64_t gq = q0 + qi;
    const int64_t my_qn = gq < a.nq ? a.qn[gq] : 0;
    const float my_rq = rsqrt_norm(my_qn);
    uint64_t keys[kMaxK];
    int64_t dots[kMaxK];
    for (int i = 0; i < k; ++i) {
        keys[i] = 0;
        dots[i] = 0;
    }
    float thr = -INFINITY;

    // staging loaders: q tile BQ x 32 dims, r tile 128 x 32 dims (int16 -> fp32)
    auto load_q = [&](int kt, int16_t (&st)[TQ * 2]) {
        // thread t covers query (t % BQ), dims [dseg*16/ (256/BQ)...]
        constexpr int per = (BQ * kKT) / kThreadsP;  // int16 per thread (= TQ*2)
        const int qq = t % BQ, seg = t / BQ;
        const int64_t gqq = q0 + qq;
        const int d0 = kt * kKT + seg * per;
        const int16_t* src = a.q + gqq * dim + d0;
        if (VEC && gqq < a.nq && d0 + per <= dim) {
#pragma unroll
            for (int u = 0; u < per / 8; ++u) *reinterpret_cast<uint4*>(&st[8 * u]) = __ldg(reinterpret_cast<const uint4*>(src) + u);
        } else {
#pragma unroll
            for (int u = 0; u < per; ++u) st[u] = (gqq < a.nq && d0 + u < dim) ? src[u] : (int16_t)0;
        }
    };
    auto load_r = [&](int64_t rb, int kt, int16_t (&st)[16]) {
        const int rr = t & 127, seg = t >> 7;
        const int64_t grr = rb + rr;
        const int d0 = kt * kKT + seg * 16;
        const int16_t* src = a.r + grr * dim + d0;
        if (VEC && grr < rend && d0 + 16 <= dim) {
            *reinterpret_cast<uint4*>(&st[0]) = __ldg(reinterpret_cast<const uint4*>(src));
            *reinterpret_cast<uint4*>(&st[8]) = __ldg(reinterpret_cast<const uint4*>(src) + 1);
        } else {
#pragma unroll
            for (int u = 0; u < 16; ++u) st[u] = (grr < rend && d0 + u < dim) ? src[u] : (int16_t)0;
        }
    };
    auto store_q = [&](int buf, const int16_t (&st)[TQ * 2]) {
        constexpr int per = (BQ * kKT) / kThreadsP;
        const int qq = t % BQ, seg = t / BQ;
        float* dst = qs + buf * kKT * QLD;
#pragma unroll
        for (int u = 0; u < per; ++u) dst[(seg * per + u) * QLD + qq] = (float)st[u];
    };
    auto store_r = [&](int buf, const int16_t (&st)[16]) {
        const int rr = t & 127, seg = t >> 7;
        float* dst = rs + buf * kKT * RLD;
#pragma unroll
        for (int u = 0; u < 16; ++u) dst[(seg * 16 + u) * RLD + rr] = (float)st[u];
    };

    for (int64_t rb = rbeg; rb < rend; rb += kBR) {
        float acc[TQ][8];
        Mid mid[TQ][8];
#pragma unroll
        for (int i = 0; i < TQ; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                acc[i][j] = 0.f;
                mid[i][j] = 0;
            }
        int nfold = 0, groups_since_fold = 0;
        if (t < kBR) {
            const int64_t g = rb + t;
            const int64_t n2 = g < rend ? a.rn[g] : 0;
            rn_s[t] = n2;
            rr_s[t] = rsqrt_norm(n2);
        }
        int16_t sq[TQ * 2], sr[16];
        load_q(0, sq);
        load_r(rb, 0, sr);
        store_q(0, sq);
        store_r(0, sr);
        __syncthreads();
        for (int kt = 0; kt < nkt; ++kt) {
            const int buf = kt & 1;
            if (kt + 1 < nkt) {
                load_q(kt + 1, sq);
                load_r(rb, kt + 1, sr);
            }
            const float* qb = qs + buf * kKT * QLD + ty * TQ;
            const float* rb0 = rs + buf * kKT * RLD + tx * 4;
#pragma unroll
            for (int g = 0; g < kKT / 4; ++g) {
#pragma unroll
                for (int dd = 0; dd < 4; ++dd) {
                    const int d = 4 * g + dd;
                    float qv[TQ], rv[8];
#pragma unroll
                    for (int u = 0; u < TQ / 4; ++u) {
                        const float4 f = *reinterpret_cast<const float4*>(qb + d * QLD + 4 * u);
                        qv[4 * u] = f.x;
                        qv[4 * u + 1] = f.y;
                        qv[4 * u + 2] = f.z;
                        qv[4 * u + 3] = f.w;
                    }
                    const float4 r0 = *reinterpret_cast<const float4*>(rb0 + d * RLD);
                    const float4 r1 = *reinterpret_cast<const float4*>(rb0 + d * RLD + 64);
                    rv[0] = r0.x; rv[1] = r0.y; rv[2] = r0.z; rv[3] = r0.w;
                    rv[4] = r1.x; rv[5] = r1.y; rv[6] = r1.z; rv[7] = r1.w;
#pragma unroll
                    for (int i = 0; i < TQ; ++i)
#pragma unroll
                        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(qv[i], rv[j], acc[i][j]);
                }
                // fold the exact fp32 partials into the integer accumulator
                // every fold_groups groups of 4 dims, and after the last tile
                if (++groups_since_fold == a.fold_groups || (kt + 1 == nkt && g == kKT / 4 - 1)) {
                    groups_since_fold = 0;
#pragma unroll
                    for (int i = 0; i < TQ; ++i)
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            if (WIDE)
                                mid[i][j] += (int64_t)(fold_bits(acc[i][j]) - kMagicBits);
                            else
                                mid[i][j] = (Mid)((uint32_t)mid[i][j] + (uint32_t)fold_bits(acc[i][j]));
                            acc[i][j] = 0.f;
                        }
                    ++nfold;
                }
            }
            if (kt + 1 < nkt) {
                store_q(buf ^ 1, sq);
                store_r(buf ^ 1, sr);
            }
            __syncthreads();
        }
        // exact dots -> shared tile [BQ][kBR+1]
#pragma unroll
        for (int i = 0; i < TQ; ++i)
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                Mid v = mid[i][j];
                if (!WIDE) v = (Mid)((uint32_t)v - (uint32_t)nfold * (uint32_t)kMagicBits);
                const int rl = (j < 4) ? (tx * 4 + j) : (64 + tx * 4 + j - 4);
                dtile[(ty * TQ + i) * (kBR + 1) + rl] = v;
            }
        __syncthreads();
        // scan: thread (qi, hh) checks references hh, hh+nh, ... of this tile
        if (gq < a.nq) {
            const Mid* drow = dtile + qi * (kBR + 1);
            for (int rl = hh; rl < kBR; rl += nh) {
                const int64_t gr = rb + rl;
                if (gr >= rend) break;
                const int64_t dot = (int64_t)drow[rl];
                const float ap = approx_score(__ll2float_rn(dot), my_rq, rr_s[rl], a.mode);
                if (ap < thr) continue;
                const float s = exact_score(dot, my_qn, rn_s[rl], a.mode);
                const uint64_t key = make_key(s, (uint32_t)gr);
                if (key <= keys[k - 1]) continue;
                list_insert(keys, dots, k, key, dot);
                if (keys[k - 1] != 0) {
                    const float sk = key_score(keys[k - 1]);
                    thr = a.mode == HDC_SCORE_DOT ? sk : sk - kFilterMargin;
                }
            }
        }
        __syncthreads();
    }

    // merge the nh partial lists of each query and write the range's result
    for (int part = 1; part < nh; ++part) {
        if (hh == part)
            for (int i = 0; i < k; ++i) {
                xkeys[qi * kMaxK + i] = keys[i];
                xdots[qi * kMaxK + i] = dots[i];
            }
        __syncthreads();
        if (hh == 0)
            for (int i = 0; i < k; ++i) {
                const uint64_t key = xkeys[qi * kMaxK + i];
                if (key <= keys[k - 1]) break;
                list_insert(keys, dots, k, key, xdots[qi * kMaxK + i]);
            }
        __syncthreads();
    }
    if (hh == 0 && gq < a.nq) {
        uint64_t* ok = a.ws_key + ((int64_t)split * a.nq + gq) * k;
        int64_t* od = a.ws_dot + ((int64_t)split * a.nq + gq) * k;
        for (int i = 0; i < k; ++i) {
            ok[i] = keys[i];
            od[i] = dots[i];
        }
    }
}

// Final merge of the per-range lists: one thread per query.
__global__ void merge_kernel(const uint64_t* __restrict__ ws_key, const int64_t* __restrict__ ws_dot, int n_splits,
                             int64_t nq, int k, const int64_t* __restrict__ qn, const int64_t* __restrict__ rn,
                             int64_t nr, float* __restrict__ out_s, int32_t* __restrict__ out_i,
                             double* __restrict__ out_c, int64_t* __restrict__ out_d) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq) return;
    uint64_t keys[kMaxK];
    int64_t dots[kMaxK];
    for (int i = 0; i < k; ++i) {
        keys[i] = ws_key[q * k + i];
        dots[i] = ws_dot[q * k + i];
    }
    for (int s = 1; s < n_splits; ++s) {
        const uint64_t* kk = ws_key + ((int64_t)s * nq + q) * k;
        const int64_t* dd = ws_dot + ((int64_t)s * nq + q) * k;
        for (int i = 0; i < k; ++i) {
            const uint64_t key = kk[i];
            if (key <= keys[k - 1]) break;
            list_insert(keys, dots, k, key, dd[i]);
        }
    }
    const int64_t nqv = qn[q];
    for (int i = 0; i < k; ++i) {
        const uint32_t idx = key_idx(keys[i]);
        // a list a search left unwritten (a bounded wait that gave up) holds stale keys: never
        // follow an index past the references
        const bool ok = keys[i] != 0 && (int64_t)idx < nr;
        out_s[q * k + i] = ok ? key_score(keys[i]) : -INFINITY;
        out_i[q * k + i] = ok ? (int32_t)idx : -1;
        if (out_c) out_c[q * k + i] = ok ? exact_cos(dots[i], nqv, rn[idx]) : 0.0;
        if (out_d) out_d[q * k + i] = ok ? dots[i] : 0;
    }
}

// ---------------------------------------------------------------- bundling
template <typename T>
__global__ void bundle_kernel(const T* __restrict__ rows, int dim, const int64_t* __restrict__ child_ptr,
                              const int32_t* __restrict__ child_idx, int64_t n_parents, int32_t* __restrict__ out) {
    const int64_t p = blockIdx.y;
    const int d = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_parents || d >= dim) return;
    int32_t s = 0;
    for (int64_t c = child_ptr[p]; c < child_ptr[p + 1]; ++c) s += (int32_t)rows[(int64_t)child_idx[c] * dim + d];
    out[p * dim + d] = s;
}

int plain_splits(const hdc_context* ctx, int64_t nq, int64_t nr, int tq) {
    const int64_t qtiles = (nq + tq * 16 - 1) / (tq * 16);
    const int64_t rtiles = std::max<int64_t>(1, (nr + kBR - 1) / kBR);
    int64_t s = std::max<int64_t>(1, (2 * (int64_t)ctx->num_sms + qtiles - 1) / qtiles);
    return (int)std::min<int64_t>(s, rtiles);
}

}  // namespace

int launch_norms(hdc_context* ctx, const void* d_hv, int elem_bytes, int64_t n, int64_t* d_norm2, int32_t* d_maxabs,
                 cudaStream_t stream) {
    if (n == 0) return HDC_OK;
    const int rows_per_block = 8;
    const int64_t grid = (n + rows_per_block - 1) / rows_per_block;
    if (grid > 0x7fffffff) return fail(HDC_ERR_INVALID, "norms: too many rows");
    if (elem_bytes == 1)
        norms_kernel<int8_t><<<(unsigned)grid, 256, 0, stream>>>(static_cast<const int8_t*>(d_hv), n, ctx->dim,
                                                                  d_norm2, d_maxabs);
    else if (elem_bytes == 2)
        norms_kernel<int16_t><<<(unsigned)grid, 256, 0, stream>>>(static_cast<const int16_t*>(d_hv), n, ctx->dim,
                                                                   d_norm2, d_maxabs);
    else if (elem_bytes == kNormsF16)
        norms_kernel<__half><<<(unsigned)grid, 256, 0, stream>>>(static_cast<const __half*>(d_hv), n, ctx->dim,
                                                                  d_norm2, d_maxabs);
    else
        norms_kernel<int32_t><<<(unsigned)grid, 256, 0, stream>>>(static_cast<const int32_t*>(d_hv), n, ctx->dim,
                                                                   d_norm2, d_maxabs);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "norms: launch");
}

size_t plain_workspace_bytes(const hdc_context* ctx, int64_t nq, int64_t nr, int k) {
    k = (int)std::min<int64_t>(k, nr);
    if (k < 1) k = 1;
    const int s = std::max(plain_splits(ctx, nq, nr, 8), plain_splits(ctx, nq, nr, 4));
    return (size_t)s * nq * k * (sizeof(uint64_t) + sizeof(int64_t));
}

template <int TQ, bool WIDE, bool VEC>
static int launch_plain_t(const PlainArgs& a, int64_t nq, cudaStream_t stream) {
    constexpr int BQ = TQ * 16;
    const size_t tiles = (size_t)2 * kKT * ((BQ + 4) + (kBR + 4)) * sizeof(float);
    const size_t dt = (size_t)BQ * (kBR + 1) * (WIDE ? 8 : 4);
    const size_t xl = (size_t)2 * BQ * kMaxK * 8;
    const size_t smem = std::max(std::max(tiles, dt), xl);
    auto kern = plain_kernel<TQ, WIDE, VEC>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "search: cudaFuncSetAttribute");
    const int64_t qtiles = (nq + BQ - 1) / BQ;
    kern<<<dim3((unsigned)qtiles, a.n_splits), kThreadsP, smem, stream>>>(a);
    e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "search: plain launch");
}

int launch_search_plain(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qn, int64_t nq, int32_t maxq,
                        const int16_t* d_r, const int64_t* d_rn, int64_t nr, int32_t maxr, int k, int mode,
                        float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot, void* d_work,
                        size_t work_bytes, cudaStream_t stream) {
    if (nq == 0) return HDC_OK;
    if (nr <= 0) return fail(HDC_ERR_INVALID, "search: empty reference set");
    if (k > nr) k = (int)nr;  // src/cosine.cu:451
    if (k < 1 || k > kMaxK) return fail(HDC_ERR_INVALID, "search: k must be in 1..32");
    if (nr > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "search: more than 2^31-1 references");
    if (maxq < 0 || maxr < 0) return fail(HDC_ERR_INVALID, "search: negative bound");
    const int64_t prod = (int64_t)std::max(maxq, 1) * std::max(maxr, 1);
    const int64_t lim = (int64_t)1 << 22;  // |fp32 partial| < 2^22 keeps FFMA chains and the fold exact
    const int64_t chunk_dims = (lim - 1) / prod;
    if (chunk_dims < 4)
        return fail(HDC_ERR_RANGE, "search: max|q|*max|r| must not exceed 2^20 (exact fp32 chunks of 4 dims)");
    const int fold_groups = (int)std::min<int64_t>(chunk_dims / 4, 1 << 24);
    const bool wide = prod * (int64_t)ctx->dim >= ((int64_t)1 << 31);
    const bool vec = (ctx->dim % 8 == 0) && ((reinterpret_cast<uintptr_t>(d_q) & 15) == 0) &&
                     ((reinterpret_cast<uintptr_t>(d_r) & 15) == 0);
    const int tq = wide || (fold_groups <= kPlainFoldTile && nr >= kPlainWideTileRefs) ? 4 : 8;
    PlainArgs a{};
    a.q = d_q;
    a.qn = d_qn;
    a.nq = nq;
    a.r = d_r;
    a.rn = d_rn;
    a.nr = nr;
    a.dim = ctx->dim;
    a.k = k;
    a.mode = mode;
    a.fold_groups = fold_groups;
    a.n_splits = plain_splits(ctx, nq, nr, tq);
    const int64_t rtiles = (nr + kBR - 1) / kBR;
    a.split_len = ((rtiles + a.n_splits - 1) / a.n_splits) * kBR;
    a.n_splits = (int)((nr + a.split_len - 1) / a.split_len);
    const size_t need = (size_t)a.n_splits * nq * k * (sizeof(uint64_t) + sizeof(int64_t));
    if (!d_work || work_bytes < need) return fail(HDC_ERR_INVALID, "search: workspace too small");
    a.ws_key = static_cast<uint64_t*>(d_work);
    a.ws_dot = reinterpret_cast<int64_t*>(a.ws_key + (size_t)a.n_splits * nq * k);
    int st;
    if (wide)
        st = vec ? launch_plain_t<4, true, true>(a, nq, stream) : launch_plain_t<4, true, false>(a, nq, stream);
    else
        st = tq == 4 ? (vec ? launch_plain_t<4, false, true>(a, nq, stream) : launch_plain_t<4, false, false>(a, nq, stream))
                     : (vec ? launch_plain_t<8, false, true>(a, nq, stream) : launch_plain_t<8, false, false>(a, nq, stream));
    if (st != HDC_OK) return st;
    return launch_merge(a.ws_key, a.ws_dot, a.n_splits, nq, k, d_qn, d_rn, nr, d_score, d_idx, d_cos, d_dot, stream);
}

int launch_merge(const uint64_t* ws_key, const int64_t* ws_dot, int n_lists, int64_t nq, int k, const int64_t* d_qn,
                 const int64_t* d_rn, int64_t nr, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot,
                 cudaStream_t stream) {
    const int mt = 128;
    merge_kernel<<<(unsigned)((nq + mt - 1) / mt), mt, 0, stream>>>(ws_key, ws_dot, n_lists, nq, k, d_qn, d_rn, nr,
                                                                  d_score, d_idx, d_cos, d_dot);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "search: merge launch");
}

int launch_bundle(hdc_context* ctx, const void* d_rows, int elem_bytes, const int64_t* d_child_ptr,
                  const int32_t* d_child_idx, int64_t n_parents, int32_t* d_out, cudaStream_t stream) {
    if (n_parents == 0) return HDC_OK;
    if (n_parents > 65535) {
        // grid.y limit: launch in slices
        for (int64_t p0 = 0; p0 < n_parents; p0 += 65535) {
            const int64_t np = std::min<int64_t>(65535, n_parents - p0);
            int st = launch_bundle(ctx, d_rows, elem_bytes, d_child_ptr + p0, d_child_idx, np,
                                   d_out + p0 * ctx->dim, stream);
            if (st != HDC_OK) return st;
        }
        return HDC_OK;
    }
    dim3 grid((ctx->dim + 255) / 256, (unsigned)n_parents);
    if (elem_bytes == 2)
        bundle_kernel<int16_t><<<grid, 256, 0, stream>>>(static_cast<const int16_t*>(d_rows), ctx->dim, d_child_ptr,
                                                         d_child_idx, n_parents, d_out);
    else
        bundle_kernel<int32_t><<<grid, 256, 0, stream>>>(static_cast<const int32_t*>(d_rows), ctx->dim, d_child_ptr,
                                                         d_child_idx, n_parents, d_out);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "bundle: launch");
}

}  // namespace hdc

// ---------------------------------------------------------------- search without device allocation
// Fixed scratch of hdc_search_plain_noalloc: the per-range top-k lists that
// hdc_search_plain keeps in the caller's workspace.  It is part of the
// library's device image, so every GPU that loads the library holds these
// HDC_NOALLOC_SCRATCH_BYTES until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[HDC_NOALLOC_SCRATCH_BYTES];

namespace hdc {
namespace {
std::mutex g_noalloc_mutex;
}  // namespace

// Device address of the fixed scratch on the context's device (which must be
// current).  In host code the array's name only stands in for the symbol, so
// the address is asked of the runtime on the first call with a context and
// kept in the context.  A context does not outlive its device's state, so
// after cudaDeviceReset the new contexts look the address up again.
static int noalloc_scratch(hdc_context* ctx, void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "search_plain_noalloc: cudaGetDevice");
    if (dev != ctx->device)
        return fail(HDC_ERR_INVALID, "search_plain_noalloc: the context's device must be the current device");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!ctx->noalloc_scratch) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "search_plain_noalloc: cudaGetSymbolAddress");
        ctx->noalloc_scratch = p;
    }
    *out = ctx->noalloc_scratch;
    return HDC_OK;
}

}  // namespace hdc

extern "C" int hdc_search_plain_noalloc(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                                        int32_t max_abs_q, const int16_t* d_r, const int64_t* d_rnorm2, int64_t nr,
                                        int32_t max_abs_r, int k, int score_mode, float* d_score, int32_t* d_idx,
                                        double* d_cos, int64_t* d_dot, void* stream) {
    using namespace hdc;
    if (!ctx) return fail(HDC_ERR_INVALID, "search_plain_noalloc: null context");
    if (nq < 0 || nr < 0) return fail(HDC_ERR_INVALID, "search_plain_noalloc: negative count");
    if (nq == 0) return HDC_OK;
    if (!valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "search_plain_noalloc: bad score mode");
    if (!d_q || !d_qnorm2 || !d_r || !d_rnorm2 || !d_score || !d_idx)
        return fail(HDC_ERR_INVALID, "search_plain_noalloc: null pointer");
    if (nr <= 0) return fail(HDC_ERR_INVALID, "search_plain_noalloc: empty reference set");
    const int64_t kk = std::min<int64_t>(k, nr);  // as hdc_search_plain: k is clamped to nr, then checked
    if (kk < 1 || kk > kMaxK) return fail(HDC_ERR_INVALID, "search_plain_noalloc: k must be in 1..32");
    const size_t need = plain_workspace_bytes(ctx, nq, nr, k);
    if (need > (size_t)HDC_NOALLOC_SCRATCH_BYTES)
        return fail(HDC_ERR_RANGE, "search_plain_noalloc: this batch needs " + std::to_string(need) +
                                       " bytes of scratch but the fixed scratch holds " +
                                       std::to_string((size_t)HDC_NOALLOC_SCRATCH_BYTES) +
                                       "; pass fewer queries per call");
    void* scratch = nullptr;
    int st = noalloc_scratch(ctx, &scratch);
    if (st != HDC_OK) return st;
    // The kernel writes every scratch entry the merge reads, so nothing is cleared.
    return launch_search_plain(ctx, d_q, d_qnorm2, nq, max_abs_q, d_r, d_rnorm2, nr, max_abs_r, k, score_mode, d_score,
                               d_idx, d_cos, d_dot, scratch, (size_t)HDC_NOALLOC_SCRATCH_BYTES,
                               static_cast<cudaStream_t>(stream));
}
