// (a) k-mer hypervector encoding on sm_103a.
//
// Semantics (bit-exact with the reference CPU encoder):
//   out[d] = sum over k-mer positions p of (2*bit_d(binder(canon(seq[p..p+k)))) - 1)
// where canon() is min(kmer, revcomp(kmer)) in A<C<G<T order and
//   binder(c)_j = 1 ^ XOR_i base[c_i][(j + i) mod 64*W]
// (src/encoder.cpp:47-74 builds binders with mult(), src/HV.cpp:98-147;
// src/encoder.cpp:106-132 bundles every position and skips k-mers holding a
// byte outside "ACGT"; src/HV.cpp:156-216 accumulates +1/-1 per bit).
//
// GB300 design
//   * One warp owns 32 W consecutive 32-bit words of the hypervector (a
//     1024 W-dim "slab"); lane l owns words W l .. W l + W - 1.  A CTA serves
//     one slab for many segments, so the slab's lookup tables are built once
//     per CTA and reused.  W = 2 where its table fits shared memory (every
//     k <= 14): the per-position work (entry load, row addresses, k-mer
//     staging) is then shared by two words.
//   * The canonical k-mer's digits are split into parts of <= 4 digits.  For
//     each part the CTA keeps in shared memory a table of all 4^len
//     pre-rotated, pre-XORed binder fragments restricted to the slab; part 0
//     also carries the all-ones start value.  A binder word is the XOR of
//     one 128 W-byte table row per part (conflict-free: the 32 lanes read the
//     32 W words of one row).
//   * Per chunk of kChunk positions each lane computes kChunk / 32 canonical
//     k-mers with a rolling 2-bit code (revcomp = bitwise NOT of the
//     little-endian code, forward = digit reversal), and writes one entry per
//     position: the byte offsets of its table rows, so a row's address is one
//     add.  Invalid k-mers and the chunk tail point at an all-zero row, which
//     contributes nothing.
//   * Bundling never unpacks bits: 16 binder words are reduced by a
//     carry-save adder tree into bit-sliced counters (ones/twos/fours/eights
//     plus NH higher planes), ~2 logic ops per word; counts are extracted
//     once per segment.
#include <cuda_bf16.h>

#include <algorithm>

#include "hdc_internal.cuh"

namespace hdc {
namespace {

constexpr int kWarps = 24;
constexpr int kThreads = kWarps * 32;
constexpr int kChunk = 64;  // positions per staged chunk
constexpr int kPerLane = kChunk / 32;
constexpr int kMaxParts = 4;
constexpr size_t kMaxEncodeSmem = 227 * 1024;  // dynamic shared memory a CTA may opt into

struct EncodeArgs {
    const uint32_t* base32;  // [4][W32], A,C,G,T
    int dim, k, W32;
    int nparts;
    int part_first[kMaxParts];  // first digit (0 = first base of the canonical k-mer)
    int part_len[kMaxParts];
    int part_row0[kMaxParts];
    int zero_row;
    int table_rows;
    const unsigned char* bytes;
    // 2-bit packed input (when set, instead of bytes): base i of the stream at bits 2 (i % 16)
    // of words[i / 16], A=0 C=1 G=2 T=3; segment offsets count bases
    const uint32_t* words;
    const int64_t* seg_off;  // explicit segments
    const int32_t* seg_len;
    const int64_t* seq_off;  // window segments: [n_seqs+1]
    const int64_t* win_off;  // [n_seqs+1]
    int64_t n_seqs;
    int window, step;
    int64_t n_segs;
    int out_kind;
    void* out;
    int64_t out_stride;
    int32_t* nkmers;
    // length-binned work queue (optional): segments are taken in the order
    // order[0], order[1], ... (longest first) from one counter per slab
    const int32_t* order;
    int* queue;  // [n_slabs] counters, zero at launch
};

__device__ __forceinline__ void csa(uint32_t& h, uint32_t& l, uint32_t a, uint32_t b, uint32_t c) {
    uint32_t u = a ^ b;
    h = (a & b) | (u & c);
    l = u ^ c;
}

__device__ __forceinline__ void get_segment(const EncodeArgs& a, int64_t g, int64_t& start, int& len) {
    if (a.seg_off) {
        start = a.seg_off[g];
        len = a.seg_len[g];
        return;
    }
    // window mode: find s with win_off[s] <= g < win_off[s+1]
    int64_t lo = 0, hi = a.n_seqs;  // invariant win_off[lo] <= g < win_off[hi]
    while (hi - lo > 1) {
        int64_t mid = (lo + hi) >> 1;
        if (a.win_off[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    start = a.seq_off[lo] + (g - a.win_off[lo]) * (int64_t)a.step;
    len = a.window;
}

// 2-bit code of an ASCII byte (A=0 C=1 G=2 T=3) and whether it is a base.
__device__ __forceinline__ uint32_t base_code(uint32_t c) { return ((c >> 1) ^ (c >> 2)) & 3u; }
__device__ __forceinline__ uint32_t is_base(uint32_t c) {
    return (c == 'A') | (c == 'C') | (c == 'G') | (c == 'T');
}

// A position's table rows, one per digit part, as byte offsets from the start of the table
// (parts past NP and invalid k-mers point at the all-zero row).
template <int NP, int W>
__device__ __forceinline__ uint4 pack_entry(const EncodeArgs& a, uint32_t canon) {
    constexpr uint32_t kRowBytes = 128u * W;
    uint32_t f[kMaxParts];
#pragma unroll
    for (int p = 0; p < kMaxParts; ++p) {
        uint32_t row = (uint32_t)a.zero_row;
        if (p < NP) {
            const int len = a.part_len[p];
            const int shift = 2 * (a.k - a.part_first[p] - len);
            row = (uint32_t)a.part_row0[p] + ((canon >> shift) & ((1u << (2 * len)) - 1u));
        }
        f[p] = row * kRowBytes;
    }
    return make_uint4(f[0], f[1], f[2], f[3]);
}

// W consecutive words of a table row from shared memory (32-bit shared address)
template <int W>
__device__ __forceinline__ void lds_words(uint32_t addr, uint32_t (&v)[W]) {
    if constexpr (W == 1) {
        asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v[0]) : "r"(addr));
    } else {
        asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(v[0]), "=r"(v[1]) : "r"(addr));
    }
}

// One word of a segment's output from its bit-sliced counters (planes: ones, twos, fours,
// eights, then hi[0 .. NH)); w32 is the word's index in the row.
template <int NH>
__device__ __forceinline__ void write_word(const EncodeArgs& a, int64_t seg, int w32, int nvalid, uint32_t ones,
                                           uint32_t twos, uint32_t fours, uint32_t eights, const uint32_t (&hi)[NH]) {
    if (a.out_kind == HDC_OUT_SIGN_BITS) {
        // a row has ceil(dim / 32) words: a word that starts at or past dim writes nothing
        // (the ring of 64-bit words can hold one more 32-bit word than that)
        if (w32 * 32 >= a.dim) return;
        // 2 count - nvalid >= 0, i.e. count >= ceil(nvalid / 2), compared plane by plane
        // from the most significant: gt = lanes already above, eq = equal so far
        const uint32_t thr = (uint32_t)(nvalid + 1) >> 1;
        uint32_t gt = 0, eq = 0xffffffffu;
        auto cmp = [&](uint32_t plane, int bit) {
            if ((thr >> bit) & 1u) {
                eq &= plane;
            } else {
                gt |= eq & plane;
                eq &= ~plane;
            }
        };
#pragma unroll
        for (int h = NH - 1; h >= 0; --h) cmp(hi[h], 4 + h);
        cmp(eights, 3);
        cmp(fours, 2);
        cmp(twos, 1);
        cmp(ones, 0);
        uint32_t bits = gt | eq;
        const int nd = min(32, a.dim - w32 * 32);
        if (nd < 32) bits &= (1u << nd) - 1u;
        reinterpret_cast<uint32_t*>(a.out)[seg * a.out_stride + w32] = bits;
        return;
    }

    // ---- counts -> output values, dims b and b+16 in 16-bit fields ----
    uint32_t val[32];
#pragma unroll
    for (int b = 0; b < 16; ++b) {
        const uint32_t M = 0x00010001u;
        uint32_t v = ((ones >> b) & M) + (((twos >> b) & M) << 1) + (((fours >> b) & M) << 2) +
                     (((eights >> b) & M) << 3);
#pragma unroll
        for (int h = 0; h < NH; ++h) v += ((hi[h] >> b) & M) << (4 + h);
        val[b] = v & 0xffffu;
        val[b + 16] = v >> 16;
    }
    const int dbase = w32 * 32;
    const int nd = min(32, a.dim - dbase);
    char* rowp = static_cast<char*>(a.out);
    if (a.out_kind == HDC_OUT_I32) {
        int32_t* o = reinterpret_cast<int32_t*>(rowp) + seg * a.out_stride + dbase;
        if (nd == 32 && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                int4 v4;
                v4.x = 2 * (int)val[4 * q + 0] - nvalid;
                v4.y = 2 * (int)val[4 * q + 1] - nvalid;
                v4.z = 2 * (int)val[4 * q + 2] - nvalid;
                v4.w = 2 * (int)val[4 * q + 3] - nvalid;
                reinterpret_cast<int4*>(o)[q] = v4;
            }
        } else {
#pragma unroll
            for (int b = 0; b < 32; ++b)
                if (b < nd) o[b] = 2 * (int)val[b] - nvalid;
        }
    } else if (a.out_kind == HDC_OUT_BIPOLAR_I8) {
        int8_t* o = reinterpret_cast<int8_t*>(rowp) + seg * a.out_stride + dbase;
        uint32_t pk[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            pk[q] = 0;
#pragma unroll
            for (int t = 0; t < 4; ++t)
                pk[q] |= (2 * (int)val[4 * q + t] - nvalid >= 0 ? 0x01u : 0xffu) << (8 * t);
        }
        if (nd == 32 && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
            reinterpret_cast<uint4*>(o)[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            reinterpret_cast<uint4*>(o)[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        } else {
#pragma unroll
            for (int b = 0; b < 32; ++b)
                if (b < nd) o[b] = (int8_t)(pk[b >> 2] >> (8 * (b & 3)));
        }
    } else {
        uint16_t* o = reinterpret_cast<uint16_t*>(rowp) + seg * a.out_stride + dbase;
        uint32_t pk[16];
#pragma unroll
        for (int q = 0; q < 16; ++q) {
            uint32_t h2[2];
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const int v = 2 * (int)val[2 * q + t] - nvalid;
                if (a.out_kind == HDC_OUT_I16)
                    h2[t] = (uint32_t)v & 0xffffu;
                else if (a.out_kind == HDC_OUT_BIPOLAR_I16)
                    h2[t] = v >= 0 ? 0x0001u : 0xffffu;
                else if (a.out_kind == HDC_OUT_BIPOLAR_F16)
                    h2[t] = v >= 0 ? 0x3c00u : 0xbc00u;  // fp16 +1 / -1
                else if (a.out_kind == HDC_OUT_F16)
                    h2[t] = __half_as_ushort(__int2half_rn(v));  // exact: |v| <= 2048
                else
                    h2[t] = v >= 0 ? 0x3f80u : 0xbf80u;  // bf16 +1 / -1
            }
            pk[q] = h2[0] | (h2[1] << 16);
        }
        if (nd == 32 && ((reinterpret_cast<uintptr_t>(o) & 15) == 0)) {
#pragma unroll
            for (int q = 0; q < 4; ++q)
                reinterpret_cast<uint4*>(o)[q] = make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
        } else {
#pragma unroll
            for (int b = 0; b < 32; ++b)
                if (b < nd) o[b] = (uint16_t)(pk[b >> 1] >> (16 * (b & 1)));
        }
    }
}

// W: words a lane owns (a slab is 32 W words; W = 2 halves the per-position work of the
// entries, addresses and k-mer staging per word, where the wider table fits shared memory)
template <int NP, int NH, int W>
__global__ void __launch_bounds__(kThreads) encode_kernel(const EncodeArgs a) {
    extern __shared__ __align__(16) uint32_t smem[];
    constexpr int SW = 32 * W;  // words per slab
    uint32_t* table = smem;     // [table_rows][SW]
    uint4* lists = reinterpret_cast<uint4*>(smem + a.table_rows * SW);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int slab = blockIdx.y;

    // ---- lookup tables for this slab ----
    for (int e = threadIdx.x; e < a.table_rows * SW; e += kThreads) {
        const int row = e / SW, w = slab * SW + (e % SW);
        uint32_t v = 0;
        if (row < a.zero_row && w < a.W32) {
            int p = 0;
            while (p + 1 < a.nparts && row >= a.part_row0[p + 1]) ++p;
            const int sub = row - a.part_row0[p], len = a.part_len[p], first = a.part_first[p];
            v = p == 0 ? ~0u : 0u;
            const int wn = (w + 1 == a.W32) ? 0 : w + 1;
            for (int t = 0; t < len; ++t) {
                const int digit = (sub >> (2 * (len - 1 - t))) & 3;
                const uint32_t* b = a.base32 + digit * a.W32;
                v ^= __funnelshift_r(b[w], b[wn], first + t);  // rot_{first+t}
            }
        }
        table[e] = v;
    }
    __syncthreads();

    // this lane's words of table row 0 (a row's W lane words are contiguous)
    const uint32_t tbase = (uint32_t)__cvta_generic_to_shared(table) + 4u * W * lane;
    uint4* list = lists + warp * kChunk;
    const uint4 zero_entry = pack_entry<0, W>(a, 0);
    const int k = a.k;
    const uint32_t mask2k = k == 16 ? 0xffffffffu : ((1u << (2 * k)) - 1u);
    const int64_t gw = (int64_t)blockIdx.x * kWarps + warp, nw = (int64_t)gridDim.x * kWarps;
    const int w0 = slab * SW + W * lane;  // this lane's first word

    int64_t next = gw;
    if (a.queue) {
        int t = 0;
        if (lane == 0) t = atomicAdd(a.queue + slab, 1);
        next = __shfl_sync(0xffffffffu, t, 0);
    }
    for (int64_t pos_q = next; pos_q < a.n_segs;) {
        const int64_t seg = a.order ? (int64_t)a.order[pos_q] : pos_q;
        int64_t start;
        int len;
        get_segment(a, seg, start, len);
        const unsigned char* s = a.words ? nullptr : a.bytes + start;
        const int npos = len >= k ? len - k + 1 : 0;
        uint32_t ones[W], twos[W], fours[W], eights[W];
        uint32_t hi[W][NH];
#pragma unroll
        for (int i = 0; i < W; ++i) {
            ones[i] = twos[i] = fours[i] = eights[i] = 0;
#pragma unroll
            for (int h = 0; h < NH; ++h) hi[i][h] = 0;
        }
        int nvalid = 0;

        for (int c0 = 0; c0 < npos; c0 += kChunk) {
            // ---- stage kPerLane canonical k-mers per lane ----
            const int p0 = c0 + lane * kPerLane;
            uint32_t x = 0, m = 0;
            auto push = [&](int pos) {
                uint32_t code, inv;
                if (a.words) {  // packed: every position of the segment is a base
                    const int64_t i = start + pos;
                    code = pos < len ? (__ldg(a.words + (i >> 4)) >> (2 * (int)(i & 15))) & 3u : 0u;
                    inv = pos < len ? 0u : 1u;
                } else {
                    const uint32_t c = pos < len ? (uint32_t)__ldg(s + pos) : 0u;
                    code = base_code(c);
                    inv = pos < len ? (is_base(c) ^ 1u) : 1u;
                }
                x = (x >> 2) | (code << (2 * (k - 1)));
                m = (m >> 1) | (inv << (k - 1));
            };
            for (int j = 0; j < k - 1; ++j) push(p0 + j);
#pragma unroll
            for (int r = 0; r < kPerLane; ++r) {
                push(p0 + r + k - 1);
                uint4 e = zero_entry;
                if (p0 + r < npos && m == 0) {
                    uint32_t rc = ~x & mask2k;
                    uint32_t y = __brev(x) >> (32 - 2 * k);
                    uint32_t fw = ((y & 0x55555555u) << 1) | ((y >> 1) & 0x55555555u);
                    e = pack_entry<NP, W>(a, fw < rc ? fw : rc);
                    ++nvalid;
                }
                list[lane * kPerLane + r] = e;
            }
            __syncwarp();

            // ---- bundle: binder words through a carry-save adder tree ----
            const int groups = (min(kChunk, npos - c0) + 15) >> 4;
            for (int g = 0; g < groups; ++g) {
                uint32_t xw[W][16];
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const uint4 e = list[g * 16 + j];
                    uint32_t v[W];
                    lds_words<W>(tbase + e.x, v);
                    if (NP > 1) {
                        uint32_t u[W];
                        lds_words<W>(tbase + e.y, u);
#pragma unroll
                        for (int i = 0; i < W; ++i) v[i] ^= u[i];
                    }
                    if (NP > 2) {
                        uint32_t u[W];
                        lds_words<W>(tbase + e.z, u);
#pragma unroll
                        for (int i = 0; i < W; ++i) v[i] ^= u[i];
                    }
                    if (NP > 3) {
                        uint32_t u[W];
                        lds_words<W>(tbase + e.w, u);
#pragma unroll
                        for (int i = 0; i < W; ++i) v[i] ^= u[i];
                    }
#pragma unroll
                    for (int i = 0; i < W; ++i) xw[i][j] = v[i];
                }
#pragma unroll
                for (int i = 0; i < W; ++i) {
                    uint32_t twosA, twosB, foursA, foursB, eightsA, eightsB, sixteens;
                    csa(twosA, ones[i], ones[i], xw[i][0], xw[i][1]);
                    csa(twosB, ones[i], ones[i], xw[i][2], xw[i][3]);
                    csa(foursA, twos[i], twos[i], twosA, twosB);
                    csa(twosA, ones[i], ones[i], xw[i][4], xw[i][5]);
                    csa(twosB, ones[i], ones[i], xw[i][6], xw[i][7]);
                    csa(foursB, twos[i], twos[i], twosA, twosB);
                    csa(eightsA, fours[i], fours[i], foursA, foursB);
                    csa(twosA, ones[i], ones[i], xw[i][8], xw[i][9]);
                    csa(twosB, ones[i], ones[i], xw[i][10], xw[i][11]);
                    csa(foursA, twos[i], twos[i], twosA, twosB);
                    csa(twosA, ones[i], ones[i], xw[i][12], xw[i][13]);
                    csa(twosB, ones[i], ones[i], xw[i][14], xw[i][15]);
                    csa(foursB, twos[i], twos[i], twosA, twosB);
                    csa(eightsB, fours[i], fours[i], foursA, foursB);
                    csa(sixteens, eights[i], eights[i], eightsA, eightsB);
                    uint32_t carry = sixteens;
#pragma unroll
                    for (int h = 0; h < NH; ++h) {
                        const uint32_t t = hi[i][h] & carry;
                        hi[i][h] ^= carry;
                        carry = t;
                    }
                }
            }
            __syncwarp();
        }
        nvalid = __reduce_add_sync(0xffffffffu, nvalid);
        if (a.nkmers && lane == 0 && slab == 0) a.nkmers[seg] = nvalid;
        // next segment: from the queue, or a fixed stride over the grid
        if (a.queue) {
            int t = 0;
            if (lane == 0) t = atomicAdd(a.queue + slab, 1);
            pos_q = __shfl_sync(0xffffffffu, t, 0);
        } else {
            pos_q += nw;
        }
#pragma unroll
        for (int i = 0; i < W; ++i)
            if (w0 + i < a.W32) write_word<NH>(a, seg, w0 + i, nvalid, ones[i], twos[i], fours[i], eights[i], hi[i]);
    }
}

// The grid: every slab served by the same number of CTAs, all of them resident at once (one
// wave).  Each warp takes a fixed share of the segments, so a CTA that had to wait for a free
// SM would run its whole share after the others finished: the call would take two CTA times.
template <int NP, int NH, int W>
int launch_np_nh(const hdc_context* ctx, const EncodeArgs& a, int n_slabs, size_t smem, cudaStream_t stream) {
    auto kern = encode_kernel<NP, NH, W>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_fail(e, "encode: cudaFuncSetAttribute");
    int per_sm = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem);
    if (e != cudaSuccess || per_sm < 1) return cuda_fail(e != cudaSuccess ? e : cudaErrorInvalidConfiguration,
                                                         "encode: occupancy");
    const int64_t fit = std::max<int64_t>(1, (int64_t)ctx->num_sms * per_sm / n_slabs);
    const int64_t need = (a.n_segs + kWarps - 1) / kWarps;
    const int grid_x = (int)std::min(fit, need);
    kern<<<dim3(grid_x, n_slabs), kThreads, smem, stream>>>(a);
    e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "encode: launch");
}

// Shared memory of a CTA whose lanes own W words: the slab's table rows and the warps' lists
size_t encode_smem(const EncodeArgs& a, int w) {
    return (size_t)a.table_rows * 32 * w * 4 + (size_t)kWarps * kChunk * sizeof(uint4);
}

// Two words a lane where that table fits a CTA's shared memory, else one
template <int NP>
int launch_np(const hdc_context* ctx, const EncodeArgs& a, int nh, cudaStream_t stream) {
    const bool w2 = encode_smem(a, 2) <= kMaxEncodeSmem;
    const int n_slabs = (a.W32 + 32 * (w2 ? 2 : 1) - 1) / (32 * (w2 ? 2 : 1));
    const size_t smem = encode_smem(a, w2 ? 2 : 1);
    if (w2) {
        if (nh <= 4) return launch_np_nh<NP, 4, 2>(ctx, a, n_slabs, smem, stream);
        if (nh <= 8) return launch_np_nh<NP, 8, 2>(ctx, a, n_slabs, smem, stream);
        return launch_np_nh<NP, 12, 2>(ctx, a, n_slabs, smem, stream);
    }
    if (nh <= 4) return launch_np_nh<NP, 4, 1>(ctx, a, n_slabs, smem, stream);
    if (nh <= 8) return launch_np_nh<NP, 8, 1>(ctx, a, n_slabs, smem, stream);
    return launch_np_nh<NP, 12, 1>(ctx, a, n_slabs, smem, stream);
}

}  // namespace

// the most slabs a call can have (one word a lane): the size of a work queue's counters
int encode_slabs(const hdc_context* ctx) { return (ctx->words32 + 31) / 32; }

namespace {
// 2-bit code of a byte as the reference packs it (src/encode.cu:169-185): A/a=0, C/c=1,
// G/g=2, T/t=3, anything else 0
__device__ __forceinline__ uint32_t pack_code(uint32_t c) {
    c &= 0xdfu;  // upper case
    return c == 'C' ? 1u : c == 'G' ? 2u : c == 'T' ? 3u : 0u;
}

// words[j] = the codes of bytes 16 j .. 16 j + 15 (a 128-bit load per word; bytes past n count 0)
__global__ void pack_2bit_kernel(const unsigned char* __restrict__ bytes, int64_t n, uint32_t* __restrict__ words,
                                 int64_t n_words) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_words; j += (int64_t)gridDim.x * blockDim.x) {
        uint32_t b[16];
        const int64_t o = j * 16;
        if (o + 16 <= n && (reinterpret_cast<uintptr_t>(bytes) & 15) == 0) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(bytes + o));
            const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int i = 0; i < 16; ++i) b[i] = (w4[i >> 2] >> (8 * (i & 3))) & 0xffu;
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) b[i] = o + i < n ? bytes[o + i] : 0u;
        }
        uint32_t w = 0;
#pragma unroll
        for (int i = 0; i < 16; ++i) w |= pack_code(b[i]) << (2 * i);
        words[j] = w;
    }
}
}  // namespace

int launch_pack_2bit(hdc_context* ctx, const char* d_bytes, int64_t n_bytes, uint32_t* d_words, cudaStream_t stream) {
    const int64_t n_words = (n_bytes + 15) / 16;
    if (n_words == 0) return HDC_OK;
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((int64_t)ctx->num_sms * 16,
                                                                          (n_words + 255) / 256));
    pack_2bit_kernel<<<grid, 256, 0, stream>>>(reinterpret_cast<const unsigned char*>(d_bytes), n_bytes, d_words,
                                               n_words);
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "pack_2bit: launch");
}

int launch_encode(hdc_context* ctx, const char* d_bytes, const int64_t* d_seg_off, const int32_t* d_seg_len,
                  const int64_t* d_seq_off, const int64_t* d_win_off, int64_t n_seqs, int64_t n_segs, int out_kind,
                  void* d_out, int64_t out_stride, int32_t* d_nkmers, int max_seg_len, cudaStream_t stream,
                  const int32_t* d_order, int* d_queue, const uint32_t* d_words) {
    if (n_segs == 0) return HDC_OK;
    EncodeArgs a{};
    a.base32 = ctx->d_base32;
    a.dim = ctx->dim;
    a.k = ctx->kmer;
    a.W32 = ctx->words32;
    // digit parts of <= 4 digits, as even as possible, longer parts first
    const int np = (a.k + 3) / 4;
    a.nparts = np;
    int first = 0, row0 = 0;
    for (int p = 0; p < np; ++p) {
        const int len = a.k / np + (p < a.k % np ? 1 : 0);
        a.part_first[p] = first;
        a.part_len[p] = len;
        a.part_row0[p] = row0;
        first += len;
        row0 += 1 << (2 * len);
    }
    a.zero_row = row0;
    a.table_rows = row0 + 1;
    a.bytes = reinterpret_cast<const unsigned char*>(d_bytes);
    a.words = d_words;
    a.seg_off = d_seg_off;
    a.seg_len = d_seg_len;
    a.seq_off = d_seq_off;
    a.win_off = d_win_off;
    a.n_seqs = n_seqs;
    a.window = ctx->window;
    a.step = ctx->step;
    a.n_segs = n_segs;
    a.out_kind = out_kind;
    a.out = d_out;
    a.out_stride = out_stride;
    a.nkmers = d_nkmers;
    a.order = d_order;
    a.queue = d_queue;

    // counters: ones..eights hold 0..15, NH higher planes hold multiples of 16
    const int64_t max_nk = max_seg_len > 0 ? std::max<int64_t>(0, (int64_t)max_seg_len - a.k + 1) : (int64_t)1 << 40;
    int nh;
    if (max_nk <= 255)
        nh = 4;
    else if (max_nk <= 4095)
        nh = 8;
    else
        nh = 12;  // counts modulo 2^16
    if (out_kind != HDC_OUT_I16 && max_nk > 65535)
        return fail(HDC_ERR_RANGE, "encode: segments longer than 65535 k-mers need HDC_OUT_I16 (counts wrap)");
    if (out_kind == HDC_OUT_F16 && max_nk > 2048)
        return fail(HDC_ERR_RANGE, "encode: fp16 counts are exact for segments of at most 2048 k-mers");

    switch (np) {
        case 1: return launch_np<1>(ctx, a, nh, stream);
        case 2: return launch_np<2>(ctx, a, nh, stream);
        case 3: return launch_np<3>(ctx, a, nh, stream);
        default: return launch_np<4>(ctx, a, nh, stream);
    }
}

}  // namespace hdc
