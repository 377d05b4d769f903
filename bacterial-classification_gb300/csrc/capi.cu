// extern "C" entry points of libhdc_gb300 (declared in include/hdc_gb300.h).
#include <cuda_runtime.h>

#include <cstring>
#include <random>
#include <string>

#include "hdc_internal.cuh"

namespace {
thread_local std::string g_last_error;
}

namespace hdc {

int fail(int status, const std::string& msg) {
    g_last_error = msg;
    return status;
}

int cuda_fail(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? HDC_ERR_NOMEM : HDC_ERR_CUDA;
}

}  // namespace hdc

using hdc::fail;

extern "C" {

const char* hdc_last_error(void) { return g_last_error.c_str(); }

const char* hdc_status_string(int status) {
    switch (status) {
        case HDC_OK: return "ok";
        case HDC_ERR_INVALID: return "invalid argument";
        case HDC_ERR_RANGE: return "value range";
        case HDC_ERR_CUDA: return "CUDA error";
        case HDC_ERR_NOMEM: return "out of device memory";
        case HDC_ERR_UNSUPPORTED: return "unsupported device";
        case HDC_ERR_TIMEOUT: return "device wait timed out";
        default: return "unknown status";
    }
}

// Base hypervectors exactly as src/HV.cpp:20-41: mt19937_64(seed), one draw per
// 64-bit word, bits at and above HV_DIM cleared; seeds A=0, C=1, T=2, G=3
// (src/HV.cpp:37-40).  Stored in code order A,C,G,T.
int hdc_context_create(int dim, int kmer, int window, int step, hdc_context** out) {
    if (!out) return fail(HDC_ERR_INVALID, "context: null output pointer");
    *out = nullptr;
    if (dim < 1 || dim > (1 << 20)) return fail(HDC_ERR_INVALID, "context: dim must be in 1..2^20");
    if (kmer < 1 || kmer > 16) return fail(HDC_ERR_INVALID, "context: kmer must be in 1..16");
    if (window < 1 || step < 1) return fail(HDC_ERR_INVALID, "context: window and step must be positive");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return hdc::cuda_fail(e, "context: cudaGetDevice");
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return hdc::cuda_fail(e, "context: cudaGetDeviceProperties");
    auto* c = new hdc_context();
    c->dim = dim;
    c->kmer = kmer;
    c->window = window;
    c->step = step;
    c->words64 = (dim + 63) / 64;
    c->words32 = 2 * c->words64;
    c->device = dev;
    c->num_sms = prop.multiProcessorCount;
    c->host_base = new uint64_t[4 * (size_t)c->words64];
    const int seed_of_code[4] = {0, 1, 3, 2};
    const int excess = c->words64 * 64 - dim;
    for (int code = 0; code < 4; ++code) {
        std::mt19937_64 rng((uint64_t)seed_of_code[code]);
        uint64_t* w = c->host_base + (size_t)code * c->words64;
        for (int i = 0; i < c->words64; ++i) w[i] = rng();
        if (excess > 0) w[c->words64 - 1] &= (~uint64_t(0)) >> excess;
    }
    e = cudaMalloc(&c->d_base32, sizeof(uint64_t) * 4 * (size_t)c->words64);
    if (e == cudaSuccess) e = cudaMalloc(&c->d_status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
        cudaFree(c->d_base32);
        cudaFree(c->d_status);
        delete[] c->host_base;
        delete c;
        return hdc::cuda_fail(e, "context: cudaMalloc");
    }
    // little-endian: 64-bit word i is 32-bit words 2i (low) and 2i+1 (high)
    e = cudaMemcpy(c->d_base32, c->host_base, sizeof(uint64_t) * 4 * (size_t)c->words64, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(c->d_base32);
        delete[] c->host_base;
        delete c;
        return hdc::cuda_fail(e, "context: upload");
    }
    *out = c;
    return HDC_OK;
}

void hdc_context_destroy(hdc_context* ctx) {
    if (!ctx) return;
    cudaFree(ctx->d_phase_ts);
    cudaFree(ctx->d_base32);
    cudaFree(ctx->d_status);
    delete[] ctx->host_base;
    delete ctx;
}

int hdc_context_base_hvs(const hdc_context* ctx, uint64_t* host_out) {
    if (!ctx || !host_out) return fail(HDC_ERR_INVALID, "base_hvs: null argument");
    std::memcpy(host_out, ctx->host_base, sizeof(uint64_t) * 4 * (size_t)ctx->words64);
    return HDC_OK;
}

int hdc_encode_segments(hdc_context* ctx, const char* d_bytes, const int64_t* d_seg_off, const int32_t* d_seg_len,
                        int64_t n_segs, int32_t max_len, int out_kind, void* d_out, int64_t out_stride,
                        int32_t* d_nkmers, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "encode: null context");
    if (n_segs < 0) return fail(HDC_ERR_INVALID, "encode: negative segment count");
    if (n_segs == 0) return HDC_OK;
    if (!d_bytes || !d_seg_off || !d_seg_len || !d_out) return fail(HDC_ERR_INVALID, "encode: null pointer");
    if (out_kind < HDC_OUT_I16 || out_kind > HDC_OUT_SIGN_BITS) return fail(HDC_ERR_INVALID, "encode: bad out_kind");
    if (out_stride < (out_kind == HDC_OUT_SIGN_BITS ? (ctx->dim + 31) / 32 : ctx->dim))
        return fail(HDC_ERR_INVALID, "encode: out_stride below the row length");
    if (max_len < 0) return fail(HDC_ERR_INVALID, "encode: negative max_len");
    return hdc::launch_encode(ctx, d_bytes, d_seg_off, d_seg_len, nullptr, nullptr, 0, n_segs, out_kind, d_out,
                              out_stride, d_nkmers, max_len, static_cast<cudaStream_t>(stream));
}

int hdc_beam_phase_times(const hdc_context* ctx, int64_t* out_ns, int max_n, int* n_out) {
    if (!ctx || !out_ns || !n_out || max_n < 0) return fail(HDC_ERR_INVALID, "beam_phase_times: null argument");
    const int n = hdc::beam_phase_times(ctx, out_ns, max_n);
    if (n < 0) return fail(HDC_ERR_CUDA, "beam_phase_times: read back");
    *n_out = n;
    return HDC_OK;
}

int hdc_binders(const hdc_context* ctx, const int64_t* codes, int64_t n, uint64_t* host_out) {
    if (!ctx || (n > 0 && (!codes || !host_out))) return fail(HDC_ERR_INVALID, "binders: null argument");
    if (n < 0) return fail(HDC_ERR_INVALID, "binders: negative count");
    const int W = ctx->words64, k = ctx->kmer;
    const int excess = W * 64 - ctx->dim;
    const uint64_t tail = excess > 0 ? (~uint64_t(0)) >> excess : ~uint64_t(0);
    const int64_t n_codes = (int64_t)1 << (2 * k);
    for (int64_t i = 0; i < n; ++i)
        if (codes[i] < 0 || codes[i] >= n_codes) return fail(HDC_ERR_RANGE, "binders: k-mer code out of range");
    for (int64_t i = 0; i < n; ++i) {
        uint64_t* out = host_out + (size_t)i * W;
        for (int w = 0; w < W; ++w) out[w] = ~uint64_t(0);
        for (int d = 0; d < k; ++d) {  // digit d (d = 0: the first base) rotated by d over the 64 W-bit ring
            const uint64_t* b = ctx->host_base + (size_t)((codes[i] >> (2 * (k - 1 - d))) & 3) * W;
            for (int w = 0; w < W; ++w) {
                const uint64_t next = b[w + 1 == W ? 0 : w + 1];
                out[w] ^= d == 0 ? b[w] : (b[w] >> d) | (next << (64 - d));
            }
        }
        out[W - 1] &= tail;
    }
    return HDC_OK;
}

int hdc_pack_2bit(hdc_context* ctx, const char* d_bytes, int64_t n_bytes, uint32_t* d_words, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "pack_2bit: null context");
    if (n_bytes < 0) return fail(HDC_ERR_INVALID, "pack_2bit: negative length");
    if (n_bytes == 0) return HDC_OK;
    if (!d_bytes || !d_words) return fail(HDC_ERR_INVALID, "pack_2bit: null pointer");
    return hdc::launch_pack_2bit(ctx, d_bytes, n_bytes, d_words, static_cast<cudaStream_t>(stream));
}

int hdc_encode_packed(hdc_context* ctx, const uint32_t* d_words, const int64_t* d_base_off, const int32_t* d_len,
                      int64_t n_segs, int32_t max_len, int out_kind, void* d_out, int64_t out_stride,
                      int32_t* d_nkmers, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "encode_packed: null context");
    if (n_segs < 0) return fail(HDC_ERR_INVALID, "encode_packed: negative segment count");
    if (n_segs == 0) return HDC_OK;
    if (!d_words || !d_base_off || !d_len || !d_out) return fail(HDC_ERR_INVALID, "encode_packed: null pointer");
    if (out_kind < HDC_OUT_I16 || out_kind > HDC_OUT_SIGN_BITS)
        return fail(HDC_ERR_INVALID, "encode_packed: bad out_kind");
    if (out_stride < (out_kind == HDC_OUT_SIGN_BITS ? (ctx->dim + 31) / 32 : ctx->dim))
        return fail(HDC_ERR_INVALID, "encode_packed: out_stride below the row length");
    if (max_len < 0) return fail(HDC_ERR_INVALID, "encode_packed: negative max_len");
    return hdc::launch_encode(ctx, nullptr, d_base_off, d_len, nullptr, nullptr, 0, n_segs, out_kind, d_out,
                              out_stride, d_nkmers, max_len, static_cast<cudaStream_t>(stream), nullptr, nullptr,
                              d_words);
}

int64_t hdc_num_windows(const hdc_context* ctx, int64_t len) {
    if (!ctx || len < ctx->window) return 0;
    return (len - ctx->window) / ctx->step + 1;
}

int hdc_encode_windows(hdc_context* ctx, const char* d_bytes, const int64_t* d_seq_off, const int64_t* d_win_off,
                       int64_t n_seqs, int64_t n_windows, int16_t* d_out, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "encode_windows: null context");
    if (n_seqs < 0 || n_windows < 0) return fail(HDC_ERR_INVALID, "encode_windows: negative count");
    if (n_seqs == 0 || n_windows == 0) return HDC_OK;
    if (!d_bytes || !d_seq_off || !d_win_off || !d_out) return fail(HDC_ERR_INVALID, "encode_windows: null pointer");
    return hdc::launch_encode(ctx, d_bytes, nullptr, nullptr, d_seq_off, d_win_off, n_seqs, n_windows, HDC_OUT_I16,
                              d_out, ctx->dim, nullptr, ctx->window, static_cast<cudaStream_t>(stream));
}

int hdc_norms_f16(hdc_context* ctx, const void* d_hv, int64_t n, int64_t* d_norm2, int32_t* d_maxabs, void* stream) {
    if (!ctx || (!d_hv && n) || (!d_norm2 && n)) return fail(HDC_ERR_INVALID, "norms: null pointer");
    if (n < 0) return fail(HDC_ERR_INVALID, "norms: negative count");
    return hdc::launch_norms(ctx, d_hv, hdc::kNormsF16, n, d_norm2, d_maxabs, static_cast<cudaStream_t>(stream));
}

int hdc_norms(hdc_context* ctx, const void* d_hv, int elem_bytes, int64_t n, int64_t* d_norm2, int32_t* d_maxabs,
              void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "norms: null context");
    if (elem_bytes != 1 && elem_bytes != 2 && elem_bytes != 4)
        return fail(HDC_ERR_INVALID, "norms: elem_bytes must be 1, 2 or 4");
    if (n < 0) return fail(HDC_ERR_INVALID, "norms: negative count");
    if (n > 0 && (!d_hv || !d_norm2)) return fail(HDC_ERR_INVALID, "norms: null pointer");
    return hdc::launch_norms(ctx, d_hv, elem_bytes, n, d_norm2, d_maxabs, static_cast<cudaStream_t>(stream));
}

size_t hdc_search_workspace_bytes(const hdc_context* ctx, int64_t nq, int64_t nr, int k) {
    if (!ctx || nq <= 0 || nr <= 0 || k <= 0) return 0;
    return hdc::plain_workspace_bytes(ctx, nq, nr, k);
}

int hdc_search_plain(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq, int32_t max_abs_q,
                     const int16_t* d_r, const int64_t* d_rnorm2, int64_t nr, int32_t max_abs_r, int k,
                     int score_mode, float* d_score, int32_t* d_idx, double* d_cos, int64_t* d_dot, void* d_work,
                     size_t work_bytes, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "search: null context");
    if (nq < 0 || nr < 0) return fail(HDC_ERR_INVALID, "search: negative count");
    if (nq == 0) return HDC_OK;
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "search: bad score mode");
    if (!d_q || !d_qnorm2 || !d_r || !d_rnorm2 || !d_score || !d_idx)
        return fail(HDC_ERR_INVALID, "search: null pointer");
    return hdc::launch_search_plain(ctx, d_q, d_qnorm2, nq, max_abs_q, d_r, d_rnorm2, nr, max_abs_r, k, score_mode,
                                    d_score, d_idx, d_cos, d_dot, d_work, work_bytes,
                                    static_cast<cudaStream_t>(stream));
}

int hdc_context_status(hdc_context* ctx, int* status) {
    if (!ctx || !status) return fail(HDC_ERR_INVALID, "status: null argument");
    cudaError_t e = cudaMemcpy(status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemset(ctx->d_status, 0, sizeof(int));
    if (e != cudaSuccess) return hdc::cuda_fail(e, "status: read");
    return HDC_OK;
}

int hdc_refdb_create(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                     hdc_refdb** out, void* stream) {
    if (!ctx || !out) return fail(HDC_ERR_INVALID, "refdb: null argument");
    *out = nullptr;
    if (elem_bytes != 2 && elem_bytes != 4) return fail(HDC_ERR_INVALID, "refdb: elem_bytes must be 2 or 4");
    if (nr < 1 || !d_ref) return fail(HDC_ERR_INVALID, "refdb: empty reference set");
    if (max_abs < 0) return fail(HDC_ERR_INVALID, "refdb: negative max_abs");
    return hdc::refdb_create(ctx, d_ref, elem_bytes, nr, max_abs, 0, out, static_cast<cudaStream_t>(stream));
}

int hdc_refdb_create_ex(hdc_context* ctx, const void* d_ref, int elem_bytes, int64_t nr, int32_t max_abs,
                        int32_t max_query_abs, hdc_refdb** out, void* stream) {
    if (!ctx || !out) return fail(HDC_ERR_INVALID, "refdb: null argument");
    *out = nullptr;
    if (elem_bytes != 2 && elem_bytes != 4) return fail(HDC_ERR_INVALID, "refdb: elem_bytes must be 2 or 4");
    if (nr < 1 || !d_ref) return fail(HDC_ERR_INVALID, "refdb: empty reference set");
    if (max_abs < 0) return fail(HDC_ERR_INVALID, "refdb: negative max_abs");
    if (max_query_abs < 1 || max_query_abs > 2048)
        return fail(HDC_ERR_RANGE, "refdb: max_query_abs must be in 1..2048 (exact fp16 queries)");
    return hdc::refdb_create(ctx, d_ref, elem_bytes, nr, max_abs, max_query_abs, out,
                             static_cast<cudaStream_t>(stream));
}

int hdc_refdb_limb_bits(const hdc_refdb* db) { return db ? db->limb_bits : 0; }

void hdc_refdb_destroy(hdc_refdb* db) { hdc::refdb_destroy(db); }

int hdc_refdb_limbs(const hdc_refdb* db) { return db ? db->L : 0; }

size_t hdc_search_tc_workspace_bytes(const hdc_context* ctx, const hdc_refdb* db, int64_t nq, int k) {
    if (!ctx || !db || nq <= 0 || k <= 0) return 0;
    return hdc::tc_workspace_bytes(ctx, nq, db, k);
}

int hdc_search_tc(hdc_context* ctx, const hdc_refdb* db, const void* d_q, const int64_t* d_qnorm2, int64_t nq,
                  int32_t max_abs_q, int k, int score_mode, float* d_score, int32_t* d_idx, double* d_cos,
                  int64_t* d_dot, void* d_work, size_t work_bytes, void* stream) {
    if (!ctx || !db) return fail(HDC_ERR_INVALID, "tc search: null context or database");
    if (nq < 0) return fail(HDC_ERR_INVALID, "tc search: negative count");
    if (nq == 0) return HDC_OK;
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "tc search: bad score mode");
    if (!d_q || !d_qnorm2 || !d_score || !d_idx) return fail(HDC_ERR_INVALID, "tc search: null pointer");
    return hdc::launch_search_tc(ctx, db, static_cast<const __half*>(d_q), d_qnorm2, nq, max_abs_q, k, score_mode,
                                 d_score, d_idx, d_cos, d_dot, d_work, work_bytes, ctx->d_status,
                                 static_cast<cudaStream_t>(stream));
}

int hdc_search_tc_last_shape(const hdc_context* ctx, int32_t shape[5]) {
    if (!ctx || !shape) return hdc::fail(HDC_ERR_INVALID, "tc shape: null argument");
    for (int i = 0; i < 5; ++i) shape[i] = ctx->tc_last_shape[i];
    return HDC_OK;
}

int hdc_search_tc_tuning(hdc_context* ctx, int group_tiles, int l2_policy, int tile_n, int m_blocks) {
    if (!ctx) return fail(HDC_ERR_INVALID, "tc tuning: null context");
    if (group_tiles < 0 || l2_policy < -1 || l2_policy > 2 || (tile_n != 0 && tile_n != 128 && tile_n != 256) ||
        m_blocks < 0 || m_blocks > 2)
        return fail(HDC_ERR_INVALID, "tc tuning: bad value");
    ctx->tc_m_blocks = m_blocks;
    ctx->tc_group = group_tiles;
    ctx->tc_policy = l2_policy;
    ctx->tc_tile_n = tile_n;
    return HDC_OK;
}

int hdc_context_option(hdc_context* ctx, int option, int value) {
    if (!ctx) return fail(HDC_ERR_INVALID, "option: null context");
    switch (option) {
        case HDC_TC_PREFETCH:
            if (value < -1 || value > 64) return fail(HDC_ERR_INVALID, "tc option: prefetch must be in -1..64");
            ctx->tc_prefetch = value;
            return HDC_OK;
        case HDC_TC_CLUSTER:
            if (value < 0 || value > 4 || value == 3)
                return fail(HDC_ERR_INVALID, "tc option: cluster must be 0, 1, 2 or 4");
            ctx->tc_cluster = value;
            return HDC_OK;
        case HDC_TC_SHARE:
            if (value < -1 || value > 1) return fail(HDC_ERR_INVALID, "tc option: share must be -1, 0 or 1");
            ctx->tc_share = value;
            return HDC_OK;
        case HDC_TC_SCATTER:
            if (value < -1 || value > 1) return fail(HDC_ERR_INVALID, "option: tile order must be -1, 0 or 1");
            ctx->tc_scatter = value;
            return HDC_OK;
        case HDC_TC_LANES:
            if (value < 0) return fail(HDC_ERR_INVALID, "option: lanes must be >= 0");
            ctx->tc_lanes = value;
            return HDC_OK;
        case HDC_TC_PAIR_MMA:
            ctx->tc_pair_mma = value < 0 ? -1 : (value != 0);
            return HDC_OK;
        case HDC_TC_KBLOCK:
            if (value != 0 && value != 32 && value != 64) return fail(HDC_ERR_INVALID, "option: K block must be 0, 32 or 64");
            ctx->tc_kblock = value;
            return HDC_OK;
        case HDC_BEAM_GROUPED:
            if (value < -1 || value > 2) return fail(HDC_ERR_INVALID, "option: beam grouping must be -1, 0, 1 or 2");
            ctx->beam_grouped = value;
            return HDC_OK;
        case HDC_BEAM_ONE_LAUNCH:
            if (value < -1 || value > 2)
                return fail(HDC_ERR_INVALID, "option: one-launch descent must be -1, 0, 1 or 2");
            ctx->beam_one = value;
            return HDC_OK;
        case HDC_WAIT_LIMIT:
            if (value < 0 || value > 4000000)
                return fail(HDC_ERR_INVALID, "option: wait limit must be 0 .. 4,000,000 thousand cycles");
            ctx->wait_cycles = (long long)value * 1000;
            return HDC_OK;
        case HDC_GREEDY_FORM:
            if (value < -1 || value > 1) return fail(HDC_ERR_INVALID, "option: greedy form must be -1, 0 or 1");
            ctx->greedy_form = value;
            return HDC_OK;
        case HDC_TEST_WITHHOLD_LOADS:
            if (value < 0 || value > 2) return fail(HDC_ERR_INVALID, "option: withhold must be 0, 1 or 2");
            ctx->test_withhold_loads = value;
            return HDC_OK;
        default:
            return fail(HDC_ERR_INVALID, "option: unknown option");
    }
}

int hdc_bundle(hdc_context* ctx, const void* d_rows, int elem_bytes, const int64_t* d_child_ptr,
               const int32_t* d_child_idx, int64_t n_parents, int32_t* d_out, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "bundle: null context");
    if (elem_bytes != 2 && elem_bytes != 4) return fail(HDC_ERR_INVALID, "bundle: elem_bytes must be 2 or 4");
    if (n_parents < 0) return fail(HDC_ERR_INVALID, "bundle: negative count");
    if (n_parents == 0) return HDC_OK;
    if (!d_rows || !d_child_ptr || !d_child_idx || !d_out) return fail(HDC_ERR_INVALID, "bundle: null pointer");
    return hdc::launch_bundle(ctx, d_rows, elem_bytes, d_child_ptr, d_child_idx, n_parents, d_out,
                              static_cast<cudaStream_t>(stream));
}

int hdc_propagate_greedy(hdc_context* ctx, const int16_t* d_hv, const int64_t* d_norm2, const int64_t* d_cand_ptr,
                         const int32_t* d_cand_idx, const int64_t* d_rep_ptr, const int32_t* d_rep_idx,
                         int64_t n_parents, double threshold, int score_mode, uint8_t* d_selected, float* d_best,
                         int32_t* d_scratch, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "propagate: null context");
    if (n_parents < 0) return fail(HDC_ERR_INVALID, "propagate: negative count");
    if (n_parents == 0) return HDC_OK;
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "propagate: bad score mode");
    if (!d_hv || !d_norm2 || !d_cand_ptr || !d_cand_idx || !d_rep_ptr || !d_selected || !d_scratch)
        return fail(HDC_ERR_INVALID, "propagate: null pointer");
    return hdc::launch_propagate_greedy(ctx, d_hv, d_norm2, d_cand_ptr, d_cand_idx, d_rep_ptr, d_rep_idx, n_parents,
                                        threshold, score_mode, d_selected, d_best, d_scratch,
                                        static_cast<cudaStream_t>(stream));
}

int hdc_beam_search(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qnorm2, int64_t nq, const int32_t* d_proto,
                    const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr, const int32_t* d_child_idx,
                    const int32_t* d_roots, int n_roots, int levels, int beam, double threshold, int score_mode,
                    int32_t* d_path, float* d_path_score, int32_t* d_depth, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "beam: null context");
    if (nq < 0 || n_nodes < 0) return fail(HDC_ERR_INVALID, "beam: negative count");
    if (nq == 0) return HDC_OK;
    if (n_nodes < 1 || n_nodes > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "beam: node count out of range");
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "beam: bad score mode");
    if (!d_q || !d_qnorm2 || !d_proto || !d_proto_norm2 || !d_child_ptr || !d_child_idx || !d_roots || !d_path ||
        !d_path_score || !d_depth)
        return fail(HDC_ERR_INVALID, "beam: null pointer");
    return hdc::launch_beam_search(ctx, d_q, nullptr, d_qnorm2, nq, d_proto, n_nodes, nullptr, d_proto_norm2, n_nodes,
                                   d_child_ptr, d_child_idx, d_roots, n_roots, 0, levels, beam, threshold, score_mode,
                                   d_path, d_path_score, d_depth, static_cast<cudaStream_t>(stream));
}

static int beam_split(hdc_context* ctx, const int8_t* d_q, const uint32_t* d_qbits, const int64_t* d_qnorm2, int64_t nq,
                          const int32_t* d_proto32, int64_t n_wide, const int16_t* d_proto16,
                          const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                          const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                          int levels, int beam, double threshold, int score_mode, int32_t* d_path,
                          float* d_path_score, int32_t* d_depth, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "beam split: null context");
    if (nq < 0 || n_nodes < 0) return fail(HDC_ERR_INVALID, "beam split: negative count");
    if (nq == 0) return HDC_OK;
    if (n_nodes < 1 || n_nodes > 0x7fffffffLL) return fail(HDC_ERR_INVALID, "beam split: node count out of range");
    if (n_wide < 0 || n_wide > n_nodes) return fail(HDC_ERR_INVALID, "beam split: n_wide must be in 0..n_nodes");
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "beam split: bad score mode");
    if (max_children < 0) return fail(HDC_ERR_INVALID, "beam split: negative max_children");
    if ((!d_q && !d_qbits) || !d_qnorm2 || (n_wide > 0 && !d_proto32) || (n_wide < n_nodes && !d_proto16) || !d_proto_norm2 ||
        !d_child_ptr || !d_child_idx || !d_roots || !d_path || !d_path_score || !d_depth)
        return fail(HDC_ERR_INVALID, "beam split: null pointer");
    return hdc::launch_beam_search(ctx, d_q, d_qbits, d_qnorm2, nq, d_proto32, n_wide, d_proto16, d_proto_norm2, n_nodes,
                                   d_child_ptr, d_child_idx, d_roots, n_roots, max_children, levels, beam, threshold,
                                   score_mode,
                                   d_path, d_path_score, d_depth, static_cast<cudaStream_t>(stream));
}

int hdc_beam_search_split(hdc_context* ctx, const int8_t* d_q, const int64_t* d_qnorm2, int64_t nq,
                          const int32_t* d_proto32, int64_t n_wide, const int16_t* d_proto16,
                          const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                          const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                          int levels, int beam, double threshold, int score_mode, int32_t* d_path,
                          float* d_path_score, int32_t* d_depth, void* stream) {
    return beam_split(ctx, d_q, nullptr, d_qnorm2, nq, d_proto32, n_wide, d_proto16, d_proto_norm2, n_nodes,
                      d_child_ptr, d_child_idx, d_roots, n_roots, max_children, levels, beam, threshold, score_mode,
                      d_path, d_path_score, d_depth, stream);
}

int hdc_beam_search_split_bits(hdc_context* ctx, const uint32_t* d_qbits, const int64_t* d_qnorm2, int64_t nq,
                               const int32_t* d_proto32, int64_t n_wide, const int16_t* d_proto16,
                               const int64_t* d_proto_norm2, int64_t n_nodes, const int64_t* d_child_ptr,
                               const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int max_children,
                               int levels, int beam, double threshold, int score_mode, int32_t* d_path,
                               float* d_path_score, int32_t* d_depth, void* stream) {
    if (!d_qbits && nq > 0) return fail(HDC_ERR_INVALID, "beam split: null pointer");
    return beam_split(ctx, nullptr, d_qbits, d_qnorm2, nq, d_proto32, n_wide, d_proto16, d_proto_norm2, n_nodes,
                      d_child_ptr, d_child_idx, d_roots, n_roots, max_children, levels, beam, threshold, score_mode,
                      d_path, d_path_score, d_depth, stream);
}

int hdc_similarity(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, const int16_t* d_rows,
                   const int64_t* d_row_norm2, const int64_t* d_ref_rows, const uint8_t* d_ref_whole,
                   const int32_t* d_pair_q, const int32_t* d_pair_ref, int64_t n_pairs, int score_mode,
                   float* d_score, int32_t* d_window, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "similarity: null context");
    if (n_pairs < 0) return fail(HDC_ERR_INVALID, "similarity: negative count");
    if (n_pairs == 0) return HDC_OK;
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "similarity: bad score mode");
    if (!d_q || !d_qnorm2 || !d_rows || !d_row_norm2 || !d_ref_rows || !d_pair_q || !d_pair_ref || !d_score ||
        !d_window)
        return fail(HDC_ERR_INVALID, "similarity: null pointer");
    return hdc::launch_similarity(ctx, d_q, d_qnorm2, d_rows, d_row_norm2, d_ref_rows, d_ref_whole, d_pair_q,
                                  d_pair_ref, n_pairs, score_mode, d_score, d_window,
                                  static_cast<cudaStream_t>(stream));
}

int hdc_identify(hdc_context* ctx, const int16_t* d_q, const int64_t* d_qnorm2, int64_t nq, const int16_t* d_rows,
                 const int64_t* d_row_norm2, const int64_t* d_node_rows, const int64_t* d_child_ptr,
                 const int32_t* d_child_idx, const int32_t* d_roots, int n_roots, int levels, int beam,
                 double threshold, int score_mode, int32_t* d_path, float* d_path_score, int32_t* d_depth,
                 int32_t* d_stop_level, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "identify: null context");
    if (nq < 0) return fail(HDC_ERR_INVALID, "identify: negative count");
    if (nq == 0) return HDC_OK;
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "identify: bad score mode");
    if (!d_q || !d_qnorm2 || !d_rows || !d_row_norm2 || !d_node_rows || !d_child_ptr || !d_child_idx ||
        (n_roots > 0 && !d_roots) || !d_path || !d_path_score || !d_depth)
        return fail(HDC_ERR_INVALID, "identify: null pointer");
    return hdc::launch_identify(ctx, d_q, d_qnorm2, nq, d_rows, d_row_norm2, d_node_rows, d_child_ptr, d_child_idx,
                                d_roots, n_roots, levels, beam, threshold, score_mode, d_path, d_path_score, d_depth,
                                d_stop_level, static_cast<cudaStream_t>(stream));
}

int hdc_fasta_parse(hdc_context* ctx, const char* d_in, int64_t n, char* d_out, int64_t* d_seq_off,
                    int32_t* d_seq_len, int64_t* d_name_off, int32_t* d_name_len, int64_t max_records,
                    int64_t* d_count, void* stream) {
    if (!ctx) return fail(HDC_ERR_INVALID, "fasta: null context");
    if (n < 0 || max_records < 0) return fail(HDC_ERR_INVALID, "fasta: negative size");
    if (!d_count || (n > 0 && (!d_in || !d_out)) ||
        (max_records > 0 && (!d_seq_off || !d_seq_len || !d_name_off || !d_name_len)))
        return fail(HDC_ERR_INVALID, "fasta: null pointer");
    return hdc::launch_fasta_parse(ctx, d_in, n, d_out, d_seq_off, d_seq_len, d_name_off, d_name_len, max_records,
                                   d_count, static_cast<cudaStream_t>(stream));
}

int hdc_device_alloc(size_t bytes, void** out) {
    if (!out) return fail(HDC_ERR_INVALID, "alloc: null output pointer");
    *out = nullptr;
    if (bytes == 0) return HDC_OK;
    cudaError_t e = cudaMalloc(out, bytes);
    return e == cudaSuccess ? HDC_OK : hdc::cuda_fail(e, "alloc: cudaMalloc");
}

int hdc_device_free(void* p) {
    cudaError_t e = cudaFree(p);
    return e == cudaSuccess ? HDC_OK : hdc::cuda_fail(e, "free: cudaFree");
}

int hdc_copy(void* dst, const void* src, size_t bytes, int to_device, void* stream) {
    if (bytes == 0) return HDC_OK;
    if (!dst || !src) return fail(HDC_ERR_INVALID, "copy: null pointer");
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost,
                                    static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? HDC_OK : hdc::cuda_fail(e, "copy: cudaMemcpyAsync");
}

int hdc_stream_sync(void* stream) {
    cudaError_t e = cudaStreamSynchronize(static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? HDC_OK : hdc::cuda_fail(e, "sync: cudaStreamSynchronize");
}

}  // extern "C"
