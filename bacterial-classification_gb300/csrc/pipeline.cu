// Batching form: a reusable encode -> search -> top-k pipeline for streams of
// reads of uneven length, replayed as one CUDA graph per batch.
//
// Per batch the host writes the reads into pinned staging buffers and a
// longest-first order; the graph then copies them to the device, encodes the
// reads with the length-binned work queue of the encoder (warps take the next
// longest read from a counter, so long reads do not straggle at the end),
// searches them on the tensor cores against the resident database and copies
// the top-k back.  The autotuner times the tensor-core schedules
// (hdc_search_tc_tuning) on the pipeline's own buffers and keeps the fastest
// before the graph is captured.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <vector>

#include "hdc_internal.cuh"

struct hdc_pipeline {
    hdc_context* ctx = nullptr;
    const hdc_refdb* db = nullptr;
    int64_t max_reads = 0, max_bytes = 0;
    int k = 0, mode = 0, max_len = 0;
    cudaStream_t stream = nullptr;
    // device
    char* d_bytes = nullptr;
    int64_t* d_off = nullptr;
    int32_t* d_len = nullptr;
    int32_t* d_order = nullptr;
    int* d_queue = nullptr;
    __half* d_q = nullptr;
    int64_t* d_qn = nullptr;
    void* d_work = nullptr;
    size_t work_bytes = 0;
    float* d_score = nullptr;
    int32_t* d_idx = nullptr;
    // pinned host staging
    char* h_bytes = nullptr;
    int64_t* h_off = nullptr;
    int32_t* h_len = nullptr;
    int32_t* h_order = nullptr;
    float* h_score = nullptr;
    int32_t* h_idx = nullptr;
    cudaGraphExec_t exec = nullptr;      // copies in, kernels, copies out
    cudaGraphExec_t exec_res = nullptr;  // kernels only, on the batch already on the device
    float tuned_ms = 0.0f;
};

namespace hdc {
namespace {

__global__ void fill_i64(int64_t* p, int64_t n, int64_t v) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

int enqueue_batch(hdc_pipeline* p, bool copies) {
    hdc_context* ctx = p->ctx;
    const cudaStream_t s = p->stream;
    cudaError_t e = cudaSuccess;
    if (copies) {
        e = cudaMemcpyAsync(p->d_bytes, p->h_bytes, (size_t)p->max_bytes, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_off, p->h_off, sizeof(int64_t) * p->max_reads, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_len, p->h_len, sizeof(int32_t) * p->max_reads, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->d_order, p->h_order, sizeof(int32_t) * p->max_reads, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_fail(e, "pipeline: copy to device");
    }
    e = cudaMemsetAsync(p->d_queue, 0, sizeof(int) * encode_slabs(ctx), s);
    if (e != cudaSuccess) return cuda_fail(e, "pipeline: reset queue");
    int st = launch_encode(ctx, p->d_bytes, p->d_off, p->d_len, nullptr, nullptr, 0, p->max_reads,
                           HDC_OUT_BIPOLAR_F16, p->d_q, ctx->dim, nullptr, p->max_len, s, p->d_order, p->d_queue);
    if (st != HDC_OK) return st;
    st = launch_search_tc(ctx, p->db, p->d_q, p->d_qn, p->max_reads, 1, p->k, p->mode, p->d_score, p->d_idx, nullptr,
                          nullptr, p->d_work, p->work_bytes, ctx->d_status, s);
    if (st != HDC_OK) return st;
    if (copies) {
        e = cudaMemcpyAsync(p->h_score, p->d_score, sizeof(float) * p->max_reads * p->k, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(p->h_idx, p->d_idx, sizeof(int32_t) * p->max_reads * p->k, cudaMemcpyDeviceToHost, s);
        if (e != cudaSuccess) return cuda_fail(e, "pipeline: copy to host");
    }
    return HDC_OK;
}

int capture_one(hdc_pipeline* p, bool copies, cudaGraphExec_t* out) {
    if (*out) {
        cudaGraphExecDestroy(*out);
        *out = nullptr;
    }
    cudaError_t e = cudaStreamBeginCapture(p->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "pipeline: begin capture");
    int st = enqueue_batch(p, copies);
    cudaGraph_t graph = nullptr;
    e = cudaStreamEndCapture(p->stream, &graph);
    if (st != HDC_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return cuda_fail(e, "pipeline: end capture");
    e = cudaGraphInstantiate(out, graph, 0);
    cudaGraphDestroy(graph);
    return e == cudaSuccess ? HDC_OK : cuda_fail(e, "pipeline: instantiate");
}

int capture(hdc_pipeline* p) {
    // one uncaptured pass sets the kernels' shared-memory attributes outside the capture
    int st = enqueue_batch(p, true);
    if (st != HDC_OK) return st;
    cudaError_t e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return cuda_fail(e, "pipeline: warm-up");
    st = capture_one(p, true, &p->exec);
    if (st != HDC_OK) return st;
    return capture_one(p, false, &p->exec_res);
}

void release(hdc_pipeline* p) {
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->exec_res) cudaGraphExecDestroy(p->exec_res);
    cudaFree(p->d_bytes);
    cudaFree(p->d_off);
    cudaFree(p->d_len);
    cudaFree(p->d_order);
    cudaFree(p->d_queue);
    cudaFree(p->d_q);
    cudaFree(p->d_qn);
    cudaFree(p->d_work);
    cudaFree(p->d_score);
    cudaFree(p->d_idx);
    cudaFreeHost(p->h_bytes);
    cudaFreeHost(p->h_off);
    cudaFreeHost(p->h_len);
    cudaFreeHost(p->h_order);
    cudaFreeHost(p->h_score);
    cudaFreeHost(p->h_idx);
    if (p->stream) cudaStreamDestroy(p->stream);
    delete p;
}

}  // namespace
}  // namespace hdc

using hdc::fail;

extern "C" {

int hdc_pipeline_create(hdc_context* ctx, const hdc_refdb* db, int64_t max_reads, int64_t max_bytes, int32_t max_len,
                        int k, int score_mode, hdc_pipeline** out) {
    if (!ctx || !db || !out) return fail(HDC_ERR_INVALID, "pipeline: null argument");
    *out = nullptr;
    if (max_reads < 1 || max_bytes < 1 || max_len < 1 || k < 1 || k > 32)
        return fail(HDC_ERR_INVALID, "pipeline: bad size or k");
    if (!hdc::valid_score_mode(score_mode)) return fail(HDC_ERR_INVALID, "pipeline: bad score mode");
    if (max_len - ctx->kmer + 1 > 65535) return fail(HDC_ERR_RANGE, "pipeline: reads longer than 65535 k-mers");
    auto* p = new hdc_pipeline();
    p->ctx = ctx;
    p->db = db;
    p->max_reads = max_reads;
    p->max_bytes = max_bytes;
    p->max_len = max_len;
    p->k = (int)std::min<int64_t>(k, db->nr);
    p->mode = score_mode;
    const size_t D = (size_t)ctx->dim;
    // room for the most reference lanes any autotuner candidate uses (SMs / 8)
    p->work_bytes = std::max(hdc::tc_workspace_bytes(ctx, max_reads, db, p->k),
                             (size_t)(ctx->num_sms / 8 + 1) * max_reads * p->k * (sizeof(uint64_t) + sizeof(int64_t)));
    cudaError_t e = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking);
    auto ok = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    ok(cudaMalloc(&p->d_bytes, (size_t)max_bytes + 16));
    ok(cudaMalloc(&p->d_off, sizeof(int64_t) * max_reads));
    ok(cudaMalloc(&p->d_len, sizeof(int32_t) * max_reads));
    ok(cudaMalloc(&p->d_order, sizeof(int32_t) * max_reads));
    ok(cudaMalloc(&p->d_queue, sizeof(int) * hdc::encode_slabs(ctx)));
    ok(cudaMalloc(&p->d_q, sizeof(__half) * D * max_reads));
    ok(cudaMalloc(&p->d_qn, sizeof(int64_t) * max_reads));
    ok(cudaMalloc(&p->d_work, std::max<size_t>(p->work_bytes, 16)));
    ok(cudaMalloc(&p->d_score, sizeof(float) * max_reads * p->k));
    ok(cudaMalloc(&p->d_idx, sizeof(int32_t) * max_reads * p->k));
    ok(cudaMallocHost(&p->h_bytes, (size_t)max_bytes + 16));
    ok(cudaMallocHost(&p->h_off, sizeof(int64_t) * max_reads));
    ok(cudaMallocHost(&p->h_len, sizeof(int32_t) * max_reads));
    ok(cudaMallocHost(&p->h_order, sizeof(int32_t) * max_reads));
    ok(cudaMallocHost(&p->h_score, sizeof(float) * max_reads * p->k));
    ok(cudaMallocHost(&p->h_idx, sizeof(int32_t) * max_reads * p->k));
    if (e != cudaSuccess) {
        hdc::release(p);
        return hdc::cuda_fail(e, "pipeline: allocation");
    }
    // +1/-1 query rows have squared norm dim
    hdc::fill_i64<<<(unsigned)((max_reads + 255) / 256), 256, 0, p->stream>>>(p->d_qn, max_reads, ctx->dim);
    std::memset(p->h_bytes, 'A', (size_t)max_bytes);
    for (int64_t i = 0; i < max_reads; ++i) {
        p->h_off[i] = 0;
        p->h_len[i] = 0;
        p->h_order[i] = (int32_t)i;
    }
    int st = hdc::capture(p);
    if (st != HDC_OK) {
        hdc::release(p);
        return st;
    }
    *out = p;
    return HDC_OK;
}

void hdc_pipeline_destroy(hdc_pipeline* p) {
    if (p) hdc::release(p);
}

// Reads i < n_reads are host bytes[off[i] .. off[i]+len[i]); outputs are
// [n_reads][k] on the host.  Synchronous.
int hdc_pipeline_run(hdc_pipeline* p, const char* bytes, const int64_t* off, const int32_t* len, int64_t n_reads,
                     float* scores, int32_t* idx) {
    if (!p || (n_reads > 0 && (!bytes || !off || !len || !scores || !idx)))
        return fail(HDC_ERR_INVALID, "pipeline run: null argument");
    if (n_reads < 0 || n_reads > p->max_reads) return fail(HDC_ERR_INVALID, "pipeline run: too many reads");
    // pack the batch into the pinned staging area, longest read first
    int64_t pos = 0;
    for (int64_t i = 0; i < n_reads; ++i) {
        if (len[i] < 0 || len[i] > p->max_len) return fail(HDC_ERR_INVALID, "pipeline run: read longer than max_len");
        if (pos + len[i] > p->max_bytes) return fail(HDC_ERR_INVALID, "pipeline run: batch exceeds max_bytes");
        std::memcpy(p->h_bytes + pos, bytes + off[i], (size_t)len[i]);
        p->h_off[i] = pos;
        p->h_len[i] = len[i];
        pos += len[i];
    }
    for (int64_t i = n_reads; i < p->max_reads; ++i) {
        p->h_off[i] = 0;
        p->h_len[i] = 0;
    }
    std::iota(p->h_order, p->h_order + p->max_reads, 0);
    std::stable_sort(p->h_order, p->h_order + p->max_reads,
                     [&](int32_t a, int32_t b) { return p->h_len[a] > p->h_len[b]; });
    cudaError_t e = cudaGraphLaunch(p->exec, p->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->stream);
    if (e != cudaSuccess) return hdc::cuda_fail(e, "pipeline run: graph");
    std::memcpy(scores, p->h_score, sizeof(float) * n_reads * p->k);
    std::memcpy(idx, p->h_idx, sizeof(int32_t) * n_reads * p->k);
    return HDC_OK;
}

// Replays encode + search on the batch already on the device (no copies),
// asynchronously on the pipeline's stream.
int hdc_pipeline_launch_resident(hdc_pipeline* p) {
    if (!p) return fail(HDC_ERR_INVALID, "pipeline: null pipeline");
    cudaError_t e = cudaGraphLaunch(p->exec_res, p->stream);
    return e == cudaSuccess ? HDC_OK : hdc::cuda_fail(e, "pipeline: graph launch");
}

void* hdc_pipeline_stream(hdc_pipeline* p) { return p ? (void*)p->stream : nullptr; }

// Times the tensor-core schedules on the pipeline's buffers (the last batch
// staged, or an empty one), keeps the fastest and re-captures the graph.
int hdc_pipeline_autotune(hdc_pipeline* p, int* best_group, int* best_policy, int* best_tile_n, int* best_m_blocks,
                          float* best_ms) {
    if (!p) return fail(HDC_ERR_INVALID, "autotune: null pipeline");
    hdc_context* ctx = p->ctx;
    const int sms = ctx->num_sms;
    struct Cand {
        int g, pol, n, mb;
    };
    // the library's automatic schedule first (group, L2 policy, tile and M-blocks left to the search)
    std::vector<Cand> cands = {{0, -1, 0, 0},       {sms, 0, 128, 1}, {sms, 1, 128, 1}, {sms / 2, 0, 128, 1},
                               {sms / 4, 0, 128, 1}, {sms, 0, 128, 2}, {sms, 0, 256, 1}, {16, 1, 128, 1},
                               {8, 1, 128, 1}};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    Cand bestc = cands[0];
    for (const Cand& c : cands) {
        ctx->tc_group = c.g;
        ctx->tc_policy = c.pol;
        ctx->tc_tile_n = c.n;
        ctx->tc_m_blocks = c.mb;
        float total = 0.0f;
        bool ok = true;
        for (int rep = 0; rep < 3 && ok; ++rep) {
            cudaEventRecord(e0, p->stream);
            ok = hdc::launch_search_tc(ctx, p->db, p->d_q, p->d_qn, p->max_reads, 1, p->k, p->mode, p->d_score,
                                       p->d_idx, nullptr, nullptr, p->d_work, p->work_bytes, ctx->d_status,
                                       p->stream) == HDC_OK;
            cudaEventRecord(e1, p->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) ok = false;
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0) total += ms;  // the first run warms the schedule up
        }
        if (ok && total / 2 < best) {
            best = total / 2;
            bestc = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->tc_group = bestc.g;
    ctx->tc_policy = bestc.pol;
    ctx->tc_tile_n = bestc.n;
    ctx->tc_m_blocks = bestc.mb;
    p->tuned_ms = best;
    if (best_group) *best_group = bestc.g;
    if (best_policy) *best_policy = bestc.pol;
    if (best_tile_n) *best_tile_n = bestc.n;
    if (best_m_blocks) *best_m_blocks = bestc.mb;
    if (best_ms) *best_ms = best;
    return hdc::capture(p);
}

}  // extern "C"
