// GPU.cuh drop-in: encode() and cosine_search() of the reference
// (src/encode.cu:197-409, src/cosine.cu:502-564) on top of the libhdc_gb300
// C ABI.  Link this file and libhdc_gb300.so in place of encode.cu and
// cosine.cu; the rest of the reference (HV.cpp, encoder.cpp, hierarchy.cpp,
// targets/, tests/) builds unchanged.
//
// Behaviour kept from the reference: per-sequence window lists, k clamped to
// the database size, results keyed by input pointer (duplicate pointers
// collapse), std::runtime_error on failure.  Behaviour fixed: every sequence
// of a batch is encoded from its own bases with L-k+1 k-mers per window, and
// the ranking is exact with ties to the lower database index.
#include <cstring>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>

#include "GPU.cuh"
#include "hdc_gb300.h"

namespace {

void check(int st, const char* what) {
    if (st != HDC_OK) throw std::runtime_error(std::string(what) + ": " + hdc_last_error());
}

hdc_context* context() {
    static std::mutex mu;
    static hdc_context* ctx = nullptr;
    std::lock_guard<std::mutex> lock(mu);
    if (!ctx) check(hdc_context_create(HV_DIM, KMER_SIZE, SEQUENCE_LENGTH, SIM_STEP, &ctx), "hdc_context_create");
    return ctx;
}

// device buffer freed on scope exit
struct DeviceBuffer {
    void* p = nullptr;
    explicit DeviceBuffer(size_t bytes) { check(hdc_device_alloc(bytes, &p), "hdc_device_alloc"); }
    ~DeviceBuffer() { hdc_device_free(p); }
    DeviceBuffer(const DeviceBuffer&) = delete;
    DeviceBuffer& operator=(const DeviceBuffer&) = delete;
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

}  // namespace

std::vector<std::vector<HV_16>> encode(const std::vector<int16_t>& kmer_map, const std::vector<std::string>& sequences) {
    (void)kmer_map;
    hdc_context* ctx = context();
    const size_t n = sequences.size();
    std::vector<std::vector<HV_16>> out(n);
    // batches bounded by the size of the window output (1 GiB of int16 rows)
    const size_t max_rows = std::max<size_t>(1, (size_t(1) << 30) / (sizeof(int16_t) * HV_DIM));
    size_t s0 = 0;
    while (s0 < n) {
        size_t s1 = s0, rows = 0, bytes = 0;
        while (s1 < n) {
            const size_t w = (size_t)hdc_num_windows(ctx, (int64_t)sequences[s1].size());
            if (s1 > s0 && rows + w > max_rows) break;
            rows += w;
            bytes += sequences[s1].size();
            ++s1;
        }
        std::vector<int64_t> seq_off(s1 - s0 + 1, 0), win_off(s1 - s0 + 1, 0);
        std::string buf;
        buf.reserve(bytes + 16);
        for (size_t i = s0; i < s1; ++i) {
            buf += sequences[i];
            seq_off[i - s0 + 1] = (int64_t)buf.size();
            win_off[i - s0 + 1] = win_off[i - s0] + hdc_num_windows(ctx, (int64_t)sequences[i].size());
        }
        if (rows > 0) {
            DeviceBuffer d_buf(buf.size() + 16), d_so(seq_off.size() * 8), d_wo(win_off.size() * 8),
                d_out(rows * HV_DIM * sizeof(int16_t));
            check(hdc_copy(d_buf.p, buf.data(), buf.size(), 1, nullptr), "hdc_copy");
            check(hdc_copy(d_so.p, seq_off.data(), seq_off.size() * 8, 1, nullptr), "hdc_copy");
            check(hdc_copy(d_wo.p, win_off.data(), win_off.size() * 8, 1, nullptr), "hdc_copy");
            check(hdc_encode_windows(ctx, d_buf.as<char>(), d_so.as<int64_t>(), d_wo.as<int64_t>(),
                                     (int64_t)(s1 - s0), (int64_t)rows, d_out.as<int16_t>(), nullptr),
                  "hdc_encode_windows");
            std::vector<int16_t> flat(rows * HV_DIM);
            check(hdc_copy(flat.data(), d_out.p, flat.size() * sizeof(int16_t), 0, nullptr), "hdc_copy");
            check(hdc_stream_sync(nullptr), "hdc_stream_sync");
            for (size_t i = s0; i < s1; ++i) {
                const int64_t w0 = win_off[i - s0], w1 = win_off[i - s0 + 1];
                out[i].resize((size_t)(w1 - w0));
                for (int64_t w = w0; w < w1; ++w)
                    out[i][(size_t)(w - w0)] = HV_16(flat.begin() + w * HV_DIM, flat.begin() + (w + 1) * HV_DIM);
            }
        }
        s0 = s1;
    }
    return out;
}

std::unordered_map<HV_16*, std::vector<std::pair<float, HV_16*>>> cosine_search(const std::vector<HV_16*>& inputs,
                                                                                const std::vector<HV_16*>& db,
                                                                                int k) {
    std::unordered_map<HV_16*, std::vector<std::pair<float, HV_16*>>> result;
    const int64_t nq = (int64_t)inputs.size(), nr = (int64_t)db.size();
    if (k > nr) k = (int)nr;  // src/cosine.cu:509
    if (nq == 0 || k <= 0) return result;
    hdc_context* ctx = context();
    std::vector<int16_t> fq((size_t)nq * HV_DIM), fr((size_t)nr * HV_DIM);
    for (int64_t i = 0; i < nq; ++i) std::memcpy(&fq[(size_t)i * HV_DIM], inputs[i]->data(), HV_DIM * 2);
    for (int64_t i = 0; i < nr; ++i) std::memcpy(&fr[(size_t)i * HV_DIM], db[i]->data(), HV_DIM * 2);
#ifdef HDC_DROPIN_NORM_SCORE
    const int mode = HDC_SCORE_NORM;
#else
    const int mode = HDC_SCORE_COS;
#endif
    DeviceBuffer d_q(fq.size() * 2), d_r(fr.size() * 2), d_qn(nq * 8), d_rn(nr * 8), d_max(8),
        d_s((size_t)nq * k * 4), d_i((size_t)nq * k * 4);
    check(hdc_copy(d_q.p, fq.data(), fq.size() * 2, 1, nullptr), "hdc_copy");
    check(hdc_copy(d_r.p, fr.data(), fr.size() * 2, 1, nullptr), "hdc_copy");
    const int32_t zero[2] = {0, 0};
    check(hdc_copy(d_max.p, zero, 8, 1, nullptr), "hdc_copy");
    check(hdc_norms(ctx, d_q.p, 2, nq, d_qn.as<int64_t>(), d_max.as<int32_t>(), nullptr), "hdc_norms");
    check(hdc_norms(ctx, d_r.p, 2, nr, d_rn.as<int64_t>(), d_max.as<int32_t>() + 1, nullptr), "hdc_norms");
    int32_t maxabs[2];
    check(hdc_copy(maxabs, d_max.p, 8, 0, nullptr), "hdc_copy");
    check(hdc_stream_sync(nullptr), "hdc_stream_sync");
    const size_t wb = hdc_search_workspace_bytes(ctx, nq, nr, k);
    DeviceBuffer d_w(wb);
    check(hdc_search_plain(ctx, d_q.as<int16_t>(), d_qn.as<int64_t>(), nq, maxabs[0], d_r.as<int16_t>(),
                           d_rn.as<int64_t>(), nr, maxabs[1], k, mode, d_s.as<float>(), d_i.as<int32_t>(), nullptr,
                           nullptr, d_w.p, wb, nullptr),
          "hdc_search_plain");
    std::vector<float> hs((size_t)nq * k);
    std::vector<int32_t> hi((size_t)nq * k);
    check(hdc_copy(hs.data(), d_s.p, hs.size() * 4, 0, nullptr), "hdc_copy");
    check(hdc_copy(hi.data(), d_i.p, hi.size() * 4, 0, nullptr), "hdc_copy");
    check(hdc_stream_sync(nullptr), "hdc_stream_sync");
    result.reserve((size_t)nq);
    for (int64_t i = 0; i < nq; ++i) {
        std::vector<std::pair<float, HV_16*>> m((size_t)k);
        for (int j = 0; j < k; ++j) m[(size_t)j] = {hs[(size_t)i * k + j], db[(size_t)hi[(size_t)i * k + j]]};
        result[inputs[i]] = std::move(m);
    }
    return result;
}
