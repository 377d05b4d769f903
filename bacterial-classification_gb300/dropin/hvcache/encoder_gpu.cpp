// HVCache of dropin/encoder.h on the GPU, through the libhdc_gb300 C ABI.
//
// The cache keeps the reference's LRU semantics (src/encoder.cpp:76-104: a
// hit moves the entry to the front, a miss inserts at the front and evicts
// the least recently used entry once max_entries are held); what a miss
// costs is one GPU encode instead of a CPU bundling pass.  Values are
// HVCache::compute's (src/encoder.cpp:106-132): int16 sums of the +1/-1
// binders of every k-mer of A, C, G, T, other k-mers skipped, wrapping like
// the reference's int16 accumulator.
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <unordered_set>
#include <vector>

#include "encoder.h"
#include "hdc_gb300.h"

namespace {

void check(int st, const char* what) {
    if (st != HDC_OK) throw std::runtime_error(std::string(what) + ": " + hdc_last_error());
}

#ifdef NORM_COSINE
constexpr int kScoreMode = HDC_SCORE_NORM;
#else
constexpr int kScoreMode = HDC_SCORE_DOT;
#endif

// window starts of HVCache::precompute (src/encoder.cpp:134-196): 0, then step, 2 step, ...
// while start + window < len; none when len < window
std::vector<size_t> precompute_starts(size_t len) {
    std::vector<size_t> xs;
    if (len < (size_t)SEQUENCE_LENGTH) return xs;
    xs.push_back(0);
    for (size_t x = SIM_STEP; x + SEQUENCE_LENGTH < len; x += SIM_STEP) xs.push_back(x);
    return xs;
}

// k-mer code (A=0 C=1 G=2 T=3, first base most significant) as its string
std::string kmer_string(int64_t code, int k) {
    static const char kBase[4] = {'A', 'C', 'G', 'T'};
    std::string s(k, 'A');
    for (int i = k - 1; i >= 0; --i, code >>= 2) s[i] = kBase[code & 3];
    return s;
}

}  // namespace

struct HVCache::Device {
    hdc_context* ctx = nullptr;
    void* bytes = nullptr;  // sequence bytes of a call
    size_t bytes_cap = 0;
    void* meta = nullptr;   // the call's small arrays (offsets, lengths, pair lists)
    size_t meta_cap = 0;
    void* rows = nullptr;   // int16 rows of a call
    size_t rows_cap = 0;

    ~Device() {
        hdc_device_free(bytes);
        hdc_device_free(meta);
        hdc_device_free(rows);
        hdc_context_destroy(ctx);
    }

    static void* grow(void*& p, size_t& cap, size_t need) {
        if (need > cap) {
            hdc_device_free(p);
            p = nullptr;
            cap = 0;
            check(hdc_device_alloc(need, &p), "hdc_device_alloc");
            cap = need;
        }
        return p;
    }

    // Upload `text`, encode its segments (byte offset, length) into int16 rows on the device.
    // Returns the device rows; `meta_tail` bytes after the offsets and lengths stay free in `meta`
    // for the caller, at the returned offset.
    int16_t* encode(const std::string& text, const std::vector<int64_t>& off, const std::vector<int32_t>& len,
                    size_t meta_tail, size_t* tail_at) {
        const int64_t n = (int64_t)off.size();
        grow(bytes, bytes_cap, text.size() + 16);
        const size_t off_bytes = (size_t)n * 8, len_at = (off_bytes + 15) & ~(size_t)15;
        const size_t tail = (len_at + (size_t)n * 4 + 15) & ~(size_t)15;
        grow(meta, meta_cap, tail + meta_tail + 16);
        grow(rows, rows_cap, (size_t)n * HV_DIM * 2);
        std::vector<unsigned char> host(len_at + (size_t)n * 4);
        std::memcpy(host.data(), off.data(), off_bytes);
        std::memcpy(host.data() + len_at, len.data(), (size_t)n * 4);
        check(hdc_copy(bytes, text.data(), text.size(), 1, nullptr), "hdc_copy");
        check(hdc_copy(meta, host.data(), host.size(), 1, nullptr), "hdc_copy");
        const int32_t max_len = n ? *std::max_element(len.begin(), len.end()) : 0;
        auto* m = static_cast<unsigned char*>(meta);
        check(hdc_encode_segments(ctx, static_cast<const char*>(bytes), reinterpret_cast<const int64_t*>(m),
                                  reinterpret_cast<const int32_t*>(m + len_at), n, max_len, HDC_OUT_I16, rows,
                                  HV_DIM, nullptr, nullptr),
              "hdc_encode_segments");
        *tail_at = tail;
        return static_cast<int16_t*>(rows);
    }

    // int16 hypervectors of the given substrings of `text`, on the host
    std::vector<HV_16> encode_host(const std::string& text, const std::vector<int64_t>& off,
                                   const std::vector<int32_t>& len) {
        std::vector<HV_16> out(off.size(), HV_16(HV_DIM));
        if (off.empty()) return out;
        size_t tail_at;
        const int16_t* d = encode(text, off, len, 0, &tail_at);
        std::vector<int16_t> all(off.size() * (size_t)HV_DIM);
        check(hdc_copy(all.data(), d, all.size() * 2, 0, nullptr), "hdc_copy");
        check(hdc_stream_sync(nullptr), "hdc_stream_sync");
        for (size_t i = 0; i < off.size(); ++i)
            std::memcpy(out[i].data(), all.data() + i * HV_DIM, (size_t)HV_DIM * 2);
        return out;
    }
};

HVCache::HVCache(size_t max_entries, size_t channel_) : capacity(max_entries), channel(channel_), dev(new Device()) {
    check(hdc_context_create(HV_DIM, (int)channel, SEQUENCE_LENGTH, SIM_STEP, &dev->ctx), "hdc_context_create");
    // kmers: every k-mer of length `channel` -> the binder of its canonical form (the smaller of it
    // and its reverse complement), as the reference's constructor builds it
    const int k = (int)channel;
    const int64_t n = (int64_t)1 << (2 * k);
    std::vector<int64_t> canon((size_t)n);
    for (int64_t code = 0; code < n; ++code) {
        int64_t rc = 0;
        for (int i = 0; i < k; ++i) rc |= (3 - ((code >> (2 * i)) & 3)) << (2 * (k - 1 - i));
        canon[(size_t)code] = std::min(code, rc);
    }
    const size_t W = HV_WORDS;
    std::vector<uint64_t> words((size_t)n * W);
    check(hdc_binders(dev->ctx, canon.data(), n, words.data()), "hdc_binders");
    kmers.reserve((size_t)n);
    for (int64_t code = 0; code < n; ++code)
        kmers.emplace(kmer_string(code, k), HV(words.begin() + (ptrdiff_t)((size_t)code * W),
                                                words.begin() + (ptrdiff_t)((size_t)(code + 1) * W)));
}

HVCache::~HVCache() { delete dev; }

HVCache::HVCache(HVCache&& o) noexcept
    : kmers(std::move(o.kmers)), capacity(o.capacity), lru(std::move(o.lru)), map(std::move(o.map)),
      channel(o.channel), dev(o.dev) {
    o.dev = nullptr;
}

const HV_16& HVCache::insert(const std::string& key, HV_16&& hv) {
    if (map.size() >= capacity && !lru.empty()) {
        map.erase(lru.back());
        lru.pop_back();
    }
    lru.push_front(key);
    return map.emplace(key, Entry{std::move(hv), lru.begin()}).first->second.hv;
}

const HV_16& HVCache::get(const std::string& seq) {
    auto it = map.find(seq);
    if (it != map.end()) {
        lru.splice(lru.begin(), lru, it->second.lru_it);
        return it->second.hv;
    }
    auto hv = dev->encode_host(seq, {0}, {(int32_t)seq.size()});
    return insert(seq, std::move(hv[0]));
}

void HVCache::precompute(const std::string& seq) {
    const std::vector<size_t> xs = precompute_starts(seq.size());
    if (xs.empty()) return;
    // the windows not cached yet, encoded in one call
    std::vector<int64_t> off;
    std::vector<int32_t> len;
    std::unordered_set<std::string> queued;
    for (size_t x : xs) {
        std::string key = seq.substr(x, SEQUENCE_LENGTH);
        if (map.count(key) || !queued.insert(key).second) continue;
        off.push_back((int64_t)x);
        len.push_back(SEQUENCE_LENGTH);
    }
    std::vector<HV_16> fresh = dev->encode_host(seq, off, len);
    std::unordered_map<std::string, size_t> at;
    for (size_t i = 0; i < off.size(); ++i) at.emplace(seq.substr((size_t)off[i], SEQUENCE_LENGTH), i);
    // then the cache updates in the reference's order: each window a hit (to the front) or an insert
    for (size_t x : xs) {
        std::string key = seq.substr(x, SEQUENCE_LENGTH);
        auto it = map.find(key);
        if (it != map.end()) {
            lru.splice(lru.begin(), lru, it->second.lru_it);
            continue;
        }
        auto f = at.find(key);
        if (f != at.end() && !fresh[f->second].empty()) {
            insert(key, std::move(fresh[f->second]));
            fresh[f->second].clear();
        } else {  // evicted again by the inserts before it in this call
            insert(key, std::move(dev->encode_host(seq, {(int64_t)x}, {SEQUENCE_LENGTH})[0]));
        }
    }
}

SIM HVCache::similarity(const std::string& query, const std::string& reference) {
    // rows: the whole reference when it is at most one window long (scored unclamped), else its
    // windows x = 0, step, ... while x + window < len (src/encoder.cpp:198-215)
    const bool whole = (size_t)SEQUENCE_LENGTH >= reference.size();
    std::vector<int64_t> off{0};
    std::vector<int32_t> len{(int32_t)query.size()};
    const int64_t rbase = (int64_t)query.size();
    if (whole) {
        off.push_back(rbase);
        len.push_back((int32_t)reference.size());
    } else {
        for (size_t x = 0; x + SEQUENCE_LENGTH < reference.size(); x += SIM_STEP) {
            off.push_back(rbase + (int64_t)x);
            len.push_back(SEQUENCE_LENGTH);
        }
    }
    const int64_t n_rows = (int64_t)off.size() - 1;
    // after the offsets and lengths: norms [1 + n_rows], ref_rows [2], whole flag, pair lists, result
    const size_t norms_at = 0, rr_at = ((size_t)(1 + n_rows) * 8 + 15) & ~(size_t)15;
    const size_t whole_at = rr_at + 16, pq_at = whole_at + 16, res_at = pq_at + 16;
    size_t tail_at;
    const int16_t* rows = dev->encode(query + reference, off, len, res_at + 16, &tail_at);
    auto* m = static_cast<unsigned char*>(dev->meta) + tail_at;
    int64_t rr[2] = {0, n_rows};
    unsigned char small[48] = {0};
    std::memcpy(small, rr, 16);
    small[16] = whole ? 1 : 0;
    const int32_t zero[2] = {0, 0};
    std::memcpy(small + 32, zero, 8);
    check(hdc_copy(m + rr_at, small, sizeof small, 1, nullptr), "hdc_copy");
    auto* norms = reinterpret_cast<int64_t*>(m + norms_at);
    check(hdc_norms(dev->ctx, rows, 2, 1 + n_rows, norms, nullptr, nullptr), "hdc_norms");
    auto* score = reinterpret_cast<float*>(m + res_at);
    auto* win = reinterpret_cast<int32_t*>(m + res_at + 8);
    check(hdc_similarity(dev->ctx, rows, norms, rows + HV_DIM, norms + 1, reinterpret_cast<const int64_t*>(m + rr_at),
                         reinterpret_cast<const uint8_t*>(m + whole_at), reinterpret_cast<const int32_t*>(m + pq_at),
                         reinterpret_cast<const int32_t*>(m + pq_at + 4), 1, kScoreMode, score, win, nullptr),
          "hdc_similarity");
    float s = 0.0f;
    int32_t w = -1;
    check(hdc_copy(&s, score, sizeof s, 0, nullptr), "hdc_copy");
    check(hdc_copy(&w, win, sizeof w, 0, nullptr), "hdc_copy");
    check(hdc_stream_sync(nullptr), "hdc_stream_sync");
    return SIM{whole || w < 0 ? 0 : (size_t)w * SIM_STEP, s};
}
