// GPU-backed drop-in for the reference's src/encoder.h (put this directory on
// the include path ahead of the reference's src/ and link encoder_gpu.cpp in
// place of src/encoder.cpp): class HVCache with
// the same public interface (src/encoder.h:16-42), so that code written
// against it -- targets/identify.cpp, targets/propogate-children.cpp,
// tests/query-test.cpp, tests/sim-test.cpp -- compiles unchanged and encodes
// and scores on the GPU through libhdc_gb300 (encoder_gpu.cpp):
//   get(seq)        HVCache::compute on the GPU (hdc_encode_segments), kept
//                   in an LRU cache of max_entries sequences as before;
//   precompute(seq) the sequence's windows encoded in one GPU call and put
//                   in the cache, each window the compute of its substring
//                   (the reference's sliding update drifts from compute
//                   after the first window, src/encoder.cpp:176);
//   similarity(q,r) the best window score in one GPU call
//                   (hdc_encode_segments + hdc_norms + hdc_similarity); the
//                   cache is not consulted or filled by it;
//   kmers           filled at construction, as by the reference (4^channel
//                   entries; values from hdc_binders).
// Scores use the reference's cosine() scale: NORM (2 (cos - 0.5)) when
// NORM_COSINE is defined, as in its release build, else the dot product.
#pragma once
#include <cstddef>
#include <list>
#include <string>
#include <unordered_map>

#include "config.h"

constexpr size_t CACHE_BYTES = 1'000'000'000;
constexpr size_t HV_MEM = HV_DIM * 2;
constexpr size_t CACHE_SIZE = CACHE_BYTES / HV_MEM;

struct SIM {
    size_t pos;
    float score;
};

class HVCache {
public:
    explicit HVCache(size_t max_entries = CACHE_SIZE, size_t channel = KMER_SIZE);
    ~HVCache();
    HVCache(HVCache&& other) noexcept;
    HVCache(const HVCache&) = delete;
    HVCache& operator=(const HVCache&) = delete;
    HVCache& operator=(HVCache&&) = delete;

    const HV_16& get(const std::string& seq);

    void precompute(const std::string& seq);

    // Require that query is SEQUENCE_LENGTH long
    SIM similarity(const std::string& query, const std::string& reference);

    std::unordered_map<std::string, HV> kmers;

private:
    struct Entry {
        HV_16 hv;
        std::list<std::string>::iterator lru_it;
    };
    struct Device;  // the library context, device buffers and stream (encoder_gpu.cpp)

    size_t capacity;
    std::list<std::string> lru;
    std::unordered_map<std::string, Entry> map;
    size_t channel;
    Device* dev;

    const HV_16& insert(const std::string& key, HV_16&& hv);
};
