// identify on the GPU: the application of targets/identify.cpp with its
// scoring (:137-159, HVCache::similarity over every sequence of every
// candidate node) and the level loop in one hdc_identify launch.
//
//   identify <sequence-directory> <taxonomy-file> <input-fasta> <output-file>
//
// Host side, as in the reference: FASTA reads (a record's name is the header
// line after '>', the first name of a repeated sequence wins, :46-71); the
// taxonomy through Hierarchy; level 0 candidates get_order("p__"); the result
// text goes to <output-file> when that file exists, else to stdout (:213-246).
// GPU side: every node's sequences are cut into similarity rows (the windows
// x = 0, step, ... while x + L < len, or the whole sequence when
// len <= L, src/encoder.cpp:198-215), encoded with compute semantics
// (hdc_encode_segments) together with the whole reads (HVCache::get), and
// hdc_identify runs the descent (beam 5, threshold 0, NORM score).
//
// The order of the result lines is the iteration order of the reference's
// unordered_maps; it is reproduced by replaying the same insertions and
// erasures on maps of the same key type (the order depends on the keys and
// on that history, not on the mapped values).
#include <cstdio>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "config.h"
#include "hdc_gb300.h"
#include "hierarchy.h"

namespace {

constexpr int kLevels = 6;
constexpr int kBeam = 5;
constexpr double kThreshold = 0.0;

void check(int st, const char* what) {
    if (st != HDC_OK) throw std::runtime_error(std::string(what) + ": " + hdc_last_error());
}

struct Dev {
    void* p = nullptr;
    explicit Dev(size_t n) { check(hdc_device_alloc(n ? n : 16, &p), "alloc"); }
    ~Dev() { hdc_device_free(p); }
    template <class T>
    T* as() const { return static_cast<T*>(p); }
};

template <class T>
void upload(Dev& d, const std::vector<T>& v) {
    if (!v.empty()) check(hdc_copy(d.p, v.data(), v.size() * sizeof(T), 1, nullptr), "copy");
}

// segments of a byte buffer to encode: (offset, length)
struct Segments {
    std::string bytes;
    std::vector<int64_t> off;
    std::vector<int32_t> len;
    int32_t max_len = 0;
    int64_t add_text(const std::string& s) {
        const int64_t o = (int64_t)bytes.size();
        bytes += s;
        return o;
    }
    void add(int64_t o, int32_t n) {
        off.push_back(o);
        len.push_back(n);
        if (n > max_len) max_len = n;
    }
};

// whole-sequence or windowed int16 encodes of `seg`, plus squared norms
void encode(hdc_context* ctx, const Segments& seg, Dev& hv, Dev& n2) {
    const int64_t n = (int64_t)seg.off.size();
    if (n == 0) return;
    Dev d_bytes(seg.bytes.size() + 16), d_off(n * 8), d_len(n * 4);
    check(hdc_copy(d_bytes.p, seg.bytes.data(), seg.bytes.size(), 1, nullptr), "copy");
    upload(d_off, seg.off);
    upload(d_len, seg.len);
    check(hdc_encode_segments(ctx, d_bytes.as<char>(), d_off.as<int64_t>(), d_len.as<int32_t>(), n, seg.max_len,
                              HDC_OUT_I16, hv.p, HV_DIM, nullptr, nullptr),
          "encode");
    check(hdc_norms(ctx, hv.p, 2, n, n2.as<int64_t>(), nullptr, nullptr), "norms");
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "Usage: identify sequence-directory taxonomy-file input-fasta output-file\n");
        return 1;
    }
    Hierarchy tree(argv[1], argv[2]);

    // reads
    std::vector<std::string> seqs;
    std::unordered_map<std::string, std::string> seq_to_name;
    if (std::filesystem::exists(argv[3])) {
        std::ifstream in(argv[3]);
        std::string line, seq, name;
        auto flush = [&] {
            if (!seq.empty()) {
                seqs.push_back(seq);
                seq_to_name.emplace(seq, name);
                seq.clear();
            }
        };
        while (std::getline(in, line)) {
            if (line.starts_with(">")) {
                flush();
                name = line.substr(1);
            } else {
                seq += line;
            }
        }
        flush();
    }
    // the reference's read map: distinct sequences, emplaced in file order
    std::unordered_map<std::string, int32_t> sequences;
    std::vector<const std::string*> reads;
    for (const auto& s : seqs)
        if (sequences.emplace(s, (int32_t)reads.size()).second) reads.push_back(&s);

    // taxonomy nodes reachable from the level-0 candidates, breadth first
    std::vector<std::string> roots = tree.get_order("p__");
    std::unordered_map<std::string, int32_t> node_id;
    std::vector<std::string> nodes;
    auto id_of = [&](const std::string& s) {
        auto it = node_id.find(s);
        if (it != node_id.end()) return it->second;
        node_id.emplace(s, (int32_t)nodes.size());
        nodes.push_back(s);
        return (int32_t)nodes.size() - 1;
    };
    std::vector<int32_t> root_ids;
    for (const auto& r : roots) root_ids.push_back(id_of(r));
    std::vector<int64_t> child_ptr(1, 0);
    std::vector<int32_t> child_idx;
    for (size_t i = 0; i < nodes.size(); ++i) {
        const std::string name = nodes[i];  // copy: id_of may grow `nodes`
        if (auto* kids = tree.get_children(name))
            for (const auto& k : *kids) child_idx.push_back(id_of(k));
        child_ptr.push_back((int64_t)child_idx.size());
    }

    // similarity rows of every node's sequences
    Segments rows;
    std::vector<int64_t> node_rows(1, 0);
    std::unordered_map<std::string, int64_t> text_at;  // each distinct sequence stored once
    for (const auto& name : nodes) {
        for (const auto& s : tree.get_sequences(name)) {
            auto it = text_at.find(s);
            const int64_t o = it != text_at.end() ? it->second : text_at.emplace(s, rows.add_text(s)).first->second;
            const size_t n = s.size();
            if (SEQUENCE_LENGTH >= n) {
                rows.add(o, (int32_t)n);
            } else {
                for (size_t x = 0; x + SEQUENCE_LENGTH < n; x += SIM_STEP) rows.add(o + (int64_t)x, SEQUENCE_LENGTH);
            }
        }
        node_rows.push_back((int64_t)rows.off.size());
    }
    Segments q;
    for (auto* r : reads) q.add(q.add_text(*r), (int32_t)r->size());

    hdc_context* ctx = nullptr;
    check(hdc_context_create(HV_DIM, KMER_SIZE, SEQUENCE_LENGTH, SIM_STEP, &ctx), "context");
    const int64_t nq = (int64_t)reads.size(), nr = (int64_t)rows.off.size();
    std::vector<int32_t> path((size_t)nq * kLevels), depth(nq), stop(nq);
    std::vector<float> path_score((size_t)nq * kLevels);
    if (nq > 0) {
        Dev d_rows((size_t)nr * HV_DIM * 2), d_rn(nr * 8), d_q((size_t)nq * HV_DIM * 2), d_qn(nq * 8);
        encode(ctx, rows, d_rows, d_rn);
        encode(ctx, q, d_q, d_qn);
        Dev d_nrows(node_rows.size() * 8), d_cp(child_ptr.size() * 8), d_ci(child_idx.size() * 4 + 4),
            d_roots(root_ids.size() * 4 + 4), d_path(path.size() * 4), d_ps(path.size() * 4), d_depth(nq * 4),
            d_stop(nq * 4);
        upload(d_nrows, node_rows);
        upload(d_cp, child_ptr);
        upload(d_ci, child_idx);
        upload(d_roots, root_ids);
        check(hdc_identify(ctx, d_q.as<int16_t>(), d_qn.as<int64_t>(), nq, d_rows.as<int16_t>(), d_rn.as<int64_t>(),
                           d_nrows.as<int64_t>(), d_cp.as<int64_t>(), d_ci.as<int32_t>(), d_roots.as<int32_t>(),
                           (int)root_ids.size(), kLevels, kBeam, kThreshold, HDC_SCORE_NORM, d_path.as<int32_t>(),
                           d_ps.as<float>(), d_depth.as<int32_t>(), d_stop.as<int32_t>(), nullptr),
              "identify");
        check(hdc_copy(path.data(), d_path.p, path.size() * 4, 0, nullptr), "copy");
        check(hdc_copy(path_score.data(), d_ps.p, path.size() * 4, 0, nullptr), "copy");
        check(hdc_copy(depth.data(), d_depth.p, nq * 4, 0, nullptr), "copy");
        check(hdc_copy(stop.data(), d_stop.p, nq * 4, 0, nullptr), "copy");
        check(hdc_stream_sync(nullptr), "sync");
    }
    hdc_context_destroy(ctx);

    // replay the reference's map history: early stops leave `sequences` level
    // by level in its iteration order (:167-189), the rest follow (:204-211)
    auto names_of = [&](int32_t r) {
        std::vector<std::string> p;
        for (int l = 0; l < depth[r]; ++l) p.push_back(nodes[path[(size_t)r * kLevels + l]]);
        return p;
    };
    std::unordered_map<std::string, std::vector<std::string>> outputs;
    for (int x = 0; x < kLevels; ++x)
        for (auto it = sequences.begin(); it != sequences.end();) {
            if (stop[it->second] == x) {
                outputs.emplace(it->first, names_of(it->second));
                it = sequences.erase(it);
            } else {
                ++it;
            }
        }
    for (auto& [target, r] : sequences) outputs[target] = names_of(r);

    std::ostream* out_stream = &std::cout;
    std::ofstream file;
    if (std::filesystem::exists(argv[4])) {
        file.open(argv[4]);
        if (file) out_stream = &file;
    }
    std::ostream& out = *out_stream;
    out << "\nRESULTS\n";
    for (auto& [key, output] : outputs) {
        out << "\n" << seq_to_name[key] << ":";
        auto it = sequences.find(key);
        if (it != sequences.end()) {  // reads that ran every level print their path with its scores
            const int32_t r = it->second;
            for (int l = 0; l < depth[r]; ++l)
                out << " " << output[l] << " (" << path_score[(size_t)r * kLevels + l] << ")";
        }
    }
    out << "\n";
    return 0;
}
