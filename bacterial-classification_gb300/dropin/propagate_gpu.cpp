// propagate-children on the GPU: the application of
// targets/propogate-children.cpp with its hot loop (:60-73) on
// hdc_propagate_greedy and its sequence encodes (HVCache::get, whole
// sequence) on hdc_encode_segments.
//
//   propagate-children <sequence-directory> <taxonomy-file>
//
// Same traversal as the reference: ranks p, c, o, f, g, s in turn; for each
// parent of the rank (Hierarchy::get_order order) the candidates are its
// descendants' sequences, collected child by child, each child's own
// sequences before its subtree (:16-33); a candidate is appended to the
// parent's FASTA when its best NORM cosine against the parent's sequences and
// the candidates already appended is below 0.75.  Appends of one rank only
// touch that rank's parents, which are not descendants of one another, so all
// parents of a rank are decided in one GPU launch and appended afterwards in
// the reference's order.
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "config.h"
#include "hdc_gb300.h"
#include "hierarchy.h"

namespace {

const std::vector<std::string> kOrder = {"k__", "p__", "c__", "o__", "f__", "g__", "s__"};
constexpr double kThreshold = 0.75;

void check(int st, const char* what) {
    if (st != HDC_OK) throw std::runtime_error(std::string(what) + ": " + hdc_last_error());
}

void collect(Hierarchy& tree, const std::string& node, std::vector<std::string>& out) {
    auto kids = tree.get_children(node);
    if (!kids) return;
    for (const auto& child : *kids) {
        const auto& seqs = tree.get_sequences(child);
        out.insert(out.end(), seqs.begin(), seqs.end());
        collect(tree, child, out);
    }
}

struct Dev {
    void* p = nullptr;
    explicit Dev(size_t n) { check(hdc_device_alloc(n ? n : 16, &p), "alloc"); }
    ~Dev() { hdc_device_free(p); }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "Usage: propagate-children sequence-directory taxonomy-file\n");
        return 1;
    }
    Hierarchy tree(argv[1], argv[2]);
    hdc_context* ctx = nullptr;
    check(hdc_context_create(HV_DIM, KMER_SIZE, SEQUENCE_LENGTH, SIM_STEP, &ctx), "context");
    long total = 0;
    for (size_t x = 1; x < kOrder.size(); ++x) {
        const auto parents = tree.get_order(kOrder[x]);
        if (parents.empty()) continue;
        // distinct sequences of this rank, candidate and representative lists
        std::unordered_map<std::string, int32_t> index;
        std::vector<const std::string*> uniq;
        auto id_of = [&](const std::string& s) {
            auto it = index.find(s);
            if (it != index.end()) return it->second;
            const int32_t id = (int32_t)uniq.size();
            uniq.push_back(&index.emplace(s, id).first->first);
            return id;
        };
        std::vector<std::vector<std::string>> cands(parents.size());
        std::vector<int64_t> cand_ptr(1, 0), rep_ptr(1, 0);
        std::vector<int32_t> cand_idx, rep_idx;
        for (size_t p = 0; p < parents.size(); ++p) {
            for (const auto& s : tree.get_sequences(parents[p])) rep_idx.push_back(id_of(s));
            collect(tree, parents[p], cands[p]);
            for (const auto& s : cands[p]) cand_idx.push_back(id_of(s));
            cand_ptr.push_back((int64_t)cand_idx.size());
            rep_ptr.push_back((int64_t)rep_idx.size());
        }
        if (cand_idx.empty()) continue;
        // whole-sequence encodes of the distinct sequences
        std::string bytes;
        std::vector<int64_t> off;
        std::vector<int32_t> len;
        int32_t max_len = 0;
        for (auto* s : uniq) {
            off.push_back((int64_t)bytes.size());
            len.push_back((int32_t)s->size());
            max_len = std::max(max_len, (int32_t)s->size());
            bytes += *s;
        }
        const int64_t n = (int64_t)uniq.size();
        Dev d_bytes(bytes.size() + 16), d_off(n * 8), d_len(n * 4), d_hv((size_t)n * HV_DIM * 2), d_n2(n * 8),
            d_cp(cand_ptr.size() * 8), d_ci(cand_idx.size() * 4), d_rp(rep_ptr.size() * 8),
            d_ri(std::max<size_t>(rep_idx.size(), 1) * 4), d_sel(cand_idx.size()), d_scr(cand_idx.size() * 4);
        check(hdc_copy(d_bytes.p, bytes.data(), bytes.size(), 1, nullptr), "copy");
        check(hdc_copy(d_off.p, off.data(), n * 8, 1, nullptr), "copy");
        check(hdc_copy(d_len.p, len.data(), n * 4, 1, nullptr), "copy");
        check(hdc_copy(d_cp.p, cand_ptr.data(), cand_ptr.size() * 8, 1, nullptr), "copy");
        check(hdc_copy(d_ci.p, cand_idx.data(), cand_idx.size() * 4, 1, nullptr), "copy");
        check(hdc_copy(d_rp.p, rep_ptr.data(), rep_ptr.size() * 8, 1, nullptr), "copy");
        if (!rep_idx.empty()) check(hdc_copy(d_ri.p, rep_idx.data(), rep_idx.size() * 4, 1, nullptr), "copy");
        check(hdc_encode_segments(ctx, (const char*)d_bytes.p, (const int64_t*)d_off.p, (const int32_t*)d_len.p, n,
                                  max_len, HDC_OUT_I16, d_hv.p, HV_DIM, nullptr, nullptr),
              "encode");
        check(hdc_norms(ctx, d_hv.p, 2, n, (int64_t*)d_n2.p, nullptr, nullptr), "norms");
        check(hdc_propagate_greedy(ctx, (const int16_t*)d_hv.p, (const int64_t*)d_n2.p, (const int64_t*)d_cp.p,
                                   (const int32_t*)d_ci.p, (const int64_t*)d_rp.p, (const int32_t*)d_ri.p,
                                   (int64_t)parents.size(), kThreshold, HDC_SCORE_NORM, (uint8_t*)d_sel.p, nullptr,
                                   (int32_t*)d_scr.p, nullptr),
              "propagate");
        std::vector<uint8_t> sel(cand_idx.size());
        check(hdc_copy(sel.data(), d_sel.p, sel.size(), 0, nullptr), "copy");
        check(hdc_stream_sync(nullptr), "sync");
        for (size_t p = 0; p < parents.size(); ++p)
            for (int64_t c = cand_ptr[p]; c < cand_ptr[p + 1]; ++c)
                if (sel[(size_t)c]) {
                    tree.append_sequence(parents[p], cands[p][(size_t)(c - cand_ptr[p])]);
                    ++total;
                }
    }
    hdc_context_destroy(ctx);
    std::printf("Propogated: %ld\n", total);
    return 0;
}
