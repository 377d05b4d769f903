// Taxonomy tree + FASTA store behind the reference's Hierarchy interface
// (src/hierarchy.h:8-29), written from this specification of its observable
// behaviour (src/hierarchy.cpp is the behaviour being matched):
//
//   taxonomy file   The first line is a header.  Every other non-empty line is
//                   "<id> TAB <lowest rank> TAB <taxonomy>"; only the third
//                   field is used.  The taxonomy is split at ';'.  A token
//                   loses its leading blanks (' ' only) and is a rank name
//                   when it contains "__" and does not end with "__"; spaces
//                   in a rank name become '_'.  Each rank name is a parent of
//                   the next rank name on the same line.
//   iteration order The reference gathers the children of a parent in an
//                   std::unordered_set as the lines are read and then builds
//                   its std::unordered_map<parent, vector<child>> by walking
//                   the map of sets.  get_order() walks that map and
//                   get_children() returns those vectors, and
//                   propagate-children's greedy selection depends on the
//                   order, so the same container types are filled with the
//                   same sequence of insertions here.
//   sequences       Category c lives in <seq_dir>/<c>.fasta (c with spaces
//                   turned into '_').  A '>' line ends the current record,
//                   other lines are concatenated; empty records are dropped.
//                   A missing file is an empty category.  Files are read on
//                   first use and kept.
//   appending       The record is added to the kept list (when the category
//                   was read already), then ">" <c> "_appended_" <n> and the
//                   sequence are appended to the file, n being the kept
//                   list's size after the addition (0 when it was never
//                   read).  Missing directories are created; a file that
//                   cannot be opened is a std::runtime_error.
//   lookups         get_order(p): every parent whose name starts with p, in
//                   map order.  get_children(c): the children of c (c used as
//                   given) or nullptr.
#include "hierarchy.h"

#include <algorithm>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string_view>
#include <unordered_set>

namespace {

std::string file_text(const std::filesystem::path& p) {
    std::ifstream in(p, std::ios::binary);
    return std::string(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}

// Calls fn(line) for every '\n'-terminated line of text and for a last
// unterminated one; the '\n' is not part of the line.
template <typename Fn>
void each_line(std::string_view text, Fn&& fn) {
    while (!text.empty()) {
        const size_t nl = text.find('\n');
        if (nl == std::string_view::npos) {
            fn(text);
            return;
        }
        fn(text.substr(0, nl));
        text.remove_prefix(nl + 1);
    }
}

std::string category_name(std::string s) {
    std::replace(s.begin(), s.end(), ' ', '_');
    return s;
}

// The third tab-separated field of an index line (the rest of the line after
// the second tab), or empty when the line has fewer than two tabs.
std::string_view taxonomy_field(std::string_view line) {
    size_t at = 0;
    for (int tabs = 0; tabs < 2; ++tabs) {
        const size_t t = line.find('\t', at);
        if (t == std::string_view::npos) return {};
        at = t + 1;
    }
    return line.substr(at);
}

// The rank names of one taxonomy string, in order.
std::vector<std::string> rank_names(std::string_view tax) {
    std::vector<std::string> out;
    size_t start = 0;
    while (start <= tax.size()) {
        size_t end = tax.find(';', start);
        if (end == std::string_view::npos) end = tax.size();
        std::string_view tok = tax.substr(start, end - start);
        const size_t lead = tok.find_first_not_of(' ');
        tok = lead == std::string_view::npos ? std::string_view() : tok.substr(lead);
        const bool marked = tok.find("__") != std::string_view::npos;
        const bool bare = tok.size() >= 2 && tok.substr(tok.size() - 2) == "__";
        if (marked && !bare) out.push_back(category_name(std::string(tok)));
        start = end + 1;
    }
    return out;
}

// The records of a FASTA file: '>' lines separate them, other lines are
// joined, empty records are dropped.
std::vector<std::string> fasta_records(const std::filesystem::path& p) {
    std::vector<std::string> recs;
    std::string cur;
    each_line(file_text(p), [&](std::string_view line) {
        if (!line.empty() && line.front() == '>') {
            if (!cur.empty()) recs.push_back(std::move(cur));
            cur.clear();
        } else {
            cur.append(line);
        }
    });
    if (!cur.empty()) recs.push_back(std::move(cur));
    return recs;
}

}  // namespace

Hierarchy::Hierarchy(std::string dir, std::string taxes_path) : seq_dir(std::move(dir)), taxes(std::move(taxes_path)) {
    std::unordered_map<std::string, std::unordered_set<std::string>> kids_of;
    bool header = true;
    each_line(file_text(taxes), [&](std::string_view line) {
        if (header) {
            header = false;
            return;
        }
        if (line.empty()) return;
        const std::vector<std::string> ranks = rank_names(taxonomy_field(line));
        for (size_t r = 0; r + 1 < ranks.size(); ++r) kids_of[ranks[r]].insert(ranks[r + 1]);
    });
    for (const auto& entry : kids_of)
        children[entry.first] = std::vector<std::string>(entry.second.begin(), entry.second.end());
}

const std::vector<std::string>& Hierarchy::get_sequences(std::string category) {
    const std::string name = category_name(std::move(category));
    auto hit = seq_cache.find(name);
    if (hit == seq_cache.end()) {
        const std::filesystem::path fasta = seq_dir / (name + ".fasta");
        hit = seq_cache.emplace(name, std::filesystem::exists(fasta) ? fasta_records(fasta)
                                                                      : std::vector<std::string>()).first;
    }
    return hit->second;
}

void Hierarchy::append_sequence(std::string category, std::string seq) {
    const std::string name = category_name(std::move(category));
    if (auto kept = seq_cache.find(name); kept != seq_cache.end()) kept->second.push_back(seq);
    const std::filesystem::path fasta = seq_dir / (name + ".fasta");
    std::filesystem::create_directories(fasta.parent_path());
    std::ofstream out(fasta, std::ios::app);
    if (!out) throw std::runtime_error("cannot append to FASTA file " + fasta.string());
    out << '>' << make_seq_id(name) << '\n' << seq << '\n';
}

std::vector<std::string> Hierarchy::get_order(std::string order) {
    std::vector<std::string> parents;
    for (const auto& entry : children)
        if (std::string_view(entry.first).substr(0, order.size()) == order) parents.push_back(entry.first);
    return parents;
}

const std::vector<std::string>* Hierarchy::get_children(std::string category) {
    const auto hit = children.find(category);
    return hit == children.end() ? nullptr : &hit->second;
}

std::string Hierarchy::make_seq_id(const std::string& category) {
    const std::string name = category_name(category);
    const auto kept = seq_cache.find(name);
    return name + "_appended_" + std::to_string(kept == seq_cache.end() ? 0 : kept->second.size());
}
