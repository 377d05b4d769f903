// Taxonomy tree + FASTA store (see hierarchy.h).  Behaviour of the reference's
// src/hierarchy.cpp:
//   * taxonomy_index.tsv: the first line is a header; each line is
//     id \t lowest-rank \t "k__x;p__y;...": tokens are trimmed of leading
//     spaces, kept when they contain "__" and do not end with it, spaces
//     become '_' (:18-55);
//   * consecutive kept ranks make parent -> child edges, gathered per parent
//     in an unordered_set and then copied into the children map (:47-55);
//   * sequences of a category live in <seq_dir>/<category>.fasta, loaded on
//     first use (:57-83); appending adds to the cache (when loaded) and to the
//     file, with the id <category>_appended_<n> (:85-108, :125-130);
//   * get_order(prefix) lists the parents whose name starts with prefix, in
//     the children map's order (:110-116).
#include "hierarchy.h"

#include <fstream>
#include <sstream>
#include <stdexcept>
#include <unordered_set>

namespace {
std::string underscores(std::string s) {
    for (char& c : s)
        if (c == ' ') c = '_';
    return s;
}
}  // namespace

Hierarchy::Hierarchy(std::string dir, std::string taxes_path) : seq_dir(dir), taxes(taxes_path) {
    std::unordered_map<std::string, std::unordered_set<std::string>> edges;
    std::ifstream in(taxes_path);
    std::string line;
    std::getline(in, line);  // header
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        std::string id, lowest, tax;
        std::stringstream fields(line);
        std::getline(fields, id, '\t');
        std::getline(fields, lowest, '\t');
        std::getline(fields, tax);
        std::vector<std::string> ranks;
        std::stringstream toks(tax);
        std::string tok;
        while (std::getline(toks, tok, ';')) {
            tok.erase(0, tok.find_first_not_of(' '));
            if (tok.find("__") != std::string::npos && !tok.ends_with("__")) ranks.push_back(underscores(tok));
        }
        for (size_t i = 1; i < ranks.size(); ++i) edges[ranks[i - 1]].insert(ranks[i]);
    }
    for (auto& [parent, kids] : edges) children[parent] = std::vector<std::string>(kids.begin(), kids.end());
}

const std::vector<std::string>& Hierarchy::get_sequences(std::string category) {
    category = underscores(category);
    auto it = seq_cache.find(category);
    if (it != seq_cache.end()) return it->second;
    std::vector<std::string> seqs;
    std::filesystem::path fasta = seq_dir / (category + ".fasta");
    if (std::filesystem::exists(fasta)) {
        std::ifstream in(fasta);
        std::string line, seq;
        while (std::getline(in, line)) {
            if (line.starts_with(">")) {
                if (!seq.empty()) {
                    seqs.push_back(seq);
                    seq.clear();
                }
            } else {
                seq += line;
            }
        }
        if (!seq.empty()) seqs.push_back(seq);
    }
    return seq_cache.emplace(category, std::move(seqs)).first->second;
}

void Hierarchy::append_sequence(std::string category, std::string seq) {
    category = underscores(category);
    auto it = seq_cache.find(category);
    if (it != seq_cache.end()) it->second.push_back(seq);
    std::filesystem::path fasta = seq_dir / (category + ".fasta");
    std::filesystem::create_directories(fasta.parent_path());
    std::ofstream out(fasta, std::ios::app);
    if (!out) throw std::runtime_error("Failed to open FASTA for append: " + fasta.string());
    out << ">" << make_seq_id(category) << "\n" << seq << "\n";
}

std::vector<std::string> Hierarchy::get_order(std::string order) {
    std::vector<std::string> out;
    for (const auto& [parent, kids] : children)
        if (parent.starts_with(order)) out.push_back(parent);
    return out;
}

const std::vector<std::string>* Hierarchy::get_children(std::string category) {
    auto it = children.find(category);
    return it == children.end() ? nullptr : &it->second;
}

std::string Hierarchy::make_seq_id(const std::string& category) {
    auto name = underscores(category);
    auto it = seq_cache.find(name);
    size_t n = it == seq_cache.end() ? 0 : it->second.size();
    return name + "_appended_" + std::to_string(n);
}
