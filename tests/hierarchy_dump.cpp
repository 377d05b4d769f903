// Test driver: prints what a Hierarchy (src/hierarchy.h interface) reports for
// a taxonomy directory -- orders, children, sequences -- then appends records
// and prints the files it wrote.  Compiled against the reference's
// src/hierarchy.cpp and against the drop-in's; the two outputs must be equal.
//   hierarchy_dump <seq_dir> <taxonomy_index.tsv> <category to read before appending>...
#include <fstream>
#include <iostream>
#include <iterator>
#include <string>
#include <vector>

#include "hierarchy.h"

static void list(const char* what, const std::string& key, const std::vector<std::string>* v) {
    std::cout << what << " [" << key << "]";
    if (!v) {
        std::cout << " null\n";
        return;
    }
    for (const auto& s : *v) std::cout << " |" << s;
    std::cout << "\n";
}

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    Hierarchy h(argv[1], argv[2]);
    const std::vector<std::string> prefixes = {"", "k__", "p__", "c__", "o__", "f__", "g__", "s__", "x"};
    for (const auto& p : prefixes) {
        auto o = h.get_order(p);
        list("order", p, &o);
    }
    auto all = h.get_order("");
    for (const auto& n : all) {
        list("children", n, h.get_children(n));
        if (const auto* kids = h.get_children(n))
            for (const auto& c : *kids) {
                list("children", c, h.get_children(c));
                list("sequences", c, &h.get_sequences(c));
            }
        list("sequences", n, &h.get_sequences(n));
    }
    list("children", "no such node", h.get_children("no such node"));
    for (int a = 3; a < argc; ++a) h.get_sequences(argv[a]);  // cached before the appends
    for (int a = 3; a < argc; ++a) {
        h.append_sequence(argv[a], "ACGTACGT" + std::to_string(a));
        h.append_sequence(argv[a], "TTTT");
    }
    h.append_sequence("new category", "GGGG");
    h.append_sequence("new category", "CCCC");
    for (int a = 3; a < argc; ++a) list("after", argv[a], &h.get_sequences(argv[a]));
    list("after", "new category", &h.get_sequences("new category"));
    std::vector<std::string> files;
    for (int a = 3; a < argc; ++a) files.push_back(argv[a]);
    files.push_back("new_category");
    for (auto f : files) {
        for (char& c : f)
            if (c == ' ') c = '_';
        std::ifstream in(std::string(argv[1]) + "/" + f + ".fasta", std::ios::binary);
        std::cout << "file " << f << "\n"
                  << std::string(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>()) << "--\n";
    }
    return 0;
}
