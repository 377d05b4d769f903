// Self-check driver of the GPU.cuh drop-in, written against the reference's
// call surface only: reads sequences (one per line) from argv[1], calls
// encode(kmer_map, sequences) and cosine_search(inputs, db, k) the way
// tests/cosine_comparison_test.cpp:74-133 does (inputs = first window of each
// sequence of the first half, db = every window of the second half), and
// writes the window hypervectors and the ranked matches as text for the
// parity test to compare with the oracle.
//   selftest <seqs.txt> <k> <out_windows.bin> <out_matches.txt>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <unordered_map>

#include "GPU.cuh"

int main(int argc, char** argv) {
    if (argc != 5) {
        std::fprintf(stderr, "usage: %s seqs.txt k windows.bin matches.txt\n", argv[0]);
        return 1;
    }
    std::vector<std::string> seqs;
    {
        std::ifstream in(argv[1]);
        std::string line;
        while (std::getline(in, line)) seqs.push_back(line);
    }
    const int k = std::atoi(argv[2]);
    std::vector<int16_t> kmer_map;  // not read by the drop-in
    auto hvs = encode(kmer_map, seqs);
    FILE* f = std::fopen(argv[3], "wb");
    for (auto& s : hvs)
        for (auto& w : s) std::fwrite(w.data(), 2, w.size(), f);
    std::fclose(f);
    const size_t half = hvs.size() / 2;
    std::vector<HV_16*> inputs, db;
    std::unordered_map<HV_16*, size_t> db_index;
    for (size_t i = 0; i < half; ++i)
        if (!hvs[i].empty()) inputs.push_back(&hvs[i][0]);
    for (size_t i = half; i < hvs.size(); ++i)
        for (auto& w : hvs[i]) {
            db_index[&w] = db.size();
            db.push_back(&w);
        }
    auto res = cosine_search(inputs, db, k);
    std::ofstream out(argv[4]);
    char buf[96];
    for (size_t q = 0; q < inputs.size(); ++q) {
        const auto& m = res.at(inputs[q]);
        for (size_t r = 0; r < m.size(); ++r) {
            std::snprintf(buf, sizeof buf, "%zu %zu %zu %.9g\n", q, r, db_index.at(m[r].second), (double)m[r].first);
            out << buf;
        }
    }
    return 0;
}
