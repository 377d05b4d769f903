// Self-check driver of the GPU-backed HVCache (dropin/encoder.h), written
// against the reference's call surface only (src/encoder.h:16-42): get(),
// precompute() then get() of every window, similarity() of given pairs, and
// kmers[] of given k-mers.  Writes what they return for the parity test to
// compare with the oracle.
//   hvcache_selftest <seqs.txt> <pairs.txt> <kmers.txt> <capacity> <out_prefix>
// out_prefix.get.bin      int16 [n_seqs][HV_DIM]: get(seq), sequences in file order, twice
//                         (the second pass hits or refills the cache)
// out_prefix.windows.bin  int16 rows: for every sequence of at least one window, after
//                         precompute(seq), get() of each window 0, step, ... (x + L < len)
// out_prefix.sim.txt      "pos score" per pair line "q r" (indices into seqs)
// out_prefix.kmers.bin    uint64 [n_kmers][HV_WORDS]: kmers.at(kmer)
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "encoder.h"

static std::vector<std::string> lines(const char* path) {
    std::vector<std::string> v;
    std::ifstream in(path);
    std::string s;
    while (std::getline(in, s)) v.push_back(s);
    return v;
}

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s seqs.txt pairs.txt kmers.txt capacity out_prefix\n", argv[0]);
        return 1;
    }
    const auto seqs = lines(argv[1]);
    const auto pairs = lines(argv[2]);
    const auto kms = lines(argv[3]);
    HVCache cache((size_t)std::atoll(argv[4]));
    const std::string pre = argv[5];
    FILE* f = std::fopen((pre + ".get.bin").c_str(), "wb");
    for (int pass = 0; pass < 2; ++pass)
        for (const auto& s : seqs) {
            const HV_16& h = cache.get(s);
            std::fwrite(h.data(), 2, h.size(), f);
        }
    std::fclose(f);
    f = std::fopen((pre + ".windows.bin").c_str(), "wb");
    for (const auto& s : seqs) {
        if (s.size() < (size_t)SEQUENCE_LENGTH) continue;
        cache.precompute(s);
        for (size_t x = 0; x == 0 || x + SEQUENCE_LENGTH < s.size(); x += SIM_STEP) {
            const HV_16& h = cache.get(s.substr(x, SEQUENCE_LENGTH));
            std::fwrite(h.data(), 2, h.size(), f);
        }
    }
    std::fclose(f);
    std::ofstream sim(pre + ".sim.txt");
    char buf[64];
    for (const auto& p : pairs) {
        const size_t sp = p.find(' ');
        const SIM r = cache.similarity(seqs.at(std::stoul(p.substr(0, sp))), seqs.at(std::stoul(p.substr(sp + 1))));
        std::snprintf(buf, sizeof buf, "%zu %.9g\n", r.pos, (double)r.score);
        sim << buf;
    }
    f = std::fopen((pre + ".kmers.bin").c_str(), "wb");
    for (const auto& k : kms) {
        const HV& h = cache.kmers.at(k);
        std::fwrite(h.data(), 8, h.size(), f);
    }
    std::fclose(f);
    std::printf("kmers %zu\n", cache.kmers.size());
    return 0;
}
