/*
 * ref_driver.cpp -- a command-line front end over the reference's own CPU
 * classes, used to generate golden vectors and to time the reference CPU
 * path.  TEST INFRASTRUCTURE ONLY (built by oracle/build_ref.sh into
 * oracle/_ref/, never linked into the product).
 *
 * It calls, unmodified:
 *   HVCache (src/encoder.h:16-42): constructor (binder table), get()
 *     (= compute(), src/encoder.cpp:76-132), kmers map, precompute(),
 *     similarity()
 *   cosine (src/HV.cpp:219-242, built with NORM_COSINE like install.sh:3)
 *   make_hv-derived bases through get_base_hv (src/HV.cpp:43-51)
 *
 * Commands (sequences are read one per line from a text file):
 *   base    <out.bin>                     4 base HVs (A,C,G,T order) as uint64 words
 *   binder  <kmers.txt> <out.bin>         cache.kmers[kmer] words per line
 *   encode  <seqs.txt> <out.bin>          cache.get(seq) as int16[HV_DIM] per line
 *   windows <seqs.txt> <out.bin>          per line: (len-L)/step+1 windows (0 if len<L),
 *                                         each cache.get(seq.substr(w*step, L))
 *   precompute <seqs.txt> <out.bin>       per line: the windows that
 *                                         HVCache::precompute caches, in order
 *   topk    <queries.txt> <refs.txt> <k> <out.txt>
 *                                         encode all, brute-force cosine, order by
 *                                         (score desc, index asc); prints
 *                                         "q rank idx score(%.9g)" lines
 *   cosine  <a.bin> <b.bin> <n> <out.txt> cosine of n int16 HV pairs
 *   similarity <queries.txt> <refs.txt> <out.txt>
 *                                         cache.similarity(q, r) for every pair,
 *                                         without precompute (compute-semantics
 *                                         windows); prints "q r score(%.9g) pos"
 *   time    <queries.txt> <refs.txt> <k>  encode + brute-force top-k; prints reads/s
 */
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>
#include <algorithm>

#include "HV.h"
#include "encoder.h"

static std::vector<std::string> read_lines(const char* path) {
    std::vector<std::string> v;
    std::ifstream in(path);
    std::string line;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        v.push_back(line);
    }
    return v;
}

static void write_bin(FILE* f, const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) {
        std::perror("fwrite");
        std::exit(2);
    }
}

struct Ranked {
    float s;
    int i;
};

static void rank_topk(const HV_16& q, const std::vector<HV_16>& refs, int k, std::vector<Ranked>& out) {
    std::vector<Ranked> all(refs.size());
    for (size_t j = 0; j < refs.size(); ++j) all[j] = {cosine(q, refs[j]), (int)j};
    std::stable_sort(all.begin(), all.end(), [](const Ranked& a, const Ranked& b) { return a.s > b.s; });
    out.assign(all.begin(), all.begin() + std::min<size_t>(k, all.size()));
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <command> ...\n", argv[0]);
        return 1;
    }
    std::string cmd = argv[1];
    HVCache cache(100000);

    if (cmd == "base") {
        FILE* f = std::fopen(argv[2], "wb");
        const char bases[4] = {'A', 'C', 'G', 'T'};
        for (char b : bases) {
            const HV& hv = get_base_hv(b);
            write_bin(f, hv.data(), hv.size() * sizeof(uint64_t));
        }
        std::fclose(f);
        return 0;
    }
    if (cmd == "binder") {
        auto kmers = read_lines(argv[2]);
        FILE* f = std::fopen(argv[3], "wb");
        for (auto& km : kmers) {
            auto it = cache.kmers.find(km);
            HV hv(HV_WORDS, 0);
            if (it != cache.kmers.end()) hv = it->second;
            write_bin(f, hv.data(), hv.size() * sizeof(uint64_t));
        }
        std::fclose(f);
        return 0;
    }
    if (cmd == "encode") {
        auto seqs = read_lines(argv[2]);
        FILE* f = std::fopen(argv[3], "wb");
        for (auto& s : seqs) {
            const HV_16& hv = cache.get(s);
            write_bin(f, hv.data(), hv.size() * sizeof(int16_t));
        }
        std::fclose(f);
        return 0;
    }
    if (cmd == "windows") {
        auto seqs = read_lines(argv[2]);
        FILE* f = std::fopen(argv[3], "wb");
        for (auto& s : seqs) {
            long len = (long)s.size();
            if (len < SEQUENCE_LENGTH) continue;
            long nw = (len - SEQUENCE_LENGTH) / SIM_STEP + 1;
            for (long w = 0; w < nw; ++w) {
                const HV_16& hv = cache.get(s.substr(w * SIM_STEP, SEQUENCE_LENGTH));
                write_bin(f, hv.data(), hv.size() * sizeof(int16_t));
            }
        }
        std::fclose(f);
        return 0;
    }
    if (cmd == "precompute") {
        auto seqs = read_lines(argv[2]);
        FILE* f = std::fopen(argv[3], "wb");
        for (auto& s : seqs) {
            HVCache c2(100000);
            c2.precompute(s);
            // the cached windows are at offsets 0, step, ... while idx+L < len
            for (size_t idx = 0; idx + SEQUENCE_LENGTH <= s.size(); idx += SIM_STEP) {
                if (idx > 0 && !(idx + SEQUENCE_LENGTH < s.size())) break;
                const HV_16& hv = c2.get(s.substr(idx, SEQUENCE_LENGTH));
                write_bin(f, hv.data(), hv.size() * sizeof(int16_t));
            }
        }
        std::fclose(f);
        return 0;
    }
    if (cmd == "topk") {
        auto qs = read_lines(argv[2]);
        auto rs = read_lines(argv[3]);
        int k = std::atoi(argv[4]);
        std::vector<HV_16> refs;
        refs.reserve(rs.size());
        for (auto& r : rs) refs.push_back(cache.get(r));
        std::ofstream out(argv[5]);
        char buf[128];
        std::vector<Ranked> top;
        for (size_t qi = 0; qi < qs.size(); ++qi) {
            HV_16 q = cache.get(qs[qi]);
            rank_topk(q, refs, k, top);
            for (size_t t = 0; t < top.size(); ++t) {
                std::snprintf(buf, sizeof buf, "%zu %zu %d %.9g\n", qi, t, top[t].i, (double)top[t].s);
                out << buf;
            }
        }
        return 0;
    }
    if (cmd == "cosine") {
        int n = std::atoi(argv[4]);
        FILE* fa = std::fopen(argv[2], "rb");
        FILE* fb = std::fopen(argv[3], "rb");
        std::ofstream out(argv[5]);
        HV_16 a(HV_DIM), b(HV_DIM);
        char buf[64];
        for (int i = 0; i < n; ++i) {
            if (std::fread(a.data(), 2, HV_DIM, fa) != (size_t)HV_DIM) return 3;
            if (std::fread(b.data(), 2, HV_DIM, fb) != (size_t)HV_DIM) return 3;
            std::snprintf(buf, sizeof buf, "%.9g\n", (double)cosine(a, b));
            out << buf;
        }
        return 0;
    }
    if (cmd == "similarity") {
        auto qs = read_lines(argv[2]);
        auto rs = read_lines(argv[3]);
        std::ofstream out(argv[4]);
        char buf[128];
        for (size_t qi = 0; qi < qs.size(); ++qi)
            for (size_t ri = 0; ri < rs.size(); ++ri) {
                SIM sim = cache.similarity(qs[qi], rs[ri]);
                std::snprintf(buf, sizeof buf, "%zu %zu %.9g %zu\n", qi, ri, (double)sim.score, sim.pos);
                out << buf;
            }
        return 0;
    }
    if (cmd == "time") {
        auto qs = read_lines(argv[2]);
        auto rs = read_lines(argv[3]);
        int k = std::atoi(argv[4]);
        std::vector<HV_16> refs;
        for (auto& r : rs) refs.push_back(cache.get(r));
        std::vector<Ranked> top;
        auto t0 = std::chrono::steady_clock::now();
        long checksum = 0;
        for (auto& q : qs) {
            // distinct reads: every get() misses the LRU and runs compute()
            rank_topk(cache.get(q), refs, k, top);
            checksum += top.empty() ? 0 : top[0].i;
        }
        auto t1 = std::chrono::steady_clock::now();
        double s = std::chrono::duration<double>(t1 - t0).count();
        std::printf("%.6f %zu %ld\n", qs.size() / s, qs.size(), checksum);
        return 0;
    }
    std::fprintf(stderr, "unknown command %s\n", cmd.c_str());
    return 1;
}
