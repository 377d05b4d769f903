// Seeded synthetic taxonomy trees, noisy copies and reads (include/hdc_synth.h).
#include "hdc_synth.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <string>
#include <thread>
#include <vector>

namespace {

const char kBases[4] = {'A', 'C', 'G', 'T'};

uint64_t splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ULL;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ULL;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBULL;
    return x ^ (x >> 31);
}

// independent stream for item (a, b) of a generator seeded with `seed`
std::mt19937_64 stream(uint64_t seed, uint64_t a, uint64_t b) {
    return std::mt19937_64(splitmix64(splitmix64(seed ^ splitmix64(a + 1)) ^ (b * 0xD1B54A32D192ED03ULL)));
}

uint64_t threshold(double p) {
    if (p <= 0) return 0;
    if (p >= 1) return ~0ULL;
    return (uint64_t)(p * 18446744073709551616.0);
}

char other_base(char c, uint64_t r) {
    int code = c == 'A' ? 0 : c == 'C' ? 1 : c == 'G' ? 2 : 3;
    return kBases[(code + 1 + (int)(r % 3)) & 3];
}

void substitute(std::string& s, double p, std::mt19937_64& g) {
    const uint64_t t = threshold(p);
    for (char& c : s)
        if (g() < t) c = other_base(c, g());
}

void insert_random(std::string& s, std::mt19937_64& g) {
    size_t pos = g() % (s.size() + 1);
    s.insert(s.begin() + pos, kBases[g() & 3]);
}

void delete_random(std::string& s, std::mt19937_64& g) {
    if (s.empty()) return;
    s.erase(s.begin() + g() % s.size());
}

template <typename F>
void parallel_for(int64_t n, int threads, F&& fn) {
    threads = std::max(1, std::min<int>(threads, (int)std::min<int64_t>(n, 256)));
    if (threads <= 1) {
        for (int64_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::vector<std::thread> th;
    for (int t = 0; t < threads; ++t)
        th.emplace_back([&, t] {
            for (int64_t i = t; i < n; i += threads) fn(i);
        });
    for (auto& x : th) x.join();
}

int emit(const std::vector<std::string>& v, char* buf, int64_t cap, int64_t* off, int32_t* len) {
    int64_t pos = 0;
    for (size_t i = 0; i < v.size(); ++i) {
        if (pos + (int64_t)v[i].size() > cap) return -1;
        std::memcpy(buf + pos, v[i].data(), v[i].size());
        off[i] = pos;
        len[i] = (int32_t)v[i].size();
        pos += (int64_t)v[i].size();
    }
    return 0;
}

int hw_threads(int t) { return t > 0 ? t : (int)std::max(1u, std::thread::hardware_concurrency()); }

}  // namespace

extern "C" {

int hdc_synth_tree(uint64_t seed, int64_t n_leaves, int root_len, const double* subst, int jitter, int min_len,
                   int max_len, char* buf, int64_t buf_cap, int64_t* off, int32_t* len, int64_t* nodes_per_rank,
                   int threads) {
    if (n_leaves < 1 || root_len < 1 || !subst || jitter < 0 || min_len > max_len || !buf || !off || !len) return -1;
    threads = hw_threads(threads);
    int64_t b = 1;
    while (true) {  // smallest b with b^6 >= n_leaves
        int64_t p = 1;
        for (int i = 0; i < 6; ++i) p *= b;
        if (p >= n_leaves) break;
        ++b;
    }
    std::vector<int64_t> count(7);
    for (int r = 0; r <= 6; ++r) {
        int64_t d = 1;
        for (int i = r; i < 6; ++i) d *= b;
        count[r] = (n_leaves + d - 1) / d;
    }
    if (nodes_per_rank)
        for (int r = 0; r <= 6; ++r) nodes_per_rank[r] = count[r];
    std::vector<std::string> level(1);
    {
        auto g = stream(seed, 0, 0);
        level[0].resize(root_len);
        for (char& c : level[0]) c = kBases[g() & 3];
    }
    for (int r = 1; r <= 6; ++r) {
        std::vector<std::string> next(count[r]);
        parallel_for(count[r], threads, [&](int64_t j) {
            auto g = stream(seed, (uint64_t)r, (uint64_t)j);
            std::string s = level[j / b];
            substitute(s, subst[r - 1], g);
            const int delta = (int)(g() % (uint64_t)(2 * jitter + 1)) - jitter;
            for (int i = 0; i < delta; ++i) insert_random(s, g);
            for (int i = 0; i < -delta; ++i) delete_random(s, g);
            if (r == 6) {
                while ((int)s.size() < min_len) insert_random(s, g);
                while ((int)s.size() > max_len) delete_random(s, g);
            }
            next[j] = std::move(s);
        });
        level.swap(next);
    }
    return emit(level, buf, buf_cap, off, len);
}

int hdc_synth_copies(uint64_t seed, const char* src, const int64_t* src_off, const int32_t* src_len, int64_t n_src,
                     int n_copies, double subst, char* buf, int64_t buf_cap, int64_t* off, int32_t* len,
                     int threads) {
    if (n_src < 0 || n_copies < 1 || !src || !buf || !off || !len) return -1;
    std::vector<std::string> out(n_src * n_copies);
    parallel_for(n_src * n_copies, hw_threads(threads), [&](int64_t t) {
        const int64_t i = t / n_copies, c = t % n_copies;
        auto g = stream(seed, (uint64_t)i, (uint64_t)c);
        std::string s(src + src_off[i], src_len[i]);
        substitute(s, subst, g);
        out[t] = std::move(s);
    });
    return emit(out, buf, buf_cap, off, len);
}

int hdc_synth_reads(uint64_t seed, const char* src, const int64_t* src_off, const int32_t* src_len, int64_t n_src,
                    int64_t n_reads, int read_len, double sigma, int min_read, int max_read, double subst,
                    double mixed_frac, double mixed_rate, char* buf, int64_t buf_cap, int64_t* off, int32_t* len,
                    int32_t* label, int threads) {
    if (n_src < 1 || n_reads < 0 || read_len < 1 || !src || !buf || !off || !len) return -1;
    std::vector<std::string> out(n_reads);
    const uint64_t t_mixed = threshold(mixed_frac), t_err = threshold(mixed_rate);
    parallel_for(n_reads, hw_threads(threads), [&](int64_t i) {
        auto g = stream(seed, (uint64_t)i, 0x5EEDULL);
        const int64_t si = (int64_t)(g() % (uint64_t)n_src);
        if (label) label[i] = (int32_t)si;
        int L = read_len;
        if (sigma > 0) {
            // Box-Muller from two 53-bit uniforms
            const double u1 = ((g() >> 11) + 1.0) * (1.0 / 9007199254740993.0);
            const double u2 = (g() >> 11) * (1.0 / 9007199254740992.0);
            const double z = std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
            L = (int)std::lround(read_len * std::exp(sigma * z));
            L = std::min(std::max(L, min_read), max_read);
        }
        L = std::min(L, (int)src_len[si]);
        const int64_t start = (int64_t)(g() % (uint64_t)(src_len[si] - L + 1));
        std::string s(src + src_off[si] + start, L);
        if (g() < t_mixed) {
            std::string e;
            e.reserve(L + L / 8 + 4);
            for (char c : s) {
                if (g() < t_err) {
                    const uint64_t kind = g() % 5;  // substitution : insertion : deletion = 3 : 1 : 1
                    if (kind < 3)
                        e.push_back(other_base(c, g()));
                    else if (kind == 3) {
                        e.push_back(kBases[g() & 3]);
                        e.push_back(c);
                    }  // kind 4: deletion
                } else {
                    e.push_back(c);
                }
            }
            s.swap(e);
        } else {
            substitute(s, subst, g);
        }
        out[i] = std::move(s);
    });
    return emit(out, buf, buf_cap, off, len);
}

}  // extern "C"
