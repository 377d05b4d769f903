/*
 * hdc_oracle.c -- CPU oracle for the k-mer hypervector encode / cosine top-k /
 * propagate-children path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only the test suite,
 * the smoke check and the CPU-baseline leg of the benchmark load it.  The
 * product library never links or calls it.
 *
 * It is a plain C restatement of the reference's CPU algorithm (citations are
 * to files of benlaflen/bacterial-classification):
 *
 *   base hypervectors   src/HV.cpp:20-41 (make_hv: mt19937_64(seed), one draw
 *                       per 64-bit word, tail bits masked; A,C,T,G use seeds
 *                       0,1,2,3; src/HV.cpp:43-51 get_base_hv)
 *   permute + bind      src/HV.cpp:98-147 (mult: out_j = l_j ^ r_{(j+s) mod 64W})
 *   k-mer binder        src/encoder.cpp:47-74 (canonical = min(s, revcomp(s)) in
 *                       std::string order; binder = ~0 ^ rot_0(b0) ^ ... ^
 *                       rot_{k-1}(b_{k-1}) over the canonical k-mer's bases)
 *   bundle              src/HV.cpp:156-216 (superpose_batch: +1 per set bit,
 *                       -1 per clear bit, int16 accumulator)
 *   sequence encode     src/encoder.cpp:106-132 (HVCache::compute: every k-mer
 *                       position 0..len-k, k-mers holding a byte outside
 *                       "ACGT" are skipped)
 *   cosine              src/HV.cpp:219-252 (int64 dot and norms; NORM_COSINE
 *                       returns float(2*(dot/(sqrt(nl)*sqrt(nr)) - 0.5)), -1 when
 *                       a norm is zero; without NORM_COSINE returns float(dot))
 *   greedy propagate    targets/propogate-children.cpp:60-73
 *
 * The mt19937_64 generator below follows the published MT19937-64 algorithm
 * (Matsumoto & Nishimura), whose parameters the C++ standard fixes for
 * std::mt19937_64.
 *
 * Ranking rule used everywhere: descending float score, ties broken by the
 * lower reference index (the first maximum wins, as in the reference's
 * brute-force CPU argmax, tests/cosine_comparison_test.cpp:146-156).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* MT19937-64                                                          */
/* ------------------------------------------------------------------ */
#define MT_N 312
#define MT_M 156
#define MT_A 0xB5026F5AA96619E9ULL
#define MT_UPPER 0xFFFFFFFF80000000ULL
#define MT_LOWER 0x000000007FFFFFFFULL

typedef struct {
    uint64_t s[MT_N];
    int i;
} orc_mt64;

static void mt_seed(orc_mt64* g, uint64_t seed) {
    g->s[0] = seed;
    for (int i = 1; i < MT_N; ++i)
        g->s[i] = 6364136223846793005ULL * (g->s[i - 1] ^ (g->s[i - 1] >> 62)) + (uint64_t)i;
    g->i = MT_N;
}

static uint64_t mt_next(orc_mt64* g) {
    if (g->i >= MT_N) {
        for (int j = 0; j < MT_N; ++j) {
            uint64_t y = (g->s[j] & MT_UPPER) | (g->s[(j + 1) % MT_N] & MT_LOWER);
            uint64_t v = g->s[(j + MT_M) % MT_N] ^ (y >> 1);
            if (y & 1ULL) v ^= MT_A;
            g->s[j] = v;
        }
        g->i = 0;
    }
    uint64_t x = g->s[g->i++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= (x >> 43);
    return x;
}

/* First n outputs of mt19937_64(seed); used to pin the generator. */
void orc_mt64_stream(uint64_t seed, int n, uint64_t* out) {
    orc_mt64 g;
    mt_seed(&g, seed);
    for (int i = 0; i < n; ++i) out[i] = mt_next(&g);
}

/* ------------------------------------------------------------------ */
/* Hypervector primitives                                              */
/* ------------------------------------------------------------------ */
static int words64(int dim) { return (dim + 63) / 64; }

static uint64_t tail_mask(int dim) {
    int excess = words64(dim) * 64 - dim;
    return excess ? (~0ULL >> excess) : ~0ULL;
}

/* code: A=0 C=1 G=2 T=3 (std::string order); anything else is invalid. */
static int base_code(char c) {
    switch (c) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return -1;
    }
}

/* Seeds per code, from get_base_hv: A->0, C->1, G->3, T->2. */
static const int SEED_OF_CODE[4] = {0, 1, 3, 2};

/* out: [4][W] words, indexed by base code (A,C,G,T). */
int orc_base_hvs(int dim, uint64_t* out) {
    int W = words64(dim);
    for (int c = 0; c < 4; ++c) {
        orc_mt64 g;
        mt_seed(&g, (uint64_t)SEED_OF_CODE[c]);
        for (int w = 0; w < W; ++w) out[c * W + w] = mt_next(&g);
        out[c * W + W - 1] &= tail_mask(dim);
    }
    return W;
}

/* mult(l, r, out, s): out_j = l_j ^ r_{(j+s) mod 64W} for s < 64, tail masked. */
static void mult(const uint64_t* l, const uint64_t* r, uint64_t* out, int W, int s, uint64_t tmask) {
    uint64_t tmp[W];
    for (int w = 0; w < W; ++w) {
        uint64_t rw;
        if (s == 0)
            rw = r[w];
        else
            rw = (r[w] >> s) | (r[(w + 1) % W] << (64 - s));
        tmp[w] = l[w] ^ rw;
    }
    memcpy(out, tmp, sizeof(uint64_t) * (size_t)W);
    out[W - 1] &= tmask;
}

/* Lexicographic code of a k-mer (first base most significant), or -1. */
static int64_t lex_code(const char* s, int k) {
    int64_t v = 0;
    for (int i = 0; i < k; ++i) {
        int c = base_code(s[i]);
        if (c < 0) return -1;
        v = (v << 2) | c;
    }
    return v;
}

/* canonical = min(s, revcomp(s)) under std::string ordering (A<C<G<T). */
int64_t orc_canonical(const char* kmer, int k) {
    int64_t f = lex_code(kmer, k);
    if (f < 0) return -1;
    int64_t r = 0;
    for (int i = k - 1; i >= 0; --i) r = (r << 2) | (3 - base_code(kmer[i]));
    return f < r ? f : r;
}

/* binder of a canonical k-mer code: start from all-ones, then mult by the
 * base of digit i rotated by i, for i = 0 (first base) .. k-1. */
void orc_binder(int dim, int k, int64_t canon, uint64_t* out) {
    int W = words64(dim);
    uint64_t tm = tail_mask(dim);
    uint64_t* base = (uint64_t*)malloc(sizeof(uint64_t) * 4 * (size_t)W);
    orc_base_hvs(dim, base);
    for (int w = 0; w < W; ++w) out[w] = ~0ULL;
    out[W - 1] &= tm;
    for (int i = 0; i < k; ++i) {
        int c = (int)((canon >> (2 * (k - 1 - i))) & 3);
        mult(out, base + (size_t)c * W, out, W, i, tm);
    }
    free(base);
}

/* Rotated base table R[i][c][W] = rot_i(base[c]); lets a binder be built as
 * ~0 ^ XOR_i R[i][c_i] (equal to the chain of mult calls: each output bit
 * depends only on the same bit of l, and the tail is masked at the end). */
typedef struct {
    int dim, k, W;
    uint64_t tmask;
    uint64_t* rot; /* [k][4][W] */
} orc_tables;

static void tables_init(orc_tables* t, int dim, int k) {
    t->dim = dim;
    t->k = k;
    t->W = words64(dim);
    t->tmask = tail_mask(dim);
    uint64_t* base = (uint64_t*)malloc(sizeof(uint64_t) * 4 * (size_t)t->W);
    orc_base_hvs(dim, base);
    t->rot = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)k * 4 * (size_t)t->W);
    uint64_t* zero = (uint64_t*)calloc((size_t)t->W, sizeof(uint64_t));
    for (int i = 0; i < k; ++i)
        for (int c = 0; c < 4; ++c)
            mult(zero, base + (size_t)c * t->W, t->rot + ((size_t)i * 4 + c) * t->W, t->W, i, ~0ULL);
    free(zero);
    free(base);
}

static void tables_free(orc_tables* t) { free(t->rot); }

static void tables_binder(const orc_tables* t, int64_t canon, uint64_t* out) {
    int W = t->W, k = t->k;
    for (int w = 0; w < W; ++w) out[w] = ~0ULL;
    for (int i = 0; i < k; ++i) {
        int c = (int)((canon >> (2 * (k - 1 - i))) & 3);
        const uint64_t* r = t->rot + ((size_t)i * 4 + c) * W;
        for (int w = 0; w < W; ++w) out[w] ^= r[w];
    }
    out[W - 1] &= t->tmask;
}

/* HVCache::compute: counts in int32, returned modulo 2^16 like the int16
 * accumulator of superpose_batch.  Returns the number of k-mers bundled. */
static int64_t encode_one(const orc_tables* t, const char* seq, int64_t len, int32_t* acc, uint64_t* scratch) {
    int dim = t->dim, k = t->k;
    memset(acc, 0, sizeof(int32_t) * (size_t)dim);
    int64_t n = 0;
    for (int64_t p = 0; p + k <= len; ++p) {
        int64_t canon = orc_canonical(seq + p, k);
        if (canon < 0) continue;
        tables_binder(t, canon, scratch);
        for (int d = 0; d < dim; ++d) acc[d] += ((scratch[d >> 6] >> (d & 63)) & 1ULL) ? 1 : -1;
        ++n;
    }
    return n;
}

/* Encode one sequence (whole-sequence semantics) into int16[dim]. */
int64_t orc_encode(int dim, int k, const char* seq, int64_t len, int16_t* out) {
    orc_tables t;
    tables_init(&t, dim, k);
    int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)t.W);
    int64_t n = encode_one(&t, seq, len, acc, tmp);
    for (int d = 0; d < dim; ++d) out[d] = (int16_t)(uint16_t)(uint32_t)acc[d];
    free(tmp);
    free(acc);
    tables_free(&t);
    return n;
}

/* ------------------------------------------------------------------ */
/* Threaded batch helpers                                              */
/* ------------------------------------------------------------------ */
typedef struct {
    const orc_tables* t;
    const char* buf;
    const int64_t* off; /* segment starts */
    const int64_t* len; /* segment lengths */
    int64_t n;
    int out_kind; /* 0: int16 counts, 1: int32 counts, 2: bipolar int8 (ties -> +1) */
    void* out;
    int64_t* nk;
    int tid, nthreads;
} enc_job;

static void* enc_worker(void* arg) {
    enc_job* j = (enc_job*)arg;
    int dim = j->t->dim;
    int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)j->t->W);
    for (int64_t s = j->tid; s < j->n; s += j->nthreads) {
        int64_t n = encode_one(j->t, j->buf + j->off[s], j->len[s], acc, tmp);
        if (j->nk) j->nk[s] = n;
        if (j->out_kind == 0) {
            int16_t* o = (int16_t*)j->out + (size_t)s * dim;
            for (int d = 0; d < dim; ++d) o[d] = (int16_t)(uint16_t)(uint32_t)acc[d];
        } else if (j->out_kind == 1) {
            memcpy((int32_t*)j->out + (size_t)s * dim, acc, sizeof(int32_t) * (size_t)dim);
        } else {
            int8_t* o = (int8_t*)j->out + (size_t)s * dim;
            for (int d = 0; d < dim; ++d) o[d] = acc[d] >= 0 ? 1 : -1;
        }
    }
    free(tmp);
    free(acc);
    return NULL;
}

/* Encode n segments buf[off[i] .. off[i]+len[i]) (whole-segment semantics). */
int orc_encode_segments(int dim, int k, const char* buf, const int64_t* off, const int64_t* len, int64_t n,
                        int out_kind, void* out, int64_t* nk, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    orc_tables t;
    tables_init(&t, dim, k);
    pthread_t th[256];
    enc_job jobs[256];
    if (nthreads > 256) nthreads = 256;
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (enc_job){&t, buf, off, len, n, out_kind, out, nk, i, nthreads};
        pthread_create(&th[i], NULL, enc_worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    tables_free(&t);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Fast CPU encoder for building large reference sets (the CPU-baseline  */
/* database).  Same result as encode_one, checked bit for bit by the     */
/* tests: binder words from per-part tables of pre-rotated, pre-XORed    */
/* base fragments (parts of <= 4 digits), counts in 64-bit bit-sliced    */
/* counters (ripple-carry add of each binder word).  Not used to time    */
/* the reference path, which is encode_one.                              */
/* ------------------------------------------------------------------ */
typedef struct {
    int dim, k, W, np;
    int first[4], len[4];
    uint64_t* tab[4]; /* [4^len][W] */
} fast_tables;

static void fast_init(fast_tables* f, const orc_tables* t) {
    f->dim = t->dim;
    f->k = t->k;
    f->W = t->W;
    f->np = (t->k + 3) / 4;
    int first = 0;
    for (int p = 0; p < f->np; ++p) {
        int len = t->k / f->np + (p < t->k % f->np ? 1 : 0);
        f->first[p] = first;
        f->len[p] = len;
        int rows = 1 << (2 * len);
        f->tab[p] = (uint64_t*)calloc((size_t)rows * f->W, sizeof(uint64_t));
        for (int r = 0; r < rows; ++r) {
            uint64_t* o = f->tab[p] + (size_t)r * f->W;
            if (p == 0)
                for (int w = 0; w < f->W; ++w) o[w] = ~0ULL;
            for (int d = 0; d < len; ++d) {
                int c = (r >> (2 * (len - 1 - d))) & 3;
                const uint64_t* rot = t->rot + ((size_t)(first + d) * 4 + c) * f->W;
                for (int w = 0; w < f->W; ++w) o[w] ^= rot[w];
            }
        }
        first += len;
    }
}

static void fast_free(fast_tables* f) {
    for (int p = 0; p < f->np; ++p) free(f->tab[p]);
}

/* ripple-carry add of one binder's bits into a bit-sliced counter */
static void planes_add(uint64_t* planes, int nplanes, int W, const uint64_t* word) {
    for (int w = 0; w < W; ++w) {
        uint64_t c = word[w];
        for (int b = 0; b < nplanes && c; ++b) {
            uint64_t t = planes[(size_t)b * W + w] & c;
            planes[(size_t)b * W + w] ^= c;
            c = t;
        }
    }
}

/* the binder of canonical k-mer code `canon` from the fragment tables */
static void fast_binder(const fast_tables* f, int64_t canon, uint64_t* word) {
    const int W = f->W, k = f->k;
    const uint64_t* rows[4];
    for (int q = 0; q < f->np; ++q) {
        int shift = 2 * (k - f->first[q] - f->len[q]);
        rows[q] = f->tab[q] + (size_t)((canon >> shift) & ((1 << (2 * f->len[q])) - 1)) * W;
    }
    for (int w = 0; w < W; ++w) {
        uint64_t x = rows[0][w];
        for (int q = 1; q < f->np; ++q) x ^= rows[q][w];
        word[w] = x;
    }
}

/* value of element d of a bit-sliced counter */
static int32_t planes_get(const uint64_t* planes, int nplanes, int W, int d) {
    int32_t c = 0;
    for (int b = 0; b < nplanes; ++b) c |= (int32_t)((planes[(size_t)b * W + (d >> 6)] >> (d & 63)) & 1) << b;
    return c;
}

/* counts[d] for d < dim into acc (int32), returns the number of k-mers */
static int64_t fast_encode_one(const fast_tables* f, const char* seq, int64_t len, int32_t* acc, uint64_t* planes,
                               int nplanes, uint64_t* word) {
    const int W = f->W, k = f->k;
    memset(planes, 0, sizeof(uint64_t) * (size_t)nplanes * W);
    int64_t n = 0;
    for (int64_t p = 0; p + k <= len; ++p) {
        int64_t canon = orc_canonical(seq + p, k);
        if (canon < 0) continue;
        fast_binder(f, canon, word);
        planes_add(planes, nplanes, W, word);
        ++n;
    }
    for (int d = 0; d < f->dim; ++d) acc[d] = 2 * planes_get(planes, nplanes, W, d) - (int32_t)n;
    return n;
}

typedef struct {
    const fast_tables* f;
    const char* buf;
    const int64_t *off, *len;
    int64_t n;
    int group; /* rows summed per output row (bundles of noisy copies) */
    int32_t* out;
    int tid, nthreads;
} fast_job;

static void* fast_worker(void* arg) {
    fast_job* j = (fast_job*)arg;
    const int dim = j->f->dim, W = j->f->W;
    const int nplanes = 17;
    int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    uint64_t* planes = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)nplanes * W);
    uint64_t* word = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)W);
    const int64_t nout = j->n / j->group;
    for (int64_t o = j->tid; o < nout; o += j->nthreads) {
        int32_t* dst = j->out + (size_t)o * dim;
        memset(dst, 0, sizeof(int32_t) * (size_t)dim);
        for (int g = 0; g < j->group; ++g) {
            int64_t s = o * j->group + g;
            fast_encode_one(j->f, j->buf + j->off[s], j->len[s], acc, planes, nplanes, word);
            for (int d = 0; d < dim; ++d) dst[d] += acc[d];
        }
    }
    free(word);
    free(planes);
    free(acc);
    return NULL;
}

/* Encode n segments (exact int32 counts; segments of < 2^17 k-mers) and sum
 * them in consecutive groups of `group` into out [n/group][dim]. */
int orc_encode_bundles(int dim, int k, const char* buf, const int64_t* off, const int64_t* len, int64_t n, int group,
                       int32_t* out, int nthreads) {
    if (group < 1 || n % group) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    orc_tables t;
    tables_init(&t, dim, k);
    fast_tables f;
    fast_init(&f, &t);
    pthread_t th[256];
    fast_job jobs[256];
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (fast_job){&f, buf, off, len, n, group, out, i, nthreads};
        pthread_create(&th[i], NULL, fast_worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    fast_free(&f);
    tables_free(&t);
    return 0;
}

/* Bundles of noisy copies, computed from differences (test infrastructure:
 * builds the same rows as orc_encode_bundles on the copies, faster).
 * out[i] = sum over c < group of encode(copy[i * group + c]).  A copy of the
 * same length as its source leaf differs from it only in the k-mers that
 * overlap a changed base, so
 *   count_bits(bundle) = group * bits(leaf) + bits(new k-mers) - bits(old k-mers)
 *   n_kmers(bundle)    = group * n(leaf)    + n(new)           - n(old)
 * and element d is 2 * count_bits[d] - n_kmers (the HVCache::compute sum,
 * src/encoder.cpp:106-132, over every copy).  A copy whose length differs is
 * encoded whole.  Three bit-sliced counters (leaf, added, removed). */
typedef struct {
    const fast_tables* f;
    const char *leaf_buf, *copy_buf;
    const int64_t *leaf_off, *leaf_len, *copy_off, *copy_len;
    int64_t n_leaves;
    int group;
    int32_t* out;
    int tid, nthreads;
} delta_job;

static void* delta_worker(void* arg) {
    delta_job* j = (delta_job*)arg;
    const fast_tables* f = j->f;
    const int dim = f->dim, W = f->W, k = f->k, np = 17;
    uint64_t* pl = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)np * W);
    uint64_t* pa = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)np * W);
    uint64_t* ps = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)np * W);
    uint64_t* word = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)W);
    int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    int64_t cap = 0;
    uint8_t* mark = NULL;
    for (int64_t i = j->tid; i < j->n_leaves; i += j->nthreads) {
        const char* leaf = j->leaf_buf + j->leaf_off[i];
        const int64_t L = j->leaf_len[i];
        if (L + 1 > cap) {
            cap = L + 1;
            mark = (uint8_t*)realloc(mark, (size_t)cap);
        }
        memset(pl, 0, sizeof(uint64_t) * (size_t)np * W);
        memset(pa, 0, sizeof(uint64_t) * (size_t)np * W);
        memset(ps, 0, sizeof(uint64_t) * (size_t)np * W);
        int64_t n_leaf = 0, n_add = 0, n_sub = 0;
        for (int64_t p = 0; p + k <= L; ++p) {
            int64_t c = orc_canonical(leaf + p, k);
            if (c < 0) continue;
            fast_binder(f, c, word);
            planes_add(pl, np, W, word);
            ++n_leaf;
        }
        for (int g = 0; g < j->group; ++g) {
            const int64_t s = i * j->group + g;
            const char* cp = j->copy_buf + j->copy_off[s];
            const int64_t CL = j->copy_len[s];
            if (CL != L) { /* not a substitution-only copy: encode it whole */
                for (int64_t p = 0; p + k <= CL; ++p) {
                    int64_t c = orc_canonical(cp + p, k);
                    if (c < 0) continue;
                    fast_binder(f, c, word);
                    planes_add(pa, np, W, word);
                    ++n_add;
                }
                /* the leaf term counted this copy as the leaf: take one leaf back out */
                for (int64_t p = 0; p + k <= L; ++p) {
                    int64_t c = orc_canonical(leaf + p, k);
                    if (c < 0) continue;
                    fast_binder(f, c, word);
                    planes_add(ps, np, W, word);
                }
                n_sub += n_leaf;
                continue;
            }
            memset(mark, 0, (size_t)cap);
            for (int64_t b = 0; b < L; ++b) {
                if (cp[b] == leaf[b]) continue;
                const int64_t lo = b - k + 1 > 0 ? b - k + 1 : 0;
                for (int64_t p = lo; p <= b && p + k <= L; ++p) mark[p] = 1;
            }
            for (int64_t p = 0; p + k <= L; ++p) {
                if (!mark[p]) continue;
                int64_t co = orc_canonical(leaf + p, k), cn = orc_canonical(cp + p, k);
                if (co >= 0) {
                    fast_binder(f, co, word);
                    planes_add(ps, np, W, word);
                    ++n_sub;
                }
                if (cn >= 0) {
                    fast_binder(f, cn, word);
                    planes_add(pa, np, W, word);
                    ++n_add;
                }
            }
        }
        const int64_t n_tot = (int64_t)j->group * n_leaf + n_add - n_sub;
        int32_t* dst = j->out + (size_t)i * dim;
        for (int d = 0; d < dim; ++d) {
            const int64_t bits = (int64_t)j->group * planes_get(pl, np, W, d) + planes_get(pa, np, W, d) -
                                 planes_get(ps, np, W, d);
            dst[d] = (int32_t)(2 * bits - n_tot);
        }
    }
    free(mark);
    free(acc);
    free(word);
    free(ps);
    free(pa);
    free(pl);
    return NULL;
}

int orc_encode_copy_bundles(int dim, int k, const char* leaf_buf, const int64_t* leaf_off, const int64_t* leaf_len,
                            int64_t n_leaves, const char* copy_buf, const int64_t* copy_off, const int64_t* copy_len,
                            int group, int32_t* out, int nthreads) {
    if (group < 1) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    orc_tables t;
    tables_init(&t, dim, k);
    fast_tables f;
    fast_init(&f, &t);
    pthread_t th[256];
    delta_job jobs[256];
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (delta_job){&f, leaf_buf, copy_buf, leaf_off, leaf_len, copy_off, copy_len, n_leaves, group, out, i,
                              nthreads};
        pthread_create(&th[i], NULL, delta_worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    fast_free(&f);
    tables_free(&t);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Cosine and ranking                                                  */
/* ------------------------------------------------------------------ */
enum { ORC_SCORE_NORM = 0, ORC_SCORE_COS = 1, ORC_SCORE_DOT = 2 };

/* Score from exact integer dot and squared norms. */
static float score_from(int64_t dot, int64_t nl, int64_t nr, int mode) {
    if (mode == ORC_SCORE_DOT) return (float)dot;
    if (nl == 0 || nr == 0) return -1.0f;
    double c = (double)dot / (sqrt((double)nl) * sqrt((double)nr));
    if (mode == ORC_SCORE_NORM) return (float)(2.0 * (c - 0.5));
    return (float)c;
}

static double cos_from(int64_t dot, int64_t nl, int64_t nr) {
    if (nl == 0 || nr == 0) return 0.0;
    return (double)dot / (sqrt((double)nl) * sqrt((double)nr));
}

/* The reference float score for given exact dots and squared norms (vectorised). */
void orc_scores_from(const int64_t* dot, const int64_t* nl, const int64_t* nr, int64_t n, int mode, float* out) {
    for (int64_t i = 0; i < n; ++i) out[i] = score_from(dot[i], nl[i], nr[i], mode);
}

float orc_cosine_i32(const int32_t* l, const int32_t* r, int dim, int mode) {
    int64_t dot = 0, nl = 0, nr = 0;
    for (int i = 0; i < dim; ++i) {
        int64_t a = l[i], b = r[i];
        dot += a * b;
        nl += a * a;
        nr += b * b;
    }
    return score_from(dot, nl, nr, mode);
}

/* ordering key: larger is better; score descending then index ascending */
static int better(float sa, int32_t ia, float sb, int32_t ib) {
    if (sa != sb) return sa > sb;
    return ia < ib;
}

typedef struct {
    const int32_t *q, *r;
    const int64_t *qn, *rn;
    int64_t nq, nr;
    int dim, k, mode;
    float* out_s;
    int32_t* out_i;
    double* out_c;
    int64_t* out_dot;
    int tid, nthreads;
} topk_job;

static void* topk_worker(void* arg) {
    topk_job* j = (topk_job*)arg;
    int k = j->k, dim = j->dim;
    float* bs = (float*)malloc(sizeof(float) * (size_t)k);
    int32_t* bi = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int64_t* bd = (int64_t*)malloc(sizeof(int64_t) * (size_t)k);
    for (int64_t qi = j->tid; qi < j->nq; qi += j->nthreads) {
        const int32_t* q = j->q + (size_t)qi * dim;
        int filled = 0;
        for (int64_t ri = 0; ri < j->nr; ++ri) {
            const int32_t* r = j->r + (size_t)ri * dim;
            int64_t dot = 0;
            for (int d = 0; d < dim; ++d) dot += (int64_t)q[d] * (int64_t)r[d];
            float s = score_from(dot, j->qn[qi], j->rn[ri], j->mode);
            if (filled == k && !better(s, (int32_t)ri, bs[k - 1], bi[k - 1])) continue;
            int pos = filled < k ? filled : k - 1;
            while (pos > 0 && better(s, (int32_t)ri, bs[pos - 1], bi[pos - 1])) {
                bs[pos] = bs[pos - 1];
                bi[pos] = bi[pos - 1];
                bd[pos] = bd[pos - 1];
                --pos;
            }
            bs[pos] = s;
            bi[pos] = (int32_t)ri;
            bd[pos] = dot;
            if (filled < k) ++filled;
        }
        for (int t = 0; t < k; ++t) {
            int ok = t < filled;
            j->out_s[qi * k + t] = ok ? bs[t] : -INFINITY;
            j->out_i[qi * k + t] = ok ? bi[t] : -1;
            if (j->out_c) j->out_c[qi * k + t] = ok ? cos_from(bd[t], j->qn[qi], j->rn[bi[t]]) : 0.0;
            if (j->out_dot) j->out_dot[qi * k + t] = ok ? bd[t] : 0;
        }
    }
    free(bd);
    free(bi);
    free(bs);
    return NULL;
}

static void norms_i32(const int32_t* v, int64_t n, int dim, int64_t* out) {
    for (int64_t i = 0; i < n; ++i) {
        int64_t s = 0;
        for (int d = 0; d < dim; ++d) s += (int64_t)v[(size_t)i * dim + d] * v[(size_t)i * dim + d];
        out[i] = s;
    }
}

/* Brute-force top-k of every query against every reference. */
int orc_topk_i32(const int32_t* q, int64_t nq, const int32_t* r, int64_t nr, int dim, int k, int mode,
                 float* out_s, int32_t* out_i, double* out_c, int64_t* out_dot, int nthreads) {
    if (k < 1) return -1;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    int64_t* qn = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nq > 0 ? nq : 1));
    int64_t* rn = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
    norms_i32(q, nq, dim, qn);
    norms_i32(r, nr, dim, rn);
    pthread_t th[256];
    topk_job jobs[256];
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (topk_job){q, r, qn, rn, nq, nr, dim, k, mode, out_s, out_i, out_c, out_dot, i, nthreads};
        pthread_create(&th[i], NULL, topk_worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(rn);
    free(qn);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Classification: encode reads then rank them against references.     */
/* This is the CPU baseline: HVCache::compute per read followed by a    */
/* brute-force cosine over every reference (encode + top-k search).     */
/* ------------------------------------------------------------------ */
typedef struct {
    const orc_tables* t;
    const char* buf;
    const int64_t *off, *len;
    int64_t n;
    const void* refs;
    int ref_bytes; /* 2: int16 rows (HV_16), 4: int32 rows */
    const int64_t* rn;
    int64_t nr;
    int k, mode, bipolar;
    int32_t max_abs_r; /* max |reference element| (int16 rows) */
    float* out_s;
    int32_t* out_i;
    double* out_c;    /* optional: FP64 cosine of each hit */
    int64_t* out_dot; /* optional: exact dot of each hit */
    int tid, nthreads;
} cls_job;

static void* cls_worker(void* arg) {
    cls_job* j = (cls_job*)arg;
    int dim = j->t->dim, k = j->k;
    int32_t* acc = (int32_t*)malloc(sizeof(int32_t) * (size_t)dim);
    uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)j->t->W);
    float* bs = (float*)malloc(sizeof(float) * (size_t)k);
    int32_t* bi = (int32_t*)malloc(sizeof(int32_t) * (size_t)k);
    int64_t* bd = (int64_t*)malloc(sizeof(int64_t) * (size_t)k);
    int16_t* q16 = (int16_t*)malloc(sizeof(int16_t) * (size_t)dim);
    for (int64_t s = j->tid; s < j->n; s += j->nthreads) {
        encode_one(j->t, j->buf + j->off[s], j->len[s], acc, tmp);
        int64_t qn = 0;
        int32_t max_q = 1;
        for (int d = 0; d < dim; ++d) {
            int32_t v = j->bipolar ? (acc[d] >= 0 ? 1 : -1) : (int32_t)(int16_t)(uint16_t)(uint32_t)acc[d];
            acc[d] = v;
            q16[d] = (int16_t)v;
            qn += (int64_t)v * v;
            if (v > max_q) max_q = v;
            if (-v > max_q) max_q = -v;
        }
        /* int16 x int16 products summed in int32 over chunks short enough that no sum can
           overflow (chunk * max|q| * max|r| < 2^31), then in int64: exact, and vectorisable */
        const int64_t bound = (int64_t)max_q * (j->max_abs_r > 0 ? j->max_abs_r : 1);
        int chunk = (int)(2147483647LL / bound);
        if (chunk < 1) chunk = 1;
        int filled = 0;
        for (int64_t ri = 0; ri < j->nr; ++ri) {
            int64_t dot = 0;
            if (j->ref_bytes == 2) {
                const int16_t* r = (const int16_t*)j->refs + (size_t)ri * dim;
                for (int d0 = 0; d0 < dim; d0 += chunk) {
                    const int d1 = dim - d0 < chunk ? dim : d0 + chunk;
                    int32_t part = 0;
                    for (int d = d0; d < d1; ++d) part += (int32_t)q16[d] * (int32_t)r[d];
                    dot += part;
                }
            } else {
                const int32_t* r = (const int32_t*)j->refs + (size_t)ri * dim;
                for (int d = 0; d < dim; ++d) dot += (int64_t)acc[d] * r[d];
            }
            float sc = score_from(dot, qn, j->rn[ri], j->mode);
            if (filled == k && !better(sc, (int32_t)ri, bs[k - 1], bi[k - 1])) continue;
            int pos = filled < k ? filled : k - 1;
            while (pos > 0 && better(sc, (int32_t)ri, bs[pos - 1], bi[pos - 1])) {
                bs[pos] = bs[pos - 1];
                bi[pos] = bi[pos - 1];
                bd[pos] = bd[pos - 1];
                --pos;
            }
            bs[pos] = sc;
            bi[pos] = (int32_t)ri;
            bd[pos] = dot;
            if (filled < k) ++filled;
        }
        for (int t = 0; t < k; ++t) {
            j->out_s[s * k + t] = t < filled ? bs[t] : -INFINITY;
            j->out_i[s * k + t] = t < filled ? bi[t] : -1;
            if (j->out_c) j->out_c[s * k + t] = t < filled ? cos_from(bd[t], qn, j->rn[bi[t]]) : 0.0;
            if (j->out_dot) j->out_dot[s * k + t] = t < filled ? bd[t] : 0;
        }
    }
    free(q16);
    free(bd);
    free(bi);
    free(bs);
    free(tmp);
    free(acc);
    return NULL;
}

typedef struct {
    const void* refs;
    int ref_bytes, dim;
    int64_t nr;
    int64_t* rn;
    int32_t max_abs; /* this thread's max |element| */
    int tid, nthreads;
} norms_job;

static void* norms_worker(void* arg) {
    norms_job* j = (norms_job*)arg;
    int32_t mx = 0;
    for (int64_t i = j->tid; i < j->nr; i += j->nthreads) {
        int64_t s = 0;
        for (int d = 0; d < j->dim; ++d) {
            const int64_t v = j->ref_bytes == 2 ? ((const int16_t*)j->refs)[(size_t)i * j->dim + d]
                                                : ((const int32_t*)j->refs)[(size_t)i * j->dim + d];
            s += v * v;
            const int64_t a = v < 0 ? -v : v;
            if (a > mx) mx = a > 0x7fffffff ? 0x7fffffff : (int32_t)a;
        }
        j->rn[i] = s;
    }
    j->max_abs = mx;
    return NULL;
}

/* Squared norms of the references (int16 or int32 rows) into rn, and the
 * largest |element|; rows split over threads. */
int32_t orc_ref_norms(const void* refs, int ref_bytes, int64_t nr, int dim, int64_t* rn, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    norms_job jobs[256];
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (norms_job){refs, ref_bytes, dim, nr, rn, 0, i, nthreads};
        pthread_create(&th[i], NULL, norms_worker, &jobs[i]);
    }
    int32_t mx = 0;
    for (int i = 0; i < nthreads; ++i) {
        pthread_join(th[i], NULL);
        if (jobs[i].max_abs > mx) mx = jobs[i].max_abs;
    }
    return mx;
}

/* Encode every read then rank it against every reference: scores and indices,
 * and, when out_c / out_dot are given, each hit's FP64 cosine and exact dot.
 * rn_in (optional): the references' squared norms from orc_ref_norms, with
 * max_abs_in their largest |element|; computed here when null. */
int orc_classify_ex(int dim, int kmer, const char* buf, const int64_t* off, const int64_t* len, int64_t n,
                    const void* refs, int ref_bytes, int64_t nr, const int64_t* rn_in, int32_t max_abs_in, int k,
                    int mode, int bipolar, float* out_s, int32_t* out_i, double* out_c, int64_t* out_dot,
                    int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    orc_tables t;
    tables_init(&t, dim, kmer);
    int64_t* rn_own = NULL;
    const int64_t* rn = rn_in;
    int32_t max_abs_r = max_abs_in;
    if (!rn) {
        rn_own = (int64_t*)malloc(sizeof(int64_t) * (size_t)(nr > 0 ? nr : 1));
        max_abs_r = orc_ref_norms(refs, ref_bytes, nr, dim, rn_own, nthreads);
        rn = rn_own;
    }
    if (ref_bytes != 2) max_abs_r = 0; /* int32 rows are summed in int64 directly */
    pthread_t th[256];
    cls_job jobs[256];
    for (int i = 0; i < nthreads; ++i) {
        jobs[i] = (cls_job){&t,    buf,      off,   len,   n,     refs,  ref_bytes, rn, nr, k, mode, bipolar, max_abs_r,
                            out_s, out_i, out_c, out_dot, i, nthreads};
        pthread_create(&th[i], NULL, cls_worker, &jobs[i]);
    }
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    free(rn_own);
    tables_free(&t);
    return 0;
}

int orc_classify(int dim, int kmer, const char* buf, const int64_t* off, const int64_t* len, int64_t n,
                 const void* refs, int ref_bytes, int64_t nr, int k, int mode, int bipolar, float* out_s,
                 int32_t* out_i, int nthreads) {
    return orc_classify_ex(dim, kmer, buf, off, len, n, refs, ref_bytes, nr, NULL, 0, k, mode, bipolar, out_s, out_i,
                           NULL, NULL, nthreads);
}

/* ------------------------------------------------------------------ */
/* Propagate-children                                                  */
/* ------------------------------------------------------------------ */

/* Bundling: parent[p] = sum of rows of its children (CSR: child_ptr[p] ..
 * child_ptr[p+1] index into child_idx), exact int32. */
int orc_bundle(const int32_t* rows, int dim, const int64_t* child_ptr, const int32_t* child_idx, int64_t nparents,
               int32_t* out) {
    for (int64_t p = 0; p < nparents; ++p) {
        int32_t* o = out + (size_t)p * dim;
        memset(o, 0, sizeof(int32_t) * (size_t)dim);
        for (int64_t c = child_ptr[p]; c < child_ptr[p + 1]; ++c) {
            const int32_t* r = rows + (size_t)child_idx[c] * dim;
            for (int d = 0; d < dim; ++d) o[d] += r[d];
        }
    }
    return 0;
}

/* Greedy representative selection for one parent
 * (targets/propogate-children.cpp:60-73): candidates are visited in order;
 * best = max(0, max score vs the parent's existing representatives and the
 * candidates already added); a candidate is added when best < threshold.
 * reps/cands are int32 rows; selected[i] = 1 if candidate i was added. */
int orc_propagate_greedy(const int32_t* reps, int64_t nreps, const int32_t* cands, int64_t ncands, int dim,
                         double threshold, int mode, uint8_t* selected, float* best_out) {
    int64_t* added = (int64_t*)malloc(sizeof(int64_t) * (size_t)(ncands > 0 ? ncands : 1));
    int64_t nadded = 0;
    for (int64_t i = 0; i < ncands; ++i) {
        const int32_t* x = cands + (size_t)i * dim;
        float best = 0.0f;
        for (int64_t r = 0; r < nreps; ++r) {
            float s = orc_cosine_i32(x, reps + (size_t)r * dim, dim, mode);
            if (s > best) best = s;
        }
        for (int64_t a = 0; a < nadded; ++a) {
            float s = orc_cosine_i32(x, cands + (size_t)added[a] * dim, dim, mode);
            if (s > best) best = s;
        }
        if (best_out) best_out[i] = best;
        selected[i] = (double)best < threshold;
        if (selected[i]) added[nadded++] = i;
    }
    free(added);
    return (int)nadded;
}
