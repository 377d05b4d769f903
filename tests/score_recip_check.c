/* CPU check of the tensor-core search's reciprocal-product exact score
 * (exact_score_recip in csrc/topk.cuh), restated in C with the same IEEE
 * operations (glibc's fma and the division operator are correctly rounded).
 *
 * For random and adversarial (dot, nq, nr) it compares the float score of the
 * fast path, with its fallback, against the reference's own formula
 *   COS  (float)(dot / (sqrt(nq) * sqrt(nr)))
 *   NORM (float)(2.0 * (dot / (sqrt(nq) * sqrt(nr)) - 0.5))   (src/HV.cpp:219-242)
 * bit for bit, and checks that the corrected quotient q1 is within one unit in
 * the last place of the correctly rounded one.  Prints one line of counts and
 * exits 1 on any mismatch.  Build with -ffp-contract=off. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next(void) {
    state ^= state << 13;
    state ^= state >> 7;
    state ^= state << 17;
    return state;
}

static uint64_t dbits(double x) {
    uint64_t b;
    memcpy(&b, &x, 8);
    return b;
}

/* far_from_float_midpoint of csrc/topk.cuh */
static int far_from_midpoint(double t) {
    const uint64_t b = dbits(t);
    const int e = (int)((b >> 52) & 0x7ff);
    const int64_t d = (int64_t)(b & 0x1fffffffull) - (int64_t)(1 << 28);
    return e >= 998 && e <= 1024 && (d < 0 ? -d : d) > ((int64_t)1 << (1025 - e));
}

static float reference_score(int64_t dot, int64_t nq, int64_t nr, int norm) {
    const double c = (double)dot / (sqrt((double)nq) * sqrt((double)nr));
    return norm ? (float)(2.0 * (c - 0.5)) : (float)c;
}

static long n_fast, n_exact, n_bad, n_far;

static float fast_score(int64_t dot, int64_t nq, int64_t nr, int norm) {
    const double sq = sqrt((double)nq), sr = sqrt((double)nr);
    const double iq = 1.0 / sq, ir = 1.0 / sr;
    const double x = (double)dot, p = sq * sr, y = iq * ir;
    const double q0 = x * y;
    const double q1 = fma(fma(-q0, p, x), y, q0);
    const double c = x / p;
    if (q1 != c && nextafter(c, q1) != q1) ++n_far;
    const double t = norm ? q1 - 0.5 : q1;
    if (!far_from_midpoint(t)) {
        ++n_exact;
        return reference_score(dot, nq, nr, norm);
    }
    ++n_fast;
    const float f = (float)t;
    return norm ? 2.0f * f : f;
}

static void check(int64_t dot, int64_t nq, int64_t nr) {
    for (int norm = 0; norm < 2; ++norm) {
        const float a = fast_score(dot, nq, nr, norm), b = reference_score(dot, nq, nr, norm);
        uint32_t ua, ub;
        memcpy(&ua, &a, 4);
        memcpy(&ub, &b, 4);
        if (ua != ub) {
            if (n_bad < 5)
                printf("mismatch dot=%lld nq=%lld nr=%lld norm=%d: %.9g vs %.9g\n", (long long)dot, (long long)nq,
                       (long long)nr, norm, a, b);
            ++n_bad;
        }
    }
}

int main(int argc, char** argv) {
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    for (long i = 0; i < n; ++i) {
        /* bipolar queries (nq = dim) or count-valued ones; references up to 2^42 */
        const int64_t nq = (next() & 1) ? (int64_t)(1000 + next() % 20000)
                                        : (int64_t)(1 + next() % (1ull << (next() % 40 + 1)));
        const int64_t nr = (int64_t)(1 + next() % (1ull << (next() % 42 + 1)));
        const double lim = sqrt((double)nq) * sqrt((double)nr);
        int64_t dot;
        switch ((int)(next() % 4)) {
            case 0: /* uniform cosine */
                dot = (int64_t)((double)(next() % 2000001) / 1e6 * lim - lim);
                break;
            case 1: { /* cosine near a float midpoint */
                const float f = (float)((double)(next() % 2000001) / 1e6 - 1.0);
                const double mid = (double)f + ldexp(1.0, ilogb(f) - 24) * ((next() & 1) ? 1 : -1);
                dot = (int64_t)llround(mid * lim) + (int64_t)(next() % 5) - 2;
                break;
            }
            case 2: { /* c - 0.5 near a float midpoint */
                const float f = (float)((double)(next() % 3000001) / 1e6 - 2.0) * 0.5f;
                const double mid = (double)f + ldexp(1.0, ilogb(f) - 24) * ((next() & 1) ? 1 : -1);
                dot = (int64_t)llround((mid + 0.5) * lim) + (int64_t)(next() % 5) - 2;
                break;
            }
            default: { /* cosine near 0.5, 1 and -1 */
                static const double at[3] = {0.5, 1.0, -1.0};
                dot = (int64_t)llround(at[next() % 3] * lim) + (int64_t)(next() % 41) - 20;
            }
        }
        if ((double)llabs(dot) > lim) dot = dot > 0 ? (int64_t)floor(lim) : -(int64_t)floor(lim);
        check(dot, nq, nr);
    }
    printf("fast %ld exact %ld mismatches %ld quotient-more-than-one-unit %ld\n", n_fast, n_exact, n_bad, n_far);
    return n_bad != 0 || n_far != 0;
}
