// Ranking keys and exact scores shared by the plain and tensor-core searches.
//
// Ranking rule: descending float score, ties to the lower reference index
// (the reference CPU argmax keeps the first maximum,
// tests/cosine_comparison_test.cpp:146-156).  A candidate is packed into a
// 64-bit key that orders exactly like that rule:
//     key = orderable(score bits) << 32 | (0xffffffff - ref index)
// so "larger key" means "ranks earlier" and key 0 is below every real key.
#pragma once

#include <stdint.h>

#include "hdc_gb300.h"

namespace hdc {

__host__ __device__ __forceinline__ uint32_t ord_float(float f) {
    uint32_t b;
    memcpy(&b, &f, 4);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

__host__ __device__ __forceinline__ float unord_float(uint32_t o) {
    uint32_t b = (o & 0x80000000u) ? (o & 0x7fffffffu) : ~o;
    float f;
    memcpy(&f, &b, 4);
    return f;
}

__host__ __device__ __forceinline__ uint64_t make_key(float score, uint32_t idx) {
    return ((uint64_t)ord_float(score) << 32) | (uint64_t)(0xffffffffu - idx);
}

__host__ __device__ __forceinline__ uint32_t key_idx(uint64_t key) { return 0xffffffffu - (uint32_t)key; }
__host__ __device__ __forceinline__ float key_score(uint64_t key) { return unord_float((uint32_t)(key >> 32)); }

// The reference's float score from the exact dot and squared norms:
//   NORM: (float)(2.0 * (dot / (sqrt(nq) * sqrt(nr)) - 0.5)), -1 on a zero norm
//         (src/HV.cpp:219-242; the float literal 0.5f is exactly 0.5)
//   COS:  (float)(dot / (sqrt(nq) * sqrt(nr))), -1 on a zero norm
//   DOT:  (float)dot (src/HV.cpp:244-252)
// Every double operation is IEEE round-to-nearest, written with explicit
// intrinsics so no contraction or reassociation can change the rounding.
__device__ __forceinline__ double exact_cos(int64_t dot, int64_t nq, int64_t nr) {
    if (nq == 0 || nr == 0) return 0.0;
    double den = __dmul_rn(__dsqrt_rn((double)nq), __dsqrt_rn((double)nr));
    return __ddiv_rn((double)dot, den);
}

__device__ __forceinline__ float exact_score(int64_t dot, int64_t nq, int64_t nr, int mode) {
    if (mode == HDC_SCORE_DOT) return __ll2float_rn(dot);
    if (nq == 0 || nr == 0) return -1.0f;
    double c = exact_cos(dot, nq, nr);
    if (mode == HDC_SCORE_NORM) return __double2float_rn(__dmul_rn(2.0, __dadd_rn(c, -0.5)));
    return __double2float_rn(c);
}

// Width of the fp32 pre-filter guard band, in score units.  The fp32
// estimate  fl(fl(dot) * fl(1/sqrt(nq)) * fl(1/sqrt(nr)))  is within about
// 5 * 2^-24 (relative, i.e. < 3.5e-7 absolute for |cos| <= 1) of the exact
// cosine, and the reference's float score is the double result rounded to
// float (another <= 6e-8); a score that can reach the current k-th best is
// therefore never rejected with a margin of 4e-6 (NORM doubles the cosine
// error, still < 1e-6).  DOT scores are exact and need no margin.
constexpr float kFilterMargin = 4e-6f;

// The same score from sq = sqrt(nq) and sr = sqrt(nr), each already rounded to
// double (0 for a zero norm): the identical sequence of IEEE operations, with
// the two square roots computed once per query and per reference.  Two steps
// leave the FP64 pipe with identical results: the zero tests read the bits (a
// square root of a non-negative integer is +0 or positive), and NORM scales by 2
// after the rounding to float, which commutes with it here (|c - 0.5| is 0 or at
// least 2^-54, far from float's subnormals, and far below overflow).
__device__ __forceinline__ float exact_score_sqrt(int64_t dot, double sq, double sr, int mode) {
    if (mode == HDC_SCORE_DOT) return __ll2float_rn(dot);
    if (__double_as_longlong(sq) == 0 || __double_as_longlong(sr) == 0) return -1.0f;
    const double c = __ddiv_rn((double)dot, __dmul_rn(sq, sr));
    if (mode == HDC_SCORE_NORM) return 2.0f * __double2float_rn(__dadd_rn(c, -0.5));
    return __double2float_rn(c);
}

// True when the double t lies more than 2^-50 from every midpoint between two
// adjacent floats, so that any value within 2^-50 of t rounds to the same float.
// The midpoints of t's binade have the 29 low mantissa bits 1000...0; 2^-50 is
// 2^(1025 - e) units of that binade (e the biased exponent).  Binades below
// 2^-27 (and zero) are never "far": the margin would not fit in those bits.
__device__ __forceinline__ bool far_from_float_midpoint(double t) {
    const uint64_t b = (uint64_t)__double_as_longlong(t);
    const int e = (int)((b >> 52) & 0x7ff);
    const int64_t d = (int64_t)(b & 0x1fffffffull) - (int64_t)(1 << 28);
    return e >= 998 && e <= 1024 && (d < 0 ? -d : d) > ((int64_t)1 << (1025 - e));
}

// exact_score_sqrt with the divide replaced by a reciprocal product and one
// correction, given also iq = fl(1/sq) and ir = fl(1/sr) (0 for a zero norm).
// y = fl(iq * ir) is within a few units in the last place of 1/p, p = fl(sq * sr),
// so q0 = fl(dot * y) is too; the residual dot - q0 * p (one FMA) and
// q1 = fl(q0 + residual * y) (the Newton correction of Markstein's division) put
// q1 within one unit of fl(dot / p), i.e. within 2^-52 of the quotient the
// reference rounds for |c| <= 1 (2^-51 with NORM's subtraction).  When the value
// to be rounded to float lies more than 2^-50 from every float midpoint, its
// rounding equals that of the reference's value; otherwise (a window of 2^-49
// around each midpoint, rarely met) the exact sequence runs.
__device__ __forceinline__ float exact_score_recip(int64_t dot, double sq, double sr, double iq, double ir,
                                                   int mode) {
    if (mode == HDC_SCORE_DOT) return __ll2float_rn(dot);
    if (__double_as_longlong(sq) == 0 || __double_as_longlong(sr) == 0) return -1.0f;
    const double x = (double)dot, p = __dmul_rn(sq, sr), y = __dmul_rn(iq, ir);
    const double q0 = __dmul_rn(x, y);
    const double q1 = __fma_rn(__fma_rn(-q0, p, x), y, q0);
    const double t = mode == HDC_SCORE_NORM ? __dadd_rn(q1, -0.5) : q1;
    if (far_from_float_midpoint(t)) {
        const float f = __double2float_rn(t);
        return mode == HDC_SCORE_NORM ? 2.0f * f : f;
    }
    return exact_score_sqrt(dot, sq, sr, mode);
}

__device__ __forceinline__ float approx_score(float dotf, float rq, float rr, int mode) {
    if (mode == HDC_SCORE_DOT) return dotf;
    const float c = dotf * rq * rr;  // rq/rr are 0 for zero norms
    return mode == HDC_SCORE_NORM ? fmaf(2.0f, c, -1.0f) : c;
}

// fp32 reciprocal square root of a squared norm, rounded from FP64
__device__ __forceinline__ float rsqrt_norm(int64_t n2) {
    return n2 == 0 ? 0.0f : __double2float_rn(__drcp_rn(__dsqrt_rn((double)n2)));
}

// Insert (key, dot) into a descending list of length k held in local memory.
__device__ __forceinline__ void list_insert(uint64_t* keys, int64_t* dots, int k, uint64_t key, int64_t dot) {
    int pos = k - 1;
    while (pos > 0 && keys[pos - 1] < key) {
        keys[pos] = keys[pos - 1];
        dots[pos] = dots[pos - 1];
        --pos;
    }
    keys[pos] = key;
    dots[pos] = dot;
}

}  // namespace hdc
