// Double-float arithmetic on the FP32 pipe, for reproducing the float rounding
// of an FP64 expression without issuing FP64 instructions.
//
// GB300 issues FP64 at 2 lanes per clock per SM against 128 for FP32, and the
// reference computes its clip points in FP64 and stores them as floats. A
// value kept as an unevaluated sum hi + lo of two floats carries ~48 bits;
// each operation below also yields an absolute bound on its own error, so the
// final value v is known to lie within E of the reference's double d. When no
// float rounding boundary (midpoint between adjacent floats) lies within E of
// v, every double in [v - E, v + E] — d among them — rounds to the same float,
// which is then the reference's float exactly (round_certified). Otherwise the
// caller evaluates the reference's own FP64 expression. With E ~ 2^-43 of the
// magnitudes against a float spacing of 2^-23, that happens about once in 10^6.
//
// Error-free transformations (Knuth's TwoSum, Dekker's product via one fused
// multiply-add), written with round-to-nearest intrinsics so that nothing is
// reassociated or contracted.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace farm {

struct dflt {
    float hi, lo;
};

// a + b = s + e exactly
__device__ __forceinline__ dflt two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

// a * b = p + e exactly (no underflow in the ranges used here)
__device__ __forceinline__ dflt two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

// renormalise so that hi = rn(hi + lo) (|a| >= |b| or a == 0)
__device__ __forceinline__ dflt fast_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// Bounds below are absolute and conservative; u = 2^-24.
constexpr float kU = 5.9604645e-08f;   // 2^-24
constexpr float kU2 = 3.5527137e-15f;  // 2^-48

// a + b; adds to *err a bound on |result - (a + b)|:
// 3u (|a.lo| + |b.lo|) + 2u^2 (|a.hi| + |b.hi|)
__device__ __forceinline__ dflt df_add(dflt a, dflt b, float *err) {
    const dflt s = two_sum(a.hi, b.hi);
    const float t = __fadd_rn(a.lo, b.lo);
    const dflt r = two_sum(s.hi, __fadd_rn(s.lo, t));
    *err = __fadd_rn(*err, __fadd_rn(__fmul_rn(3.f * kU, __fadd_rn(fabsf(a.lo), fabsf(b.lo))),
                                     __fmul_rn(2.f * kU2, __fadd_rn(fabsf(a.hi), fabsf(b.hi)))));
    return r;
}

// a * b; adds 10u^2 |a b| to *err
__device__ __forceinline__ dflt df_mul(dflt a, dflt b, float *err) {
    const dflt p = two_prod(a.hi, b.hi);
    const float c = __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi));
    const dflt r = two_sum(p.hi, __fadd_rn(p.lo, c));
    *err = __fadd_rn(*err, __fmul_rn(10.f * kU2, fabsf(r.hi)));
    return r;
}

// a / b for a float b; adds 8u^2 |a / b| to *err
__device__ __forceinline__ dflt df_div_f(dflt a, float b, float *err) {
    const float q1 = __fdiv_rn(a.hi, b);
    const dflt p = two_prod(q1, b);
    // remainder a - q1 b, exact up to the rounding of the low parts
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo);
    const float q2 = __fdiv_rn(r, b);
    const dflt q = fast_two_sum(q1, q2);
    *err = __fadd_rn(*err, __fmul_rn(8.f * kU2, fabsf(q.hi)));
    return q;
}

// float b / double-float a; adds 16u^2 |b / a| to *err
__device__ __forceinline__ dflt df_rdiv(float b, dflt a, float *err) {
    const float q1 = __fdiv_rn(b, a.hi);
    // b - q1 * a = b - q1 a.hi - q1 a.lo
    const dflt p = two_prod(q1, a.hi);
    const float r = __fsub_rn(__fsub_rn(__fsub_rn(b, p.hi), p.lo), __fmul_rn(q1, a.lo));
    const float q2 = __fdiv_rn(r, a.hi);
    const dflt q = fast_two_sum(q1, q2);
    *err = __fadd_rn(*err, __fmul_rn(16.f * kU2, fabsf(q.hi)));
    return q;
}

// a / b for double-floats; adds 10u^2 |a / b| to *err
__device__ __forceinline__ dflt df_div(dflt a, dflt b, float *err) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const dflt p = two_prod(q1, b.hi);
    const float r = __fsub_rn(__fadd_rn(__fsub_rn(__fsub_rn(a.hi, p.hi), p.lo), a.lo), __fmul_rn(q1, b.lo));
    const float q2 = __fdiv_rn(r, b.hi);
    const dflt q = fast_two_sum(q1, q2);
    *err = __fadd_rn(*err, __fmul_rn(10.f * kU2, fabsf(q.hi)));
    return q;
}

// A value of the reference's FP64 computation tracked in double-float: v and
// a bound e on |v - the reference's double|. Each operation adds its own
// double-float error, the propagation of its inputs' bounds, and the
// reference's rounding of its result (2^-53 relative, counted as 2^-52).
struct cval {
    dflt v;
    float e;
};
constexpr float kRef = 2.220446e-16f;  // 2^-52

__device__ __forceinline__ float mag(const cval &a) { return fabsf(a.v.hi); }

// a float the reference promotes to double: exact
__device__ __forceinline__ cval cv_f(float f) { return {{f, 0.f}, 0.f}; }
// a double the reference holds, given as its split hi + lo (within u^2)
__device__ __forceinline__ cval cv_d(dflt c) { return {c, __fmul_rn(2.f * kU2, fabsf(c.hi))}; }
__device__ __forceinline__ cval cv_neg(cval a) { return {{-a.v.hi, -a.v.lo}, a.e}; }

__device__ __forceinline__ cval cv_add(cval a, cval b) {
    float e = __fadd_rn(a.e, b.e);
    const dflt v = df_add(a.v, b.v, &e);
    return {v, __fadd_rn(e, __fmul_rn(kRef, fabsf(v.hi)))};
}

__device__ __forceinline__ cval cv_mul(cval a, cval b) {
    float e = __fadd_rn(__fadd_rn(__fmul_rn(mag(a), b.e), __fmul_rn(mag(b), a.e)), __fmul_rn(a.e, b.e));
    const dflt v = df_mul(a.v, b.v, &e);
    return {v, __fadd_rn(e, __fmul_rn(kRef, fabsf(v.hi)))};
}

// a / b, |b| well away from its error bound (the caller checks)
__device__ __forceinline__ cval cv_div(cval a, cval b) {
    float e = 0.f;
    const dflt v = df_div(a.v, b.v, &e);
    const float bb = fabsf(b.v.hi);
    // |a/b - a'/b'| <= (e_a + |a/b| e_b) / (|b| - e_b)
    const float prop = __fdiv_rn(__fadd_rn(a.e, __fmul_rn(fabsf(v.hi), b.e)), __fsub_rn(bb, b.e));
    return {v, __fadd_rn(__fadd_rn(e, prop), __fmul_rn(kRef, fabsf(v.hi)))};
}

// The float nearest to the reference's double d, given v = x.hi + x.lo with
// |v - d| <= err: true when every real within err of v rounds to the same
// float (no rounding midpoint in between), which is then written to *out.
// Zero, subnormal and near-overflow results are left to the caller.
__device__ __forceinline__ bool round_certified(dflt x, float err, float *out) {
    const dflt n = fast_two_sum(x.hi, x.lo);  // hi = rn(hi + lo) up to a tie
    const float f = n.hi, af = fabsf(f);
    if (!(af >= 7.8886091e-31f) || !(af <= 1.0e37f)) return false;  // [2^-100, 1e37]
    // distances from |f| to the rounding midpoints on either side of it
    const int b = __float_as_int(af);
    const float half_above = __fmul_rn(__fsub_rn(__int_as_float(b + 1), af), 0.5f);  // exact: powers of two
    const float half_below = __fmul_rn(__fsub_rn(af, __int_as_float(b - 1)), 0.5f);
    const float lo = f < 0.f ? -n.lo : n.lo;  // the remainder in the direction of |f|
    const float e = __fmul_rn(err, 1.0625f);  // slack for the rounding of the two tests
    if (__fadd_rn(lo, e) < half_above && __fsub_rn(lo, e) > -half_below) {
        *out = f;
        return true;
    }
    return false;
}

}  // namespace farm
