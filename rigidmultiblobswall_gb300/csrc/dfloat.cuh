// Double-float ("df64") arithmetic on the FP32 pipe: a value is hi + lo with
// |lo| <= ulp(hi)/2, about 48 significant bits.  Built from the error-free
// transformations TwoSum (Knuth), FastTwoSum (Dekker) and the FMA-based exact
// product; additions use the cheap ("sloppy") variant, whose error is bounded
// by ~2^-47 (|a| + |b|) - the same form as an FP64 addition, 30x looser.
//
// Every rounding step of these transformations uses the _rn intrinsics:
// the compiler never contracts them into an FMA.  A contracted
// `p = x*y; s = p + c` becomes s = fma(x, y, c), no longer the rounded sum of
// the p that the error term is computed from, and the transformation stops
// being error-free (a ~2^-24 relative error leaks into the result).
#pragma once
#include <cuda_runtime.h>

namespace rmw {

struct df {
    float hi, lo;
};

__device__ __forceinline__ df df_from(float h) { return {h, 0.0f}; }

__device__ __forceinline__ df fast_two_sum(float a, float b)
{
    const float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ df two_sum_df(float a, float b)
{
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}

__device__ __forceinline__ df operator+(df a, df b)
{
    const df s = two_sum_df(a.hi, b.hi);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator+(df a, float b)
{
    const df s = two_sum_df(a.hi, b);
    return fast_two_sum(s.hi, __fadd_rn(s.lo, a.lo));
}
__device__ __forceinline__ df operator+(float a, df b) { return b + a; }
__device__ __forceinline__ df operator-(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator-(df a, float b) { return a + (-b); }
__device__ __forceinline__ df operator-(float a, df b) { return (-b) + a; }

__device__ __forceinline__ df operator*(df a, df b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df operator*(df a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df operator*(float a, df b) { return b * a; }

// Products left unnormalised, (p, e) with |e| <= ~2^-22.4 |p|: for operands
// that go straight into a sum (whose two-sum renormalises), where the skipped
// fast two-sum would be redone anyway.
__device__ __forceinline__ df mul_u(df a, df b)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return {p, e};
}
__device__ __forceinline__ df mul_u(df a, float b)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    return {p, e};
}
__device__ __forceinline__ df sqr_u(df a)
{
    const float p = __fmul_rn(a.hi, a.hi);
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return {p, e};
}

// Sums left unnormalised (the exact two-sum of the high parts plus the low
// parts): for operands of a further sum, or of a product when the high parts
// cannot cancel (after cancellation the value sits in the low part, and a
// double-float product drops lo * lo).
__device__ __forceinline__ df add_u(df a, df b)
{
    const df s = two_sum_df(a.hi, b.hi);
    return {s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo))};
}
__device__ __forceinline__ df sub_u(df a, df b) { return add_u(a, {-b.hi, -b.lo}); }
// a*b + c, unnormalised
__device__ __forceinline__ df mad_u(df a, df b, df c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const df t = two_sum_df(p, c.hi);
    return {t.hi, __fadd_rn(t.lo, __fadd_rn(e, c.lo))};
}
__device__ __forceinline__ df mad_u(df a, float b, df c)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    const df t = two_sum_df(p, c.hi);
    return {t.hi, __fadd_rn(t.lo, __fadd_rn(e, c.lo))};
}

// a*b + c with a single renormalisation
__device__ __forceinline__ df mad(df a, df b, df c)
{
    const float p = __fmul_rn(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    const df t = two_sum_df(p, c.hi);
    return fast_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(e, c.lo)));
}
__device__ __forceinline__ df mad(df a, float b, df c)
{
    const float p = __fmul_rn(a.hi, b);
    float e = fmaf(a.hi, b, -p);
    e = fmaf(a.lo, b, e);
    const df t = two_sum_df(p, c.hi);
    return fast_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(e, c.lo)));
}
// a*b + c*d with a single renormalisation
__device__ __forceinline__ df mad2(df a, df b, df c, df d)
{
    const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi);
    float e1 = fmaf(a.hi, b.hi, -p1);
    e1 = fmaf(a.hi, b.lo, e1);
    e1 = fmaf(a.lo, b.hi, e1);
    float e2 = fmaf(c.hi, d.hi, -p2);
    e2 = fmaf(c.hi, d.lo, e2);
    e2 = fmaf(c.lo, d.hi, e2);
    const df t = two_sum_df(p1, p2);
    return fast_two_sum(t.hi, __fadd_rn(t.lo, __fadd_rn(e1, e2)));
}
// a*b + c*d + e*f with a single renormalisation
__device__ __forceinline__ df dot3(df a, df b, df c, df d, df e, df f)
{
    const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi), p3 = __fmul_rn(e.hi, f.hi);
    float e1 = fmaf(a.hi, b.hi, -p1);
    e1 = fmaf(a.hi, b.lo, e1);
    e1 = fmaf(a.lo, b.hi, e1);
    float e2 = fmaf(c.hi, d.hi, -p2);
    e2 = fmaf(c.hi, d.lo, e2);
    e2 = fmaf(c.lo, d.hi, e2);
    float e3 = fmaf(e.hi, f.hi, -p3);
    e3 = fmaf(e.hi, f.lo, e3);
    e3 = fmaf(e.lo, f.hi, e3);
    const df t1 = two_sum_df(p1, p2);
    const df t2 = two_sum_df(t1.hi, p3);
    return fast_two_sum(t2.hi, __fadd_rn(__fadd_rn(t1.lo, t2.lo), __fadd_rn(__fadd_rn(e1, e2), e3)));
}

// acc += a*b + c*d without renormalising acc (as acc_add)
__device__ __forceinline__ void acc_dot2(df &acc, df a, df b, df c, df d)
{
    const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi);
    float e1 = fmaf(a.hi, b.hi, -p1);
    e1 = fmaf(a.hi, b.lo, e1);
    e1 = fmaf(a.lo, b.hi, e1);
    float e2 = fmaf(c.hi, d.hi, -p2);
    e2 = fmaf(c.hi, d.lo, e2);
    e2 = fmaf(c.lo, d.hi, e2);
    const df t1 = two_sum_df(acc.hi, p1);
    const df t2 = two_sum_df(t1.hi, p2);
    acc.hi = t2.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(__fadd_rn(t1.lo, t2.lo), __fadd_rn(e1, e2)));
}

// acc += a*b + c*d + e*f without renormalising acc
__device__ __forceinline__ void acc_dot3(df &acc, df a, df b, df c, df d, df e, df f)
{
    const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi), p3 = __fmul_rn(e.hi, f.hi);
    float e1 = fmaf(a.hi, b.hi, -p1);
    e1 = fmaf(a.hi, b.lo, e1);
    e1 = fmaf(a.lo, b.hi, e1);
    float e2 = fmaf(c.hi, d.hi, -p2);
    e2 = fmaf(c.hi, d.lo, e2);
    e2 = fmaf(c.lo, d.hi, e2);
    float e3 = fmaf(e.hi, f.hi, -p3);
    e3 = fmaf(e.hi, f.lo, e3);
    e3 = fmaf(e.lo, f.hi, e3);
    const df t1 = two_sum_df(acc.hi, p1);
    const df t2 = two_sum_df(t1.hi, p2);
    const df t3 = two_sum_df(t2.hi, p3);
    acc.hi = t3.hi;
    const float lo = __fadd_rn(__fadd_rn(t1.lo, t2.lo), t3.lo);
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(lo, __fadd_rn(__fadd_rn(e1, e2), e3)));
}

// acc += a*b + c*d + e*f + g*h without renormalising acc
__device__ __forceinline__ void acc_dot4(df &acc, df a, df b, df c, df d, df e, df f, df g, df h)
{
    const float p1 = __fmul_rn(a.hi, b.hi), p2 = __fmul_rn(c.hi, d.hi);
    const float p3 = __fmul_rn(e.hi, f.hi), p4 = __fmul_rn(g.hi, h.hi);
    float e1 = fmaf(a.hi, b.hi, -p1);
    e1 = fmaf(a.hi, b.lo, e1);
    e1 = fmaf(a.lo, b.hi, e1);
    float e2 = fmaf(c.hi, d.hi, -p2);
    e2 = fmaf(c.hi, d.lo, e2);
    e2 = fmaf(c.lo, d.hi, e2);
    float e3 = fmaf(e.hi, f.hi, -p3);
    e3 = fmaf(e.hi, f.lo, e3);
    e3 = fmaf(e.lo, f.hi, e3);
    float e4 = fmaf(g.hi, h.hi, -p4);
    e4 = fmaf(g.hi, h.lo, e4);
    e4 = fmaf(g.lo, h.hi, e4);
    const df t1 = two_sum_df(acc.hi, p1);
    const df t2 = two_sum_df(t1.hi, p2);
    const df t3 = two_sum_df(t2.hi, p3);
    const df t4 = two_sum_df(t3.hi, p4);
    acc.hi = t4.hi;
    const float lo = __fadd_rn(__fadd_rn(t1.lo, t2.lo), __fadd_rn(t3.lo, t4.lo));
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(lo, __fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, e4))));
}

// acc += x without renormalising acc (the running low part absorbs the
// rounding errors; fold before converting)
__device__ __forceinline__ void acc_add(df &acc, df x)
{
    const df t = two_sum_df(acc.hi, x.hi);
    acc.hi = t.hi;
    acc.lo = __fadd_rn(acc.lo, __fadd_rn(t.lo, x.lo));
}

// exact scaling by a power of two
__device__ __forceinline__ df scale2(df a, float p2) { return {__fmul_rn(a.hi, p2), __fmul_rn(a.lo, p2)}; }

__device__ __forceinline__ df sqr(df a)
{
    const float p = __fmul_rn(a.hi, a.hi);
    float e = fmaf(a.hi, a.hi, -p);
    e = fmaf(2.0f * a.hi, a.lo, e);
    return fast_two_sum(p, e);
}

// exact product of two floats
__device__ __forceinline__ df two_prod(float a, float b)
{
    const float p = __fmul_rn(a, b);
    return {p, fmaf(a, b, -p)};
}

// 1/sqrt(x): hardware estimate, one FP32 Newton step (to ~1 ulp of float),
// then one Newton step in double-float: y1 = y + y (1 - x y^2) / 2, where the
// residual 1 - x y^2 is formed in double-float and the (tiny) correction in
// FP32.  Relative error ~ 1.5 * (2^-24)^2 + 2^-47.
__device__ __forceinline__ df rsqrt_df(df x)
{
    float y = rsqrtf(x.hi);
    y = y * fmaf(-0.5f * x.hi, y * y, 1.5f);
    const df t = mul_u(x, two_prod(y, y));
    const float e = __fsub_rn(__fsub_rn(1.0f, t.hi), t.lo);
    return fast_two_sum(y, __fmul_rn(__fmul_rn(0.5f, y), e));
}

__device__ __forceinline__ bool operator>(df a, float b) { return a.hi > b || (a.hi == b && a.lo > 0.0f); }
__device__ __forceinline__ bool operator>=(df a, float b) { return a.hi > b || (a.hi == b && a.lo >= 0.0f); }

__device__ __forceinline__ double to_double(df a) { return (double)a.hi + (double)a.lo; }

// double -> double-float (round hi, exact remainder in lo)
__device__ __forceinline__ df df_of_double(double d)
{
    const float h = (float)d;
    return {h, (float)(d - (double)h)};
}

}  // namespace rmw
