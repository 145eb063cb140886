// Arithmetic policies of the 7-point star update
//   u_new = c0*u + cx*(w+e) + cy*(s+n) + cz*(b+t) + cf*F
// in FP64, plain FP32 and compensated FP32 pairs, shared by the plain sweep
// and the batched ensemble kernels.
#pragma once

#include "star7.cuh"

namespace scafes {

// ---- arithmetic policies ---------------------------------------------------

struct PolF64 {
    using T = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from_double(double d) { return d; }
    static __device__ __forceinline__ double to_double(T v) { return v; }
    template <bool HAS_F>
    static __device__ __forceinline__ T star(const Star7Coeffs& c, T u, T w, T e,
                                             T s, T n, T b, T t, T f) {
        double v = c.c0 * u;
        v = fma(c.cx, w + e, v);
        v = fma(c.cy, s + n, v);
        v = fma(c.cz, b + t, v);
        if (HAS_F) v = fma(c.cf, f, v);
        return v;
    }
    static __device__ __forceinline__ T mirror(T u, T uo, const Split& corr) {
        return (u + uo) - corr.d;
    }
    static __device__ __forceinline__ T src(T fa, T fb, const Split& time, bool has_b) {
        return has_b ? fa + time.d * fb : fa;
    }
};

struct PolF32 {
    using T = float;
    static __device__ __forceinline__ T zero() { return 0.0f; }
    static __device__ __forceinline__ T from_double(double d) { return (float)d; }
    static __device__ __forceinline__ double to_double(T v) { return (double)v; }
    template <bool HAS_F>
    static __device__ __forceinline__ T star(const Star7Coeffs& c, T u, T w, T e,
                                             T s, T n, T b, T t, T f) {
        float v = c.c0h * u;
        v = fmaf(c.cxh, w + e, v);
        v = fmaf(c.cyh, s + n, v);
        v = fmaf(c.czh, b + t, v);
        if (HAS_F) v = fmaf(c.cfh, f, v);
        return v;
    }
    static __device__ __forceinline__ T mirror(T u, T uo, const Split& corr) {
        return (u + uo) - corr.hi;
    }
    static __device__ __forceinline__ T src(T fa, T fb, const Split& time, bool has_b) {
        return has_b ? fmaf(time.hi, fb, fa) : fa;
    }
};

// Compensated FP32 pair.  The value of a node is hi + lo.  The update
// computes the exact sums of the hi parts per axis (TwoSum), the exact
// products of those sums with the hi part of each coefficient (FMA TwoProd)
// and their exact sum (TwoSum); everything of relative size 2^-24 (lo parts,
// coefficient tails, rounding errors) is accumulated in plain FP32, which
// contributes errors of relative size 2^-48 that average out over steps.
// Each coefficient is carried to ~72 bits (hi + lo + lo2): a coefficient
// rounded to 48 bits would perturb the operator itself, and that error
// would grow linearly with the number of steps.  A final FastTwoSum
// renormalises the pair.
struct PolF32x2 {
    using T = float2;
    static __device__ __forceinline__ T zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ T from_double(double d) {
        f2 p = split_double(d);
        return make_float2(p.hi, p.lo);
    }
    static __device__ __forceinline__ double to_double(T v) { return (double)v.x + (double)v.y; }
    template <bool HAS_F>
    static __device__ __forceinline__ T star(const Star7Coeffs& c, T u, T w, T e,
                                             T s, T n, T b, T t, T f) {
        // Pair sums per axis: exact hi sum + FP32 tail.
        f2 sx = two_sum(w.x, e.x);
        f2 sy = two_sum(s.x, n.x);
        f2 sz = two_sum(b.x, t.x);
        float tx = sx.lo + (w.y + e.y);
        float ty = sy.lo + (s.y + n.y);
        float tz = sz.lo + (b.y + t.y);
        // Products with the hi coefficient, exact via FMA; tails in FP32.
        float p0 = c.c0h * u.x;
        float r0 = fmaf(c.c0h, u.x, -p0);
        r0 = fmaf(c.c0l, u.x, r0);
        r0 = fmaf(c.c0h, u.y, r0);
        r0 = fmaf(c.c0ll, u.x, r0);
        float px = c.cxh * sx.hi;
        float rx = fmaf(c.cxh, sx.hi, -px);
        rx = fmaf(c.cxl, sx.hi, rx);
        rx = fmaf(c.cxh, tx, rx);
        rx = fmaf(c.cxll, sx.hi, rx);
        float py = c.cyh * sy.hi;
        float ry = fmaf(c.cyh, sy.hi, -py);
        ry = fmaf(c.cyl, sy.hi, ry);
        ry = fmaf(c.cyh, ty, ry);
        ry = fmaf(c.cyll, sy.hi, ry);
        float pz = c.czh * sz.hi;
        float rz = fmaf(c.czh, sz.hi, -pz);
        rz = fmaf(c.czl, sz.hi, rz);
        rz = fmaf(c.czh, tz, rz);
        rz = fmaf(c.czll, sz.hi, rz);
        // Exact sum of the main products.
        f2 a1 = two_sum(p0, px);
        f2 a2 = two_sum(a1.hi, py);
        f2 a3 = two_sum(a2.hi, pz);
        float r = ((r0 + rx) + (ry + rz)) + ((a1.lo + a2.lo) + a3.lo);
        float hi = a3.hi;
        if (HAS_F) {
            float pf = c.cfh * f.x;
            float rf = fmaf(c.cfh, f.x, -pf);
            rf = fmaf(c.cfl, f.x, rf);
            rf = fmaf(c.cfh, f.y, rf);
            rf = fmaf(c.cfll, f.x, rf);
            f2 a4 = two_sum(hi, pf);
            hi = a4.hi;
            r += rf + a4.lo;
        }
        f2 out = fast_two_sum(hi, r);
        return make_float2(out.hi, out.lo);
    }
    static __device__ __forceinline__ T mirror(T u, T uo, const Split& corr) {
        // (u + uo) - corr with corr a power of two (exact in FP32).
        f2 s = two_sum(u.x, uo.x);
        float lo = s.lo + (u.y + uo.y);
        f2 d = two_sum(s.hi, -corr.hi);
        f2 out = fast_two_sum(d.hi, d.lo + lo);
        return make_float2(out.hi, out.lo);
    }
    static __device__ __forceinline__ T src(T fa, T fb, const Split& time, bool has_b) {
        if (!has_b) return fa;
        // fa + time * fb in pair arithmetic with time split on the host: no
        // FP64 instruction on this path (a predicated FP64 instruction would
        // still occupy the GB300's narrow FP64 pipe in every lane).
        float p = time.hi * fb.x;
        float e = fmaf(time.hi, fb.x, -p);
        e = fmaf(time.hi, fb.y, e);
        e = fmaf(time.lo, fb.x, e);
        f2 s = two_sum(fa.x, p);
        f2 out = fast_two_sum(s.hi, s.lo + (fa.y + e));
        return make_float2(out.hi, out.lo);
    }
};


}  // namespace scafes
