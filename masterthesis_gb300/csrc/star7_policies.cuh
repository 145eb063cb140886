// Arithmetic policies of the 7-point star update
//   u_new = c0*u + cx*(w+e) + cy*(s+n) + cz*(b+t) + cf*F
// in FP64, plain FP32 and compensated FP32 pairs, shared by the plain sweep
// and the batched ensemble kernels.
#pragma once

#include "dadd_int.cuh"
#include "star7.cuh"

namespace scafes {

// ---- arithmetic policies ---------------------------------------------------

struct PolF64 {
    using T = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from_double(double d) { return d; }
    static __device__ __forceinline__ double to_double(T v) { return v; }
    static __device__ __forceinline__ double int_sum(double a, double b, bool& ok, bool skip) {
        bool o;
        const uint64_t r = dadd_same_sign_bits((uint64_t)__double_as_longlong(a),
                                               (uint64_t)__double_as_longlong(b), o);
        ok = ok && (o || skip);
        return __longlong_as_double((long long)r);
    }
    // The three neighbour sums of R nodes, sx/sy/sz[k] = w+e, s+n, b+t of
    // node k, added on the integer pipe (dadd_int.cuh: the FP64 adder's
    // exact bits) instead of the FP64 pipe, which bounds the FP64 sweep.  A
    // warp with a lane outside the integer adder's range (a zero border
    // value, opposite signs) adds that axis's sums in FP64, in a call: a
    // predicated FP64 add inline would hold the FP64 pipe in every warp.
    // Bit k of `skip` marks row k's result as replaced (a border rule, or
    // not stored): its sums do not call for the FP64 adds.
    template <int R>
    static __device__ __forceinline__ void sums(const T (&w)[R], const T (&e)[R], const T (&s)[R], const T (&n)[R],
                                                const T (&b)[R], const T (&t)[R], T (&sx)[R], T (&sy)[R],
                                                T (&sz)[R], unsigned skip) {
        bool okx = true, oky = true, okz = true;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const bool sk = (skip >> k) & 1u;
            sx[k] = int_sum(w[k], e[k], okx, sk);
            sy[k] = int_sum(s[k], n[k], oky, sk);
            sz[k] = int_sum(b[k], t[k], okz, sk);
        }
        const unsigned lanes = __activemask();
        if (__any_sync(lanes, !okx)) fp64_sums<R>(w, e, sx);
        if (__any_sync(lanes, !oky)) fp64_sums<R>(s, n, sy);
        if (__any_sync(lanes, !okz)) fp64_sums<R>(b, t, sz);
    }
    template <int R>
    struct Nodes {
        double v[R];
    };
    template <int R>
    static __device__ __noinline__ Nodes<R> fp64_add(Nodes<R> a, Nodes<R> b) {
        Nodes<R> r;
#pragma unroll
        for (int k = 0; k < R; ++k) r.v[k] = a.v[k] + b.v[k];
        return r;
    }
    template <int R>
    static __device__ __forceinline__ void fp64_sums(const T (&a)[R], const T (&b)[R], T (&out)[R]) {
        Nodes<R> x, y;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            x.v[k] = a[k];
            y.v[k] = b[k];
        }
        const Nodes<R> r = fp64_add<R>(x, y);
#pragma unroll
        for (int k = 0; k < R; ++k) out[k] = r.v[k];
    }
    template <bool HAS_F>
    static __device__ __forceinline__ T star_of_sums(const Star7Coeffs& c, T u, T sx, T sy, T sz, T f) {
        double v = c.c0 * u;
        v = fma(c.cx, sx, v);
        v = fma(c.cy, sy, v);
        v = fma(c.cz, sz, v);
        if (HAS_F) v = fma(c.cf, f, v);
        return v;
    }
    template <bool HAS_F>
    static __device__ __forceinline__ T star(const Star7Coeffs& c, T u, T w, T e,
                                             T s, T n, T b, T t, T f) {
        T sx[1], sy[1], sz[1];
        const T w1[1] = {w}, e1[1] = {e}, s1[1] = {s}, n1[1] = {n}, b1[1] = {b}, t1[1] = {t};
        sums<1>(w1, e1, s1, n1, b1, t1, sx, sy, sz, 0u);
        return star_of_sums<HAS_F>(c, u, sx[0], sy[0], sz[0], f);
    }
    static __device__ __forceinline__ T mirror(T u, T uo, const Split& corr) {
        return (u + uo) - corr.d;
    }
    static __device__ __forceinline__ T src(T fa, T fb, const Split& time, bool has_b) {
        return has_b ? fa + time.d * fb : fa;
    }

    // Variable coefficients: c0x * u + cax * (cx (w+e) + cy (s+n) + cz (b+t))
    // + f, with the node's own C0 and CA and the source with weight 1
    // (8 FP64 operations, the three sums on the integer pipe as in sums()).
    template <bool HAS_F>
    static __device__ __forceinline__ T star_vc_of_sums(const Star7Coeffs& c, T u, T sx, T sy, T sz, T f, T c0x,
                                                        T cax) {
        double l = c.cx * sx;
        l = fma(c.cy, sy, l);
        l = fma(c.cz, sz, l);
        const double v = HAS_F ? fma(c0x, u, f) : c0x * u;
        return fma(cax, l, v);
    }
    template <bool HAS_F>
    static __device__ __forceinline__ T star_vc(const Star7Coeffs& c, T u, T w, T e, T s, T n, T b, T t, T f,
                                                T c0x, T cax) {
        T sx[1], sy[1], sz[1];
        const T w1[1] = {w}, e1[1] = {e}, s1[1] = {s}, n1[1] = {n}, b1[1] = {b}, t1[1] = {t};
        sums<1>(w1, e1, s1, n1, b1, t1, sx, sy, sz, 0u);
        return star_vc_of_sums<HAS_F>(c, u, sx[0], sy[0], sz[0], f, c0x, cax);
    }
    // All R rows of one thread with the coefficients c0[k * stride],
    // ca[k * stride] of row k; `skip` as for star_rows.
    template <bool HAS_F, int R>
    static __device__ __forceinline__ void star_vc_rows(const Star7Coeffs& c, const T (&below)[R],
                                                        const T (&cur)[R], const T (&above)[R], T ym, T yp,
                                                        const T (&w)[R], const T (&e)[R], const T (&f)[R],
                                                        const T* c0, const T* ca, int stride, T (&v)[R],
                                                        unsigned skip) {
        T s[R], n[R], sx[R], sy[R], sz[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            s[k] = k == 0 ? ym : cur[k - 1];
            n[k] = k == R - 1 ? yp : cur[k + 1];
        }
        sums<R>(w, e, s, n, below, above, sx, sy, sz, skip);
#pragma unroll
        for (int k = 0; k < R; ++k)
            v[k] = star_vc_of_sums<HAS_F>(c, cur[k], sx[k], sy[k], sz[k], f[k], c0[k * stride], ca[k * stride]);
    }
    // All R rows of one thread (row k's s/n neighbours are rows k-1/k+1,
    // ym/yp beyond the ends).  Bit k of `skip`: row k's result is replaced
    // by the caller.
    template <bool HAS_F, int R>
    static __device__ __forceinline__ void star_rows(const Star7Coeffs& c, const T (&below)[R], const T (&cur)[R],
                                                     const T (&above)[R], T ym, T yp, const T (&w)[R],
                                                     const T (&e)[R], const T (&f)[R], T (&v)[R],
                                                     unsigned skip = 0u) {
        T s[R], n[R], sx[R], sy[R], sz[R];
#pragma unroll
        for (int k = 0; k < R; ++k) {
            s[k] = k == 0 ? ym : cur[k - 1];
            n[k] = k == R - 1 ? yp : cur[k + 1];
        }
        sums<R>(w, e, s, n, below, above, sx, sy, sz, skip);
#pragma unroll
        for (int k = 0; k < R; ++k) v[k] = star_of_sums<HAS_F>(c, cur[k], sx[k], sy[k], sz[k], f[k]);
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
    template <bool HAS_F>
    static __device__ __forceinline__ T star_vc(const Star7Coeffs& c, T u, T w, T e, T s, T n, T b, T t, T f,
                                                T c0x, T cax) {
        float l = c.cxh * (w + e);
        l = fmaf(c.cyh, s + n, l);
        l = fmaf(c.czh, b + t, l);
        const float v = HAS_F ? fmaf(c0x, u, f) : c0x * u;
        return fmaf(cax, l, v);
    }
    template <bool HAS_F, int R>
    static __device__ __forceinline__ void star_vc_rows(const Star7Coeffs& c, const T (&below)[R],
                                                        const T (&cur)[R], const T (&above)[R], T ym, T yp,
                                                        const T (&w)[R], const T (&e)[R], const T (&f)[R],
                                                        const T* c0, const T* ca, int stride, T (&v)[R],
                                                        unsigned) {
#pragma unroll
        for (int k = 0; k < R; ++k)
            v[k] = star_vc<HAS_F>(c, cur[k], w[k], e[k], k == 0 ? ym : cur[k - 1], k == R - 1 ? yp : cur[k + 1],
                                  below[k], above[k], f[k], c0[k * stride], ca[k * stride]);
    }
    // All R rows of one thread (row k's s/n neighbours are rows k-1/k+1,
    // ym/yp beyond the ends).
    template <bool HAS_F, int R>
    static __device__ __forceinline__ void star_rows(const Star7Coeffs& c, const T (&below)[R], const T (&cur)[R],
                                                     const T (&above)[R], T ym, T yp, const T (&w)[R],
                                                     const T (&e)[R], const T (&f)[R], T (&v)[R],
                                                     unsigned skip = 0u) {
#pragma unroll
        for (int k = 0; k < R; ++k)
            v[k] = star<HAS_F>(c, cur[k], w[k], e[k], k == 0 ? ym : cur[k - 1], k == R - 1 ? yp : cur[k + 1],
                               below[k], above[k], f[k]);
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
    // Two rows at once on the paired FP32 instructions of sm_100+ (FFMA2,
    // FADD2, FMUL2): component .x carries row k, .y row k+1, with exactly the
    // operations of star() per component, so the results are bit-identical
    // while half the arithmetic instructions are issued.  The main products
    // are formed negated (a negated coefficient times the value is exact),
    // so the FMA TwoProd takes -p without a separate negation; TwoSum and
    // FastTwoSum are symmetric under negation, and the result is negated
    // back at the end.
    template <bool HAS_F>
    static __device__ __forceinline__ void star2(const Star7Coeffs& c, T u0, T u1, T w0, T w1, T e0, T e1,
                                                 T s0, T s1, T n0, T n1, T b0, T b1, T t0, T t1, T f0, T f1,
                                                 T& o0, T& o1) {
        const float2 M1 = make_float2(-1.f, -1.f);
        auto bc = [](float v) { return make_float2(v, v); };
        auto sub = [&](float2 a, float2 b) { return __ffma2_rn(b, M1, a); };  // a - b, one rounding
        auto tsum = [&](float2 a, float2 b, float2& err) {
            const float2 sm = __fadd2_rn(a, b);
            const float2 bb = sub(sm, a);
            err = __fadd2_rn(sub(a, sub(sm, bb)), sub(b, bb));
            return sm;
        };
        auto hi = [](T a, T b) { return make_float2(a.x, b.x); };
        auto lo = [](T a, T b) { return make_float2(a.y, b.y); };
        // Axis sums: exact hi sums + FP32 tails.
        float2 ex, ey, ez;
        const float2 SX = tsum(hi(w0, w1), hi(e0, e1), ex);
        const float2 SY = tsum(hi(s0, s1), hi(n0, n1), ey);
        const float2 SZ = tsum(hi(b0, b1), hi(t0, t1), ez);
        const float2 TX = __fadd2_rn(ex, __fadd2_rn(lo(w0, w1), lo(e0, e1)));
        const float2 TY = __fadd2_rn(ey, __fadd2_rn(lo(s0, s1), lo(n0, n1)));
        const float2 TZ = __fadd2_rn(ez, __fadd2_rn(lo(b0, b1), lo(t0, t1)));
        const float2 UH = hi(u0, u1), UL = lo(u0, u1);
        // Negated main products and their (positive) FP32 tails.
        const float2 NP0 = __fmul2_rn(bc(-c.c0h), UH);
        float2 R0 = __ffma2_rn(bc(c.c0h), UH, NP0);
        R0 = __ffma2_rn(bc(c.c0l), UH, R0);
        R0 = __ffma2_rn(bc(c.c0h), UL, R0);
        R0 = __ffma2_rn(bc(c.c0ll), UH, R0);
        const float2 NPX = __fmul2_rn(bc(-c.cxh), SX);
        float2 RX = __ffma2_rn(bc(c.cxh), SX, NPX);
        RX = __ffma2_rn(bc(c.cxl), SX, RX);
        RX = __ffma2_rn(bc(c.cxh), TX, RX);
        RX = __ffma2_rn(bc(c.cxll), SX, RX);
        const float2 NPY = __fmul2_rn(bc(-c.cyh), SY);
        float2 RY = __ffma2_rn(bc(c.cyh), SY, NPY);
        RY = __ffma2_rn(bc(c.cyl), SY, RY);
        RY = __ffma2_rn(bc(c.cyh), TY, RY);
        RY = __ffma2_rn(bc(c.cyll), SY, RY);
        const float2 NPZ = __fmul2_rn(bc(-c.czh), SZ);
        float2 RZ = __ffma2_rn(bc(c.czh), SZ, NPZ);
        RZ = __ffma2_rn(bc(c.czl), SZ, RZ);
        RZ = __ffma2_rn(bc(c.czh), TZ, RZ);
        RZ = __ffma2_rn(bc(c.czll), SZ, RZ);
        // Exact sum of the negated products.
        float2 a1, a2, a3;
        const float2 H1 = tsum(NP0, NPX, a1);
        const float2 H2 = tsum(H1, NPY, a2);
        float2 NH = tsum(H2, NPZ, a3);
        // Negated tail: -(((r0 + rx) + (ry + rz)) + ((a1 + a2) + a3)).
        const float2 rt = __fadd2_rn(__fadd2_rn(R0, RX), __fadd2_rn(RY, RZ));
        float2 NR = sub(__fadd2_rn(__fadd2_rn(a1, a2), a3), rt);
        if (HAS_F) {
            const float2 FH = hi(f0, f1), FL = lo(f0, f1);
            const float2 NPF = __fmul2_rn(bc(-c.cfh), FH);
            float2 RF = __ffma2_rn(bc(c.cfh), FH, NPF);
            RF = __ffma2_rn(bc(c.cfl), FH, RF);
            RF = __ffma2_rn(bc(c.cfh), FL, RF);
            RF = __ffma2_rn(bc(c.cfll), FH, RF);
            float2 a4;
            NH = tsum(NH, NPF, a4);
            NR = sub(NR, sub(RF, a4));
        }
        // FastTwoSum of the negated pair, then negate back.
        const float2 S = __fadd2_rn(NH, NR);
        const float2 E = sub(NR, sub(S, NH));
        o0 = make_float2(-S.x, -E.x);
        o1 = make_float2(-S.y, -E.y);
    }

    template <bool HAS_F, int R>
    static __device__ __forceinline__ void star_rows(const Star7Coeffs& c, const T (&below)[R], const T (&cur)[R],
                                                     const T (&above)[R], T ym, T yp, const T (&w)[R],
                                                     const T (&e)[R], const T (&f)[R], T (&v)[R],
                                                     unsigned skip = 0u) {
#pragma unroll
        for (int k = 0; k + 1 < R; k += 2) {
            const T s0 = k == 0 ? ym : cur[k - 1];
            const T n1 = k + 1 == R - 1 ? yp : cur[k + 2];
            star2<HAS_F>(c, cur[k], cur[k + 1], w[k], w[k + 1], e[k], e[k + 1], s0, cur[k], cur[k + 1], n1,
                         below[k], below[k + 1], above[k], above[k + 1], f[k], f[k + 1], v[k], v[k + 1]);
        }
        if (R % 2 == 1) {
            const int k = R - 1;
            v[k] = star<HAS_F>(c, cur[k], w[k], e[k], k == 0 ? ym : cur[k - 1], yp, below[k], above[k], f[k]);
        }
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
