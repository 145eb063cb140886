// Multi-field leapfrog workloads: the Lame-Navier elastic wave (3
// displacement components, mixed second derivatives) and the Yee FDTD
// scheme for Maxwell's equations (6 staggered fields).
//
// In ScaFES these are problems with several unknown data fields and a
// second update phase (the leapfrog "update2" of src/ScaFES_Problem.hpp:
// 2604-2619, :2875-2918).  The Yee problem of the reference
// (examples/EMFDTD/EMFDTD.hpp:295-385: H in updateInner, D/E/I in
// updateInner2) is not built by the reference (examples/Makefile.am:14) and
// its Lame-Navier example cannot advance (examples/LameNavierEqnFDM/
// LameNavierEqnFDM.hpp:23-25: only one old time level is exposed), so the
// schemes here follow the textbook forms written out in the oracle
// (orc_lame, orc_yee), which the tests use as the reference.
//
// Both are FP64-issue-bound on GB300 (Lame: ~57 FP64 operations per node,
// Yee: ~24 per cell and step), so the kernels read neighbours straight from
// global memory through L1 instead of staging tiles: one thread per (x, y)
// column marches a chunk of 16 z-planes.  The FP32-pair Lame kernel
// (k_lame_x2_tma) stages the three components through TMA instead (its
// pair arithmetic needs the loads' latency hidden); FP32 and FP32-pair Yee
// run the fused one-pass step (k_yee_tma) below.
#include <cstdarg>
#include <cmath>
#include <cstdio>
#include <string>

#include "scafes_common.cuh"
#include "star7.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

using namespace scafes;

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

constexpr int MX = 32, MY = 8, MZ = 16;

struct LameCoef {
    double a[3][3];   // a[c][p]: weight of d_pp on component c (includes tau^2/rho/h_p^2)
    double b[3][3];   // b[c][q]: weight of d_cq u_q (includes tau^2/rho/(4 h_c h_q))
};

// u_new (written over uprev) = 2u - uprev + sum ... on inner nodes; 0 on border.
__global__ void __launch_bounds__(MX * MY)
k_lame(const double* __restrict__ u, double* __restrict__ up, LameCoef K, Layout L, long long comp) {
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
    const long long st[3] = {1, L.pitch, L.plane};
    const int z0 = blockIdx.z * MZ, z1 = min(z0 + MZ, L.nz);
    for (int z = z0; z < z1; ++z) {
        const long long m = L.idx(x, y, z);
        if (colb || z == 0 || z == L.nz - 1) {
            up[m] = 0.0;
            up[m + comp] = 0.0;
            up[m + 2 * comp] = 0.0;
            continue;
        }
        double out[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const double* uc = u + c * comp;
            const double uv = uc[m];
            double acc = 2.0 * uv - up[m + c * comp];
#pragma unroll
            for (int p = 0; p < 3; ++p)
                acc = fma(K.a[c][p], (uc[m + st[p]] + uc[m - st[p]]) - 2.0 * uv, acc);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q == c) continue;
                const double* uq = u + q * comp;
                const long long sp = st[c], sq = st[q];
                acc = fma(K.b[c][q], (uq[m + sp + sq] - uq[m + sp - sq]) - (uq[m - sp + sq] - uq[m - sp - sq]), acc);
            }
            out[c] = acc;
        }
        up[m] = out[0];
        up[m + comp] = out[1];
        up[m + 2 * comp] = out[2];
    }
}

// Yee H half step (see orc_yee for the staggering).
template <class T>
__global__ void __launch_bounds__(MX * MY)
k_yee_h(const T* __restrict__ ex, const T* __restrict__ ey, const T* __restrict__ ez, T* __restrict__ hx,
        T* __restrict__ hy, T* __restrict__ hz, Layout L, T ch) {
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const int z0 = blockIdx.z * MZ, z1 = min(z0 + MZ, L.nz);
    for (int z = z0; z < z1; ++z) {
        const long long m = L.idx(x, y, z);
        const bool xi = x + 1 < L.nx, yi = y + 1 < L.ny, zi = z + 1 < L.nz;
        if (yi && zi) hx[m] -= ch * ((ez[m + L.pitch] - ez[m]) - (ey[m + L.plane] - ey[m]));
        if (xi && zi) hy[m] -= ch * ((ex[m + L.plane] - ex[m]) - (ez[m + 1] - ez[m]));
        if (xi && yi) hz[m] -= ch * ((ey[m + 1] - ey[m]) - (ex[m + L.pitch] - ex[m]));
    }
}

// Yee E step with PEC walls and the soft current source.
template <class T>
__global__ void __launch_bounds__(MX * MY)
k_yee_e(T* __restrict__ ex, T* __restrict__ ey, T* __restrict__ ez, const T* __restrict__ hx,
        const T* __restrict__ hy, const T* __restrict__ hz, Layout L, T ch, long long src, T src_val) {
    const int x = blockIdx.x * MX + threadIdx.x, y = blockIdx.y * MY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const int z0 = blockIdx.z * MZ, z1 = min(z0 + MZ, L.nz);
    const bool xin = x > 0 && x + 1 < L.nx, yin = y > 0 && y + 1 < L.ny;
    for (int z = z0; z < z1; ++z) {
        const long long m = L.idx(x, y, z);
        const bool zin = z > 0 && z + 1 < L.nz;
        if (x + 1 < L.nx && yin && zin) ex[m] += ch * ((hz[m] - hz[m - L.pitch]) - (hy[m] - hy[m - L.plane]));
        if (y + 1 < L.ny && xin && zin) ey[m] += ch * ((hx[m] - hx[m - L.plane]) - (hz[m] - hz[m - 1]));
        if (z + 1 < L.nz && xin && yin) {
            T v = ez[m] + ch * ((hy[m] - hy[m - 1]) - (hx[m] - hx[m - L.pitch]));
            if (m == src) v -= src_val;
            ez[m] = v;
        }
    }
}

// ---- compensated FP32 pairs (SCAFES_PREC_F32X2) -----------------------------
//
// Each value is a pair hi + lo of floats (8 bytes, as FP64).  A node update
// is a sum of products c * S of host-split coefficients (c = h + l + ll,
// ~72 bits) and operands S formed from neighbour differences or sums whose
// hi parts are combined exactly (TwoSum) and whose lo parts and rounding
// errors ride along in an FP32 tail.  The products' hi parts are exact
// (FMA TwoProd) and summed with TwoSum; everything of relative size 2^-24
// goes into one FP32 error term, so a step carries errors of relative size
// about 2^-48, and the pair is renormalised once per node (FastTwoSum).
// No FP64 instruction is issued.

struct C3 { float h, l, ll; };

C3 split3(double d) {
    C3 c;
    c.h = (float)d;
    const double r = d - (double)c.h;
    c.l = (float)r;
    c.ll = (float)(r - (double)c.l);
    return c;
}

struct LameCoefX2 {
    C3 d[3];      // centre weight of component c: 2 - 2 sum_p a[c][p]
    C3 a[3][3];   // as LameCoef
    C3 b[3][3];
};

// An operand S + t: hi part exact, t its FP32 tail.
struct Op { float s, t; };

__device__ __forceinline__ Op op_diff(float2 a, float2 b) {
    const f2 r = two_sum(a.x, -b.x);
    return {r.hi, r.lo + (a.y - b.y)};
}

// (a - b) - (c - d)
__device__ __forceinline__ Op op_diff2(float2 a, float2 b, float2 c, float2 d) {
    const Op p = op_diff(a, b), q = op_diff(c, d);
    const f2 r = two_sum(p.s, -q.s);
    return {r.hi, r.lo + (p.t - q.t)};
}

// Running sum: H exact-ish hi, E the FP32 error term.
struct PAcc { float H, E; };

// acc += c * (S + t)
__device__ __forceinline__ void pa_prod(PAcc& acc, const C3& c, Op o) {
    const float p = c.h * o.s;
    float e = fmaf(c.h, o.s, -p);
    e = fmaf(c.l, o.s, e);
    e = fmaf(c.h, o.t, e);
    e = fmaf(c.ll, o.s, e);
    const f2 r = two_sum(acc.H, p);
    acc.H = r.hi;
    acc.E += r.lo + e;
}

// acc += sign * v (a pair)
__device__ __forceinline__ void pa_add(PAcc& acc, float2 v, float sign) {
    const f2 r = two_sum(acc.H, sign * v.x);
    acc.H = r.hi;
    acc.E += r.lo + sign * v.y;
}

__device__ __forceinline__ float2 pa_result(PAcc acc) {
    const f2 r = fast_two_sum(acc.H, acc.E);
    return make_float2(r.hi, r.lo);
}

// Lame-Navier step on pairs: u^{n+1} = d_c u + sum_p a_cp (u(+p) + u(-p))
// + sum_q b_cq ((u_q(+c+q) - u_q(+c-q)) - (u_q(-c+q) - u_q(-c-q))) - u^{n-1},
// the FP64 form rearranged with the centre weight d_c = 2 - 2 sum_p a_cp.
// The three components of u^n are staged by TMA: a CTA owns an LX x LY
// column tile (LX x LY/2 threads, two rows each) and marches LZ planes; per
// input plane one mbarrier covers the three components' boxes with a
// one-node halo in x and y (x from x0-2 for 16-byte alignment), in a ring
// of LNS planes: planes z-1, z, z+1 are read from shared memory while the
// next LNS-3 are in flight.  u^{n-1} is read a plane ahead and u^{n+1}
// written with plain coalesced accesses of the nodes themselves.  The terms
// come in the order of the FP64 kernel's.  Every wait is bounded (status
// word, drain, return).
constexpr int LX = 32, LY = 8, LZ = 32, LNS = 6;
constexpr int LBW = LX + 4, LBH = LY + 2;                     // box: x0-2 .. x0+33, y0-1 .. y0+8
constexpr int LBOX = (LBW * LBH + 15) / 16 * 16;              // float2 per box, 128-byte multiple
constexpr int LSLOT = 3 * LBOX;                               // float2 per ring slot
constexpr uint32_t LTX_BYTES = (uint32_t)(3 * LBW * LBH * 8);
constexpr size_t LAME_SMEM = (size_t)LNS * LSLOT * 8 + LNS * 8;

// Two nodes per thread (rows y and y+1) on the paired FP32 instructions of
// sm_100+ (FFMA2, FADD2, FMUL2): lane .x carries the first node, .y the
// second, with exactly the operations of pa_prod / pa_add / op_sum /
// op_diff2 / pa_result per lane (bit-identical to the one-node form) and
// half the arithmetic instructions issued.
struct PAcc2 { float2 H, E; };

__device__ __forceinline__ float2 bc2(float v) { return make_float2(v, v); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // a - b, one rounding
    return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
}
__device__ __forceinline__ float2 tsum2(float2 a, float2 b, float2& err) {
    const float2 sm = __fadd2_rn(a, b);
    const float2 bb = sub2(sm, a);
    err = __fadd2_rn(sub2(a, sub2(sm, bb)), sub2(b, bb));
    return sm;
}
__device__ __forceinline__ float2 hi2(float2 a, float2 b) { return make_float2(a.x, b.x); }
__device__ __forceinline__ float2 lo2(float2 a, float2 b) { return make_float2(a.y, b.y); }

// (S, t) of a + b for the two nodes' pairs (a0, a1), (b0, b1).
__device__ __forceinline__ void op_sum2(float2 a0, float2 a1, float2 b0, float2 b1, float2& S, float2& t) {
    float2 e;
    S = tsum2(hi2(a0, a1), hi2(b0, b1), e);
    t = __fadd2_rn(e, __fadd2_rn(lo2(a0, a1), lo2(b0, b1)));
}
// (S, t) of a - b.
__device__ __forceinline__ void op_diff_2(float2 ah, float2 al, float2 bh, float2 bl, float2& S, float2& t) {
    float2 e;
    S = tsum2(ah, make_float2(-bh.x, -bh.y), e);
    t = __fadd2_rn(e, sub2(al, bl));
}
// (S, t) of (a - b) - (c - d).
__device__ __forceinline__ void op_diff2_2(float2 a0, float2 a1, float2 b0, float2 b1, float2 c0, float2 c1,
                                           float2 d0, float2 d1, float2& S, float2& t) {
    float2 ps, pt, qs, qt, e;
    op_diff_2(hi2(a0, a1), lo2(a0, a1), hi2(b0, b1), lo2(b0, b1), ps, pt);
    op_diff_2(hi2(c0, c1), lo2(c0, c1), hi2(d0, d1), lo2(d0, d1), qs, qt);
    S = tsum2(ps, make_float2(-qs.x, -qs.y), e);
    t = __fadd2_rn(e, sub2(pt, qt));
}
// acc += c * (S + t): the negated tail chain -e (exact negation of pa_prod's
// e, its roundings being symmetric), added back as E + (r - (-e)).
__device__ __forceinline__ void pa_prod2(PAcc2& acc, const C3& c, float2 S, float2 t) {
    const float2 P = __fmul2_rn(bc2(c.h), S);
    float2 ne = __ffma2_rn(bc2(-c.h), S, P);
    ne = __ffma2_rn(bc2(-c.l), S, ne);
    ne = __ffma2_rn(bc2(-c.h), t, ne);
    ne = __ffma2_rn(bc2(-c.ll), S, ne);
    float2 r;
    acc.H = tsum2(acc.H, P, r);
    acc.E = __fadd2_rn(acc.E, sub2(r, ne));
}
// acc -= v for the two nodes' pairs v0, v1.
__device__ __forceinline__ void pa_sub2(PAcc2& acc, float2 v0, float2 v1) {
    const float2 vh = hi2(v0, v1), vl = lo2(v0, v1);
    float2 r;
    acc.H = tsum2(acc.H, make_float2(-vh.x, -vh.y), r);
    acc.E = __fadd2_rn(acc.E, sub2(r, vl));
}
__device__ __forceinline__ void pa_result2(const PAcc2& acc, float2& o0, float2& o1) {
    const float2 S = __fadd2_rn(acc.H, acc.E);
    const float2 E = sub2(acc.E, sub2(S, acc.H));
    o0 = make_float2(S.x, E.x);
    o1 = make_float2(S.y, E.y);
}

__global__ void __launch_bounds__(LX * LY / 2)
k_lame_x2_tma(const __grid_constant__ CUtensorMap t0, const __grid_constant__ CUtensorMap t1,
              const __grid_constant__ CUtensorMap t2, float2* __restrict__ up, LameCoefX2 K, Layout L,
              long long comp, int* __restrict__ status) {
    extern __shared__ __align__(128) float2 lsm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(lsm + LNS * LSLOT);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * LX + tx;
    const int x0 = blockIdx.x * LX, y0 = blockIdx.y * LY;
    const int z0 = blockIdx.z * LZ, z1 = min(z0 + LZ, L.nz);
    if (__syncthreads_or(tid == 0 && *(volatile int*)status != 0)) return;
    if (tid == 0) {
        for (int b = 0; b < LNS; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncthreads();
    // Input plane j is z0-1+j (j = 0 .. n_in-1), in ring slot j % LNS.
    const int n_in = z1 - z0 + 2;
    auto issue = [&](int j) {
        const int sl = j % LNS, z = z0 - 1 + j;
        float2* d = lsm + sl * LSLOT;
        mbar_arrive_expect_tx(&bar[sl], LTX_BYTES);
        tma_load_3d(d, &t0, x0 - 2, y0 - 1, z, &bar[sl]);
        tma_load_3d(d + LBOX, &t1, x0 - 2, y0 - 1, z, &bar[sl]);
        tma_load_3d(d + 2 * LBOX, &t2, x0 - 2, y0 - 1, z, &bar[sl]);
    };
    if (tid == 0)
        for (int j = 0; j < LNS && j < n_in; ++j) issue(j);
    auto wait = [&](int j) { return bounded_wait(&bar[j % LNS], (uint32_t)(j / LNS) & 1u); };
    auto fail = [&](int last_issued) {
        if (tid == 0) {
            atomicExch(status, SCAFES_ERR_TIMEOUT);
            for (int j = last_issued - (LNS - 1); j <= last_issued; ++j)
                if (j >= 0 && j < n_in) bounded_wait(&bar[j % LNS], (uint32_t)(j / LNS) & 1u, kWaitLimitNs / 16);
        }
    };
    // This thread's two nodes: rows y and y+1 of column x.
    const int x = x0 + tx, y = y0 + 2 * ty;
    const bool live0 = x < L.nx && y < L.ny, live1 = x < L.nx && y + 1 < L.ny;
    const bool xb = x == 0 || x == L.nx - 1;
    const bool colb0 = xb || y == 0 || y == L.ny - 1, colb1 = xb || y + 1 == 0 || y + 1 == L.ny - 1;
    const int bc = (2 * ty + 1) * LBW + tx + 2;             // first node in a box
    const float2 zero = make_float2(0.f, 0.f);
    bool ok = wait(0);
    ok = wait(1) && ok;
    int issued = min(LNS, n_in) - 1;
    long long o = live0 ? L.idx(x, y, z0) : 0;
    // u^{n-1} of both nodes one plane ahead, in registers.
    float2 pn0[3] = {zero, zero, zero}, pn1[3] = {zero, zero, zero};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (live0) pn0[c] = up[o + c * comp];
        if (live1) pn1[c] = up[o + L.pitch + c * comp];
    }
    for (int z = z0; z < z1; ++z, o += L.plane) {
        const int jc = z - z0 + 1;  // input plane of z
        if (!__syncthreads_and(ok)) {  // plane z-2's slot is free; all waits so far succeeded
            fail(issued);
            return;
        }
        if (tid == 0 && jc + LNS - 2 < n_in && jc + LNS - 2 > issued) {
            fence_proxy_async_smem();
            issue(jc + LNS - 2);
            issued = jc + LNS - 2;
        }
        float2 pc0[3], pc1[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            pc0[c] = pn0[c];
            pc1[c] = pn1[c];
        }
        if (z + 1 < z1)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                if (live0) pn0[c] = up[o + L.plane + c * comp];
                if (live1) pn1[c] = up[o + L.plane + L.pitch + c * comp];
            }
        ok = wait(jc + 1) && ok;  // plane z+1
        if (!live0) continue;
        const bool zb = z == 0 || z == L.nz - 1;
        const float2* pb = lsm + ((jc - 1) % LNS) * LSLOT;  // plane z-1
        const float2* pc = lsm + (jc % LNS) * LSLOT;        // plane z
        const float2* pa = lsm + ((jc + 1) % LNS) * LSLOT;  // plane z+1
        // Component q of u^n at offset (dx, dy, dz) from node r (0, 1).
        auto U = [&](int r, int q, int dx, int dy, int dz) -> float2 {
            const float2* pl = dz < 0 ? pb : (dz > 0 ? pa : pc);
            return pl[q * LBOX + bc + r * LBW + dx + dy * LBW];
        };
        float2 out0[3], out1[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const float2 u0 = U(0, c, 0, 0, 0), u1 = U(1, c, 0, 0, 0);
            PAcc2 acc{make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
            pa_prod2(acc, K.d[c], hi2(u0, u1), lo2(u0, u1));
            pa_sub2(acc, pc0[c], pc1[c]);
#pragma unroll
            for (int p = 0; p < 3; ++p) {
                const int dx = p == 0, dy = p == 1, dz = p == 2;
                float2 S, t;
                op_sum2(U(0, c, dx, dy, dz), U(1, c, dx, dy, dz), U(0, c, -dx, -dy, -dz), U(1, c, -dx, -dy, -dz),
                        S, t);
                pa_prod2(acc, K.a[c][p], S, t);
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                if (q == c) continue;
                // (u_q(+c+q) - u_q(+c-q)) - (u_q(-c+q) - u_q(-c-q))
                const int cx = c == 0, cy = c == 1, cz = c == 2, qx = q == 0, qy = q == 1, qz = q == 2;
                float2 S, t;
                op_diff2_2(U(0, q, cx + qx, cy + qy, cz + qz), U(1, q, cx + qx, cy + qy, cz + qz),
                           U(0, q, cx - qx, cy - qy, cz - qz), U(1, q, cx - qx, cy - qy, cz - qz),
                           U(0, q, -cx + qx, -cy + qy, -cz + qz), U(1, q, -cx + qx, -cy + qy, -cz + qz),
                           U(0, q, -cx - qx, -cy - qy, -cz - qz), U(1, q, -cx - qx, -cy - qy, -cz - qz), S, t);
                pa_prod2(acc, K.b[c][q], S, t);
            }
            pa_result2(acc, out0[c], out1[c]);
        }
        // Border nodes (any face) are held at zero.
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            up[o + c * comp] = (colb0 || zb) ? zero : out0[c];
            if (live1) up[o + L.pitch + c * comp] = (colb1 || zb) ? zero : out1[c];
        }
    }
    if (!__syncthreads_and(ok)) fail(issued);
}

// v + sign * ch * ((a - b) - (c - d)) on pairs.
__device__ __forceinline__ float2 yee_upd(float2 v, const C3& ch, float sign, float2 a, float2 b, float2 c,
                                          float2 d) {
    PAcc acc{v.x, v.y};
    const C3 cs{sign * ch.h, sign * ch.l, sign * ch.ll};
    pa_prod(acc, cs, op_diff2(a, b, c, d));
    return pa_result(acc);
}

// One FP32 or FP32-pair Yee step (H half step, then E with the new H) in
// one pass over the fields, where the two-kernel form is bandwidth- and
// latency-bound (it moves 72 bytes per cell and step in FP32, 144 in pairs;
// this moves the 48 / 96 of reading E, H and writing E, H once).  The
// element policy (YeeF32, YeeF32x2) gives the arithmetic.  It reads the old set of six fields and writes the
// other (ping-pong: a CTA recomputes the new H of its x-1 / y-1 halo from
// old values that its neighbours must not have overwritten yet).
//
// A CTA owns a YX x YY column tile and marches z-planes.  TMA brings, per
// plane, a box of each old E field (rows y0-1 .. y0+YY) and of each old H
// field (rows y0-1 .. y0+YY-1), columns x0-4 .. x0+YX+3 (x0-4 keeps the
// 16-byte alignment TMA needs; out-of-grid cells read as 0 and are never
// used): E through a ring of three planes (z, z+1, z+2 in flight), H through
// two.  Per plane the CTA computes the new H on the tile plus a one-cell halo
// on the low x and y sides, then the new E of its own columns from the new H
// of plane z (shared) and z-1 (registers).  Same operations, in the same
// order, as k_yee_h + k_yee_e.  Every wait is bounded; on a timeout the
// kernel records the status, drains its loads and returns.
constexpr int YX = 32, YY = 8;
constexpr int YBW = YX + 8;                            // box width (x0-4 .. x0+YX+3)
constexpr int YE_BOX = YBW * (YY + 2);                 // E box: rows y0-1 .. y0+YY
constexpr int YH_BOX = YBW * (YY + 1);                 // H box: rows y0-1 .. y0+YY-1
// Elements per E / H box of ESZ-byte elements, 128-byte aligned.
__host__ __device__ constexpr int ye_pad(int esz) { return (YE_BOX * esz + 127) / 128 * 128 / esz; }
__host__ __device__ constexpr int yh_pad(int esz) { return (YH_BOX * esz + 127) / 128 * 128 / esz; }
constexpr int YHS = YX + 1, YHN = YHS * (YY + 1);     // new-H cells: x0-1 .. x0+YX-1, y0-1 ..
constexpr size_t yee_smem(int esz) {
    return (size_t)(9 * ye_pad(esz) + 6 * yh_pad(esz) + 6 * YH_BOX) * esz + 5 * 8;
}

// Element policies of the fused step: v + sign * ch * ((a - b) - (c - d))
// and v - s, in FP32 (one FMA: the arithmetic of k_yee_h / k_yee_e) or in
// FP32 pairs (the arithmetic of k_yee_h_x2 / k_yee_e_x2).
struct YeeF32 {
    using T = float;
    using C = float;
    static constexpr int MINB = 4;  // CTAs per SM
    static __device__ __forceinline__ T zero() { return 0.f; }
    static __device__ __forceinline__ T upd(T v, C ch, float sign, T a, T b, T c, T d) {
        return v + (sign * ch) * ((a - b) - (c - d));
    }
    static __device__ __forceinline__ T sub(T v, T s) { return v - s; }
};

struct YeeF32x2 {
    using T = float2;
    using C = C3;
    static constexpr int MINB = 3;
    static __device__ __forceinline__ T zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ T upd(T v, const C& ch, float sign, T a, T b, T c, T d) {
        return yee_upd(v, ch, sign, a, b, c, d);
    }
    static __device__ __forceinline__ T sub(T v, T s) {
        PAcc acc{v.x, v.y};
        pa_add(acc, s, -1.f);
        return pa_result(acc);
    }
};

template <class P>
__global__ void __launch_bounds__(YX * YY, P::MINB)
k_yee_tma(const __grid_constant__ CUtensorMap tex, const __grid_constant__ CUtensorMap tey,
          const __grid_constant__ CUtensorMap tez, const __grid_constant__ CUtensorMap thx,
          const __grid_constant__ CUtensorMap thy, const __grid_constant__ CUtensorMap thz,
          typename P::T* __restrict__ exn, typename P::T* __restrict__ eyn, typename P::T* __restrict__ ezn,
          typename P::T* __restrict__ hxn, typename P::T* __restrict__ hyn, typename P::T* __restrict__ hzn,
          Layout L, typename P::C ch, long long src, typename P::T src_val, int zchunk, int* __restrict__ status) {
    using T = typename P::T;
    constexpr int ESZ = sizeof(T);
    constexpr int YE_PAD = ye_pad(ESZ), YH_PAD = yh_pad(ESZ);
    constexpr int NT = YX * YY;
    constexpr int HPT = (YHN + NT - 1) / NT;
    extern __shared__ __align__(128) unsigned char ysm_raw[];
    T* se = reinterpret_cast<T*>(ysm_raw);  // [3 slots][ex, ey, ez][YE_PAD]
    T* sho = se + 9 * YE_PAD;               // [2 slots][hx, hy, hz][YH_PAD]   old H
    T* shn = sho + 6 * YH_PAD;              // [2 slots][hx, hy, hz][YH_BOX]   new H
    uint64_t* bar = reinterpret_cast<uint64_t*>(shn + 6 * YH_BOX);  // E slots 0-2, H slots 3-4
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * YX + tx;
    const int x0 = blockIdx.x * YX, y0 = blockIdx.y * YY;
    const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, L.nz);
    const int zs = z0 > 0 ? z0 - 1 : 0;  // plane z0-1 only gives the new H below z0
    const int np = z1 - zs;              // planes whose new H is computed

    // A sweep after one that timed out has nothing valid to work on.
    if (__syncthreads_or(tid == 0 && *(volatile int*)status != 0)) return;
    if (tid == 0) {
        for (int b = 0; b < 5; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncthreads();
    auto issue_e = [&](int p, int slot) {  // old E of plane zs+p into a ring slot
        uint64_t* b = &bar[slot];
        T* d = se + slot * 3 * YE_PAD;
        mbar_arrive_expect_tx(b, 3u * YE_BOX * (uint32_t)ESZ);
        tma_load_3d(d, &tex, x0 - 4, y0 - 1, zs + p, b);
        tma_load_3d(d + YE_PAD, &tey, x0 - 4, y0 - 1, zs + p, b);
        tma_load_3d(d + 2 * YE_PAD, &tez, x0 - 4, y0 - 1, zs + p, b);
    };
    auto issue_h = [&](int p) {  // old H of plane zs+p into slot p % 2
        uint64_t* b = &bar[3 + (p & 1)];
        T* d = sho + (p & 1) * 3 * YH_PAD;
        mbar_arrive_expect_tx(b, 3u * YH_BOX * (uint32_t)ESZ);
        tma_load_3d(d, &thx, x0 - 4, y0 - 1, zs + p, b);
        tma_load_3d(d + YH_PAD, &thy, x0 - 4, y0 - 1, zs + p, b);
        tma_load_3d(d + 2 * YH_PAD, &thz, x0 - 4, y0 - 1, zs + p, b);
    };
    // E planes 0 .. np and H planes 0 .. np-1 are loaded, each exactly once.
    if (tid == 0) {
        issue_e(0, 0);
        issue_e(1, 1);
        issue_h(0);
    }

    // Per-thread constants: the new-H cells this thread computes (box index,
    // in-grid and boundary tests) and its own column.
    int hb[HPT];
    bool hin[HPT], hxi[HPT], hyi[HPT];
#pragma unroll
    for (int k = 0; k < HPT; ++k) {
        const int i = tid + k * NT;
        const int lx = i % YHS, ly = i / YHS;
        const int gx = x0 - 1 + lx, gy = y0 - 1 + ly;
        hb[k] = ly * YBW + lx + 3;
        hin[k] = i < YHN && gx >= 0 && gx < L.nx && gy >= 0 && gy < L.ny;
        hxi[k] = gx + 1 < L.nx;
        hyi[k] = gy + 1 < L.ny;
    }
    const int x = x0 + tx, y = y0 + ty;
    const bool live = x < L.nx && y < L.ny;
    const long long oo = (long long)y * L.pitch + x;
    const int ob = (ty + 1) * YBW + tx + 4;  // own cell in a box
    const bool ex_upd = x + 1 < L.nx && y > 0 && y + 1 < L.ny;
    const bool ey_upd = y + 1 < L.ny && x > 0 && x + 1 < L.nx;
    const bool ez_upd = x > 0 && x + 1 < L.nx && y > 0 && y + 1 < L.ny;

    // Ring state without divisions: s0, s1, s2 are the slots of E planes
    // p, p+1, p+2; bit s of eph is the parity of slot s's next phase.
    int s0 = 0, s1 = 1, s2 = 2;
    uint32_t eph = 0;
    bool ok = bounded_wait(&bar[0], 0);  // E plane 0
    eph ^= 1u;
    T hx_prev = P::zero(), hy_prev = P::zero();
    for (int p = 0; p < np; ++p) {
        const int z = zs + p;
        __syncthreads();  // iteration p-1 is done with the slots refilled below
        if (tid == 0) {
            fence_proxy_async_smem();
            if (p + 2 <= np) issue_e(p + 2, s2);
            if (p + 1 < np) issue_h(p + 1);
        }
        ok = bounded_wait(&bar[s1], (eph >> s1) & 1u) && ok;   // E plane p+1
        eph ^= 1u << s1;
        ok = bounded_wait(&bar[3 + (p & 1)], (p >> 1) & 1) && ok;  // old H plane p
        const T* ea = se + s0 * 3 * YE_PAD;
        const T* eb = se + s1 * 3 * YE_PAD;
        const T* ho = sho + (p & 1) * 3 * YH_PAD;
        T* hn = shn + (p & 1) * 3 * YH_BOX;
        const bool zi = z + 1 < L.nz;
        if (ok) {
#pragma unroll
            for (int k = 0; k < HPT; ++k) {
                if (tid + k * NT >= YHN) break;
                const int b = hb[k];
                T vhx = P::zero(), vhy = P::zero(), vhz = P::zero();
                if (hin[k]) {
                    vhx = ho[b];
                    vhy = ho[YH_PAD + b];
                    vhz = ho[2 * YH_PAD + b];
                    const T ex0 = ea[b], ey0 = ea[YE_PAD + b], ez0 = ea[2 * YE_PAD + b];
                    if (hyi[k] && zi) vhx = P::upd(vhx, ch, -1.f, ea[2 * YE_PAD + b + YBW], ez0, eb[YE_PAD + b], ey0);
                    if (hxi[k] && zi) vhy = P::upd(vhy, ch, -1.f, eb[b], ex0, ea[2 * YE_PAD + b + 1], ez0);
                    if (hxi[k] && hyi[k]) vhz = P::upd(vhz, ch, -1.f, ea[YE_PAD + b + 1], ey0, ea[b + YBW], ex0);
                }
                hn[b] = vhx;
                hn[YH_BOX + b] = vhy;
                hn[2 * YH_BOX + b] = vhz;
            }
        }
        if (!__syncthreads_and(ok)) {
            if (tid == 0) {
                // A load never completed: report, drain what was issued, stop.
                // (eph already counts the wait on s1, so its pending phase
                // has the other parity.)
                atomicExch(status, SCAFES_ERR_TIMEOUT);
                bounded_wait(&bar[s1], ((eph >> s1) & 1u) ^ 1u, kWaitLimitNs / 8);
                bounded_wait(&bar[3 + (p & 1)], (p >> 1) & 1, kWaitLimitNs / 8);
                if (p + 2 <= np) bounded_wait(&bar[s2], (eph >> s2) & 1u, kWaitLimitNs / 8);
                if (p + 1 < np) bounded_wait(&bar[3 + ((p + 1) & 1)], ((p + 1) >> 1) & 1, kWaitLimitNs / 8);
            }
            return;
        }
        const T hx = hn[ob], hy = hn[YH_BOX + ob], hz = hn[2 * YH_BOX + ob];
        if (live && z >= z0) {
            const long long m = (long long)z * L.plane + oo;
            hxn[m] = hx;
            hyn[m] = hy;
            hzn[m] = hz;
            T ex = ea[ob], ey = ea[YE_PAD + ob], ez = ea[2 * YE_PAD + ob];
            const bool zin = z > 0 && zi;
            if (ex_upd && zin) ex = P::upd(ex, ch, 1.f, hz, hn[2 * YH_BOX + ob - YBW], hy, hy_prev);
            if (ey_upd && zin) ey = P::upd(ey, ch, 1.f, hx, hx_prev, hz, hn[2 * YH_BOX + ob - 1]);
            if (ez_upd && zi) {
                T v = P::upd(ez, ch, 1.f, hy, hn[YH_BOX + ob - 1], hx, hn[ob - YBW]);
                if (m == src) v = P::sub(v, src_val);
                ez = v;
            }
            exn[m] = ex;
            eyn[m] = ey;
            ezn[m] = ez;
        }
        hx_prev = hx;
        hy_prev = hy;
        const int t = s0;
        s0 = s1;
        s1 = s2;
        s2 = t;
    }
}

template <class T>
__global__ void k_dense_to_field(const double* __restrict__ d, T* __restrict__ f, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % L.nx);
        const long long r = i / L.nx;
        f[L.idx(x, (int)(r % L.ny), (int)(r / L.ny))] = (T)d[i];
    }
}

template <class T>
__global__ void k_field_to_dense(const T* __restrict__ f, double* __restrict__ d, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int x = (int)(i % L.nx);
        const long long r = i / L.nx;
        d[i] = (double)f[L.idx(x, (int)(r % L.ny), (int)(r / L.ny))];
    }
}

}  // namespace

struct scafes_mf {
    scafes_mf_cfg cfg;
    Layout L;
    size_t esz = 8;
    int nfields = 0;
    void* mem = nullptr;      // all fields, component-major
    double* stage = nullptr;  // dense doubles for transfers
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int cur = 0;              // Lame: which half of mem holds u^n;
                              // FP32 Yee: which set of 6 fields is current
    int t = 0;
    bool timed = false;
    int* status = nullptr;    // device status word of the TMA sweeps (0 = ok)
    CUtensorMap ytm[2][6];    // FP32 Yee: per field set, the TMA maps of Ex..Hz
    bool ytm_ok = false;
    CUtensorMap ltm[2][3];    // pair Lame: per half of mem, the TMA maps of its three components
    bool ltm_ok = false;
    std::string err;
};

namespace {

int mfail(scafes_mf* h, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (h) h->err = buf;
    scafes::set_last_error(buf);
    return code;
}

#define MTRY(h, call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return mfail(h, SCAFES_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                                  \
    } while (0)

// z-planes per CTA of the fused Yee step: long chunks (the plane below a
// chunk is recomputed), shorter ones while the grid has few column tiles.
int yee_zchunk(const Layout& L) {
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 1;
    }
    const long long tiles = (long long)((L.nx + YX - 1) / YX) * ((L.ny + YY - 1) / YY);
    int zc = 32;
    while (zc > 4 && tiles * ((L.nz + zc - 1) / zc) < (long long)sms * 8) zc >>= 1;
    while ((L.nz + zc - 1) / zc > 65535) zc <<= 1;  // grid.z limit
    return zc;
}

dim3 mgrid(const Layout& L) { return dim3((L.nx + MX - 1) / MX, (L.ny + MY - 1) / MY, (L.nz + MZ - 1) / MZ); }

char* field_ptr(scafes_mf* h, int f) { return (char*)h->mem + (size_t)f * h->L.size() * h->esz; }

}  // namespace

extern "C" const char* scafes_mf_last_error(const scafes_mf* h) { return h ? h->err.c_str() : ""; }

extern "C" void scafes_mf_destroy(scafes_mf* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->mem);
    cudaFree(h->stage);
    cudaFree(h->status);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int scafes_mf_create(const scafes_mf_cfg* cfg, scafes_mf** out) {
    if (!cfg || !out) return mfail(nullptr, SCAFES_ERR_ARG, "scafes_mf_create: NULL argument");
    *out = nullptr;
    if (cfg->kind != SCAFES_MF_LAME && cfg->kind != SCAFES_MF_YEE)
        return mfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_mf_create: kind %d", cfg->kind);
    for (int p = 0; p < 3; ++p)
        if (cfg->n_nodes[p] < 3 || cfg->n_nodes[p] > (1 << 16))
            return mfail(nullptr, SCAFES_ERR_ARG, "scafes_mf_create: n_nodes[%d]=%d out of [3, 65536]", p, cfg->n_nodes[p]);
    if (cfg->kind == SCAFES_MF_LAME && cfg->precision != SCAFES_PREC_F64 && cfg->precision != SCAFES_PREC_F32X2)
        return mfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_mf_create: Lame-Navier runs in FP64 or FP32 pairs");
    if (cfg->kind == SCAFES_MF_YEE && cfg->precision != SCAFES_PREC_F64 && cfg->precision != SCAFES_PREC_F32 &&
        cfg->precision != SCAFES_PREC_F32X2)
        return mfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_mf_create: Yee runs in FP64, FP32 or FP32 pairs");
    if (cfg->kind == SCAFES_MF_YEE)
        for (int p = 0; p < 3; ++p)
            if (cfg->src[p] < 0 || cfg->src[p] >= cfg->n_nodes[p])
                return mfail(nullptr, SCAFES_ERR_ARG, "scafes_mf_create: source index out of the grid");
    if (cfg->kind == SCAFES_MF_YEE && cfg->precision != SCAFES_PREC_F64) {
        const Layout Lp = make_layout(cfg->n_nodes[0], cfg->n_nodes[1], cfg->n_nodes[2]);
        if (Lp.plane > 0x7fffffffLL)  // the fused step keeps in-plane offsets in 32 bits
            return mfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_mf_create: a z-plane of %lld cells is too large",
                         Lp.plane);
    }
    scafes_mf* h = new (std::nothrow) scafes_mf();
    if (!h) return mfail(nullptr, SCAFES_ERR_NOMEM, "scafes_mf_create: out of host memory");
    h->cfg = *cfg;
    h->L = make_layout(cfg->n_nodes[0], cfg->n_nodes[1], cfg->n_nodes[2]);
    h->esz = cfg->precision == SCAFES_PREC_F32 ? 4 : 8;
    h->nfields = 6;  // Lame: u^n (3) + u^{n-1} (3); Yee: Ex..Hz
    // The fused Yee step (FP32, FP32 pairs) reads one set of six fields and
    // writes another.
    const bool fused = cfg->kind == SCAFES_MF_YEE && cfg->precision != SCAFES_PREC_F64;
    const int sets = fused ? 2 : 1;
    cudaError_t e = cudaSuccess;
    if (cfg->stream) h->stream = (cudaStream_t)cfg->stream;
    else { e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking); h->own_stream = true; }
    const size_t bytes = (size_t)sets * h->nfields * h->L.size() * h->esz;
    if (e == cudaSuccess) e = cudaMalloc(&h->mem, bytes);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->mem, 0, bytes, h->stream);
    if (e == cudaSuccess) e = cudaMalloc(&h->stage, (size_t)h->L.nx * h->L.ny * h->L.nz * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&h->status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(h->status, 0, sizeof(int), h->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->e1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? SCAFES_ERR_NOMEM : SCAFES_ERR_CUDA;
        mfail(nullptr, code, "scafes_mf_create: %s", cudaGetErrorString(e));
        scafes_mf_destroy(h);
        return code;
    }
    *out = h;
    return SCAFES_OK;
}

// Lame fields 0..2 are u^n, 3..5 u^{n-1}; the halves swap every step.
static int phys_field(const scafes_mf* h, int field) {
    if (h->cfg.kind != SCAFES_MF_LAME) return h->cur * 6 + field;  // Yee: the current set
    const int half = field / 3, comp = field % 3;
    return ((half ^ h->cur) * 3) + comp;
}

// Reads and clears the status word of the TMA sweeps.
static int mf_status(scafes_mf* h) {
    int st = 0;
    MTRY(h, cudaMemcpyAsync(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    MTRY(h, cudaStreamSynchronize(h->stream));
    if (st != 0) {
        cudaMemsetAsync(h->status, 0, sizeof(int), h->stream);
        return mfail(h, SCAFES_ERR_TIMEOUT, "a multi-field sweep gave up waiting for its TMA loads; results are invalid");
    }
    return SCAFES_OK;
}

// TMA maps of both halves (pair Lame): 36 x 10 boxes of each component.
static int lame_maps(scafes_mf* h) {
    if (h->ltm_ok) return SCAFES_OK;
    const Layout& L = h->L;
    for (int half = 0; half < 2; ++half)
        for (int c = 0; c < 3; ++c) {
            const CUresult r = make_tensor_map_3d(&h->ltm[half][c], field_ptr(h, 3 * half + c), 8, L.nx, L.ny, L.nz,
                                                  (size_t)L.pitch * 8, (size_t)L.plane * 8, LBW, LBH);
            if (r != CUDA_SUCCESS) return mfail(h, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        }
    const cudaError_t e = cudaFuncSetAttribute(k_lame_x2_tma, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)LAME_SMEM);
    if (e != cudaSuccess) return mfail(h, SCAFES_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    h->ltm_ok = true;
    return SCAFES_OK;
}

// TMA maps of both field sets (FP32 Yee): E fields with a box of YY+2 rows,
// H fields with YY+1, YBW columns.
static int yee_maps(scafes_mf* h) {
    if (h->ytm_ok) return SCAFES_OK;
    const Layout& L = h->L;
    for (int set = 0; set < 2; ++set)
        for (int f = 0; f < 6; ++f) {
            const CUresult r = make_tensor_map_3d(&h->ytm[set][f], field_ptr(h, set * 6 + f), (int)h->esz, L.nx,
                                                  L.ny, L.nz, (size_t)L.pitch * h->esz, (size_t)L.plane * h->esz,
                                                  YBW, f < 3 ? YY + 2 : YY + 1);
            if (r != CUDA_SUCCESS) return mfail(h, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
        }
    if (h->esz == 8) {
        const cudaError_t e = cudaFuncSetAttribute(k_yee_tma<YeeF32x2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                   (int)yee_smem(8));
        if (e != cudaSuccess) return mfail(h, SCAFES_ERR_CUDA, "cudaFuncSetAttribute: %s", cudaGetErrorString(e));
    }
    h->ytm_ok = true;
    return SCAFES_OK;
}

extern "C" int scafes_mf_upload(scafes_mf* h, int field, const double* host, size_t n) {
    if (!h || !host) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_upload: NULL argument");
    if (field < 0 || field >= h->nfields) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_upload: field %d", field);
    if (n != (size_t)h->L.nx * h->L.ny * h->L.nz) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_upload: wrong size");
    MTRY(h, cudaMemcpyAsync(h->stage, host, n * sizeof(double), cudaMemcpyHostToDevice, h->stream));
    char* f = field_ptr(h, phys_field(h, field));
    if (h->cfg.precision == SCAFES_PREC_F32X2) MTRY(h, convert_to_device(SCAFES_PREC_F32X2, h->stage, f, h->L, h->stream));
    else if (h->esz == 8) k_dense_to_field<double><<<256, 256, 0, h->stream>>>(h->stage, (double*)f, h->L);
    else k_dense_to_field<float><<<256, 256, 0, h->stream>>>(h->stage, (float*)f, h->L);
    MTRY(h, cudaGetLastError());
    MTRY(h, cudaStreamSynchronize(h->stream));
    h->t = 0;
    return SCAFES_OK;
}

extern "C" int scafes_mf_download(scafes_mf* h, int field, double* host, size_t n) {
    if (!h || !host) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_download: NULL argument");
    if (field < 0 || field >= h->nfields) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_download: field %d", field);
    if (n != (size_t)h->L.nx * h->L.ny * h->L.nz) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_download: wrong size");
    const int st = mf_status(h);
    if (st) return st;
    const char* f = field_ptr(h, phys_field(h, field));
    if (h->cfg.precision == SCAFES_PREC_F32X2)
        MTRY(h, convert_from_device(SCAFES_PREC_F32X2, f, h->stage, h->L, h->stream));
    else if (h->esz == 8) k_field_to_dense<double><<<256, 256, 0, h->stream>>>((const double*)f, h->stage, h->L);
    else k_field_to_dense<float><<<256, 256, 0, h->stream>>>((const float*)f, h->stage, h->L);
    MTRY(h, cudaGetLastError());
    MTRY(h, cudaMemcpyAsync(host, h->stage, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    MTRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_mf_step(scafes_mf* h, int n_steps) {
    if (!h) return mfail(nullptr, SCAFES_ERR_ARG, "scafes_mf_step: NULL handle");
    if (n_steps < 0) return mfail(h, SCAFES_ERR_ARG, "scafes_mf_step: n_steps < 0");
    const Layout& L = h->L;
    const scafes_mf_cfg& c = h->cfg;
    MTRY(h, cudaEventRecord(h->e0, h->stream));
    if (c.kind == SCAFES_MF_LAME) {
        const double lam = c.p[0], mu = c.p[1], rho = c.p[2];
        double hh[3];
        for (int p = 0; p < 3; ++p) hh[p] = (c.coord_last[p] - c.coord_first[p]) / (c.n_nodes[p] - 1);
        const double s = c.tau * c.tau / rho;
        LameCoef K;
        for (int cc = 0; cc < 3; ++cc)
            for (int p = 0; p < 3; ++p) {
                K.a[cc][p] = s * (p == cc ? lam + 2.0 * mu : mu) / (hh[p] * hh[p]);
                K.b[cc][p] = (p == cc) ? 0.0 : s * (lam + mu) / (4.0 * hh[cc] * hh[p]);
            }
        const long long comp = L.size();
        LameCoefX2 K2;
        for (int cc = 0; cc < 3; ++cc) {
            double sa = 0.0;
            for (int p = 0; p < 3; ++p) {
                K2.a[cc][p] = split3(K.a[cc][p]);
                K2.b[cc][p] = split3(K.b[cc][p]);
                sa += K.a[cc][p];
            }
            K2.d[cc] = split3(2.0 - 2.0 * sa);
        }
        const bool x2 = c.precision == SCAFES_PREC_F32X2;
        if (x2) {
            const int rc = lame_maps(h);
            if (rc) return rc;
        }
        const dim3 lgrid((L.nx + LX - 1) / LX, (L.ny + LY - 1) / LY, (L.nz + LZ - 1) / LZ);
        for (int st = 0; st < n_steps; ++st) {
            void* u = field_ptr(h, 3 * h->cur);
            void* up = field_ptr(h, 3 * (h->cur ^ 1));
            if (x2) {
                const CUtensorMap* t = h->ltm[h->cur];
                k_lame_x2_tma<<<lgrid, dim3(LX, LY / 2), LAME_SMEM, h->stream>>>(t[0], t[1], t[2], (float2*)up, K2,
                                                                                L, comp, h->status);
            } else {
                k_lame<<<mgrid(L), dim3(MX, MY), 0, h->stream>>>((const double*)u, (double*)up, K, L, comp);
            }
            MTRY(h, cudaGetLastError());
            h->cur ^= 1;
            h->t += 1;
        }
    } else {
        const double hgrid = (c.coord_last[0] - c.coord_first[0]) / (c.n_nodes[0] - 1);
        const double ch = c.tau / hgrid;
        const long long src = L.idx(c.src[0], c.src[1], c.src[2]);
        const double amp = c.p[0], t0 = c.p[1], w = c.p[2], freq = c.p[3];
        for (int st = 0; st < n_steps; ++st) {
            const double time = c.t_start + (h->t + 1) * c.tau;
            const double a = (time - t0) / w;
            const double sv = c.tau * amp * std::exp(-a * a) * std::sin(2.0 * 3.14159265358979323846 * freq * time);
            if (c.precision == SCAFES_PREC_F32X2) {
                const int rc = yee_maps(h);
                if (rc) return rc;
                float2* g[6];
                for (int i = 0; i < 6; ++i) g[i] = (float2*)field_ptr(h, (h->cur ^ 1) * 6 + i);
                const CUtensorMap* t = h->ytm[h->cur];
                const int zc = yee_zchunk(L);
                const dim3 grid((L.nx + YX - 1) / YX, (L.ny + YY - 1) / YY, (L.nz + zc - 1) / zc);
                const f2 sp = split_double(sv);
                k_yee_tma<YeeF32x2><<<grid, dim3(YX, YY), yee_smem(8), h->stream>>>(
                    t[0], t[1], t[2], t[3], t[4], t[5], g[0], g[1], g[2], g[3], g[4], g[5], L, split3(ch), src,
                    make_float2(sp.hi, sp.lo), zc, h->status);
                h->cur ^= 1;
            } else if (h->esz == 8) {
                double* f[6];
                for (int i = 0; i < 6; ++i) f[i] = (double*)field_ptr(h, i);
                k_yee_h<double><<<mgrid(L), dim3(MX, MY), 0, h->stream>>>(f[0], f[1], f[2], f[3], f[4], f[5], L, ch);
                k_yee_e<double><<<mgrid(L), dim3(MX, MY), 0, h->stream>>>(f[0], f[1], f[2], f[3], f[4], f[5], L, ch,
                                                                          src, sv);
            } else {
                const int rc = yee_maps(h);
                if (rc) return rc;
                float* g[6];
                for (int i = 0; i < 6; ++i) g[i] = (float*)field_ptr(h, (h->cur ^ 1) * 6 + i);
                const CUtensorMap* t = h->ytm[h->cur];
                const int zc = yee_zchunk(L);
                const dim3 grid((L.nx + YX - 1) / YX, (L.ny + YY - 1) / YY, (L.nz + zc - 1) / zc);
                k_yee_tma<YeeF32><<<grid, dim3(YX, YY), yee_smem(4), h->stream>>>(
                    t[0], t[1], t[2], t[3], t[4], t[5], g[0], g[1], g[2], g[3], g[4], g[5], L, (float)ch, src,
                    (float)sv, zc, h->status);
                h->cur ^= 1;
            }
            MTRY(h, cudaGetLastError());
            h->t += 1;
        }
    }
    MTRY(h, cudaEventRecord(h->e1, h->stream));
    h->timed = true;
    return SCAFES_OK;
}

extern "C" int scafes_mf_last_ms(const scafes_mf* h, float* ms) {
    if (!h || !ms) return mfail(nullptr, SCAFES_ERR_ARG, "scafes_mf_last_ms: NULL argument");
    if (!h->timed) return mfail(nullptr, SCAFES_ERR_STATE, "scafes_mf_last_ms: nothing ran yet");
    cudaError_t e = cudaEventSynchronize(h->e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, h->e0, h->e1);
    if (e != cudaSuccess) return mfail(nullptr, SCAFES_ERR_CUDA, "scafes_mf_last_ms: %s", cudaGetErrorString(e));
    return SCAFES_OK;
}
