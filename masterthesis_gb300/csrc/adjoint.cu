// Hand-written adjoint of the flux-form variable-conductivity heat update,
// with binomial checkpointing.
//
// Forward update (inner nodes; border nodes keep their value):
//   u'_i = u_i + sum_p [ K_p[i] (u_{i+p} - u_i) - K_p[i-p] (u_i - u_{i-p}) ]
//   K_p[i] = (tau/h_p^2) * (k_i + k_{i+p}) / 2     (conductivity of face i|i+p)
// Objective J = 1/2 ||u_T - target||^2.  Gradients dJ/dk and dJ/du0.
//
// The reference obtains gradients by taping the update with ADOL-C and
// evaluating the tape in forward mode with one direction per parameter
// (src/ScaFES_Problem.hpp:5843-5967 traceTypeTwo, :6633-6747
// evalFovForwardTypeTwo, ::fov_forward at :6714).  Here the reverse-time
// (adjoint) sweep is hand-written: the update is linear in u and its
// matrix is symmetric on the inner nodes, so the adjoint step has the same
// stencil as the forward step applied to lambda (zero on border nodes),
// plus the accumulation, per node, of the conductivity gradient
//   dJ/dk_i = sum_p (tau/h_p^2)/2 (G_p[i] + G_p[i-p]),
//   G_p[j] = sum over steps of (u_{j+p} - u_j) (lambda_j - lambda_{j+p}),
// the two faces of node i along each axis, in FP32-pair arithmetic.
// The forward states the adjoint needs are recomputed from snapshots kept
// in device memory; the split points follow the optimal binomial schedule
// (Griewank & Walther, "Algorithm 799: revolve", ACM TOMS 26(1), 2000),
// computed here by dynamic programming over (steps, free snapshots).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#include "adjoint.cuh"
#include "scafes_common.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

using namespace scafes;

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

constexpr int AX = 32, AY = 8;

// Face conductivities K_p[i] = w_p (k_i + k_{i+p}) / 2, zero where i+p is
// outside the grid, and the diagonal d_i = 1 - sum of the six faces of i.
__global__ void k_faces(const double* __restrict__ k, double* __restrict__ kx, double* __restrict__ ky,
                        double* __restrict__ kz, double* __restrict__ dg, Layout L, double wx, double wy,
                        double wz) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        const double kc = k[o];
        const double fxp = x + 1 < L.nx ? wx * 0.5 * (kc + k[o + 1]) : 0.0;
        const double fyp = y + 1 < L.ny ? wy * 0.5 * (kc + k[o + L.pitch]) : 0.0;
        const double fzp = z + 1 < L.nz ? wz * 0.5 * (kc + k[o + L.plane]) : 0.0;
        const double fxm = x > 0 ? wx * 0.5 * (k[o - 1] + kc) : 0.0;
        const double fym = y > 0 ? wy * 0.5 * (k[o - L.pitch] + kc) : 0.0;
        const double fzm = z > 0 ? wz * 0.5 * (k[o - L.plane] + kc) : 0.0;
        kx[o] = fxp;
        ky[o] = fyp;
        kz[o] = fzp;
        dg[o] = 1.0 - (((fxp + fxm) + (fyp + fym)) + (fzp + fzm));
    }
}

// One forward step (inner nodes; border nodes copied), in the diagonal
// form u'_i = d_i u_i + sum_f K_f u_nb: 7 FP64 operations per node (the
// flux form takes 12), summed in the order diagonal, +x, -x, +y, -y, +z,
// -z, which the reverse sweep's recomputation repeats bit for bit.
__global__ void __launch_bounds__(AX * AY)
k_forward(const double* __restrict__ u, double* __restrict__ un, const double* __restrict__ kx,
          const double* __restrict__ ky, const double* __restrict__ kz, const double* __restrict__ dg, Layout L) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
    const int zb = blockIdx.z * 16, ze = min(zb + 16, L.nz);
    for (int z = zb; z < ze; ++z) {
        const long long o = L.idx(x, y, z);
        const double uc = u[o];
        if (colb || z == 0 || z == L.nz - 1) {
            un[o] = uc;
            continue;
        }
        double v = dg[o] * uc;
        v = fma(kx[o], u[o + 1], v);
        v = fma(kx[o - 1], u[o - 1], v);
        v = fma(ky[o], u[o + L.pitch], v);
        v = fma(ky[o - L.pitch], u[o - L.pitch], v);
        v = fma(kz[o], u[o + L.plane], v);
        v = fma(kz[o - L.plane], u[o - L.plane], v);
        un[o] = v;
    }
}

// A double as an FP32 pair (split_bits: integer instructions only).
__device__ __forceinline__ float2 pbits(double d) {
    const f2 p = split_bits(d);
    return make_float2(p.hi, p.lo);
}

// lambda_T = u_T - target (or the given cotangent when `seed`): inner part
// into lam, border part into bnd; per-CTA partial sums of 0.5 (u_T -
// target)^2 into part (0 when `seed`).
__global__ void k_terminal(const double* __restrict__ uT, const double* __restrict__ target,
                           double* __restrict__ lam, double* __restrict__ bnd, double* __restrict__ part, Layout L,
                           bool seed) {
    __shared__ double sh[AX * AY];
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    double acc = 0.0;
    if (x < L.nx && y < L.ny) {
        const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
        for (int z = 0; z < L.nz; ++z) {
            const long long o = L.idx(x, y, z);
            const double d = seed ? target[o] : uT[o] - target[o];
            if (!seed) acc += 0.5 * d * d;
            const bool border = colb || z == 0 || z == L.nz - 1;
            lam[o] = border ? 0.0 : d;
            bnd[o] = border ? d : 0.0;
        }
    }
    const int t = threadIdx.y * AX + threadIdx.x;
    sh[t] = acc;
    __syncthreads();
    for (int s = AX * AY / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    if (t == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

// dJ/dk = the per-node gradient pair; dJ/du0 = lambda_0 + border part
// (FP64 sweeps: lambda and bnd FP64).
__global__ void k_finalize(const float2* __restrict__ g, const double* __restrict__ lam,
                           const double* __restrict__ bnd, double* __restrict__ dk, double* __restrict__ du0,
                           Layout L) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        dk[o] = join_pair(g[o].x, g[o].y);
        du0[o] = lam[o] + bnd[o];
    }
}

// ---- compensated FP32-pair (f32x2) sweeps ----------------------------------
//
// The same update in its diagonal form u'_i = d_i u_i + sum_f K_f u_nb with
// d_i = 1 - sum_f K_f (K and d prepared in FP64, then split into pairs).
// Products are exact in their hi parts (FMA TwoProd) with the cross terms
// in FP32; sums are TwoSum-exact in the hi parts; every pair is
// renormalised once per node (FastTwoSum).  No FP64 instruction is issued
// in the per-step kernels.

// p = a * b as an unnormalised pair.
__device__ __forceinline__ f2 pmul(float2 a, float2 b) {
    const float p = a.x * b.x;
    float e = fmaf(a.x, b.x, -p);
    e = fmaf(a.x, b.y, e);
    e = fmaf(a.y, b.x, e);
    return {p, e};
}

// acc += p (unnormalised).
__device__ __forceinline__ void pacc(f2& acc, f2 p) {
    const f2 s = two_sum(acc.hi, p.hi);
    acc.hi = s.hi;
    acc.lo += s.lo + p.lo;
}

// a - b as an unnormalised pair.
__device__ __forceinline__ f2 psub(float2 a, float2 b) {
    const f2 s = two_sum(a.x, -b.x);
    return {s.hi, s.lo + (a.y - b.y)};
}

__device__ __forceinline__ float2 pnorm(f2 a) {
    const f2 r = fast_two_sum(a.hi, a.lo);
    return make_float2(r.hi, r.lo);
}

__device__ __forceinline__ float2 psplit(double d) {
    const f2 p = split_double(d);
    return make_float2(p.hi, p.lo);
}

__device__ __forceinline__ double pjoin(float2 a) { return (double)a.x + (double)a.y; }

// In-place conversions of a padded field between FP64 and pairs (each
// element keeps its 8 bytes).
__global__ void k_to_pair(void* buf, Layout L) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        const double d = reinterpret_cast<const double*>(buf)[o];
        reinterpret_cast<float2*>(buf)[o] = psplit(d);
    }
}

__global__ void k_from_pair(void* buf, Layout L) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        const float2 p = reinterpret_cast<const float2*>(buf)[o];
        reinterpret_cast<double*>(buf)[o] = pjoin(p);
    }
}

// Face conductivities and the diagonal from k (FP64), stored as pairs.
__global__ void k_prep_x2(const double* __restrict__ k, float2* __restrict__ kx, float2* __restrict__ ky,
                          float2* __restrict__ kz, float2* __restrict__ dg, Layout L, double wx, double wy,
                          double wz) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        const double kc = k[o];
        const double fxp = x + 1 < L.nx ? wx * 0.5 * (kc + k[o + 1]) : 0.0;
        const double fyp = y + 1 < L.ny ? wy * 0.5 * (kc + k[o + L.pitch]) : 0.0;
        const double fzp = z + 1 < L.nz ? wz * 0.5 * (kc + k[o + L.plane]) : 0.0;
        const double fxm = x > 0 ? wx * 0.5 * (k[o - 1] + kc) : 0.0;
        const double fym = y > 0 ? wy * 0.5 * (k[o - L.pitch] + kc) : 0.0;
        const double fzm = z > 0 ? wz * 0.5 * (k[o - L.plane] + kc) : 0.0;
        kx[o] = psplit(fxp);
        ky[o] = psplit(fyp);
        kz[o] = psplit(fzp);
        dg[o] = psplit(1.0 - (((fxp + fxm) + (fyp + fym)) + (fzp + fzm)));
    }
}

// One forward step on FP32 pairs, u' = d u + sum_f K_f u_nb over the six
// faces (border nodes copied), with every operand staged through TMA: a
// column-per-thread kernel with plain loads stalled on their latency (ncu:
// long-scoreboard stalls, 0.63 of HBM).  A CTA owns an FTX x FTY column tile
// and marches FZ_ planes; per plane one mbarrier covers five boxes -- u with
// a one-node halo (x from x0-2 for 16-byte alignment), the x faces from
// x0-2, the y faces from row y0-1, the z faces and the diagonal of the tile
// -- in a ring of four planes (planes z, z+1 in use, z+2, z+3 in flight).
// u and the z face of the plane below come from register queues.  The
// products are accumulated in a fixed order (diagonal, +x, -x, +y, -y, +z,
// -z), which the reverse sweep's recomputation repeats bit for bit.  Every
// wait is bounded (status word, drain, return).
constexpr int FTX = 32, FTY = 8, FZ_ = 32, FNS = 4;
constexpr int FUW = FTX + 4, FUH = FTY + 2;             // u box: x0-2 .. x0+33, y0-1 .. y0+8
constexpr int FXW = FTX + 4, FXH = FTY;                 // x faces: x0-2 .. x0+33, own rows
constexpr int FYW = FTX, FYH = FTY + 1;                 // y faces: own columns, y0-1 .. y0+7
constexpr int FKW = FTX, FKH = FTY;                     // z faces, diagonal: the tile
constexpr int pad16(int n) { return (n + 15) / 16 * 16; }  // float2 count -> 128-byte multiple
constexpr int FO_U = 0, FO_X = pad16(FUW * FUH), FO_Y = FO_X + pad16(FXW * FXH);
constexpr int FO_Z = FO_Y + pad16(FYW * FYH), FO_D = FO_Z + pad16(FKW * FKH);
constexpr int FSLOT = FO_D + pad16(FKW * FKH);          // float2 per ring slot
constexpr uint32_t FTX_BYTES = (uint32_t)(FUW * FUH + FXW * FXH + FYW * FYH + 2 * FKW * FKH) * 8u;
constexpr size_t FSMEM = (size_t)FNS * FSLOT * 8 + FNS * 8;

__global__ void __launch_bounds__(FTX * FTY)
k_forward_x2_tma(const __grid_constant__ CUtensorMap tu, const __grid_constant__ CUtensorMap tkx,
                 const __grid_constant__ CUtensorMap tky, const __grid_constant__ CUtensorMap tkz,
                 const __grid_constant__ CUtensorMap tdg, float2* __restrict__ un, Layout L,
                 int* __restrict__ status) {
    extern __shared__ __align__(128) float2 fsm[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(fsm + FNS * FSLOT);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * FTX + tx;
    const int x0 = blockIdx.x * FTX, y0 = blockIdx.y * FTY;
    const int z0 = blockIdx.z * FZ_, z1 = min(z0 + FZ_, L.nz);
    if (__syncthreads_or(tid == 0 && *(volatile int*)status != 0)) return;
    if (tid == 0) {
        for (int b = 0; b < FNS; ++b) scafes::mbar_init(&bar[b], 1);
        scafes::fence_barrier_init();
    }
    __syncthreads();
    // Input plane j is z0-1+j (j = 0 .. n_in-1), in ring slot j % FNS.
    const int n_in = z1 - z0 + 2;
    auto issue = [&](int j) {
        const int s = j & (FNS - 1), z = z0 - 1 + j;
        float2* d = fsm + s * FSLOT;
        scafes::mbar_arrive_expect_tx(&bar[s], FTX_BYTES);
        scafes::tma_load_3d(d + FO_U, &tu, x0 - 2, y0 - 1, z, &bar[s]);
        scafes::tma_load_3d(d + FO_X, &tkx, x0 - 2, y0, z, &bar[s]);
        scafes::tma_load_3d(d + FO_Y, &tky, x0, y0 - 1, z, &bar[s]);
        scafes::tma_load_3d(d + FO_Z, &tkz, x0, y0, z, &bar[s]);
        scafes::tma_load_3d(d + FO_D, &tdg, x0, y0, z, &bar[s]);
    };
    if (tid == 0)
        for (int j = 0; j < FNS && j < n_in; ++j) issue(j);
    auto wait = [&](int j) { return scafes::bounded_wait(&bar[j & (FNS - 1)], (uint32_t)(j >> 2) & 1u); };
    auto fail = [&](int last_issued) {
        if (tid == 0) {
            atomicExch(status, SCAFES_ERR_TIMEOUT);
            // Only the last FNS planes issued can still be in flight (a slot
            // is refilled only after its previous plane was waited on).
            for (int j = last_issued - (FNS - 1); j <= last_issued; ++j)
                if (j >= 0 && j < n_in)
                    scafes::bounded_wait(&bar[j & (FNS - 1)], (uint32_t)(j >> 2) & 1u, scafes::kWaitLimitNs / 16);
        }
    };
    const int x = x0 + tx, y = y0 + ty;
    const bool live = x < L.nx && y < L.ny;
    const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
    const int bu = (ty + 1) * FUW + tx + 2, bx = ty * FXW + tx + 2, by = (ty + 1) * FYW + tx, bk = ty * FKW + tx;
    const float2 zero = make_float2(0.f, 0.f);
    bool ok = wait(0);
    const float2* s0 = fsm;
    float2 ub = z0 > 0 ? s0[FO_U + bu] : zero;  // plane z0-1
    float2 kzb = z0 > 0 ? s0[FO_Z + bk] : zero;
    ok = wait(1) && ok;
    float2 uc = fsm[FSLOT + FO_U + bu];         // plane z0
    int issued = FNS - 1;
    for (int z = z0; z < z1; ++z) {
        const int jc = z - z0 + 1;  // input plane of z
        if (!__syncthreads_and(ok)) {  // plane z-1's slot is free; all waits so far succeeded
            fail(issued);
            return;
        }
        if (tid == 0 && jc + 3 < n_in && jc + 3 > issued) {
            scafes::fence_proxy_async_smem();
            issue(jc + 3);
            issued = jc + 3;
        }
        ok = wait(jc + 1) && ok;  // plane z+1 (its u above this node)
        const float2* sc = fsm + (jc & (FNS - 1)) * FSLOT;
        const float2* sa = fsm + ((jc + 1) & (FNS - 1)) * FSLOT;
        const float2 ua = z + 1 < L.nz ? sa[FO_U + bu] : zero;
        const float2 kzc = sc[FO_Z + bk];
        if (live) {
            const long long o = L.idx(x, y, z);
            if (colb || z == 0 || z == L.nz - 1) {
                un[o] = uc;
            } else {
                f2 acc = pmul(sc[FO_D + bk], uc);
                pacc(acc, pmul(sc[FO_X + bx], sc[FO_U + bu + 1]));
                pacc(acc, pmul(sc[FO_X + bx - 1], sc[FO_U + bu - 1]));
                pacc(acc, pmul(sc[FO_Y + by], sc[FO_U + bu + FUW]));
                pacc(acc, pmul(sc[FO_Y + by - FYW], sc[FO_U + bu - FUW]));
                pacc(acc, pmul(kzc, ua));
                pacc(acc, pmul(kzb, ub));
                un[o] = pnorm(acc);
            }
        }
        ub = uc;
        uc = ua;
        kzb = kzc;
    }
    if (!__syncthreads_and(ok)) fail(issued);
}

// One adjoint step: lambda' = A^T lambda (the transposed
// diagonal form; border rows pass what they receive into bnd) and the
// conductivity gradient at the state u_t, accumulated per node:
//   g_i -= sum_p w_p/2 [ P_p(i) + P_p(i-p) ],
//   P_p(j) = (u_{j+p} - u_j)(lambda_{j+p} - lambda_j),
// the two faces of node i along each axis (dJ/dk_i directly; one pair per
// node read and written instead of three face accumulators: 72 bytes per
// node instead of 104).  A face to a node outside the grid or between two
// border nodes contributes nothing: lambda is zero there.
// The operands are staged through TMA on the forward step's tile (RTX x
// RTY columns, RZ_ planes, a ring of four planes on four mbarriers).  Per
// plane one mbarrier covers six boxes: lambda and u with a one-node halo
// (x from x0-2), the x faces from x0-2, the y faces from row y0-1, the z
// faces and the diagonal.  lambda, u and the z face of the plane below and
// the z-face product of the plane below come from register queues; g is
// read with plain loads one plane ahead and written in place.
// Out-of-range box elements read as zero.  Every wait is bounded (status
// word, drain, return).
constexpr int RTX = FTX, RTY = FTY, RZ_ = FZ_, RNS = FNS;
constexpr int RLW = FUW, RLH = FUH;                       // lambda and u boxes: the forward's u box
constexpr int RO_L = 0, RO_U = pad16(RLW * RLH), RO_X = RO_U + pad16(RLW * RLH);
constexpr int RO_Y = RO_X + pad16(FXW * FXH), RO_Z = RO_Y + pad16(FYW * FYH), RO_D = RO_Z + pad16(FKW * FKH);
constexpr int RSLOT = RO_D + pad16(FKW * FKH);
constexpr uint32_t RTX_BYTES = (uint32_t)(2 * RLW * RLH + FXW * FXH + FYW * FYH + 2 * FKW * FKH) * 8u;
constexpr size_t RSMEM = (size_t)RNS * RSLOT * 8 + RNS * 8;
// FP64 fields: the lambda and u boxes of two planes also as FP32 pairs.
constexpr int RPAIR = pad16(RLW * RLH);
constexpr size_t RSMEM_F64 = (size_t)RNS * RSLOT * 8 + (size_t)4 * RPAIR * 8 + RNS * 8;
static_assert(RSLOT * 8 % 128 == 0 && RO_U * 8 % 128 == 0 && RO_X * 8 % 128 == 0, "TMA destinations 128-byte aligned");

// (u_b - u_a)(l_b - l_a) as an unnormalised pair.
__device__ __forceinline__ f2 pface(float2 ua, float2 ub, float2 la, float2 lb) {
    const f2 du = psub(ub, ua);
    const f2 dl = psub(lb, la);
    const float p = du.hi * dl.hi;
    float e = fmaf(du.hi, dl.hi, -p);
    e = fmaf(du.hi, dl.lo, e);
    e = fmaf(du.lo, dl.hi, e);
    return {p, e};
}

// c * (a + b) for a pair constant c (an axis weight w_p / 2), unnormalised.
__device__ __forceinline__ f2 pscale2(float2 c, f2 a, f2 b) {
    f2 s = a;
    pacc(s, b);
    const float p = c.x * s.hi;
    float e = fmaf(c.x, s.hi, -p);
    e = fmaf(c.x, s.lo, e);
    e = fmaf(c.y, s.hi, e);
    return {p, e};
}

// A stored value as a pair: FP32-pair fields as they are, FP64 fields split
// with integer instructions.
__device__ __forceinline__ float2 pview(float2 v) { return v; }
__device__ __forceinline__ float2 pview(double v) { return pbits(v); }

// E = float2: every field an FP32 pair, the lambda update in pair
// arithmetic.  E = double: lambda, u, the faces and the diagonal FP64 and
// the lambda update in FP64 in the order of k_forward (diagonal, +x, -x,
// +y, -y, +z, -z; 7 FP64 operations per node), the gradient in FP32 pairs
// from integer splits of u and lambda (no FP64 instruction).  With FP64
// fields the lambda and u boxes of each plane are split once, cooperatively,
// into a two-plane ring of pairs in shared memory when the plane arrives
// (each node's neighbours then read pairs instead of splitting them again);
// the centre values' pairs travel in registers from the plane above.
template <class E>
__global__ void __launch_bounds__(RTX * RTY)
k_adjoint_x2_tma(const __grid_constant__ CUtensorMap tl, const __grid_constant__ CUtensorMap tu,
                 const __grid_constant__ CUtensorMap tkx, const __grid_constant__ CUtensorMap tky,
                 const __grid_constant__ CUtensorMap tkz, const __grid_constant__ CUtensorMap tdg,
                 E* __restrict__ lamn, float2* __restrict__ g, E* __restrict__ bnd, float2 hx2,
                 float2 hy2, float2 hz2, Layout L, int* __restrict__ status) {
    constexpr bool F64 = std::is_same<E, double>::value;
    extern __shared__ __align__(128) unsigned char rsm_raw[];
    E* rsm = reinterpret_cast<E*>(rsm_raw);
    float2* pring = reinterpret_cast<float2*>(rsm + RNS * RSLOT);  // F64: [2 planes][lambda, u][RPAIR]
    uint64_t* bar = reinterpret_cast<uint64_t*>(rsm + RNS * RSLOT + (F64 ? 4 * RPAIR : 0));
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * RTX + tx;
    const int x0 = blockIdx.x * RTX, y0 = blockIdx.y * RTY;
    const int z0 = blockIdx.z * RZ_, z1 = min(z0 + RZ_, L.nz);
    if (__syncthreads_or(tid == 0 && *(volatile int*)status != 0)) return;
    if (tid == 0) {
        for (int b = 0; b < RNS; ++b) scafes::mbar_init(&bar[b], 1);
        scafes::fence_barrier_init();
    }
    __syncthreads();
    // Input plane j is z0-1+j (j = 0 .. n_in-1), in ring slot j % RNS.
    const int n_in = z1 - z0 + 2;
    auto issue = [&](int j) {
        const int s = j & (RNS - 1), z = z0 - 1 + j;
        E* d = rsm + s * RSLOT;
        scafes::mbar_arrive_expect_tx(&bar[s], RTX_BYTES);
        scafes::tma_load_3d(d + RO_L, &tl, x0 - 2, y0 - 1, z, &bar[s]);
        scafes::tma_load_3d(d + RO_U, &tu, x0 - 2, y0 - 1, z, &bar[s]);
        scafes::tma_load_3d(d + RO_X, &tkx, x0 - 2, y0, z, &bar[s]);
        scafes::tma_load_3d(d + RO_Y, &tky, x0, y0 - 1, z, &bar[s]);
        scafes::tma_load_3d(d + RO_Z, &tkz, x0, y0, z, &bar[s]);
        scafes::tma_load_3d(d + RO_D, &tdg, x0, y0, z, &bar[s]);
    };
    if (tid == 0)
        for (int j = 0; j < RNS && j < n_in; ++j) issue(j);
    auto wait = [&](int j) { return scafes::bounded_wait(&bar[j & (RNS - 1)], (uint32_t)(j >> 2) & 1u); };
    auto fail = [&](int last_issued) {
        if (tid == 0) {
            atomicExch(status, SCAFES_ERR_TIMEOUT);
            for (int j = last_issued - (RNS - 1); j <= last_issued; ++j)
                if (j >= 0 && j < n_in)
                    scafes::bounded_wait(&bar[j & (RNS - 1)], (uint32_t)(j >> 2) & 1u, scafes::kWaitLimitNs / 16);
        }
    };
    const int x = x0 + tx, y = y0 + ty;
    const bool live = x < L.nx && y < L.ny;
    const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
    const int bl = (ty + 1) * RLW + tx + 2, bx = ty * FXW + tx + 2, by = (ty + 1) * FYW + tx;
    const int bk = ty * FKW + tx;
    const float2 zero = make_float2(0.f, 0.f);
    const E ezero = E{};
    constexpr int NT = RTX * RTY;
    // F64: input plane j's lambda and u boxes as pairs into ring slot j & 1.
    auto to_pairs = [&](int j) {
        if constexpr (F64) {
            const E* sj = rsm + (j & (RNS - 1)) * RSLOT;
            float2* pj = pring + (j & 1) * 2 * RPAIR;
            for (int i = tid; i < RLW * RLH; i += NT) {
                pj[i] = pview(sj[RO_L + i]);
                pj[RPAIR + i] = pview(sj[RO_U + i]);
            }
        }
    };
    long long o = live ? L.idx(x, y, z0) : 0;
    float2 gn = live ? g[o] : zero;
    bool ok = wait(0);
    E lb = z0 > 0 ? rsm[RO_L + bl] : ezero;  // plane z0-1
    E ub = z0 > 0 ? rsm[RO_U + bl] : ezero;
    E kzb = z0 > 0 ? rsm[RO_Z + bk] : ezero;
    ok = wait(1) && ok;
    to_pairs(1);
    // Pairs of the centre values of plane z0, then of each plane in turn.
    float2 plc = pview(rsm[RSLOT + RO_L + bl]), puc = pview(rsm[RSLOT + RO_U + bl]);
    // The z-face product of the plane below (face z-1 | z).
    f2 pzb = z0 > 0 ? pface(pview(ub), puc, pview(lb), plc) : f2{0.f, 0.f};
    int issued = RNS - 1;
    for (int z = z0; z < z1; ++z, o += L.plane) {
        const int jc = z - z0 + 1;  // input plane of z
        if (!__syncthreads_and(ok)) {  // plane z-1's slot is free; all waits so far succeeded
            fail(issued);
            return;
        }
        if (tid == 0 && jc + 3 < n_in && jc + 3 > issued) {
            scafes::fence_proxy_async_smem();
            issue(jc + 3);
            issued = jc + 3;
        }
        const float2 gc = gn;
        if (live && z + 1 < z1) gn = g[o + L.plane];
        ok = wait(jc + 1) && ok;  // plane z+1
        to_pairs(jc + 1);         // read from the next iteration on (after its barrier)
        const E* sc = rsm + (jc & (RNS - 1)) * RSLOT;
        const E* sa = rsm + ((jc + 1) & (RNS - 1)) * RSLOT;
        const float2* ppl = pring + (jc & 1) * 2 * RPAIR;  // F64: plane z's pairs
        const float2* ppu = ppl + RPAIR;
        auto PL = [&](int i) -> float2 {
            if constexpr (F64) return ppl[i];
            else return pview(sc[RO_L + i]);
        };
        auto PU = [&](int i) -> float2 {
            if constexpr (F64) return ppu[i];
            else return pview(sc[RO_U + i]);
        };
        const bool top = z + 1 < L.nz;
        const E la = top ? sa[RO_L + bl] : ezero;
        const E ua = top ? sa[RO_U + bl] : ezero;
        const E lc = sc[RO_L + bl];
        const E kzc = sc[RO_Z + bk];
        const float2 pla = pview(la), pua = pview(ua);
        const f2 pza = pface(puc, pua, plc, pla);  // face z | z+1
        if (live) {
            const bool border = colb || z == 0 || z == L.nz - 1;
            const E lxp = sc[RO_L + bl + 1], lxm = sc[RO_L + bl - 1];
            const E lyp = sc[RO_L + bl + RLW], lym = sc[RO_L + bl - RLW];
            // dJ/dk_i: the two faces along each axis.
            f2 gk = pscale2(hx2, pface(puc, PU(bl + 1), plc, PL(bl + 1)), pface(PU(bl - 1), puc, PL(bl - 1), plc));
            pacc(gk, pscale2(hy2, pface(puc, PU(bl + RLW), plc, PL(bl + RLW)),
                             pface(PU(bl - RLW), puc, PL(bl - RLW), plc)));
            pacc(gk, pscale2(hz2, pza, pzb));
            f2 gsum{gc.x, gc.y};
            pacc(gsum, {-gk.hi, -gk.lo});
            g[o] = pnorm(gsum);
            const E kxp = sc[RO_X + bx], kyp = sc[RO_Y + by];
            const E kxm = sc[RO_X + bx - 1], kym = sc[RO_Y + by - FYW];
            if constexpr (F64) {
                // lambda' in FP64; a border row passes its inflow into bnd.
                double v = border ? kxp * lxp : sc[RO_D + bk] * lc;
                if (!border) v = fma(kxp, lxp, v);
                v = fma(kxm, lxm, v);
                v = fma(kyp, lyp, v);
                v = fma(kym, lym, v);
                v = fma(kzc, la, v);
                v = fma(kzb, lb, v);
                if (border) {
                    bnd[o] += v;
                    lamn[o] = 0.0;
                } else {
                    lamn[o] = v;
                }
            } else {
                f2 acc = border ? f2{0.f, 0.f} : pmul(sc[RO_D + bk], lc);
                pacc(acc, pmul(kxp, lxp));
                pacc(acc, pmul(kxm, lxm));
                pacc(acc, pmul(kyp, lyp));
                pacc(acc, pmul(kym, lym));
                pacc(acc, pmul(kzc, la));
                pacc(acc, pmul(kzb, lb));
                if (border) {
                    const float2 bo = bnd[o];
                    pacc(acc, {bo.x, bo.y});
                    bnd[o] = pnorm(acc);
                    lamn[o] = zero;
                } else {
                    lamn[o] = pnorm(acc);
                }
            }
        }
        lb = lc;
        kzb = kzc;
        pzb = pza;
        plc = pla;
        puc = pua;
    }
    if (!__syncthreads_and(ok)) fail(issued);
}

// lambda_T = u_T - target or the cotangent (u_T pairs, target FP64): inner
// part into lam, border part into bnd, per-CTA partial sums of J into part.
__global__ void k_terminal_x2(const float2* __restrict__ uT, const double* __restrict__ target,
                              float2* __restrict__ lam, float2* __restrict__ bnd, double* __restrict__ part, Layout L,
                              bool seed) {
    __shared__ double sh[AX * AY];
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    double acc = 0.0;
    if (x < L.nx && y < L.ny) {
        const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
        for (int z = 0; z < L.nz; ++z) {
            const long long o = L.idx(x, y, z);
            const double d = seed ? target[o] : pjoin(uT[o]) - target[o];
            if (!seed) acc += 0.5 * d * d;
            const bool border = colb || z == 0 || z == L.nz - 1;
            lam[o] = border ? make_float2(0.f, 0.f) : psplit(d);
            bnd[o] = border ? psplit(d) : make_float2(0.f, 0.f);
        }
    }
    const int t = threadIdx.y * AX + threadIdx.x;
    sh[t] = acc;
    __syncthreads();
    for (int s = AX * AY / 2; s > 0; s >>= 1) {
        if (t < s) sh[t] += sh[t + s];
        __syncthreads();
    }
    if (t == 0) part[blockIdx.y * gridDim.x + blockIdx.x] = sh[0];
}

__global__ void k_finalize_x2(const float2* __restrict__ g, const float2* __restrict__ lam,
                              const float2* __restrict__ bnd, double* __restrict__ dk, double* __restrict__ du0,
                              Layout L) {
    const int x = blockIdx.x * AX + threadIdx.x, y = blockIdx.y * AY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    for (int z = 0; z < L.nz; ++z) {
        const long long o = L.idx(x, y, z);
        dk[o] = pjoin(g[o]);
        du0[o] = pjoin(lam[o]) + pjoin(bnd[o]);
    }
}

}  // namespace

struct scafes_adj {
    Layout L;
    double tau = 0.0, w[3] = {0, 0, 0};
    int n_snap = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int precision = SCAFES_PREC_F64;
    // Every field holds 8 bytes per node: FP64 values, or FP32 pairs when
    // precision is SCAFES_PREC_F32X2.
    double *kx = nullptr, *ky = nullptr, *kz = nullptr;
    double *dg = nullptr;      // diagonal of the update, d_i = 1 - sum of i's faces
    double *u[2] = {nullptr, nullptr}, *lam[2] = {nullptr, nullptr};
    double *gx = nullptr, *bnd = nullptr;  // gx: the per-node gradient (an FP32 pair per node)
    double *snaps = nullptr;   // n_snap fields
    double *work = nullptr;    // staging of host arrays (dense doubles)
    double *part = nullptr;    // J partial sums
    int part_n = 0;
    bool have_k = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float fwd_ms = 0.f, grad_ms = 0.f;
    long long fwd_steps = 0, adj_steps = 0;
    // Optimal first splits of the binomial schedule, keyed by (steps, free slots).
    std::unordered_map<long long, int> split_memo;
    // The pair steps' TMA descriptors: one per state buffer and box shape
    // (u[0], u[1], snapshot slots, lambda; encoded on first use) and the
    // four coefficient fields.
    struct StateMap { const void* base; int box; CUtensorMap map; };
    std::vector<StateMap> umaps;
    CUtensorMap cmaps[4];
    bool cmaps_ok = false;
    int* status = nullptr;     // device word: nonzero once a bounded wait ran out
    std::string err;
};

namespace {

int afail(scafes_adj* a, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (a) a->err = buf;
    scafes::set_last_error(buf);
    return code;
}

#define ATRY(a, call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return afail(a, SCAFES_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                                  \
    } while (0)

dim3 grid2(const Layout& L) { return dim3((L.nx + AX - 1) / AX, (L.ny + AY - 1) / AY, 1); }
dim3 grid3(const Layout& L) { return dim3((L.nx + AX - 1) / AX, (L.ny + AY - 1) / AY, (L.nz + 15) / 16); }
size_t field_bytes(const scafes_adj* a) { return (size_t)a->L.size() * sizeof(double); }
double* snap(scafes_adj* a, int s) { return a->snaps + (size_t)s * a->L.size(); }

bool pairs(const scafes_adj* a) { return a->precision == SCAFES_PREC_F32X2; }
const float2* P2(const double* p) { return reinterpret_cast<const float2*>(p); }
float2* P2(double* p) { return reinterpret_cast<float2*>(p); }

// Descriptor of a field of 8-byte elements (FP64 or an FP32 pair) for a box
// of bw x bh nodes.
int pair_map(scafes_adj* a, CUtensorMap* m, const void* base, int bw, int bh) {
    const CUresult r = scafes::make_tensor_map_3d(m, base, 8, a->L.nx, a->L.ny, a->L.nz, (size_t)a->L.pitch * 8,
                                                  (size_t)a->L.plane * 8, bw, bh);
    if (r != CUDA_SUCCESS) return afail(a, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return SCAFES_OK;
}

// State boxes: a one-node halo (the forward step's u, the adjoint step's
// lambda and u).
enum { BOX_HALO = 0 };

// Copies the descriptor of `src` for `box` into *out (the cache may grow,
// so no pointer into it is handed out).
int state_map(scafes_adj* a, const double* src, int box, CUtensorMap* out) {
    for (const auto& e : a->umaps)
        if (e.base == src && e.box == box) {
            *out = e.map;
            return SCAFES_OK;
        }
    scafes_adj::StateMap m{src, box, {}};
    if (int rc = pair_map(a, &m.map, src, FUW, FUH))
        return rc;
    a->umaps.push_back(m);
    *out = m.map;
    return SCAFES_OK;
}

int coefficient_maps(scafes_adj* a) {
    if (a->cmaps_ok) return SCAFES_OK;
    int rc = pair_map(a, &a->cmaps[0], a->kx, FXW, FXH);
    if (!rc) rc = pair_map(a, &a->cmaps[1], a->ky, FYW, FYH);
    if (!rc) rc = pair_map(a, &a->cmaps[2], a->kz, FKW, FKH);
    if (!rc) rc = pair_map(a, &a->cmaps[3], a->dg, FKW, FKH);
    if (rc) return rc;
    ATRY(a, cudaFuncSetAttribute(k_forward_x2_tma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FSMEM));
    ATRY(a, cudaFuncSetAttribute(k_adjoint_x2_tma<float2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RSMEM));
    ATRY(a, cudaFuncSetAttribute(k_adjoint_x2_tma<float2>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
    ATRY(a, cudaFuncSetAttribute(k_adjoint_x2_tma<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)RSMEM_F64));
    ATRY(a, cudaFuncSetAttribute(k_adjoint_x2_tma<double>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 (int)cudaSharedmemCarveoutMaxShared));
    a->cmaps_ok = true;
    return SCAFES_OK;
}

int fwd_x2_tma(scafes_adj* a, const double* src, double* dst) {
    if (int rc = coefficient_maps(a)) return rc;
    CUtensorMap mu;
    if (int rc = state_map(a, src, BOX_HALO, &mu)) return rc;
    const dim3 grid((a->L.nx + FTX - 1) / FTX, (a->L.ny + FTY - 1) / FTY, (a->L.nz + FZ_ - 1) / FZ_);
    k_forward_x2_tma<<<grid, dim3(FTX, FTY), FSMEM, a->stream>>>(mu, a->cmaps[0], a->cmaps[1], a->cmaps[2],
                                                                  a->cmaps[3], P2(dst), a->L, a->status);
    return SCAFES_OK;
}

// Reads the device status word after the work queued so far and clears it.
int check_status(scafes_adj* a, const char* who) {
    int st = 0;
    ATRY(a, cudaMemcpyAsync(&st, a->status, sizeof(int), cudaMemcpyDeviceToHost, a->stream));
    ATRY(a, cudaStreamSynchronize(a->stream));
    if (st == 0) return SCAFES_OK;
    ATRY(a, cudaMemsetAsync(a->status, 0, sizeof(int), a->stream));
    ATRY(a, cudaStreamSynchronize(a->stream));
    return afail(a, st, "%s: a bounded device wait ran out (status %d); the result is invalid", who, st);
}

int fwd(scafes_adj* a, const double* src, double* dst) {
    if (pairs(a)) {
        const int rc = fwd_x2_tma(a, src, dst);
        if (rc) return rc;
    } else
        k_forward<<<grid3(a->L), dim3(AX, AY), 0, a->stream>>>(src, dst, a->kx, a->ky, a->kz, a->dg, a->L);
    ATRY(a, cudaGetLastError());
    ++a->fwd_steps;
    return SCAFES_OK;
}

// lambda_T, the border part of dJ/du0 and the partial sums of J from u_T.
int terminal(scafes_adj* a, const double* uT, const double* target, double* lam, double* Jpart, bool seed) {
    if (pairs(a))
        k_terminal_x2<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(P2(uT), target, P2(lam), P2(a->bnd), Jpart, a->L,
                                                                   seed);
    else
        k_terminal<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(uT, target, lam, a->bnd, Jpart, a->L, seed);
    ATRY(a, cudaGetLastError());
    return SCAFES_OK;
}

// Converts a field in place between host-facing FP64 and the sweep's type.
int to_sweep_type(scafes_adj* a, double* buf) {
    if (!pairs(a)) return SCAFES_OK;
    k_to_pair<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(buf, a->L);
    ATRY(a, cudaGetLastError());
    return SCAFES_OK;
}

int from_sweep_type(scafes_adj* a, double* buf) {
    if (!pairs(a)) return SCAFES_OK;
    k_from_pair<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(buf, a->L);
    ATRY(a, cudaGetLastError());
    return SCAFES_OK;
}

// Optimal binomial schedule.  cost(n, s) = fewest forward steps that
// reverse n steps starting from a stored state with s free snapshots, the
// minimum of
//   cost(1, s) = 0,  cost(n, 0) = n(n-1)/2,
//   cost(n, s) = min_m  m + cost(n - m, s - 1) + cost(m, s)
// (advance m steps, store the state, reverse the right part with one slot
// fewer, then the left part).  Its closed form (Griewank 1992; Griewank &
// Walther, "Algorithm 799: revolve", ACM TOMS 26(1), 2000): with c = s + 1
// checkpoints and r the fewest repetitions for which C(c + r, c) >= n,
//   cost(n, s) = r n - C(c + r, c + 1),
// which the tests check against the recursion.  The first split of a
// reversal is an m that attains the minimum, found by a scan and memoised
// per (n, s): no table grows with the snapshot count, so every slot the
// caller gives is used.
long long binomial_cost(long long n, long long s) {
    if (n <= 1) return 0;
    if (s <= 0) return n * (n - 1) / 2;
    if (s >= n - 1) return n - 1;
    const long long c = s + 1;
    long long r = 0, beta = 1;  // beta = C(c + r, c)
    while (beta < n) {
        ++r;
        beta = beta * (c + r) / r;
    }
    return r * n - beta * r / (c + 1);  // C(c + r, c + 1) = C(c + r, c) r / (c + 1)
}

int split_of(scafes_adj* a, int n, int s) {
    if (s >= n - 1) return 1;
    const long long key = (long long)n * 4194304LL + s;
    const auto it = a->split_memo.find(key);
    if (it != a->split_memo.end()) return it->second;
    const long long best = binomial_cost(n, s);
    int m_best = 1;
    for (int m = 1; m < n; ++m)
        if (m + binomial_cost(n - m, s - 1) + binomial_cost(m, s) == best) {
            m_best = m;
            break;
        }
    a->split_memo.emplace(key, m_best);
    return m_best;
}

// Free snapshot slots the schedule uses: all states when they fit, else
// every slot but the one holding u0.
int schedule_slots(int n_snap, int n_steps) {
    const int free = n_snap - 1;
    return free >= n_steps - 1 ? n_steps - 1 : free;
}

struct Rev {
    scafes_adj* a;
    const double* target;  // J's target, or dJ/du_T itself when `seed`
    int T;
    int cur;  // lambda buffer holding lambda_b
    bool started;
    double* Jpart;
    bool seed;
    // Border nodes reset to a fixed value every step (a Dirichlet border)
    // instead of held at u0's values: u0's border then enters only the first
    // step, and the border part of dJ/du0 is that step's alone.
    bool reset_border = false;
};

int adj_step(Rev& R, const double* u_t) {
    scafes_adj* a = R.a;
    if (R.reset_border && a->adj_steps == R.T - 1)
        ATRY(a, cudaMemsetAsync(a->bnd, 0, field_bytes(a), a->stream));  // the last step is t = 0 -> 1
    if (int rc = coefficient_maps(a)) return rc;
    CUtensorMap ml, mu;
    if (int rc = state_map(a, a->lam[R.cur], BOX_HALO, &ml)) return rc;
    if (int rc = state_map(a, u_t, BOX_HALO, &mu)) return rc;
    const dim3 grid((a->L.nx + RTX - 1) / RTX, (a->L.ny + RTY - 1) / RTY, (a->L.nz + RZ_ - 1) / RZ_);
    auto half = [](double w) {
        const f2 p = split_double(0.5 * w);
        return make_float2(p.hi, p.lo);
    };
    if (pairs(a))
        k_adjoint_x2_tma<float2><<<grid, dim3(RTX, RTY), RSMEM, a->stream>>>(
            ml, mu, a->cmaps[0], a->cmaps[1], a->cmaps[2], a->cmaps[3], P2(a->lam[R.cur ^ 1]), P2(a->gx),
            P2(a->bnd), half(a->w[0]), half(a->w[1]), half(a->w[2]), a->L, a->status);
    else
        k_adjoint_x2_tma<double><<<grid, dim3(RTX, RTY), RSMEM_F64, a->stream>>>(
            ml, mu, a->cmaps[0], a->cmaps[1], a->cmaps[2], a->cmaps[3], a->lam[R.cur ^ 1], P2(a->gx), a->bnd,
            half(a->w[0]), half(a->w[1]), half(a->w[2]), a->L, a->status);
    ATRY(a, cudaGetLastError());
    R.cur ^= 1;
    ++a->adj_steps;
    return SCAFES_OK;
}

// Reverses steps [lo, hi): the state u_lo is in snapshot slot `slot`;
// `free` further slots (slot+1 .. slot+free) may be used.
int reverse(Rev& R, int lo, int hi, int slot, int free) {
    scafes_adj* a = R.a;
    int rc;
    if (hi - lo == 1) {
        if (!R.started) {
            // Bottom of the first descent: u_T from u_{T-1} gives J and lambda_T.
            if ((rc = fwd(a, snap(a, slot), a->u[0]))) return rc;
            if ((rc = terminal(a, a->u[0], R.target, a->lam[R.cur], R.Jpart, R.seed))) return rc;
            R.started = true;
        }
        return adj_step(R, snap(a, slot));
    }
    if (free == 0) {
        // No slot left: recompute every state from u_lo.
        for (int t = hi - 1; t >= lo; --t) {
            const double* src = snap(a, slot);
            int buf = 0;
            for (int s = lo; s < t; ++s) {
                if ((rc = fwd(a, src, a->u[buf]))) return rc;
                src = a->u[buf];
                buf ^= 1;
            }
            if (t == hi - 1 && !R.started) {
                if ((rc = fwd(a, src, a->u[buf]))) return rc;
                if ((rc = terminal(a, a->u[buf], R.target, a->lam[R.cur], R.Jpart, R.seed))) return rc;
                R.started = true;
            }
            if ((rc = adj_step(R, src))) return rc;
        }
        return SCAFES_OK;
    }
    const int m = lo + split_of(a, hi - lo, free);
    // Advance u_lo -> u_m into slot+1.
    const double* src = snap(a, slot);
    int buf = 0;
    for (int s = lo; s < m - 1; ++s) {
        if ((rc = fwd(a, src, a->u[buf]))) return rc;
        src = a->u[buf];
        buf ^= 1;
    }
    if ((rc = fwd(a, src, snap(a, slot + 1)))) return rc;
    if ((rc = reverse(R, m, hi, slot + 1, free - 1))) return rc;
    return reverse(R, lo, m, slot, free);
}

int upload_dense(scafes_adj* a, const double* host, double* dev) {
    const Layout& L = a->L;
    ATRY(a, cudaMemcpy2DAsync(dev, (size_t)L.pitch * sizeof(double), host, (size_t)L.nx * sizeof(double),
                              (size_t)L.nx * sizeof(double), (size_t)L.ny * L.nz, cudaMemcpyHostToDevice, a->stream));
    return SCAFES_OK;
}

int download_dense(scafes_adj* a, const double* dev, double* host) {
    const Layout& L = a->L;
    ATRY(a, cudaMemcpy2DAsync(host, (size_t)L.nx * sizeof(double), dev, (size_t)L.pitch * sizeof(double),
                              (size_t)L.nx * sizeof(double), (size_t)L.ny * L.nz, cudaMemcpyDeviceToHost, a->stream));
    return SCAFES_OK;
}

}  // namespace

extern "C" const char* scafes_adj_last_error(const scafes_adj* a) { return a ? a->err.c_str() : ""; }

extern "C" void scafes_adj_destroy(scafes_adj* a) {
    if (!a) return;
    if (a->stream) cudaStreamSynchronize(a->stream);
    double* bufs[] = {a->kx, a->ky, a->kz, a->dg, a->u[0], a->u[1], a->lam[0], a->lam[1], a->gx, a->bnd,
                      a->snaps, a->work, a->part};
    for (double* b : bufs) cudaFree(b);
    cudaFree(a->status);
    if (a->e0) cudaEventDestroy(a->e0);
    if (a->e1) cudaEventDestroy(a->e1);
    if (a->own_stream && a->stream) cudaStreamDestroy(a->stream);
    delete a;
}

extern "C" int scafes_adj_create(const int n_nodes[3], const double coord_first[3], const double coord_last[3],
                                 double tau, int n_snapshots, void* stream, scafes_adj** out) {
    if (!out || !n_nodes || !coord_first || !coord_last)
        return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_create: NULL argument");
    *out = nullptr;
    for (int p = 0; p < 3; ++p)
        if (n_nodes[p] < 3 || n_nodes[p] > (1 << 16))
            return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_create: n_nodes[%d]=%d out of [3, 65536]", p, n_nodes[p]);
    if (n_snapshots < 2) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_create: need at least 2 snapshots");
    if (!(tau > 0.0)) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_create: tau must be > 0");
    scafes_adj* a = new (std::nothrow) scafes_adj();
    if (!a) return afail(nullptr, SCAFES_ERR_NOMEM, "scafes_adj_create: out of host memory");
    a->L = make_layout(n_nodes[0], n_nodes[1], n_nodes[2]);
    a->tau = tau;
    for (int p = 0; p < 3; ++p) {
        const double h = (coord_last[p] - coord_first[p]) / (n_nodes[p] - 1);
        a->w[p] = tau / (h * h);
    }
    a->n_snap = n_snapshots;
    const size_t fb = field_bytes(a);
    cudaError_t e = cudaSuccess;
    if (stream) a->stream = (cudaStream_t)stream;
    else { e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking); a->own_stream = true; }
    double** fields[] = {&a->kx, &a->ky, &a->kz, &a->dg, &a->u[0], &a->u[1], &a->lam[0], &a->lam[1], &a->gx,
                         &a->bnd, &a->work};
    for (double** f : fields)
        if (e == cudaSuccess) e = cudaMalloc(f, fb);
    if (e == cudaSuccess) e = cudaMalloc(&a->snaps, fb * (size_t)n_snapshots);
    a->part_n = grid2(a->L).x * grid2(a->L).y;
    if (e == cudaSuccess) e = cudaMalloc(&a->part, sizeof(double) * a->part_n);
    if (e == cudaSuccess) e = cudaMalloc(&a->status, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(a->status, 0, sizeof(int), a->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(a->snaps, 0, fb * (size_t)n_snapshots, a->stream);
    for (double** f : fields)
        if (e == cudaSuccess) e = cudaMemsetAsync(*f, 0, fb, a->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&a->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&a->e1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(a->stream);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? SCAFES_ERR_NOMEM : SCAFES_ERR_CUDA;
        afail(nullptr, code, "scafes_adj_create: %s (%d snapshots of %zu bytes)", cudaGetErrorString(e), n_snapshots, fb);
        scafes_adj_destroy(a);
        return code;
    }
    *out = a;
    return SCAFES_OK;
}

extern "C" int scafes_adj_set_precision(scafes_adj* a, int precision) {
    if (!a) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_set_precision: NULL handle");
    if (precision != SCAFES_PREC_F64 && precision != SCAFES_PREC_F32X2)
        return afail(a, SCAFES_ERR_UNSUPPORTED, "scafes_adj_set_precision: precision %d (F64 or F32X2 only)", precision);
    a->precision = precision;
    a->have_k = false;
    return SCAFES_OK;
}

namespace {

__global__ void k_fill(double* __restrict__ f, long long n, double v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        f[i] = v;
}

// Face conductivities (and the pair diagonal) from the node values in `work`.
int prepare_faces(scafes_adj* a) {
    if (pairs(a))
        k_prep_x2<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(a->work, P2(a->kx), P2(a->ky), P2(a->kz), P2(a->dg),
                                                               a->L, a->w[0], a->w[1], a->w[2]);
    else
        k_faces<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(a->work, a->kx, a->ky, a->kz, a->dg, a->L, a->w[0],
                                                             a->w[1], a->w[2]);
    ATRY(a, cudaGetLastError());
    ATRY(a, cudaStreamSynchronize(a->stream));
    a->have_k = true;
    return SCAFES_OK;
}

}  // namespace

extern "C" int scafes_adj_set_conductivity(scafes_adj* a, const double* k, size_t n) {
    if (!a || !k) return afail(a, SCAFES_ERR_ARG, "scafes_adj_set_conductivity: NULL argument");
    if (n != (size_t)a->L.nx * a->L.ny * a->L.nz)
        return afail(a, SCAFES_ERR_ARG, "scafes_adj_set_conductivity: expected %zu values",
                     (size_t)a->L.nx * a->L.ny * a->L.nz);
    int rc = upload_dense(a, k, a->work);
    if (rc) return rc;
    return prepare_faces(a);
}

extern "C" int scafes_adj_set_conductivity_uniform(scafes_adj* a, double k) {
    if (!a) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_set_conductivity_uniform: NULL handle");
    if (!(k > 0.0) || !std::isfinite(k))
        return afail(a, SCAFES_ERR_ARG, "scafes_adj_set_conductivity_uniform: k = %g must be finite and > 0", k);
    k_fill<<<1024, 256, 0, a->stream>>>(a->work, a->L.size(), k);
    ATRY(a, cudaGetLastError());
    return prepare_faces(a);
}

extern "C" int scafes_adj_forward(scafes_adj* a, const double* u0, int n_steps, double* uT, size_t n) {
    if (!a || !u0 || !uT || n_steps < 0) return afail(a, SCAFES_ERR_ARG, "scafes_adj_forward: bad arguments");
    if (n != (size_t)a->L.nx * a->L.ny * a->L.nz) return afail(a, SCAFES_ERR_ARG, "scafes_adj_forward: wrong size");
    if (!a->have_k) return afail(a, SCAFES_ERR_STATE, "scafes_adj_forward: set the conductivity first");
    int rc = upload_dense(a, u0, a->u[0]);
    if (rc) return rc;
    if ((rc = to_sweep_type(a, a->u[0]))) return rc;
    a->fwd_steps = 0;
    ATRY(a, cudaEventRecord(a->e0, a->stream));
    int cur = 0;
    for (int s = 0; s < n_steps; ++s) {
        if ((rc = fwd(a, a->u[cur], a->u[cur ^ 1]))) return rc;
        cur ^= 1;
    }
    ATRY(a, cudaEventRecord(a->e1, a->stream));
    if ((rc = from_sweep_type(a, a->u[cur]))) return rc;
    if ((rc = download_dense(a, a->u[cur], uT))) return rc;
    ATRY(a, cudaStreamSynchronize(a->stream));
    if ((rc = check_status(a, "scafes_adj_forward"))) return rc;
    ATRY(a, cudaEventElapsedTime(&a->fwd_ms, a->e0, a->e1));
    return SCAFES_OK;
}

// The reverse sweep from u0 over n_steps: `target` is J's target
// (J = 0.5 |u_T - target|^2) or, with `seed`, the cotangent dJ/du_T.
// With u0_dev, u0 is a device field in the handle's padded FP64 layout.
static int gradient_impl(scafes_adj* a, const char* who, const double* u0, const double* target, bool seed,
                         int n_steps, double* J, double* grad_k, double* grad_u0, size_t n, bool u0_dev = false,
                         bool reset_border = false) {
    if (!a || !u0 || !target || !grad_k || !grad_u0 || n_steps < 1)
        return afail(a, SCAFES_ERR_ARG, "%s: bad arguments", who);
    if (n != (size_t)a->L.nx * a->L.ny * a->L.nz) return afail(a, SCAFES_ERR_ARG, "%s: wrong size", who);
    if (!a->have_k) return afail(a, SCAFES_ERR_STATE, "%s: set the conductivity first", who);
    const int free = schedule_slots(a->n_snap, n_steps);
    const size_t fb = field_bytes(a);
    int rc = SCAFES_OK;
    if (u0_dev)
        ATRY(a, cudaMemcpyAsync(snap(a, 0), u0, fb, cudaMemcpyDeviceToDevice, a->stream));
    else if ((rc = upload_dense(a, u0, snap(a, 0))))
        return rc;
    if ((rc = to_sweep_type(a, snap(a, 0)))) return rc;
    // The target goes to u[1]'s slot only transiently: keep it in `work`.
    if ((rc = upload_dense(a, target, a->work))) return rc;
    ATRY(a, cudaMemsetAsync(a->gx, 0, fb, a->stream));
    a->fwd_steps = 0;
    a->adj_steps = 0;
    ATRY(a, cudaEventRecord(a->e0, a->stream));
    Rev R{a, a->work, n_steps, 0, false, a->part, seed, reset_border};
    if ((rc = reverse(R, 0, n_steps, 0, free))) return rc;
    if (pairs(a))
        k_finalize_x2<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(P2(a->gx), P2(a->lam[R.cur]), P2(a->bnd),
                                                                   a->u[0], a->u[1], a->L);
    else
        k_finalize<<<grid2(a->L), dim3(AX, AY), 0, a->stream>>>(P2(a->gx), a->lam[R.cur], a->bnd, a->u[0],
                                                                a->u[1], a->L);
    ATRY(a, cudaGetLastError());
    ATRY(a, cudaEventRecord(a->e1, a->stream));
    std::vector<double> part(a->part_n);
    ATRY(a, cudaMemcpyAsync(part.data(), a->part, sizeof(double) * a->part_n, cudaMemcpyDeviceToHost, a->stream));
    if ((rc = download_dense(a, a->u[0], grad_k))) return rc;
    if ((rc = download_dense(a, a->u[1], grad_u0))) return rc;
    ATRY(a, cudaStreamSynchronize(a->stream));
    if ((rc = check_status(a, who))) return rc;
    ATRY(a, cudaEventElapsedTime(&a->grad_ms, a->e0, a->e1));
    if (J) {
        double s = 0.0;
        for (double v : part) s += v;
        *J = s;
    }
    return SCAFES_OK;
}

extern "C" int scafes_adj_gradient(scafes_adj* a, const double* u0, const double* target, int n_steps, double* J,
                                   double* grad_k, double* grad_u0, size_t n) {
    if (!J) return afail(a, SCAFES_ERR_ARG, "scafes_adj_gradient: bad arguments");
    return gradient_impl(a, "scafes_adj_gradient", u0, target, false, n_steps, J, grad_k, grad_u0, n);
}

extern "C" int scafes_adj_backward(scafes_adj* a, const double* u0, const double* dJ_duT, int n_steps,
                                   double* grad_k, double* grad_u0, size_t n) {
    return gradient_impl(a, "scafes_adj_backward", u0, dJ_duT, true, n_steps, nullptr, grad_k, grad_u0, n);
}

namespace scafes {
int adj_backward_device_u0(scafes_adj* a, const double* u0_dev, const double* dJ_duT, int n_steps, double* grad_k,
                           double* grad_u0, size_t n) {
    return gradient_impl(a, "scafes_gpu_adjoint", u0_dev, dJ_duT, true, n_steps, nullptr, grad_k, grad_u0, n, true,
                         true);
}
}  // namespace scafes

extern "C" int scafes_adj_inject_status(scafes_adj* a, int code) {
    if (!a) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_inject_status: NULL handle");
    if (code > 0) return afail(a, SCAFES_ERR_ARG, "scafes_adj_inject_status: code %d > 0", code);
    ATRY(a, cudaMemcpyAsync(a->status, &code, sizeof(int), cudaMemcpyHostToDevice, a->stream));
    ATRY(a, cudaStreamSynchronize(a->stream));
    return SCAFES_OK;
}

extern "C" int scafes_adj_stats(const scafes_adj* a, float* forward_ms, float* gradient_ms, long long* forward_steps,
                                long long* adjoint_steps, int* snapshots) {
    if (!a) return afail(nullptr, SCAFES_ERR_ARG, "scafes_adj_stats: NULL handle");
    if (forward_ms) *forward_ms = a->fwd_ms;
    if (gradient_ms) *gradient_ms = a->grad_ms;
    if (forward_steps) *forward_steps = a->fwd_steps;
    if (adjoint_steps) *adjoint_steps = a->adj_steps;
    if (snapshots) *snapshots = a->n_snap;
    return SCAFES_OK;
}

extern "C" long long scafes_adj_schedule_cost(int n_steps, int n_snapshots) {
    if (n_steps < 1 || n_snapshots < 1) return -1;
    const int free = schedule_slots(n_snapshots, n_steps);
    if (free >= n_steps - 1) return n_steps;  // one sweep, every state stored
    return binomial_cost(n_steps, free) + 1;  // + the step that gives u_T
}
