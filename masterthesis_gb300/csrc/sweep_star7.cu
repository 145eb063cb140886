// Plain 7-point sweep: one launch advances the whole grid by one time step.
//
// Replaces the per-node loop of ScaFES's evalTypeTwoAt
// (src/ScaFES_Problem.hpp:5399-5476) for the heat-type callbacks
// (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218,
//  tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168) and
// their Dirichlet border (.../Dirichlet/Dirichlet.hpp:125-131), and the copy
// old->new that precedes it (:5078-5082): every node is written each step.
//
// Mapping: a CTA owns a BX x BY column tile and marches it through a chunk
// of z-planes.  Each thread keeps u(z-1), u(z), u(z+1) of its column in
// registers; the x/y neighbours come from the current plane staged in
// double-buffered shared memory (one __syncthreads per plane).  Global loads
// and stores are row-contiguous across a warp (32 consecutive x).
#include "star7.cuh"
#include "../../include/scafes_gb300.h"

namespace scafes {

// ---- arithmetic policies ---------------------------------------------------

struct PolF64 {
    using T = double;
    static __device__ __forceinline__ T zero() { return 0.0; }
    static __device__ __forceinline__ T from_double(double d) { return d; }
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
    static __device__ __forceinline__ T mirror(T u, T uo, double corr) {
        return (u + uo) - corr;
    }
    static __device__ __forceinline__ T src(T fa, T fb, double time, bool has_b) {
        return has_b ? fa + time * fb : fa;
    }
};

struct PolF32 {
    using T = float;
    static __device__ __forceinline__ T zero() { return 0.0f; }
    static __device__ __forceinline__ T from_double(double d) { return (float)d; }
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
    static __device__ __forceinline__ T mirror(T u, T uo, double corr) {
        return (u + uo) - (float)corr;
    }
    static __device__ __forceinline__ T src(T fa, T fb, double time, bool has_b) {
        return has_b ? fa + (float)time * fb : fa;
    }
};

// Compensated FP32 pair.  The value of a node is hi + lo.  The update
// computes the exact sums of the hi parts per axis (TwoSum), the exact
// products of those sums with the hi part of each coefficient (FMA TwoProd)
// and their exact sum (TwoSum); everything of relative size 2^-24 (lo parts,
// coefficient tails, rounding errors) is accumulated in plain FP32, which
// contributes errors of relative size 2^-48.  A final FastTwoSum renormalises.
struct PolF32x2 {
    using T = float2;
    static __device__ __forceinline__ T zero() { return make_float2(0.f, 0.f); }
    static __device__ __forceinline__ T from_double(double d) {
        f2 p = split_double(d);
        return make_float2(p.hi, p.lo);
    }
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
        // Products with the hi coefficient, exact via FMA.
        float p0 = c.c0h * u.x;
        float r0 = fmaf(c.c0h, u.x, -p0);
        r0 = fmaf(c.c0l, u.x, r0);
        r0 = fmaf(c.c0h, u.y, r0);
        float px = c.cxh * sx.hi;
        float rx = fmaf(c.cxh, sx.hi, -px);
        rx = fmaf(c.cxl, sx.hi, rx);
        rx = fmaf(c.cxh, tx, rx);
        float py = c.cyh * sy.hi;
        float ry = fmaf(c.cyh, sy.hi, -py);
        ry = fmaf(c.cyl, sy.hi, ry);
        ry = fmaf(c.cyh, ty, ry);
        float pz = c.czh * sz.hi;
        float rz = fmaf(c.czh, sz.hi, -pz);
        rz = fmaf(c.czl, sz.hi, rz);
        rz = fmaf(c.czh, tz, rz);
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
            f2 a4 = two_sum(hi, pf);
            hi = a4.hi;
            r += rf + a4.lo;
        }
        f2 out = fast_two_sum(hi, r);
        return make_float2(out.hi, out.lo);
    }
    static __device__ __forceinline__ T mirror(T u, T uo, double corr) {
        // (u + uo) - corr with corr a power of two (exact in FP32).
        f2 s = two_sum(u.x, uo.x);
        float lo = s.lo + (u.y + uo.y);
        f2 d = two_sum(s.hi, -(float)corr);
        f2 out = fast_two_sum(d.hi, d.lo + lo);
        return make_float2(out.hi, out.lo);
    }
    static __device__ __forceinline__ T src(T fa, T fb, double time, bool has_b) {
        if (!has_b) return fa;
        // fa + time * fb in FP64 is cheap here: F_B is rare (time-dependent
        // sources only); split the result back.
        double v = ((double)fa.x + (double)fa.y) + time * ((double)fb.x + (double)fb.y);
        return from_double(v);
    }
};

// ---- the sweep kernel --------------------------------------------------------

constexpr int BX = 32;
constexpr int BY = 8;

template <class P, bool HAS_F, int BORDER>
__global__ void __launch_bounds__(BX * BY)
star7_sweep(const typename P::T* __restrict__ uo, typename P::T* __restrict__ un,
            const typename P::T* __restrict__ fa, const typename P::T* __restrict__ fb,
            const double* __restrict__ ga, const double* __restrict__ gb,
            Layout L, Star7Coeffs c, double time_old, double time_new,
            double corr, int zchunk)
{
    using T = typename P::T;
    __shared__ T sm[2][BY + 2][BX + 2];

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int x = blockIdx.x * BX + tx;
    const int y = blockIdx.y * BY + ty;
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, L.nz);
    const bool active = (x < L.nx) && (y < L.ny);
    const bool col_border = active && (x == 0 || x == L.nx - 1 || y == 0 || y == L.ny - 1);
    const long long col = (long long)y * L.pitch + x;
    const bool has_fb = (fb != nullptr);
    const bool has_gb = (gb != nullptr);

    T below = P::zero(), cur = P::zero(), above = P::zero();
    if (active) {
        if (z0 > 0) below = uo[col + (long long)(z0 - 1) * L.plane];
        cur = uo[col + (long long)z0 * L.plane];
    }
    for (int z = z0; z < z1; ++z) {
        const long long off = col + (long long)z * L.plane;
        if (active && z + 1 < L.nz) above = uo[off + L.plane];
        const int buf = (z - z0) & 1;
        sm[buf][ty + 1][tx + 1] = cur;
        if (tx == 0)
            sm[buf][ty + 1][0] = (active && x > 0) ? uo[off - 1] : P::zero();
        if (tx == BX - 1)
            sm[buf][ty + 1][BX + 1] = (y < L.ny && x + 1 < L.nx) ? uo[off + 1] : P::zero();
        if (ty == 0)
            sm[buf][0][tx + 1] = (active && y > 0) ? uo[off - L.pitch] : P::zero();
        if (ty == BY - 1)
            sm[buf][BY + 1][tx + 1] = (x < L.nx && y + 1 < L.ny) ? uo[off + L.pitch] : P::zero();
        __syncthreads();
        if (active) {
            const bool border = col_border || z == 0 || z == L.nz - 1;
            T v;
            if (!border) {
                T f = P::zero();
                if (HAS_F) f = P::src(fa[off], has_fb ? fb[off] : P::zero(), time_old, has_fb);
                v = P::template star<HAS_F>(c, cur,
                                            sm[buf][ty + 1][tx], sm[buf][ty + 1][tx + 2],
                                            sm[buf][ty][tx + 1], sm[buf][ty + 2][tx + 1],
                                            below, above, f);
            } else if (BORDER == SCAFES_BORDER_DIRICHLET) {
                double g = ga ? ga[off] : 0.0;
                if (has_gb) g += time_new * gb[off];
                v = P::from_double(g);
            } else {
                // Mirror border: the last face (in direction order x-, x+,
                // y-, y+, z-, z+) the node lies on decides.
                T opp;
                double cc;
                if (z == L.nz - 1)      { opp = below; cc = -corr; }
                else if (z == 0)        { opp = above; cc = corr; }
                else if (y == L.ny - 1) { opp = sm[buf][ty][tx + 1]; cc = -corr; }
                else if (y == 0)        { opp = sm[buf][ty + 2][tx + 1]; cc = corr; }
                else if (x == L.nx - 1) { opp = sm[buf][ty + 1][tx]; cc = -corr; }
                else                    { opp = sm[buf][ty + 1][tx + 2]; cc = corr; }
                v = P::mirror(cur, opp, cc);
            }
            un[off] = v;
        }
        below = cur;
        cur = above;
    }
}

// ---- host side ---------------------------------------------------------------

Star7Coeffs make_star7_coeffs(double c0, const double cp[3], double cf) {
    Star7Coeffs c;
    c.c0 = c0; c.cx = cp[0]; c.cy = cp[1]; c.cz = cp[2]; c.cf = cf;
    f2 s;
    s = split_double(c0);    c.c0h = s.hi; c.c0l = s.lo;
    s = split_double(cp[0]); c.cxh = s.hi; c.cxl = s.lo;
    s = split_double(cp[1]); c.cyh = s.hi; c.cyl = s.lo;
    s = split_double(cp[2]); c.czh = s.hi; c.czl = s.lo;
    s = split_double(cf);    c.cfh = s.hi; c.cfl = s.lo;
    return c;
}

size_t element_size(int precision) {
    switch (precision) {
        case SCAFES_PREC_F64: return sizeof(double);
        case SCAFES_PREC_F32X2: return sizeof(float2);
        case SCAFES_PREC_F32: return sizeof(float);
        default: return 0;
    }
}

static int num_sms() {
    static int n = 0;
    if (n == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

template <class P, bool HAS_F, int BORDER>
static cudaError_t launch_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    const Layout& L = a.L;
    dim3 block(BX, BY, 1);
    const int gx = (L.nx + BX - 1) / BX, gy = (L.ny + BY - 1) / BY;
    // Enough CTAs for ~8 per SM; each z-chunk re-reads one halo plane.
    const long long tiles = (long long)gx * gy;
    const long long want = (long long)num_sms() * 8;
    int nchunks = (int)((want + tiles - 1) / tiles);
    if (nchunks < 1) nchunks = 1;
    int zchunk = (L.nz + nchunks - 1) / nchunks;
    if (zchunk < 8) zchunk = 8;
    nchunks = (L.nz + zchunk - 1) / zchunk;
    dim3 grid(gx, gy, nchunks);
    star7_sweep<P, HAS_F, BORDER><<<grid, block, 0, stream>>>(
        (const T*)a.uo, (T*)a.un, (const T*)a.fa, (const T*)a.fb, a.ga, a.gb, L, a.c,
        a.time_old, a.time_new, a.mirror_corr, zchunk);
    return cudaGetLastError();
}

template <class P>
static cudaError_t launch_prec(const Star7Launch& a, cudaStream_t stream) {
    const bool has_f = (a.fa != nullptr) && (a.c.cf != 0.0);
    if (a.border == SCAFES_BORDER_DIRICHLET) {
        return has_f ? launch_typed<P, true, SCAFES_BORDER_DIRICHLET>(a, stream)
                     : launch_typed<P, false, SCAFES_BORDER_DIRICHLET>(a, stream);
    }
    return has_f ? launch_typed<P, true, SCAFES_BORDER_MIRROR_POW2>(a, stream)
                 : launch_typed<P, false, SCAFES_BORDER_MIRROR_POW2>(a, stream);
}

cudaError_t launch_star7(const Star7Launch& a, cudaStream_t stream) {
    switch (a.precision) {
        case SCAFES_PREC_F64: return launch_prec<PolF64>(a, stream);
        case SCAFES_PREC_F32: return launch_prec<PolF32>(a, stream);
        case SCAFES_PREC_F32X2: return launch_prec<PolF32x2>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

// ---- layout conversion kernels ---------------------------------------------

template <int PREC>
__global__ void k_to_device(const double* __restrict__ dense, void* __restrict__ field, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % L.nx);
        const long long r = m / L.nx;
        const int j = (int)(r % L.ny);
        const int k = (int)(r / L.ny);
        const long long o = L.idx(i, j, k);
        const double v = dense[m];
        if (PREC == SCAFES_PREC_F64) ((double*)field)[o] = v;
        else if (PREC == SCAFES_PREC_F32) ((float*)field)[o] = (float)v;
        else { f2 p = split_double(v); ((float2*)field)[o] = make_float2(p.hi, p.lo); }
    }
}

template <int PREC>
__global__ void k_from_device(const void* __restrict__ field, double* __restrict__ dense, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % L.nx);
        const long long r = m / L.nx;
        const int j = (int)(r % L.ny);
        const int k = (int)(r / L.ny);
        const long long o = L.idx(i, j, k);
        double v;
        if (PREC == SCAFES_PREC_F64) v = ((const double*)field)[o];
        else if (PREC == SCAFES_PREC_F32) v = (double)((const float*)field)[o];
        else { float2 p = ((const float2*)field)[o]; v = join_pair(p.x, p.y); }
        dense[m] = v;
    }
}

cudaError_t convert_to_device(int precision, const double* dense, void* field,
                              const Layout& L, cudaStream_t stream) {
    const int blocks = num_sms() * 4, threads = 256;
    switch (precision) {
        case SCAFES_PREC_F64: k_to_device<SCAFES_PREC_F64><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        case SCAFES_PREC_F32: k_to_device<SCAFES_PREC_F32><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        case SCAFES_PREC_F32X2: k_to_device<SCAFES_PREC_F32X2><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t convert_from_device(int precision, const void* field, double* dense,
                                const Layout& L, cudaStream_t stream) {
    const int blocks = num_sms() * 4, threads = 256;
    switch (precision) {
        case SCAFES_PREC_F64: k_from_device<SCAFES_PREC_F64><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        case SCAFES_PREC_F32: k_from_device<SCAFES_PREC_F32><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        case SCAFES_PREC_F32X2: k_from_device<SCAFES_PREC_F32X2><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace scafes
