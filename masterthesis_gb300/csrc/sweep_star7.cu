// Plain 7-point sweep: one launch advances the whole grid by one time step.
//
// Replaces the per-node loop of ScaFES's evalTypeTwoAt
// (src/ScaFES_Problem.hpp:5399-5476) for the heat-type callbacks
// (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218,
//  tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168) and
// their Dirichlet border (.../Dirichlet/Dirichlet.hpp:125-131), and the copy
// old->new that precedes it (:5078-5082): every node is written each step.
// Each CTA runs one tile (star7_tile.cuh) over a chunk of z-planes.
#include "star7_tile.cuh"

namespace scafes {

template <class P, int SRC, int BORDER, int BY, int R, int NS, bool FS>
__global__ void __launch_bounds__(BX * (BY / R))
star7_tma(const __grid_constant__ CUtensorMap tm, const __grid_constant__ CUtensorMap tmf,
          typename P::T* __restrict__ un,
          const typename P::T* __restrict__ fa, const typename P::T* __restrict__ fb,
          const typename P::T* __restrict__ ga, const typename P::T* __restrict__ gb, typename P::T gval,
          Layout L, Star7Coeffs c, Split time_old, Split time_new,
          Split corr, const BorderTable* __restrict__ table, int zchunk, int* __restrict__ status)
{
    using T = typename P::T;
    using G = Tile<T, BY, NS, FS>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* st = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NS * G::STRIDE * G::ESZ);
    ring_init<NS>(bar);
    TileJob<T> J{&tm, &tmf, un, fa, fb, ga, gb, gval, L, time_old, time_new, corr, table};
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, L.nz);
    uint32_t base = 0;
    star7_tile<P, SRC, BORDER, BY, R, NS, FS>(J, c, blockIdx.x * BX, blockIdx.y * BY, z0, z1, st, bar, base, status);
}

// ---- host side ---------------------------------------------------------------

Star7Coeffs make_star7_coeffs(double c0, const double cp[3], double cf) {
    Star7Coeffs c;
    c.c0 = c0; c.cx = cp[0]; c.cy = cp[1]; c.cz = cp[2]; c.cf = cf;
    auto split3 = [](double v, float& h, float& l, float& ll) {
        h = (float)v;
        double r = v - (double)h;
        l = (float)r;
        ll = (float)(r - (double)l);
    };
    split3(c0, c.c0h, c.c0l, c.c0ll);
    split3(cp[0], c.cxh, c.cxl, c.cxll);
    split3(cp[1], c.cyh, c.cyl, c.cyll);
    split3(cp[2], c.czh, c.czl, c.czll);
    split3(cf, c.cfh, c.cfl, c.cfll);
    return c;
}

int star7_box_width(int precision) {
    return BX + 2 * (16 / (int)element_size(precision));
}

int star7_box_height(int tile) {
    return kTiles[tile].by + 2;
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

int star7_default_tile(const Layout& L) {
    // Four rows per thread once the grid has enough tiles to fill the GPU.
    const long long cols = (long long)L.nx * L.ny;
    return cols >= 256LL * 256LL ? 2 : 0;
}

// z-chunk length: 16 planes keep ~8 CTAs per SM streaming with two halo
// planes per chunk; shorter chunks give enough CTAs on small grids.
static int choose_zchunk(const Layout& L, int by) {
    const long long tiles = (long long)((L.nx + BX - 1) / BX) * ((L.ny + by - 1) / by);
    const long long want = (long long)num_sms() * 16;
    int zc = 16;
    while (zc > 4 && tiles * ((L.nz + zc - 1) / zc) < want) zc >>= 1;
    return zc;
}

// A double as the element type of a precision (host side).
static inline void to_elem(double d, double& out) { out = d; }
static inline void to_elem(double d, float& out) { out = (float)d; }
static inline void to_elem(double d, float2& out) {
    f2 p = split_double(d);
    out = make_float2(p.hi, p.lo);
}

template <class P, int SRC, int BORDER, int BY, int R, int NS0>
static cudaError_t launch_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    constexpr bool FS = SRC == SRC_A;  // a source without a time term is staged with the iterate
    constexpr int NS = ring_stages(NS0, FS);
    using G = Tile<T, BY, NS, FS>;
    const Layout& L = a.L;
    if (FS && a.tm_f == nullptr) return cudaErrorInvalidValue;
    auto kern = star7_tma<P, SRC, BORDER, BY, R, NS, FS>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
        // The ring lives in shared memory: ask for the largest carveout so
        // that occupancy is not capped by a small L1/shared split.
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             cudaSharedmemCarveoutMaxShared);
        attr = true;
    }
    T gval;
    to_elem(a.gconst, gval);
    const int zchunk = choose_zchunk(L, BY);
    dim3 block(BX, BY / R, 1);
    dim3 grid((L.nx + BX - 1) / BX, (L.ny + BY - 1) / BY, (L.nz + zchunk - 1) / zchunk);
    kern<<<grid, block, G::SMEM, stream>>>(*a.tm_uo, FS ? *a.tm_f : *a.tm_uo, (T*)a.un, (const T*)a.fa, (const T*)a.fb, (const T*)a.ga,
                                           (const T*)a.gb, gval, L,
                                           a.c, make_split(a.time_old), make_split(a.time_new),
                                           make_split(a.mirror_corr), a.table, zchunk, a.status);
    return cudaGetLastError();
}

template <class P, int SRC, int BORDER>
static cudaError_t launch_tile(const Star7Launch& a, cudaStream_t stream) {
    switch (a.tile) {
        case 0: return launch_typed<P, SRC, BORDER, kTiles[0].by, kTiles[0].r, kTiles[0].ns>(a, stream);
        case 1: return launch_typed<P, SRC, BORDER, kTiles[1].by, kTiles[1].r, kTiles[1].ns>(a, stream);
        case 2: return launch_typed<P, SRC, BORDER, kTiles[2].by, kTiles[2].r, kTiles[2].ns>(a, stream);
        case 3: return launch_typed<P, SRC, BORDER, kTiles[3].by, kTiles[3].r, kTiles[3].ns>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

template <class P, int BORDER>
static cudaError_t launch_src(const Star7Launch& a, cudaStream_t stream) {
    if (a.fa == nullptr || a.c.cf == 0.0) return launch_tile<P, SRC_NONE, BORDER>(a, stream);
    if (a.fb == nullptr) return launch_tile<P, SRC_A, BORDER>(a, stream);
    return launch_tile<P, SRC_AB, BORDER>(a, stream);
}

template <class P>
static cudaError_t launch_prec(const Star7Launch& a, cudaStream_t stream) {
    switch (a.border) {
        case SCAFES_BORDER_DIRICHLET: return launch_src<P, SCAFES_BORDER_DIRICHLET>(a, stream);
        case SCAFES_BORDER_MIRROR_POW2: return launch_src<P, SCAFES_BORDER_MIRROR_POW2>(a, stream);
        case SCAFES_BORDER_TABLE:
            if (a.table == nullptr) return cudaErrorInvalidValue;
            return launch_src<P, SCAFES_BORDER_TABLE>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_star7(const Star7Launch& a, cudaStream_t stream) {
    switch (a.precision) {
        case SCAFES_PREC_F64: return launch_prec<PolF64>(a, stream);
        case SCAFES_PREC_F32: return launch_prec<PolF32>(a, stream);
        case SCAFES_PREC_F32X2: return launch_prec<PolF32x2>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace scafes
