// Plain 7-point sweep: one launch advances the whole grid by one time step.
//
// Replaces the per-node loop of ScaFES's evalTypeTwoAt
// (src/ScaFES_Problem.hpp:5399-5476) for the heat-type callbacks
// (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218,
//  tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168) and
// their Dirichlet border (.../Dirichlet/Dirichlet.hpp:125-131), and the copy
// old->new that precedes it (:5078-5082): every node is written each step.
//
// Mapping: a CTA owns a 32 x BY column tile and marches it through a chunk
// of z-planes.  One elected thread streams the tile's planes (with a one-
// node halo in x and y) from HBM into an NSTAGE-deep ring of shared-memory
// stages with 3D TMA loads, each stage completing on its own mbarrier, so
// that several planes per CTA are in flight.  Each thread owns R consecutive
// rows of one column: it keeps u(z-1), u(z), u(z+1) of those rows in
// registers (the z-marching queue), takes the y-neighbours inside its rows
// from registers and the x-neighbours (and the two outer y-neighbours) from
// the staged plane.  Blocking R rows per thread amortises the per-plane
// wait, barrier and index work over R node updates.  Out-of-domain halo
// cells are zero-filled by the TMA unit.  Stores are row-contiguous per warp.
#include "star7_policies.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

namespace scafes {

constexpr int BX = 32;
constexpr int NSTAGE = 8;  // power of two: stage/phase indices are shifts

template <class T, int BY>
struct Tile {
    static constexpr int ESZ = (int)sizeof(T);
    static constexpr int LP = 16 / ESZ;          // left halo padded to 16 bytes
    static constexpr int W = BX + 2 * LP;        // box width (elements)
    static constexpr int H = BY + 2;             // box height (rows)
    static constexpr uint32_t TX_BYTES = W * H * ESZ;
    static constexpr int STRIDE = ((W * H * ESZ + 127) / 128) * 128 / ESZ;  // elements per stage
    static constexpr size_t SMEM = (size_t)NSTAGE * STRIDE * ESZ + NSTAGE * sizeof(uint64_t);
};

// Tile variants {BY, R}: CTA tile 32 x BY, R rows per thread.
struct TileShape { int by, r; };
constexpr TileShape kTiles[STAR7_NUM_TILES] = {{8, 1}, {16, 2}, {32, 4}, {16, 4}};

template <class P, bool HAS_F, int BORDER, int BY, int R>
__global__ void __launch_bounds__(BX * (BY / R))
star7_tma(const __grid_constant__ CUtensorMap tm, typename P::T* __restrict__ un,
          const typename P::T* __restrict__ fa, const typename P::T* __restrict__ fb,
          const double* __restrict__ ga, const double* __restrict__ gb,
          Layout L, Star7Coeffs c, double time_old, double time_new,
          double corr, int zchunk, int* __restrict__ status)
{
    using T = typename P::T;
    using G = Tile<T, BY>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* st = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NSTAGE * G::STRIDE * G::ESZ);

    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * BX + tx;
    const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
    const int x = x0 + tx;
    const int yb = y0 + ty * R;  // first row of this thread
    const int rb = ty * R + 1;   // its row inside a stage
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, L.nz);
    const int np = z1 - z0 + 2;  // planes z0-1 .. z1 (index p <-> z = z0 - 1 + p)

    if (tid == 0) {
        for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (tid == 0) {
        const int pre = np < NSTAGE ? np : NSTAGE;
        for (int p = 0; p < pre; ++p) {
            mbar_arrive_expect_tx(&bar[p], G::TX_BYTES);
            tma_load_3d(st + p * G::STRIDE, &tm, x0 - G::LP, y0 - 1, z0 - 1 + p, &bar[p]);
        }
    }

    const bool xin = x < L.nx;
    const bool xb = (x == 0 || x == L.nx - 1);
    const bool has_fb = (fb != nullptr);
    const bool has_gb = (gb != nullptr);
    const int cc = G::LP + tx;  // this thread's column inside a stage row

    bool ok = bounded_wait(&bar[0], 0);
    ok = bounded_wait(&bar[1], 0) && ok;
    T below[R], cur[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        below[k] = st[0 * G::STRIDE + (rb + k) * G::W + cc];
        cur[k] = st[1 * G::STRIDE + (rb + k) * G::W + cc];
    }
    int p = 1;
    for (int z = z0; z < z1; ++z, ++p) {
        const int sa = (p + 1) & (NSTAGE - 1);
        ok = bounded_wait(&bar[sa], ((p + 1) / NSTAGE) & 1) && ok;
        const T* pl = st + (p & (NSTAGE - 1)) * G::STRIDE + cc;
        const T* pa = st + sa * G::STRIDE + cc;
        T above[R];
#pragma unroll
        for (int k = 0; k < R; ++k) above[k] = pa[(rb + k) * G::W];
        if (xin && ok) {
            const bool zb = (z == 0 || z == L.nz - 1);
            const long long zoff = (long long)z * L.plane + x;
            const T ym = pl[(rb - 1) * G::W];
            const T yp = pl[(rb + R) * G::W];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int y = yb + k;
                if (y < L.ny) {
                    const long long off = zoff + (long long)y * L.pitch;
                    const T s = (k == 0) ? ym : cur[k - 1];
                    const T n = (k == R - 1) ? yp : cur[k + 1];
                    const T w = pl[(rb + k) * G::W - 1];
                    const T e = pl[(rb + k) * G::W + 1];
                    const bool border = xb || zb || y == 0 || y == L.ny - 1;
                    T v;
                    if (!border) {
                        T f = P::zero();
                        if (HAS_F) f = P::src(fa[off], has_fb ? fb[off] : P::zero(), time_old, has_fb);
                        v = P::template star<HAS_F>(c, cur[k], w, e, s, n, below[k], above[k], f);
                    } else if (BORDER == SCAFES_BORDER_DIRICHLET) {
                        double g = ga ? ga[off] : 0.0;
                        if (has_gb) g += time_new * gb[off];
                        v = P::from_double(g);
                    } else {
                        // Mirror border: the last face (in direction order
                        // x-, x+, y-, y+, z-, z+) the node lies on decides.
                        T opp;
                        double cs;
                        if (z == L.nz - 1)      { opp = below[k]; cs = -corr; }
                        else if (z == 0)        { opp = above[k]; cs = corr; }
                        else if (y == L.ny - 1) { opp = s; cs = -corr; }
                        else if (y == 0)        { opp = n; cs = corr; }
                        else if (x == L.nx - 1) { opp = w; cs = -corr; }
                        else                    { opp = e; cs = corr; }
                        v = P::mirror(cur[k], opp, cs);
                    }
                    un[off] = v;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < R; ++k) {
            below[k] = cur[k];
            cur[k] = above[k];
        }
        // Everyone is done with plane p-1: its stage takes plane p-1+NSTAGE.
        if (!__syncthreads_and(ok)) break;
        if (tid == 0) {
            const int pn = p - 1 + NSTAGE;
            if (pn < np) {
                const int s = pn & (NSTAGE - 1);
                fence_proxy_async_smem();
                mbar_arrive_expect_tx(&bar[s], G::TX_BYTES);
                tma_load_3d(st + s * G::STRIDE, &tm, x0 - G::LP, y0 - 1, z0 - 1 + pn, &bar[s]);
            }
        }
    }
    if (!__syncthreads_and(ok) && tid == 0) {
        // A stage never completed: report, drain what was issued, return.
        atomicExch(status, SCAFES_ERR_TIMEOUT);
        for (int q = (p > 0 ? p - 1 : 0); q < np && q < p - 1 + NSTAGE; ++q)
            bounded_wait(&bar[q & (NSTAGE - 1)], (q / NSTAGE) & 1, kWaitLimitNs / 8);
    }
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

template <class P, bool HAS_F, int BORDER, int BY, int R>
static cudaError_t launch_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    using G = Tile<T, BY>;
    const Layout& L = a.L;
    auto kern = star7_tma<P, HAS_F, BORDER, BY, R>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
        attr = true;
    }
    const int zchunk = choose_zchunk(L, BY);
    dim3 block(BX, BY / R, 1);
    dim3 grid((L.nx + BX - 1) / BX, (L.ny + BY - 1) / BY, (L.nz + zchunk - 1) / zchunk);
    kern<<<grid, block, G::SMEM, stream>>>(*a.tm_uo, (T*)a.un, (const T*)a.fa, (const T*)a.fb, a.ga, a.gb, L,
                                           a.c, a.time_old, a.time_new, a.mirror_corr, zchunk, a.status);
    return cudaGetLastError();
}

template <class P, bool HAS_F, int BORDER>
static cudaError_t launch_tile(const Star7Launch& a, cudaStream_t stream) {
    switch (a.tile) {
        case 0: return launch_typed<P, HAS_F, BORDER, kTiles[0].by, kTiles[0].r>(a, stream);
        case 1: return launch_typed<P, HAS_F, BORDER, kTiles[1].by, kTiles[1].r>(a, stream);
        case 2: return launch_typed<P, HAS_F, BORDER, kTiles[2].by, kTiles[2].r>(a, stream);
        case 3: return launch_typed<P, HAS_F, BORDER, kTiles[3].by, kTiles[3].r>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

template <class P>
static cudaError_t launch_prec(const Star7Launch& a, cudaStream_t stream) {
    const bool has_f = (a.fa != nullptr) && (a.c.cf != 0.0);
    if (a.border == SCAFES_BORDER_DIRICHLET) {
        return has_f ? launch_tile<P, true, SCAFES_BORDER_DIRICHLET>(a, stream)
                     : launch_tile<P, false, SCAFES_BORDER_DIRICHLET>(a, stream);
    }
    return has_f ? launch_tile<P, true, SCAFES_BORDER_MIRROR_POW2>(a, stream)
                 : launch_tile<P, false, SCAFES_BORDER_MIRROR_POW2>(a, stream);
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
