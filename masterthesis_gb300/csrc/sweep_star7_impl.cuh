// Sweep kernel template and its launch dispatch, included by one
// translation unit per element type (sweep_star7_f64.cu, _f32x2.cu, _f32.cu)
// so that the instantiations compile in parallel.
#pragma once

#include "star7_tb.cuh"
#include "star7_tile.cuh"

namespace scafes {

// Minimum resident CTAs per SM asked of the compiler: 8 for the one-row
// FP64 tile without a source and with a Dirichlet or mirror border, whose
// integer-pipe neighbour sums are latency-bound and gain more from 64
// resident warps (32 registers, 32-44 bytes spilled to L1: 113.9 against
// 110.6 GLUP/s at 512^3) than they lose to the spills.  The source and
// table-border variants would spill 92-228 bytes: no constraint for them
// or for any other tile.
template <class P, int R, int SRC, int BORDER>
constexpr int star7_min_ctas() {
    return (R == 1 && std::is_same<P, PolF64>::value && SRC == SRC_NONE &&
            (BORDER == SCAFES_BORDER_DIRICHLET || BORDER == SCAFES_BORDER_MIRROR_POW2))
               ? 8
               : 0;
}

template <class P, int SRC, int BORDER, int BY, int R, int NS, bool FS, bool ML>
__global__ void __launch_bounds__(BX * (BY / R), star7_min_ctas<P, R, SRC, BORDER>())
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
    // After a sweep gave up on a TMA load (status set), the results are
    // invalid until the host reads the status: later sweeps return at once
    // instead of each waiting out its own limit.
    if (__syncthreads_or(threadIdx.x == 0 && threadIdx.y == 0 && *(volatile int*)status != 0)) return;
    ring_init<NS>(bar);
    TileJob<T> J{&tm, &tmf, un, fa, fb, ga, gb, gval, L, time_old, time_new, corr, table};
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, L.nz);
    uint32_t base = 0;
    star7_tile<P, SRC, BORDER, BY, R, NS, FS, ML>(J, c, blockIdx.x * BX, blockIdx.y * BY, z0, z1, st, bar, base, status);
}

// Per-node border rules (FP64 and FP32 sweeps) leave the x-face nodes
// outside the y and z border rows to k_xface_node_rules: otherwise every
// warp of an x-face tile evaluates a rule for one or two lanes (FP64
// instructions that hold the narrow FP64 pipe; rule loads it waits for).
template <class P, int BORDER>
constexpr bool XFACE_PASS =
    (std::is_same<P, PolF64>::value || std::is_same<P, PolF32>::value) && BORDER == SCAFES_BORDER_NODES;

// The per-node rules of the nodes on the two x faces outside the y and z
// border rows (one border layer), from the old iterate: what node_rule
// computes for them, in the same order and arithmetic (FP64 rules for
// double fields, the FP32 copy of the rules for float fields; a neighbour
// outside the grid reads 0, as from the TMA halo).  One thread per
// (face, y, z).
template <typename T>
static __global__ void k_xface_node_rules(const T* __restrict__ uo, T* __restrict__ un,
                                          const scafes_border_node_rule* __restrict__ nodes, Layout L) {
    const long long rows = (long long)(L.ny - 2) * (L.nz - 2);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < 2 * rows;
         i += (long long)gridDim.x * blockDim.x) {
        const int side = (int)(i / rows);
        const long long r = i % rows;
        const int y = 1 + (int)(r % (L.ny - 2)), z = 1 + (int)(r / (L.ny - 2));
        const int x = side ? L.nx - 1 : 0;
        const long long o = L.idx(x, y, z);
        const T w = x > 0 ? uo[o - 1] : T(0), e = x < L.nx - 1 ? uo[o + 1] : T(0);
        if constexpr (std::is_same<T, float>::value) {
            const float* R = reinterpret_cast<const float*>(nodes) + 8 * border_node_index(L, x, y, z);
            float v = fmaf(R[0], uo[o], R[7]);
            v = fmaf(R[1], w, v);
            v = fmaf(R[2], e, v);
            v = fmaf(R[3], uo[o - L.pitch], v);
            v = fmaf(R[4], uo[o + L.pitch], v);
            v = fmaf(R[5], uo[o - L.plane], v);
            v = fmaf(R[6], uo[o + L.plane], v);
            un[o] = v;
        } else {
            const scafes_border_node_rule& R = nodes[border_node_index(L, x, y, z)];
            double v = fma(R.cu, uo[o], R.cst);
            v = fma(R.cn[0], w, v);
            v = fma(R.cn[1], e, v);
            v = fma(R.cn[2], uo[o - L.pitch], v);
            v = fma(R.cn[3], uo[o + L.pitch], v);
            v = fma(R.cn[4], uo[o - L.plane], v);
            v = fma(R.cn[5], uo[o + L.plane], v);
            un[o] = v;
        }
    }
}

// The variable-coefficient sweep: as star7_tma, with the coefficient fields
// C0 and CA staged by TMA with every plane (and F_A with them when the
// source is present), and the Dirichlet, table or per-node border.
// The variable-coefficient one-row FP64 tile asks for 6 CTAs per SM (40
// registers, up to 12 bytes spilled): 89.5 against 85.8 GLUP/s on the
// 512^3 tissue workload (5 CTAs: 85.8).
template <class P, int R>
constexpr int star7_vc_min_ctas() {
    return (R == 1 && std::is_same<P, PolF64>::value) ? 6 : 0;
}

template <class P, int SRC, int BORDER, int BY, int R, int NS>
__global__ void __launch_bounds__(BX * (BY / R), star7_vc_min_ctas<P, R>())
star7_vc_tma(const __grid_constant__ CUtensorMap tm, const __grid_constant__ CUtensorMap tmf,
             const __grid_constant__ CUtensorMap tmc0, const __grid_constant__ CUtensorMap tmca,
             typename P::T* __restrict__ un, const typename P::T* __restrict__ fa,
             const typename P::T* __restrict__ ga, typename P::T gval, Layout L, Star7Coeffs c, Split time_old,
             Split time_new, const BorderTable* __restrict__ table,
             const scafes_border_node_rule* __restrict__ nodes, int zchunk, int* __restrict__ status)
{
    using T = typename P::T;
    constexpr bool FS = SRC == SRC_A;
    using G = Tile<T, BY, NS, FS, true>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    T* st = reinterpret_cast<T*>(smem_raw);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + (size_t)NS * G::STRIDE * G::ESZ);
    if (__syncthreads_or(threadIdx.x == 0 && threadIdx.y == 0 && *(volatile int*)status != 0)) return;
    ring_init<NS>(bar);
    TileJob<T> J{&tm, &tmf, un, fa, nullptr, ga, nullptr, gval, L, time_old, time_new, Split{0.0, 0.f, 0.f}, table,
                 &tmc0, &tmca, nodes, XFACE_PASS<P, BORDER>};
    const int z0 = blockIdx.z * zchunk;
    const int z1 = min(z0 + zchunk, L.nz);
    uint32_t base = 0;
    star7_tile<P, SRC, BORDER, BY, R, NS, FS, false, true>(J, c, blockIdx.x * BX, blockIdx.y * BY, z0, z1, st,
                                                           bar, base, status);
}

// ---- host side ---------------------------------------------------------------

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

// z-chunk length: 16 planes keep ~8 CTAs per SM streaming with two halo
// planes per chunk; shorter chunks give enough CTAs on small grids.
static int choose_zchunk(const Layout& L, int by) {
    const long long tiles = (long long)((L.nx + BX - 1) / BX) * ((L.ny + by - 1) / by);
    const long long want = (long long)num_sms() * 16;
    int zc = 16;
    while (zc > 4 && tiles * ((L.nz + zc - 1) / zc) < want) zc >>= 1;
    while ((L.nz + zc - 1) / zc > 65535) zc <<= 1;  // grid.z limit
    return zc;
}

// A double as the element type of a precision (host side).
static inline void to_elem(double d, double& out) { out = d; }
static inline void to_elem(double d, float& out) { out = (float)d; }
static inline void to_elem(double d, float2& out) {
    f2 p = split_double(d);
    out = make_float2(p.hi, p.lo);
}

template <class P, int SRC, int BORDER, int BY, int R, int NS0, bool ML>
static cudaError_t launch_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    constexpr bool FS = SRC == SRC_A;  // a source without a time term is staged with the iterate
    constexpr int NS = ring_stages(NS0, FS);
    using G = Tile<T, BY, NS, FS>;
    const Layout& L = a.L;
    if (FS && a.tm_f == nullptr) return cudaErrorInvalidValue;
    auto kern = star7_tma<P, SRC, BORDER, BY, R, NS, FS, ML>;
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
    if (a.L.nl != 1) {
        // More than one border layer (rare; not a bandwidth case): one tile
        // variant reads the layer count from the layout.  Its TMA boxes must
        // be the ones the descriptors were encoded for, so any other tile is
        // refused here rather than launched.
        constexpr int T1 = STAR7_MULTI_LAYER_TILE;
        if (BORDER == SCAFES_BORDER_MIRROR_POW2 || a.tile != T1) return cudaErrorInvalidValue;
        return launch_typed<P, SRC, BORDER, kTiles[T1].by, kTiles[T1].r, kTiles[T1].ns, true>(a, stream);
    }
    switch (a.tile) {
        case 0: return launch_typed<P, SRC, BORDER, kTiles[0].by, kTiles[0].r, kTiles[0].ns, false>(a, stream);
        case 1: return launch_typed<P, SRC, BORDER, kTiles[1].by, kTiles[1].r, kTiles[1].ns, false>(a, stream);
        case 2: return launch_typed<P, SRC, BORDER, kTiles[2].by, kTiles[2].r, kTiles[2].ns, false>(a, stream);
        case 3: return launch_typed<P, SRC, BORDER, kTiles[3].by, kTiles[3].r, kTiles[3].ns, false>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

// Stages of the variable-coefficient ring: each stage holds up to three
// extra boxes, so four stages keep shared memory within a few CTAs per SM.
constexpr int kVcStages = 4;

template <class P, int SRC, int BORDER, int BY, int R>
static cudaError_t launch_vc_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    constexpr bool FS = SRC == SRC_A;
    constexpr int NS = kVcStages;
    using G = Tile<T, BY, NS, FS, true>;
    const Layout& L = a.L;
    if ((FS && a.tm_f == nullptr) || a.tm_c0 == nullptr || a.tm_ca == nullptr) return cudaErrorInvalidValue;
    auto kern = star7_vc_tma<P, SRC, BORDER, BY, R, NS>;
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM);
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
        attr = true;
    }
    T gval;
    to_elem(a.gconst, gval);
    const int zchunk = choose_zchunk(L, BY);
    dim3 block(BX, BY / R, 1);
    dim3 grid((L.nx + BX - 1) / BX, (L.ny + BY - 1) / BY, (L.nz + zchunk - 1) / zchunk);
    kern<<<grid, block, G::SMEM, stream>>>(*a.tm_uo, FS ? *a.tm_f : *a.tm_uo, *a.tm_c0, *a.tm_ca, (T*)a.un,
                                           (const T*)a.fa, (const T*)a.ga, gval, L, a.c, make_split(a.time_old),
                                           make_split(a.time_new), a.table, a.nodes, zchunk, a.status);
    if constexpr (XFACE_PASS<P, BORDER>) {
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        const long long work = 2LL * (L.ny - 2) * (L.nz - 2);
        const int blocks = (int)std::min<long long>((work + 255) / 256, (long long)num_sms() * 8);
        k_xface_node_rules<T><<<blocks, 256, 0, stream>>>((const T*)a.uo, (T*)a.un, a.nodes, L);
    }
    return cudaGetLastError();
}

template <class P, int SRC, int BORDER>
static cudaError_t launch_vc_tile(const Star7Launch& a, cudaStream_t stream) {
    switch (a.tile) {
        case 0: return launch_vc_typed<P, SRC, BORDER, kTiles[0].by, kTiles[0].r>(a, stream);
        case 1: return launch_vc_typed<P, SRC, BORDER, kTiles[1].by, kTiles[1].r>(a, stream);
        case 2: return launch_vc_typed<P, SRC, BORDER, kTiles[2].by, kTiles[2].r>(a, stream);
        case 3: return launch_vc_typed<P, SRC, BORDER, kTiles[3].by, kTiles[3].r>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

template <class P, int BORDER>
static cudaError_t launch_vc_src(const Star7Launch& a, cudaStream_t stream) {
    if (a.fb != nullptr) return cudaErrorInvalidValue;  // static source only
    if (a.fa == nullptr || a.c.cf == 0.0) return launch_vc_tile<P, SRC_NONE, BORDER>(a, stream);
    return launch_vc_tile<P, SRC_A, BORDER>(a, stream);
}

// The variable-coefficient family: FP64 and FP32, one border layer.
template <class P>
static cudaError_t launch_vc(const Star7Launch& a, cudaStream_t stream) {
    if constexpr (std::is_same<P, PolF32x2>::value) {
        return cudaErrorInvalidValue;
    } else {
        if (a.L.nl != 1) return cudaErrorInvalidValue;
        switch (a.border) {
            case SCAFES_BORDER_DIRICHLET: return launch_vc_src<P, SCAFES_BORDER_DIRICHLET>(a, stream);
            case SCAFES_BORDER_TABLE:
                if (a.table == nullptr) return cudaErrorInvalidValue;
                return launch_vc_src<P, SCAFES_BORDER_TABLE>(a, stream);
            case SCAFES_BORDER_NODES:
                if (a.nodes == nullptr) return cudaErrorInvalidValue;
                return launch_vc_src<P, SCAFES_BORDER_NODES>(a, stream);
            default: return cudaErrorInvalidValue;
        }
    }
}

template <class P, int BORDER>
static cudaError_t launch_src(const Star7Launch& a, cudaStream_t stream) {
    if (a.fa == nullptr || a.c.cf == 0.0) return launch_tile<P, SRC_NONE, BORDER>(a, stream);
    if (a.fb == nullptr) return launch_tile<P, SRC_A, BORDER>(a, stream);
    return launch_tile<P, SRC_AB, BORDER>(a, stream);
}

// z-planes per CTA of a depth-2 pass: long chunks (each recomputes two
// intermediate planes and reads four extra input planes), shorter ones
// while the grid has few column tiles.
static int tb_zchunk(const Layout& L) {
    const long long tiles = (long long)((L.nx + TB_X - 1) / TB_X) * ((L.ny + TB_Y - 1) / TB_Y);
    int zc = 64;
    while (zc > 8 && tiles * ((L.nz + zc - 1) / zc) < (long long)num_sms() * 8) zc >>= 1;
    while ((L.nz + zc - 1) / zc > 65535) zc <<= 1;  // grid.z limit
    return zc;
}

// Shared-memory attributes of the depth-2 kernel (once; also callable
// before a stream capture that launches it).
template <class P, bool HAS_F>
static cudaError_t tb_attributes() {
    static cudaError_t done = cudaErrorNotReady;
    if (done == cudaErrorNotReady) {
        auto kern = star7_tb2<P, HAS_F>;
        constexpr size_t SMEM = tb_smem(sizeof(typename P::T));
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        done = e;
    }
    return done;
}

template <class P>
cudaError_t prepare_tb_prec() {
    const cudaError_t e = tb_attributes<P, false>();
    return e != cudaSuccess ? e : tb_attributes<P, true>();
}

template <class P, bool HAS_F>
static cudaError_t launch_tb_typed(const Star7Launch& a, cudaStream_t stream) {
    using T = typename P::T;
    auto kern = star7_tb2<P, HAS_F>;
    constexpr size_t SMEM = tb_smem(sizeof(T));
    if (const cudaError_t e = tb_attributes<P, HAS_F>()) return e;
    T gval;
    to_elem(a.gconst, gval);
    const Layout& L = a.L;
    const int zc = tb_zchunk(L);
    const dim3 grid((L.nx + TB_X - 1) / TB_X, (L.ny + TB_Y - 1) / TB_Y, (L.nz + zc - 1) / zc);
    kern<<<grid, dim3(TB_X, TB_TY), SMEM, stream>>>(*a.tm_tb, (T*)a.un, (const T*)a.fa, (const T*)a.ga,
                                                     (const T*)a.gb, gval, L, a.c, make_split(a.time_new),
                                                     make_split(a.time_new2), zc, a.status);
    return cudaGetLastError();
}

template <class P>
cudaError_t launch_tb_prec(const Star7Launch& a, cudaStream_t stream) {
    if (!star7_tb_eligible(a) || a.tm_tb == nullptr) return cudaErrorInvalidValue;
    if (a.fa == nullptr || a.c.cf == 0.0) return launch_tb_typed<P, false>(a, stream);
    return launch_tb_typed<P, true>(a, stream);
}

template <class P>
cudaError_t launch_prec(const Star7Launch& a, cudaStream_t stream) {
    if (a.vc) return launch_vc<P>(a, stream);
    switch (a.border) {
        case SCAFES_BORDER_DIRICHLET: return launch_src<P, SCAFES_BORDER_DIRICHLET>(a, stream);
        case SCAFES_BORDER_MIRROR_POW2: return launch_src<P, SCAFES_BORDER_MIRROR_POW2>(a, stream);
        case SCAFES_BORDER_TABLE:
            if (a.table == nullptr) return cudaErrorInvalidValue;
            return launch_src<P, SCAFES_BORDER_TABLE>(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace scafes
