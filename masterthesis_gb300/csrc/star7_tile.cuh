// One CTA tile of the 7-point sweep: a 32 x BY column tile marched through
// the z-planes [z0, z1), fed by a ring of TMA-loaded shared-memory stages.
// Shared by the plain sweep (one tile per CTA) and the batched ensemble
// (a persistent CTA works through many tiles of many instances).
//
// Mapping: one elected thread streams the tile's planes (with a one-node
// halo in x and y, x padded to 16 bytes) into an NS-deep ring of
// stages with 3D TMA loads, each stage completing on its own mbarrier.
// Each thread owns R consecutive rows of one column and keeps u(z-1),
// u(z), u(z+1) of them in registers (the z-marching queue); y-neighbours
// inside its rows come from registers, x-neighbours and the two outer
// y-neighbours from the staged plane.  Out-of-domain halo cells are
// zero-filled by the TMA unit.  Stores are row-contiguous per warp.
#pragma once

#include <type_traits>

#include "star7_policies.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

namespace scafes {

// NS: stages of the shared-memory ring, a power of two (stage and phase
// indices are shifts).  Fewer stages leave room for more CTAs per SM.
// FS: each stage also holds the source F_A of its plane (a 32 x BY box
// without halo), streamed by TMA with the iterate instead of read per node.
// VC: each stage also holds the coefficient fields C0 and CA of its plane
// (two more 32 x BY boxes), for the variable-coefficient update.
template <class T, int BY, int NS, bool FS = false, bool VC = false>
struct Tile {
    static constexpr int ESZ = (int)sizeof(T);
    static constexpr int LP = 16 / ESZ;          // left halo padded to 16 bytes
    static constexpr int W = BX + 2 * LP;        // box width (elements)
    static constexpr int H = BY + 2;             // box height (rows)
    static constexpr uint32_t TX_BYTES = W * H * ESZ;
    static constexpr int USTRIDE = ((W * H * ESZ + 127) / 128) * 128 / ESZ;  // iterate box, elements
    static constexpr int XSTRIDE = ((BX * BY * ESZ + 127) / 128) * 128 / ESZ;  // one extra box, elements
    static constexpr int NXB = (FS ? 1 : 0) + (VC ? 2 : 0);  // extra boxes per stage
    static constexpr uint32_t X_BYTES = NXB * BX * BY * ESZ;
    static constexpr int C0OFF = USTRIDE + (FS ? XSTRIDE : 0);  // C0 box inside a stage
    static constexpr int CAOFF = C0OFF + XSTRIDE;                // CA box
    static constexpr int STRIDE = USTRIDE + NXB * XSTRIDE;
    static constexpr size_t SMEM = (size_t)NS * STRIDE * ESZ + NS * sizeof(uint64_t);
};

// Ring depth of a kernel: tiles that also stage F_A use 4 stages (their
// stages are larger; 4 keep 2-3 planes in flight).
constexpr int ring_stages(int ns, bool fs) { return fs ? 4 : ns; }

// Tile variants {BY, R, NS}: CTA tile 32 x BY, R rows per thread, NS ring
// stages.
struct TileShape { int by, r, ns; };
constexpr TileShape kTiles[STAR7_NUM_TILES] = {{8, 1, 8}, {16, 2, 8}, {32, 4, 8}, {16, 4, 4}};

// Everything one tile needs besides its position.
template <class T>
struct TileJob {
    const CUtensorMap* tm;   // TMA descriptor of the old iterate
    const CUtensorMap* tmf;  // TMA descriptor of F_A (box 32 x BY), staged tiles only
    T* un;                   // new iterate
    const T* fa;             // source F_A or null
    const T* fb;             // source F_B or null
    const T* ga;             // border value G_A or null (then gval)
    const T* gb;             // border value G_B or null
    T gval;                  // border value when ga is null
    Layout L;
    Split time_old, time_new, corr;  // time(t), time(t+1), mirror correction
    const BorderTable* table;  // border rules (SCAFES_BORDER_TABLE)
    const CUtensorMap* tmc0 = nullptr;  // TMA descriptors of C0, CA (box 32 x BY), VC tiles only
    const CUtensorMap* tmca = nullptr;
    const scafes_border_node_rule* nodes = nullptr;  // per-node rules (SCAFES_BORDER_NODES)
    // Per-node rules: the nodes on an x face outside the y and z border
    // rows are left to a separate pass (k_xface_node_rules), so that no
    // warp of an x-face tile evaluates a rule for one lane.
    bool xface_pass = false;
};

// The rule of one border node of a SCAFES_BORDER_NODES problem:
// u_new = cu*u + sum_d cn[d]*u_d + cst, in FP64, except for the FP32 sweep,
// whose rules the host stores as 8 floats per node (cu, cn[0..5], cst) and
// which evaluates them in FP32: on an x-face tile every warp calls this for
// one or two lanes, and a warp's FP64 instructions (and FP32<->FP64
// conversions) hold GB300's narrow FP64 pipe whatever the active lanes.
template <class P>
__device__ __noinline__ typename P::T node_rule(const TileJob<typename P::T>& J, int x, int y, int z,
                                                 typename P::T u, typename P::T w, typename P::T e,
                                                 typename P::T s, typename P::T n, typename P::T b,
                                                 typename P::T t) {
    if constexpr (std::is_same<P, PolF32>::value) {
        const float* Rf = reinterpret_cast<const float*>(J.nodes) + 8 * border_node_index(J.L, x, y, z);
        float v = fmaf(Rf[0], u, Rf[7]);
        v = fmaf(Rf[1], w, v);
        v = fmaf(Rf[2], e, v);
        v = fmaf(Rf[3], s, v);
        v = fmaf(Rf[4], n, v);
        v = fmaf(Rf[5], b, v);
        v = fmaf(Rf[6], t, v);
        return v;
    }
    const scafes_border_node_rule& R = J.nodes[border_node_index(J.L, x, y, z)];
    double v = fma(R.cu, P::to_double(u), R.cst);
    v = fma(R.cn[0], P::to_double(w), v);
    v = fma(R.cn[1], P::to_double(e), v);
    v = fma(R.cn[2], P::to_double(s), v);
    v = fma(R.cn[3], P::to_double(n), v);
    v = fma(R.cn[4], P::to_double(b), v);
    v = fma(R.cn[5], P::to_double(t), v);
    return P::from_double(v);
}

// The table rule of a border node, in FP64 whatever the element type (border
// nodes are a thin layer; the rule needs the reference's rounding, not
// speed).  mask: faces the node lies on; off: its element offset.
template <class P, bool HAS_F, bool HAS_FB>
__device__ __noinline__ typename P::T table_rule(const TileJob<typename P::T>& J, int mask, long long off,
                                                  typename P::T u, typename P::T w, typename P::T e,
                                                  typename P::T s, typename P::T n, typename P::T b,
                                                  typename P::T t) {
    const BorderTable& B = *J.table;
    const scafes_border_form& R = B.rule[mask];
    const double ud = P::to_double(u);
    double v = R.cu * ud;
    v = fma(R.cn[0], P::to_double(w), v);
    v = fma(R.cn[1], P::to_double(e), v);
    v = fma(R.cn[2], P::to_double(s), v);
    v = fma(R.cn[3], P::to_double(n), v);
    v = fma(R.cn[4], P::to_double(b), v);
    v = fma(R.cn[5], P::to_double(t), v);
    if (HAS_F) {
        double f = P::to_double(J.fa[off]);
        if (HAS_FB) f = fma(J.time_old.d, P::to_double(J.fb[off]), f);
        v = fma(R.cf, f, v);
    }
    // G(t) = G_A + s (G_B + s (G_C + s (G_D + s G_E))), s = (time - tc) * rate;
    // with the default basis and no higher orders this is G_A + time * G_B.
    const double g0 = J.ga ? P::to_double(J.ga[off]) : P::to_double(J.gval);
    const double g1 = J.gb ? P::to_double(J.gb[off]) : 0.0;
    double gh[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) gh[k] = B.g_hi[k] ? B.g_hi[k][off] : 0.0;
    auto G = [&](double time) {
        const double s = __dmul_rn(__dsub_rn(time, B.t_center), B.t_rate);
        double g = fma(gh[2], s, gh[1]);
        g = fma(g, s, gh[0]);
        g = fma(g, s, g1);
        return fma(g, s, g0);
    };
    v = fma(R.cg_old, G(J.time_old.d), v);
    v = fma(R.cg_new, G(J.time_new.d), v);
    if (R.cu4 != 0.0) {
        const double u2 = ud * ud;
        v = fma(R.cu4, u2 * u2, v);
    }
    return P::from_double(v);
}

// Initialises the ring's mbarriers (thread 0) -- once per CTA.
template <int NS>
__device__ __forceinline__ void ring_init(uint64_t* bar) {
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
}

// Source term of the update, fixed at compile time so that no predicated
// arithmetic of an absent term is issued: none, F_A, or F_A + time * F_B.
enum : int { SRC_NONE = 0, SRC_A = 1, SRC_AB = 2 };

// Processes planes [z0, z1) of the tile at (x0, y0).  `base` counts the
// planes this CTA has streamed through the ring so far (it fixes the stage
// and phase of every plane); it is advanced by the planes this tile used.
// Returns false (and records SCAFES_ERR_TIMEOUT) when a stage never
// arrived; the caller must then stop.
template <class P, int SRC, int BORDER, int BY, int R, int NS, bool FS, bool ML = false, bool VC = false>
__device__ __forceinline__ bool star7_tile(const TileJob<typename P::T>& J, const Star7Coeffs& c,
                                           int x0, int y0, int z0, int z1,
                                           typename P::T* st, uint64_t* bar, uint32_t& base,
                                           int* status) {
    using T = typename P::T;
    using G = Tile<T, BY, NS, FS, VC>;
    constexpr bool HAS_F = SRC != SRC_NONE;
    constexpr bool has_fb = SRC == SRC_AB;
    static_assert(!FS || SRC == SRC_A, "only F_A is staged");
    static_assert(!VC || SRC != SRC_AB, "the variable-coefficient update takes a static source");
    static_assert(BORDER != SCAFES_BORDER_NODES || VC, "per-node border rules come with variable coefficients");
    const Layout& L = J.L;
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * BX + tx;
    const int x = x0 + tx;
    const int yb = y0 + ty * R;  // first row of this thread
    const int rb = ty * R + 1;   // its row inside a stage
    const int np = z1 - z0 + 2;  // planes z0-1 .. z1 (index p <-> z = z0 - 1 + p)
    const uint32_t b0 = base;

    // Streams plane q (z = z0 - 1 + q) into its stage; the planes that are
    // computed (1 <= q <= np - 2) bring their F_A box along.
    auto issue = [&](int q) {
        const uint32_t s = (b0 + (uint32_t)q) & (NS - 1);
        const bool wx = G::NXB > 0 && q >= 1 && q <= np - 2;
        mbar_arrive_expect_tx(&bar[s], G::TX_BYTES + (wx ? G::X_BYTES : 0u));
        tma_load_3d(st + s * G::STRIDE, J.tm, x0 - G::LP, y0 - 1, z0 - 1 + q, &bar[s]);
        if (wx && FS) tma_load_3d(st + s * G::STRIDE + G::USTRIDE, J.tmf, x0, y0, z0 - 1 + q, &bar[s]);
        if (wx && VC) {
            tma_load_3d(st + s * G::STRIDE + G::C0OFF, J.tmc0, x0, y0, z0 - 1 + q, &bar[s]);
            tma_load_3d(st + s * G::STRIDE + G::CAOFF, J.tmca, x0, y0, z0 - 1 + q, &bar[s]);
        }
    };
    if (tid == 0) {
        const int pre = np < NS ? np : NS;
        fence_proxy_async_smem();
        for (int p = 0; p < pre; ++p) issue(p);
    }

    const bool xin = x < L.nx;
    // Border nodes: within nl nodes of a face (src/ScaFES_Problem.hpp:
    // 3952-3971).  ML kernels read nl from the layout; the others are built
    // for one layer, the reference's default, which keeps the tests out of
    // the registers of the hot loop.
    const int nl = ML ? L.nl : 1;
    const bool xb = (x < nl || x > L.nx - 1 - nl);
    const bool has_gb = (J.gb != nullptr);
    // The whole 32 x BY tile holds inner columns: no per-node border tests.
    const bool tile_inner = x0 >= nl && x0 + BX <= L.nx - nl && y0 >= nl && y0 + BY <= L.ny - nl;
    const int cc = G::LP + tx;  // this thread's column inside a stage row
    auto slot = [&](int p) { return (b0 + (uint32_t)p) & (NS - 1); };
    auto phase = [&](int p) { return ((b0 + (uint32_t)p) / NS) & 1; };

    bool ok = bounded_wait(&bar[slot(0)], phase(0));
    ok = bounded_wait(&bar[slot(1)], phase(1)) && ok;
    // z-marching queue: three register blocks whose roles (below, current,
    // above) rotate from plane to plane, so no values are moved.
    T qa[R], qb[R], qc[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        qa[k] = st[slot(0) * G::STRIDE + (rb + k) * G::W + cc];
        qb[k] = st[slot(1) * G::STRIDE + (rb + k) * G::W + cc];
    }
    int p = 1;  // plane index of the current z (plane p holds z = z0 - 1 + p)
    int z = z0;

    // One z-plane: `below`, `cur` hold planes p-1, p; `above` receives p+1.
    // Returns false when a stage did not arrive in any thread of the CTA.
    auto plane = [&](const T (&below)[R], const T (&cur)[R], T (&above)[R]) -> bool {
        const uint32_t sa = slot(p + 1);
        ok = bounded_wait(&bar[sa], phase(p + 1)) && ok;
        const T* pl = st + slot(p) * G::STRIDE + cc;
        const T* pa = st + sa * G::STRIDE + cc;
#pragma unroll
        for (int k = 0; k < R; ++k) above[k] = pa[(rb + k) * G::W];
        const bool zb = (z < nl || z > L.nz - 1 - nl);
        const T ym = pl[(rb - 1) * G::W];
        const T yp = pl[(rb + R) * G::W];
        // A plane that is not a z-border plane.  Every node takes the star;
        // on a tile that touches an x or y face the border nodes then take
        // the border rule instead (a select, not a branch around the star:
        // the y test is uniform per warp, the x test hits one or two lanes).
        auto rows = [&](auto all_inner) {
            constexpr bool INNER = decltype(all_inner)::value;
            const long long o0 = (long long)z * L.plane + (long long)yb * L.pitch + x;
            T w[R], e[R], f[R], v[R];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const long long off = o0 + (long long)k * L.pitch;
                const bool live = INNER || (xin && yb + k < L.ny);
                w[k] = pl[(rb + k) * G::W - 1];
                e[k] = pl[(rb + k) * G::W + 1];
                f[k] = P::zero();
                if (FS)
                    f[k] = st[slot(p) * G::STRIDE + G::USTRIDE + (ty * R + k) * BX + tx];
                else if (HAS_F && live)
                    f[k] = P::src(J.fa[off], has_fb ? J.fb[off] : P::zero(), J.time_old, has_fb);
            }
            // Rows whose result the border rule replaces (or that are not
            // stored) set their bit in `skip`.
            unsigned skip = 0u;
            if constexpr (!INNER) {
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int y = yb + k;
                    if (!xin || y >= L.ny || xb || y < nl || y > L.ny - 1 - nl) skip |= 1u << k;
                }
            }
            if constexpr (VC) {
                const T* c0b = st + slot(p) * G::STRIDE + G::C0OFF + ty * R * BX + tx;
                const T* cab = st + slot(p) * G::STRIDE + G::CAOFF + ty * R * BX + tx;
                P::template star_vc_rows<HAS_F, R>(c, below, cur, above, ym, yp, w, e, f, c0b, cab, BX, v, skip);
            } else {
                P::template star_rows<HAS_F, R>(c, below, cur, above, ym, yp, w, e, f, v, skip);
            }
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const long long off = o0 + (long long)k * L.pitch;
                const int y = yb + k;
                bool live = INNER || (xin && y < L.ny);
                const bool ybord = y < nl || y > L.ny - 1 - nl;
                if (BORDER == SCAFES_BORDER_NODES && !INNER && J.xface_pass && xb && !ybord)
                    live = false;  // written by the x-face pass
                if (!INNER && live && (xb || ybord)) {
                    const T s = (k == 0) ? ym : cur[k - 1];
                    const T n = (k == R - 1) ? yp : cur[k + 1];
                    if (BORDER == SCAFES_BORDER_NODES) {
                        v[k] = node_rule<P>(J, x, y, z, cur[k], w[k], e[k], s, n, below[k], above[k]);
                    } else if (BORDER == SCAFES_BORDER_TABLE) {
                        const int mask = (x == 0) | ((x == L.nx - 1) << 1) | ((y == 0) << 2) |
                                         ((y == L.ny - 1) << 3);
                        v[k] = table_rule<P, HAS_F, has_fb>(J, mask, off, cur[k], w[k], e[k], s, n, below[k],
                                                            above[k]);
                    } else if (BORDER == SCAFES_BORDER_DIRICHLET) {
                        v[k] = J.ga ? J.ga[off] : J.gval;
                        if (has_gb) v[k] = P::src(v[k], J.gb[off], J.time_new, true);
                    } else {
                        // Mirror rule of an x or y face (see the z-border
                        // path below for the face order).
                        T opp;
                        bool minus;
                        if (y == L.ny - 1)      { opp = s; minus = true; }
                        else if (y == 0)        { opp = n; minus = false; }
                        else if (x == L.nx - 1) { opp = w[k]; minus = true; }
                        else                    { opp = e[k]; minus = false; }
                        v[k] = P::mirror(cur[k], opp, minus ? negated(J.corr) : J.corr);
                    }
                }
                if (live) J.un[off] = v[k];
            }
        };
        if (ok && !zb) {
            if (tile_inner) rows(std::true_type{});
            else rows(std::false_type{});
        } else if (ok && xin) {
            const long long zoff = (long long)z * L.plane + x;
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int y = yb + k;
                if (y < L.ny) {
                    const long long off = zoff + (long long)y * L.pitch;
                    const T s = (k == 0) ? ym : cur[k - 1];
                    const T n = (k == R - 1) ? yp : cur[k + 1];
                    const T w = pl[(rb + k) * G::W - 1];
                    const T e = pl[(rb + k) * G::W + 1];
                    const bool border = xb || zb || y < nl || y > L.ny - 1 - nl;
                    T v;
                    if (!border) {
                        T f = P::zero();
                        if (HAS_F) f = P::src(J.fa[off], has_fb ? J.fb[off] : P::zero(), J.time_old, has_fb);
                        if constexpr (VC) {
                            const int bo = (ty * R + k) * BX + tx;
                            v = P::template star_vc<HAS_F>(c, cur[k], w, e, s, n, below[k], above[k], f,
                                                           st[slot(p) * G::STRIDE + G::C0OFF + bo],
                                                           st[slot(p) * G::STRIDE + G::CAOFF + bo]);
                        } else {
                            v = P::template star<HAS_F>(c, cur[k], w, e, s, n, below[k], above[k], f);
                        }
                    } else if (BORDER == SCAFES_BORDER_NODES) {
                        v = node_rule<P>(J, x, y, z, cur[k], w, e, s, n, below[k], above[k]);
                    } else if (BORDER == SCAFES_BORDER_TABLE) {
                        const int mask = (x == 0) | ((x == L.nx - 1) << 1) | ((y == 0) << 2) |
                                         ((y == L.ny - 1) << 3) | ((z == 0) << 4) | ((z == L.nz - 1) << 5);
                        v = table_rule<P, HAS_F, has_fb>(J, mask, off, cur[k], w, e, s, n, below[k], above[k]);
                    } else if (BORDER == SCAFES_BORDER_DIRICHLET) {
                        // Border values are stored in the element type, so
                        // this branch does no FP64 work on the FP32 paths.
                        v = J.ga ? J.ga[off] : J.gval;
                        if (has_gb) v = P::src(v, J.gb[off], J.time_new, true);
                    } else {
                        // Mirror border: the last face (in direction order
                        // x-, x+, y-, y+, z-, z+) the node lies on decides.
                        T opp;
                        bool minus;
                        if (z == L.nz - 1)      { opp = below[k]; minus = true; }
                        else if (z == 0)        { opp = above[k]; minus = false; }
                        else if (y == L.ny - 1) { opp = s; minus = true; }
                        else if (y == 0)        { opp = n; minus = false; }
                        else if (x == L.nx - 1) { opp = w; minus = true; }
                        else                    { opp = e; minus = false; }
                        v = P::mirror(cur[k], opp, minus ? negated(J.corr) : J.corr);
                    }
                    J.un[off] = v;
                }
            }
        }
        // Everyone is done with plane p-1: its stage takes plane p-1+NS.
        if (!__syncthreads_and(ok)) return false;
        if (tid == 0) {
            const int pn = p - 1 + NS;
            if (pn < np) {
                fence_proxy_async_smem();
                issue(pn);
            }
        }
        ++p;
        ++z;
        return true;
    };

    bool all_ok = true;
    while (z < z1) {
        if (!(all_ok = plane(qa, qb, qc)) || z >= z1) break;
        if (!(all_ok = plane(qb, qc, qa)) || z >= z1) break;
        if (!(all_ok = plane(qc, qa, qb))) break;
    }
    if (!all_ok) {
        if (tid == 0) {
            // A stage never completed: report, drain what was issued, stop.
            atomicExch(status, SCAFES_ERR_TIMEOUT);
            for (int q = (p > 0 ? p - 1 : 0); q < np && q < p - 1 + NS; ++q)
                bounded_wait(&bar[slot(q)], phase(q), kWaitLimitNs / 8);
        }
        return false;
    }
    base = b0 + (uint32_t)np;
    return true;
}

}  // namespace scafes
