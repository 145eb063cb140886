// Temporal blocking of the plain sweep: two time steps per pass over the
// field (depth 2), for the Dirichlet border with one border layer and a
// source that is absent or static.  Each step is the update of
// sweep_star7 (the reference's evalTypeTwoAt loop, src/ScaFES_Problem.hpp:
// 5399-5476, over the heat / Pennes callbacks and Dirichlet.hpp:125-131), in
// the same arithmetic per node (the policies' star), so a pass gives the
// same bits as two single-step sweeps while reading and writing the field
// once.
//
// A CTA owns a TB_X x TB_Y column tile of the output and marches z.  TMA
// brings, per plane, a box of the old iterate with a two-node halo in x and
// y (its x start padded down to 16 bytes) through a ring of TB_NS planes.
// At input plane q the CTA computes the intermediate step on plane q-1 over
// the tile plus a one-node halo (each thread two tile nodes and at most one
// halo node, centre and z-neighbours from register queues, x/y neighbours
// from the staged plane), then the second step on plane q-2 over its own
// nodes (intermediate z-neighbours from registers, x/y neighbours from the
// intermediate plane in shared memory), written to the new buffer: one
// block barrier per plane.  Each CTA recomputes the intermediate values its
// halo needs; nothing is exchanged between CTAs.  Every wait is bounded
// (status word, drain, return).
#pragma once

#include "star7.cuh"
#include "star7_policies.cuh"
#include "tma.cuh"

namespace scafes {

constexpr int TB_X = 32, TB_Y = 32;        // output tile
constexpr int TB_TY = 8, TB_R = 4;         // thread rows; each thread owns TB_R consecutive rows
constexpr int TB_NS = 4;                   // input ring: planes q-1, q in use, q+1, q+2 in flight
constexpr int TB_U1W = TB_X + 2, TB_U1H = TB_Y + 2, TB_U1 = TB_U1W * TB_U1H;  // intermediate region
constexpr int TB_BH = TB_Y + 4;            // input box rows: y0-2 .. y0+TB_Y+1
constexpr int TB_HALO = 2 * TB_U1W + 2 * TB_Y;  // intermediate cells around the output tile
static_assert(TB_Y == TB_TY * TB_R, "each thread row owns TB_R tile rows");
static_assert(TB_HALO <= TB_X * TB_TY, "one halo cell per thread at most");

// Left pad of the input box in elements (16 bytes of alignment, at least
// the two halo nodes) and its width.
__host__ __device__ constexpr int tb_lp(int esz) { return esz == 4 ? 4 : 2; }
__host__ __device__ constexpr int tb_bw(int esz) { return TB_X + 2 * tb_lp(esz); }
__host__ __device__ constexpr int tb_slot(int esz) {  // input slot, elements, 128-byte aligned
    return ((tb_bw(esz) * TB_BH * esz + 127) / 128) * 128 / esz;
}
__host__ __device__ constexpr size_t tb_smem(int esz) {
    return (size_t)(TB_NS * tb_slot(esz) + 2 * TB_U1) * esz + TB_NS * 8;
}

template <class P, bool HAS_F>
__global__ void __launch_bounds__(TB_X * TB_TY)
star7_tb2(const __grid_constant__ CUtensorMap tm, typename P::T* __restrict__ un,
          const typename P::T* __restrict__ fa, const typename P::T* __restrict__ ga,
          const typename P::T* __restrict__ gb, typename P::T gval, Layout L, Star7Coeffs c, Split time1,
          Split time2, int zchunk, int* __restrict__ status) {
    using T = typename P::T;
    constexpr int ESZ = sizeof(T);
    constexpr int LP = tb_lp(ESZ), BW = tb_bw(ESZ), SLOT = tb_slot(ESZ);
    constexpr int R = TB_R;
    extern __shared__ __align__(128) unsigned char tb_raw[];
    T* sin = reinterpret_cast<T*>(tb_raw);  // [TB_NS][SLOT]   input planes
    T* su1 = sin + TB_NS * SLOT;            // [2][TB_U1]      intermediate planes
    uint64_t* bar = reinterpret_cast<uint64_t*>(su1 + 2 * TB_U1);
    const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TB_X + tx;
    const int x0 = blockIdx.x * TB_X, y0 = blockIdx.y * TB_Y;
    const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, L.nz);
    const bool has_gb = gb != nullptr;

    if (__syncthreads_or(tid == 0 && *(volatile int*)status != 0)) return;
    if (tid == 0) {
        for (int b = 0; b < TB_NS; ++b) mbar_init(&bar[b], 1);
        fence_barrier_init();
    }
    __syncthreads();
    constexpr uint32_t TX_BYTES = (uint32_t)(BW * TB_BH * ESZ);
    // Input plane z0-2+i goes to ring slot i % TB_NS.
    auto issue = [&](int i, int slot) {
        mbar_arrive_expect_tx(&bar[slot], TX_BYTES);
        tma_load_3d(sin + slot * SLOT, &tm, x0 - LP, y0 - 2, z0 - 2 + i, &bar[slot]);
    };
    const int n_in = z1 - z0 + 4;  // input planes z0-2 .. z1+1
    if (tid == 0)
        for (int i = 0; i < TB_NS && i < n_in; ++i) issue(i, i);

    // The whole intermediate region holds inner nodes of the x/y faces: no
    // per-node border test except on the z-border planes.
    const bool inner_xy = x0 >= 2 && x0 + TB_X + 1 <= L.nx - 2 && y0 >= 2 && y0 + TB_Y + 1 <= L.ny - 2;
    // Own block: column tx, rows R*ty .. R*ty+R-1 of the tile.
    const int x = x0 + tx, yb = y0 + R * ty;
    const int ob = (R * ty + 2) * BW + tx + LP;         // its first node in an input slot
    const int ou = (R * ty + 1) * TB_U1W + tx + 1;      // ... in an intermediate plane
    const long long oo = (long long)yb * L.pitch + x;  // ... in a plane of the field
    // Halo item (threads tid < TB_HALO): one intermediate cell around the tile.
    int hlx, hly;
    {
        const int h = tid < TB_HALO ? tid : 0;
        if (h < TB_U1W) { hlx = h; hly = 0; }
        else if (h < 2 * TB_U1W) { hlx = h - TB_U1W; hly = TB_U1H - 1; }
        else if (h < 2 * TB_U1W + TB_Y) { hlx = 0; hly = h - 2 * TB_U1W + 1; }
        else { hlx = TB_U1W - 1; hly = h - 2 * TB_U1W - TB_Y + 1; }
    }
    const bool has_h = tid < TB_HALO;
    const int hgx = x0 - 1 + hlx, hgy = y0 - 1 + hly;
    const int hb = (hly + 1) * BW + hlx - 1 + LP, hu = hly * TB_U1W + hlx;
    const bool h_in = has_h && hgx >= 0 && hgx < L.nx && hgy >= 0 && hgy < L.ny;
    const bool h_xy = hgx == 0 || hgx == L.nx - 1 || hgy == 0 || hgy == L.ny - 1;
    const long long ho = (long long)hgy * L.pitch + hgx;

    // The value of a border node at a time level.
    auto border_value = [&](long long off, const Split& tm_) {
        T v = ga ? ga[off] : gval;
        if (has_gb) v = P::src(v, gb[off], tm_, true);
        return v;
    };

    // Input ring: sl[] are the slots of planes q-1, q, q+1, q+2; bit s of
    // ph is the parity of slot s's next phase.
    int sl[TB_NS] = {0, 1, 2, 3};
    uint32_t ph = 0;
    bool ok = bounded_wait(&bar[0], 0);
    ph ^= 1u;
    ok = bounded_wait(&bar[1], 0) && ok;
    ph ^= 2u;
    // z-queues (registers): input values at planes q-2 (qb), q-1 (qc) of the
    // own block and the halo cell; intermediate values of the own block at
    // planes q-3 (ub), q-2 (uc), q-1 (ua).
    T qb[R], qc[R], qa[R], ub[R], uc[R], ua[R];
    T hqb, hqc;
#pragma unroll
    for (int k = 0; k < R; ++k) {
        qb[k] = sin[0 * SLOT + ob + k * BW];  // slot 0: plane z0-2
        qc[k] = sin[1 * SLOT + ob + k * BW];  // slot 1: plane z0-1
        ub[k] = uc[k] = ua[k] = P::zero();
    }
    hqb = sin[hb];
    hqc = sin[SLOT + hb];
    // Plane z0-2 now lives in registers: its slot takes plane z0+2.
    __syncthreads();
    if (tid == 0) {
        fence_proxy_async_smem();
        if (TB_NS < n_in) issue(TB_NS, 0);
    }
    sl[0] = 1;  // plane z0-1
    sl[1] = 2;  // plane z0
    sl[2] = 3;  // plane z0+1
    sl[3] = 0;  // plane z0+2

    // A load never completed: report, drain whatever may still be in flight
    // (both phases of every slot: a completed phase returns at once; an
    // error path may spend a second here).
    auto fail = [&]() {
        if (tid == 0) {
            atomicExch(status, SCAFES_ERR_TIMEOUT);
            for (int b = 0; b < TB_NS; ++b) {
                bounded_wait(&bar[b], (ph >> b) & 1u, kWaitLimitNs / 16);
                bounded_wait(&bar[b], ((ph >> b) & 1u) ^ 1u, kWaitLimitNs / 16);
            }
        }
    };
    // (A loop unrolled by three with rotating queue roles instead of the
    // register moves below took more registers and ran slower.)
    for (int q = z0; q <= z1 + 1; ++q) {
        const int i_q = q - z0 + 2;  // index of input plane q
        // One barrier per plane: the previous plane's reads are done (its
        // slot may be refilled) and every wait so far succeeded.  A plane
        // whose wait failed is computed on whatever arrived; the next
        // barrier (or the one after the loop) stops the CTA and reports it.
        if (!__syncthreads_and(ok)) {
            fail();
            return;
        }
        if (q > z0 && tid == 0) {
            fence_proxy_async_smem();
            if (i_q + 2 < n_in) issue(i_q + 2, sl[3]);
        }
        ok = bounded_wait(&bar[sl[1]], (ph >> sl[1]) & 1u) && ok;  // input plane q
        ph ^= 1u << sl[1];
        const T* pc = sin + sl[0] * SLOT;  // input plane q-1
        const T* pa = sin + sl[1] * SLOT;  // input plane q
        T* w1 = su1 + ((q - 1) & 1) * TB_U1;        // receives the intermediate plane q-1
        const T* r1 = su1 + ((q - 2) & 1) * TB_U1;  // intermediate plane q-2
        const int l1 = q - 1;
        const bool l1_in = l1 >= 0 && l1 < L.nz;
        const bool l1_zb = l1 == 0 || l1 == L.nz - 1;

        // First step on plane q-1: the own block (rows in registers) ...
        {
            T w[R], e[R], f[R], v[R];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                qa[k] = pa[ob + k * BW];
                w[k] = pc[ob + k * BW - 1];
                e[k] = pc[ob + k * BW + 1];
                f[k] = P::zero();
                if (HAS_F && l1_in && x < L.nx && yb + k < L.ny) f[k] = fa[(long long)l1 * L.plane + oo + (long long)k * L.pitch];
            }
            const T ym = pc[ob - BW], yp = pc[ob + R * BW];
            unsigned skip = 0u;  // rows the border rule replaces
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int y = yb + k;
                if (!l1_in || l1_zb || x <= 0 || x >= L.nx - 1 || y <= 0 || y >= L.ny - 1) skip |= 1u << k;
            }
            P::template star_rows<HAS_F, R>(c, qb, qc, qa, ym, yp, w, e, f, v, skip);
            if (!inner_xy || l1_zb || !l1_in) {
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int y = yb + k;
                    if (!l1_in || x >= L.nx || y >= L.ny) v[k] = P::zero();
                    else if (l1_zb || x == 0 || x == L.nx - 1 || y == 0 || y == L.ny - 1)
                        v[k] = border_value((long long)l1 * L.plane + oo + (long long)k * L.pitch, time1);
                }
            }
#pragma unroll
            for (int k = 0; k < R; ++k) {
                w1[ou + k * TB_U1W] = v[k];
                ub[k] = uc[k];
                uc[k] = ua[k];
                ua[k] = v[k];
                qb[k] = qc[k];
                qc[k] = qa[k];
            }
        }
        // ... and the halo cell.
        if (has_h) {
            const T hqa = pa[hb];
            T v = P::zero();
            if (l1_in && h_in) {
                const long long off = (long long)l1 * L.plane + ho;
                if (l1_zb || h_xy) {
                    v = border_value(off, time1);
                } else {
                    T f = P::zero();
                    if (HAS_F) f = fa[off];
                    v = P::template star<HAS_F>(c, hqc, pc[hb - 1], pc[hb + 1], pc[hb - BW], pc[hb + BW], hqb, hqa,
                                                f);
                }
            }
            w1[hu] = v;
            hqb = hqc;
            hqc = hqa;
        }

        // Second step on plane q-2 for the own block: z-neighbours from the
        // queues, x/y neighbours from the intermediate plane q-2 (complete
        // since the barrier that opened this plane).
        const int l2 = q - 2;
        if (l2 >= z0) {
            const bool l2_zb = l2 == 0 || l2 == L.nz - 1;
            T w[R], e[R], f[R], v[R];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                w[k] = r1[ou + k * TB_U1W - 1];
                e[k] = r1[ou + k * TB_U1W + 1];
                f[k] = P::zero();
                if (HAS_F && x < L.nx && yb + k < L.ny) f[k] = fa[(long long)l2 * L.plane + oo + (long long)k * L.pitch];
            }
            const T ym = r1[ou - TB_U1W], yp = r1[ou + R * TB_U1W];
            unsigned skip = 0u;  // rows the border rule replaces
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int y = yb + k;
                if (l2_zb || x <= 0 || x >= L.nx - 1 || y <= 0 || y >= L.ny - 1) skip |= 1u << k;
            }
            P::template star_rows<HAS_F, R>(c, ub, uc, ua, ym, yp, w, e, f, v, skip);
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int y = yb + k;
                if (inner_xy && !l2_zb) {
                    un[(long long)l2 * L.plane + oo + (long long)k * L.pitch] = v[k];
                } else if (x < L.nx && y < L.ny) {
                    const long long off = (long long)l2 * L.plane + oo + (long long)k * L.pitch;
                    if (l2_zb || x == 0 || x == L.nx - 1 || y == 0 || y == L.ny - 1) v[k] = border_value(off, time2);
                    un[off] = v[k];
                }
            }
        }
        // Rotate the input ring: plane q-1's slot takes plane q+3.
        const int s0 = sl[0];
        sl[0] = sl[1];
        sl[1] = sl[2];
        sl[2] = sl[3];
        sl[3] = s0;
    }
    if (!__syncthreads_and(ok)) fail();  // the last plane's wait
}

}  // namespace scafes
