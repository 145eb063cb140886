// Internal interface between the C ABI (capi.cu) and the plain 7-point sweep
// kernels (sweep_star7.cu).
#pragma once

#include <cuda.h>

#include "scafes_common.cuh"
#include "../../include/scafes_gb300.h"

namespace scafes {

// Number of CTA tile variants of the plain sweep (32 x BY columns, R rows
// per thread): {8,1}, {16,2}, {32,4}, {16,4}.
constexpr int STAR7_NUM_TILES = 4;
// The one tile variant built for more than one border layer; a launch with
// L.nl != 1 must use it (its TMA descriptors are encoded for that tile).
constexpr int STAR7_MULTI_LAYER_TILE = 1;

// Coefficients of u_new = c0*u + sum_p cp*(u_{p-}+u_{p+}) + cf*F, in double
// and split into FP32 triples (hi + lo + lo2, ~72 bits) for the
// compensated path.
// Width (nodes along x) of every sweep tile: one warp per row.
constexpr int BX = 32;

struct Star7Coeffs {
    double c0, cx, cy, cz, cf;
    float c0h, c0l, c0ll, cxh, cxl, cxll, cyh, cyl, cyll, czh, czl, czll, cfh, cfl, cfll;
};

Star7Coeffs make_star7_coeffs(double c0, const double cp[3], double cf);

// A scalar in double and split into an FP32 pair (hi + lo), prepared on the
// host so that the FP32 kernels never convert doubles themselves.
struct Split {
    double d;
    float hi, lo;
};

inline Split make_split(double v) {
    Split s;
    s.d = v;
    f2 p = split_double(v);
    s.hi = p.hi;
    s.lo = p.lo;
    return s;
}

__host__ __device__ inline Split negated(const Split& s) {
    Split r;
    r.d = -s.d;
    r.hi = -s.hi;
    r.lo = -s.lo;
    return r;
}

// Width (elements) of the TMA box of the sweep for a precision: the 32-wide
// tile plus a halo padded to 16 bytes on each side.
int star7_box_width(int precision);
// Height (rows) of the TMA box of tile variant `tile`.
int star7_box_height(int tile);
// Tile variant used when none is chosen: {8,1} for FP64; otherwise {32,4}
// on large grids and {8,1} else.
int star7_default_tile(const Layout& L, int precision);

// Device block of a SCAFES_BORDER_TABLE problem: the rule of each border
// class and the border field's higher time orders and time variable
// (scafes_gpu_set_border_time_basis).
struct BorderTable {
    scafes_border_form rule[SCAFES_BORDER_CLASSES];
    const double* g_hi[3] = {nullptr, nullptr, nullptr};  // G_C, G_D, G_E (FP64) or null
    double t_center = 0.0, t_rate = 1.0;
};

// Border nodes (within nl of a face) of an nx x ny x nz grid.
__host__ __device__ inline long long border_node_count(int nx, int ny, int nz, int nl) {
    const long long full = (long long)nx * ny * nz;
    const long long in = (long long)(nx - 2 * nl) * (ny - 2 * nl) * (nz - 2 * nl);
    return full - (in > 0 ? in : 0);
}

// Position of border node (x, y, z) among the border nodes in Fortran order
// (x fastest).  A plane within nl of a z face is all border nodes; another
// plane has nl full rows at each y face and 2*nl nodes in every other row.
__host__ __device__ inline long long border_node_index(const Layout& L, int x, int y, int z) {
    const int nl = L.nl;
    const long long pb = (long long)L.nx * L.ny;                                   // border plane
    const long long pi = 2LL * nl * L.nx + (long long)(L.ny - 2 * nl) * 2 * nl;   // other plane
    const int zb = (z < nl ? z : nl) + (z > L.nz - nl ? z - (L.nz - nl) : 0);  // border planes below z
    long long idx = (long long)zb * pb + (long long)(z - zb) * pi;
    if (z < nl || z >= L.nz - nl) return idx + (long long)y * L.nx + x;
    const int yb = (y < nl ? y : nl) + (y > L.ny - nl ? y - (L.ny - nl) : 0);  // full rows below y
    idx += (long long)yb * L.nx + (long long)(y - yb) * 2 * nl;
    if (y < nl || y >= L.ny - nl) return idx + x;
    return idx + (x < nl ? x : nl + (x - (L.nx - nl)));
}

struct Star7Launch {
    int precision;        // enum scafes_precision
    int border;           // enum scafes_border
    int tile;             // tile variant 0 .. STAR7_NUM_TILES-1
    Layout L;
    const CUtensorMap* tm_uo;  // TMA descriptor of the old iterate
    const CUtensorMap* tm_f;   // TMA descriptor of F_A, box 32 x BY of the tile (F_A-only sources)
    int* status;          // device status word (0 = ok)
    const void* uo;       // old iterate (element type per precision)
    void* un;             // new iterate
    const void* fa;       // source F_A (element type per precision) or null
    const void* fb;       // source F_B or null
    const void* ga;       // border value G_A (element type per precision) or null
    const void* gb;       // border value G_B or null
    double gconst;        // border value when ga is null
    Star7Coeffs c;
    double time_old;      // time(t)   : F is read at the old time
    double time_new;      // time(t+1) : G is read at the new time
    double time_new2;     // time(t+2) : the second step of a depth-2 pass
    const CUtensorMap* tm_tb;  // TMA descriptor of the old iterate for depth-2 passes
    double mirror_corr;   // 2^t for SCAFES_BORDER_MIRROR_POW2
    const BorderTable* table;  // device rules for SCAFES_BORDER_TABLE
    // Variable coefficients (slots C0 and CA uploaded): C0, CA staged by TMA
    // with the iterate (boxes 32 x BY of the tile), like F_A.
    bool vc = false;
    const CUtensorMap* tm_c0 = nullptr;
    const CUtensorMap* tm_ca = nullptr;
    const scafes_border_node_rule* nodes = nullptr;  // SCAFES_BORDER_NODES rules
};

// Enqueues one sweep (one time step) on `stream`.  Returns cudaSuccess or the
// launch error.
cudaError_t launch_star7(const Star7Launch& a, cudaStream_t stream);

// Enqueues one depth-2 pass (two time steps; star7_tb.cuh) on `stream`:
// Dirichlet border, one border layer, no time-dependent source, a.tm_tb
// encoded by star7_tb_box.  Returns cudaErrorInvalidValue for any other
// problem.
cudaError_t launch_star7_tb(const Star7Launch& a, cudaStream_t stream);
// Sets the depth-2 kernels' attributes of a precision (before a stream
// capture that launches them).
cudaError_t launch_star7_tb_prepare(int precision);
// TMA box (width, rows) of the depth-2 pass for a precision.
void star7_tb_box(int precision, int* width, int* rows);
// Whether a problem can take depth-2 passes.
bool star7_tb_eligible(const Star7Launch& a);

// Conversions between host-layout doubles (dense, x fastest) staged on the
// device and the padded device layout of each precision.
cudaError_t convert_to_device(int precision, const double* dense, void* field,
                              const Layout& L, cudaStream_t stream);
cudaError_t convert_from_device(int precision, const void* field,
                                double* dense, const Layout& L,
                                cudaStream_t stream);

size_t element_size(int precision);

}  // namespace scafes
