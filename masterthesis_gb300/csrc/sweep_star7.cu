// Plain 7-point sweep: one launch advances the whole grid by one time step.
//
// Replaces the per-node loop of ScaFES's evalTypeTwoAt
// (src/ScaFES_Problem.hpp:5399-5476) for the heat-type callbacks
// (tests/system/HeatEqnFDM/HeatEqnFDM.hpp:205-218,
//  tests/system/PennesBioheatEqnFDM/PennesBioheatEqnFDM.hpp:153-168) and
// their Dirichlet border (.../Dirichlet/Dirichlet.hpp:125-131), and the copy
// old->new that precedes it (:5078-5082): every node is written each step.
// Each CTA runs one tile (star7_tile.cuh) over a chunk of z-planes; the
// kernels are instantiated per element type in sweep_star7_{f64,f32x2,f32}.cu.
// This file holds the host helpers and the dispatch on the element type.
#include "star7_tb.cuh"
#include "star7_tile.cuh"

namespace scafes {

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

int star7_default_tile(const Layout& L, int precision) {
    // FP64: one row per thread (the integer-pipe sums want resident warps,
    // not registers; the autotuner's choice at every size measured).  Else
    // four rows per thread once the grid has enough tiles to fill the GPU.
    if (precision == SCAFES_PREC_F64) return 0;
    const long long cols = (long long)L.nx * L.ny;
    return cols >= 256LL * 256LL ? 2 : 0;
}

cudaError_t launch_star7_f64(const Star7Launch& a, cudaStream_t stream);
cudaError_t launch_star7_f32(const Star7Launch& a, cudaStream_t stream);
cudaError_t launch_star7_f32x2(const Star7Launch& a, cudaStream_t stream);
cudaError_t launch_star7_tb_f64(const Star7Launch& a, cudaStream_t stream);
cudaError_t launch_star7_tb_f32(const Star7Launch& a, cudaStream_t stream);
cudaError_t launch_star7_tb_f32x2(const Star7Launch& a, cudaStream_t stream);
cudaError_t prepare_star7_tb_f64();
cudaError_t prepare_star7_tb_f32();
cudaError_t prepare_star7_tb_f32x2();

bool star7_tb_eligible(const Star7Launch& a) {
    return a.border == SCAFES_BORDER_DIRICHLET && a.L.nl == 1 && a.fb == nullptr && !a.vc;
}

void star7_tb_box(int precision, int* width, int* rows) {
    const int esz = (int)element_size(precision);
    *width = tb_bw(esz);
    *rows = TB_BH;
}

cudaError_t launch_star7_tb(const Star7Launch& a, cudaStream_t stream) {
    switch (a.precision) {
        case SCAFES_PREC_F64: return launch_star7_tb_f64(a, stream);
        case SCAFES_PREC_F32: return launch_star7_tb_f32(a, stream);
        case SCAFES_PREC_F32X2: return launch_star7_tb_f32x2(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_star7_tb_prepare(int precision) {
    switch (precision) {
        case SCAFES_PREC_F64: return prepare_star7_tb_f64();
        case SCAFES_PREC_F32: return prepare_star7_tb_f32();
        case SCAFES_PREC_F32X2: return prepare_star7_tb_f32x2();
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_star7(const Star7Launch& a, cudaStream_t stream) {
    switch (a.precision) {
        case SCAFES_PREC_F64: return launch_star7_f64(a, stream);
        case SCAFES_PREC_F32: return launch_star7_f32(a, stream);
        case SCAFES_PREC_F32X2: return launch_star7_f32x2(a, stream);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace scafes
