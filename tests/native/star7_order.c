/* One 7-point star sweep of the interior nodes in the FP64 sweep kernel's
 * own operation order, for bit-for-bit checks of that kernel:
 *   v = c0*u;  v = fma(cx, w+e, v);  v = fma(cy, s+n, v);  v = fma(cz, b+t, v)
 * (C99 fma is the correctly rounded fused multiply-add, as the GPU's).
 * Field layout x fastest, then y, then z.  Border nodes of `out` are set to
 * `border`.  Compile with -ffp-contract=off. */
#include <math.h>

void star7_sweep_f64(const double* u, double* out, int nx, int ny, int nz, double c0, double cx, double cy,
                     double cz, double border) {
    const long long px = 1, py = nx, pz = (long long)nx * ny;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const long long o = x * px + y * py + z * pz;
                if (x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1) {
                    out[o] = border;
                    continue;
                }
                double v = c0 * u[o];
                v = fma(cx, u[o - px] + u[o + px], v);
                v = fma(cy, u[o - py] + u[o + py], v);
                v = fma(cz, u[o - pz] + u[o + pz], v);
                out[o] = v;
            }
}

/* The variable-coefficient sweep's order (per-node C0 and CA, no source):
 *   l = cx*(w+e);  l = fma(cy, s+n, l);  l = fma(cz, b+t, l);  v = fma(ca, l, c0*u) */
void star7_vc_sweep_f64(const double* u, const double* c0f, const double* caf, double* out, int nx, int ny,
                        int nz, double cx, double cy, double cz, double border) {
    const long long px = 1, py = nx, pz = (long long)nx * ny;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) {
                const long long o = x * px + y * py + z * pz;
                if (x == 0 || y == 0 || z == 0 || x == nx - 1 || y == ny - 1 || z == nz - 1) {
                    out[o] = border;
                    continue;
                }
                double l = cx * (u[o - px] + u[o + px]);
                l = fma(cy, u[o - py] + u[o + py], l);
                l = fma(cz, u[o - pz] + u[o + pz], l);
                out[o] = fma(caf[o], l, c0f[o] * u[o]);
            }
}
