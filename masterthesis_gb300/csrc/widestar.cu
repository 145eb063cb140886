// Wider stencils with a width per data field: the averaging update of
// tests/system/HeatEqnFdmStencilWidthVar/HeatEqnFdmStencilWidthVar.hpp:120-165
// (the reference's test of per-field ghost widths, src/ScaFES_Problem.hpp:
// 1495-1514).  Every node, inner or border, takes
//   u' = 2 + (sum of the values within `w` nodes along each axis, truncated
//             at the grid's faces, + u - cc) / count
// where cc sums the signed offsets that were added (+r to the right, -r to
// the left) and count is 1 + the number of values added.  The sum runs in
// the reference's order (axes x, y, z; per axis the left side r = 1..w, then
// the right side), with the same single division, so results are bit-exact
// to the reference.
//
// One thread per (x, y) column marches a chunk of z-planes; neighbours come
// through L1/L2 (the update is an FP64 sum plus one FP64 division per node,
// so the FP64 pipe, not HBM, bounds it on GB300).  Each field of a handle
// has its own width; one launch per field per step.
#include <cstdarg>
#include <cstdio>
#include <string>
#include <vector>

#include "scafes_common.cuh"
#include "../../include/scafes_gb300.h"

using namespace scafes;

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

constexpr int WX = 32, WY = 8, WZ = 16;

__global__ void __launch_bounds__(WX * WY)
k_wide(const double* __restrict__ u, double* __restrict__ un, Layout L, int w, int wz) {
    const int x = blockIdx.x * WX + threadIdx.x, y = blockIdx.y * WY + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const int zb = blockIdx.z * wz, ze = min(zb + wz, L.nz);
    const int ms_x = min(x, w), me_x = min(L.nx - 1 - x, w);
    const int ms_y = min(y, w), me_y = min(L.ny - 1 - y, w);
    for (int z = zb; z < ze; ++z) {
        const long long o = L.idx(x, y, z);
        const int ms_z = min(z, w), me_z = min(L.nz - 1 - z, w);
        double sum = 0.0;
        int cc = 0;
        for (int r = 1; r <= ms_x; ++r) { sum += u[o - r]; cc -= r; }
        for (int r = 1; r <= me_x; ++r) { sum += u[o + r]; cc += r; }
        for (int r = 1; r <= ms_y; ++r) { sum += u[o - (long long)r * L.pitch]; cc -= r; }
        for (int r = 1; r <= me_y; ++r) { sum += u[o + (long long)r * L.pitch]; cc += r; }
        for (int r = 1; r <= ms_z; ++r) { sum += u[o - (long long)r * L.plane]; cc -= r; }
        for (int r = 1; r <= me_z; ++r) { sum += u[o + (long long)r * L.plane]; cc += r; }
        const int cnt = 1 + ms_x + me_x + ms_y + me_y + ms_z + me_z;
        // Two separate roundings as in the reference: no contraction here.
        const double num = __dsub_rn(__dadd_rn(sum, u[o]), (double)cc);
        un[o] = __dadd_rn(2.0, __ddiv_rn(num, (double)cnt));
    }
}

}  // namespace

struct scafes_wide {
    Layout L;
    std::vector<int> widths;
    std::vector<double*> buf[2];  // per field: current and next iterate
    int cur = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    bool timed = false;
    std::string err;
};

namespace {

int wfail(scafes_wide* h, int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof(b), fmt, ap);
    va_end(ap);
    if (h) h->err = b;
    scafes::set_last_error(b);
    return code;
}

#define WTRY(h, call)                                                                          \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess)                                                                 \
            return wfail(h, SCAFES_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                         __FILE__, __LINE__);                                                  \
    } while (0)

int check_field(scafes_wide* h, int field, const void* host, size_t n, const char* who) {
    if (!h) return wfail(nullptr, SCAFES_ERR_ARG, "%s: handle is NULL", who);
    if (field < 0 || field >= (int)h->widths.size())
        return wfail(h, SCAFES_ERR_ARG, "%s: field %d out of range [0, %d)", who, field, (int)h->widths.size());
    const size_t nn = (size_t)h->L.nx * h->L.ny * h->L.nz;
    if (!host || n != nn) return wfail(h, SCAFES_ERR_ARG, "%s: expected %zu values, got %zu", who, nn, n);
    return SCAFES_OK;
}

}  // namespace

extern "C" const char* scafes_wide_last_error(const scafes_wide* h) { return h ? h->err.c_str() : ""; }

extern "C" void scafes_wide_destroy(scafes_wide* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (int b = 0; b < 2; ++b)
        for (double* p : h->buf[b]) cudaFree(p);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int scafes_wide_create(const int n_nodes[3], int n_fields, const int* widths, void* stream,
                                  scafes_wide** out) {
    if (!out || !n_nodes || !widths || n_fields < 1)
        return wfail(nullptr, SCAFES_ERR_ARG, "scafes_wide_create: bad arguments");
    *out = nullptr;
    for (int p = 0; p < 3; ++p)
        if (n_nodes[p] < 1 || n_nodes[p] > (1 << 20))
            return wfail(nullptr, SCAFES_ERR_ARG, "scafes_wide_create: n_nodes[%d]=%d out of [1, 2^20]", p,
                         n_nodes[p]);
    for (int f = 0; f < n_fields; ++f)
        if (widths[f] < 0 || widths[f] > SCAFES_WIDE_MAX_WIDTH)
            return wfail(nullptr, SCAFES_ERR_ARG, "scafes_wide_create: width %d of field %d out of [0, %d]",
                         widths[f], f, SCAFES_WIDE_MAX_WIDTH);
    scafes_wide* h = new (std::nothrow) scafes_wide();
    if (!h) return wfail(nullptr, SCAFES_ERR_NOMEM, "scafes_wide_create: out of host memory");
    h->L = make_layout(n_nodes[0], n_nodes[1], n_nodes[2]);
    h->widths.assign(widths, widths + n_fields);
    cudaError_t e = cudaSuccess;
    if (stream) {
        h->stream = (cudaStream_t)stream;
    } else {
        e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
        h->own_stream = true;
    }
    const size_t bytes = (size_t)h->L.size() * sizeof(double);
    for (int b = 0; b < 2; ++b) h->buf[b].assign(n_fields, nullptr);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b)
        for (int f = 0; f < n_fields && e == cudaSuccess; ++f) {
            e = cudaMalloc(&h->buf[b][f], bytes);
            if (e == cudaSuccess) e = cudaMemsetAsync(h->buf[b][f], 0, bytes, h->stream);
        }
    if (e == cudaSuccess) e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->e1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? SCAFES_ERR_NOMEM : SCAFES_ERR_CUDA;
        wfail(nullptr, code, "scafes_wide_create: %s", cudaGetErrorString(e));
        scafes_wide_destroy(h);
        return code;
    }
    *out = h;
    return SCAFES_OK;
}

extern "C" int scafes_wide_upload(scafes_wide* h, int field, const double* host, size_t n) {
    int rc = check_field(h, field, host, n, "scafes_wide_upload");
    if (rc) return rc;
    const Layout& L = h->L;
    WTRY(h, cudaMemcpy2DAsync(h->buf[h->cur][field], (size_t)L.pitch * sizeof(double), host,
                              (size_t)L.nx * sizeof(double), (size_t)L.nx * sizeof(double), (size_t)L.ny * L.nz,
                              cudaMemcpyHostToDevice, h->stream));
    WTRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_wide_download(scafes_wide* h, int field, double* host, size_t n) {
    int rc = check_field(h, field, host, n, "scafes_wide_download");
    if (rc) return rc;
    const Layout& L = h->L;
    WTRY(h, cudaMemcpy2DAsync(host, (size_t)L.nx * sizeof(double), h->buf[h->cur][field],
                              (size_t)L.pitch * sizeof(double), (size_t)L.nx * sizeof(double), (size_t)L.ny * L.nz,
                              cudaMemcpyDeviceToHost, h->stream));
    WTRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_wide_step(scafes_wide* h, int n_steps) {
    if (!h) return wfail(nullptr, SCAFES_ERR_ARG, "scafes_wide_step: handle is NULL");
    if (n_steps < 0) return wfail(h, SCAFES_ERR_ARG, "scafes_wide_step: n_steps=%d < 0", n_steps);
    const Layout& L = h->L;
    int wz = WZ;
    while ((L.nz + wz - 1) / wz > 65535) wz <<= 1;  // grid.z limit
    const dim3 grid((L.nx + WX - 1) / WX, (L.ny + WY - 1) / WY, (L.nz + wz - 1) / wz);
    WTRY(h, cudaEventRecord(h->e0, h->stream));
    for (int s = 0; s < n_steps; ++s) {
        for (size_t f = 0; f < h->widths.size(); ++f) {
            k_wide<<<grid, dim3(WX, WY), 0, h->stream>>>(h->buf[h->cur][f], h->buf[h->cur ^ 1][f], L, h->widths[f],
                                                         wz);
            WTRY(h, cudaGetLastError());
        }
        h->cur ^= 1;
    }
    WTRY(h, cudaEventRecord(h->e1, h->stream));
    h->timed = true;
    return SCAFES_OK;
}

extern "C" int scafes_wide_last_ms(const scafes_wide* h, float* ms) {
    if (!h || !ms) return wfail(nullptr, SCAFES_ERR_ARG, "scafes_wide_last_ms: NULL argument");
    if (!h->timed) return wfail(nullptr, SCAFES_ERR_STATE, "scafes_wide_last_ms: nothing ran yet");
    cudaError_t e = cudaEventSynchronize(h->e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, h->e0, h->e1);
    if (e != cudaSuccess) return wfail(nullptr, SCAFES_ERR_CUDA, "scafes_wide_last_ms: %s", cudaGetErrorString(e));
    return SCAFES_OK;
}
