// C ABI of the plain (single-instance) problem: handle life cycle, field
// transfer, the time-step loop and the L-infinity error check.
//
// The handle plays the role of the field lumps the ScaFES Problem
// constructor allocates (src/ScaFES_Problem.hpp:1604-1674): two ping-pong
// buffers of the unknown field (the old/new pair swapped by
// swapPointersOfUnknownDfs, :3273-3316) plus the known fields.
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint.cuh"
#include "star7.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

using namespace scafes;

namespace {

thread_local std::string g_last_error;

int fail(std::string* where, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    if (where) *where = buf;
    return code;
}

// Bytes of host staging used for precision conversions (per slab).
constexpr size_t kStageBytes = 64ull << 20;

}  // namespace

struct scafes_handle {
    scafes_cfg cfg;
    Layout L;
    size_t esz = 0;
    void* u[2] = {nullptr, nullptr};
    CUtensorMap tm[2][STAR7_NUM_TILES];   // TMA descriptors of u[0], u[1] per tile
    bool tm_ok[2][STAR7_NUM_TILES] = {};
    CUtensorMap tmf[STAR7_NUM_TILES];     // TMA descriptors of F_A (box 32 x BY) per tile
    bool tmf_ok[STAR7_NUM_TILES] = {};
    CUtensorMap tmc[2][STAR7_NUM_TILES];  // TMA descriptors of C0 and CA (box 32 x BY) per tile
    bool tmc_ok[2][STAR7_NUM_TILES] = {};
    scafes_border_node_rule* nodes = nullptr;  // per-node border rules (SCAFES_BORDER_NODES)
    int tile = 0;                         // tile variant of the sweep
    int depth = 1;                        // temporal blocking depth (1 or 2)
    CUtensorMap tm_tb[2];                 // TMA descriptors of u[0], u[1] for depth-2 passes
    bool tm_tb_ok[2] = {};
    int* status = nullptr;                // device status word of the kernels
    int cur = 0;
    void* fld[SCAFES_FIELD_COUNT] = {};   // known slots (U slot unused here)
    bool has[SCAFES_FIELD_COUNT] = {};
    double* stage = nullptr;              // device staging for conversions
    size_t stage_elems = 0;
    double* red = nullptr;                // err_linf partial maxima (scratch)
    int red_blocks = 0;
    double* red_host = nullptr;           // pinned result of err_linf
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    int launches = 0;
    int t = 0;
    bool uploaded = false;
    // Border rules of a SCAFES_BORDER_TABLE problem (device copy) and whether
    // any rule reads the source field.
    BorderTable* table = nullptr;          // device copy of table_host
    BorderTable table_host;
    bool table_needs_f = false;
    // Snapshot writer (allocated on first use): a dense FP64 copy of the
    // iterate on the device, two pinned host buffers, a copy stream.
    double* snap_dev = nullptr;
    double* snap_host[2] = {nullptr, nullptr};
    cudaStream_t snap_stream = nullptr;
    cudaEvent_t snap_conv = nullptr, snap_copied[2] = {nullptr, nullptr};
    // Backward entry: with keep_initial, every upload of the unknown field
    // also lands as FP64 in u0keep, the state scafes_gpu_adjoint starts
    // from; the adjoint engine is created on first use.
    bool keep_initial = false;
    bool u0keep_valid = false;
    double* u0keep = nullptr;
    int* mismatch = nullptr;               // border check of scafes_gpu_adjoint
    scafes_adj* adj = nullptr;
    int adj_snaps = 0, adj_prec = -1;
    std::string err;
};

#define CUDA_TRY(h, call)                                                           \
    do {                                                                            \
        cudaError_t e_ = (call);                                                    \
        if (e_ != cudaSuccess)                                                      \
            return fail((h) ? &(h)->err : nullptr, SCAFES_ERR_CUDA, "%s: %s (%s:%d)", \
                        #call, cudaGetErrorString(e_), __FILE__, __LINE__);         \
    } while (0)

namespace scafes {
// Lets other translation units of the library record a message for
// scafes_last_error().
void set_last_error(const char* msg) { g_last_error = msg ? msg : ""; }
}  // namespace scafes

extern "C" const char* scafes_last_error(void) { return g_last_error.c_str(); }

extern "C" const char* scafes_gpu_last_error(const scafes_handle* h) {
    return h ? h->err.c_str() : g_last_error.c_str();
}

extern "C" int scafes_star7_heat_coeffs(scafes_cfg* cfg, double coeff_a,
                                        double rho_c, double perf) {
    if (!cfg || cfg->dim != 3 || rho_c == 0.0)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_star7_heat_coeffs: bad arguments");
    double sum = 0.0;
    for (int p = 0; p < 3; ++p) {
        if (cfg->n_nodes[p] < 2)
            return fail(nullptr, SCAFES_ERR_ARG, "scafes_star7_heat_coeffs: n_nodes[%d] < 2", p);
        const double h = (cfg->coord_last[p] - cfg->coord_first[p]) / (cfg->n_nodes[p] - 1);
        cfg->cp[p] = cfg->tau * coeff_a / (h * h);
        sum += cfg->cp[p];
    }
    cfg->c0 = 1.0 - 2.0 * sum - cfg->tau * perf;
    cfg->cf = cfg->tau * (1.0 / rho_c);
    return SCAFES_OK;
}

static int validate(const scafes_cfg* c) {
    if (!c) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_create: cfg is NULL");
    if (c->dim != 3)
        return fail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_create: dim=%d (only 3 is supported)", c->dim);
    for (int p = 0; p < 3; ++p)
        if (c->n_nodes[p] < 3 || c->n_nodes[p] > (1 << 20))
            return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_create: n_nodes[%d]=%d out of range [3, 2^20]",
                        p, c->n_nodes[p]);
    int nmin = c->n_nodes[0];
    for (int p = 1; p < 3; ++p) nmin = c->n_nodes[p] < nmin ? c->n_nodes[p] : nmin;
    if (c->n_layers_at_border < 1 || 2 * c->n_layers_at_border > nmin)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_create: n_layers_at_border=%d out of [1, %d]",
                    c->n_layers_at_border, nmin / 2);
    if (c->n_layers_at_border != 1 && c->border == SCAFES_BORDER_MIRROR_POW2)
        return fail(nullptr, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_create: the mirror border is a one-layer rule (n_layers_at_border=%d)",
                    c->n_layers_at_border);
    if (c->precision != SCAFES_PREC_F64 && c->precision != SCAFES_PREC_F32X2 &&
        c->precision != SCAFES_PREC_F32)
        return fail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_create: precision %d not supported", c->precision);
    if (c->border != SCAFES_BORDER_DIRICHLET && c->border != SCAFES_BORDER_MIRROR_POW2 &&
        c->border != SCAFES_BORDER_TABLE && c->border != SCAFES_BORDER_NODES)
        return fail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_create: border kind %d not supported", c->border);
    if (c->border == SCAFES_BORDER_NODES && (c->n_layers_at_border != 1 || c->precision == SCAFES_PREC_F32X2))
        return fail(nullptr, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_create: per-node border rules take one border layer and F64 or F32");
    if (c->tile < 0 || c->tile > STAR7_NUM_TILES)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_create: tile=%d out of range [0, %d]", c->tile,
                    STAR7_NUM_TILES);
    return SCAFES_OK;
}

extern "C" void scafes_gpu_destroy(scafes_handle* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    scafes_adj_destroy(h->adj);
    cudaFree(h->u0keep);
    cudaFree(h->mismatch);
    for (int i = 0; i < 2; ++i) cudaFree(h->u[i]);
    cudaFree(h->status);
    for (int i = 0; i < SCAFES_FIELD_COUNT; ++i) cudaFree(h->fld[i]);
    cudaFree(h->stage);
    cudaFree(h->table);
    cudaFree(h->nodes);
    cudaFree(h->snap_dev);
    for (int i = 0; i < 2; ++i) {
        if (h->snap_host[i]) cudaFreeHost(h->snap_host[i]);
        if (h->snap_copied[i]) cudaEventDestroy(h->snap_copied[i]);
    }
    if (h->snap_conv) cudaEventDestroy(h->snap_conv);
    if (h->snap_stream) cudaStreamDestroy(h->snap_stream);
    cudaFree(h->red);
    if (h->red_host) cudaFreeHost(h->red_host);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int scafes_gpu_create(const scafes_cfg* cfg, scafes_handle** out) {
    if (!out) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_create: out is NULL");
    *out = nullptr;
    int rc = validate(cfg);
    if (rc != SCAFES_OK) return rc;
    scafes_handle* h = new (std::nothrow) scafes_handle();
    if (!h) return fail(nullptr, SCAFES_ERR_NOMEM, "scafes_gpu_create: out of host memory");
    h->cfg = *cfg;
    h->L = make_layout(cfg->n_nodes[0], cfg->n_nodes[1], cfg->n_nodes[2]);
    h->L.nl = cfg->n_layers_at_border;
    h->esz = element_size(cfg->precision);
    const size_t bytes = (size_t)h->L.size() * h->esz;
    auto bail = [&](int code, const char* what, cudaError_t e) {
        int r = fail(nullptr, code, "scafes_gpu_create: %s: %s", what, cudaGetErrorString(e));
        scafes_gpu_destroy(h);
        return r;
    };
    cudaError_t e;
    if (cfg->stream) {
        h->stream = (cudaStream_t)cfg->stream;
    } else {
        if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess)
            return bail(SCAFES_ERR_CUDA, "cudaStreamCreate", e);
        h->own_stream = true;
    }
    for (int i = 0; i < 2; ++i) {
        if ((e = cudaMalloc(&h->u[i], bytes)) != cudaSuccess)
            return bail(SCAFES_ERR_NOMEM, "cudaMalloc(u)", e);
        if ((e = cudaMemsetAsync(h->u[i], 0, bytes, h->stream)) != cudaSuccess)
            return bail(SCAFES_ERR_CUDA, "cudaMemset(u)", e);
    }
    h->tile = cfg->tile > 0 ? cfg->tile - 1 : star7_default_tile(h->L, cfg->precision);
    if ((e = cudaMalloc(&h->status, sizeof(int))) != cudaSuccess)
        return bail(SCAFES_ERR_NOMEM, "cudaMalloc(status)", e);
    if ((e = cudaMemsetAsync(h->status, 0, sizeof(int), h->stream)) != cudaSuccess)
        return bail(SCAFES_ERR_CUDA, "cudaMemset(status)", e);
    if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess) return bail(SCAFES_ERR_CUDA, "cudaEventCreate", e);
    if ((e = cudaEventCreate(&h->ev1)) != cudaSuccess) return bail(SCAFES_ERR_CUDA, "cudaEventCreate", e);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    h->red_blocks = sms * 4;
    if ((e = cudaMalloc(&h->red, sizeof(double) * 2 * (h->red_blocks + 1))) != cudaSuccess)
        return bail(SCAFES_ERR_NOMEM, "cudaMalloc(scratch)", e);
    if ((e = cudaMallocHost(&h->red_host, sizeof(double) * 2)) != cudaSuccess)
        return bail(SCAFES_ERR_NOMEM, "cudaMallocHost", e);
    if ((e = cudaStreamSynchronize(h->stream)) != cudaSuccess) return bail(SCAFES_ERR_CUDA, "sync", e);
    *out = h;
    return SCAFES_OK;
}

// Exact-solution slots stay double (only the error check reads them);
// source and border slots use the element type of the unknown field.
static bool slot_is_double(int field) {
    return field == SCAFES_FIELD_E_A || field == SCAFES_FIELD_E_B ||
           (field >= SCAFES_FIELD_G_C && field <= SCAFES_FIELD_G_E);
}

// Copies the host image of the border table (rules, higher time orders of
// G, time basis) to the device, once the rules exist there.
static int sync_table(scafes_handle* h) {
    if (!h->table) return SCAFES_OK;
    CUDA_TRY(h, cudaMemcpyAsync(h->table, &h->table_host, sizeof(BorderTable), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

static int ensure_stage(scafes_handle* h) {
    if (h->stage) return SCAFES_OK;
    const size_t plane_elems = (size_t)h->L.nx * h->L.ny;
    size_t planes = kStageBytes / (plane_elems * sizeof(double));
    if (planes < 1) planes = 1;
    if (planes > (size_t)h->L.nz) planes = h->L.nz;
    h->stage_elems = planes * plane_elems;
    CUDA_TRY(h, cudaMalloc(&h->stage, h->stage_elems * sizeof(double)));
    return SCAFES_OK;
}

// host dense -> device field of element type `prec` (or double when prec < 0)
static int h2d(scafes_handle* h, void* dst, int prec, const double* host) {
    const Layout& L = h->L;
    if (prec == SCAFES_PREC_F64) {
        if (L.pitch == L.nx)  // unpadded rows: one contiguous copy
            CUDA_TRY(h, cudaMemcpyAsync(dst, host, (size_t)L.size() * sizeof(double), cudaMemcpyHostToDevice,
                                        h->stream));
        else
            CUDA_TRY(h, cudaMemcpy2DAsync(dst, (size_t)L.pitch * sizeof(double), host,
                                          (size_t)L.nx * sizeof(double), (size_t)L.nx * sizeof(double),
                                          (size_t)L.ny * L.nz, cudaMemcpyHostToDevice, h->stream));
        return SCAFES_OK;
    }
    int rc = ensure_stage(h);
    if (rc) return rc;
    const size_t plane_elems = (size_t)L.nx * L.ny;
    const int planes = (int)(h->stage_elems / plane_elems);
    const size_t esz = element_size(prec);
    for (int z0 = 0; z0 < L.nz; z0 += planes) {
        const int nzs = (z0 + planes <= L.nz) ? planes : L.nz - z0;
        CUDA_TRY(h, cudaMemcpyAsync(h->stage, host + (size_t)z0 * plane_elems,
                                    (size_t)nzs * plane_elems * sizeof(double),
                                    cudaMemcpyHostToDevice, h->stream));
        Layout S = L;
        S.nz = nzs;
        char* d = (char*)dst + (size_t)z0 * L.plane * esz;
        CUDA_TRY(h, convert_to_device(prec, h->stage, d, S, h->stream));
    }
    return SCAFES_OK;
}

static int d2h(scafes_handle* h, const void* src, int prec, double* host) {
    const Layout& L = h->L;
    if (prec == SCAFES_PREC_F64) {
        if (L.pitch == L.nx)
            CUDA_TRY(h, cudaMemcpyAsync(host, src, (size_t)L.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                        h->stream));
        else
            CUDA_TRY(h, cudaMemcpy2DAsync(host, (size_t)L.nx * sizeof(double), src,
                                          (size_t)L.pitch * sizeof(double), (size_t)L.nx * sizeof(double),
                                          (size_t)L.ny * L.nz, cudaMemcpyDeviceToHost, h->stream));
        return SCAFES_OK;
    }
    int rc = ensure_stage(h);
    if (rc) return rc;
    const size_t plane_elems = (size_t)L.nx * L.ny;
    const int planes = (int)(h->stage_elems / plane_elems);
    const size_t esz = element_size(prec);
    for (int z0 = 0; z0 < L.nz; z0 += planes) {
        const int nzs = (z0 + planes <= L.nz) ? planes : L.nz - z0;
        Layout S = L;
        S.nz = nzs;
        const char* s = (const char*)src + (size_t)z0 * L.plane * esz;
        CUDA_TRY(h, convert_from_device(prec, s, h->stage, S, h->stream));
        CUDA_TRY(h, cudaMemcpyAsync(host + (size_t)z0 * plane_elems, h->stage,
                                    (size_t)nzs * plane_elems * sizeof(double),
                                    cudaMemcpyDeviceToHost, h->stream));
    }
    return SCAFES_OK;
}

static size_t n_nodes(const scafes_handle* h) {
    return (size_t)h->L.nx * h->L.ny * h->L.nz;
}

// Reads (and clears) the kernels' status word after the stream drained: a
// bounded device wait that ran out is reported here instead of a hang.
static int check_status(scafes_handle* h) {
    int st = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&st, h->status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (st != 0) {
        cudaMemsetAsync(h->status, 0, sizeof(int), h->stream);
        return fail(&h->err, SCAFES_ERR_TIMEOUT,
                    "a sweep kernel gave up waiting for its TMA loads (status %d); results are invalid", st);
    }
    return SCAFES_OK;
}

extern "C" int scafes_gpu_upload(scafes_handle* h, int field, const double* host, size_t n) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_upload: handle is NULL");
    if (field < 0 || field >= SCAFES_FIELD_COUNT)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_upload: field %d out of range", field);
    if (!host || n != n_nodes(h))
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_upload: expected %zu values, got %zu%s",
                    n_nodes(h), n, host ? "" : " (NULL pointer)");
    int rc;
    if (field == SCAFES_FIELD_U) {
        rc = h2d(h, h->u[0], h->cfg.precision, host);
        if (rc) return rc;
        h->u0keep_valid = false;
        if (h->keep_initial) {
            if (!h->u0keep) CUDA_TRY(h, cudaMalloc(&h->u0keep, (size_t)h->L.size() * sizeof(double)));
            if ((rc = h2d(h, h->u0keep, SCAFES_PREC_F64, host))) return rc;
            h->u0keep_valid = true;
        }
        h->cur = 0;
        h->t = 0;
        h->uploaded = true;
    } else {
        const bool dbl = slot_is_double(field);
        const size_t esz = dbl ? sizeof(double) : h->esz;
        if (!h->fld[field]) {
            CUDA_TRY(h, cudaMalloc(&h->fld[field], (size_t)h->L.size() * esz));
            CUDA_TRY(h, cudaMemsetAsync(h->fld[field], 0, (size_t)h->L.size() * esz, h->stream));
        }
        rc = h2d(h, h->fld[field], dbl ? SCAFES_PREC_F64 : h->cfg.precision, host);
        if (rc) return rc;
        h->has[field] = true;
        if (field >= SCAFES_FIELD_G_C && field <= SCAFES_FIELD_G_E) {
            h->table_host.g_hi[field - SCAFES_FIELD_G_C] = (const double*)h->fld[field];
            rc = sync_table(h);
            if (rc) return rc;
        }
    }
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_gpu_download(scafes_handle* h, int field, double* host, size_t n) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_download: handle is NULL");
    if (field < 0 || field >= SCAFES_FIELD_COUNT)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_download: field %d out of range", field);
    if (!host || n != n_nodes(h))
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_download: expected %zu values, got %zu",
                    n_nodes(h), n);
    int rc;
    if (field == SCAFES_FIELD_U) {
        if (!h->uploaded)
            return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_download: the unknown field was never uploaded");
        rc = check_status(h);
        if (rc) return rc;
        rc = d2h(h, h->u[h->cur], h->cfg.precision, host);
    } else {
        if (!h->has[field])
            return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_download: slot %d was never uploaded", field);
        rc = d2h(h, h->fld[field], slot_is_double(field) ? SCAFES_PREC_F64 : h->cfg.precision, host);
    }
    if (rc) return rc;
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_gpu_upload_async(scafes_handle* h, const double* host, size_t n) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_upload_async: handle is NULL");
    if (!host || n != n_nodes(h))
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_upload_async: expected %zu values, got %zu%s",
                    n_nodes(h), n, host ? "" : " (NULL pointer)");
    if (h->keep_initial && !h->u0keep)
        CUDA_TRY(h, cudaMalloc(&h->u0keep, (size_t)h->L.size() * sizeof(double)));
    int rc = h2d(h, h->u[0], h->cfg.precision, host);
    if (rc) return rc;
    h->u0keep_valid = false;
    if (h->keep_initial) {
        if ((rc = h2d(h, h->u0keep, SCAFES_PREC_F64, host))) return rc;
        h->u0keep_valid = true;
    }
    h->cur = 0;
    h->t = 0;
    h->uploaded = true;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_download_async(scafes_handle* h, double* host, size_t n) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_download_async: handle is NULL");
    if (!host || n != n_nodes(h))
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_download_async: expected %zu values, got %zu",
                    n_nodes(h), n);
    if (!h->uploaded)
        return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_download_async: the unknown field was never uploaded");
    return d2h(h, h->u[h->cur], h->cfg.precision, host);
}

extern "C" int scafes_gpu_synchronize(scafes_handle* h) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_synchronize: handle is NULL");
    return check_status(h);
}

// TMA descriptor of buffer `buf` for tile variant `tile` (encoded on first use).
static const CUtensorMap* tensor_map(scafes_handle* h, int buf, int tile) {
    if (!h->tm_ok[buf][tile]) {
        CUresult r = make_tensor_map_3d(&h->tm[buf][tile], h->u[buf], (int)h->esz, h->L.nx, h->L.ny, h->L.nz,
                                        (size_t)h->L.pitch * h->esz, (size_t)h->L.plane * h->esz,
                                        star7_box_width(h->cfg.precision), star7_box_height(tile));
        if (r != CUDA_SUCCESS) {
            fail(&h->err, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
            return nullptr;
        }
        h->tm_ok[buf][tile] = true;
    }
    return &h->tm[buf][tile];
}

// TMA descriptor of the source F_A for tile variant `tile`: a 32 x BY box
// without halo (the F_A slot keeps its device buffer once uploaded).
static const CUtensorMap* source_map(scafes_handle* h, int tile) {
    if (!h->tmf_ok[tile]) {
        CUresult r = make_tensor_map_3d(&h->tmf[tile], h->fld[SCAFES_FIELD_F_A], (int)h->esz, h->L.nx, h->L.ny,
                                        h->L.nz, (size_t)h->L.pitch * h->esz, (size_t)h->L.plane * h->esz, BX,
                                        star7_box_height(tile) - 2);
        if (r != CUDA_SUCCESS) {
            fail(&h->err, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled (source) failed (%d)", (int)r);
            return nullptr;
        }
        h->tmf_ok[tile] = true;
    }
    return &h->tmf[tile];
}

// TMA descriptor of coefficient slot C0 (k = 0) or CA (k = 1) for tile
// variant `tile`: a 32 x BY box without halo, like the source.
static const CUtensorMap* coeff_map(scafes_handle* h, int k, int tile) {
    if (!h->tmc_ok[k][tile]) {
        CUresult r = make_tensor_map_3d(&h->tmc[k][tile], h->fld[k == 0 ? SCAFES_FIELD_C0 : SCAFES_FIELD_CA],
                                        (int)h->esz, h->L.nx, h->L.ny, h->L.nz, (size_t)h->L.pitch * h->esz,
                                        (size_t)h->L.plane * h->esz, BX, star7_box_height(tile) - 2);
        if (r != CUDA_SUCCESS) {
            fail(&h->err, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled (coefficients) failed (%d)", (int)r);
            return nullptr;
        }
        h->tmc_ok[k][tile] = true;
    }
    return &h->tmc[k][tile];
}

// Whether the handle runs the variable-coefficient update (C0 and CA uploaded).
static bool var_coeffs(const scafes_handle* h) {
    return h->has[SCAFES_FIELD_C0] && h->has[SCAFES_FIELD_CA];
}

// TMA descriptor of buffer `buf` for the depth-2 pass (encoded on first use).
static const CUtensorMap* tb_map(scafes_handle* h, int buf) {
    if (!h->tm_tb_ok[buf]) {
        int bw = 0, bh = 0;
        star7_tb_box(h->cfg.precision, &bw, &bh);
        CUresult r = make_tensor_map_3d(&h->tm_tb[buf], h->u[buf], (int)h->esz, h->L.nx, h->L.ny, h->L.nz,
                                        (size_t)h->L.pitch * h->esz, (size_t)h->L.plane * h->esz, bw, bh);
        if (r != CUDA_SUCCESS) {
            fail(&h->err, SCAFES_ERR_CUDA, "cuTensorMapEncodeTiled (depth 2) failed (%d)", (int)r);
            return nullptr;
        }
        h->tm_tb_ok[buf] = true;
    }
    return &h->tm_tb[buf];
}

static int step_impl(scafes_handle* h, int n_steps, int tile, bool timed, int depth) {
    if (h->L.nl != 1) tile = STAR7_MULTI_LAYER_TILE;  // the only variant built for several layers
    Star7Launch a;
    a.precision = h->cfg.precision;
    a.border = h->cfg.border;
    a.tile = tile;
    for (int b = 0; b < 2; ++b)
        if (!tensor_map(h, b, tile)) return SCAFES_ERR_CUDA;
    a.L = h->L;
    a.fa = h->has[SCAFES_FIELD_F_A] ? h->fld[SCAFES_FIELD_F_A] : nullptr;
    a.fb = h->has[SCAFES_FIELD_F_B] ? h->fld[SCAFES_FIELD_F_B] : nullptr;
    a.ga = h->has[SCAFES_FIELD_G_A] ? h->fld[SCAFES_FIELD_G_A] : nullptr;
    a.gb = h->has[SCAFES_FIELD_G_B] ? h->fld[SCAFES_FIELD_G_B] : nullptr;
    a.gconst = 0.0;
    a.c = make_star7_coeffs(h->cfg.c0, h->cfg.cp, h->cfg.cf);
    a.table = h->table;
    a.tm_f = nullptr;
    if (a.fa && !a.fb && h->cfg.cf != 0.0 && !(a.tm_f = source_map(h, tile))) return SCAFES_ERR_CUDA;
    if (!h->has[SCAFES_FIELD_F_A] && h->has[SCAFES_FIELD_F_B])
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_step: upload F_A (possibly zeros) when F_B is used");
    const bool g_hi = h->has[SCAFES_FIELD_G_C] || h->has[SCAFES_FIELD_G_D] || h->has[SCAFES_FIELD_G_E];
    if (h->cfg.border != SCAFES_BORDER_TABLE &&
        (g_hi || h->table_host.t_center != 0.0 || h->table_host.t_rate != 1.0))
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_step: higher time orders of G (slots G_C..G_E) or another time basis need "
                    "SCAFES_BORDER_TABLE; this border reads G = G_A + time*G_B");
    if (h->cfg.border == SCAFES_BORDER_TABLE) {
        if (!h->table)
            return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_step: set the border rules first "
                                                   "(scafes_gpu_set_border_forms)");
        if (h->table_needs_f && (a.fa == nullptr || h->cfg.cf == 0.0))
            return fail(&h->err, SCAFES_ERR_STATE,
                        "scafes_gpu_step: a border rule reads the source F, but no F_A is uploaded or cf == 0");
    }
    a.vc = var_coeffs(h);
    if (h->has[SCAFES_FIELD_C0] != h->has[SCAFES_FIELD_CA])
        return fail(&h->err, SCAFES_ERR_STATE,
                    "scafes_gpu_step: the variable-coefficient update needs both slots C0 and CA uploaded");
    if (h->cfg.border == SCAFES_BORDER_NODES) {
        if (!a.vc)
            return fail(&h->err, SCAFES_ERR_STATE,
                        "scafes_gpu_step: per-node border rules need the coefficient slots C0 and CA");
        if (!h->nodes)
            return fail(&h->err, SCAFES_ERR_STATE,
                        "scafes_gpu_step: set the per-node border rules first (scafes_gpu_set_border_node_rules)");
        a.nodes = h->nodes;
    }
    if (a.vc) {
        if (h->cfg.precision == SCAFES_PREC_F32X2)
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_step: the variable-coefficient update runs in F64 or F32, not F32X2");
        if (h->L.nl != 1)
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_step: the variable-coefficient update takes one border layer");
        if (a.fb)
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_step: the variable-coefficient update takes a static source (no F_B)");
        if (a.fa && h->cfg.cf != 0.0 && h->cfg.cf != 1.0)
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_step: with variable coefficients the source enters with cf = 1 (fold other "
                        "factors into F_A) or cf = 0");
        if (h->cfg.border == SCAFES_BORDER_MIRROR_POW2)
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_step: the variable-coefficient update takes the Dirichlet, table or per-node border");
        if (!(a.tm_c0 = coeff_map(h, 0, tile)) || !(a.tm_ca = coeff_map(h, 1, tile))) return SCAFES_ERR_CUDA;
    }
    a.tm_tb = nullptr;
    const bool tb = depth == 2 && star7_tb_eligible(a);
    if (tb)
        for (int b = 0; b < 2; ++b)
            if (!tb_map(h, b)) return SCAFES_ERR_CUDA;
    if (timed) CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream));
    a.status = h->status;
    int launches = 0;
    for (int s = 0; s < n_steps;) {
        a.tm_uo = &h->tm[h->cur][tile];
        a.uo = h->u[h->cur];
        a.un = h->u[h->cur ^ 1];
        a.time_old = h->cfg.t_start + h->t * h->cfg.tau;          // time(t)
        a.time_new = h->cfg.t_start + (h->t + 1) * h->cfg.tau;    // time(t+1)
        a.time_new2 = h->cfg.t_start + (h->t + 2) * h->cfg.tau;   // time(t+2)
        a.mirror_corr = ldexp(1.0, h->t);                          // 2^(t_new - 1)
        const int adv = (tb && n_steps - s >= 2) ? 2 : 1;
        a.tm_tb = adv == 2 ? &h->tm_tb[h->cur] : nullptr;
        cudaError_t e = adv == 2 ? launch_star7_tb(a, h->stream) : launch_star7(a, h->stream);
        if (e != cudaSuccess)
            return fail(&h->err, SCAFES_ERR_CUDA, "scafes_gpu_step: launch failed: %s", cudaGetErrorString(e));
        h->cur ^= 1;
        h->t += adv;
        s += adv;
        ++launches;
    }
    if (timed) {
        CUDA_TRY(h, cudaEventRecord(h->ev1, h->stream));
        h->timed = true;
        h->launches = launches;
    }
    return SCAFES_OK;
}

extern "C" int scafes_gpu_inject_status(scafes_handle* h, int code) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_inject_status: handle is NULL");
    if (code > 0) return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_inject_status: code %d > 0", code);
    CUDA_TRY(h, cudaMemcpyAsync(h->status, &code, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_gpu_set_temporal_depth(scafes_handle* h, int depth) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_set_temporal_depth: handle is NULL");
    if (depth != 1 && depth != 2)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_set_temporal_depth: depth %d (1 or 2)", depth);
    h->depth = depth;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_temporal_depth(const scafes_handle* h, int* depth) {
    if (!h || !depth) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_temporal_depth: NULL argument");
    Star7Launch a;
    a.border = h->cfg.border;
    a.L = h->L;
    a.fb = h->has[SCAFES_FIELD_F_B] ? h->fld[SCAFES_FIELD_F_B] : nullptr;
    a.vc = var_coeffs(h);
    *depth = (h->depth == 2 && star7_tb_eligible(a)) ? 2 : 1;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_set_border_forms(scafes_handle* h, const scafes_border_form forms[64]) {
    if (!h || !forms) return fail(h ? &h->err : nullptr, SCAFES_ERR_ARG, "scafes_gpu_set_border_forms: NULL argument");
    if (h->cfg.border != SCAFES_BORDER_TABLE)
        return fail(&h->err, SCAFES_ERR_STATE,
                    "scafes_gpu_set_border_forms: the problem was created with border kind %d, not "
                    "SCAFES_BORDER_TABLE", h->cfg.border);
    // A weight on a neighbour that a class's nodes do not have would read
    // the zero halo silently: refuse it.
    bool needs_f = false;
    for (int m = 1; m < SCAFES_BORDER_CLASSES; ++m) {
        for (int d = 0; d < 6; ++d)
            if ((m >> d) & 1 && forms[m].cn[d] != 0.0)
                return fail(&h->err, SCAFES_ERR_ARG,
                            "scafes_gpu_set_border_forms: class %d weights neighbour %d, which lies outside the grid",
                            m, d);
        if ((m & 3) == 3 || (m & 12) == 12 || (m & 48) == 48)
            continue;  // a node cannot be on both faces of an axis (n >= 3)
        needs_f = needs_f || forms[m].cf != 0.0;
    }
    // With more than one border layer, class 0 is the rule of the border
    // nodes that lie on no face.
    if (h->L.nl > 1) needs_f = needs_f || forms[0].cf != 0.0;
    if (!h->table) CUDA_TRY(h, cudaMalloc(&h->table, sizeof(BorderTable)));
    std::memcpy(h->table_host.rule, forms, sizeof(scafes_border_form) * SCAFES_BORDER_CLASSES);
    const int rc = sync_table(h);
    if (rc) return rc;
    h->table_needs_f = needs_f;
    return SCAFES_OK;
}

extern "C" int scafes_border_node_count(const scafes_cfg* cfg, long long* count) {
    if (!cfg || !count) return fail(nullptr, SCAFES_ERR_ARG, "scafes_border_node_count: NULL argument");
    const int nl = cfg->n_layers_at_border;
    for (int p = 0; p < 3; ++p)
        if (cfg->n_nodes[p] < 3 || nl < 1 || 2 * nl > cfg->n_nodes[p])
            return fail(nullptr, SCAFES_ERR_ARG, "scafes_border_node_count: n_nodes / n_layers_at_border out of range");
    *count = border_node_count(cfg->n_nodes[0], cfg->n_nodes[1], cfg->n_nodes[2], nl);
    return SCAFES_OK;
}

extern "C" int scafes_gpu_set_border_node_rules(scafes_handle* h, const scafes_border_node_rule* rules, size_t n) {
    if (!h || !rules)
        return fail(h ? &h->err : nullptr, SCAFES_ERR_ARG, "scafes_gpu_set_border_node_rules: NULL argument");
    if (h->cfg.border != SCAFES_BORDER_NODES)
        return fail(&h->err, SCAFES_ERR_STATE,
                    "scafes_gpu_set_border_node_rules: the problem was created with border kind %d, not "
                    "SCAFES_BORDER_NODES", h->cfg.border);
    const long long count = border_node_count(h->L.nx, h->L.ny, h->L.nz, h->L.nl);
    if ((long long)n != count)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_set_border_node_rules: expected %lld rules, got %zu", count,
                    n);
    // A weight on a neighbour outside the grid would read the zero halo
    // silently: refuse it (faces in direction order x-, x+, y-, y+, z-, z+).
    long long r = 0;
    for (int z = 0; z < h->L.nz; ++z)
        for (int y = 0; y < h->L.ny; ++y)
            for (int x = 0; x < h->L.nx; ++x) {
                const bool inner = x > 0 && x < h->L.nx - 1 && y > 0 && y < h->L.ny - 1 && z > 0 && z < h->L.nz - 1;
                if (inner) continue;
                const bool out[6] = {x == 0, x == h->L.nx - 1, y == 0, y == h->L.ny - 1, z == 0, z == h->L.nz - 1};
                for (int d = 0; d < 6; ++d)
                    if (out[d] && rules[r].cn[d] != 0.0)
                        return fail(&h->err, SCAFES_ERR_ARG,
                                    "scafes_gpu_set_border_node_rules: the rule of node (%d,%d,%d) weights neighbour "
                                    "%d, which lies outside the grid", x, y, z, d);
                ++r;
            }
    if (!h->nodes) CUDA_TRY(h, cudaMalloc(&h->nodes, (size_t)count * sizeof(scafes_border_node_rule)));
    if (h->cfg.precision == SCAFES_PREC_F32) {
        // The FP32 sweep evaluates the rules in FP32: 8 floats per node
        // (cu, cn[0..5], cst) in the same allocation.
        std::vector<float> f((size_t)count * 8);
        for (long long i = 0; i < count; ++i) {
            f[i * 8] = (float)rules[i].cu;
            for (int d = 0; d < 6; ++d) f[i * 8 + 1 + d] = (float)rules[i].cn[d];
            f[i * 8 + 7] = (float)rules[i].cst;
        }
        CUDA_TRY(h, cudaMemcpyAsync(h->nodes, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice,
                                    h->stream));
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        return SCAFES_OK;
    }
    CUDA_TRY(h, cudaMemcpyAsync(h->nodes, rules, (size_t)count * sizeof(scafes_border_node_rule),
                                cudaMemcpyHostToDevice, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_gpu_set_border_time_basis(scafes_handle* h, double t_center, double t_rate) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_set_border_time_basis: handle is NULL");
    if (!std::isfinite(t_center) || !std::isfinite(t_rate) || t_rate == 0.0)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_set_border_time_basis: t_center=%g, t_rate=%g", t_center,
                    t_rate);
    h->table_host.t_center = t_center;
    h->table_host.t_rate = t_rate;
    return sync_table(h);
}

extern "C" int scafes_border_forms_flux(const scafes_cfg* cfg, int kind, double lambda, double alpha,
                                        scafes_border_form forms[64]) {
    if (!cfg || !forms || cfg->dim != 3 || lambda == 0.0)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_border_forms_flux: bad arguments");
    if (kind != SCAFES_FLUX_NEUMANN && kind != SCAFES_FLUX_CAUCHY && kind != SCAFES_FLUX_RADIATION)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_border_forms_flux: kind %d", kind);
    double h[3];
    for (int p = 0; p < 3; ++p) {
        if (cfg->n_nodes[p] < 3) return fail(nullptr, SCAFES_ERR_ARG, "scafes_border_forms_flux: n_nodes[%d] < 3", p);
        h[p] = (cfg->coord_last[p] - cfg->coord_first[p]) / (cfg->n_nodes[p] - 1);
    }
    for (int m = 0; m < SCAFES_BORDER_CLASSES; ++m) {
        scafes_border_form& F = forms[m];
        F = scafes_border_form{};
        // Class 0 (border nodes on no face, n_layers_at_border > 1) takes
        // the branch of the max-face classes with no face: the inner update.
        if (m & (1 | 4 | 16)) {  // on a min face: Dirichlet (the "index 0" branch of Neumann.hpp, Cauchy.hpp, Radiation.hpp)
            F.cg_new = 1.0;
            continue;
        }
        // Max faces only: the inner update, with the missing neighbour of each
        // max-face direction replaced by the inner one plus the flux term.
        F.cu = cfg->c0;
        F.cf = cfg->cf;
        for (int p = 0; p < 3; ++p) {
            const bool on_max = (m >> (2 * p + 1)) & 1;
            if (on_max) {
                F.cn[2 * p] = 2.0 * cfg->cp[p];
                const double flux = cfg->cp[p] * (2.0 * h[p] / lambda);
                if (kind == SCAFES_FLUX_NEUMANN) {
                    F.cg_old -= flux;
                } else if (kind == SCAFES_FLUX_CAUCHY) {
                    F.cu -= flux * alpha;
                    F.cg_old += flux;
                } else {
                    F.cu4 -= flux * alpha;
                    F.cg_old += flux;
                }
            } else {
                F.cn[2 * p] = cfg->cp[p];
                F.cn[2 * p + 1] = cfg->cp[p];
            }
        }
    }
    return SCAFES_OK;
}

extern "C" int scafes_gpu_step(scafes_handle* h, int n_steps) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_step: handle is NULL");
    if (n_steps < 0) return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_step: n_steps=%d < 0", n_steps);
    if (!h->uploaded)
        return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_step: upload the unknown field first");
    return step_impl(h, n_steps, h->tile, true, h->depth);
}

// ---- snapshots ----------------------------------------------------------------

namespace {

const char kSnapMagic[8] = {'S', 'C', 'A', 'F', 'E', 'S', 'S', '1'};

struct SnapHeader {
    char magic[8];
    int32_t version;
    int32_t n[3];
    int32_t reserved[2];
};

struct SnapRecord {
    int64_t step;
    double time;
};

int snap_setup(scafes_handle* h) {
    if (h->snap_dev) return SCAFES_OK;
    const size_t bytes = n_nodes(h) * sizeof(double);
    CUDA_TRY(h, cudaMalloc(&h->snap_dev, bytes));
    for (int i = 0; i < 2; ++i) {
        CUDA_TRY(h, cudaMallocHost(&h->snap_host[i], bytes));
        CUDA_TRY(h, cudaEventCreateWithFlags(&h->snap_copied[i], cudaEventDisableTiming));
    }
    CUDA_TRY(h, cudaEventCreateWithFlags(&h->snap_conv, cudaEventDisableTiming));
    CUDA_TRY(h, cudaStreamCreateWithFlags(&h->snap_stream, cudaStreamNonBlocking));
    return SCAFES_OK;
}

// Enqueues the copy of the current iterate into pinned buffer b: dense FP64
// on the device (on the compute stream, after the previous copy out of the
// device buffer finished), then device -> host on the copy stream.
int snap_enqueue(scafes_handle* h, int b, int prev) {
    const Layout& L = h->L;
    if (prev >= 0) CUDA_TRY(h, cudaStreamWaitEvent(h->stream, h->snap_copied[prev], 0));
    if (h->cfg.precision == SCAFES_PREC_F64)
        CUDA_TRY(h, cudaMemcpy2DAsync(h->snap_dev, (size_t)L.nx * sizeof(double), h->u[h->cur],
                                      (size_t)L.pitch * sizeof(double), (size_t)L.nx * sizeof(double),
                                      (size_t)L.ny * L.nz, cudaMemcpyDeviceToDevice, h->stream));
    else
        CUDA_TRY(h, convert_from_device(h->cfg.precision, h->u[h->cur], h->snap_dev, L, h->stream));
    CUDA_TRY(h, cudaEventRecord(h->snap_conv, h->stream));
    CUDA_TRY(h, cudaStreamWaitEvent(h->snap_stream, h->snap_conv, 0));
    CUDA_TRY(h, cudaMemcpyAsync(h->snap_host[b], h->snap_dev, n_nodes(h) * sizeof(double), cudaMemcpyDeviceToHost,
                                h->snap_stream));
    CUDA_TRY(h, cudaEventRecord(h->snap_copied[b], h->snap_stream));
    return SCAFES_OK;
}

// Waits for pinned buffer b and appends it to the file.
int snap_write(scafes_handle* h, FILE* f, int b, long long step) {
    CUDA_TRY(h, cudaEventSynchronize(h->snap_copied[b]));
    SnapRecord r{(int64_t)step, h->cfg.t_start + step * h->cfg.tau};
    const size_t n = n_nodes(h);
    if (std::fwrite(&r, sizeof(r), 1, f) != 1 || std::fwrite(h->snap_host[b], sizeof(double), n, f) != n)
        return fail(&h->err, SCAFES_ERR_IO, "scafes_gpu_step_snapshots: writing the snapshot of step %lld failed",
                    step);
    return SCAFES_OK;
}

}  // namespace

extern "C" int scafes_gpu_step_snapshots(scafes_handle* h, int n_steps, int interval, int flags, const char* path) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_step_snapshots: handle is NULL");
    if (n_steps < 0 || interval < 0 || !path)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_step_snapshots: bad arguments");
    if (!h->uploaded)
        return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_step_snapshots: upload the unknown field first");
    int rc = snap_setup(h);
    if (rc) return rc;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(&h->err, SCAFES_ERR_IO, "scafes_gpu_step_snapshots: cannot open %s for writing", path);
    SnapHeader hd{};
    std::memcpy(hd.magic, kSnapMagic, sizeof(kSnapMagic));
    hd.version = 1;
    hd.n[0] = h->L.nx; hd.n[1] = h->L.ny; hd.n[2] = h->L.nz;
    if (std::fwrite(&hd, sizeof(hd), 1, f) != 1) {
        std::fclose(f);
        return fail(&h->err, SCAFES_ERR_IO, "scafes_gpu_step_snapshots: cannot write %s", path);
    }
    // Snapshot points: the current step (START), every step t with
    // t % interval == 0 (the reference's nTimesteps/nSnapshots rule), the
    // last step (END).  A snapshot is written while the next steps run.
    const long long t0 = h->t, t1 = h->t + (long long)n_steps;
    int pending = -1, b = 0;
    long long pending_step = 0, done = t0;
    CUDA_TRY(h, cudaEventRecord(h->ev0, h->stream));
    auto snap = [&](long long t) -> int {
        int r = snap_enqueue(h, b, pending);
        if (r == SCAFES_OK && pending >= 0) r = snap_write(h, f, pending, pending_step);
        pending = b;
        pending_step = t;
        b ^= 1;
        return r;
    };
    if (flags & SCAFES_SNAP_START) rc = snap(t0);
    for (long long t = t0 + 1; t <= t1 && rc == SCAFES_OK; ++t) {
        const bool at = (interval > 0 && t % interval == 0) || (t == t1 && (flags & SCAFES_SNAP_END));
        if (!at) continue;
        rc = step_impl(h, (int)(t - done), h->tile, false, h->depth);
        done = t;
        if (rc == SCAFES_OK) rc = snap(t);
    }
    if (rc == SCAFES_OK && done < t1) rc = step_impl(h, (int)(t1 - done), h->tile, false, h->depth);
    if (rc == SCAFES_OK) {
        cudaError_t e = cudaEventRecord(h->ev1, h->stream);
        if (e != cudaSuccess) rc = fail(&h->err, SCAFES_ERR_CUDA, "scafes_gpu_step_snapshots: %s", cudaGetErrorString(e));
    }
    if (rc == SCAFES_OK && pending >= 0) rc = snap_write(h, f, pending, pending_step);
    if (std::fclose(f) != 0 && rc == SCAFES_OK)
        rc = fail(&h->err, SCAFES_ERR_IO, "scafes_gpu_step_snapshots: closing %s failed", path);
    if (rc) return rc;
    h->timed = true;
    h->launches = n_steps;
    return check_status(h);
}

extern "C" int scafes_snapshot_info(const char* path, int n_nodes_out[3], int* count) {
    if (!path || !n_nodes_out || !count) return fail(nullptr, SCAFES_ERR_ARG, "scafes_snapshot_info: NULL argument");
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(nullptr, SCAFES_ERR_IO, "scafes_snapshot_info: cannot open %s", path);
    SnapHeader hd{};
    const bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, kSnapMagic, 8) == 0 &&
                    hd.version == 1 && hd.n[0] > 0 && hd.n[1] > 0 && hd.n[2] > 0;
    long long size = -1;
    if (ok && std::fseek(f, 0, SEEK_END) == 0) size = std::ftell(f);
    std::fclose(f);
    if (!ok || size < 0) return fail(nullptr, SCAFES_ERR_IO, "scafes_snapshot_info: %s is not a snapshot file", path);
    const long long rec = (long long)sizeof(SnapRecord) + (long long)hd.n[0] * hd.n[1] * hd.n[2] * 8;
    for (int p = 0; p < 3; ++p) n_nodes_out[p] = hd.n[p];
    *count = (int)((size - (long long)sizeof(hd)) / rec);
    return SCAFES_OK;
}

extern "C" int scafes_snapshot_read(const char* path, int index, double* host, size_t n, long long* step,
                                    double* time) {
    int nn[3], count = 0;
    int rc = scafes_snapshot_info(path, nn, &count);
    if (rc) return rc;
    const size_t total = (size_t)nn[0] * nn[1] * nn[2];
    if (!host || n != total)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_snapshot_read: expected %zu values, got %zu", total, n);
    if (index < 0 || index >= count)
        return fail(nullptr, SCAFES_ERR_ARG, "scafes_snapshot_read: index %d out of [0, %d)", index, count);
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(nullptr, SCAFES_ERR_IO, "scafes_snapshot_read: cannot open %s", path);
    const long long off = (long long)sizeof(SnapHeader) + (long long)index * ((long long)sizeof(SnapRecord) + 8LL * total);
    SnapRecord r{};
    const bool ok = std::fseek(f, off, SEEK_SET) == 0 && std::fread(&r, sizeof(r), 1, f) == 1 &&
                    std::fread(host, sizeof(double), total, f) == total;
    std::fclose(f);
    if (!ok) return fail(nullptr, SCAFES_ERR_IO, "scafes_snapshot_read: %s is truncated", path);
    if (step) *step = r.step;
    if (time) *time = r.time;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_autotune(scafes_handle* h, int n_steps, int* chosen, float* ms_per_tile) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_autotune: handle is NULL");
    if (n_steps < 1) return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_autotune: n_steps=%d < 1", n_steps);
    if (!h->uploaded)
        return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_autotune: upload the unknown field first");
    // Trial steps run on a copy: the iterate and the step counter are
    // restored afterwards.
    const size_t bytes = (size_t)h->L.size() * h->esz;
    void* save = nullptr;
    CUDA_TRY(h, cudaMalloc(&save, bytes));
    const int t_save = h->t, cur_save = h->cur;
    cudaError_t e = cudaMemcpyAsync(save, h->u[h->cur], bytes, cudaMemcpyDeviceToDevice, h->stream);
    int best = h->tile, rc = SCAFES_OK;
    float best_ms = 0.f;
    for (int tile = 0; tile < STAR7_NUM_TILES && e == cudaSuccess && rc == SCAFES_OK; ++tile) {
        rc = step_impl(h, 1, tile, false, 1);  // warm-up (and first-use setup)
        if (rc == SCAFES_OK) rc = step_impl(h, n_steps, tile, true, 1);
        float ms = 0.f;
        if (rc == SCAFES_OK) {
            e = cudaEventSynchronize(h->ev1);
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, h->ev0, h->ev1);
        }
        if (ms_per_tile) ms_per_tile[tile] = ms / n_steps;
        if (rc == SCAFES_OK && e == cudaSuccess && (tile == 0 || ms < best_ms)) {
            best_ms = ms;
            best = tile;
        }
    }
    // Temporal blocking: depth 2 (its own tile) against the best depth-1 tile.
    int best_depth = 1;
    int dep = 0;
    const int n2 = n_steps + (n_steps & 1);
    if (e == cudaSuccess && rc == SCAFES_OK && scafes_gpu_temporal_depth(h, &dep) == SCAFES_OK) {
        const int keep = h->depth;
        h->depth = 2;
        if (scafes_gpu_temporal_depth(h, &dep) == SCAFES_OK && dep == 2) {
            rc = step_impl(h, 2, best, false, 2);
            if (rc == SCAFES_OK) rc = step_impl(h, n2, best, true, 2);
            float ms = 0.f;
            if (rc == SCAFES_OK) {
                e = cudaEventSynchronize(h->ev1);
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, h->ev0, h->ev1);
            }
            // Keep depth 2 only when it is clearly faster (3 %), so that
            // timing noise does not flip the choice between runs.
            if (rc == SCAFES_OK && e == cudaSuccess && ms / n2 < 0.97f * best_ms / n_steps) best_depth = 2;
        }
        h->depth = keep;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h->u[cur_save], save, bytes, cudaMemcpyDeviceToDevice, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    cudaFree(save);
    h->t = t_save;
    h->cur = cur_save;
    h->timed = false;
    if (rc != SCAFES_OK) return rc;
    if (e != cudaSuccess)
        return fail(&h->err, SCAFES_ERR_CUDA, "scafes_gpu_autotune: %s", cudaGetErrorString(e));
    rc = check_status(h);
    if (rc) return rc;
    h->tile = best;
    h->depth = best_depth;
    if (chosen) *chosen = best + 1;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_timestep(const scafes_handle* h, int* t) {
    if (!h || !t) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_timestep: NULL argument");
    *t = h->t;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_last_step_ms(const scafes_handle* h, float* ms) {
    if (!h || !ms) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_last_step_ms: NULL argument");
    if (!h->timed) return fail(nullptr, SCAFES_ERR_STATE, "scafes_gpu_last_step_ms: no step yet");
    cudaError_t e = cudaEventSynchronize(h->ev1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(ms, h->ev0, h->ev1);
    if (e != cudaSuccess)
        return fail(nullptr, SCAFES_ERR_CUDA, "scafes_gpu_last_step_ms: %s", cudaGetErrorString(e));
    return SCAFES_OK;
}

extern "C" int scafes_gpu_last_step_launches(const scafes_handle* h, int* launches) {
    if (!h || !launches) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_last_step_launches: NULL argument");
    *launches = h->launches;
    return SCAFES_OK;
}

// ---- L-infinity error (DataField::compErrLinf) -------------------------------

template <class T>
__device__ __forceinline__ double load_as_double(const T* p, long long o);
template <>
__device__ __forceinline__ double load_as_double<double>(const double* p, long long o) { return p[o]; }
template <>
__device__ __forceinline__ double load_as_double<float>(const float* p, long long o) { return (double)p[o]; }
template <>
__device__ __forceinline__ double load_as_double<float2>(const float2* p, long long o) {
    float2 v = p[o];
    return join_pair(v.x, v.y);
}

__device__ __forceinline__ double nan_to_inf(double d) { return (d != d) ? __longlong_as_double(0x7ff0000000000000LL) : d; }

// Pass 1: per-CTA maxima of |u - E| and |E| into part[2*blockIdx.x + {0,1}].
template <class T>
__global__ void k_err_partial(const T* __restrict__ u, const double* __restrict__ ea,
                              const double* __restrict__ eb, double time, Layout L,
                              double* __restrict__ part) {
    __shared__ double s_err[8], s_ref[8];
    double me = 0.0, mr = 0.0;
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % L.nx);
        const long long r = m / L.nx;
        const long long o = L.idx(i, (int)(r % L.ny), (int)(r / L.ny));
        double e = ea ? ea[o] : 0.0;
        if (eb) e += time * eb[o];
        const double d = nan_to_inf(fabs(load_as_double<T>(u, o) - e));
        me = fmax(me, d);
        mr = fmax(mr, fabs(e));
    }
    for (int s = 16; s > 0; s >>= 1) {
        me = fmax(me, __shfl_down_sync(0xffffffffu, me, s));
        mr = fmax(mr, __shfl_down_sync(0xffffffffu, mr, s));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { s_err[w] = me; s_ref[w] = mr; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { me = fmax(me, s_err[k]); mr = fmax(mr, s_ref[k]); }
        part[2 * blockIdx.x] = me;
        part[2 * blockIdx.x + 1] = mr;
    }
}

// Pass 2: one CTA folds the partial maxima into out[0..1].
__global__ void k_err_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    double me = 0.0, mr = 0.0;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        me = fmax(me, part[2 * k]);
        mr = fmax(mr, part[2 * k + 1]);
    }
    for (int s = 16; s > 0; s >>= 1) {
        me = fmax(me, __shfl_down_sync(0xffffffffu, me, s));
        mr = fmax(mr, __shfl_down_sync(0xffffffffu, mr, s));
    }
    __shared__ double s_err[32], s_ref[32];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { s_err[w] = me; s_ref[w] = mr; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) { me = fmax(me, s_err[k]); mr = fmax(mr, s_ref[k]); }
        out[0] = me;
        out[1] = mr;
    }
}

extern "C" int scafes_gpu_err_linf(scafes_handle* h, double* err, double* max_ref) {
    if (!h || !err || !max_ref) return fail(h ? &h->err : nullptr, SCAFES_ERR_ARG, "scafes_gpu_err_linf: NULL argument");
    if (!h->uploaded) return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_err_linf: upload the unknown field first");
    const double* ea = h->has[SCAFES_FIELD_E_A] ? (const double*)h->fld[SCAFES_FIELD_E_A] : nullptr;
    const double* eb = h->has[SCAFES_FIELD_E_B] ? (const double*)h->fld[SCAFES_FIELD_E_B] : nullptr;
    const double time = h->cfg.t_start + h->t * h->cfg.tau;
    double* part = h->red;
    double* out = h->red + 2 * h->red_blocks;
    const void* u = h->u[h->cur];
    switch (h->cfg.precision) {
        case SCAFES_PREC_F64: k_err_partial<double><<<h->red_blocks, 256, 0, h->stream>>>((const double*)u, ea, eb, time, h->L, part); break;
        case SCAFES_PREC_F32: k_err_partial<float><<<h->red_blocks, 256, 0, h->stream>>>((const float*)u, ea, eb, time, h->L, part); break;
        default: k_err_partial<float2><<<h->red_blocks, 256, 0, h->stream>>>((const float2*)u, ea, eb, time, h->L, part); break;
    }
    CUDA_TRY(h, cudaGetLastError());
    k_err_final<<<1, 1024, 0, h->stream>>>(part, h->red_blocks, out);
    CUDA_TRY(h, cudaGetLastError());
    CUDA_TRY(h, cudaMemcpyAsync(h->red_host, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    *err = h->red_host[0];
    *max_ref = h->red_host[1];
    return check_status(h);
}

// ---- backward entry -------------------------------------------------------

// Counts the global-border nodes where the initial iterate differs from the
// Dirichlet value G_A (0 where G_A was not uploaded).  With pairs, G_A holds
// FP32 pairs and the iterate is compared as the pair it becomes.
__global__ void k_border_mismatch(const double* __restrict__ u0, const void* __restrict__ ga, int pairs, Layout L,
                                  int* __restrict__ count) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= L.nx || y >= L.ny) return;
    const bool colb = x == 0 || y == 0 || x == L.nx - 1 || y == L.ny - 1;
    int bad = 0;
    for (int z = 0; z < L.nz; ++z) {
        if (!colb && z != 0 && z != L.nz - 1) continue;
        const long long o = L.idx(x, y, z);
        double u = u0[o], g = 0.0;
        if (pairs) {
            const f2 p = split_double(u);
            u = (double)p.hi + (double)p.lo;
            if (ga) g = (double)((const float2*)ga)[o].x + (double)((const float2*)ga)[o].y;
        } else if (ga) {
            g = ((const double*)ga)[o];
        }
        bad += u != g;
    }
    if (bad) atomicAdd(count, bad);
}

extern "C" int scafes_gpu_keep_initial(scafes_handle* h, int on) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_keep_initial: handle is NULL");
    h->keep_initial = on != 0;
    if (!h->keep_initial) {
        CUDA_TRY(h, cudaStreamSynchronize(h->stream));
        cudaFree(h->u0keep);
        h->u0keep = nullptr;
        h->u0keep_valid = false;
    }
    return SCAFES_OK;
}

extern "C" int scafes_gpu_adjoint(scafes_handle* h, const double* dJ_du_T, double* dJ_dk, double* dJ_du0,
                                  int n_checkpoints) {
    if (!h) return fail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_adjoint: handle is NULL");
    if (!dJ_du_T || !dJ_dk || !dJ_du0) return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_adjoint: NULL array");
    if (h->has[SCAFES_FIELD_C0] || h->has[SCAFES_FIELD_CA])
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_adjoint: problems with coefficient fields are not covered");
    if (n_checkpoints < 2)
        return fail(&h->err, SCAFES_ERR_ARG, "scafes_gpu_adjoint: n_checkpoints = %d (at least 2)", n_checkpoints);
    const scafes_cfg& c = h->cfg;
    if (c.precision != SCAFES_PREC_F64 && c.precision != SCAFES_PREC_F32X2)
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_adjoint: precision %d (F64 or F32X2 only)",
                    c.precision);
    if (c.border != SCAFES_BORDER_DIRICHLET || c.n_layers_at_border != 1)
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_adjoint: the Dirichlet border with one border layer only");
    if (h->has[SCAFES_FIELD_G_B])
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_adjoint: the border value must not depend on time");
    if (c.cf != 0.0 && (h->has[SCAFES_FIELD_F_A] || h->has[SCAFES_FIELD_F_B]))
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_adjoint: problems with a source are not covered");
    // The inner update must be the heat form c0 = 1 - 2 sum cp, cp[p] = tau a / h_p^2: then it is the flux form
    // with the uniform conductivity a.
    double a = 0.0, sum_cp = 0.0;
    for (int p = 0; p < 3; ++p) {
        const double hp = (c.coord_last[p] - c.coord_first[p]) / (c.n_nodes[p] - 1);
        const double ap = c.cp[p] * hp * hp / c.tau;
        if (p == 0) a = ap;
        else if (std::fabs(ap - a) > 1e-12 * std::fabs(a))
            return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                        "scafes_gpu_adjoint: cp[%d] is not tau*a/h^2 for the a of cp[0] (anisotropic heat)", p);
        sum_cp += c.cp[p];
    }
    if (!(a > 0.0) || std::fabs(c.c0 - (1.0 - 2.0 * sum_cp)) > 1e-12)
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_adjoint: the inner update is not the heat form (c0 = 1 - 2 sum cp, a > 0)");
    if (!h->u0keep_valid)
        return fail(&h->err, SCAFES_ERR_STATE,
                    "scafes_gpu_adjoint: call scafes_gpu_keep_initial(h, 1) before uploading the initial iterate");
    if (h->t < 1) return fail(&h->err, SCAFES_ERR_STATE, "scafes_gpu_adjoint: no step since the upload");
    // The border is held at the initial iterate's values: they must be the Dirichlet value.
    if (!h->mismatch) CUDA_TRY(h, cudaMalloc(&h->mismatch, sizeof(int)));
    CUDA_TRY(h, cudaMemsetAsync(h->mismatch, 0, sizeof(int), h->stream));
    const void* ga = h->has[SCAFES_FIELD_G_A] ? h->fld[SCAFES_FIELD_G_A] : nullptr;
    const dim3 blk(32, 8), grd((h->L.nx + 31) / 32, (h->L.ny + 7) / 8);
    k_border_mismatch<<<grd, blk, 0, h->stream>>>(h->u0keep, ga, c.precision == SCAFES_PREC_F32X2, h->L,
                                                  h->mismatch);
    CUDA_TRY(h, cudaGetLastError());
    int bad = 0;
    CUDA_TRY(h, cudaMemcpyAsync(&bad, h->mismatch, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    if (bad)
        return fail(&h->err, SCAFES_ERR_UNSUPPORTED,
                    "scafes_gpu_adjoint: %d border nodes of the initial iterate differ from the Dirichlet value", bad);
    if (!h->adj || h->adj_snaps != n_checkpoints || h->adj_prec != c.precision) {
        scafes_adj_destroy(h->adj);
        h->adj = nullptr;
        int rc = scafes_adj_create(c.n_nodes, c.coord_first, c.coord_last, c.tau, n_checkpoints, h->stream, &h->adj);
        if (!rc) rc = scafes_adj_set_precision(h->adj, c.precision);
        if (!rc) rc = scafes_adj_set_conductivity_uniform(h->adj, a);
        if (rc) {
            fail(&h->err, rc, "scafes_gpu_adjoint: %s",
                 h->adj ? scafes_adj_last_error(h->adj) : scafes_last_error());
            scafes_adj_destroy(h->adj);
            h->adj = nullptr;
            return rc;
        }
        h->adj_snaps = n_checkpoints;
        h->adj_prec = c.precision;
    }
    const int rc = scafes::adj_backward_device_u0(h->adj, h->u0keep, dJ_du_T, h->t, dJ_dk, dJ_du0, n_nodes(h));
    if (rc) return fail(&h->err, rc, "%s", scafes_adj_last_error(h->adj));
    return SCAFES_OK;
}
