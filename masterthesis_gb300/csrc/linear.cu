// Linear multi-field stencils with an optional second (leapfrog) phase:
// the device form of update callbacks that couple several unknown fields,
//   u_new[f](i) = cst + sum_k w_k * u_old[src_k](i + d_k),
// one rule per (phase, field, node class) -- class 0 the inner nodes,
// classes 1..63 the border nodes by the faces they lie on (bit 0 x = 0,
// bit 1 x = nx-1, bit 2 y = 0, bit 3 y = ny-1, bit 4 z = 0, bit 5 z = nz-1)
// -- as the drop-in Problem records them from updateInner/updateBorder and
// updateInner2/updateBorder2.  A step runs phase 1 (old -> new) and, for a
// leapfrog problem, phase 2 on the result of phase 1 (the reference's
// evalUpdatePhase, pointer swap, evalUpdate2Phase, src/ScaFES_Problem.hpp:
// 2596-2619, 2829-2918; every node of the new iterate starts as a copy of
// the old one, :5078-5082, which a recorded rule already contains).
// FP64, plain loads: a correctness path for the problems the fused kernels
// (Lame-Navier, Yee) do not cover as recorded callbacks.  Each field has its
// own pair of buffers; a field that a phase leaves alone on every node (its
// rule the identity) is neither copied nor swapped in that phase.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "scafes_common.cuh"
#include "../../include/scafes_gb300.h"

using namespace scafes;

namespace scafes {
void set_last_error(const char* msg);
}

namespace {

struct Rule {
    int off, n;  // terms [off, off + n)
    double cst;
};

struct Term {
    long long d;  // element offset of the neighbour (padded layout)
    int src;      // source field
    double w;
};

constexpr int kClasses = SCAFES_BORDER_CLASSES;

// Where each field of one phase is read from and written to.  A field whose
// rule is the identity on every node class in this phase is neither
// written nor swapped (out = nullptr): its current buffer stays current.
struct FieldPtrs {
    const double* in[SCAFES_LIN_MAX_FIELDS];
    double* out[SCAFES_LIN_MAX_FIELDS];
};

__global__ void k_linear(FieldPtrs P, const Rule* __restrict__ rules, const Term* __restrict__ terms, int n_fields,
                         Layout L) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y, z = blockIdx.z;
    if (x >= L.nx || y >= L.ny) return;
    const int cls = (x == 0) | ((x == L.nx - 1) << 1) | ((y == 0) << 2) | ((y == L.ny - 1) << 3) | ((z == 0) << 4) |
                    ((z == L.nz - 1) << 5);
    const long long o = L.idx(x, y, z);
    for (int f = 0; f < n_fields; ++f) {
        if (P.out[f] == nullptr) continue;
        const Rule r = rules[f * kClasses + cls];
        double v = r.cst;
        for (int k = r.off; k < r.off + r.n; ++k) {
            const Term t = terms[k];
            v = fma(t.w, P.in[t.src][o + t.d], v);
        }
        P.out[f][o] = v;
    }
}

}  // namespace

struct scafes_lin {
    Layout L;
    int n_fields = 0, n_phases = 1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    double* buf[2] = {nullptr, nullptr};  // all fields, padded layout, field after field
    int cur[SCAFES_LIN_MAX_FIELDS] = {};  // per field, the buffer holding its current values
    std::vector<bool> ident;              // [phase][field]: the identity on every class
    // Host rules: [phase][field][class] -> terms; the device copies are
    // rebuilt when a rule changes.
    std::vector<std::vector<scafes_lin_term>> host_terms;
    std::vector<double> host_cst;
    std::vector<bool> host_set;
    Rule* rules = nullptr;
    Term* terms = nullptr;
    bool dirty = true;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = 0.f;
    std::string err;
};

namespace {

int lfail(scafes_lin* h, int code, const char* fmt, ...) {
    char b[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(b, sizeof(b), fmt, ap);
    va_end(ap);
    if (h) h->err = b;
    scafes::set_last_error(b);
    return code;
}

#define LTRY(h, call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return lfail(h, SCAFES_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

size_t slot(const scafes_lin* h, int phase, int field, int cls) {
    return ((size_t)phase * h->n_fields + field) * kClasses + cls;
}

long long field_stride(const scafes_lin* h) { return h->L.size(); }

// Uploads the rule tables (both phases) once after a change.
int sync_rules(scafes_lin* h) {
    if (!h->dirty) return SCAFES_OK;
    std::vector<Rule> r(h->host_terms.size());
    std::vector<Term> t;
    for (size_t s = 0; s < r.size(); ++s) {
        if (!h->host_set[s]) {
            return lfail(h, SCAFES_ERR_STATE, "scafes_lin_step: no rule for phase %d, field %d, class %d",
                         (int)(s / ((size_t)h->n_fields * kClasses)),
                         (int)(s / kClasses % h->n_fields), (int)(s % kClasses));
        }
        r[s].off = (int)t.size();
        r[s].n = (int)h->host_terms[s].size();
        r[s].cst = h->host_cst[s];
        for (const auto& q : h->host_terms[s]) t.push_back(Term{h->L.idx(q.dx, q.dy, q.dz), q.src, q.w});
    }
    h->ident.assign((size_t)h->n_phases * h->n_fields, true);
    for (size_t s = 0; s < r.size(); ++s) {
        const int ph = (int)(s / ((size_t)h->n_fields * kClasses)), f = (int)(s / kClasses % h->n_fields);
        const auto& tl = h->host_terms[s];
        const bool id = h->host_cst[s] == 0.0 && tl.size() == 1 && tl[0].src == f && tl[0].dx == 0 &&
                        tl[0].dy == 0 && tl[0].dz == 0 && tl[0].w == 1.0;
        if (!id) h->ident[(size_t)ph * h->n_fields + f] = false;
    }
    cudaFree(h->rules);
    cudaFree(h->terms);
    h->rules = nullptr;
    h->terms = nullptr;
    LTRY(h, cudaMalloc(&h->rules, sizeof(Rule) * r.size()));
    LTRY(h, cudaMalloc(&h->terms, sizeof(Term) * (t.empty() ? 1 : t.size())));
    LTRY(h, cudaMemcpyAsync(h->rules, r.data(), sizeof(Rule) * r.size(), cudaMemcpyHostToDevice, h->stream));
    if (!t.empty())
        LTRY(h, cudaMemcpyAsync(h->terms, t.data(), sizeof(Term) * t.size(), cudaMemcpyHostToDevice, h->stream));
    LTRY(h, cudaStreamSynchronize(h->stream));
    h->dirty = false;
    return SCAFES_OK;
}

}  // namespace

extern "C" const char* scafes_lin_last_error(const scafes_lin* h) { return h ? h->err.c_str() : ""; }

extern "C" void scafes_lin_destroy(scafes_lin* h) {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->buf[0]);
    cudaFree(h->buf[1]);
    cudaFree(h->rules);
    cudaFree(h->terms);
    if (h->e0) cudaEventDestroy(h->e0);
    if (h->e1) cudaEventDestroy(h->e1);
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

extern "C" int scafes_lin_create(const int n_nodes[3], int n_fields, int n_phases, void* stream, scafes_lin** out) {
    if (!out || !n_nodes) return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_create: NULL argument");
    *out = nullptr;
    if (n_fields < 1 || n_fields > SCAFES_LIN_MAX_FIELDS || (n_phases != 1 && n_phases != 2))
        return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_create: %d fields (1..%d), %d phases (1 or 2)", n_fields,
                     SCAFES_LIN_MAX_FIELDS, n_phases);
    // z is the launch grid's third dimension (at most 65535 blocks).
    for (int p = 0; p < 3; ++p)
        if (n_nodes[p] < 3 || n_nodes[p] > 65535)
            return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_create: n_nodes[%d]=%d out of [3, 65535]", p, n_nodes[p]);
    scafes_lin* h = new (std::nothrow) scafes_lin();
    if (!h) return lfail(nullptr, SCAFES_ERR_NOMEM, "scafes_lin_create: out of host memory");
    h->L = make_layout(n_nodes[0], n_nodes[1], n_nodes[2]);
    h->n_fields = n_fields;
    h->n_phases = n_phases;
    const size_t nrules = (size_t)n_phases * n_fields * kClasses;
    h->host_terms.assign(nrules, {});
    h->host_cst.assign(nrules, 0.0);
    h->host_set.assign(nrules, false);
    cudaError_t e = cudaSuccess;
    if (stream) h->stream = (cudaStream_t)stream;
    else { e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking); h->own_stream = true; }
    const size_t bytes = (size_t)h->L.size() * n_fields * sizeof(double);
    for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
        e = cudaMalloc(&h->buf[b], bytes);
        if (e == cudaSuccess) e = cudaMemsetAsync(h->buf[b], 0, bytes, h->stream);
    }
    if (e == cudaSuccess) e = cudaEventCreate(&h->e0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->e1);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        const int code = e == cudaErrorMemoryAllocation ? SCAFES_ERR_NOMEM : SCAFES_ERR_CUDA;
        lfail(nullptr, code, "scafes_lin_create: %s", cudaGetErrorString(e));
        scafes_lin_destroy(h);
        return code;
    }
    *out = h;
    return SCAFES_OK;
}

extern "C" int scafes_lin_set_rule(scafes_lin* h, int phase, int field, int cls, const scafes_lin_term* terms,
                                   int n_terms, double cst) {
    if (!h) return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_set_rule: handle is NULL");
    if (phase < 1 || phase > h->n_phases || field < 0 || field >= h->n_fields || cls < 0 || cls >= kClasses ||
        n_terms < 0 || n_terms > SCAFES_LIN_MAX_TERMS || (n_terms > 0 && !terms))
        return lfail(h, SCAFES_ERR_ARG, "scafes_lin_set_rule: phase %d, field %d, class %d, %d terms out of range",
                     phase, field, cls, n_terms);
    const bool out[6] = {(cls & 1) != 0, (cls & 2) != 0, (cls & 4) != 0, (cls & 8) != 0, (cls & 16) != 0,
                         (cls & 32) != 0};
    for (int k = 0; k < n_terms; ++k) {
        const scafes_lin_term& t = terms[k];
        if (t.src < 0 || t.src >= h->n_fields || t.dx < -1 || t.dx > 1 || t.dy < -1 || t.dy > 1 || t.dz < -1 ||
            t.dz > 1)
            return lfail(h, SCAFES_ERR_ARG, "scafes_lin_set_rule: term %d reads field %d at (%d,%d,%d)", k, t.src,
                         t.dx, t.dy, t.dz);
        // A node of this class has no neighbour beyond the faces it lies on.
        if ((t.dx < 0 && out[0]) || (t.dx > 0 && out[1]) || (t.dy < 0 && out[2]) || (t.dy > 0 && out[3]) ||
            (t.dz < 0 && out[4]) || (t.dz > 0 && out[5]))
            return lfail(h, SCAFES_ERR_ARG, "scafes_lin_set_rule: class %d has no neighbour at (%d,%d,%d)", cls, t.dx,
                         t.dy, t.dz);
    }
    const size_t s = slot(h, phase - 1, field, cls);
    h->host_terms[s].assign(terms, terms + n_terms);
    h->host_cst[s] = cst;
    h->host_set[s] = true;
    h->dirty = true;
    return SCAFES_OK;
}

extern "C" int scafes_lin_upload(scafes_lin* h, int field, const double* host, size_t n) {
    if (!h || !host) return lfail(h, SCAFES_ERR_ARG, "scafes_lin_upload: NULL argument");
    const Layout& L = h->L;
    if (field < 0 || field >= h->n_fields || n != (size_t)L.nx * L.ny * L.nz)
        return lfail(h, SCAFES_ERR_ARG, "scafes_lin_upload: field %d / %zu values", field, n);
    double* d = h->buf[h->cur[field]] + (size_t)field * field_stride(h);
    LTRY(h, cudaMemcpy2DAsync(d, (size_t)L.pitch * 8, host, (size_t)L.nx * 8, (size_t)L.nx * 8, (size_t)L.ny * L.nz,
                              cudaMemcpyHostToDevice, h->stream));
    LTRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_lin_download(scafes_lin* h, int field, double* host, size_t n) {
    if (!h || !host) return lfail(h, SCAFES_ERR_ARG, "scafes_lin_download: NULL argument");
    const Layout& L = h->L;
    if (field < 0 || field >= h->n_fields || n != (size_t)L.nx * L.ny * L.nz)
        return lfail(h, SCAFES_ERR_ARG, "scafes_lin_download: field %d / %zu values", field, n);
    const double* d = h->buf[h->cur[field]] + (size_t)field * field_stride(h);
    LTRY(h, cudaMemcpy2DAsync(host, (size_t)L.nx * 8, d, (size_t)L.pitch * 8, (size_t)L.nx * 8, (size_t)L.ny * L.nz,
                              cudaMemcpyDeviceToHost, h->stream));
    LTRY(h, cudaStreamSynchronize(h->stream));
    return SCAFES_OK;
}

extern "C" int scafes_lin_step(scafes_lin* h, int n_steps) {
    if (!h) return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_step: handle is NULL");
    if (n_steps < 0) return lfail(h, SCAFES_ERR_ARG, "scafes_lin_step: n_steps < 0");
    if (int rc = sync_rules(h)) return rc;
    const Layout& L = h->L;
    const dim3 grid((L.nx + 31) / 32, (L.ny + 7) / 8, L.nz), block(32, 8);
    const size_t per_phase = (size_t)h->n_fields * kClasses;
    LTRY(h, cudaEventRecord(h->e0, h->stream));
    for (int s = 0; s < n_steps; ++s)
        for (int ph = 0; ph < h->n_phases; ++ph) {
            FieldPtrs P;
            for (int f = 0; f < SCAFES_LIN_MAX_FIELDS; ++f) {
                P.in[f] = nullptr;
                P.out[f] = nullptr;
            }
            for (int f = 0; f < h->n_fields; ++f) {
                const size_t fo = (size_t)f * field_stride(h);
                P.in[f] = h->buf[h->cur[f]] + fo;
                if (!h->ident[(size_t)ph * h->n_fields + f]) P.out[f] = h->buf[h->cur[f] ^ 1] + fo;
            }
            k_linear<<<grid, block, 0, h->stream>>>(P, h->rules + ph * per_phase, h->terms, h->n_fields, L);
            LTRY(h, cudaGetLastError());
            for (int f = 0; f < h->n_fields; ++f)
                if (P.out[f]) h->cur[f] ^= 1;
        }
    LTRY(h, cudaEventRecord(h->e1, h->stream));
    LTRY(h, cudaEventSynchronize(h->e1));
    LTRY(h, cudaEventElapsedTime(&h->ms, h->e0, h->e1));
    return SCAFES_OK;
}

extern "C" int scafes_lin_last_ms(const scafes_lin* h, float* ms) {
    if (!h || !ms) return lfail(nullptr, SCAFES_ERR_ARG, "scafes_lin_last_ms: NULL argument");
    *ms = h->ms;
    return SCAFES_OK;
}
