// An ensemble assembled one instance at a time: scafes_gpu_batch_create,
// _enqueue (one parameter set with its initial iterate and source), _run.
// This is the shape of the reference's callers of whole runs -- its MCMC
// drivers (examples/MRIDataPBHEqnFDM/startMCMCFit.py) start one ScaFES run
// per parameter set -- turned into one device ensemble: the instances
// enqueued before the first run become one scafes_batch (one pool, one
// persistent kernel per step, the time loop in a CUDA graph).  Host code
// only; the kernels are those of batch.cu.
#include <cstdarg>
#include <cstdio>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/scafes_gb300.h"

namespace scafes {
void set_last_error(const char* msg);
}

struct scafes_gpu_batch {
    int precision = SCAFES_PREC_F64;
    void* stream = nullptr;
    std::vector<scafes_batch_instance> inst;
    std::vector<std::vector<double>> u0, f;  // host copies until the first run
    scafes_batch* b = nullptr;
    std::string err;
};

namespace {

int qfail(scafes_gpu_batch* q, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (q) q->err = buf;
    scafes::set_last_error(buf);
    return code;
}

size_t nodes(const scafes_batch_instance& in) {
    return (size_t)in.n_nodes[0] * in.n_nodes[1] * in.n_nodes[2];
}

// Builds the device ensemble from the enqueued instances and uploads their
// fields; the host copies are released afterwards.
int materialise(scafes_gpu_batch* q) {
    if (q->inst.empty()) return qfail(q, SCAFES_ERR_STATE, "scafes_gpu_batch_run: no instance enqueued");
    int rc = scafes_batch_create(q->inst.data(), (int)q->inst.size(), q->precision, q->stream, &q->b);
    if (rc) return qfail(q, rc, "scafes_gpu_batch_run: %s", scafes_last_error());
    for (size_t i = 0; i < q->inst.size(); ++i) {
        rc = scafes_batch_upload(q->b, (int)i, SCAFES_FIELD_U, q->u0[i].data(), q->u0[i].size());
        if (!rc && !q->f[i].empty())
            rc = scafes_batch_upload(q->b, (int)i, SCAFES_FIELD_F_A, q->f[i].data(), q->f[i].size());
        if (rc) {
            qfail(q, rc, "scafes_gpu_batch_run: %s", scafes_batch_last_error(q->b));
            scafes_batch_destroy(q->b);  // the next run starts over from the host copies
            q->b = nullptr;
            return rc;
        }
    }
    std::vector<std::vector<double>>().swap(q->u0);
    std::vector<std::vector<double>>().swap(q->f);
    return SCAFES_OK;
}

}  // namespace

extern "C" int scafes_gpu_batch_create(int precision, void* stream, scafes_gpu_batch** out) {
    if (!out) return qfail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_batch_create: out is NULL");
    *out = nullptr;
    if (precision != SCAFES_PREC_F64 && precision != SCAFES_PREC_F32X2 && precision != SCAFES_PREC_F32)
        return qfail(nullptr, SCAFES_ERR_UNSUPPORTED, "scafes_gpu_batch_create: precision %d not supported", precision);
    scafes_gpu_batch* q = new (std::nothrow) scafes_gpu_batch();
    if (!q) return qfail(nullptr, SCAFES_ERR_NOMEM, "scafes_gpu_batch_create: out of host memory");
    q->precision = precision;
    q->stream = stream;
    *out = q;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_batch_enqueue(scafes_gpu_batch* q, const scafes_batch_instance* inst, const double* u0,
                                        const double* f, int* index) {
    if (!q || !inst || !u0) return qfail(q, SCAFES_ERR_ARG, "scafes_gpu_batch_enqueue: NULL argument");
    if (q->b)
        return qfail(q, SCAFES_ERR_STATE,
                     "scafes_gpu_batch_enqueue: the ensemble already runs; enqueue before the first run");
    for (int p = 0; p < 3; ++p)
        if (inst->n_nodes[p] < 3 || inst->n_nodes[p] > 32767)
            return qfail(q, SCAFES_ERR_ARG, "scafes_gpu_batch_enqueue: n_nodes[%d]=%d out of [3, 32767]", p,
                         inst->n_nodes[p]);
    const size_t n = nodes(*inst);
    try {
        std::vector<double> a(u0, u0 + n), s = f ? std::vector<double>(f, f + n) : std::vector<double>();
        q->inst.reserve(q->inst.size() + 1);
        q->u0.reserve(q->u0.size() + 1);
        q->f.reserve(q->f.size() + 1);
        q->inst.push_back(*inst);  // no allocation after the reserves
        q->u0.push_back(std::move(a));
        q->f.push_back(std::move(s));
    } catch (const std::bad_alloc&) {
        return qfail(q, SCAFES_ERR_NOMEM, "scafes_gpu_batch_enqueue: out of host memory");
    }
    if (index) *index = (int)q->inst.size() - 1;
    return SCAFES_OK;
}

extern "C" int scafes_gpu_batch_run(scafes_gpu_batch* q, int n_steps) {
    if (!q) return qfail(nullptr, SCAFES_ERR_ARG, "scafes_gpu_batch_run: handle is NULL");
    if (n_steps < 0) return qfail(q, SCAFES_ERR_ARG, "scafes_gpu_batch_run: n_steps=%d < 0", n_steps);
    if (!q->b) {
        const int rc = materialise(q);
        if (rc) return rc;
    }
    const int rc = scafes_batch_step(q->b, n_steps);
    return rc ? qfail(q, rc, "scafes_gpu_batch_run: %s", scafes_batch_last_error(q->b)) : SCAFES_OK;
}

extern "C" int scafes_gpu_batch_download(scafes_gpu_batch* q, int index, double* host, size_t n) {
    if (!q || !host) return qfail(q, SCAFES_ERR_ARG, "scafes_gpu_batch_download: NULL argument");
    if (!q->b) return qfail(q, SCAFES_ERR_STATE, "scafes_gpu_batch_download: the ensemble has not run yet");
    const int rc = scafes_batch_download(q->b, index, SCAFES_FIELD_U, host, n);
    return rc ? qfail(q, rc, "scafes_gpu_batch_download: %s", scafes_batch_last_error(q->b)) : SCAFES_OK;
}

extern "C" scafes_batch* scafes_gpu_batch_ensemble(scafes_gpu_batch* q) { return q ? q->b : nullptr; }

extern "C" const char* scafes_gpu_batch_last_error(const scafes_gpu_batch* q) { return q ? q->err.c_str() : ""; }

extern "C" void scafes_gpu_batch_destroy(scafes_gpu_batch* q) {
    if (!q) return;
    if (q->b) scafes_batch_destroy(q->b);
    delete q;
}
