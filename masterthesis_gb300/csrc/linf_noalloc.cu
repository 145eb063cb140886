// Max-norm error check that allocates nothing.
//
// Who needs this: some callers of the stencil engine are not allowed to
// call cudaMalloc at the point where they want an error check.  Examples
// are a serving or real-time loop whose owner forbids allocation after
// start-up because cudaMalloc can synchronise the device and fail under
// memory pressure at any moment, and a host program that hands us device
// memory from its own pool allocator and must not have us grab memory
// behind its back.  scafes_gpu_err_linf keeps its partial
// maxima in a buffer that scafes_gpu_create allocates, so it is not usable
// without a handle; this entry point works on caller-owned device arrays and
// keeps its partial maxima in a fixed array in the library's device image.
//
// The scratch array below is part of the module: every GPU that loads the
// library holds it (256 KiB) until the process exits.  All calls share it,
// on every stream, so calls that overlap in time on the GPU race on it and
// give wrong results; callers must order them (one stream, or events).
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/scafes_gb300.h"

namespace scafes {
void set_last_error(const char* msg);  // capi.cu: feeds scafes_last_error()
}

namespace {

constexpr int kThreads = 256;
constexpr long long kChunk = 32768;   // elements per CTA (128 per thread)
constexpr int kMaxBlocks = 16384;     // CTAs whose partial maxima fit the scratch
constexpr int kMaxDevices = 64;
static_assert((long long)kMaxBlocks * kChunk == SCAFES_ERR_LINF_NOALLOC_MAX_N,
              "header limit must match the scratch array");

int reject(int code, const char* what) {
    scafes::set_last_error(what);
    return code;
}

// Two doubles (max |u - exact|, max |exact|) per CTA of the first pass.
// Every slot a call reads was written earlier by the same call, so nothing
// has to start at zero; the previous call's values are simply overwritten.
static __device__ __align__(256) double g_linf_scratch[2 * kMaxBlocks];

// Per device: the scratch address and the ID of the CUDA context it belongs
// to.  A module's device addresses are only valid in the context that loaded
// it; after cudaDeviceReset (or any teardown of the primary context) the next
// context loads the module again, possibly elsewhere, so an address is reused
// only while the current context is the one it was looked up in.
struct ScratchSlot {
    unsigned long long ctx_id;
    double* ptr;
};
ScratchSlot g_scratch[kMaxDevices] = {};
std::mutex g_setup_mutex;

__device__ __forceinline__ double to_inf_if_nan(double d) {
    return (d != d) ? __longlong_as_double(0x7ff0000000000000LL) : d;
}

__device__ __forceinline__ void block_max2(double& a, double& b) {
    __shared__ double sa[kThreads / 32], sb[kThreads / 32];
    for (int s = 16; s > 0; s >>= 1) {
        a = fmax(a, __shfl_down_sync(0xffffffffu, a, s));
        b = fmax(b, __shfl_down_sync(0xffffffffu, b, s));
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { sa[w] = a; sb[w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int k = 1; k < kThreads / 32; ++k) { a = fmax(a, sa[k]); b = fmax(b, sb[k]); }
    }
}

// Pass 1: CTA b reduces elements [b*kChunk, (b+1)*kChunk) into part[2b..2b+1].
__global__ void __launch_bounds__(kThreads)
k_linf_part(const double* __restrict__ u, const double* __restrict__ ex, long long n,
            double* __restrict__ part) {
    const long long lo = blockIdx.x * kChunk;
    const long long hi = lo + kChunk < n ? lo + kChunk : n;
    double me = 0.0, mr = 0.0;
    for (long long m = lo + threadIdx.x; m < hi; m += kThreads) {
        const double e = ex[m];
        me = fmax(me, to_inf_if_nan(fabs(u[m] - e)));
        mr = fmax(mr, fabs(e));
    }
    block_max2(me, mr);
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = me;
        part[2 * blockIdx.x + 1] = mr;
    }
}

// Pass 2: one CTA folds the nb partial pairs into out[0..1].
__global__ void __launch_bounds__(kThreads)
k_linf_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
    double me = 0.0, mr = 0.0;
    for (int k = threadIdx.x; k < nb; k += kThreads) {
        me = fmax(me, part[2 * k]);
        mr = fmax(mr, part[2 * k + 1]);
    }
    block_max2(me, mr);
    if (threadIdx.x == 0) {
        out[0] = me;
        out[1] = mr;
    }
}

// ID of the current CUDA context (cuCtxGetCurrent + cuCtxGetId, reached
// through the runtime's driver entry points, so the library needs no link
// against libcuda).  Returns false when the driver does not provide them.
using PfnCtxGetCurrent = int (*)(void**);
using PfnCtxGetId = int (*)(void*, unsigned long long*);

bool current_context_id(unsigned long long* id) {
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<PfnCtxGetCurrent>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<PfnCtxGetId>(p);
    }
    if (!get_current || !get_id) return false;
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return false;
    return get_id(ctx, id) == 0;
}

// Device address of the scratch array in the current context.  The first
// call on a device, and the first call after that device's context was
// replaced, looks it up (cudaGetSymbolAddress, which may load the module);
// later calls in the same context reuse it.
int scratch_on_current_device(double** ptr) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess)
        return reject(SCAFES_ERR_CUDA, "scafes_err_linf_noalloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices)
        return reject(SCAFES_ERR_UNSUPPORTED, "scafes_err_linf_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchSlot& slot = g_scratch[dev];
    unsigned long long id = 0;
    if (slot.ptr && current_context_id(&id) && slot.ctx_id == id) {
        *ptr = slot.ptr;
        return SCAFES_OK;
    }
    // First call on this device, or its context changed since the lookup:
    // look the address up in the current context (this makes the device's
    // primary context current if none is) and remember which context it was.
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_linf_scratch) != cudaSuccess || !p)
        return reject(SCAFES_ERR_CUDA, "scafes_err_linf_noalloc: cudaGetSymbolAddress of the scratch failed");
    slot.ptr = static_cast<double*>(p);
    // Without the driver's context IDs, every call looks the address up again.
    slot.ctx_id = current_context_id(&id) ? id : 0;
    if (slot.ctx_id == 0) {
        *ptr = slot.ptr;
        slot.ptr = nullptr;
        return SCAFES_OK;
    }
    *ptr = slot.ptr;
    return SCAFES_OK;
}

}  // namespace

extern "C" int scafes_err_linf_noalloc(const double* u, const double* exact, long long n,
                                       double* out, void* stream) {
    if (!u || !exact || !out)
        return reject(SCAFES_ERR_ARG, "scafes_err_linf_noalloc: NULL device pointer");
    if (n < 1) return reject(SCAFES_ERR_ARG, "scafes_err_linf_noalloc: n must be >= 1");
    if (n > SCAFES_ERR_LINF_NOALLOC_MAX_N) {
        char msg[200];
        snprintf(msg, sizeof(msg),
                 "scafes_err_linf_noalloc: n = %lld exceeds the fixed scratch capacity of %lld values",
                 n, (long long)SCAFES_ERR_LINF_NOALLOC_MAX_N);
        return reject(SCAFES_ERR_ARG, msg);
    }
    double* part = nullptr;
    const int rc = scratch_on_current_device(&part);
    if (rc != SCAFES_OK) return rc;
    const int nb = (int)((n + kChunk - 1) / kChunk);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    k_linf_part<<<nb, kThreads, 0, s>>>(u, exact, n, part);
    if (cudaGetLastError() != cudaSuccess)
        return reject(SCAFES_ERR_CUDA, "scafes_err_linf_noalloc: launch of the partial pass failed");
    k_linf_final<<<1, kThreads, 0, s>>>(part, nb, out);
    if (cudaGetLastError() != cudaSuccess)
        return reject(SCAFES_ERR_CUDA, "scafes_err_linf_noalloc: launch of the final pass failed");
    return SCAFES_OK;
}
