// Issue-rate probes for the roofline of the sweep kernels: the FP64 FMA rate
// and the FP32 FMA rate of the current GPU, measured with CUDA events.
// On GB300 the FP64 rate, not HBM, bounds an FP64 7-point sweep, so the
// benchmark reports that bound beside the HBM one.
#include <cuda_runtime.h>

#include "dadd_int.cuh"
#include "tma.cuh"
#include "../../include/scafes_gb300.h"

namespace {

constexpr int kIters = 2048;

__global__ void k_dfma_rate(double* out, double a, double b) {
    double x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
    for (int i = 0; i < kIters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ffma_rate(float* out, float a, float b) {
    float x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
#pragma unroll 4
    for (int i = 0; i < 4 * kIters; ++i) {
        x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
        x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

// One CTA waits, with the bounded wait of the sweep kernels, on an
// mbarrier that nothing arrives at: the wait must give up after limit_ns
// and the kernel report it in the status word, as a sweep whose TMA load
// never completed does.
__global__ void k_wait_probe(unsigned long long limit_ns, int* status, unsigned long long* waited_ns) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        scafes::mbar_init(&bar, 1);
        scafes::fence_barrier_init();
    }
    __syncthreads();
    const unsigned long long t0 = scafes::global_timer_ns();
    const bool ok = scafes::bounded_wait(&bar, 0, limit_ns);
    if (!__syncthreads_and(ok) && threadIdx.x == 0) {
        atomicExch(status, SCAFES_ERR_TIMEOUT);
        *waited_ns = scafes::global_timer_ns() - t0;
    }
}

// The integer-pipe addition of the FP64 sweep, element by element.
__global__ void k_dadd_int(const uint64_t* a, const uint64_t* b, uint64_t* sum, unsigned char* ok, long long n) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride) {
        bool o;
        sum[i] = scafes::dadd_same_sign_bits(a[i], b[i], o);
        ok[i] = o ? 1 : 0;
    }
}

}  // namespace

// No counterpart in the reference: runs the integer-pipe binary64 addition
// of the FP64 sweep on the device for n pairs of bit patterns (host arrays,
// 1 <= n <= 2^26), for a check against the FP64 adder.  sum[i] is defined
// where ok[i] is 1.
extern "C" int scafes_probe_dadd_int(const unsigned long long* a, const unsigned long long* b,
                                     unsigned long long* sum, unsigned char* ok, long long n) {
    if (!a || !b || !sum || !ok || n < 1 || n > (1ll << 26)) return SCAFES_ERR_ARG;
    const size_t bytes = sizeof(uint64_t) * (size_t)n;
    uint64_t* d = nullptr;
    if (cudaMalloc(&d, 3 * bytes + (size_t)n) != cudaSuccess) return SCAFES_ERR_NOMEM;
    unsigned char* d_ok = reinterpret_cast<unsigned char*>(d + 3 * n);
    cudaError_t e = cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        const long long blocks = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
        k_dadd_int<<<(unsigned)blocks, 256>>>(d, d + n, d + 2 * n, d_ok, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(sum, d + 2 * n, bytes, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(ok, d_ok, (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(d);
    return e == cudaSuccess ? SCAFES_OK : SCAFES_ERR_CUDA;
}

// No counterpart in the reference: exercises the timeout path of the
// bounded device waits without any fault (no load is ever issued; the
// barrier simply never completes).  limit_us in [1, 1e6].  Writes the
// status the kernel recorded (SCAFES_ERR_TIMEOUT expected) and the time it
// waited; synchronises the device.
extern "C" int scafes_probe_wait_timeout(unsigned limit_us, int* status, double* waited_ms) {
    if (!status || !waited_ms || limit_us < 1 || limit_us > 1000000) return SCAFES_ERR_ARG;
    int* d_status = nullptr;
    unsigned long long* d_waited = nullptr;
    if (cudaMalloc(&d_status, sizeof(int)) != cudaSuccess) return SCAFES_ERR_CUDA;
    if (cudaMalloc(&d_waited, sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d_status);
        return SCAFES_ERR_CUDA;
    }
    int st = 0;
    unsigned long long w = 0;
    cudaError_t e = cudaMemset(d_status, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d_waited, 0, sizeof(unsigned long long));
    if (e == cudaSuccess) {
        k_wait_probe<<<1, 64>>>((unsigned long long)limit_us * 1000ull, d_status, d_waited);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&w, d_waited, sizeof(w), cudaMemcpyDeviceToHost);
    cudaFree(d_status);
    cudaFree(d_waited);
    if (e != cudaSuccess) return SCAFES_ERR_CUDA;
    *status = st;
    *waited_ms = (double)w * 1e-6;
    return SCAFES_OK;
}

// No counterpart in the reference: a measurement utility for the roofline.
extern "C" int scafes_probe_pipe_rates(double* fp64_gops, double* fp32_gops) {
    if (!fp64_gops || !fp32_gops) return SCAFES_ERR_ARG;
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess) return SCAFES_ERR_CUDA;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int blocks = sms * 8, threads = 256;
    double* buf = nullptr;
    if (cudaMalloc(&buf, sizeof(double) * blocks * threads) != cudaSuccess) return SCAFES_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0.f;
    const double lanes = (double)blocks * threads * 8;
    k_dfma_rate<<<blocks, threads>>>(buf, 1.0000001, 1e-9);  // warm-up
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) k_dfma_rate<<<blocks, threads>>>(buf, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    *fp64_gops = lanes * kIters * 3 / (ms * 1e-3) / 1e9;
    k_ffma_rate<<<blocks, threads>>>((float*)buf, 1.0000001f, 1e-9f);
    cudaEventRecord(e0);
    for (int r = 0; r < 3; ++r) k_ffma_rate<<<blocks, threads>>>((float*)buf, 1.0000001f, 1e-9f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    *fp32_gops = lanes * 4 * kIters * 3 / (ms * 1e-3) / 1e9;
    cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(buf);
    return err == cudaSuccess ? SCAFES_OK : SCAFES_ERR_CUDA;
}
