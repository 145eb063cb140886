// Conversions between host-layout doubles (dense, x fastest) staged on the
// device and the padded device layout of each precision.
#include "star7.cuh"
#include "../../include/scafes_gb300.h"

namespace scafes {

size_t element_size(int precision) {
    switch (precision) {
        case SCAFES_PREC_F64: return sizeof(double);
        case SCAFES_PREC_F32X2: return sizeof(float2);
        case SCAFES_PREC_F32: return sizeof(float);
        default: return 0;
    }
}

static int conv_blocks() {
    static int n = 0;
    if (n == 0) {
        int dev = 0, sms = 1;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        n = sms * 4;
    }
    return n;
}

template <int PREC>
__global__ void k_to_device(const double* __restrict__ dense, void* __restrict__ field, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % L.nx);
        const long long r = m / L.nx;
        const int j = (int)(r % L.ny);
        const int k = (int)(r / L.ny);
        const long long o = L.idx(i, j, k);
        const double v = dense[m];
        if (PREC == SCAFES_PREC_F64) ((double*)field)[o] = v;
        else if (PREC == SCAFES_PREC_F32) ((float*)field)[o] = (float)v;
        else { f2 p = split_double(v); ((float2*)field)[o] = make_float2(p.hi, p.lo); }
    }
}

template <int PREC>
__global__ void k_from_device(const void* __restrict__ field, double* __restrict__ dense, Layout L) {
    const long long n = (long long)L.nx * L.ny * L.nz;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < n;
         m += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(m % L.nx);
        const long long r = m / L.nx;
        const int j = (int)(r % L.ny);
        const int k = (int)(r / L.ny);
        const long long o = L.idx(i, j, k);
        double v;
        if (PREC == SCAFES_PREC_F64) v = ((const double*)field)[o];
        else if (PREC == SCAFES_PREC_F32) v = (double)((const float*)field)[o];
        else { float2 p = ((const float2*)field)[o]; v = join_pair(p.x, p.y); }
        dense[m] = v;
    }
}

cudaError_t convert_to_device(int precision, const double* dense, void* field,
                              const Layout& L, cudaStream_t stream) {
    const int blocks = conv_blocks(), threads = 256;
    switch (precision) {
        case SCAFES_PREC_F64: k_to_device<SCAFES_PREC_F64><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        case SCAFES_PREC_F32: k_to_device<SCAFES_PREC_F32><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        case SCAFES_PREC_F32X2: k_to_device<SCAFES_PREC_F32X2><<<blocks, threads, 0, stream>>>(dense, field, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t convert_from_device(int precision, const void* field, double* dense,
                                const Layout& L, cudaStream_t stream) {
    const int blocks = conv_blocks(), threads = 256;
    switch (precision) {
        case SCAFES_PREC_F64: k_from_device<SCAFES_PREC_F64><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        case SCAFES_PREC_F32: k_from_device<SCAFES_PREC_F32><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        case SCAFES_PREC_F32X2: k_from_device<SCAFES_PREC_F32X2><<<blocks, threads, 0, stream>>>(field, dense, L); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace scafes
