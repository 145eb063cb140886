// Shared device helpers: status plumbing, padded field layout and
// compensated FP32-pair ("f32x2") arithmetic.
//
// The f32x2 helpers implement the published error-free transformations:
//   TwoSum      Knuth, TAOCP vol. 2 (1969), 4.2.2 Thm B: s = fl(a+b) and the
//               exact rounding error e with a + b = s + e, 6 flops;
//   FastTwoSum  Dekker (1971): same, 3 flops, valid when |a| >= |b|;
//   TwoProd     with a fused multiply-add, p = fl(a*b), e = fma(a, b, -p)
//               is exact (a*b = p + e) for FP32 without underflow.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace scafes {

// Row pitch (in elements) of every device field: rows start on 256-byte
// boundaries for 8-byte elements, 128-byte boundaries for 4-byte ones.
__host__ __device__ inline int row_pitch(int nx) { return (nx + 31) & ~31; }

struct Layout {
    int nx, ny, nz;
    int pitch;          // elements per row
    long long plane;    // elements per z-plane (pitch * ny)
    int nl;             // border layers: a node is a border node when it lies
                        // within nl nodes of a face (nLayersAtBorder)
    __host__ __device__ long long idx(int i, int j, int k) const {
        return (long long)k * plane + (long long)j * pitch + i;
    }
    __host__ __device__ long long size() const { return plane * nz; }
};

inline Layout make_layout(int nx, int ny, int nz) {
    Layout L;
    L.nx = nx; L.ny = ny; L.nz = nz;
    L.pitch = row_pitch(nx);
    L.plane = (long long)L.pitch * ny;
    L.nl = 1;
    return L;
}

// ---- compensated FP32 pairs ------------------------------------------------

struct f2 { float hi, lo; };

__device__ __forceinline__ f2 two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}

__device__ __forceinline__ f2 fast_two_sum(float a, float b) {
    float s = __fadd_rn(a, b);
    float e = __fsub_rn(b, __fsub_rn(s, a));
    return {s, e};
}

// Split a double into hi + lo (round-to-nearest hi, remainder rounded).
__host__ __device__ inline f2 split_double(double x) {
    float hi = (float)x;
    float lo = (float)(x - (double)hi);
    return {hi, lo};
}

__host__ __device__ inline double join_pair(float hi, float lo) {
    return (double)hi + (double)lo;
}

// Split a double into hi + lo with integer instructions only (no FP64
// operation, which GB300 issues at a small fraction of its FP32 rate, not
// even a predicated one on a rare path): hi is the value with its
// significand truncated to 24 bits, lo the remaining 29 bits rounded to a
// float (one I2F).  |v - (hi + lo)| <= 2^-48 |v| for 2^-74 <= |v| < 2^128;
// smaller |v| down to 2^-126 keep only hi (truncated); below that (FP32
// subnormals, double subnormals, zero) the result is a signed zero;
// |v| >= 2^128 gives a signed infinity, infinities and NaN keep their kind.
__device__ __forceinline__ f2 split_bits(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
    const int e = (int)((b >> 52) & 0x7FF);
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const int ef = e - 1023 + 127;
    if (ef <= 0) return {__int_as_float((int)sign), 0.f};  // below the FP32 normal range
    if (ef >= 255) {                                         // above it: infinity, or NaN for a NaN
        const unsigned nan = (e == 0x7FF && m != 0) ? 0x400000u : 0u;
        return {__int_as_float((int)(sign | 0x7F800000u | nan)), 0.f};
    }
    const float hi = __int_as_float((int)(sign | ((unsigned)ef << 23) | (unsigned)(m >> 29)));
    const int es = e - 1075 + 127;
    if (es <= 0) return {hi, 0.f};
    const float l = __uint2float_rn((unsigned)(m & 0x1FFFFFFFull)) * __int_as_float(es << 23);
    return {hi, sign ? -l : l};
}

}  // namespace scafes
