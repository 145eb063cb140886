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

}  // namespace scafes
