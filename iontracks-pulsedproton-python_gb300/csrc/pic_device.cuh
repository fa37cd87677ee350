// pic_device.cuh -- device-side helpers shared by the step and deposition
// kernels: four-wide vector access to a k-row, compensated FP32 tallies and
// the block/grid reduction that turns per-thread tallies into one float64
// record per step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pic_gb300.h"

namespace pic {

// Four consecutive k elements of one (i, j) column. The field rows are
// 32-byte aligned (kpitch is a multiple of 8) and every vector starts at a
// multiple of 4 elements, so float loads are single 128-bit accesses and
// double loads two 128-bit accesses.
template <typename T>
struct V4 {
    T v[4];
};

__device__ __forceinline__ V4<float> load4(const float *p) {
    float4 t = __ldg(reinterpret_cast<const float4 *>(p));
    return {{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ V4<double> load4(const double *p) {
    double2 a = __ldg(reinterpret_cast<const double2 *>(p));
    double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    return {{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void store4(float *p, const V4<float> &v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void store4(double *p, const V4<double> &v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v.v[0], v.v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v.v[2], v.v[3]);
}

// Running sum of one tally. FP32 partials are Kahan-compensated: a thread
// adds thousands of voxel values, and plain float accumulation would lose
// ~1e-5 of the total; the compensation keeps it at float64-like accuracy
// using only FP32 instructions (the GPU's FP64 rate is a small fraction of
// its FP32 rate). FP64 fields accumulate plainly.
template <typename T>
struct Tally {
    T s = 0, c = 0;
    __device__ __forceinline__ void add(T v) {
        T y = v - c;
        T t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};
template <>
struct Tally<double> {
    double s = 0;
    __device__ __forceinline__ void add(double v) { s += v; }
    __device__ __forceinline__ double value() const { return s; }
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of four doubles, result valid in thread 0. Fixed tree order.
template <int BLOCK>
__device__ __forceinline__ void block_sum4(double (&v)[4], double (*smem)[4]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < 4; ++q) v[q] = warp_sum(v[q]);
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) smem[warp][q] = v[q];
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double x = lane < BLOCK / 32 ? smem[lane][q] : 0.0;
            v[q] = warp_sum(x);
        }
    }
    __syncthreads();
}

// Completes a step's tallies: every block stores its partial, the last block
// to finish (completion counter) sums all partials in block order and writes
// tally[0..3]. Deterministic for a given grid size; no float atomics.
// partial order in memory: {injected (dimensionless), recombined, n+, n-}.
template <int BLOCK>
__device__ void finish_tally(double (&v)[4], double *partials, unsigned int *counter, double *tally,
                             double injected_scale) {
    __shared__ double red[BLOCK / 32][4];
    __shared__ bool last;
    block_sum4<BLOCK>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) partials[4 * (int64_t)blockIdx.x + q] = v[q];
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += BLOCK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += __ldcg(partials + 4 * (int64_t)b + q);
    }
    block_sum4<BLOCK>(acc, red);
    if (threadIdx.x == 0) {
        tally[0] = acc[0] * injected_scale;
        tally[1] = acc[1];
        tally[2] = acc[2];
        tally[3] = acc[3];
        *counter = 0u;  // ready for the next step
        __threadfence();
    }
}

}  // namespace pic
