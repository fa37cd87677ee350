// pic_device.cuh -- device-side helpers shared by the step and deposition
// kernels: four-wide vector access to a k-row, compensated FP32 tallies and
// the block/grid reduction that turns per-thread tallies into one float64
// record per step.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pic_gb300.h"

namespace pic {

// The centre weight of the Lax-Wendroff stencil in the field type. The four
// weights sum to one (zm + zp + 4 lat + cen = 1: the scheme conserves carriers
// between recombination and collection). Rounded one by one to float32 they
// sum to 1 + O(3e-8), and that bias acts on every voxel at every step: over
// the few hundred steps a carrier lives it shifts the densities, and through
// the recombination term k_s, by ~1e-5. So the float32 centre weight absorbs
// the rounding of the other three, leaving the float32 sum within half an ulp
// of cen (~1e-9) of the float64 one; float64 fields take cen as it is.
template <typename T>
__host__ __device__ inline T centre_weight(double lat, double zm, double zp, double cen) {
    if (sizeof(T) == sizeof(double)) return (T)cen;
    const double d = ((double)(float)zm - zm) + ((double)(float)zp - zp) + 4.0 * ((double)(float)lat - lat);
    return (T)(cen - d);
}

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
// Coherent forms for kernels that read data written earlier in the same
// launch by other blocks (the persistent kernels): loads cached in L2 only
// (ld.global.cg). Neither the read-only path of __ldg nor an SM's L1 is kept
// coherent with other SMs' writes; L2 is the point of coherence.
__device__ __forceinline__ V4<float> load4c(const float *p) {
    const float4 t = __ldcg(reinterpret_cast<const float4 *>(p));
    return {{t.x, t.y, t.z, t.w}};
}
__device__ __forceinline__ V4<double> load4c(const double *p) {
    const double2 a = __ldcg(reinterpret_cast<const double2 *>(p));
    const double2 b = __ldcg(reinterpret_cast<const double2 *>(p) + 1);
    return {{a.x, a.y, b.x, b.y}};
}
__device__ __forceinline__ void store4(float *p, const V4<float> &v) {
    *reinterpret_cast<float4 *>(p) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void store4(double *p, const V4<double> &v) {
    reinterpret_cast<double2 *>(p)[0] = make_double2(v.v[0], v.v[1]);
    reinterpret_cast<double2 *>(p)[1] = make_double2(v.v[2], v.v[3]);
}

// One cell of the 2D deposition of a step: (G * density, G * the sum of the
// density of its four lateral neighbours), G the track peak density. The step
// kernels add the first to the cell's gap layers and the second to the
// lateral sum of its stencil, one load per column.
template <typename T> struct PairOf;
template <> struct PairOf<float> { using type = float2; };
template <> struct PairOf<double> { using type = double2; };
template <typename T> using pair_t = typename PairOf<T>::type;

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

// Double-float: the unevaluated sum hi + lo of two floats, added with the
// error-free TwoSum of Knuth (TAOCP vol. 2, 4.2.2) and renormalised with
// Dekker's FastTwoSum (1971) -- about 44 significant bits from FP32
// instructions only. The block and grid reductions of the float32 kernels use
// it in place of float64, whose rate on GB300 is a small fraction of FP32's
// (a float64 reduction tree was several microseconds of every small-grid step).
// Additions only: nothing here can be contracted into an FMA.
struct DF {
    float hi, lo;
};
__device__ __forceinline__ DF df_add(DF a, DF b) {
    const float s = a.hi + b.hi;
    const float v = s - a.hi;
    const float e = (a.hi - (s - v)) + (b.hi - v);
    const float lo = e + (a.lo + b.lo);
    const float h = s + lo;
    return {h, lo - (h - s)};
}
// A Kahan running sum (s, c) holds s - c.
__device__ __forceinline__ DF df_of(const Tally<float> &t) {
    const float h = t.s - t.c;
    return {h, (t.s - h) - t.c};
}
__device__ __forceinline__ double df_value(DF a) { return (double)a.hi + (double)a.lo; }

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

__device__ __forceinline__ DF warp_sum(DF a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const DF b{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
        a = df_add(a, b);
    }
    return a;
}

// Block-wide sum of four doubles (or double-floats), result valid in thread
// 0. Fixed tree order.
template <int BLOCK, typename A>
__device__ __forceinline__ void block_sum4(A (&v)[4], A (*smem)[4]) {
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
            A x = lane < BLOCK / 32 ? smem[lane][q] : A{};
            v[q] = warp_sum(x);
        }
    }
    __syncthreads();
}

// The double-float form of finish_tally (below) for float32 kernels: the
// partials are float2 (hi, lo) pairs in the same 8-byte slots.
template <int BLOCK>
__device__ void finish_tally_df(DF (&v)[4], double *partials_d, unsigned int *counter, double *tally,
                                double injected_scale) {
    __shared__ DF red[BLOCK / 32][4];
    __shared__ bool last;
    float2 *partials = reinterpret_cast<float2 *>(partials_d);
    block_sum4<BLOCK>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) partials[4 * (int64_t)blockIdx.x + q] = make_float2(v[q].hi, v[q].lo);
        __threadfence();
        unsigned int prev = atomicAdd(counter, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    DF acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += BLOCK) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float2 p = __ldcg(partials + 4 * (int64_t)b + q);
            acc[q] = df_add(acc[q], DF{p.x, p.y});
        }
    }
    block_sum4<BLOCK>(acc, red);
    if (threadIdx.x == 0) {
        tally[0] = df_value(acc[0]) * injected_scale;
        tally[1] = df_value(acc[1]);
        tally[2] = df_value(acc[2]);
        tally[3] = df_value(acc[3]);
        *counter = 0u;  // ready for the next step
        __threadfence();
    }
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
