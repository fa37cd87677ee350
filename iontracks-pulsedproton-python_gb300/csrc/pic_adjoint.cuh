// pic_adjoint.cuh -- device helpers shared by the two adjoint step kernels
// (adjoint.cu: flat; adjoint_stream.cu: streaming): the five derivative sums
// and their double-float (float32 fields) or double (float64 fields) slots.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_device.cuh"

namespace pic {

constexpr int kAdjGrad = 5;  // dR/ds+, dR/dc+, dR/ds-, dR/dc-, dR/da

// Reduction helpers over kAdjGrad values (double-float for float32 fields).
template <typename T> struct AdjRed { using type = double; };
template <> struct AdjRed<float> { using type = DF; };
__device__ __forceinline__ double adj_of(const Tally<double> &t) { return t.value(); }
__device__ __forceinline__ DF adj_of(const Tally<float> &t) { return df_of(t); }
__device__ __forceinline__ void adj_store(double *slot, double v) { *slot = v; }
__device__ __forceinline__ void adj_store(double *slot, DF v) {
    *reinterpret_cast<float2 *>(slot) = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ void adj_load_add(double &acc, const double *slot) { acc += __ldcg(slot); }
__device__ __forceinline__ void adj_load_add(DF &acc, const double *slot) {
    const float2 p = __ldcg(reinterpret_cast<const float2 *>(slot));
    acc = df_add(acc, DF{p.x, p.y});
}
__device__ __forceinline__ double adj_value(double v) { return v; }
__device__ __forceinline__ double adj_value(DF v) { return df_value(v); }
// slot += v, by the one thread that owns the slot
__device__ __forceinline__ void adj_accumulate(double *slot, double v) { *slot += v; }
__device__ __forceinline__ void adj_accumulate(double *slot, DF v) {
    float2 *p = reinterpret_cast<float2 *>(slot);
    const float2 o = *p;
    const DF s = df_add(DF{o.x, o.y}, v);
    *p = make_float2(s.hi, s.lo);
}

}  // namespace pic
