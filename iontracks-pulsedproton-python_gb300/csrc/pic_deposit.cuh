// pic_deposit.cuh -- the per-track deposition body (one or more warps per track),
// shared by the single-grid kernel (deposit.cu) and the batched one
// (batched.cu). See deposit.cu for what it computes.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pic_device.cuh"

namespace pic {

__device__ __forceinline__ float gauss1(double d, float h2b2) {
    const float f = (float)d;
    return expf(-(f * f) * h2b2);
}
__device__ __forceinline__ double gauss1(double d, double h2b2) { return exp(-(d * d) * h2b2); }

__device__ __forceinline__ void add_pair(float2 *p, float c, float l) { atomicAdd(p, make_float2(c, l)); }
__device__ __forceinline__ void add_pair(double2 *p, double c, double l) {
    atomicAdd(&p->x, c);
    atomicAdd(&p->y, l);
}

// One track, by `nparts` warps (this one is `part`; lane = this thread's
// lane): its truncated separable Gaussian added into the step's deposition
// pairs (row pitch dp), its centre counted once. With g_i = exp(-(i-x)^2 h^2/b^2)
// inside the truncation box [i_lo, i_hi) and 0 outside it (the same for j),
// cell (i, j) receives
//   G g_i g_j                                         (its density), and
//   G ((g_{i-1} + g_{i+1}) g_j + g_i (g_{j-1} + g_{j+1}))  (its neighbours'),
// so the written box is the truncation box widened by one cell each way.
// Part p takes the written box's rows i0 + p, i0 + p + nparts, ...: a step
// with few tracks spreads each box over several warps.
template <typename T>
__device__ __forceinline__ void deposit_track(double x, double y, int64_t n, int64_t dp, double cut, T h2b2, T gfac,
                                              pair_t<T> *__restrict__ dens, uint32_t *__restrict__ counts, int lane,
                                              int part = 0, int nparts = 1) {
    int64_t i_lo = (int64_t)ceil(x - cut), i_hi = (int64_t)floor(x + cut) + 1;
    int64_t j_lo = (int64_t)ceil(y - cut), j_hi = (int64_t)floor(y + cut) + 1;
    i_lo = i_lo < 0 ? 0 : i_lo;
    j_lo = j_lo < 0 ? 0 : j_lo;
    i_hi = i_hi > n ? n : i_hi;
    j_hi = j_hi > n ? n : j_hi;
    if (counts && lane == 0 && part == 0) {
        // int(x) floors for x >= 0; centres lie in [0, no_xy). A recomputed
        // step passes no counter: its tracks were counted once.
        int64_t ix = (int64_t)x, iy = (int64_t)y;
        if (ix >= 0 && ix < n && iy >= 0 && iy < n) atomicAdd(counts + ix * n + iy, 1u);
    }
    if (i_lo >= i_hi || j_lo >= j_hi) return;
    auto gi = [&](int64_t i) { return (i >= i_lo && i < i_hi) ? gauss1((double)i - x, h2b2) : T(0); };
    auto gj = [&](int64_t j) { return (j >= j_lo && j < j_hi) ? gauss1((double)j - y, h2b2) : T(0); };
    const int64_t oi_lo = i_lo > 0 ? i_lo - 1 : 0, oi_hi = i_hi < n ? i_hi + 1 : n;
    const int64_t oj_lo = j_lo > 0 ? j_lo - 1 : 0, oj_hi = j_hi < n ? j_hi + 1 : n;
    const int64_t box_rows = oi_hi - oi_lo;
    const int64_t nrows = box_rows > part ? (box_rows - part + nparts - 1) / nparts : 0;
    // Each lane evaluates one exponential per column chunk and one per row
    // chunk; the neighbouring factors come from the adjacent lanes (the edge
    // lanes evaluate the one factor beyond the chunk).
    for (int64_t jb = oj_lo; jb < oj_hi; jb += 32) {
        const int64_t j = jb + lane;
        const bool jok = j < oj_hi;
        const T gjo = gj(j);
        T gjm = __shfl_up_sync(0xffffffffu, gjo, 1), gjp = __shfl_down_sync(0xffffffffu, gjo, 1);
        if (lane == 0) gjm = gj(j - 1);
        if (lane == 31) gjp = gj(j + 1);
        const T Gj = jok ? gfac * gjo : T(0);
        const T Hj = jok ? gfac * (gjm + gjp) : T(0);
        for (int64_t tb = 0; tb < nrows; tb += 32) {
            const int rows = (int)((nrows - tb) < 32 ? (nrows - tb) : 32);
            const int64_t i0 = oi_lo + part + nparts * tb;  // row of r = 0
            const int64_t il = i0 + (int64_t)nparts * lane;
            const T gio = gi(il);
            T him;
            if (nparts == 1) {  // rows il -1 / +1 belong to the adjacent lanes
                T gim = __shfl_up_sync(0xffffffffu, gio, 1), gip = __shfl_down_sync(0xffffffffu, gio, 1);
                if (lane == 0) gim = gi(il - 1);
                if (lane == 31) gip = gi(il + 1);
                him = gim + gip;
            } else {
                him = gi(il - 1) + gi(il + 1);
            }
            const T gi_lane = lane < rows ? gio : T(0);
            const T hi_lane = lane < rows ? him : T(0);
            for (int r = 0; r < rows; ++r) {
                const T g_i = __shfl_sync(0xffffffffu, gi_lane, r);
                const T h_i = __shfl_sync(0xffffffffu, hi_lane, r);
                const T c = g_i * Gj, l = h_i * Gj + g_i * Hj;
                if (jok && (c != T(0) || l != T(0))) add_pair(dens + (i0 + (int64_t)nparts * r) * dp + j, c, l);
            }
        }
    }
}

}  // namespace pic
