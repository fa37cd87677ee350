// pic_deposit.cuh -- the per-track deposition body (one or more warps per track),
// shared by the single-grid kernel (deposit.cu) and the batched one
// (batched.cu). See deposit.cu for what it computes.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

namespace pic {

__device__ __forceinline__ float gauss1(double d, float h2b2) {
    const float f = (float)d;
    return expf(-(f * f) * h2b2);
}
__device__ __forceinline__ double gauss1(double d, double h2b2) { return exp(-(d * d) * h2b2); }

// One track, by `nparts` warps (this one is `part`; lane = this thread's
// lane): its truncated separable Gaussian added into dens (row pitch dp), its
// centre counted once. Part p takes the box rows i_lo + p, i_lo + p + nparts,
// ...: a step with few tracks spreads each box over several warps.
template <typename T>
__device__ __forceinline__ void deposit_track(double x, double y, int64_t n, int64_t dp, double cut, T h2b2,
                                              T *__restrict__ dens, uint32_t *__restrict__ counts, int lane,
                                              int part = 0, int nparts = 1) {
    int64_t i_lo = (int64_t)ceil(x - cut), i_hi = (int64_t)floor(x + cut) + 1;
    int64_t j_lo = (int64_t)ceil(y - cut), j_hi = (int64_t)floor(y + cut) + 1;
    i_lo = i_lo < 0 ? 0 : i_lo;
    j_lo = j_lo < 0 ? 0 : j_lo;
    i_hi = i_hi > n ? n : i_hi;
    j_hi = j_hi > n ? n : j_hi;
    if (lane == 0 && part == 0) {
        // int(x) floors for x >= 0; centres lie in [0, no_xy).
        int64_t ix = (int64_t)x, iy = (int64_t)y;
        if (ix >= 0 && ix < n && iy >= 0 && iy < n) atomicAdd(counts + ix * n + iy, 1u);
    }
    const int64_t box_rows = i_hi - i_lo;
    const int64_t nrows = box_rows > part ? (box_rows - part + nparts - 1) / nparts : 0;
    for (int64_t jb = j_lo; jb < j_hi; jb += 32) {
        const int64_t j = jb + lane;
        const bool jok = j < j_hi;
        const T gj = jok ? gauss1((double)j - y, h2b2) : T(0);
        for (int64_t tb = 0; tb < nrows; tb += 32) {
            const int rows = (int)((nrows - tb) < 32 ? (nrows - tb) : 32);
            const int64_t i0 = i_lo + part + nparts * tb;  // row of r = 0
            const T gi_lane = lane < rows ? gauss1((double)(i0 + (int64_t)nparts * lane) - x, h2b2) : T(0);
            for (int r = 0; r < rows; ++r) {
                const T gi = __shfl_sync(0xffffffffu, gi_lane, r);
                if (jok) atomicAdd(dens + (i0 + (int64_t)nparts * r) * dp + j, gi * gj);
            }
        }
    }
}

}  // namespace pic
