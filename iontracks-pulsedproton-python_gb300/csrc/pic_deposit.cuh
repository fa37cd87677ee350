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
__device__ __forceinline__ float exp_neg(float a) { return expf(-a); }
__device__ __forceinline__ double exp_neg(double a) { return exp(-a); }

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

// ---------------------------------------------------------------------------
// Outer-product form of the deposition, for grids whose tracks overlap
// heavily (a small grid with hundreds of tracks a step: there the per-track
// form's atomics all land on the same few thousand cells and serialise in L2).
// Over a step's tracks t the pairs of cell (i, j) are sums of outer products,
//   c(i, j) = sum_t gx_t(i) Gy_t(j),
//   l(i, j) = sum_t hx_t(i) Gy_t(j) + gx_t(i) Hy_t(j),
// with gx_t the track's row factors, Gy_t = G gy_t its column factors,
// hx_t(i) = gx_t(i-1) + gx_t(i+1) and Hy_t(j) = Gy_t(j-1) + Gy_t(j+1) (the
// per-track terms of deposit_track). A block owns a kDepTile x kDepTile tile
// and a part of the step's tracks; it stages the factors of kDepBatch tracks
// that reach the tile at a time in shared memory, and each thread forms a
// 4 x 4 block of cells (rows and columns 16 apart) with 48 FMAs per track from
// 16 shared loads; at the end each cell's sums are added once per part.
constexpr int kDepTile = 64;      // cells per tile side
constexpr int kDepThreads = 256;  // 16 x 16 threads, 4 x 4 cells each
constexpr int kDepBatch = 16;     // tracks whose factors are staged together

__host__ __device__ inline int64_t deposit_tiles(int64_t n) {
    const int64_t t = (n + kDepTile - 1) / kDepTile;
    return t * t;
}
// Parts a tile's tracks are split into (one block each): one per
// kDepPartTracks tracks, at most 32. Every block scans its task's tracks and
// adds each cell of its tile once, so fewer, longer parts scan and add less,
// but more parts keep more SMs busy: the 64-configuration sweep's batched run
// took 1.27 s with parts of 32 tracks and 1.30-1.31 s with parts of 128.
constexpr int kDepPartTracks = 32;
__host__ __device__ inline int deposit_tile_parts(int64_t m) {
    const int64_t p = (m + kDepPartTracks - 1) / kDepPartTracks;
    return (int)(p < 1 ? 1 : (p > 32 ? 32 : p));
}

template <typename T>
struct DepTileShared {
    int sel[kDepThreads];  // tracks of the current chunk that reach the tile (offsets from t0)
    int wcount[kDepThreads / 32];
    int lo[kDepBatch][2], hi[kDepBatch][2], ci[kDepBatch][2];  // truncation box and centre cell per axis
    T cf[kDepBatch][2];                  // centre minus its cell, in [0, 1)
    T g[kDepBatch][2][kDepTile + 2];     // gx over rows i0-1 .. i0+kDepTile; Gy over the columns
    T h[kDepBatch][2][kDepTile];         // hx over rows i0 .. ; Hy over the columns
};

// Tracks [t0, t1) of the step into tile `tile` (row-major over the
// ceil(n / kDepTile)^2 tiles) of the pairs (zero on entry); counts (if
// non-null) once per track by the tile holding its centre column.
template <typename T>
__device__ __forceinline__ void deposit_tile(const double *__restrict__ xs, const double *__restrict__ ys, int64_t t0,
                                             int64_t t1, int64_t n, int64_t dp, double cut, T h2b2, T gfac,
                                             pair_t<T> *__restrict__ dens, uint32_t *__restrict__ counts, int64_t tile,
                                             DepTileShared<T> &sh) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t tr = (n + kDepTile - 1) / kDepTile;
    const int64_t i0 = (tile / tr) * kDepTile, j0 = (tile % tr) * kDepTile;
    const int ty = threadIdx.x >> 4, tx = threadIdx.x & 15;  // cells (i0 + ty + 16a, j0 + tx + 16b)
    T acc_c[4][4], acc_l[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc_c[a][b] = acc_l[a][b] = T(0);
    // conservative reach of a track's written box (truncation box widened by
    // one cell, plus a margin for the float test)
    const float reach = (float)cut + 2.0f;
    for (int64_t c0 = t0; c0 < t1; c0 += kDepThreads) {
        const int64_t t = c0 + threadIdx.x;
        bool hit = false;
        if (t < t1) {
            const double x = xs[t], y = ys[t];
            if (counts) {
                const int64_t ix = (int64_t)x, iy = (int64_t)y;  // int() floors for centres in [0, n)
                if (ix >= i0 && ix < i0 + kDepTile && iy >= j0 && iy < j0 + kDepTile && ix < n && iy < n)
                    atomicAdd(counts + ix * n + iy, 1u);
            }
            const float xf = (float)x, yf = (float)y;
            hit = xf + reach >= (float)i0 && xf - reach <= (float)(i0 + kDepTile - 1) && yf + reach >= (float)j0 &&
                  yf - reach <= (float)(j0 + kDepTile - 1);
        }
        // order-preserving compaction of this chunk's hits
        const unsigned bal = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) sh.wcount[warp] = __popc(bal);
        __syncthreads();
        int base = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kDepThreads / 32; ++w) {
            base += w < warp ? sh.wcount[w] : 0;
            total += sh.wcount[w];
        }
        if (hit) sh.sel[base + __popc(bal & ((1u << lane) - 1u))] = (int)(t - t0);
        __syncthreads();
        for (int b0 = 0; b0 < total; b0 += kDepBatch) {
            const int kb = total - b0 < kDepBatch ? total - b0 : kDepBatch;
            // per track and axis: the truncation box [ceil(c - cut), floor(c + cut)]
            // clipped to the grid (solver_numba.py:86-89), the centre's cell and
            // its offset in it (float64 once per track, the field type after)
            if (threadIdx.x < 2 * kDepBatch) {
                const int k = threadIdx.x >> 1, ax = threadIdx.x & 1;
                if (k < kb) {
                    const double c = ax ? ys[t0 + sh.sel[b0 + k]] : xs[t0 + sh.sel[b0 + k]];
                    const int64_t lo = (int64_t)ceil(c - cut), hi = (int64_t)floor(c + cut) + 1;
                    const double fl = floor(c);
                    sh.lo[k][ax] = (int)(lo < 0 ? 0 : lo);
                    sh.hi[k][ax] = (int)(hi > n ? n : hi);
                    sh.ci[k][ax] = (int)fl;
                    sh.cf[k][ax] = (T)(c - fl);
                }
            }
            __syncthreads();
            // the factors: g at offsets (cell - ci) - cf, an exact integer less
            // the centre's fraction, rounded once to the field type as
            // deposit_track rounds its float64 offset; zero outside the box
            for (int q = threadIdx.x; q < kDepBatch * 2 * (kDepTile + 2); q += kDepThreads) {
                const int k = q / (2 * (kDepTile + 2)), rem = q - k * 2 * (kDepTile + 2);
                const int ax = rem / (kDepTile + 2), e = rem - ax * (kDepTile + 2);
                T v = T(0);
                if (k < kb) {
                    const int cell = (int)(ax ? j0 : i0) - 1 + e;
                    if (cell >= sh.lo[k][ax] && cell < sh.hi[k][ax]) {
                        const T d = (T)(cell - sh.ci[k][ax]) - sh.cf[k][ax];
                        v = exp_neg(d * d * h2b2);
                        if (ax) v *= gfac;
                    }
                }
                sh.g[k][ax][e] = v;
            }
            __syncthreads();
            for (int q = threadIdx.x; q < kDepBatch * 2 * kDepTile; q += kDepThreads) {
                const int k = q / (2 * kDepTile), rem = q - k * 2 * kDepTile;
                const int ax = rem / kDepTile, e = rem - ax * kDepTile;
                sh.h[k][ax][e] = sh.g[k][ax][e] + sh.g[k][ax][e + 2];
            }
            __syncthreads();
            for (int k = 0; k < kb; ++k) {
                T gx[4], hx[4], gy[4], hy[4];
#pragma unroll
                for (int a = 0; a < 4; ++a) {
                    gx[a] = sh.g[k][0][ty + 16 * a + 1];
                    hx[a] = sh.h[k][0][ty + 16 * a];
                    gy[a] = sh.g[k][1][tx + 16 * a + 1];
                    hy[a] = sh.h[k][1][tx + 16 * a];
                }
#pragma unroll
                for (int a = 0; a < 4; ++a)
#pragma unroll
                    for (int b = 0; b < 4; ++b) {
                        acc_c[a][b] += gx[a] * gy[b];
                        acc_l[a][b] += hx[a] * gy[b] + gx[a] * hy[b];
                    }
            }
            __syncthreads();
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        const int64_t i = i0 + ty + 16 * a;
        if (i >= n) continue;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            const int64_t j = j0 + tx + 16 * b;
            if (j < n && (acc_c[a][b] != T(0) || acc_l[a][b] != T(0)))
                add_pair(dens + i * dp + j, acc_c[a][b], acc_l[a][b]);
        }
    }
}

}  // namespace pic
