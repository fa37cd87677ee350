// pic_binned.cuh -- the binned tile form of the deposition, shared by the
// single-grid launches (deposit.cu: up to kBinSteps steps of one grid per
// launch pair) and the batched step (batched.cu: the tracks of every grid of
// one global step per launch pair). deposit.cu describes what it computes.
//
// A launch pair serves a list of slots; a slot is one grid's tracks of one
// step with everything the kernels need of that grid. The first launch
// (bin_kernel) takes the launch's tracks four to a warp: it forms each
// track's truncation box and Gaussian factors once, counts its centre in its
// grid's histogram and lists it in every tile of its slot that its box meets.
// The second (binned_kernel) gives each tile of each slot one block.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pic_deposit.cuh"
#include "pic_internal.h"

namespace pic {

constexpr int kBinC = kBinOut + 2;  // density tile side: output cells and a one-cell halo
constexpr int kBinThreads = 256;    // 16 x 16 threads, 4 x 4 density cells each
constexpr int kBinBatch = 16;       // tracks whose factors are staged together
constexpr int kBinWarpTracks = 4;   // tracks per warp of the binning launch
constexpr int kBinChunk = 512;      // tracks whose boxes the tile block stages at once
static_assert(kBinC == 64 && kBinBox == 64, "a thread's 4 x 4 cells of 16 x 16 threads assume 64-cell tiles");

// One slot: a grid's tracks of one step. Launch track t of the slot (first
// <= t < last) has its centre at xs[t - first], ys[t - first].
template <typename T>
struct BinSlot {
    const double *xs, *ys;
    pair_t<T> *dens;     // the step's deposition pairs of this grid
    uint32_t *hist;      // the grid's track histogram (null: not counted)
    int *count;          // [tps^2] tracks listed per tile (zero between launches)
    int *list;           // [tps^2][kBinCap] launch track indices per tile
    int64_t first, last;
    double cut;          // truncation half-width in voxels
    T h2b2, gfac;        // h^2 / b^2 and G
    int32_t n, dp, tps;  // grid side, pair row pitch, tiles per side
    int32_t block0;      // the slot's first block in the tile launch
    int32_t add;         // 1: add to the pairs (a later piece of one step's tracks)
};

// The launch's per-track scratch: truncation boxes and factors (launch track
// index t: box[t], fac[t][2][kBinBox] = gx from lo_i, G gy from lo_j).
template <typename T>
struct BinScratch {
    short4 *box;
    T *fac;
};

// Slots passed by value (a segment's steps of one grid: at most kBinSteps).
template <typename T>
struct BinSlotsValue {
    BinSlot<T> s[kBinSteps];
    int count;
    int64_t tracks;  // the launch's tracks (the last slot's last)
    __device__ __forceinline__ const BinSlot<T> &operator[](int k) const { return s[k]; }
    __device__ __forceinline__ int of_track(int64_t t) const {
        int k = 0;
        while (k + 1 < count && s[k + 1].first <= t) ++k;
        return k;
    }
    __device__ __forceinline__ int of_block(int64_t b) const {
        int k = 0;
        while (k + 1 < count && s[k + 1].block0 <= b) ++k;
        return k;
    }
};

// Slots in device memory (a batched global step's grids, written by the
// step's preparation kernel): binary searches over first and block0.
template <typename T>
struct BinSlotsDevice {
    const BinSlot<T> *s;
    int count;
    int64_t tracks;
    __device__ __forceinline__ const BinSlot<T> &operator[](int k) const { return s[k]; }
    __device__ __forceinline__ int of_track(int64_t t) const {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s[mid].first <= t) lo = mid; else hi = mid - 1;
        }
        return lo;
    }
    __device__ __forceinline__ int of_block(int64_t b) const {
        int lo = 0, hi = count - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s[mid].block0 <= b) lo = mid; else hi = mid - 1;
        }
        return lo;
    }
};

// The two launches over `slots` (deposit.cu): the binning, then `blocks`
// tile blocks (at least the slots' tiles; blocks past a slot's tiles exit).
template <typename T, typename S>
int binned_launches(const S &slots, const BinScratch<T> &sc, int64_t blocks, cudaStream_t st);

// The truncation box [lo, hi) of a track along one axis, clipped to the grid
// (solver_numba.py:86-89).
__device__ __forceinline__ void track_box(double c, double cut, int64_t n, int64_t &lo, int64_t &hi) {
    lo = (int64_t)ceil(c - cut);
    hi = (int64_t)floor(c + cut) + 1;
    lo = lo < 0 ? 0 : lo;
    hi = hi > n ? n : hi;
}

// A warp per kBinWarpTracks tracks. Lane 2 q + a forms track q's box along
// axis a (i, j) and the centre's cell and offset (float64, one lane per track
// and axis); then for each track every lane forms two row and two column
// factors, g at offsets (cell - ci) - cf as in deposit_tile (zero past the
// box); the centre is counted once, and lanes 2 q and 2 q + 1 list track q in
// every tile of its slot whose density rows [62 t - 1, 62 t + 63) and columns
// meet its box.
template <typename T, typename S>
__global__ void __launch_bounds__(256) bin_kernel(S slots, BinScratch<T> sc) {
    const int lane = threadIdx.x & 31, ax = lane & 1;
    const int64_t m = slots.tracks;
    const int64_t t0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * kBinWarpTracks;
    if (t0 >= m) return;
    const int64_t tl = t0 + (lane >> 1);
    int lo = 0, hi = 0, ci = 0, k = 0;
    T cf = T(0);
    if (lane < 2 * kBinWarpTracks && tl < m) {
        k = slots.of_track(tl);
        const BinSlot<T> &Sl = slots[k];
        const double c = (ax ? Sl.ys : Sl.xs)[tl - Sl.first];
        int64_t a, b;
        track_box(c, Sl.cut, Sl.n, a, b);
        const double fl = floor(c);
        lo = (int)a, hi = (int)b, ci = (int)fl;
        cf = (T)(c - fl);
    }
    const int nt = m - t0 < kBinWarpTracks ? (int)(m - t0) : kBinWarpTracks;
    for (int q = 0; q < nt; ++q) {
        const int64_t t = t0 + q;
        const int lo_i = __shfl_sync(0xffffffffu, lo, 2 * q), hi_i = __shfl_sync(0xffffffffu, hi, 2 * q);
        const int lo_j = __shfl_sync(0xffffffffu, lo, 2 * q + 1), hi_j = __shfl_sync(0xffffffffu, hi, 2 * q + 1);
        const int ci_i = __shfl_sync(0xffffffffu, ci, 2 * q), ci_j = __shfl_sync(0xffffffffu, ci, 2 * q + 1);
        const T cf_i = __shfl_sync(0xffffffffu, cf, 2 * q), cf_j = __shfl_sync(0xffffffffu, cf, 2 * q + 1);
        const int kq = __shfl_sync(0xffffffffu, k, 2 * q);
        const BinSlot<T> &Sq = slots[kq];
        const T h2b2 = Sq.h2b2, gfac = Sq.gfac;
        T *F = sc.fac + t * (2 * kBinBox);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int e = lane + 32 * h;
            T gx = T(0), gy = T(0);
            if (lo_i + e < hi_i) {
                const T d = (T)(lo_i + e - ci_i) - cf_i;
                gx = exp_neg(d * d * h2b2);
            }
            if (lo_j + e < hi_j) {
                const T d = (T)(lo_j + e - ci_j) - cf_j;
                gy = exp_neg(d * d * h2b2) * gfac;
            }
            F[e] = gx;
            F[kBinBox + e] = gy;
        }
        if (lane == 0) {
            sc.box[t] = make_short4((short)lo_i, (short)hi_i, (short)lo_j, (short)hi_j);
            // int(x) floors for centres in [0, n)
            const int n = Sq.n;
            if (Sq.hist && ci_i >= 0 && ci_i < n && ci_j >= 0 && ci_j < n)
                atomicAdd(Sq.hist + (int64_t)ci_i * n + ci_j, 1u);
        }
    }
    // the tiles of track lane / 2, split between its two lanes
    const int lo_i = __shfl_sync(0xffffffffu, lo, lane & ~1), hi_i = __shfl_sync(0xffffffffu, hi, lane & ~1);
    const int lo_j = __shfl_sync(0xffffffffu, lo, lane | 1), hi_j = __shfl_sync(0xffffffffu, hi, lane | 1);
    const int q = lane >> 1;
    if (q >= nt || lo_i >= hi_i || lo_j >= hi_j) return;
    const BinSlot<T> &Sl = slots[k];
    const int T_ = Sl.tps;
    // tile t meets [lo, hi) iff kBinOut t - 1 < hi and kBinOut t + kBinC - 1 > lo
    const int ti0 = lo_i >= kBinC - 1 ? (lo_i - (kBinC - 1)) / kBinOut + 1 : 0;
    const int tj0 = lo_j >= kBinC - 1 ? (lo_j - (kBinC - 1)) / kBinOut + 1 : 0;
    const int ti1 = hi_i / kBinOut < T_ - 1 ? hi_i / kBinOut : T_ - 1;
    const int tj1 = hi_j / kBinOut < T_ - 1 ? hi_j / kBinOut : T_ - 1;
    const int nj = tj1 - tj0 + 1, ntiles = (ti1 - ti0 + 1) * nj;
    const int t = (int)(t0 + q);
    int *count = Sl.count;
    int *list = Sl.list;
    // the first two tiles of this lane: both counters bumped before either
    // list entry is written (one round trip), the rest one at a time
    const int qa = ax, qb = ax + 2;
    const int64_t ta = qa < ntiles ? (int64_t)(ti0 + qa / nj) * T_ + tj0 + qa % nj : -1;
    const int64_t tb = qb < ntiles ? (int64_t)(ti0 + qb / nj) * T_ + tj0 + qb % nj : -1;
    const int sa = ta >= 0 ? atomicAdd(count + ta, 1) : kBinCap;
    const int sb = tb >= 0 ? atomicAdd(count + tb, 1) : kBinCap;
    if (sa < kBinCap) list[ta * kBinCap + sa] = t;
    if (sb < kBinCap) list[tb * kBinCap + sb] = t;
    for (int qq = ax + 4; qq < ntiles; qq += 2) {
        const int64_t tile = (int64_t)(ti0 + qq / nj) * T_ + tj0 + qq % nj;
        const int e = atomicAdd(count + tile, 1);
        if (e < kBinCap) list[tile * kBinCap + e] = t;
    }
}

// A thread's 4 x 4 density cells (rows 4 ty + a, columns 4 tx + b) and the
// outer-product update of one track: float in packed FP32x2 FMAs (each lane
// rounded as fmaf), double in plain FMAs.
template <typename T>
struct BinAcc;
template <>
struct BinAcc<float> {
    float2 c[4][2];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < 4; ++a) c[a][0] = c[a][1] = make_float2(0.f, 0.f);
    }
    __device__ __forceinline__ void add(const float *gx, const float *gy) {
        const float4 x = *reinterpret_cast<const float4 *>(gx), y = *reinterpret_cast<const float4 *>(gy);
        const float2 y01 = make_float2(y.x, y.y), y23 = make_float2(y.z, y.w);
        const float xa[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            const float2 xx = make_float2(xa[a], xa[a]);
            c[a][0] = __ffma2_rn(xx, y01, c[a][0]);
            c[a][1] = __ffma2_rn(xx, y23, c[a][1]);
        }
    }
    __device__ __forceinline__ float get(int a, int b) const { return (b & 1) ? c[a][b >> 1].y : c[a][b >> 1].x; }
};
template <>
struct BinAcc<double> {
    double c[4][4];
    __device__ __forceinline__ void zero() {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) c[a][b] = 0.0;
    }
    __device__ __forceinline__ void add(const double *gx, const double *gy) {
        const double2 x0 = *reinterpret_cast<const double2 *>(gx), x1 = *reinterpret_cast<const double2 *>(gx + 2);
        const double2 y0 = *reinterpret_cast<const double2 *>(gy), y1 = *reinterpret_cast<const double2 *>(gy + 2);
        const double xa[4] = {x0.x, x0.y, x1.x, x1.y}, yb[4] = {y0.x, y0.y, y1.x, y1.y};
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) c[a][b] = fma(xa[a], yb[b], c[a][b]);
    }
    __device__ __forceinline__ double get(int a, int b) const { return c[a][b]; }
};


// Dynamic shared memory of deposit_binned_kernel: the tile's track list
// (later the density tile), two buffers of staged factors, and the boxes of a
// chunk of tracks.
template <typename T>
struct BinSmem {
    static constexpr int kListBytes = kBinCap * 4;
    static constexpr int kTileBytes = kBinC * (kBinC + 1) * (int)sizeof(T);
    static constexpr int kUnion = ((kListBytes > kTileBytes ? kListBytes : kTileBytes) + 15) / 16 * 16;
    static constexpr int kFactorBytes = 2 * kBinBatch * 2 * kBinC * (int)sizeof(T);
    static constexpr int kBoxBytes = 4 * kBinChunk * 2;  // int16: lo_i hi_i lo_j hi_j
    static constexpr int kBytes = kUnion + kFactorBytes + kBoxBytes + (kBinThreads / 32) * 4;
};

// A block per tile of a slot: the tile's tracks in ascending index order
// (sorted in shared memory), their factor windows staged 16 at a time and
// prefetched one batch ahead, c = sum gx Gy as outer products, then each
// output cell's pair (c and its four neighbours' sum) stored once (added,
// for a later piece of one step).
template <typename T, typename S>
__global__ void __launch_bounds__(kBinThreads) binned_kernel(S slots, BinScratch<T> sc) {
    extern __shared__ __align__(16) unsigned char bin_smem[];
    using SM = BinSmem<T>;
    constexpr int C = kBinChunk, FB = kBinBatch * 2 * kBinC;  // factors per buffer
    int *list = reinterpret_cast<int *>(bin_smem);
    T *ctile = reinterpret_cast<T *>(bin_smem);  // [kBinC][kBinC + 1], after the sums
    T *fac = reinterpret_cast<T *>(bin_smem + SM::kUnion);  // [2][kBinBatch][2][kBinC]
    short *mbox = reinterpret_cast<short *>(fac + 2 * FB);  // [4][C]: lo_i hi_i lo_j hi_j
    int *wcount = reinterpret_cast<int *>(mbox + 4 * C);
    __shared__ int s_count;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int k = slots.of_block(blockIdx.x);
    const BinSlot<T> &SL = slots[k];
    const int tps = SL.tps;
    const int64_t tile = (int64_t)blockIdx.x - SL.block0;
    if (tile >= (int64_t)tps * tps) return;  // past the slot's tiles (a launch sized for the largest grid)
    const int64_t n = SL.n, dp = SL.dp;
    const int i0 = (int)((tile / tps) * kBinOut - 1), j0 = (int)((tile % tps) * kBinOut - 1);
    int *count = SL.count + tile;
    const int *tile_list = SL.list + tile * kBinCap;
    pair_t<T> *__restrict__ dens = SL.dens;
    const int add = SL.add;
    const int64_t m0 = SL.first, m1 = SL.last;
    if (tid == 0) s_count = *count;
    __syncthreads();
    const int cnt = s_count;
    if (cnt == 0) {
        // no track reaches the tile: zero pairs (or, adding, nothing)
        if (!add)
            for (int q = tid; q < kBinOut * kBinOut; q += kBinThreads) {
                const int64_t i = i0 + 1 + q / kBinOut, j = j0 + 1 + q % kBinOut;
                if (i < n && j < n) dens[i * dp + j] = pair_t<T>{T(0), T(0)};
            }
        return;
    }

    const int ty = tid >> 4, tx = tid & 15;  // density cells (4 ty + a, 4 tx + b)
    BinAcc<T> acc;
    acc.zero();

    // Factors of the staged chunk's tracks b0 .. b0 + kBinBatch - 1 (k of
    // them) over the tile's rows and columns: a warp takes (track, axis)
    // pairs warp, warp + 8, ..., its lanes cells lane and lane + 32 (zero past
    // the box).
    constexpr int PPW = 2 * kBinBatch / (kBinThreads / 32);  // pairs per warp
    auto load = [&](const int *idx, int b0, int k, T v[2 * PPW]) {
#pragma unroll
        for (int u = 0; u < PPW; ++u) {
            const int p = warp + u * (kBinThreads / 32), r = b0 + (p >> 1), ax = p & 1;
            v[2 * u] = v[2 * u + 1] = T(0);
            if (r < k) {
                const int lo = mbox[(2 * ax) * C + r], w = mbox[(2 * ax + 1) * C + r] - lo;
                const int off = (ax ? j0 : i0) - lo;
                const T *F = sc.fac + (int64_t)idx[r] * (2 * kBinBox) + ax * kBinBox;
                const int k0 = off + lane, k1 = off + lane + 32;
                if (k0 >= 0 && k0 < w) v[2 * u] = F[k0];
                if (k1 >= 0 && k1 < w) v[2 * u + 1] = F[k1];
            }
        }
    };
    auto store = [&](int buf, const T v[2 * PPW]) {
        T *f = fac + buf * FB;
#pragma unroll
        for (int u = 0; u < PPW; ++u) {
            const int p = warp + u * (kBinThreads / 32);
            f[p * kBinC + lane] = v[2 * u];
            f[p * kBinC + lane + 32] = v[2 * u + 1];
        }
    };
    // Sums the tracks idx[0 .. k) (k <= C, in this order) into acc.
    auto sum_chunk = [&](const int *idx, int k) {
        for (int q = tid; q < k; q += kBinThreads) {
            const short4 b = sc.box[idx[q]];
            mbox[q] = b.x, mbox[C + q] = b.y, mbox[2 * C + q] = b.z, mbox[3 * C + q] = b.w;
        }
        __syncthreads();
        T v[2 * PPW];
        if (k > 0) {
            load(idx, 0, k, v);
            store(0, v);
        }
        __syncthreads();
        for (int b0 = 0, buf = 0; b0 < k; b0 += kBinBatch, buf ^= 1) {
            const bool more = b0 + kBinBatch < k;
            if (more) load(idx, b0 + kBinBatch, k, v);  // in flight while this batch is summed
            // a whole batch: the slots past the chunk's last track hold zeros
            const T *f = fac + buf * FB;
#pragma unroll
            for (int q = 0; q < kBinBatch; ++q) acc.add(f + (2 * q) * kBinC + 4 * ty, f + (2 * q + 1) * kBinC + 4 * tx);
            if (more) store(buf ^ 1, v);
            __syncthreads();
        }
    };

    if (cnt <= kBinCap) {
        for (int q = tid; q < cnt; q += kBinThreads) list[q] = tile_list[q];
        __syncthreads();
        // ascending track order: rank sort for short lists, bitonic otherwise
        if (cnt <= kBinThreads) {
            int v = 0, r = 0;
            if (tid < cnt) {
                v = list[tid];
                for (int q = 0; q < cnt; ++q) r += list[q] < v;
            }
            __syncthreads();
            if (tid < cnt) list[r] = v;
        } else {
            int p2 = kBinThreads;
            while (p2 < cnt) p2 <<= 1;
            for (int q = cnt + tid; q < p2; q += kBinThreads) list[q] = 0x7fffffff;
            __syncthreads();
            for (int k = 2; k <= p2; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int q = tid; q < p2; q += kBinThreads) {
                        const int o = q ^ j;
                        if (o > q) {
                            const int a = list[q], b = list[o];
                            if ((a > b) == ((q & k) == 0)) {
                                list[q] = b;
                                list[o] = a;
                            }
                        }
                    }
                    __syncthreads();
                }
        }
        __syncthreads();
        for (int c0 = 0; c0 < cnt; c0 += C) sum_chunk(list + c0, cnt - c0 < C ? cnt - c0 : C);
    } else {
        // more tracks than the list holds: scan the slot's tracks in order, a
        // chunk of kBinThreads at a time, keeping those whose box meets the tile
        for (int64_t c0 = m0; c0 < m1; c0 += kBinThreads) {
            const int64_t t = c0 + tid;
            bool hit = false;
            if (t < m1) {
                const short4 b = sc.box[t];
                hit = b.x < b.y && b.z < b.w && b.x < i0 + kBinC && b.y > i0 && b.z < j0 + kBinC && b.w > j0;
            }
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (lane == 0) wcount[warp] = __popc(bal);
            __syncthreads();
            int base = 0, total = 0;
#pragma unroll
            for (int w = 0; w < kBinThreads / 32; ++w) {
                base += w < warp ? wcount[w] : 0;
                total += wcount[w];
            }
            if (hit) list[base + __popc(bal & ((1u << lane) - 1u))] = (int)t;
            __syncthreads();
            sum_chunk(list, total);
        }
    }

    // the density tile, then each output cell's pair: c and its four
    // neighbours' sum (a warp per row, its lanes along the row)
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) ctile[(4 * ty + a) * (kBinC + 1) + 4 * tx + b] = acc.get(a, b);
    __syncthreads();
    for (int r = 1 + warp; r <= kBinOut; r += kBinThreads / 32) {
        const int64_t i = i0 + r;
        if (i >= n) break;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = 1 + lane + 32 * h;
            const int64_t j = j0 + c;
            if (c > kBinOut || j >= n) continue;
            const T *row = ctile + r * (kBinC + 1) + c;
            const T l = (row[-(kBinC + 1)] + row[kBinC + 1]) + (row[-1] + row[1]);
            pair_t<T> *d = dens + i * dp + j;
            pair_t<T> v;
            if (add) {
                v = *d;
                v.x += row[0];
                v.y += l;
            } else {
                v.x = row[0];
                v.y = l;
            }
            *d = v;
        }
    }
    if (tid == 0) *count = 0;  // the next binning starts from zero
}

}  // namespace pic
