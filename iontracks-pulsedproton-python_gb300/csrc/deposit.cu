// deposit.cu -- one step's Gaussian ion tracks summed into the 2D density.
//
// A track is a line through the whole gap at constant LET, so its density is
// the same in every gap layer: only the (i, j) cross-section is accumulated
// here (already multiplied by gaussian_factor), and the fused step adds it to
// each gap layer as it reads the fields. The cross-section is separable,
//   exp(-((i-x)^2 + (j-y)^2) h^2/b^2) = g_i * g_j,
// so a track costs one exponential per stencil row and column and one multiply
// per cell (the identities of solver_numba.py:10-26). The stencil box is
// [ceil(x - cut), floor(x + cut)] clipped to [0, no_xy), as in
// solver_numba.py:86-89.
//
// The deposition is laid out [no_xy][dens_pitch(no_xy)] pairs (G * density,
// G * the density of the four lateral neighbours; rows padded to 4 pairs).
// Three forms. Binned tiles (large grids, where a step's thousands of tracks
// overlap on many cells; needs the step workspace): described at
// deposit_binned_kernel below. Per track (large grids, tracks spread over many cells): one to
// eight warps per track (more when the step has few tracks), splitting the
// box's rows. Lanes own stencil columns j; row factors are computed 32 rows at
// a time, one row per lane, and broadcast by shuffle. Each cell's pair is
// added with one vector atomic: tracks overlap, and the L2 resolves the
// collisions. Per tile (small grids, where hundreds of tracks a step pile onto
// the same cells and those atomics serialise): a block sums every track that
// reaches its 64 x 64 tile as sums of outer products of the tracks' row and
// column factors, in registers, and adds each cell once per part
// (deposit_tile in pic_deposit.cuh). In both, the offset (i - x) is formed
// from the float64 track centre before it is rounded, so the Gaussian is not
// shifted by the float32 spacing of x (up to 6e-5 voxel at x ~ 1000).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pic_deposit.cuh"
#include "pic_device.cuh"
#include "pic_internal.h"

namespace pic {

// `parts` warps per track (a power of two dividing WARPS).
template <typename T, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) deposit_kernel(const double *__restrict__ xs,
                                                              const double *__restrict__ ys, int64_t m,
                                                              pair_t<T> *__restrict__ dens,
                                                              uint32_t *__restrict__ counts, int64_t n, int64_t dp,
                                                              double cut, T h2b2, T gfac, int parts) {
    const int warp = threadIdx.x >> 5;
    const int64_t t = (int64_t)blockIdx.x * (WARPS / parts) + warp / parts;
    if (t >= m) return;
    deposit_track<T>(xs[t], ys[t], n, dp, cut, h2b2, gfac, dens, counts, threadIdx.x & 31, warp % parts, parts);
}


// The tile form (pic_deposit.cuh): block b sums part b % parts of the tracks
// into tile b / parts.
template <typename T>
__global__ void __launch_bounds__(kDepThreads) deposit_tile_kernel(const double *__restrict__ xs,
                                                                   const double *__restrict__ ys, int64_t m,
                                                                   pair_t<T> *__restrict__ dens,
                                                                   uint32_t *__restrict__ counts, int64_t n,
                                                                   int64_t dp, double cut, T h2b2, T gfac, int parts) {
    __shared__ DepTileShared<T> sh;
    const int64_t tile = blockIdx.x / parts;
    const int part = (int)(blockIdx.x % parts);
    deposit_tile<T>(xs, ys, m * part / parts, m * (part + 1) / parts, n, dp, cut, h2b2, gfac, dens, counts, tile,
                    sh);
}

// ---------------------------------------------------------------------------
// Binned tile form, for large grids (one grid of ~10^6 cells and thousands of
// tracks a step, each over a 57 x 57 box: the per-track form's ~27 M vector
// atomics a step are its cost). Over a step's tracks t the density is
//   c(i, j) = sum_t gx_t(i) Gy_t(j)   (Gy = G gy),
// and the neighbours' sum of the per-track form,
//   sum_t (gx_t(i-1) + gx_t(i+1)) Gy_t(j) + gx_t(i) (Gy_t(j-1) + Gy_t(j+1)),
// is c(i-1, j) + c(i+1, j) + c(i, j-1) + c(i, j+1): with the factors zero
// outside each track's box, both are the same sums of the same products. So a
// block forms c on a 64 x 64 tile (its 62 x 62 output cells and a one-cell
// halo), one FMA per cell and track, and the neighbours' sum from the tile
// afterwards. deposit_bin_kernel evaluates each track's factors once (a track
// meets about four tiles) and lists the track in the tiles it reaches; the
// tile's block takes its tracks in ascending index order (the lists are
// sorted in shared memory), so the result does not depend on the order the
// binning's atomics ran in: two runs give identical pairs. Every cell of a
// tile some track reaches is stored once, without atomics; a tile no track
// reaches is left as it is (zero: the buffer is zero on entry, as for the
// other forms). One pair of launches serves up to kBinSteps steps of a
// segment, one slot each (BinLaunch), which gives the GPU eight times the
// blocks of one step; a step with more than kBinTracks tracks runs in pieces,
// the later ones adding to the cells the first stored.
constexpr int kBinC = kBinOut + 2;  // density tile side: output cells and a one-cell halo
constexpr int kBinThreads = 256;    // 16 x 16 threads, 4 x 4 density cells each
constexpr int kBinBatch = 16;       // tracks whose factors are staged together
static_assert(kBinC == 64 && kBinBox == 64, "a thread's 4 x 4 cells of 16 x 16 threads assume 64-cell tiles");

template <typename T>
struct DepBins {
    int *count;     // [kBinSteps][tiles]
    int *list;      // [kBinSteps][tiles][kBinCap], track indices within the launch
    short4 *box;    // [kBinTracks]: lo_i, hi_i, lo_j, hi_j (the truncation box)
    T *fac;         // [kBinTracks][2][kBinBox]: gx from lo_i, G gy from lo_j
    char *dens;     // [kBinSteps] pair buffers of bin_dens_bytes
    int64_t tps;    // tiles per side
    int64_t tiles;  // tps^2
};
template <typename T>
inline DepBins<T> dep_bins(void *ws, int64_t n) {
    const int64_t es = sizeof(T);
    char *b = static_cast<char *>(ws) + kWorkspaceBytes;
    char *list = b + bin_count_bytes(n), *box = list + bin_list_bytes(n), *fac = box + bin_box_bytes();
    char *dens = fac + bin_fac_bytes(es);
    const int64_t t = bin_tiles_per_side(n);
    return DepBins<T>{reinterpret_cast<int *>(b), reinterpret_cast<int *>(list), reinterpret_cast<short4 *>(box),
                      reinterpret_cast<T *>(fac), dens, t, t * t};
}

// The slots of one pair of binned launches: slot k holds the launch's tracks
// [first[k], first[k + 1]) (counted from the launch's first track) and writes
// its pairs to dens[k]. add = 0: every cell of every tile is stored (zero
// where no track reaches); add = 1 (a later piece of one step): the sums are
// added to the cells and tiles no track reaches are left alone.
template <typename T>
struct BinLaunch {
    int64_t first[kBinSteps + 1];
    pair_t<T> *dens[kBinSteps];
    int slots;
    int add;
};

// The truncation box [lo, hi) of a track along one axis, clipped to the grid
// (solver_numba.py:86-89).
__device__ __forceinline__ void track_box(double c, double cut, int64_t n, int64_t &lo, int64_t &hi) {
    lo = (int64_t)ceil(c - cut);
    hi = (int64_t)floor(c + cut) + 1;
    lo = lo < 0 ? 0 : lo;
    hi = hi > n ? n : hi;
}

// A warp per kBinWarpTracks tracks. Lane 2 q + a forms track q's box along axis a (i, j)
// and the centre's cell and offset (float64, one lane per track and axis);
// then for each track every lane forms two row and two column factors, g at
// offsets (cell - ci) - cf as in deposit_tile (zero past the box); the centre
// is counted once, and lanes 2 q and 2 q + 1 list track q in every tile whose
// density rows [62 t - 1, 62 t + 63) and columns meet its box.
constexpr int kBinWarpTracks = 4;
template <typename T>
__global__ void __launch_bounds__(256) deposit_bin_kernel(const double *__restrict__ xs,
                                                          const double *__restrict__ ys, int64_t n, double cut,
                                                          T h2b2, T gfac, uint32_t *__restrict__ counts,
                                                          DepBins<T> bins, BinLaunch<T> L) {
    const int lane = threadIdx.x & 31, ax = lane & 1;
    const int64_t m = L.first[L.slots];
    const int64_t t0 = ((int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * kBinWarpTracks;
    if (t0 >= m) return;
    const int64_t tl = t0 + (lane >> 1);
    int lo = 0, hi = 0, ci = 0;
    T cf = T(0);
    if (lane < 2 * kBinWarpTracks && tl < m) {
        const double c = ax ? ys[tl] : xs[tl];
        int64_t a, b;
        track_box(c, cut, n, a, b);
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
        T *F = bins.fac + t * (2 * kBinBox);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int k = lane + 32 * h;
            T gx = T(0), gy = T(0);
            if (lo_i + k < hi_i) {
                const T d = (T)(lo_i + k - ci_i) - cf_i;
                gx = exp_neg(d * d * h2b2);
            }
            if (lo_j + k < hi_j) {
                const T d = (T)(lo_j + k - ci_j) - cf_j;
                gy = exp_neg(d * d * h2b2) * gfac;
            }
            F[k] = gx;
            F[kBinBox + k] = gy;
        }
        if (lane == 0) {
            bins.box[t] = make_short4((short)lo_i, (short)hi_i, (short)lo_j, (short)hi_j);
            // int(x) floors for centres in [0, n)
            if (counts && ci_i >= 0 && ci_i < n && ci_j >= 0 && ci_j < n)
                atomicAdd(counts + (int64_t)ci_i * n + ci_j, 1u);
        }
    }
    // the tiles of track lane / 2, split between its two lanes
    const int lo_i = __shfl_sync(0xffffffffu, lo, lane & ~1), hi_i = __shfl_sync(0xffffffffu, hi, lane & ~1);
    const int lo_j = __shfl_sync(0xffffffffu, lo, lane | 1), hi_j = __shfl_sync(0xffffffffu, hi, lane | 1);
    const int q = lane >> 1;
    if (q >= nt || lo_i >= hi_i || lo_j >= hi_j) return;
    const int T_ = (int)bins.tps;
    // tile t meets [lo, hi) iff kBinOut t - 1 < hi and kBinOut t + kBinC - 1 > lo
    const int ti0 = lo_i >= kBinC - 1 ? (lo_i - (kBinC - 1)) / kBinOut + 1 : 0;
    const int tj0 = lo_j >= kBinC - 1 ? (lo_j - (kBinC - 1)) / kBinOut + 1 : 0;
    const int ti1 = hi_i / kBinOut < T_ - 1 ? hi_i / kBinOut : T_ - 1;
    const int tj1 = hi_j / kBinOut < T_ - 1 ? hi_j / kBinOut : T_ - 1;
    const int nj = tj1 - tj0 + 1, ntiles = (ti1 - ti0 + 1) * nj;
    const int t = (int)(t0 + q);
    int k = 0;  // the track's slot
    while (k + 1 < L.slots && L.first[k + 1] <= t) ++k;
    int *count = bins.count + k * bins.tiles;
    int *list = bins.list + k * bins.tiles * kBinCap;
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

constexpr int kBinChunk = 512;  // tracks whose boxes are staged at once

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

template <typename T>
__global__ void __launch_bounds__(kBinThreads) deposit_binned_kernel(int64_t n, int64_t dp, DepBins<T> bins,
                                                                     BinLaunch<T> L) {
    extern __shared__ __align__(16) unsigned char bin_smem[];
    using S = BinSmem<T>;
    constexpr int C = kBinChunk, FB = kBinBatch * 2 * kBinC;  // factors per buffer
    int *list = reinterpret_cast<int *>(bin_smem);
    T *ctile = reinterpret_cast<T *>(bin_smem);  // [kBinC][kBinC + 1], after the sums
    T *fac = reinterpret_cast<T *>(bin_smem + S::kUnion);  // [2][kBinBatch][2][kBinC]
    short *mbox = reinterpret_cast<short *>(fac + 2 * FB);  // [4][C]: lo_i hi_i lo_j hi_j
    int *wcount = reinterpret_cast<int *>(mbox + 4 * C);
    __shared__ int s_count;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int slot = (int)(blockIdx.x / bins.tiles);
    const int64_t tile = blockIdx.x - slot * bins.tiles;
    const int i0 = (int)((tile / bins.tps) * kBinOut - 1), j0 = (int)((tile % bins.tps) * kBinOut - 1);
    int *count = bins.count + slot * bins.tiles + tile;
    const int *tile_list = bins.list + (slot * bins.tiles + tile) * kBinCap;
    pair_t<T> *__restrict__ dens = L.dens[slot];
    const int add = L.add;
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
                const T *F = bins.fac + (int64_t)idx[r] * (2 * kBinBox) + ax * kBinBox;
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
            const short4 b = bins.box[idx[q]];
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
        const int64_t m0 = L.first[slot], m1 = L.first[slot + 1];
        for (int64_t c0 = m0; c0 < m1; c0 += kBinThreads) {
            const int64_t t = c0 + tid;
            bool hit = false;
            if (t < m1) {
                const short4 b = bins.box[t];
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

template <typename T>
int binned_launches(const pic_grid *g, const double *xs, const double *ys, uint32_t *counts, const DepBins<T> &bins,
                    const BinLaunch<T> &L, cudaStream_t st) {
    constexpr int smem = BinSmem<T>::kBytes;
    static int configured = 0;  // per instantiation
    if (smem > 48 * 1024 && !configured) {
        cudaError_t e =
            cudaFuncSetAttribute(deposit_binned_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(deposit_binned_kernel)", e);
        configured = 1;
    }
    const int64_t warps = (L.first[L.slots] + kBinWarpTracks - 1) / kBinWarpTracks;
    deposit_bin_kernel<T><<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(
        xs, ys, g->no_xy, g->cutoff_voxels, (T)g->h2_over_b2, (T)g->gaussian_factor, counts, bins, L);
    int rc = check_launch("deposit_bin_kernel");
    if (rc) return rc;
    deposit_binned_kernel<T><<<(unsigned)(L.slots * bins.tiles), kBinThreads, smem, st>>>(
        g->no_xy, dens_pitch(g->no_xy), bins, L);
    return check_launch("deposit_binned_kernel");
}

// One step's tracks into the caller's pairs, in pieces of kBinTracks.
template <typename T>
int launch_binned(const pic_grid *g, const double *xs, const double *ys, int64_t m, void *dens, uint32_t *counts,
                  void *ws, cudaStream_t st) {
    const DepBins<T> bins = dep_bins<T>(ws, g->no_xy);
    for (int64_t g0 = 0; g0 < m; g0 += kBinTracks) {
        BinLaunch<T> L{};
        L.slots = 1;
        L.first[0] = 0;
        L.first[1] = m - g0 < kBinTracks ? m - g0 : kBinTracks;
        L.dens[0] = static_cast<pair_t<T> *>(dens);
        L.add = g0 > 0;
        int rc = binned_launches<T>(g, xs + g0, ys + g0, counts, bins, L, st);
        if (rc) return rc;
    }
    return PIC_OK;
}

template <typename T>
int launch_binned_steps(const pic_grid *g, const double *xs, const double *ys, const int64_t *off, int64_t s0,
                        int64_t s1, uint32_t *counts, void *ws, void *const *targets, const void **dens,
                        cudaStream_t st) {
    const DepBins<T> bins = dep_bins<T>(ws, g->no_xy);
    const int64_t slot_bytes = bin_dens_bytes(g->no_xy, sizeof(T));
    BinLaunch<T> L{};
    L.add = 0;
    int k = 0;
    for (int64_t s = s0; s < s1; ++s) {
        dens[s - s0] = nullptr;
        if (off[s + 1] == off[s]) continue;
        if (k == kBinSteps) return set_error(PIC_E_INVALID, "more than kBinSteps depositing steps in one launch");
        L.first[k] = off[s] - off[s0];
        L.dens[k] = reinterpret_cast<pair_t<T> *>(targets ? static_cast<char *>(targets[k]) : bins.dens + k * slot_bytes);
        dens[s - s0] = L.dens[k];
        ++k;
    }
    if (k == 0) return PIC_OK;
    L.slots = k;
    L.first[k] = off[s1] - off[s0];
    if (L.first[k] > kBinTracks) return set_error(PIC_E_INVALID, "more than kBinTracks tracks in one launch");
    return binned_launches<T>(g, xs + off[s0], ys + off[s0], counts, bins, L, st);
}

int launch_deposit_steps(const pic_grid *g, const double *xs, const double *ys, const int64_t *off, int64_t s0,
                         int64_t s1, uint32_t *counts, void *ws, void *const *targets, const void **dens,
                         cudaStream_t st) {
    return g->dtype == PIC_F64 ? launch_binned_steps<double>(g, xs, ys, off, s0, s1, counts, ws, targets, dens, st)
                               : launch_binned_steps<float>(g, xs, ys, off, s0, s1, counts, ws, targets, dens, st);
}

int64_t next_deposit_group(const int64_t *off, int64_t s0, int64_t n_steps, int64_t *n_dep) {
    int64_t s1 = s0, nd = 0;
    while (s1 < n_steps && s1 - s0 < kBinSpan) {
        const int64_t m = off[s1 + 1] - off[s1];
        if (m > 0 && (nd == kBinSteps || off[s1 + 1] - off[s0] > kBinTracks)) break;
        nd += m > 0;
        ++s1;
    }
    *n_dep = nd;
    return s1;
}

bool deposit_binned(const pic_grid *g, const void *ws, int64_t ws_bytes, int64_t most) {
    const int64_t bin_bytes = dep_bin_bytes(g);
    const bool bins = ws && bin_bytes > 0 && ws_bytes >= kWorkspaceBytes + bin_bytes;
    if (!bins || g->deposit_variant == PIC_DEPOSIT_TRACKS) return false;
    if (g->deposit_variant == PIC_DEPOSIT_BINNED) return true;
    const int64_t tiles = bin_tiles_per_side(g->no_xy) * bin_tiles_per_side(g->no_xy);
    if (most < 0) return tiles >= (int64_t)kBinAutoTilesPerSm * sm_count();  // one step alone
    // grouped: enough blocks for the SMs, or tiles short enough for one block
    const double per_axis = (2.0 * g->cutoff_voxels + kBinC) / kBinOut;  // tiles a track meets along an axis
    return tiles * kBinSteps >= sm_count() || (double)most * per_axis * per_axis / (double)tiles <= kBinAutoPerTile;
}

// Track-tile pairs a step's deposition may scan in the tile form: beyond it
// (a large grid) the per-track form, whose atomics then spread over many
// cells, is cheaper than every tile scanning every track.
constexpr int64_t kDepTileScanMax = 1000000;
// ... and only when a step's tiles and parts give enough blocks to fill the
// GPU: a single small grid with a few hundred tracks is faster with the
// per-track warps spread over every SM (a 48 x 48 grid's whole run: 21 ms
// per track, 31 ms in tiles); the batched step always deposits in tiles,
// where every grid's tiles together fill the GPU.
constexpr int64_t kDepTileMinBlocks = 1024;

int launch_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t m, void *dens, uint32_t *counts,
                   cudaStream_t st, void *ws, int64_t ws_bytes) {
    if (m <= 0) return PIC_OK;
    if (g->deposit_variant == PIC_DEPOSIT_BINNED && !deposit_binned(g, ws, ws_bytes, -1))
        return set_error(PIC_E_INVALID,
                         "the binned deposition needs the step workspace of pic_step_workspace_bytes (pic_run_segment "
                         "and the gradient drivers; no_xy <= 4096, cutoff_voxels < 31.5)");
    if (deposit_binned(g, ws, ws_bytes, -1))
        return g->dtype == PIC_F64 ? launch_binned<double>(g, xs, ys, m, dens, counts, ws, st)
                                   : launch_binned<float>(g, xs, ys, m, dens, counts, ws, st);
    const int64_t tiles = deposit_tiles(g->no_xy);
    const int parts_est = deposit_tile_parts(m);
    if (g->deposit_variant == PIC_DEPOSIT_AUTO && tiles * m <= kDepTileScanMax &&
        tiles * parts_est >= kDepTileMinBlocks) {
        const int parts = deposit_tile_parts(m);
        const unsigned blocks = (unsigned)(tiles * parts);
        if (g->dtype == PIC_F64)
            deposit_tile_kernel<double><<<blocks, kDepThreads, 0, st>>>(
                xs, ys, m, (double2 *)dens, counts, g->no_xy, dens_pitch(g->no_xy), g->cutoff_voxels,
                g->h2_over_b2, g->gaussian_factor, parts);
        else
            deposit_tile_kernel<float><<<blocks, kDepThreads, 0, st>>>(
                xs, ys, m, (float2 *)dens, counts, g->no_xy, dens_pitch(g->no_xy), g->cutoff_voxels,
                (float)g->h2_over_b2, (float)g->gaussian_factor, parts);
        return check_launch("deposit_tile_kernel");
    }
    constexpr int WARPS = 8;
    const int parts = deposit_parts(m, sm_count());
    const int per_block = WARPS / parts;
    const int64_t blocks = (m + per_block - 1) / per_block;
    if (g->dtype == PIC_F64) {
        deposit_kernel<double, WARPS><<<(unsigned)blocks, WARPS * 32, 0, st>>>(
            xs, ys, m, (double2 *)dens, counts, g->no_xy, dens_pitch(g->no_xy), g->cutoff_voxels, g->h2_over_b2,
            g->gaussian_factor, parts);
    } else {
        deposit_kernel<float, WARPS><<<(unsigned)blocks, WARPS * 32, 0, st>>>(
            xs, ys, m, (float2 *)dens, counts, g->no_xy, dens_pitch(g->no_xy), g->cutoff_voxels,
            (float)g->h2_over_b2, (float)g->gaussian_factor, parts);
    }
    return check_launch("deposit_kernel");
}

}  // namespace pic
