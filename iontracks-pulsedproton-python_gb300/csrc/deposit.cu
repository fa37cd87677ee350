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
// Two forms. Per track (large grids, tracks spread over many cells): one to
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
                   cudaStream_t st) {
    if (m <= 0) return PIC_OK;
    const int64_t tiles = deposit_tiles(g->no_xy);
    const int parts_est = deposit_tile_parts(m);
    if (tiles * m <= kDepTileScanMax && tiles * parts_est >= kDepTileMinBlocks) {
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
