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
// pic_binned.cuh and below. Per track (large grids, tracks spread over many cells): one to
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

#include "pic_binned.cuh"
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
// afterwards. bin_kernel evaluates each track's factors once (a track
// meets about four tiles) and lists the track in the tiles it reaches; the
// tile's block takes its tracks in ascending index order (the lists are
// sorted in shared memory), so the result does not depend on the order the
// binning's atomics ran in: two runs give identical pairs. Every cell of a
// tile some track reaches is stored once, without atomics; a tile no track
// reaches is left as it is (zero: the buffer is zero on entry, as for the
// other forms). One pair of launches serves up to kBinSteps steps of a
// segment, one slot each (BinSlot), which gives the GPU eight times the
// blocks of one step; a step with more than kBinTracks tracks runs in pieces,
// the later ones adding to the cells the first stored.
template <typename T>
struct DepBins {
    int *count;     // [kBinSteps][tiles]
    int *list;      // [kBinSteps][tiles][kBinCap], track indices within the launch
    BinScratch<T> scratch;  // boxes and factors of kBinTracks tracks
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
    return DepBins<T>{reinterpret_cast<int *>(b), reinterpret_cast<int *>(list),
                      BinScratch<T>{reinterpret_cast<short4 *>(box), reinterpret_cast<T *>(fac)}, dens, t, t * t};
}

// Slot k of a launch over one grid: tracks [first, last) of the launch (whose
// first track is xs[0]), pairs into dens, lists in the k-th block of the bins.
template <typename T>
inline BinSlot<T> grid_slot(const pic_grid *g, const DepBins<T> &bins, int k, const double *xs, const double *ys,
                            int64_t first, int64_t last, void *dens, uint32_t *hist, int add) {
    BinSlot<T> s;
    s.xs = xs + first;
    s.ys = ys + first;
    s.dens = static_cast<pair_t<T> *>(dens);
    s.hist = hist;
    s.count = bins.count + k * bins.tiles;
    s.list = bins.list + k * bins.tiles * kBinCap;
    s.first = first;
    s.last = last;
    s.cut = g->cutoff_voxels;
    s.h2b2 = (T)g->h2_over_b2;
    s.gfac = (T)g->gaussian_factor;
    s.n = (int32_t)g->no_xy;
    s.dp = (int32_t)dens_pitch(g->no_xy);
    s.tps = (int32_t)bins.tps;
    s.block0 = (int32_t)(k * bins.tiles);
    s.add = add;
    return s;
}

template <typename T, typename S>
int binned_launches(const S &slots, const BinScratch<T> &sc, int64_t blocks, cudaStream_t st) {
    constexpr int smem = BinSmem<T>::kBytes;
    static int configured = 0;  // per instantiation
    if (smem > 48 * 1024 && !configured) {
        cudaError_t e =
            cudaFuncSetAttribute(binned_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(binned_kernel)", e);
        configured = 1;
    }
    const int64_t warps = (slots.tracks + kBinWarpTracks - 1) / kBinWarpTracks;
    bin_kernel<T, S><<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(slots, sc);
    int rc = check_launch("bin_kernel");
    if (rc) return rc;
    binned_kernel<T, S><<<(unsigned)blocks, kBinThreads, smem, st>>>(slots, sc);
    return check_launch("binned_kernel");
}
template int binned_launches<float, BinSlotsDevice<float>>(const BinSlotsDevice<float> &,
                                                           const BinScratch<float> &, int64_t, cudaStream_t);
template int binned_launches<double, BinSlotsDevice<double>>(const BinSlotsDevice<double> &,
                                                             const BinScratch<double> &, int64_t, cudaStream_t);

// One step's tracks into the caller's pairs, in pieces of kBinTracks.
template <typename T>
int launch_binned(const pic_grid *g, const double *xs, const double *ys, int64_t m, void *dens, uint32_t *counts,
                  void *ws, cudaStream_t st) {
    const DepBins<T> bins = dep_bins<T>(ws, g->no_xy);
    for (int64_t g0 = 0; g0 < m; g0 += kBinTracks) {
        const int64_t mg = m - g0 < kBinTracks ? m - g0 : kBinTracks;
        BinSlotsValue<T> S{};
        S.count = 1;
        S.tracks = mg;
        S.s[0] = grid_slot<T>(g, bins, 0, xs + g0, ys + g0, 0, mg, dens, counts, g0 > 0);
        int rc = binned_launches<T>(S, bins.scratch, bins.tiles, st);
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
    BinSlotsValue<T> S{};
    int k = 0;
    const double *x0 = xs + off[s0], *y0 = ys + off[s0];
    for (int64_t s = s0; s < s1; ++s) {
        dens[s - s0] = nullptr;
        if (off[s + 1] == off[s]) continue;
        if (k == kBinSteps) return set_error(PIC_E_INVALID, "more than kBinSteps depositing steps in one launch");
        void *out = targets ? targets[k] : static_cast<void *>(bins.dens + k * slot_bytes);
        S.s[k] = grid_slot<T>(g, bins, k, x0, y0, off[s] - off[s0], off[s + 1] - off[s0], out, counts, 0);
        dens[s - s0] = out;
        ++k;
    }
    if (k == 0) return PIC_OK;
    S.count = k;
    S.tracks = off[s1] - off[s0];
    if (S.tracks > kBinTracks) return set_error(PIC_E_INVALID, "more than kBinTracks tracks in one launch");
    return binned_launches<T>(S, bins.scratch, k * bins.tiles, st);
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
