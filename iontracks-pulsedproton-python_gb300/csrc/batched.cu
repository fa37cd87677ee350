// batched.cu -- many independent chamber configurations advanced together.
//
// The grids of a batch live at their own offsets in packed buffers (fields,
// 2D deposition pairs, track histograms, tallies), described by a device table of
// pic_batch_cfg entries (each grid's pic_grid scalars and offsets). One global
// step advances every active grid by one of its own time steps with two
// launches for the whole batch:
//   * batched_deposit_kernel -- the tile form of the deposition (pic_deposit.cuh)
//     over the tracks of every grid: a task list gives each grid's tracks of
//     the step, each task takes its grid's tiles times its parts of blocks;
//   * batched_step_kernel -- the flat fused step (pic_flat.cuh) over a work
//     table that gives each block one grid and a contiguous range of that
//     grid's items; a grid's blocks are consecutive in the table, and the
//     last of them to finish (per-grid completion counter) writes the grid's
//     tallies for this step.
// Grids differ in size, time step, coefficients, step count and schedule; a
// grid that has finished is simply absent from the work table and the task
// list of later steps (the caller builds one table per set of active grids).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "pic_binned.cuh"
#include "pic_deposit.cuh"
#include "pic_device.cuh"
#include "pic_barrier.cuh"
#include "pic_flat.cuh"
#include "pic_internal.h"

namespace pic {

// A grid's step arguments without the buffers (filled per block from the
// step's packed buffers and the offsets): built once per launch chunk by
// batched_prep_kernel, copied by each block instead of recomputed.
template <typename T>
struct GridEntry {
    StepArgs<T> a;
    int64_t field_off, dens_off;
};

template <typename T>
struct BatchStepArgs {
    const pic_batch_cfg *cfgs;
    const GridEntry<T> *table;  // [n_cfgs]
    const int32_t *blk_cfg;
    const int64_t *blk_item0, *blk_item1;
    const int32_t *cfg_blk0, *cfg_nblk;
    const T *pos_in, *neg_in;
    T *pos_out, *neg_out;
    const pair_t<T> *dens;  // packed deposition pairs of this step
    pair_t<T> *dens_zero;   // packed pairs of the next step, cleared here (null: none)
    double *tally;    // packed [rows][4]
    double *partials; // [n_blocks][4]
    unsigned int *counters;  // [n_cfgs]
    int64_t step;     // global step index (row within each grid's tallies)
};

template <typename T>
__device__ void grid_args(const pic_batch_cfg &C, StepArgs<T> &a) {
    const pic_grid &g = C.grid;
    a.pos_in = a.neg_in = nullptr;
    a.pos_out = a.neg_out = nullptr;
    a.dens = nullptr;
    a.dens_zero = nullptr;
    a.tally = a.partials = nullptr;
    a.counter = nullptr;
    a.n = g.no_xy;
    a.kp = g.kpitch;
    a.c4 = g.kpitch / 4;
    a.items = g.no_xy * g.no_xy * a.c4;
    a.dp = (g.no_xy + 3) / 4 * 4;
    a.nzb = (int)g.nzb;
    a.nze = (int)g.nze;
    a.gap_end = (int)(g.nze + g.no_z);
    a.reflecting = g.wall == PIC_WALL_REFLECTING;
    a.p_lat = (T)g.p_lat; a.p_zm = (T)g.p_zm; a.p_zp = (T)g.p_zp;
    a.p_cen = centre_weight<T>(g.p_lat, g.p_zm, g.p_zp, g.p_cen);
    a.n_lat = (T)g.n_lat; a.n_zm = (T)g.n_zm; a.n_zp = (T)g.n_zp;
    a.n_cen = centre_weight<T>(g.n_lat, g.n_zm, g.n_zp, g.n_cen);
    a.alpha_dt = (T)g.alpha_dt;
    a.gfac = (T)g.gaussian_factor;
    a.score.two_mid = (int64_t)(2.0 * g.mid_xy);
    const double r4 = 4.0 * g.scoring_radius_sq;
    a.score.thr4 = r4 >= 4.0e18 ? (int64_t)4.0e18 : (int64_t)ceil(r4) - 1;
    a.injected_scale = (double)g.no_z;
    a.div_c4 = make_fastdiv(a.c4);
    a.div_n = make_fastdiv(a.n);
}

template <typename T>
__global__ void batched_prep_kernel(const pic_batch_cfg *cfgs, int n_cfgs, GridEntry<T> *table) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_cfgs) return;
    GridEntry<T> e;
    grid_args(cfgs[c], e.a);
    e.field_off = cfgs[c].field_off;
    e.dens_off = cfgs[c].dens_off;
    table[c] = e;
}

// Reduction type of a grid's tallies: double-float for float32 fields (no
// float64 arithmetic), float64 for float64 fields; partial slots are 8 bytes
// either way.
template <typename T> struct RedT { using type = double; };
template <> struct RedT<float> { using type = DF; };
__device__ __forceinline__ double red_value(double v) { return v; }
__device__ __forceinline__ double red_value(DF v) { return df_value(v); }
__device__ __forceinline__ void red_store(double *slot, double v) { *slot = v; }
__device__ __forceinline__ void red_store(double *slot, DF v) {
    *reinterpret_cast<float2 *>(slot) = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ void red_load_add(double &acc, const double *slot) { acc += __ldcg(slot); }
__device__ __forceinline__ void red_load_add(DF &acc, const double *slot) {
    const float2 p = __ldcg(reinterpret_cast<const float2 *>(slot));
    acc = df_add(acc, DF{p.x, p.y});
}
__device__ __forceinline__ double red_of(const Tally<double> &t) { return t.value(); }
__device__ __forceinline__ DF red_of(const Tally<float> &t) { return df_of(t); }

// One entry of the work table (blk): a range of one grid's items, its
// tallies reduced per block and, by the grid's last block to finish, into the
// grid's tally row. `red`, `last` and `a` are the caller's shared memory.
template <typename T, int BLOCK, typename I, bool COH = false>
__device__ __forceinline__ void batched_step_block(const BatchStepArgs<T> &b, int blk,
                                                   typename RedT<T>::type (*red)[4], bool &last, StepArgs<T> &a) {
    using R = typename RedT<T>::type;
    const int c = b.blk_cfg[blk];
    const pic_batch_cfg &C = b.cfgs[c];
    if (threadIdx.x < 32) {  // one warp copies the grid's prepared arguments
        const GridEntry<T> *E = b.table + c;
        const uint32_t *src = reinterpret_cast<const uint32_t *>(&E->a);
        uint32_t *dst = reinterpret_cast<uint32_t *>(&a);
        for (int w = threadIdx.x; w < (int)(sizeof(StepArgs<T>) / 4); w += 32) dst[w] = src[w];
        __syncwarp();
        if (threadIdx.x == 0) {
            a.pos_in = b.pos_in + E->field_off;
            a.neg_in = b.neg_in + E->field_off;
            a.pos_out = b.pos_out + E->field_off;
            a.neg_out = b.neg_out + E->field_off;
            a.dens = b.dens + E->dens_off;
            a.dens_zero = b.dens_zero ? b.dens_zero + E->dens_off : nullptr;  // null: nothing to clear
        }
    }
    __syncthreads();
    Tally<T> t_rec, t_p, t_n, t_inj;
    // The grid's blocks stride through its items together (block r of nb
    // takes items r*BLOCK + t + k*nb*BLOCK): resident blocks of a grid then
    // sweep one contiguous front through it, and each item's i-1 / i+1
    // neighbours are read while still in L2 (a contiguous chunk per block left
    // hundreds of separate windows in flight across the batch).
    {
        const I r = (I)(blk - b.cfg_blk0[c]), stride = (I)b.cfg_nblk[c] * BLOCK, items = (I)a.items;
        for (I item = r * BLOCK + threadIdx.x; item < items; item += stride)
            flat_item<T, I, COH>(a, item, t_rec, t_p, t_n, t_inj);
    }
    R v[4] = {red_of(t_inj), red_of(t_rec), red_of(t_p), red_of(t_n)};
    block_sum4<BLOCK>(v, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) red_store(b.partials + 4 * (int64_t)blk + q, v[q]);
        __threadfence();
        last = (atomicAdd(b.counters + c, 1u) == (unsigned)b.cfg_nblk[c] - 1u);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int b0 = b.cfg_blk0[c], nb = b.cfg_nblk[c];
    R acc[4] = {R{}, R{}, R{}, R{}};
    for (int k = threadIdx.x; k < nb; k += BLOCK)
#pragma unroll
        for (int q = 0; q < 4; ++q) red_load_add(acc[q], b.partials + 4 * (int64_t)(b0 + k) + q);
    block_sum4<BLOCK>(acc, red);
    if (threadIdx.x == 0) {
        double *t = b.tally + 4 * (C.tally_off + b.step);
        t[0] = red_value(acc[0]) * a.injected_scale;
        t[1] = red_value(acc[1]);
        t[2] = red_value(acc[2]);
        t[3] = red_value(acc[3]);
        b.counters[c] = 0u;
        __threadfence();
    }
}

// float32: four resident blocks per SM (64 registers, a little spilled to
// local memory) hide more of the heavy phase's global-load latency than three
// at 80 registers (the 64-grid sweep: 1.12 against 1.15-1.19 s)
template <typename T, int BLOCK, typename I>
__global__ void __launch_bounds__(BLOCK, sizeof(T) == 4 ? 4 : 1) batched_step_kernel(BatchStepArgs<T> b) {
    __shared__ typename RedT<T>::type red[BLOCK / 32][4];
    __shared__ bool last;
    // the block's grid arguments, staged once in shared memory and read by
    // broadcast (keeps them out of the registers of every thread)
    __shared__ StepArgs<T> a;
    batched_step_block<T, BLOCK, I>(b, blockIdx.x, red, last, a);
}

// Block `blk` of a global step's deposition (the tile form of
// pic_deposit.cuh): the step's tasks (grid, first track, tracks before it) are
// scanned in order, each taking tiles(grid) x parts(its tracks) blocks, to
// find this block's task, tile and part. `total` = the step's tracks.
template <typename T>
__device__ __forceinline__ void batched_deposit_block(const pic_batch_cfg *cfgs, const int32_t *task_cfg,
                                                      const int64_t *task_first, const int64_t *task_prefix,
                                                      int n_tasks, int64_t total, int64_t blk, const double *xs,
                                                      const double *ys, pair_t<T> *dens, uint32_t *counts,
                                                      DepTileShared<T> &sh) {
    int64_t acc = 0;
    for (int t = 0; t < n_tasks; ++t) {
        const int64_t m = (t + 1 < n_tasks ? task_prefix[t + 1] : total) - task_prefix[t];
        const pic_batch_cfg &C = cfgs[task_cfg[t]];
        const int64_t n = C.grid.no_xy;
        const int parts = deposit_tile_parts(m);
        const int64_t nb = deposit_tiles(n) * parts;
        if (blk < acc + nb) {
            const int64_t local = blk - acc, tile = local / parts;
            const int part = (int)(local % parts);
            const int64_t f = task_first[t];
            deposit_tile<T>(xs + f, ys + f, m * part / parts, m * (part + 1) / parts, n, (n + 3) / 4 * 4,
                            C.grid.cutoff_voxels, (T)C.grid.h2_over_b2, (T)C.grid.gaussian_factor,
                            dens + C.dens_off, counts + C.counts_off, tile, sh);
            return;
        }
        acc += nb;
    }
}

template <typename T>
__global__ void __launch_bounds__(kDepThreads) batched_deposit_kernel(const pic_batch_cfg *cfgs,
                                                                       const int32_t *task_cfg,
                                                                       const int64_t *task_first,
                                                                       const int64_t *task_prefix, int n_tasks,
                                                                       int64_t total, const double *xs,
                                                                       const double *ys, pair_t<T> *dens,
                                                                       uint32_t *counts) {
    __shared__ DepTileShared<T> sh;
    batched_deposit_block<T>(cfgs, task_cfg, task_first, task_prefix, n_tasks, total, blockIdx.x, xs, ys, dens,
                             counts, sh);
}

// Blocks of one global step's deposition (every thread of the persistent
// kernel forms the same number; the per-step launches take the host's).
__device__ __forceinline__ int64_t batched_deposit_blocks(const pic_batch_cfg *cfgs, const int32_t *task_cfg,
                                                          const int64_t *task_prefix, int n_tasks, int64_t total) {
    int64_t acc = 0;
    for (int t = 0; t < n_tasks; ++t) {
        const int64_t m = (t + 1 < n_tasks ? task_prefix[t + 1] : total) - task_prefix[t];
        acc += deposit_tiles(cfgs[task_cfg[t]].grid.no_xy) * deposit_tile_parts(m);
    }
    return acc;
}

// Workspace layout: [per-grid completion counters, n_cfgs x u32, padded to
// 256 bytes | the persistent kernel's barrier and status, 256 bytes | the
// prepared grid arguments, n_cfgs slots, padded to 256 bytes | per-block
// partials, n_blocks x 4 doubles]. The counters sit at a fixed place
// whatever the block count of a launch (which changes when grids finish), so
// they stay zero between steps.
static int64_t counters_bytes(int32_t n_cfgs) { return ((int64_t)n_cfgs * 4 + 255) / 256 * 256; }
constexpr int64_t kBarrierBytes = 256;

struct GridBarrier {
    unsigned int count;  // blocks arrived at the current barrier
    unsigned int gen;    // barriers completed
    int status;          // 0, or the code of a wait that gave up
};

// prepared grid arguments, one slot per grid (the larger, float64 form)
static int64_t table_bytes(int32_t n_cfgs) {
    return ((int64_t)n_cfgs * (int64_t)sizeof(GridEntry<double>) + 255) / 256 * 256;
}

static GridBarrier *barrier_of(const BatchLaunch &L) {
    return reinterpret_cast<GridBarrier *>(static_cast<char *>(L.workspace) + counters_bytes(L.n_cfgs));
}
template <typename T>
static GridEntry<T> *table_of(const BatchLaunch &L) {
    return reinterpret_cast<GridEntry<T> *>(static_cast<char *>(L.workspace) + counters_bytes(L.n_cfgs) +
                                            kBarrierBytes);
}
static double *partials_of(const BatchLaunch &L) {
    return reinterpret_cast<double *>(static_cast<char *>(L.workspace) + counters_bytes(L.n_cfgs) + kBarrierBytes +
                                      table_bytes(L.n_cfgs));
}

int batched_workspace_bytes(int32_t n_blocks, int32_t n_cfgs, int64_t *bytes) {
    if (n_blocks < 1 || n_cfgs < 1) return set_error(PIC_E_INVALID, "n_blocks and n_cfgs must be >= 1");
    *bytes = counters_bytes(n_cfgs) + kBarrierBytes + table_bytes(n_cfgs) + (int64_t)n_blocks * 4 * 8;
    return PIC_OK;
}

template <typename T>
static int prep_table(const BatchLaunch &L, cudaStream_t st) {
    batched_prep_kernel<T><<<(L.n_cfgs + 127) / 128, 128, 0, st>>>(L.cfgs, L.n_cfgs, table_of<T>(L));
    return check_launch("batched_prep_kernel");
}

__device__ __forceinline__ BarrierRef barrier_ref(GridBarrier *b) { return BarrierRef{&b->count, &b->gen, &b->status}; }

template <typename T>
struct BatchPersistArgs {
    BatchStepArgs<T> b;  // step and parity fields set per step
    const void *pos[2], *neg[2], *dens[2];
    const int32_t *task_cfg;
    const int64_t *task_first, *task_prefix;
    const int64_t *step_task_off, *step_tracks;  // device, by global step
    const double *xs, *ys;
    uint32_t *counts;
    int n_blocks, sms;
    int64_t first_step, n_steps;
    GridBarrier *bar;
};

// A chunk of global steps in one launch: per step, the deposition of every
// grid's tracks (warps over the step's tracks), a barrier, the fused step over
// the work table (blocks loop over its entries), a barrier.
template <typename T, typename I>
__global__ void __launch_bounds__(256) batched_persistent_kernel(BatchPersistArgs<T> p) {
    constexpr int BLOCK = 256, WARPS = BLOCK / 32;
    __shared__ typename RedT<T>::type red[BLOCK / 32][4];
    __shared__ bool last;
    __shared__ StepArgs<T> a;
    __shared__ DepTileShared<T> dep;
    static_assert(BLOCK == kDepThreads, "the persistent kernel's blocks run the tile deposition");
    for (int64_t s = p.first_step; s < p.first_step + p.n_steps; ++s) {
        const int bi = (int)(s & 1), bo = bi ^ 1;
        const int64_t t0 = p.step_task_off[s], t1 = p.step_task_off[s + 1], tracks = p.step_tracks[s];
        if (tracks > 0 && t1 > t0) {
            const int nt = (int)(t1 - t0);
            const int64_t nblk = batched_deposit_blocks(p.b.cfgs, p.task_cfg + t0, p.task_prefix + t0, nt, tracks);
            for (int64_t vb = blockIdx.x; vb < nblk; vb += gridDim.x) {
                __syncthreads();  // shared staging of the previous tile is done with
                batched_deposit_block<T>(p.b.cfgs, p.task_cfg + t0, p.task_first + t0, p.task_prefix + t0, nt,
                                         tracks, vb, p.xs, p.ys, (pair_t<T> *)p.dens[bi], p.counts, dep);
            }
            if (!grid_barrier(barrier_ref(p.bar))) return;
        }
        BatchStepArgs<T> b = p.b;
        b.pos_in = (const T *)p.pos[bi];
        b.neg_in = (const T *)p.neg[bi];
        b.pos_out = (T *)p.pos[bo];
        b.neg_out = (T *)p.neg[bo];
        b.dens = (const pair_t<T> *)p.dens[bi];
        b.dens_zero = (pair_t<T> *)p.dens[bo];
        b.step = s;
        for (int vb = blockIdx.x; vb < p.n_blocks; vb += gridDim.x) {
            __syncthreads();  // shared staging of the previous entry is done with
            batched_step_block<T, BLOCK, I, true>(b, vb, red, last, a);
        }
        if (!grid_barrier(barrier_ref(p.bar))) return;
    }
}

template <typename T, typename I>
static int launch_persistent(const BatchLaunch &L, const int64_t *sto, const int64_t *stt, cudaStream_t st) {
    static int per_sm = 0;  // resident blocks per SM of this instantiation
    if (per_sm == 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batched_persistent_kernel<T, I>, 256, 0);
        if (e != cudaSuccess || per_sm < 1) {
            per_sm = 0;
            return set_cuda_error("cudaOccupancyMaxActiveBlocksPerMultiprocessor(batched_persistent_kernel)", e);
        }
    }
    BatchPersistArgs<T> p;
    int rc = prep_table<T>(L, st);
    if (rc) return rc;
    p.b = BatchStepArgs<T>{L.cfgs, table_of<T>(L), L.blk_cfg, L.blk_item0, L.blk_item1, L.cfg_blk0, L.cfg_nblk,
                           nullptr, nullptr,
                           nullptr, nullptr, nullptr, nullptr, L.tally, partials_of(L),
                           reinterpret_cast<unsigned int *>(L.workspace), 0};
    for (int q = 0; q < 2; ++q) {
        p.pos[q] = L.pos[q];
        p.neg[q] = L.neg[q];
        p.dens[q] = L.dens[q];
    }
    p.task_cfg = L.task_cfg;
    p.task_first = L.task_first;
    p.task_prefix = L.task_prefix;
    p.step_task_off = sto;
    p.step_tracks = stt;
    p.xs = L.xs;
    p.ys = L.ys;
    p.counts = L.counts;
    p.n_blocks = L.n_blocks;
    p.sms = sm_count();
    p.first_step = L.first_step;
    p.n_steps = L.n_steps;
    p.bar = barrier_of(L);
    cudaError_t e = cudaMemsetAsync(p.bar, 0, sizeof(GridBarrier), st);
    if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(barrier)", e);
    const unsigned grid = (unsigned)(per_sm * sm_count());
    void *args[] = {&p};
    e = cudaLaunchCooperativeKernel((const void *)batched_persistent_kernel<T, I>, dim3(grid), dim3(256), args, 0, st);
    if (e != cudaSuccess) return set_cuda_error("cudaLaunchCooperativeKernel(batched_persistent_kernel)", e);
    count_launches(1);
    return PIC_OK;
}

int batched_persistent(const BatchLaunch &L, const int64_t *step_task_off, const int64_t *step_tracks,
                       cudaStream_t st) {
    if (L.dtype == PIC_F64)
        return L.index32 ? launch_persistent<double, uint32_t>(L, step_task_off, step_tracks, st)
                         : launch_persistent<double, int64_t>(L, step_task_off, step_tracks, st);
    return L.index32 ? launch_persistent<float, uint32_t>(L, step_task_off, step_tracks, st)
                     : launch_persistent<float, int64_t>(L, step_task_off, step_tracks, st);
}

int batched_status(const BatchLaunch &L, cudaStream_t st, int32_t *status) {
    int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, &barrier_of(L)->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error("reading the batched status word", e);
    *status = v;
    return PIC_OK;
}

template <typename T, typename I>
static void launch_batched_step(const BatchLaunch &L, int bi, int bo, double *partials, unsigned int *counters,
                                int64_t step, cudaStream_t st, const void *dens, void *dens_zero) {
    constexpr int BLOCK = 256;
    BatchStepArgs<T> b{L.cfgs, table_of<T>(L), L.blk_cfg, L.blk_item0, L.blk_item1, L.cfg_blk0, L.cfg_nblk,
                       (const T *)L.pos[bi], (const T *)L.neg[bi], (T *)L.pos[bo], (T *)L.neg[bo],
                       (const pair_t<T> *)dens, (pair_t<T> *)dens_zero, L.tally, partials, counters, step};
    batched_step_kernel<T, BLOCK, I><<<(unsigned)L.n_blocks, BLOCK, 0, st>>>(b);
}

// ---------------------------------------------------------------------------
// The binned deposition (pic_binned.cuh) of up to kBinSteps global steps per
// launch pair: a slot per task (a grid with tracks in a step), built on the
// device by batched_bin_prep_kernel from the task list and the grid table,
// then the binning and tile launches over those slots. Step q of a group
// writes its pairs into the q-th packed pair buffer of the workspace (zeroed
// first), which its batched step then reads. Workspace layout: [slots,
// kBinSteps x n_cfgs, padded to 256 bytes | per-tile counts, kBinSteps x
// total_tiles ints, padded | per-tile lists, kBinSteps x total_tiles x
// kBinCap ints | boxes, max_tracks short4, padded | factors, max_tracks x 2 x
// kBinBox of the field type, padded | kBinSteps packed pair buffers, each
// dens_bytes padded to 256].
static int64_t pad256(int64_t b) { return (b + 255) / 256 * 256; }

int64_t batched_deposit_bytes(int32_t n_cfgs, int32_t total_tiles, int64_t max_tracks, int64_t dens_bytes,
                              int32_t dtype) {
    const int64_t es = dtype == PIC_F64 ? 8 : 4;
    const int64_t slot = dtype == PIC_F64 ? (int64_t)sizeof(BinSlot<double>) : (int64_t)sizeof(BinSlot<float>);
    const int64_t tiles = (int64_t)kBinSteps * total_tiles;
    return pad256(kBinSteps * n_cfgs * slot) + pad256(tiles * 4) + tiles * kBinCap * 4 + pad256(max_tracks * 8) +
           pad256(max_tracks * 2 * kBinBox * es) + kBinSteps * pad256(dens_bytes);
}

template <typename T>
struct BatchedBins {
    BinSlot<T> *slots;
    int *count, *list;
    BinScratch<T> sc;
    char *dens;  // kBinSteps packed pair buffers
    int64_t dens_stride;
};
template <typename T>
static BatchedBins<T> batched_bins(const BatchLaunch &L) {
    const int64_t tiles = (int64_t)kBinSteps * L.dep_total_tiles;
    char *b = static_cast<char *>(L.dep_workspace);
    char *count = b + pad256((int64_t)kBinSteps * L.n_cfgs * sizeof(BinSlot<T>));
    char *list = count + pad256(tiles * 4);
    char *box = list + tiles * kBinCap * 4;
    char *fac = box + pad256(L.dep_max_tracks * 8);
    char *dens = fac + pad256(L.dep_max_tracks * 2 * kBinBox * (int64_t)sizeof(T));
    return BatchedBins<T>{reinterpret_cast<BinSlot<T> *>(b), reinterpret_cast<int *>(count),
                          reinterpret_cast<int *>(list),
                          BinScratch<T>{reinterpret_cast<short4 *>(box), reinterpret_cast<T *>(fac)}, dens,
                          pad256(L.dep_dens_bytes)};
}

// The steps of one group, by value: step q's tasks are [task_off[q],
// task_off[q + 1]) of the group's (counted from its first task), its tracks
// start at launch track track_base[q], its pairs go to dens[q].
template <typename T>
struct BinGroup {
    int64_t task_off[kBinSteps + 1];
    int64_t track_base[kBinSteps + 1];
    pair_t<T> *dens[kBinSteps];
    int steps;
};

// Task t's slot (its grid's scalars, tracks, pairs and histogram); the
// tiles before it, a block-wide prefix sum carried over chunks of the block's
// size, place its counts, lists and blocks.
template <typename T>
__global__ void __launch_bounds__(kBinMaxSlots) batched_bin_prep_kernel(
    const pic_batch_cfg *cfgs, const int32_t *task_cfg, const int64_t *task_first, const int64_t *task_prefix,
    int n_tasks, BinGroup<T> G, const double *xs, const double *ys, uint32_t *counts, int *count_base,
    int *list_base, BinSlot<T> *out) {
    __shared__ int64_t pre[kBinMaxSlots];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    for (int c0 = 0; c0 < n_tasks; c0 += blockDim.x) {
        const int t = c0 + (int)threadIdx.x;
        BinSlot<T> s{};
        int64_t tiles = 0;
        if (t < n_tasks) {
            int q = 0;
            while (q + 1 < G.steps && G.task_off[q + 1] <= t) ++q;
            const pic_batch_cfg &C = cfgs[task_cfg[t]];
            const pic_grid &g = C.grid;
            const int n = (int)g.no_xy;
            s.xs = xs + task_first[t];
            s.ys = ys + task_first[t];
            s.dens = G.dens[q] + C.dens_off;
            s.hist = counts + C.counts_off;
            s.first = G.track_base[q] + task_prefix[t];
            s.last = t + 1 < G.task_off[q + 1] ? G.track_base[q] + task_prefix[t + 1] : G.track_base[q + 1];
            s.cut = g.cutoff_voxels;
            s.h2b2 = (T)g.h2_over_b2;
            s.gfac = (T)g.gaussian_factor;
            s.n = n;
            s.dp = (n + 3) / 4 * 4;
            s.tps = (n + kBinOut - 1) / kBinOut;
            s.add = 0;
            tiles = (int64_t)s.tps * s.tps;
        }
        pre[threadIdx.x] = tiles;
        __syncthreads();
        for (int d = 1; d < (int)blockDim.x; d <<= 1) {
            const int64_t v = (int)threadIdx.x >= d ? pre[threadIdx.x - d] : 0;
            __syncthreads();
            pre[threadIdx.x] += v;
            __syncthreads();
        }
        if (t < n_tasks) {
            const int64_t base = carry + pre[threadIdx.x] - tiles;
            s.count = count_base + base;
            s.list = list_base + base * kBinCap;
            s.block0 = (int32_t)base;
            out[t] = s;
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += pre[threadIdx.x];
        __syncthreads();
    }
}

// Global steps s0 .. s1 - 1 of the launch (at most kBinSteps, their tracks
// within dep_max_tracks) deposited together. pairs[s - s0]: step s's pairs
// (a zeroed workspace buffer holding its tracks), or null for a step
// without tracks.
template <typename T>
static int batched_binned_deposit(const BatchLaunch &L, int64_t s0, int64_t s1, const void **pairs, cudaStream_t st) {
    const BatchedBins<T> B = batched_bins<T>(L);
    BinGroup<T> G{};
    const int64_t t0 = L.step_task_off[s0];
    int64_t tracks = 0;
    G.steps = (int)(s1 - s0);
    for (int q = 0; q < G.steps; ++q) {
        const int64_t s = s0 + q;
        G.task_off[q] = L.step_task_off[s] - t0;
        G.track_base[q] = tracks;
        const bool dep = L.step_tracks[s] > 0 && L.step_task_off[s + 1] > L.step_task_off[s];
        G.dens[q] = reinterpret_cast<pair_t<T> *>(B.dens + q * B.dens_stride);
        if (dep) {
            cudaError_t e = cudaMemsetAsync(G.dens[q], 0, (size_t)L.dep_dens_bytes, st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(batched deposition pairs)", e);
        }
        pairs[q] = dep ? G.dens[q] : nullptr;
        tracks += dep ? L.step_tracks[s] : 0;
    }
    G.task_off[G.steps] = L.step_task_off[s1] - t0;
    G.track_base[G.steps] = tracks;
    const int nt = (int)(L.step_task_off[s1] - t0);
    if (nt == 0 || tracks == 0) return PIC_OK;
    batched_bin_prep_kernel<T><<<1, nt < kBinMaxSlots ? (nt + 31) / 32 * 32 : kBinMaxSlots, 0, st>>>(
        L.cfgs, L.task_cfg + t0, L.task_first + t0, L.task_prefix + t0, nt, G, L.xs, L.ys, L.counts, B.count,
        B.list, B.slots);
    int rc = check_launch("batched_bin_prep_kernel");
    if (rc) return rc;
    const BinSlotsDevice<T> S{B.slots, nt, tracks};
    return binned_launches<T>(S, B.sc, (int64_t)nt * L.dep_max_tiles, st);
}

int batched_loop(const BatchLaunch &L, cudaStream_t st) { return batched_loop_stream(L, nullptr, st); }

int batched_loop_stream(const BatchLaunch &L, const pic_batch_stream *B, cudaStream_t st) {
    unsigned int *counters = B ? nullptr : reinterpret_cast<unsigned int *>(L.workspace);
    double *partials = B ? nullptr : partials_of(L);
    if (L.n_steps > 0 && !B) {
        int rc = L.dtype == PIC_F64 ? prep_table<double>(L, st) : prep_table<float>(L, st);
        if (rc) return rc;
    }
    auto step_launch = [&](int64_t step, int bi, int bo, const void *dens, void *dens_zero) {
        if (B) return batched_stream_step(L, *B, bi, bo, step, dens, dens_zero, st);
        if (L.dtype == PIC_F64) {
            if (L.index32) launch_batched_step<double, uint32_t>(L, bi, bo, partials, counters, step, st, dens, dens_zero);
            else launch_batched_step<double, int64_t>(L, bi, bo, partials, counters, step, st, dens, dens_zero);
        } else {
            if (L.index32) launch_batched_step<float, uint32_t>(L, bi, bo, partials, counters, step, st, dens, dens_zero);
            else launch_batched_step<float, int64_t>(L, bi, bo, partials, counters, step, st, dens, dens_zero);
        }
        return check_launch("batched_step_kernel");
    };
    if (L.dep_workspace) {
        // groups of up to kBinSteps global steps (dep_max_tracks tracks):
        // their binned deposition into the workspace's pair buffers, then
        // their steps (flat or streaming), which read those buffers (no pairs
        // to clear: the launch's own dens buffers stay zero)
        const void *pairs[kBinSteps];
        for (int64_t s0 = 0; s0 < L.n_steps;) {
            int64_t s1 = s0, tr = 0;
            while (s1 < L.n_steps && s1 - s0 < kBinSteps && tr + L.step_tracks[s1] <= L.dep_max_tracks)
                tr += L.step_tracks[s1++];
            if (s1 == s0) return set_error(PIC_E_INVALID, "a global step has more tracks than dep_max_tracks");
            int rc = L.dtype == PIC_F64 ? batched_binned_deposit<double>(L, s0, s1, pairs, st)
                                        : batched_binned_deposit<float>(L, s0, s1, pairs, st);
            if (rc) return rc;
            for (int64_t s = s0; s < s1; ++s) {
                const int64_t step = L.first_step + s;
                const int bi = (int)(step & 1);
                if ((rc = step_launch(step, bi, bi ^ 1, pairs[s - s0] ? pairs[s - s0] : L.dens[bi], nullptr)))
                    return rc;
            }
            s0 = s1;
        }
        return PIC_OK;
    }
    for (int64_t s = 0; s < L.n_steps; ++s) {
        const int64_t step = L.first_step + s;
        const int bi = (int)(step & 1), bo = bi ^ 1;
        const int64_t t0 = L.step_task_off[s], t1 = L.step_task_off[s + 1];
        const int64_t tracks = L.step_tracks[s];
        if (tracks > 0 && t1 > t0) {
            const unsigned blocks = (unsigned)L.step_blocks[s];
            if (L.dtype == PIC_F64)
                batched_deposit_kernel<double><<<blocks, kDepThreads, 0, st>>>(
                    L.cfgs, L.task_cfg + t0, L.task_first + t0, L.task_prefix + t0, (int)(t1 - t0), tracks, L.xs,
                    L.ys, (double2 *)L.dens[bi], L.counts);
            else
                batched_deposit_kernel<float><<<blocks, kDepThreads, 0, st>>>(
                    L.cfgs, L.task_cfg + t0, L.task_first + t0, L.task_prefix + t0, (int)(t1 - t0), tracks, L.xs,
                    L.ys, (float2 *)L.dens[bi], L.counts);
            int rc = check_launch("batched_deposit_kernel");
            if (rc) return rc;
        }
        int rc = step_launch(step, bi, bo, L.dens[bi], L.dens[bo]);
        if (rc) return rc;
    }
    return PIC_OK;
}

}  // namespace pic
