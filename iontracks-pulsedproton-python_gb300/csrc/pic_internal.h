// pic_internal.h -- host-side declarations shared by the translation units of
// libpic_gb300.so (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/pic_gb300.h"

namespace pic {

// Upper bound on the fused step's grid (blocks); sizes its tally workspace.
constexpr int64_t kMaxStepBlocks = 152 * 32;

struct Workspace {
    double *partials;       // [kMaxStepBlocks][4]
    unsigned int *counter;  // completion counter, zero between steps
    int *status;            // 0, or the code of a bounded wait that expired
};

inline Workspace workspace_layout(void *ws) {
    Workspace w;
    char *base = reinterpret_cast<char *>(ws);
    w.partials = reinterpret_cast<double *>(base);
    w.counter = reinterpret_cast<unsigned int *>(base + kMaxStepBlocks * 4 * sizeof(double));
    w.status = reinterpret_cast<int *>(base + kMaxStepBlocks * 4 * sizeof(double) + 128);
    return w;
}

// Largest CTA of the streaming step kernel: 16 consumer warps + 1 producer.
constexpr int kStreamMaxThreads = 17 * 32;
// Block-size bound of the streaming kernel instantiated for IPT items per
// consumer thread; a smaller bound leaves each thread more registers, so the
// IPT items of a plane can be unrolled without spilling.
__host__ __device__ constexpr int stream_max_threads(int ipt) {
    return ipt <= 1 ? 17 * 32 : (ipt == 2 ? 13 * 32 : (ipt == 3 ? 11 * 32 : 9 * 32));
}
// Wider instantiations for 2 to 4 items a thread allow up to 16 consumer
// warps: more warps per SM to hide latency, each thread held to fewer
// registers (65536 / the block rounded up to 128 threads). A launch takes the
// narrowest instantiation its threads fit.
constexpr int kStreamWide1 = 16 * 32, kStreamWide2 = 17 * 32;
__host__ __device__ constexpr int stream_thread_limit(int ipt) {
    return (ipt >= 2 && ipt <= 4) ? kStreamWide2 : stream_max_threads(ipt);
}
// items (k-vectors of a plane) per consumer thread: 1 .. kStreamMaxIpt
constexpr int kStreamMaxIpt = 6;
constexpr int kStreamMaxSmem = 227 * 1024;
// Division by an invariant divisor d >= 1 of dividends n < 2^31, by one
// multiply and shift (T. Granlund and P. Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994): with l = ceil(log2 d) and
// m = ceil(2^(31+l) / d), n / d = (n * m) >> (31 + l) exactly (m < 2^33, so
// the product fits 64 bits).
struct FastDiv {
    uint64_t m;
    int sh;
};
__host__ __device__ inline FastDiv make_fastdiv(int64_t d) {
    int l = 0;
    while (((int64_t)1 << l) < d) ++l;
    const int sh = 31 + l;
    return FastDiv{(((uint64_t)1 << sh) + (uint64_t)d - 1) / (uint64_t)d, sh};
}
__host__ __device__ __forceinline__ uint32_t fast_div(uint32_t n, FastDiv f) {
    return (uint32_t)(((unsigned long long)n * f.m) >> f.sh);
}

// Warps per track of a deposition: a step's tracks alone rarely fill the GPU
// (a few to a few thousand per step), so with few tracks each box is shared by
// up to 8 warps.
__host__ __device__ inline int deposit_parts(int64_t m, int sms) {
    const int64_t warps = (int64_t)sms * 32;  // half the resident warps of the GPU
    int p = 8;
    while (p > 1 && m * p > warps) p >>= 1;
    return p;
}

// AUTO picks the streaming kernel from this many allocated cells (no_xy^2 * kpitch)
constexpr int64_t kStreamMinCells = 100000000;

// Launch shape of the streaming step kernel.
struct StreamShape {
    int tile_rows, planes_per_item, stages, consumer_warps, ctas_per_sm, sm_count;
};

int stream_smem_bytes(int tj, int kp, int stages);
int launch_stream_step(const pic_grid *g, const StreamShape &sh, const void *pos_in, const void *neg_in,
                       void *pos_out, void *neg_out, const void *dens, void *dens_zero, double *tally, void *ws,
                       cudaStream_t st);
// Fills the shape fields of *g (variant .. ctas_per_sm) where they are 0.
int resolve_shape(pic_grid *g);
constexpr int64_t kWorkspaceBytes = kMaxStepBlocks * 4 * (int64_t)sizeof(double) + 256;

// The scored-column test of the reference, (i - mid)^2 + (j - mid)^2 < r2
// with mid = no_xy / 2 (pulsed_ion_chamber/config.py:254-255), in exact
// integer form: with dx = 2 i - 2 mid and dy = 2 j - 2 mid (integers), the
// float64 comparison is exact (half-integer squares are exact) and equals
// dx^2 + dy^2 <= ceil(4 r2) - 1. Keeps float64 off the per-voxel path (the
// GPU's FP64 rate is ~1/64 of its FP32 rate).
struct ScoreTest {
    int64_t two_mid;
    int64_t thr4;
};
int score_test(const pic_grid *g, ScoreTest *out);
__host__ __device__ inline bool scored_column(const ScoreTest &t, int64_t i, int64_t j) {
    const int64_t dx = 2 * i - t.two_mid, dy = 2 * j - t.two_mid;
    return dx * dx + dy * dy <= t.thr4;
}

// Row pitch of the 2D density: no_xy rounded up to 4 elements, so every row
// starts 16-byte aligned and a row segment can be fetched by a bulk copy.
inline int64_t dens_pitch(int64_t no_xy) { return (no_xy + 3) / 4 * 4; }

// A named NVTX range over an entry point's host-side work (header-only NVTX:
// a no-op unless a profiler is attached), so that a kernel launch list taken
// with ncu --nvtx splits by phase: segments, graph replays, batched steps,
// gradient passes.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

int set_error(int code, const std::string &msg);
int set_cuda_error(const char *what, cudaError_t e);
int check_launch(const char *what);

// Largest useful grid for the step kernel on the current device (SMs x
// resident blocks), cached per device.
int64_t step_grid_cap(int f64);
int sm_count();
int step_occupancy(int dtype, int *blocks_per_sm);

int launch_step(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                const void *dens, void *dens_zero, double *tally, void *ws, cudaStream_t st);
// The deposition of one step's m tracks into dens. ws / ws_bytes: the step
// workspace when the caller has one (null otherwise); its track lists, behind
// the fixed part, let the binned form run.
int launch_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t m, void *dens,
                   uint32_t *counts, cudaStream_t st, void *ws = nullptr, int64_t ws_bytes = 0);

// Binned tile deposition (deposit.cu): a binning launch evaluates each
// track's Gaussian row and column factors once and lists the track in the
// tiles of kBinOut x kBinOut cells its written box meets; then one block per
// tile sums its tracks' outer products in a fixed order and stores each cell
// once. One pair of launches serves up to kBinSteps steps of a segment (their
// tracks together at most kBinTracks), each step a slot with its own track
// lists and its own pair buffer in the workspace. The scratch sits in the
// step workspace behind kWorkspaceBytes: a count per slot and tile (zero
// between launches; the tile's block clears it), kBinCap track indices per
// slot and tile (a tile with more scans its slot's tracks), the boxes and
// factors of kBinTracks tracks, and kBinSteps pair buffers.
constexpr int kBinOut = 62;
constexpr int kBinCap = 4096;
constexpr int kBinSteps = 8;
constexpr int kBinTracks = 65536;
constexpr int kBinBox = 64;               // factors kept per track and axis
constexpr int64_t kBinMaxNoXy = 4096;     // largest grid with track lists
// AUTO: the binned form for a segment's steps (up to eight per launch pair)
// where those launches give every SM a block (tiles x 8 >= SMs) or a tile
// meets about kBinAutoPerTile tracks of a step at most, so one block's serial
// sum stays short. Measured on GB300, per step against the per-track warps:
// 1068^2 with 8 500 tracks 20 against 64 us, 608^2 with 27 000 106 against
// 133, 208^2 with 300 6 against 11, 128^2 with 109 4.5 against 7.7, 48^2
// with 101 3.5 against 3.8 and with ~290 (~630 a tile) a 10 um column's
// whole run 18.3 against 22.1 ms; 108^2 with 632 (~350 a tile) 8.1 against
// 6.9; 48^2 with 1 011 (~2 200 a tile) 16 against 10.5. One step alone (the
// checkpointed gradient) only where the grid's tiles give at least
// kBinAutoTilesPerSm blocks per SM (no_xy >= 1055 on 152 SMs; 608^2 with
// 27 000 tracks 158 against 132 us, 208^2 20 against 11).
constexpr int kBinAutoTilesPerSm = 2;
constexpr int kBinAutoPerTile = 1024;
constexpr int kBinSpan = 256;  // steps one launch pair may span, idle steps between included
inline int64_t bin_tiles_per_side(int64_t n) { return (n + kBinOut - 1) / kBinOut; }
inline int64_t bin_align(int64_t b) { return (b + 255) / 256 * 256; }
inline int64_t bin_count_bytes(int64_t n) {
    const int64_t t = bin_tiles_per_side(n);
    return bin_align(kBinSteps * t * t * 4);
}
inline int64_t bin_list_bytes(int64_t n) {
    const int64_t t = bin_tiles_per_side(n);
    return kBinSteps * t * t * kBinCap * 4;
}
inline int64_t bin_box_bytes() { return bin_align((int64_t)kBinTracks * 8); }
inline int64_t bin_fac_bytes(int64_t es) { return (int64_t)kBinTracks * 2 * kBinBox * es; }
inline int64_t bin_dens_bytes(int64_t n, int64_t es) { return bin_align(n * dens_pitch(n) * 2 * es); }
// A grid takes the binned form when its track lists fit (no_xy <= 4096) and
// every truncation box, [ceil(c - cut), floor(c + cut)], spans at most
// kBinBox cells (floor(2 cut) + 1 of them at most).
inline bool bin_eligible(const pic_grid *g) {
    return g->no_xy <= kBinMaxNoXy && g->cutoff_voxels > 0.0 && 2.0 * g->cutoff_voxels + 1.0 < (double)kBinBox;
}
inline int64_t dep_bin_bytes(const pic_grid *g) {
    if (!bin_eligible(g)) return 0;
    const int64_t es = g->dtype == PIC_F64 ? 8 : 4;
    return bin_count_bytes(g->no_xy) + bin_list_bytes(g->no_xy) + bin_box_bytes() + bin_fac_bytes(es) +
           kBinSteps * bin_dens_bytes(g->no_xy, es);
}
// The binned deposition of a batched global step (batched.cu): its workspace
// (a slot per grid, per-tile counts and lists, per-track boxes and factors).
constexpr int kBinMaxSlots = 1024;
int64_t batched_deposit_bytes(int32_t n_cfgs, int32_t total_tiles, int64_t max_tracks, int64_t dens_bytes,
                              int32_t dtype);

// Whether the deposition takes the binned form for this grid and workspace:
// for a segment's steps together (most = the most tracks one of them has),
// or with most < 0 for one step alone.
bool deposit_binned(const pic_grid *g, const void *ws, int64_t ws_bytes, int64_t most);
// The end of the next launch pair's steps from s0: at most kBinSteps of them
// with tracks (*n_dep), kBinTracks tracks and kBinSpan steps.
int64_t next_deposit_group(const int64_t *off, int64_t s0, int64_t n_steps, int64_t *n_dep);
// The binned deposition of steps s0 .. s1 - 1 (tracks xs/ys[off[s] ..
// off[s + 1]), a group of next_deposit_group) into targets[k] for the k-th
// step with tracks, or with targets null into the workspace's pair buffers:
// dens[s - s0] is step s's pairs, or null for a step without tracks.
int launch_deposit_steps(const pic_grid *g, const double *xs, const double *ys, const int64_t *off, int64_t s0,
                         int64_t s1, uint32_t *counts, void *ws, void *const *targets, const void **dens,
                         cudaStream_t st);
// Kernel launches issued by this library so far (every launch site reports
// to check_launch; a captured graph's launches count at each replay).
void count_launches(int64_t n);

using BatchLaunch = pic_batch_launch;
int batched_workspace_bytes(int32_t n_blocks, int32_t n_cfgs, int64_t *bytes);
int batched_loop(const BatchLaunch &L, cudaStream_t st);
int batched_persistent(const BatchLaunch &L, const int64_t *step_task_off, const int64_t *step_tracks,
                       cudaStream_t st);
int batched_status(const BatchLaunch &L, cudaStream_t st, int32_t *status);
// The streaming batched step (batched_stream.cu).
int batched_stream_workspace_bytes(int32_t n_cfgs, int32_t n_items, int32_t consumer_warps, int64_t *bytes);
int batched_stream_prepare(const pic_batch_cfg *cfgs, int32_t n_cfgs, const int32_t *items, int32_t n_items,
                           const int32_t *tile_rows, int32_t consumer_warps, void *ws, int64_t ws_bytes,
                           cudaStream_t st, pic_batch_stream *out);
// dens: the step's deposition pairs in the packed layout; dens_zero: pairs the
// step clears for the next one (null: none)
int batched_stream_step(const BatchLaunch &L, const pic_batch_stream &B, int bi, int bo, int64_t step,
                        const void *dens, void *dens_zero, cudaStream_t st);
int batched_stream_status(const pic_batch_stream &B, int32_t reset, cudaStream_t st, int32_t *status);
// batched_loop with B non-null runs the streaming step instead of the flat one.
int batched_loop_stream(const BatchLaunch &L, const pic_batch_stream *B, cudaStream_t st);

// Several steps of one grid per cooperative launch (multistep.cu): for a
// resolved FLAT grid with steps_per_launch > 1.
constexpr int kMaxMultiSteps = 256;
bool multistep_eligible(const pic_grid *resolved);
int launch_multistep(const pic_grid *g, void *const pos[2], void *const neg[2], int parity, int n_steps,
                     const double *xs, const double *ys, const int64_t *off, void *const dens[2], int dens_parity,
                     uint32_t *counts, double *tally, void *ws, cudaStream_t st);

int step_noalloc(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                 const double *xs, const double *ys, int64_t n_tracks, uint32_t *counts, double *tally,
                 cudaStream_t st);
int step_noalloc_status(int32_t reset, cudaStream_t st, int32_t *status);

int adjoint_workspace_bytes(int64_t *bytes);
int launch_adjoint(const pic_grid *g, const void *pos, const void *neg, const void *dens, void *lp_in, void *ln_in,
                   void *lp_out, void *ln_out, double *grad, void *ws, cudaStream_t st, bool accumulate = false);
int adjoint_accumulate_begin(const pic_grid *g, void *ws, cudaStream_t st);
// The streaming adjoint (adjoint_stream.cu): float32 grids with
// adjoint_variant STREAM, or AUTO and at least kAdjStreamMinCells cells (the
// grid no longer fits L2 and the flat kernel waits on its neighbour loads).
constexpr int64_t kAdjStreamMinCells = (int64_t)1 << 24;
bool adjoint_stream_eligible(const pic_grid *g);
int launch_adjoint_stream(const pic_grid *g, const void *pos, const void *neg, const void *dens, const void *lp_in,
                          const void *ln_in, void *lp_out, void *ln_out, double *grad, unsigned int *counter,
                          int *status, double *partials, int64_t max_blocks, cudaStream_t st, bool accumulate);
int adjoint_accumulate_end(const pic_grid *g, void *ws, double *grad, cudaStream_t st);

// Binomial checkpointing (revolve.cu).
int revolve_plan(int64_t n_steps, int64_t n_slots, int64_t *recompute_steps, int64_t *spine_levels);
int revolve_spine(int64_t n_steps, int64_t n_slots, int64_t *steps, int64_t cap, int64_t *n_levels);
int revolve_trace(int64_t n_steps, int64_t n_slots, int64_t *events, int64_t cap, int64_t *n_events,
                  int64_t *advanced);
int revolve_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                    const double *xs, const double *ys, const int64_t *off, void *dens, uint32_t *counts,
                    double *tally, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots, void *ws,
                    int64_t ws_bytes, cudaStream_t st);
int revolve_backward(const pic_grid *g, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots,
                     int64_t n_steps, const double *xs, const double *ys, const int64_t *off, void *dens,
                     void *work_pos0, void *work_neg0, void *work_pos1, void *work_neg1, void *lam_pos0,
                     void *lam_neg0, void *lam_pos1, void *lam_neg1, double *grad, void *ws, int64_t ws_bytes,
                     void *adj_ws, cudaStream_t st);

int selftest_waits(int32_t *barrier_status, int32_t *mbarrier_status, cudaStream_t st);

int sample_disc(const double *u, int64_t n_pairs, double scale, double mid, double radius_sq, int64_t n_wanted,
                double *xs, double *ys, int64_t *n_accepted, int64_t *n_pairs_used);
int arrival_counts_pcg64(uint64_t *st, int64_t n, double duration, const double *edges, int64_t n_edges,
                         int64_t *counts);
int sample_disc_pcg64(uint64_t *st, double scale, double mid, double radius_sq, int64_t n_wanted, int64_t max_pairs,
                      double *xs, double *ys, int64_t *n_accepted, int64_t *n_draws);

}  // namespace pic
