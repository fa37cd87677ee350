// capi.cu -- the extern "C" entry points of libpic_gb300.so (declared in
// include/pic_gb300.h): argument checks, error reporting, the per-segment
// host loop and its CUDA-graph capture.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <atomic>
#include <cmath>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "pic_internal.h"

namespace pic {

static thread_local std::string g_last_error;

int set_error(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

int set_cuda_error(const char *what, cudaError_t e) {
    return set_error(PIC_E_CUDA, std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")");
}

// Kernel launches this library has issued. A thread capturing a graph
// (pic_graph_create, pic_capture_begin .. _end) counts its launches into the
// graph instead, and every replay of the graph adds them.
static std::atomic<int64_t> g_launches{0};
static thread_local int64_t t_captured = -1;  // >= 0 while this thread captures
static std::mutex g_graph_mu;
static std::unordered_map<uintptr_t, int64_t> g_graph_launches;

void count_launches(int64_t n) {
    if (t_captured >= 0)
        t_captured += n;
    else
        g_launches += n;
}

static void graph_launches_set(uintptr_t exec, int64_t n) {
    std::lock_guard<std::mutex> lock(g_graph_mu);
    g_graph_launches[exec] = n;
}

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_cuda_error(what, e);
    count_launches(1);
    return PIC_OK;
}

int64_t step_grid_cap(int f64) {
    static std::mutex mu;
    static std::vector<int64_t> cache[2];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return kMaxStepBlocks;
    std::lock_guard<std::mutex> lock(mu);
    auto &c = cache[f64 ? 1 : 0];
    if ((int)c.size() <= dev) c.resize(dev + 1, 0);
    if (c[dev] == 0) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (step_occupancy(f64 ? PIC_F64 : PIC_F32, &per_sm) != PIC_OK || per_sm < 1) per_sm = 1;
        int64_t cap = (int64_t)sms * per_sm;
        c[dev] = cap < 1 ? 1 : (cap > kMaxStepBlocks ? kMaxStepBlocks : cap);
    }
    return c[dev];
}

int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = sms > 0 ? sms : 152;
    }
    return cached[dev];
}

int score_test(const pic_grid *g, ScoreTest *out) {
    const double two_mid = 2.0 * g->mid_xy;
    if (!(two_mid == std::floor(two_mid)) || two_mid < 0.0 || two_mid > 4.0 * (double)g->no_xy)
        return set_error(PIC_E_INVALID, "mid_xy must be a multiple of 0.5 inside the grid (no_xy / 2)");
    out->two_mid = (int64_t)two_mid;
    const double r4 = 4.0 * g->scoring_radius_sq;  // exact: power-of-two scaling
    const double cap = 4.0e18;
    if (!(r4 > 0.0)) return set_error(PIC_E_INVALID, "scoring_radius_sq must be positive");
    if (r4 >= cap) {
        out->thr4 = (int64_t)cap;
    } else {
        out->thr4 = (int64_t)std::ceil(r4) - 1;
    }
    return PIC_OK;
}

int resolve_shape(pic_grid *g) {
    // Measured on GB300 (graph-replayed steps, idle / pulse): the flat kernel
    // is faster up to a few hundred lateral cells (62.6 / 77.9 us vs 86.4 /
    // 95.8 us at 208x208x408; 146 / 174 vs 176 / 191 us at 328x328x408); the
    // streaming kernel in its 13-consumer-warp form wins from 608x608x408
    // (437 / 438 vs 454 / 492 us) to the 1068x1068x408 full electrode (1.250 /
    // 1.255 ms vs 1.73 / 1.95 ms).
    if (g->variant == PIC_VARIANT_AUTO)
        g->variant = (g->dtype == PIC_F32 && g->no_xy >= 64 && g->no_xy * g->no_xy * g->kpitch >= kStreamMinCells)
                         ? PIC_VARIANT_STREAM
                         : PIC_VARIANT_FLAT;
    if (g->variant == PIC_VARIANT_FLAT) return PIC_OK;
    if (g->variant != PIC_VARIANT_STREAM) return set_error(PIC_E_INVALID, "variant must be PIC_VARIANT_AUTO, _FLAT or _STREAM");
    if (g->dtype != PIC_F32) return set_error(PIC_E_INVALID, "the stream variant supports float32 fields only");
    if (g->no_xy < 4) return set_error(PIC_E_INVALID, "the stream variant needs no_xy >= 4");
    const int kp = (int)g->kpitch, c4 = kp / 4;
    // default: 13 consumer warps (one 512-thread form, 128 registers a
    // thread) and tiles of about three k-vectors a thread -- on the full
    // electrode 12 rows x 5 stages, 1.216 ms a step, within 1.1 % of the
    // fastest of 2 150 shapes timed by the full autotuner (15 warps, 1.202 ms)
    if (g->consumer_warps <= 0) g->consumer_warps = 13;
    if (g->consumer_warps > kStreamMaxThreads / 32 - 1)
        return set_error(PIC_E_INVALID, "consumer_warps must be <= " + std::to_string(kStreamMaxThreads / 32 - 1));
    const int nct = g->consumer_warps * 32;
    if (g->tile_rows <= 0) {
        int tj = (3 * nct) / c4;
        if (tj < 1) tj = 1;
        if (tj > 16) tj = 16;
        while (tj > 1 && 2 * (tj + 2) * kp * 4 > 48 * 1024) --tj;
        g->tile_rows = tj;
    }
    if (g->tile_rows > (int)g->no_xy - 2) g->tile_rows = (int)g->no_xy - 2;
    if (g->tile_rows * c4 > kStreamMaxIpt * nct)
        return set_error(PIC_E_INVALID, "stream variant: tile_rows * kpitch/4 must be <= " +
                                            std::to_string(kStreamMaxIpt) + " * 32 * consumer_warps");
    {
        const int ipt = (g->tile_rows * c4 + nct - 1) / nct;
        if (nct + 32 > stream_thread_limit(ipt))
            return set_error(PIC_E_INVALID, "stream variant: " + std::to_string(g->consumer_warps) +
                                                " consumer warps exceed the register budget of " +
                                                std::to_string(ipt) + " items per thread");
    }
    const int stage_bytes = (2 * (g->tile_rows + 2) * kp + 2 * ((g->tile_rows + 8) & ~3)) * 4;
    // static shared memory of the kernel (reduction scratch, flags) is < 2 KB
    const int budget = kStreamMaxSmem - 2048;
    if (g->stages <= 0) {
        int s = (budget - 256) / stage_bytes;
        g->stages = s > 16 ? 16 : s;
    }
    if (g->stages < 4) return set_error(PIC_E_CAPACITY, "the stream variant needs 4 shared-memory stages for this k extent");
    if (g->stages > 16) return set_error(PIC_E_INVALID, "stream variant: at most 16 stages");
    if (stream_smem_bytes(g->tile_rows, kp, g->stages) > budget)
        return set_error(PIC_E_CAPACITY, "stream variant: tile_rows x stages exceed shared memory");
    if (g->planes_per_item <= 0) {
        // about 12 work items per SM (a whole item per CTA keeps the load
        // balanced and the ring full), between 4 and 64 planes per item
        const int64_t jt = (g->no_xy - 2 + g->tile_rows - 1) / g->tile_rows;
        const int64_t target = 12LL * sm_count();
        int64_t li = ((g->no_xy - 2) * jt + target - 1) / target;
        g->planes_per_item = (int32_t)(li < 4 ? 4 : (li > 64 ? 64 : li));
    }
    if (g->ctas_per_sm <= 0) g->ctas_per_sm = 1;
    return PIC_OK;
}

static bool aligned(const void *p, uintptr_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

static int check_grid(const pic_grid *g) {
    if (!g) return set_error(PIC_E_INVALID, "grid descriptor is null");
    if (g->dtype != PIC_F32 && g->dtype != PIC_F64) return set_error(PIC_E_INVALID, "dtype must be PIC_F32 or PIC_F64");
    if (g->wall != PIC_WALL_ABSORBING && g->wall != PIC_WALL_REFLECTING)
        return set_error(PIC_E_INVALID, "wall must be PIC_WALL_ABSORBING or PIC_WALL_REFLECTING");
    if (g->no_xy < 3) return set_error(PIC_E_INVALID, "no_xy must be >= 3");
    if (g->nzb < 3) return set_error(PIC_E_INVALID, "no_z_with_buffer must be >= 3");
    if (g->kpitch != pic_kpitch(g->nzb)) return set_error(PIC_E_INVALID, "kpitch must equal pic_kpitch(no_z_with_buffer)");
    if (g->nze < 1) return set_error(PIC_E_INVALID, "no_z_electrode must be >= 1 (k = 0 is the fixed end plane)");
    if (g->no_z < 1 || g->nze + g->no_z > g->nzb - 1)
        return set_error(PIC_E_INVALID, "gap layers [no_z_electrode, no_z_electrode + no_z) must lie inside 1 .. nzb-2");
    if (g->no_xy > (int64_t)1 << 20 || g->nzb > (int64_t)1 << 20)
        return set_error(PIC_E_CAPACITY, "grid extent beyond 2^20 voxels per axis");
    if (!(g->cutoff_voxels > 0.0)) return set_error(PIC_E_INVALID, "cutoff_voxels must be positive");
    if (g->steps_per_launch < 0 || g->steps_per_launch > kMaxMultiSteps)
        return set_error(PIC_E_INVALID, "steps_per_launch must be 0 .. 256");
    if (g->adjoint_variant != PIC_VARIANT_AUTO && g->adjoint_variant != PIC_VARIANT_FLAT &&
        g->adjoint_variant != PIC_VARIANT_STREAM)
        return set_error(PIC_E_INVALID, "adjoint_variant must be PIC_VARIANT_AUTO, _FLAT or _STREAM");
    if (g->adjoint_variant == PIC_VARIANT_STREAM && g->dtype != PIC_F32)
        return set_error(PIC_E_INVALID, "the stream adjoint variant supports float32 fields only");
    if (g->deposit_variant != PIC_DEPOSIT_AUTO && g->deposit_variant != PIC_DEPOSIT_TRACKS &&
        g->deposit_variant != PIC_DEPOSIT_BINNED)
        return set_error(PIC_E_INVALID, "deposit_variant must be PIC_DEPOSIT_AUTO, _TRACKS or _BINNED");
    ScoreTest t;
    return score_test(g, &t);
}

static int check_fields(const void *a, const void *b, const void *c, const void *d) {
    const void *ps[4] = {a, b, c, d};
    for (const void *p : ps) {
        if (!p) return set_error(PIC_E_INVALID, "field pointer is null");
        if (!aligned(p, 32)) return set_error(PIC_E_INVALID, "field pointers must be 32-byte aligned");
    }
    return PIC_OK;
}

static int run_loop(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                    int64_t n_steps, const double *xs, const double *ys, const int64_t *off, void *dens0,
                    void *dens1, int64_t dens_parity, uint32_t *counts, double *tally, void *ws,
                    int64_t ws_bytes, cudaStream_t st) {
    void *pos[2] = {pos0, pos1}, *neg[2] = {neg0, neg1}, *dens[2] = {dens0, dens1};
    pic_grid r = *g;
    int rc0 = resolve_shape(&r);
    if (rc0) return rc0;
    if (multistep_eligible(&r)) {
        // up to steps_per_launch steps per cooperative launch
        const int64_t K = r.steps_per_launch;
        unsigned int *bar = workspace_layout(ws).counter + 16;
        for (int64_t s0 = 0; s0 < n_steps; s0 += K) {
            const int64_t m = n_steps - s0 < K ? n_steps - s0 : K;
            cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned int), st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(barrier)", e);
            int rc = launch_multistep(&r, pos, neg, (int)((parity + s0) & 1), (int)m, xs, ys, off + s0, dens,
                                      (int)((dens_parity + s0) & 1), counts, tally + 4 * s0, ws, st);
            if (rc) return rc;
        }
        return PIC_OK;
    }
    int64_t most = 0;
    for (int64_t s = 0; s < n_steps; ++s) most = std::max(most, off[s + 1] - off[s]);
    if (most > 0 && most <= kBinTracks && deposit_binned(g, ws, ws_bytes, most)) {
        // the binned deposition of up to kBinSteps steps (kBinTracks tracks)
        // at a time into the workspace's pair buffers, then those steps
        const void *dp[kBinSpan];
        const void *last_pairs = nullptr;  // the pairs of the segment's last step (null: no tracks)
        for (int64_t s0 = 0; s0 < n_steps;) {
            int64_t nd = 0;
            const int64_t s1 = next_deposit_group(off, s0, n_steps, &nd);
            int rc = launch_deposit_steps(g, xs, ys, off, s0, s1, counts, ws, nullptr, dp, st);
            if (rc) return rc;
            for (int64_t s = s0; s < s1; ++s) {
                const int bi = (int)((parity + s) & 1);
                if ((rc = launch_step(g, pos[bi], neg[bi], pos[bi ^ 1], neg[bi ^ 1], dp[s - s0], nullptr, tally + 4 * s,
                                      ws, st)))
                    return rc;
            }
            if (s1 == n_steps) last_pairs = dp[s1 - 1 - s0];
            s0 = s1;
        }
        // The caller's pair buffers, as the per-step forms leave them: the
        // last step's pairs if it deposited, and a zero buffer for the step
        // after the segment.
        const int64_t pb = dens_pitch(g->no_xy) * 2 * g->no_xy * (g->dtype == PIC_F64 ? 8 : 4);
        const int last = (int)((dens_parity + n_steps - 1) & 1);
        if (last_pairs) {
            cudaError_t e = cudaMemcpyAsync(dens[last], last_pairs, (size_t)pb, cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemcpyAsync(deposition pairs)", e);
        }
        cudaError_t e = cudaMemsetAsync(dens[last ^ 1], 0, (size_t)pb, st);
        return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaMemsetAsync(deposition pairs)", e);
    }
    for (int64_t s = 0; s < n_steps; ++s) {
        const int bi = (int)((parity + s) & 1), bo = bi ^ 1;
        const int di = (int)((dens_parity + s) & 1);
        const int64_t m = off[s + 1] - off[s];
        if (m > 0) {
            int rc = launch_deposit(g, xs + off[s], ys + off[s], m, dens[di], counts, st, ws, ws_bytes);
            if (rc) return rc;
        }
        // The buffer step s+1 accumulates into was last written at step s-1.
        const bool zero_next = (s == 0) || (off[s] - off[s - 1] > 0);
        int rc = launch_step(g, pos[bi], neg[bi], pos[bo], neg[bo], m > 0 ? dens[di] : nullptr,
                             zero_next ? dens[di ^ 1] : nullptr, tally + 4 * s, ws, st);
        if (rc) return rc;
    }
    return PIC_OK;
}

static int check_segment(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                         const double *xs, const double *ys, const int64_t *off, void *dens0, void *dens1,
                         uint32_t *counts, double *tally, void *ws, int64_t ws_bytes) {
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(pos0, neg0, pos1, neg1))) return rc;
    if (n_steps < 0) return set_error(PIC_E_INVALID, "n_steps must be >= 0");
    if (!off || !tally || !dens0 || !dens1 || !counts) return set_error(PIC_E_INVALID, "null pointer argument");
    if (!ws || ws_bytes < kWorkspaceBytes) return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    for (int64_t s = 0; s < n_steps; ++s)
        if (off[s + 1] < off[s]) return set_error(PIC_E_INVALID, "track_offsets must be non-decreasing");
    if (n_steps > 0 && off[n_steps] > off[0] && (!xs || !ys)) return set_error(PIC_E_INVALID, "track arrays are null");
    return PIC_OK;
}

// What every batched launch needs: buffers, step range and task tables.
static int check_batch_common(const pic_batch_launch *L) {
    if (!L) return set_error(PIC_E_INVALID, "launch descriptor is null");
    if (L->dtype != PIC_F32 && L->dtype != PIC_F64) return set_error(PIC_E_INVALID, "dtype must be PIC_F32 or PIC_F64");
    if (L->n_cfgs < 1) return set_error(PIC_E_INVALID, "n_cfgs must be >= 1");
    if (L->n_steps < 0 || L->first_step < 0) return set_error(PIC_E_INVALID, "step range must be non-negative");
    if (!L->cfgs || !L->counts || !L->tally || !L->dens[0] || !L->dens[1])
        return set_error(PIC_E_INVALID, "null pointer in the batch launch descriptor");
    int rc = check_fields(L->pos[0], L->neg[0], L->pos[1], L->neg[1]);
    if (rc) return rc;
    if (!L->step_task_off || !L->step_tracks || !L->step_blocks)
        return set_error(PIC_E_INVALID, "step task tables are null");
    for (int64_t s = 0; s < L->n_steps; ++s) {
        if (L->step_task_off[s + 1] < L->step_task_off[s] || L->step_tracks[s] < 0)
            return set_error(PIC_E_INVALID, "step task offsets must be non-decreasing");
        if (L->step_tracks[s] > 0 && (!L->task_cfg || !L->task_first || !L->task_prefix || !L->xs || !L->ys))
            return set_error(PIC_E_INVALID, "track or task arrays are null");
        if (L->step_tracks[s] > 0 && !L->dep_workspace &&
            (L->step_blocks[s] < 1 || L->step_blocks[s] > 0x7fffffffLL))
            return set_error(PIC_E_INVALID, "step_blocks must give each depositing step 1 .. 2^31-1 blocks");
        if (L->dep_workspace && L->step_tracks[s] > L->dep_max_tracks)
            return set_error(PIC_E_INVALID, "a global step has more tracks than dep_max_tracks");
    }
    if (L->dep_workspace) {
        if (L->n_cfgs > kBinMaxSlots) return set_error(PIC_E_INVALID, "the binned batched deposition takes at most 1024 grids");
        if (L->dep_total_tiles < 1 || L->dep_max_tiles < 1 || L->dep_max_tiles > L->dep_total_tiles ||
            L->dep_max_tracks < 0 || L->dep_dens_bytes < 1)
            return set_error(PIC_E_INVALID,
                             "dep_total_tiles, dep_max_tiles, dep_max_tracks and dep_dens_bytes are inconsistent");
        if (!aligned(L->dep_workspace, 256) ||
            L->dep_workspace_bytes < batched_deposit_bytes(L->n_cfgs, L->dep_total_tiles, L->dep_max_tracks,
                                                           L->dep_dens_bytes, L->dtype))
            return set_error(PIC_E_INVALID, "dep_workspace too small or not 256-byte aligned (pic_batched_deposit_bytes)");
    }
    return PIC_OK;
}

static int check_batch(const pic_batch_launch *L) {
    int rc = check_batch_common(L);
    if (rc) return rc;
    if (L->n_blocks < 1) return set_error(PIC_E_INVALID, "n_cfgs and n_blocks must be >= 1");
    if (L->index32 != 0 && L->index32 != 1) return set_error(PIC_E_INVALID, "index32 must be 0 or 1");
    if (!L->blk_cfg || !L->blk_item0 || !L->blk_item1 || !L->cfg_blk0 || !L->cfg_nblk || !L->workspace)
        return set_error(PIC_E_INVALID, "null pointer in the batch launch descriptor");
    int64_t need = 0;
    if ((rc = batched_workspace_bytes(L->n_blocks, L->n_cfgs, &need))) return rc;
    if (L->workspace_bytes < need) return set_error(PIC_E_INVALID, "workspace too small (pic_batched_workspace_bytes)");
    return PIC_OK;
}

}  // namespace pic

using namespace pic;

extern "C" {

const char *pic_last_error(void) { return g_last_error.c_str(); }

// The Python binding mirrors pic_grid field by field (ABI 5: 5 int64, 14
// double, 9 int32, padded to 8 bytes).
static_assert(sizeof(pic_grid) == 200, "pic_grid layout changed: bump pic_abi_version and the bindings");

int pic_abi_version(void) { return 8; }

int64_t pic_kpitch(int64_t nzb) { return (nzb + 7) / 8 * 8; }

int64_t pic_dens_pitch(int64_t no_xy) { return dens_pitch(no_xy); }

int pic_device_info(int32_t *sm_count, int64_t *total_bytes, int32_t *cc_major, int32_t *cc_minor) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error("cudaGetDevice", e);
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return set_cuda_error("cudaGetDeviceProperties", e);
    if (sm_count) *sm_count = prop.multiProcessorCount;
    if (total_bytes) *total_bytes = (int64_t)prop.totalGlobalMem;
    if (cc_major) *cc_major = prop.major;
    if (cc_minor) *cc_minor = prop.minor;
    if (prop.major != 10 || prop.minor != 3)
        return set_error(PIC_E_DEVICE, "libpic_gb300 is built for sm_103a (GB300); current device is sm_" +
                                           std::to_string(prop.major) + std::to_string(prop.minor));
    return PIC_OK;
}

int pic_step_workspace_bytes(const pic_grid *g, int64_t *bytes) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!bytes) return set_error(PIC_E_INVALID, "bytes is null");
    *bytes = kWorkspaceBytes + dep_bin_bytes(g);
    return PIC_OK;
}

int pic_workspace_status(void *workspace, int32_t reset, uintptr_t stream, int32_t *status) {
    if (!workspace || !status) return set_error(PIC_E_INVALID, "null pointer argument");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    Workspace w = workspace_layout(workspace);
    int32_t v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, w.status, sizeof(v), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error("pic_workspace_status", e);
    *status = v;
    if (reset && v != 0) {
        e = cudaMemsetAsync(w.status, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error("pic_workspace_status reset", e);
    }
    return PIC_OK;
}

int pic_resolve_shape(const pic_grid *g, pic_grid *resolved) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!resolved) return set_error(PIC_E_INVALID, "resolved is null");
    *resolved = *g;
    return resolve_shape(resolved);
}

int pic_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t n_tracks, void *dens,
                uint32_t *counts, uintptr_t stream) {
    NvtxRange nvtx_range("pic_deposit");
    int rc = check_grid(g);
    if (rc) return rc;
    if (n_tracks < 0) return set_error(PIC_E_INVALID, "n_tracks must be >= 0");
    if (n_tracks == 0) return PIC_OK;
    if (!xs || !ys || !dens || !counts) return set_error(PIC_E_INVALID, "null pointer argument");
    return launch_deposit(g, xs, ys, n_tracks, dens, counts, reinterpret_cast<cudaStream_t>(stream));
}

int pic_step(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
             const void *dens, void *dens_zero, double *tally, void *workspace, int64_t workspace_bytes,
             uintptr_t stream) {
    NvtxRange nvtx_range("pic_step");
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(pos_in, neg_in, pos_out, neg_out))) return rc;
    if (pos_in == pos_out || neg_in == neg_out) return set_error(PIC_E_INVALID, "input and output fields must differ");
    if (!tally) return set_error(PIC_E_INVALID, "tally is null");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
        return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    return launch_step(g, pos_in, neg_in, pos_out, neg_out, dens, dens_zero, tally, workspace,
                       reinterpret_cast<cudaStream_t>(stream));
}

int pic_step_noalloc(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                     const double *xs, const double *ys, int64_t n_tracks, uint32_t *counts, double *tally,
                     uintptr_t stream) {
    NvtxRange nvtx_range("pic_step_noalloc");
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(pos_in, neg_in, pos_out, neg_out))) return rc;
    if (pos_in == pos_out || neg_in == neg_out) return set_error(PIC_E_INVALID, "input and output fields must differ");
    if (!tally || !counts) return set_error(PIC_E_INVALID, "null pointer argument");
    if (n_tracks < 0) return set_error(PIC_E_INVALID, "n_tracks must be >= 0");
    if (n_tracks > 0 && (!xs || !ys)) return set_error(PIC_E_INVALID, "track arrays are null");
    return step_noalloc(g, pos_in, neg_in, pos_out, neg_out, xs, ys, n_tracks, counts, tally,
                        reinterpret_cast<cudaStream_t>(stream));
}

int pic_step_noalloc_status(int32_t reset, uintptr_t stream, int32_t *status) {
    if (!status) return set_error(PIC_E_INVALID, "status is null");
    return step_noalloc_status(reset, reinterpret_cast<cudaStream_t>(stream), status);
}

int pic_sample_disc(const double *u, int64_t n_pairs, double scale, double mid, double radius_sq, int64_t n_wanted,
                    double *xs, double *ys, int64_t *n_accepted, int64_t *n_pairs_used) {
    if (n_pairs < 0 || n_wanted < 0) return set_error(PIC_E_INVALID, "n_pairs and n_wanted must be >= 0");
    if (!n_accepted || !n_pairs_used) return set_error(PIC_E_INVALID, "null pointer argument");
    if ((n_pairs > 0 && !u) || (n_wanted > 0 && (!xs || !ys))) return set_error(PIC_E_INVALID, "null pointer argument");
    return sample_disc(u, n_pairs, scale, mid, radius_sq, n_wanted, xs, ys, n_accepted, n_pairs_used);
}

int pic_arrival_counts_pcg64(uint64_t *state, int64_t n, double duration, const double *edges, int64_t n_edges,
                             int64_t *counts) {
    if (!state || !edges || !counts) return set_error(PIC_E_INVALID, "null pointer argument");
    if (n < 1 || n_edges < 2) return set_error(PIC_E_INVALID, "n must be >= 1 and n_edges >= 2");
    if ((state[3] & 1u) == 0u) return set_error(PIC_E_INVALID, "a PCG64 increment is odd");
    for (int64_t b = 0; b + 1 < n_edges; ++b)
        if (!(edges[b] <= edges[b + 1])) return set_error(PIC_E_INVALID, "edges must be non-decreasing");
    return arrival_counts_pcg64(state, n, duration, edges, n_edges, counts);
}

int pic_sample_disc_pcg64(uint64_t *state, double scale, double mid, double radius_sq, int64_t n_wanted,
                          int64_t max_pairs, double *xs, double *ys, int64_t *n_accepted, int64_t *n_draws) {
    if (!state || !n_accepted || !n_draws) return set_error(PIC_E_INVALID, "null pointer argument");
    if (n_wanted < 0 || max_pairs < 0) return set_error(PIC_E_INVALID, "n_wanted and max_pairs must be >= 0");
    if (n_wanted > 0 && (!xs || !ys)) return set_error(PIC_E_INVALID, "null pointer argument");
    if ((state[3] & 1u) == 0u) return set_error(PIC_E_INVALID, "a PCG64 increment is odd");
    return sample_disc_pcg64(state, scale, mid, radius_sq, n_wanted, max_pairs, xs, ys, n_accepted, n_draws);
}

int pic_adjoint_workspace_bytes(const pic_grid *g, int64_t *bytes) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!bytes) return set_error(PIC_E_INVALID, "bytes is null");
    return adjoint_workspace_bytes(bytes);
}

int pic_adjoint_step(const pic_grid *g, const void *pos, const void *neg, const void *dens, void *lam_pos_in,
                     void *lam_neg_in, void *lam_pos_out, void *lam_neg_out, double *grad, void *workspace,
                     int64_t workspace_bytes, uintptr_t stream) {
    NvtxRange nvtx_range("pic_adjoint_step");
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(pos, neg, lam_pos_in, lam_neg_in)) || (rc = check_fields(lam_pos_out, lam_neg_out, pos, neg)))
        return rc;
    if (lam_pos_in == lam_pos_out || lam_neg_in == lam_neg_out)
        return set_error(PIC_E_INVALID, "adjoint input and output buffers must differ");
    if (!grad) return set_error(PIC_E_INVALID, "grad is null");
    int64_t need = 0;
    adjoint_workspace_bytes(&need);
    if (!workspace || workspace_bytes < need) return set_error(PIC_E_INVALID, "workspace too small (pic_adjoint_workspace_bytes)");
    return launch_adjoint(g, pos, neg, dens, lam_pos_in, lam_neg_in, lam_pos_out, lam_neg_out, grad, workspace,
                          reinterpret_cast<cudaStream_t>(stream));
}

// Slots of the kept densities: the d-th step with tracks uses slot d.
static int kept_slots(const int64_t *off, int64_t n_steps, int64_t *n_dep) {
    int64_t d = 0;
    for (int64_t s = 0; s < n_steps; ++s) {
        if (off[s + 1] < off[s]) return set_error(PIC_E_INVALID, "track_offsets must be non-decreasing");
        d += off[s + 1] > off[s];
    }
    *n_dep = d;
    return PIC_OK;
}

int pic_adjoint_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                        const double *xs, const double *ys, const int64_t *track_offsets, void *dens_keep,
                        uint32_t *counts, double *tally, void *ckpt_pos, void *ckpt_neg, int64_t ckpt_every,
                        int64_t state_stride, void *workspace, int64_t workspace_bytes, uintptr_t stream) {
    NvtxRange nvtx_range("pic_adjoint_forward");
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(pos0, neg0, pos1, neg1)) || (rc = check_fields(ckpt_pos, ckpt_neg, ckpt_pos, ckpt_neg)))
        return rc;
    if (n_steps < 0 || ckpt_every < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and ckpt_every >= 1");
    if (!track_offsets || !counts || !tally) return set_error(PIC_E_INVALID, "null pointer argument");
    const int64_t field = g->no_xy * g->no_xy * g->kpitch;
    if (state_stride < field || state_stride % 8 != 0)
        return set_error(PIC_E_INVALID, "state_stride must be >= no_xy^2 * kpitch and a multiple of 8 elements");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
        return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    int64_t n_dep = 0;
    if ((rc = kept_slots(track_offsets, n_steps, &n_dep))) return rc;
    if (n_dep > 0 && (!xs || !ys || !dens_keep)) return set_error(PIC_E_INVALID, "track or density arrays are null");
    if (n_dep > 0 && !aligned(dens_keep, 16)) return set_error(PIC_E_INVALID, "dens_keep must be 16-byte aligned");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t es = g->dtype == PIC_F64 ? 8 : 4;
    const int64_t dslot = 2 * g->no_xy * dens_pitch(g->no_xy);  // elements of one step's pairs
    if (n_dep > 0) {
        cudaError_t e = cudaMemsetAsync(dens_keep, 0, (size_t)(n_dep * dslot * es), st);
        if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(dens_keep)", e);
    }
    void *pos[2] = {pos0, pos1}, *neg[2] = {neg0, neg1};
    char *D = static_cast<char *>(dens_keep);
    auto checkpoint = [&](int64_t s) -> int {
        if (s % ckpt_every != 0) return PIC_OK;
        const int b = (int)(s & 1);
        const int64_t c = s / ckpt_every;
        cudaError_t e = cudaMemcpyAsync(static_cast<char *>(ckpt_pos) + c * state_stride * es, pos[b],
                                        (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(static_cast<char *>(ckpt_neg) + c * state_stride * es, neg[b], (size_t)(field * es),
                                cudaMemcpyDeviceToDevice, st);
        return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaMemcpyAsync(checkpoint)", e);
    };
    int64_t most = 0;
    for (int64_t s = 0; s < n_steps; ++s) most = std::max(most, track_offsets[s + 1] - track_offsets[s]);
    if (most > 0 && most <= kBinTracks && deposit_binned(g, workspace, workspace_bytes, most)) {
        // each launch pair deposits up to kBinSteps steps straight into their
        // kept slots
        const void *dp[kBinSpan];
        void *targets[kBinSteps];
        int64_t d = 0;
        for (int64_t s0 = 0; s0 < n_steps;) {
            int64_t nd = 0;
            const int64_t s1 = next_deposit_group(track_offsets, s0, n_steps, &nd);
            for (int64_t k = 0; k < nd; ++k) targets[k] = D + (d + k) * dslot * es;
            if ((rc = launch_deposit_steps(g, xs, ys, track_offsets, s0, s1, counts, workspace, targets, dp, st)))
                return rc;
            d += nd;
            for (int64_t s = s0; s < s1; ++s) {
                const int b = (int)(s & 1);
                if ((rc = checkpoint(s))) return rc;
                if ((rc = launch_step(g, pos[b], neg[b], pos[b ^ 1], neg[b ^ 1], dp[s - s0], nullptr, tally + 4 * s,
                                      workspace, st)))
                    return rc;
            }
            s0 = s1;
        }
        return PIC_OK;
    }
    int64_t d = 0;
    for (int64_t s = 0; s < n_steps; ++s) {
        const int b = (int)(s & 1);
        if (s % ckpt_every == 0) {
            const int64_t c = s / ckpt_every;
            cudaError_t e = cudaMemcpyAsync(static_cast<char *>(ckpt_pos) + c * state_stride * es, pos[b],
                                            (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess)
                e = cudaMemcpyAsync(static_cast<char *>(ckpt_neg) + c * state_stride * es, neg[b],
                                    (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemcpyAsync(checkpoint)", e);
        }
        const int64_t m = track_offsets[s + 1] - track_offsets[s];
        void *dens = nullptr;
        if (m > 0) {
            dens = D + (d++) * dslot * es;
            if ((rc = launch_deposit(g, xs + track_offsets[s], ys + track_offsets[s], m, dens, counts, st, workspace,
                                     workspace_bytes)))
                return rc;
        }
        rc = launch_step(g, pos[b], neg[b], pos[b ^ 1], neg[b ^ 1], dens, nullptr, tally + 4 * s, workspace, st);
        if (rc) return rc;
    }
    return PIC_OK;
}

int pic_adjoint_backward(const pic_grid *g, const void *ckpt_pos, const void *ckpt_neg, int64_t state_stride,
                         int64_t n_steps, int64_t ckpt_every, const int64_t *track_offsets, const void *dens_keep,
                         void *states_pos, void *states_neg, void *lam_pos0, void *lam_neg0, void *lam_pos1,
                         void *lam_neg1, double *grad, void *workspace,
                         int64_t workspace_bytes, void *adj_workspace, int64_t adj_workspace_bytes, uintptr_t stream) {
    NvtxRange nvtx_range("pic_adjoint_backward");
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(ckpt_pos, ckpt_neg, states_pos, states_neg)) ||
        (rc = check_fields(lam_pos0, lam_neg0, lam_pos1, lam_neg1)))
        return rc;
    if (n_steps < 0 || ckpt_every < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and ckpt_every >= 1");
    if (!track_offsets || !grad) return set_error(PIC_E_INVALID, "null pointer argument");
    const int64_t field = g->no_xy * g->no_xy * g->kpitch;
    if (state_stride < field || state_stride % 8 != 0)
        return set_error(PIC_E_INVALID, "state_stride must be >= no_xy^2 * kpitch and a multiple of 8 elements");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
        return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    int64_t need = 0;
    adjoint_workspace_bytes(&need);
    if (!adj_workspace || adj_workspace_bytes < need)
        return set_error(PIC_E_INVALID, "adjoint workspace too small (pic_adjoint_workspace_bytes)");
    int64_t n_dep = 0;
    if ((rc = kept_slots(track_offsets, n_steps, &n_dep))) return rc;
    if (n_dep > 0 && !dens_keep) return set_error(PIC_E_INVALID, "dens_keep is null");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const int64_t es = g->dtype == PIC_F64 ? 8 : 4;
    const int64_t dslot = 2 * g->no_xy * dens_pitch(g->no_xy);  // elements of one step's pairs
    const char *D = static_cast<const char *>(dens_keep);
    char *SP = static_cast<char *>(states_pos), *SN = static_cast<char *>(states_neg);
    // slot of every step's kept density (-1: none)
    std::vector<int64_t> slot(n_steps > 0 ? n_steps : 1);
    {
        int64_t d = 0;
        for (int64_t s = 0; s < n_steps; ++s) slot[s] = track_offsets[s + 1] > track_offsets[s] ? d++ : -1;
    }
    auto dens_of = [&](int64_t s) -> const void * { return slot[s] < 0 ? nullptr : D + slot[s] * dslot * es; };
    void *lp[2] = {lam_pos0, lam_pos1}, *ln[2] = {lam_neg0, lam_neg1};
    int cur = 0;  // lambda_{n_steps} = 0 in buffer 0
    const int64_t n_seg = (n_steps + ckpt_every - 1) / ckpt_every;
    if ((rc = adjoint_accumulate_begin(g, adj_workspace, st))) return rc;
    for (int64_t c = n_seg - 1; c >= 0; --c) {
        const int64_t s0 = c * ckpt_every, s1 = (s0 + ckpt_every < n_steps) ? s0 + ckpt_every : n_steps;
        const int64_t L = s1 - s0;
        cudaError_t e = cudaMemcpyAsync(SP, static_cast<const char *>(ckpt_pos) + c * state_stride * es,
                                        (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(SN, static_cast<const char *>(ckpt_neg) + c * state_stride * es, (size_t)(field * es),
                                cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return set_cuda_error("cudaMemcpyAsync(checkpoint)", e);
        // recompute states s0 .. s1-1 of the segment (state j at slot j - s0)
        for (int64_t j = 0; j + 1 < L; ++j) {
            rc = launch_step(g, SP + j * state_stride * es, SN + j * state_stride * es, SP + (j + 1) * state_stride * es,
                             SN + (j + 1) * state_stride * es, dens_of(s0 + j), nullptr, nullptr, workspace, st);
            if (rc) return rc;
        }
        // adjoint steps s1-1 .. s0
        for (int64_t j = L - 1; j >= 0; --j) {
            rc = launch_adjoint(g, SP + j * state_stride * es, SN + j * state_stride * es, dens_of(s0 + j), lp[cur],
                                ln[cur], lp[cur ^ 1], ln[cur ^ 1], nullptr, adj_workspace, st, true);
            if (rc) return rc;
            cur ^= 1;
        }
    }
    return adjoint_accumulate_end(g, adj_workspace, grad, st);
}

int pic_selftest_waits(int32_t *barrier_status, int32_t *mbarrier_status, uintptr_t stream) {
    if (!barrier_status || !mbarrier_status) return set_error(PIC_E_INVALID, "null pointer argument");
    return selftest_waits(barrier_status, mbarrier_status, reinterpret_cast<cudaStream_t>(stream));
}

int pic_revolve_plan(int64_t n_steps, int64_t n_slots, int64_t *recompute_steps, int64_t *spine_levels) {
    return revolve_plan(n_steps, n_slots, recompute_steps, spine_levels);
}

int pic_revolve_spine(int64_t n_steps, int64_t n_slots, int64_t *steps, int64_t cap, int64_t *n_levels) {
    if (!n_levels || (cap > 0 && !steps)) return set_error(PIC_E_INVALID, "null pointer argument");
    return revolve_spine(n_steps, n_slots, steps, cap, n_levels);
}

int pic_revolve_trace(int64_t n_steps, int64_t n_slots, int64_t *events, int64_t cap, int64_t *n_events,
                      int64_t *advanced) {
    if (!n_events || !advanced || (cap > 0 && !events)) return set_error(PIC_E_INVALID, "null pointer argument");
    return revolve_trace(n_steps, n_slots, events, cap, n_events, advanced);
}

// Checks shared by the two revolve passes: slots, stride, offsets, scratch.
static int check_revolve(const pic_grid *g, const void *slots_pos, const void *slots_neg, int64_t state_stride,
                         int64_t n_slots, int64_t n_steps, const double *xs, const double *ys,
                         const int64_t *track_offsets, const void *dens) {
    int rc = check_grid(g);
    if (rc) return rc;
    if ((rc = check_fields(slots_pos, slots_neg, slots_pos, slots_neg))) return rc;
    if (n_steps < 0 || n_slots < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and n_slots >= 1");
    if (!track_offsets) return set_error(PIC_E_INVALID, "track_offsets is null");
    const int64_t field = g->no_xy * g->no_xy * g->kpitch;
    if (state_stride < field || state_stride % 8 != 0)
        return set_error(PIC_E_INVALID, "state_stride must be >= no_xy^2 * kpitch and a multiple of 8 elements");
    int64_t n_dep = 0;
    if ((rc = kept_slots(track_offsets, n_steps, &n_dep))) return rc;
    if (n_dep > 0 && (!xs || !ys || !dens)) return set_error(PIC_E_INVALID, "track or deposition arrays are null");
    if (n_dep > 0 && !aligned(dens, 16)) return set_error(PIC_E_INVALID, "the deposition scratch must be 16-byte aligned");
    return revolve_plan(n_steps, n_slots, nullptr, nullptr);
}

int pic_revolve_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                        const double *xs, const double *ys, const int64_t *track_offsets, void *dens,
                        uint32_t *counts, double *tally, void *slots_pos, void *slots_neg, int64_t state_stride,
                        int64_t n_slots, void *workspace, int64_t workspace_bytes, uintptr_t stream) {
    NvtxRange nvtx_range("pic_revolve_forward");
    int rc = check_revolve(g, slots_pos, slots_neg, state_stride, n_slots, n_steps, xs, ys, track_offsets, dens);
    if (rc) return rc;
    if ((rc = check_fields(pos0, neg0, pos1, neg1))) return rc;
    if (!counts || !tally) return set_error(PIC_E_INVALID, "null pointer argument");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
        return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    return revolve_forward(g, pos0, neg0, pos1, neg1, n_steps, xs, ys, track_offsets, dens, counts, tally, slots_pos,
                           slots_neg, state_stride, n_slots, workspace, workspace_bytes,
                           reinterpret_cast<cudaStream_t>(stream));
}

int pic_revolve_backward(const pic_grid *g, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots,
                         int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                         void *dens, void *work_pos0, void *work_neg0, void *work_pos1, void *work_neg1,
                         void *lam_pos0, void *lam_neg0, void *lam_pos1, void *lam_neg1, double *grad,
                         void *workspace, int64_t workspace_bytes, void *adj_workspace, int64_t adj_workspace_bytes,
                         uintptr_t stream) {
    NvtxRange nvtx_range("pic_revolve_backward");
    int rc = check_revolve(g, slots_pos, slots_neg, state_stride, n_slots, n_steps, xs, ys, track_offsets, dens);
    if (rc) return rc;
    if ((rc = check_fields(work_pos0, work_neg0, work_pos1, work_neg1)) ||
        (rc = check_fields(lam_pos0, lam_neg0, lam_pos1, lam_neg1)))
        return rc;
    if (!grad) return set_error(PIC_E_INVALID, "grad is null");
    if (!workspace || workspace_bytes < kWorkspaceBytes)
        return set_error(PIC_E_INVALID, "workspace too small (pic_step_workspace_bytes)");
    int64_t need = 0;
    adjoint_workspace_bytes(&need);
    if (!adj_workspace || adj_workspace_bytes < need)
        return set_error(PIC_E_INVALID, "adjoint workspace too small (pic_adjoint_workspace_bytes)");
    return revolve_backward(g, slots_pos, slots_neg, state_stride, n_slots, n_steps, xs, ys, track_offsets, dens,
                            work_pos0, work_neg0, work_pos1, work_neg1, lam_pos0, lam_neg0, lam_pos1, lam_neg1, grad,
                            workspace, workspace_bytes, adj_workspace, reinterpret_cast<cudaStream_t>(stream));
}

int pic_run_segment(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                    int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                    void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                    void *workspace, int64_t workspace_bytes, uintptr_t stream) {
    NvtxRange nvtx_range("pic_run_segment");
    int rc = check_segment(g, pos0, neg0, pos1, neg1, n_steps, xs, ys, track_offsets, dens0, dens1, counts, tally,
                           workspace, workspace_bytes);
    if (rc) return rc;
    return run_loop(g, pos0, neg0, pos1, neg1, parity, n_steps, xs, ys, track_offsets, dens0, dens1, dens_parity,
                    counts, tally, workspace, workspace_bytes, reinterpret_cast<cudaStream_t>(stream));
}

int pic_graph_create(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                     int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                     void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                     void *workspace, int64_t workspace_bytes, uintptr_t stream, uintptr_t *graph_out) {
    NvtxRange nvtx_range("pic_graph_create");
    if (!graph_out) return set_error(PIC_E_INVALID, "graph_out is null");
    *graph_out = 0;
    int rc = check_segment(g, pos0, neg0, pos1, neg1, n_steps, xs, ys, track_offsets, dens0, dens1, counts, tally,
                           workspace, workspace_bytes);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaStream_t own = nullptr;
    if (st == nullptr) {
        cudaError_t e = cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
        if (e != cudaSuccess) return set_cuda_error("cudaStreamCreateWithFlags", e);
        st = own;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        if (own) cudaStreamDestroy(own);
        return set_cuda_error("cudaStreamBeginCapture", e);
    }
    t_captured = 0;
    rc = run_loop(g, pos0, neg0, pos1, neg1, parity, n_steps, xs, ys, track_offsets, dens0, dens1, dens_parity,
                  counts, tally, workspace, workspace_bytes, st);
    const int64_t captured = t_captured;
    t_captured = -1;
    e = cudaStreamEndCapture(st, &graph);
    if (own) cudaStreamDestroy(own);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return set_cuda_error("cudaStreamEndCapture", e);
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return set_cuda_error("cudaGraphInstantiate", e);
    *graph_out = reinterpret_cast<uintptr_t>(exec);
    graph_launches_set(*graph_out, captured);
    return PIC_OK;
}

int pic_capture_begin(uintptr_t stream) {
    NvtxRange nvtx_range("pic_capture_begin");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    if (st == nullptr || st == cudaStreamLegacy || st == cudaStreamPerThread)
        return set_error(PIC_E_INVALID, "capture needs a stream created by the caller (not the default stream)");
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return set_cuda_error("cudaStreamBeginCapture", e);
    t_captured = 0;
    return PIC_OK;
}

int pic_capture_end(uintptr_t stream, uintptr_t *graph_out) {
    NvtxRange nvtx_range("pic_capture_end");
    if (!graph_out) return set_error(PIC_E_INVALID, "graph_out is null");
    *graph_out = 0;
    cudaGraph_t graph = nullptr;
    const int64_t captured = t_captured < 0 ? 0 : t_captured;
    t_captured = -1;
    cudaError_t e = cudaStreamEndCapture(reinterpret_cast<cudaStream_t>(stream), &graph);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return set_cuda_error("cudaStreamEndCapture", e);
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return set_cuda_error("cudaGraphInstantiate", e);
    *graph_out = reinterpret_cast<uintptr_t>(exec);
    graph_launches_set(*graph_out, captured);
    return PIC_OK;
}

int pic_batched_workspace_bytes(int32_t n_blocks, int32_t n_cfgs, int64_t *bytes) {
    if (!bytes) return set_error(PIC_E_INVALID, "bytes is null");
    return batched_workspace_bytes(n_blocks, n_cfgs, bytes);
}

int pic_batched_deposit_bytes(int32_t n_cfgs, int32_t total_tiles, int64_t max_tracks, int64_t dens_bytes,
                              int32_t dtype, int64_t *bytes) {
    if (!bytes) return set_error(PIC_E_INVALID, "bytes is null");
    if (n_cfgs < 1 || n_cfgs > kBinMaxSlots) return set_error(PIC_E_INVALID, "n_cfgs must be 1 .. 1024");
    if (total_tiles < 1 || max_tracks < 0 || dens_bytes < 1)
        return set_error(PIC_E_INVALID, "total_tiles >= 1, max_tracks >= 0 and dens_bytes >= 1");
    if (dtype != PIC_F32 && dtype != PIC_F64) return set_error(PIC_E_INVALID, "dtype must be PIC_F32 or PIC_F64");
    *bytes = batched_deposit_bytes(n_cfgs, total_tiles, max_tracks, dens_bytes, dtype);
    return PIC_OK;
}

int pic_batched_segment(const pic_batch_launch *launch, uintptr_t stream) {
    NvtxRange nvtx_range("pic_batched_segment");
    int rc = check_batch(launch);
    if (rc) return rc;
    return batched_loop(*launch, reinterpret_cast<cudaStream_t>(stream));
}

int pic_batched_persistent(const pic_batch_launch *launch, const int64_t *step_task_off_dev,
                           const int64_t *step_tracks_dev, uintptr_t stream) {
    NvtxRange nvtx_range("pic_batched_persistent");
    int rc = check_batch(launch);  // validates the host copies of the step tables
    if (rc) return rc;
    if (!step_task_off_dev || !step_tracks_dev) return set_error(PIC_E_INVALID, "device step tables are null");
    if (launch->n_steps == 0) return PIC_OK;
    return batched_persistent(*launch, step_task_off_dev, step_tracks_dev, reinterpret_cast<cudaStream_t>(stream));
}

int pic_batched_status(const pic_batch_launch *launch, uintptr_t stream, int32_t *status) {
    if (!launch || !launch->workspace || !status) return set_error(PIC_E_INVALID, "null pointer argument");
    return batched_status(*launch, reinterpret_cast<cudaStream_t>(stream), status);
}

int pic_batched_stream_workspace_bytes(int32_t n_cfgs, int32_t n_items, int32_t consumer_warps, int64_t *bytes) {
    if (!bytes) return set_error(PIC_E_INVALID, "bytes is null");
    return batched_stream_workspace_bytes(n_cfgs, n_items, consumer_warps, bytes);
}

int pic_batched_stream_prepare(const pic_batch_cfg *cfgs_host, int32_t n_cfgs, const int32_t *items_host,
                               int32_t n_items, const int32_t *tile_rows_host, int32_t consumer_warps,
                               void *workspace, int64_t workspace_bytes, uintptr_t stream, pic_batch_stream *out) {
    NvtxRange nvtx_range("pic_batched_stream_prepare");
    return batched_stream_prepare(cfgs_host, n_cfgs, items_host, n_items, tile_rows_host, consumer_warps, workspace,
                                  workspace_bytes, reinterpret_cast<cudaStream_t>(stream), out);
}

int pic_batched_stream_segment(const pic_batch_launch *launch, const pic_batch_stream *bs, uintptr_t stream) {
    NvtxRange nvtx_range("pic_batched_stream_segment");
    int rc = check_batch_common(launch);
    if (rc) return rc;
    if (!bs || !bs->workspace) return set_error(PIC_E_INVALID, "prepared stream tables are null");
    if (launch->dtype != PIC_F32) return set_error(PIC_E_INVALID, "the batched streaming step takes float32 batches");
    if (bs->n_cfgs != launch->n_cfgs) return set_error(PIC_E_INVALID, "prepared tables are for another batch");
    if (bs->n_items < 1 || bs->consumer_warps < 1 || bs->consumer_warps > 15 || bs->stages < 4 ||
        bs->ipt < 1 || bs->ipt > 3 || bs->stage_floats < 1)
        return set_error(PIC_E_INVALID, "pic_batch_stream was not filled by pic_batched_stream_prepare");
    return batched_loop_stream(*launch, bs, reinterpret_cast<cudaStream_t>(stream));
}

int pic_batched_stream_status(const pic_batch_stream *bs, int32_t reset, uintptr_t stream, int32_t *status) {
    if (!bs || !bs->workspace || !status) return set_error(PIC_E_INVALID, "null pointer argument");
    return batched_stream_status(*bs, reset, reinterpret_cast<cudaStream_t>(stream), status);
}

int pic_batched_graph_create(const pic_batch_launch *launch, uintptr_t stream, uintptr_t *graph_out) {
    NvtxRange nvtx_range("pic_batched_graph_create");
    if (!graph_out) return set_error(PIC_E_INVALID, "graph_out is null");
    *graph_out = 0;
    int rc = check_batch(launch);
    if (rc) return rc;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaStream_t own = nullptr;
    if (st == nullptr) {
        cudaError_t e = cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking);
        if (e != cudaSuccess) return set_cuda_error("cudaStreamCreateWithFlags", e);
        st = own;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        if (own) cudaStreamDestroy(own);
        return set_cuda_error("cudaStreamBeginCapture", e);
    }
    rc = batched_loop(*launch, st);
    e = cudaStreamEndCapture(st, &graph);
    if (own) cudaStreamDestroy(own);
    if (rc) {
        if (graph) cudaGraphDestroy(graph);
        return rc;
    }
    if (e != cudaSuccess) return set_cuda_error("cudaStreamEndCapture", e);
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return set_cuda_error("cudaGraphInstantiate", e);
    *graph_out = reinterpret_cast<uintptr_t>(exec);
    return PIC_OK;
}

int pic_graph_launch(uintptr_t graph, uintptr_t stream) {
    NvtxRange nvtx_range("pic_graph_launch");
    if (!graph) return set_error(PIC_E_INVALID, "graph handle is null");
    cudaError_t e = cudaGraphLaunch(reinterpret_cast<cudaGraphExec_t>(graph), reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return set_cuda_error("cudaGraphLaunch", e);
    int64_t n = 0;
    {
        std::lock_guard<std::mutex> lock(g_graph_mu);
        auto it = g_graph_launches.find(graph);
        if (it != g_graph_launches.end()) n = it->second;
    }
    count_launches(n);
    return PIC_OK;
}

int64_t pic_kernel_launches(void) { return g_launches.load(); }

int pic_graph_destroy(uintptr_t graph) {
    if (!graph) return PIC_OK;
    {
        std::lock_guard<std::mutex> lock(g_graph_mu);
        g_graph_launches.erase(graph);
    }
    cudaError_t e = cudaGraphExecDestroy(reinterpret_cast<cudaGraphExec_t>(graph));
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaGraphExecDestroy", e);
}

}  // extern "C"
