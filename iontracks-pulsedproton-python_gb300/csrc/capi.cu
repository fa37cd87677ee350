// capi.cu -- the extern "C" entry points of libpic_gb300.so (declared in
// include/pic_gb300.h): argument checks, error reporting, the per-segment
// host loop and its CUDA-graph capture.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <mutex>
#include <string>
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

int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? PIC_OK : set_cuda_error(what, e);
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
    return PIC_OK;
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
                    cudaStream_t st) {
    void *pos[2] = {pos0, pos1}, *neg[2] = {neg0, neg1}, *dens[2] = {dens0, dens1};
    for (int64_t s = 0; s < n_steps; ++s) {
        const int bi = (int)((parity + s) & 1), bo = bi ^ 1;
        const int di = (int)((dens_parity + s) & 1);
        const int64_t m = off[s + 1] - off[s];
        if (m > 0) {
            int rc = launch_deposit(g, xs + off[s], ys + off[s], m, dens[di], counts, st);
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

}  // namespace pic

using namespace pic;

extern "C" {

const char *pic_last_error(void) { return g_last_error.c_str(); }

int pic_abi_version(void) { return 1; }

int64_t pic_kpitch(int64_t nzb) { return (nzb + 7) / 8 * 8; }

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
    *bytes = kWorkspaceBytes;
    return PIC_OK;
}

int pic_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t n_tracks, void *dens,
                uint32_t *counts, uintptr_t stream) {
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

int pic_run_segment(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                    int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                    void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                    void *workspace, int64_t workspace_bytes, uintptr_t stream) {
    int rc = check_segment(g, pos0, neg0, pos1, neg1, n_steps, xs, ys, track_offsets, dens0, dens1, counts, tally,
                           workspace, workspace_bytes);
    if (rc) return rc;
    return run_loop(g, pos0, neg0, pos1, neg1, parity, n_steps, xs, ys, track_offsets, dens0, dens1, dens_parity,
                    counts, tally, workspace, reinterpret_cast<cudaStream_t>(stream));
}

int pic_graph_create(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                     int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                     void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                     void *workspace, int64_t workspace_bytes, uintptr_t stream, uintptr_t *graph_out) {
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
    rc = run_loop(g, pos0, neg0, pos1, neg1, parity, n_steps, xs, ys, track_offsets, dens0, dens1, dens_parity,
                  counts, tally, workspace, st);
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
    if (!graph) return set_error(PIC_E_INVALID, "graph handle is null");
    cudaError_t e = cudaGraphLaunch(reinterpret_cast<cudaGraphExec_t>(graph), reinterpret_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaGraphLaunch", e);
}

int pic_graph_destroy(uintptr_t graph) {
    if (!graph) return PIC_OK;
    cudaError_t e = cudaGraphExecDestroy(reinterpret_cast<cudaGraphExec_t>(graph));
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaGraphExecDestroy", e);
}

}  // extern "C"
