// noalloc.cu -- pic_step_noalloc: one whole time step (this step's track
// deposition, then the fused step) that allocates no device memory.
//
// Who needs it: callers that can hand the library device pointers but cannot
// allocate device memory themselves -- for example a binding in another
// language that only receives the field and track buffers owned by some
// other runtime and has no CUDA allocator of its own, or a caller working
// under a strict memory budget or inside a loop where cudaMalloc (which may
// synchronise the whole device) is not allowed. pic_step needs two
// caller-allocated scratch buffers (the 2D track density and the tally
// workspace); this entry point keeps both in one file-scope device array
// instead, so the caller passes only inputs (fields, track centres) and
// outputs (next fields, track histogram, tallies).
//
// Limits and behaviour:
//   * the array holds the 2D deposition pairs (rows padded to 4 pairs) of up
//     to kNoAllocDensBytes (16 MiB): no_xy <= 1448 for float32 fields,
//     <= 1024 for float64; larger grids are refused with PIC_E_CAPACITY;
//   * every GPU that loads the library holds the array (16 MiB + the tally
//     workspace) until the process exits;
//   * every call shares the array and it keeps the last call's contents: the
//     pairs are cleared at the start of each call, the tally counter is
//     left at zero by each step (an aborted one included: every block of the
//     step still takes part in the tally reduction);
//   * calls that overlap on the GPU (different streams, or different host
//     threads) race on the array and give wrong results: serialise them;
//   * each call looks up the array's device address (cudaGetSymbolAddress)
//     with the caller's device current, so the address is right again after a
//     cudaDeviceReset; the first call on a device also loads the library's
//     device code there, so make it before any stream capture;
//   * the streaming step waits on its copy ring with bounded waits; if one
//     runs out it records a code in the array's status word and the step's
//     fields are wrong. pic_step_noalloc_status reads that word (and, asked
//     to, clears it together with the tally counter); a caller checks it
//     after a run of steps.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "pic_internal.h"

namespace pic {

constexpr int64_t kNoAllocDensBytes = 16LL << 20;
constexpr int64_t kNoAllocScratchBytes = kNoAllocDensBytes + kWorkspaceBytes;

// Device scratch of pic_step_noalloc: [2D deposition pairs (16 MiB) | tally
// workspace].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array on the current device. Looked up on every call
// (a host-side lookup once the module is loaded) rather than cached, so that
// a device reset, which may load the module at another address, cannot leave
// a stale pointer behind. The host-side symbol is only a stand-in, not a
// device address.
static int noalloc_scratch(void **out) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return set_cuda_error("cudaGetSymbolAddress(g_noalloc_scratch)", e);
    *out = p;
    return PIC_OK;
}

int step_noalloc(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                 const double *xs, const double *ys, int64_t n_tracks, uint32_t *counts, double *tally,
                 cudaStream_t st) {
    const int64_t es = g->dtype == PIC_F64 ? 8 : 4;
    const int64_t dens_bytes = 2 * g->no_xy * dens_pitch(g->no_xy) * es;  // deposition pairs
    if (dens_bytes > kNoAllocDensBytes)
        return set_error(PIC_E_CAPACITY,
                         "pic_step_noalloc: the 2D density of a " + std::to_string(g->no_xy) + " x " +
                             std::to_string(g->no_xy) + " grid (" + std::to_string(dens_bytes) +
                             " bytes) exceeds the static scratch of " + std::to_string(kNoAllocDensBytes) +
                             " bytes; use pic_deposit + pic_step with caller-allocated buffers");
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    unsigned char *dens = static_cast<unsigned char *>(base);
    void *ws = dens + kNoAllocDensBytes;
    if (n_tracks > 0) {
        cudaError_t e = cudaMemsetAsync(dens, 0, (size_t)dens_bytes, st);
        if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(static density)", e);
        rc = launch_deposit(g, xs, ys, n_tracks, dens, counts, st);
        if (rc) return rc;
    }
    return launch_step(g, pos_in, neg_in, pos_out, neg_out, n_tracks > 0 ? dens : nullptr, nullptr, tally, ws, st);
}

// Reads the status word of the array's tally workspace (0 = ok, else the code
// of the bounded wait that ran out), after the stream's work so far; with
// reset, clears it and the completion counter.
int step_noalloc_status(int32_t reset, cudaStream_t st, int32_t *status) {
    void *base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    Workspace w = workspace_layout(static_cast<unsigned char *>(base) + kNoAllocDensBytes);
    int32_t v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, w.status, sizeof(v), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error("pic_step_noalloc_status", e);
    *status = v;
    if (reset) {
        e = cudaMemsetAsync(w.status, 0, sizeof(int32_t), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(w.counter, 0, sizeof(unsigned int), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error("pic_step_noalloc_status reset", e);
    }
    return PIC_OK;
}

}  // namespace pic
