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
//     left at zero by each completed step;
//   * calls that overlap on the GPU (different streams, or different host
//     threads) race on the array and give wrong results: serialise them;
//   * the first call on a device looks up the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture.
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <string>

#include "pic_internal.h"

namespace pic {

constexpr int64_t kNoAllocDensBytes = 16LL << 20;
constexpr int64_t kNoAllocScratchBytes = kNoAllocDensBytes + kWorkspaceBytes;

// Device scratch of pic_step_noalloc: [2D deposition pairs (16 MiB) | tally
// workspace].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array, looked up once per device with that device
// current (the host-side symbol is only a stand-in, not a device address).
static int noalloc_scratch(void **out) {
    static std::mutex mu;
    static void *addr[64] = {nullptr};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_cuda_error("cudaGetDevice", e);
    if (dev < 0 || dev >= 64) return set_error(PIC_E_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return set_cuda_error("cudaGetSymbolAddress(g_noalloc_scratch)", e);
        addr[dev] = p;
    }
    *out = addr[dev];
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

}  // namespace pic
