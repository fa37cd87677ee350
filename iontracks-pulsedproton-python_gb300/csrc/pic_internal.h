// pic_internal.h -- host-side declarations shared by the translation units of
// libpic_gb300.so (not part of the public C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/pic_gb300.h"

namespace pic {

// Upper bound on the fused step's grid (blocks); sizes its tally workspace.
constexpr int64_t kMaxStepBlocks = 152 * 32;

struct Workspace {
    double *partials;       // [kMaxStepBlocks][4]
    unsigned int *counter;  // completion counter, zero between steps
};

inline Workspace workspace_layout(void *ws) {
    Workspace w;
    w.partials = reinterpret_cast<double *>(ws);
    w.counter = reinterpret_cast<unsigned int *>(reinterpret_cast<char *>(ws) + kMaxStepBlocks * 4 * sizeof(double));
    return w;
}
constexpr int64_t kWorkspaceBytes = kMaxStepBlocks * 4 * (int64_t)sizeof(double) + 256;

int set_error(int code, const std::string &msg);
int set_cuda_error(const char *what, cudaError_t e);
int check_launch(const char *what);

// Largest useful grid for the step kernel on the current device (SMs x
// resident blocks), cached per device.
int64_t step_grid_cap(int f64);
int step_occupancy(int dtype, int *blocks_per_sm);

int launch_step(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                const void *dens, void *dens_zero, double *tally, void *ws, cudaStream_t st);
int launch_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t m, void *dens,
                   uint32_t *counts, cudaStream_t st);

}  // namespace pic
