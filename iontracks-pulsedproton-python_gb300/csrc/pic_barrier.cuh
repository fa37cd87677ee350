// pic_barrier.cuh -- the device-wide barrier of the persistent kernels
// (cooperative launches: every block is resident).
//
// Arrival is one atomic on a shared count; the last block to arrive resets
// the count and advances the generation, the others poll the generation with
// a short sleep. Every wait is bounded: after kBarrierPolls polls the waiter
// sets the status word, and every block leaves at its next barrier (the host
// then reads the status). Returns false when the kernel must stop.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pic {

constexpr long long kBarrierPolls = 1LL << 24;  // x >= 100 ns: a few seconds
constexpr int kBarrierTimeout = 5;               // status code of an expired wait

struct BarrierRef {
    unsigned int *count;  // blocks arrived at the current barrier (0 between barriers)
    unsigned int *gen;    // barriers completed
    int *status;          // 0, or the code of a wait that gave up
};

__device__ __forceinline__ bool grid_barrier(BarrierRef bar, long long limit = kBarrierPolls) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int *vgen = bar.gen;
        volatile int *vstatus = bar.status;
        const unsigned int g = *vgen;
        __threadfence();  // this block's writes before its arrival
        ok = 1;
        if (atomicAdd(bar.count, 1u) == gridDim.x - 1) {
            atomicExch(bar.count, 0u);
            __threadfence();
            atomicAdd(bar.gen, 1u);
        } else {
            long long polls = 0;
            while (*vgen == g) {
                if (*vstatus != 0) {
                    ok = 0;
                    break;
                }
                if (++polls > limit) {
                    atomicCAS(bar.status, 0, kBarrierTimeout);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();  // the other blocks' writes before this block reads
    }
    __syncthreads();
    return ok != 0;
}

}  // namespace pic
