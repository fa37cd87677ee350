// selftest.cu -- the bounded waits of the kernels, run against partners that
// never come, so that a test can check on the GPU that an expired wait
// returns an error status and leaves the context usable (no fault, no hang).
//
// barrier: two blocks; block 1 leaves at once, block 0 waits at the
//   device-wide barrier of the persistent and multi-step kernels
//   (pic_barrier.cuh) with a short poll limit;
// mbarrier: one block initialises an mbarrier that nothing arrives on and
//   waits on its first phase with the streaming kernels' bounded wait
//   (pic_async.cuh), with a short try-wait limit.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_async.cuh"
#include "pic_barrier.cuh"
#include "pic_internal.h"

namespace pic {

namespace {

constexpr long long kSelftestPolls = 1LL << 12;
constexpr int kSelftestMbarCode = 91;

__global__ void selftest_barrier_kernel(unsigned int *count, unsigned int *gen, int *status) {
    if (blockIdx.x == 1) return;  // the partner that never arrives
    grid_barrier(BarrierRef{count, gen, status}, kSelftestPolls);
}

__global__ void selftest_mbarrier_kernel(int *status) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) mbar_wait(&bar, 0u, status, kSelftestMbarCode, kSelftestPolls);
}

}  // namespace

int selftest_waits(int32_t *barrier_status, int32_t *mbarrier_status, cudaStream_t st) {
    // [count, gen, barrier status, mbarrier status]
    int *d = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&d), 4 * sizeof(int), st);
    if (e != cudaSuccess) return set_cuda_error("cudaMallocAsync(selftest)", e);
    int host[4] = {0, 0, 0, 0};
    e = cudaMemsetAsync(d, 0, 4 * sizeof(int), st);
    if (e == cudaSuccess) {
        selftest_barrier_kernel<<<2, 32, 0, st>>>(reinterpret_cast<unsigned int *>(d),
                                                  reinterpret_cast<unsigned int *>(d + 1), d + 2);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        selftest_mbarrier_kernel<<<1, 32, 0, st>>>(d + 3);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(host, d, sizeof(host), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(d, st);
    if (e != cudaSuccess) return set_cuda_error("selftest_waits", e);
    *barrier_status = host[2];
    *mbarrier_status = host[3];
    return PIC_OK;
}

}  // namespace pic
