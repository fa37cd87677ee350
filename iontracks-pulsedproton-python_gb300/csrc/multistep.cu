// multistep.cu -- several time steps of one grid in ONE cooperative launch
// (temporal blocking in time), for grids whose steps are latency-bound.
//
// A small grid (tens of thousands to a few million cells) has its fields in
// L2 and runs a step in a few microseconds of memory work, but a step is two
// launches (deposition, fused step) plus the step's tally reduction: on the
// 53 x 53 x 208 grid of the saturation sweep, 14.5 us a step with CUDA
// graphs. Here one launch runs up to kMaxMultiSteps steps. Per step:
//   the deposition of the step's tracks (deposit.cu's per-track warps,
//     spread over all blocks), then a device-wide barrier (skipped on a step
//     without tracks);
//   the fused step over the flat items (step.cu's flat_item; loads from L2
//     only, since other blocks wrote the fields earlier in this launch), the
//     block's tally partial stored into one of two partial buffers, then a
//     device-wide barrier;
//   block 0 sums the previous step's partials into its tally while the
//     others start this step (the buffers alternate, so no completion counter
//     and no third barrier).
// The arithmetic of every item and every deposition is that of the per-step
// kernels; only the tally partials are summed over a different block count.
// The track offsets of the launch travel in the kernel arguments.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_barrier.cuh"
#include "pic_deposit.cuh"
#include "pic_device.cuh"
#include "pic_flat.cuh"
#include "pic_internal.h"

namespace pic {

namespace {

constexpr int kMultiBlock = 256;

template <typename T> struct MultiRed { using type = double; };
template <> struct MultiRed<float> { using type = DF; };

template <typename T>
struct MultiArgs {
    StepArgs<T> a;  // grid scalars; fields, pairs and tally set per step
    T *pos[2], *neg[2];
    pair_t<T> *dens[2];
    const double *xs, *ys;
    uint32_t *counts;
    double *tally;     // [n_steps][4]
    double *partials;  // [2][gridDim.x][4] 8-byte slots
    BarrierRef bar;
    int n_steps, parity, dens_parity, sms;
    double cut;
    T h2b2, gfac;
    int64_t off[kMaxMultiSteps + 1];  // tracks of step s: [off[s], off[s+1]) of xs/ys
};

__device__ __forceinline__ double red_of(const Tally<double> &t) { return t.value(); }
__device__ __forceinline__ DF red_of(const Tally<float> &t) { return df_of(t); }
__device__ __forceinline__ void red_store(double *slot, double v) { *slot = v; }
__device__ __forceinline__ void red_store(double *slot, DF v) {
    *reinterpret_cast<float2 *>(slot) = make_float2(v.hi, v.lo);
}
__device__ __forceinline__ void red_load_add(double &acc, const double *slot) { acc += __ldcg(slot); }
__device__ __forceinline__ void red_load_add(DF &acc, const double *slot) {
    const float2 p = __ldcg(reinterpret_cast<const float2 *>(slot));
    acc = df_add(acc, DF{p.x, p.y});
}
__device__ __forceinline__ double red_value(double v) { return v; }
__device__ __forceinline__ double red_value(DF v) { return df_value(v); }

// Block 0: step s's tally from the partials of buffer s & 1 (block order).
template <typename T>
__device__ void finish_step(const MultiArgs<T> &p, int s, typename MultiRed<T>::type (*red)[4]) {
    using R = typename MultiRed<T>::type;
    const double *part = p.partials + (int64_t)(s & 1) * gridDim.x * 4;
    R acc[4] = {R{}, R{}, R{}, R{}};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kMultiBlock)
#pragma unroll
        for (int q = 0; q < 4; ++q) red_load_add(acc[q], part + 4 * (int64_t)b + q);
    block_sum4<kMultiBlock>(acc, red);
    if (threadIdx.x == 0) {
        double *t = p.tally + 4 * (int64_t)s;
        t[0] = red_value(acc[0]) * p.a.injected_scale;
        t[1] = red_value(acc[1]);
        t[2] = red_value(acc[2]);
        t[3] = red_value(acc[3]);
    }
}

template <typename T, typename I>
__global__ void __launch_bounds__(kMultiBlock) multistep_kernel(MultiArgs<T> p) {
    using R = typename MultiRed<T>::type;
    constexpr int WARPS = kMultiBlock / 32;
    __shared__ R red[kMultiBlock / 32][4];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const I items = (I)p.a.items, stride = (I)gridDim.x * kMultiBlock;
    for (int s = 0; s < p.n_steps; ++s) {
        const int bi = (p.parity + s) & 1, bo = bi ^ 1;
        const int di = (p.dens_parity + s) & 1;
        const int64_t o0 = p.off[s], m = p.off[s + 1] - o0;
        if (s > 0 && blockIdx.x == 0) finish_step<T>(p, s - 1, red);
        if (m > 0) {
            const int parts = deposit_parts(m, p.sms);
            for (int64_t w = (int64_t)blockIdx.x * WARPS + warp; w < m * parts; w += (int64_t)gridDim.x * WARPS)
                deposit_track<T>(p.xs[o0 + w / parts], p.ys[o0 + w / parts], p.a.n, p.a.dp, p.cut, p.h2b2, p.gfac,
                                 p.dens[di], p.counts, lane, (int)(w % parts), parts);
            if (!grid_barrier(p.bar)) return;
        }
        StepArgs<T> a = p.a;
        a.pos_in = p.pos[bi];
        a.neg_in = p.neg[bi];
        a.pos_out = p.pos[bo];
        a.neg_out = p.neg[bo];
        a.dens = m > 0 ? p.dens[di] : nullptr;
        // the buffer step s+1 deposits into was last written at step s-1
        const bool zero_next = (s == 0) || (p.off[s] > p.off[s - 1]);
        a.dens_zero = zero_next ? p.dens[di ^ 1] : nullptr;
        Tally<T> t_rec, t_p, t_n, t_inj;
        for (I item = (I)blockIdx.x * kMultiBlock + threadIdx.x; item < items; item += stride)
            flat_item<T, I, true>(a, item, t_rec, t_p, t_n, t_inj);
        R v[4] = {red_of(t_inj), red_of(t_rec), red_of(t_p), red_of(t_n)};
        block_sum4<kMultiBlock>(v, red);
        if (threadIdx.x == 0) {
            double *part = p.partials + ((int64_t)(s & 1) * gridDim.x + blockIdx.x) * 4;
#pragma unroll
            for (int q = 0; q < 4; ++q) red_store(part + q, v[q]);
        }
        if (!grid_barrier(p.bar)) return;
    }
    if (p.n_steps > 0 && blockIdx.x == 0) finish_step<T>(p, p.n_steps - 1, red);
}

template <typename T, typename I>
int launch_t(const pic_grid *g, void *const pos[2], void *const neg[2], int parity, int n_steps, const double *xs,
             const double *ys, const int64_t *off, void *const dens[2], int dens_parity, uint32_t *counts,
             double *tally, void *ws, cudaStream_t st) {
    static int per_sm = 0;  // resident blocks per SM of this instantiation
    if (per_sm == 0) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, multistep_kernel<T, I>, kMultiBlock, 0);
        if (e != cudaSuccess || per_sm < 1) {
            per_sm = 0;
            return set_cuda_error("cudaOccupancyMaxActiveBlocksPerMultiprocessor(multistep_kernel)", e);
        }
    }
    MultiArgs<T> p;
    StepArgs<T> &a = p.a;
    a.pos_in = a.neg_in = nullptr;
    a.pos_out = a.neg_out = nullptr;
    a.dens = nullptr;
    a.dens_zero = nullptr;
    a.tally = nullptr;
    a.partials = nullptr;
    a.counter = nullptr;
    a.n = g->no_xy;
    a.kp = g->kpitch;
    a.c4 = g->kpitch / 4;
    a.items = g->no_xy * g->no_xy * a.c4;
    a.dp = dens_pitch(g->no_xy);
    a.nzb = (int)g->nzb;
    a.nze = (int)g->nze;
    a.gap_end = (int)(g->nze + g->no_z);
    a.reflecting = g->wall == PIC_WALL_REFLECTING;
    a.p_lat = (T)g->p_lat; a.p_zm = (T)g->p_zm; a.p_zp = (T)g->p_zp;
    a.p_cen = centre_weight<T>(g->p_lat, g->p_zm, g->p_zp, g->p_cen);
    a.n_lat = (T)g->n_lat; a.n_zm = (T)g->n_zm; a.n_zp = (T)g->n_zp;
    a.n_cen = centre_weight<T>(g->n_lat, g->n_zm, g->n_zp, g->n_cen);
    a.alpha_dt = (T)g->alpha_dt;
    a.gfac = (T)g->gaussian_factor;
    int rc = score_test(g, &a.score);
    if (rc) return rc;
    a.injected_scale = (double)g->no_z;
    a.div_c4 = make_fastdiv(a.c4);
    a.div_n = make_fastdiv(a.n);
    for (int q = 0; q < 2; ++q) {
        p.pos[q] = (T *)pos[q];
        p.neg[q] = (T *)neg[q];
        p.dens[q] = (pair_t<T> *)dens[q];
    }
    p.xs = xs;
    p.ys = ys;
    p.counts = counts;
    p.tally = tally;
    Workspace w = workspace_layout(ws);
    p.partials = w.partials;
    // the barrier's count and generation sit in the workspace's tail, beside
    // the step counter (which stays 0) and the status word
    p.bar = BarrierRef{w.counter + 16, w.counter + 17, w.status};
    p.n_steps = n_steps;
    p.parity = parity;
    p.dens_parity = dens_parity;
    p.sms = sm_count();
    p.cut = g->cutoff_voxels;
    p.h2b2 = (T)g->h2_over_b2;
    p.gfac = (T)g->gaussian_factor;
    for (int s = 0; s <= n_steps; ++s) p.off[s] = off[s];
    // one item a thread where the blocks can all be resident (each item waits
    // on its L2 loads: items a thread walks one after another add up), never
    // more than can be resident (a cooperative launch), nor than the partial
    // buffers hold
    int64_t blocks = (a.items + kMultiBlock - 1) / kMultiBlock;
    const int64_t resident = (int64_t)per_sm * p.sms;
    if (blocks > resident) blocks = resident;
    if (blocks > kMaxStepBlocks / 2) blocks = kMaxStepBlocks / 2;
    if (blocks < 1) blocks = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(kMultiBlock);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = cudaLaunchKernelEx(&cfg, multistep_kernel<T, I>, p);
    if (e != cudaSuccess) return set_cuda_error("cudaLaunchKernelEx(multistep_kernel)", e);
    count_launches(1);
    return PIC_OK;
}

}  // namespace

bool multistep_eligible(const pic_grid *resolved) {
    return resolved->variant == PIC_VARIANT_FLAT && resolved->steps_per_launch > 1;
}

int launch_multistep(const pic_grid *g, void *const pos[2], void *const neg[2], int parity, int n_steps,
                     const double *xs, const double *ys, const int64_t *off, void *const dens[2], int dens_parity,
                     uint32_t *counts, double *tally, void *ws, cudaStream_t st) {
    if (n_steps < 1 || n_steps > kMaxMultiSteps)
        return set_error(PIC_E_INVALID, "multistep launch: 1 .. kMaxMultiSteps steps");
    const bool i32 = flat_index32(g->no_xy, g->kpitch);
    if (g->dtype == PIC_F64)
        return i32 ? launch_t<double, uint32_t>(g, pos, neg, parity, n_steps, xs, ys, off, dens, dens_parity, counts,
                                                tally, ws, st)
                   : launch_t<double, int64_t>(g, pos, neg, parity, n_steps, xs, ys, off, dens, dens_parity, counts,
                                               tally, ws, st);
    return i32 ? launch_t<float, uint32_t>(g, pos, neg, parity, n_steps, xs, ys, off, dens, dens_parity, counts, tally,
                                           ws, st)
               : launch_t<float, int64_t>(g, pos, neg, parity, n_steps, xs, ys, off, dens, dens_parity, counts, tally,
                                          ws, st);
}

}  // namespace pic
