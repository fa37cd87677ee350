// stream.cu -- the fused time step as a 2.5D streaming kernel for large
// float32 grids: bulk asynchronous copies (cp.async.bulk + mbarrier) stage
// whole (j-tile x k-row) planes into a shared-memory ring while consumer
// warps march along i.
//
// Work item: a tile of TJ interior rows j = [cj_lo, cj_hi) with every k, over
// LI interior planes i = [ci_lo, ci_hi). Because k is the contiguous axis and
// the tile spans whole k-rows, the rows cj_lo-1 .. cj_hi of one plane (tile
// plus its two j-halo rows) are ONE contiguous block of memory per species,
// copied by one bulk copy. The producer warp streams the planes
// ci_lo-1 .. ci_hi of the item into an S-stage ring; consumers compute plane
// ci from the stages of ci-1, ci, ci+1, so every stencil neighbour is read
// from shared memory and each field value crosses HBM once per step (plus the
// j-halo rows, which the neighbouring tile reads at the same time, from L2).
//
// The arithmetic, the deposition-on-read, the wall handling and the tallies
// are those of step_kernel in step.cu (the reference's
// _lax_wendroff_step_numba, solver_numba.py:130-213, with the broadcast of
// solver_numba_parallel.py:222-277 fused in and state.py:113-176 for the
// ring). Ring columns are written by the interior column next to them:
// reflecting copies the new interior value (corners take the diagonal
// interior column), absorbing carries the ring's own input plus this step's
// deposition.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_async.cuh"
#include "pic_device.cuh"
#include "pic_internal.h"
#include "pic_stream.cuh"

namespace pic {

__device__ __forceinline__ void item_geometry(const StreamArgs &a, int w, int &cj_lo, int &cj_hi, int &ci_lo,
                                              int &ci_hi) {
    const int u = w / a.jt, t = w - u * a.jt;
    cj_lo = 1 + t * a.tj;
    cj_hi = min(cj_lo + a.tj, a.n - 1);
    ci_lo = 1 + u * a.li;
    ci_hi = min(ci_lo + a.li, a.n - 1);
}

// Runtime-block-size version of finish_tally (pic_device.cuh).
__device__ void finish_tally_rt(double (&v)[4], double *partials, unsigned int *counter, double *tally,
                                double injected_scale) {
    __shared__ double red[32][4];
    __shared__ bool last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    auto bsum = [&](double (&x)[4]) {
#pragma unroll
        for (int q = 0; q < 4; ++q) x[q] = warp_sum(x[q]);
        if (lane == 0)
#pragma unroll
            for (int q = 0; q < 4; ++q) red[warp][q] = x[q];
        __syncthreads();
        if (warp == 0)
#pragma unroll
            for (int q = 0; q < 4; ++q) x[q] = warp_sum(lane < nw ? red[lane][q] : 0.0);
        __syncthreads();
    };
    bsum(v);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) partials[4 * (int64_t)blockIdx.x + q] = v[q];
        __threadfence();
        last = (atomicAdd(counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[q] += __ldcg(partials + 4 * (int64_t)b + q);
    bsum(acc);
    if (threadIdx.x == 0) {
        tally[0] = acc[0] * injected_scale;
        tally[1] = acc[1];
        tally[2] = acc[2];
        tally[3] = acc[3];
        *counter = 0u;
        __threadfence();
    }
}

template <int IPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) stream_step_kernel(StreamArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ volatile int abort_flag;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + a.stages;
    const int bar_bytes = (2 * a.stages * 8 + 127) / 128 * 128;
    float *stage0 = reinterpret_cast<float *>(smem_raw + bar_bytes);
    const int stage_floats = stream_stage_floats(a.tj, a.kp);
    const int S = a.stages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = a.consumer_warps;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            // full: the producer's expect-tx arrival; the bulk copies' bytes
            // complete it.
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], cw);
        }
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();

    Tally<float> t_rec, t_p, t_n, t_inj;

    if (warp == cw) {
        // ---------------- producer warp: lane 0 issues every copy ----------------
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < a.n_items && ok; w += gridDim.x) {
                int cj_lo, cj_hi, ci_lo, ci_hi;
                item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
                for (int pl = ci_lo - 1; pl <= ci_hi; ++pl, ++g) {
                    const int slot = (int)(g % S);
                    if (g >= S && !mbar_wait(&empty[slot], (uint32_t)(((g / S) - 1) & 1), a.status, 1)) {
                        abort_flag = 1;
                        ok = false;
                        break;
                    }
                    if (abort_flag) {
                        ok = false;
                        break;
                    }
                    stream_issue_plane(a, pl, cj_lo, cj_hi, stage0 + (size_t)slot * stage_floats, &full[slot]);
                }
            }
            if (!ok) {
                // drain: every copy still in flight must land before exit
                for (long long gg = g - S < 0 ? 0 : g - S; gg < g; ++gg)
                    mbar_wait(&full[gg % S], (uint32_t)((gg / S) & 1), a.status, 2);
            }
        }
    } else {
        // ---------------- consumers ----------------
        const StreamConsts K = stream_consts(a);
        long long g = 0;
        for (int w = blockIdx.x; w < a.n_items; w += gridDim.x) {
            int cj_lo, cj_hi, ci_lo, ci_hi;
            item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
            if (!stream_consume_item<IPT>(a, K, cj_lo, cj_hi, ci_lo, ci_hi, stage0, stage_floats, full, empty, S, g,
                                          abort_flag, threadIdx.x, cw * 32, t_rec, t_p, t_n, t_inj))
                break;
        }
    }
    if (!a.tally) return;  // no tallies wanted (a recomputation): no reduction
    double v[4] = {t_inj.value(), t_rec.value(), t_p.value(), t_n.value()};
    finish_tally_rt(v, a.partials, a.counter, a.tally, a.injected_scale);
}

template <int IPT, int MAXT = stream_max_threads(IPT)>
static int launch_ipt(const StreamArgs &a, unsigned blocks, int threads, int smem, cudaStream_t st) {
    static int configured = 0;  // per instantiation: largest dynamic smem set so far
    if (smem > configured) {
        cudaError_t e =
            cudaFuncSetAttribute(stream_step_kernel<IPT, MAXT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(stream_step_kernel)", e);
        configured = smem;
    }
    stream_step_kernel<IPT, MAXT><<<blocks, threads, smem, st>>>(a);
    return check_launch("stream_step_kernel");
}

// The narrowest instantiation of IPT items a thread that takes `threads`.
template <int IPT>
static int launch_fit(const StreamArgs &a, unsigned blocks, int threads, int smem, cudaStream_t st) {
    if (threads <= stream_max_threads(IPT)) return launch_ipt<IPT>(a, blocks, threads, smem, st);
    if constexpr (stream_max_threads(IPT) < kStreamWide1)
        if (threads <= kStreamWide1) return launch_ipt<IPT, kStreamWide1>(a, blocks, threads, smem, st);
    return launch_ipt<IPT, kStreamWide2>(a, blocks, threads, smem, st);
}

int stream_smem_bytes(int tj, int kp, int stages) {
    return (2 * stages * 8 + 127) / 128 * 128 + stages * stream_stage_floats(tj, kp) * 4;
}

int launch_stream_step(const pic_grid *g, const StreamShape &sh, const void *pos_in, const void *neg_in,
                       void *pos_out, void *neg_out, const void *dens, void *dens_zero, double *tally, void *ws,
                       cudaStream_t st) {
    StreamArgs a;
    a.pos_in = (const float *)pos_in;
    a.neg_in = (const float *)neg_in;
    a.pos_out = (float *)pos_out;
    a.neg_out = (float *)neg_out;
    a.dens = (const float2 *)dens;
    a.dens_zero = (float2 *)dens_zero;
    a.tally = tally;
    Workspace w = workspace_layout(ws);
    a.partials = w.partials;
    a.counter = w.counter;
    a.status = w.status;
    a.n = (int)g->no_xy;
    a.kp = (int)g->kpitch;
    a.c4 = a.kp / 4;
    a.nzb = (int)g->nzb;
    a.nze = (int)g->nze;
    a.gap_end = (int)(g->nze + g->no_z);
    a.reflecting = g->wall == PIC_WALL_REFLECTING;
    a.dp = (int)dens_pitch(g->no_xy);
    a.tj = sh.tile_rows;
    a.li = sh.planes_per_item;
    a.jt = (a.n - 2 + a.tj - 1) / a.tj;
    const int ic = (a.n - 2 + a.li - 1) / a.li;
    a.n_items = a.jt * ic;
    a.stages = sh.stages;
    a.consumer_warps = sh.consumer_warps;
    a.p_lat = (float)g->p_lat; a.p_zm = (float)g->p_zm; a.p_zp = (float)g->p_zp;
    a.p_cen = centre_weight<float>(g->p_lat, g->p_zm, g->p_zp, g->p_cen);
    a.n_lat = (float)g->n_lat; a.n_zm = (float)g->n_zm; a.n_zp = (float)g->n_zp;
    a.n_cen = centre_weight<float>(g->n_lat, g->n_zm, g->n_zp, g->n_cen);
    a.alpha_dt = (float)g->alpha_dt;
    a.gfac = (float)g->gaussian_factor;
    ScoreTest sc;
    int rc = score_test(g, &sc);
    if (rc) return rc;
    if (g->no_xy > 16383) return set_error(PIC_E_CAPACITY, "stream variant: no_xy must be <= 16383");
    a.two_mid = (int)sc.two_mid;
    // (2i - two_mid)^2 + (2j - two_mid)^2 < 2^31 for no_xy <= 16383
    a.thr4 = sc.thr4 < 0 ? 0u : (sc.thr4 > 0x7fffffffLL ? 0xffffffffu : (uint32_t)sc.thr4);
    a.injected_scale = (double)g->no_z;  // the pairs carry G already
    const int smem = stream_smem_bytes(a.tj, a.kp, a.stages);
    int64_t blocks = (int64_t)sh.sm_count * sh.ctas_per_sm;
    if (blocks > a.n_items) blocks = a.n_items;
    if (blocks > kMaxStepBlocks) blocks = kMaxStepBlocks;
    const int threads = (a.consumer_warps + 1) * 32;
    const int ipt = (a.tj * a.c4 + a.consumer_warps * 32 - 1) / (a.consumer_warps * 32);
    if (ipt >= 1 && ipt <= kStreamMaxIpt && threads > stream_thread_limit(ipt))
        return set_error(PIC_E_INVALID, "stream variant: too many consumer warps for this tile (registers)");
    switch (ipt) {
        case 1: return launch_ipt<1>(a, (unsigned)blocks, threads, smem, st);
        case 2: return launch_fit<2>(a, (unsigned)blocks, threads, smem, st);
        case 3: return launch_fit<3>(a, (unsigned)blocks, threads, smem, st);
        case 4: return launch_fit<4>(a, (unsigned)blocks, threads, smem, st);
        case 5: return launch_ipt<5>(a, (unsigned)blocks, threads, smem, st);
        case 6: return launch_ipt<6>(a, (unsigned)blocks, threads, smem, st);
        default:
            return set_error(PIC_E_INVALID, "stream variant: tile_rows x k-vectors exceed 6 items per consumer thread");
    }
}

}  // namespace pic
