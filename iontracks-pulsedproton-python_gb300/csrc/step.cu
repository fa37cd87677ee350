// step.cu -- the fused time step (deposition broadcast + Lax-Wendroff sweep +
// recombination sink + lateral wall + scored tallies) for one grid.
//
// One work item is four consecutive k of one (i, j) column: a 128-bit load or
// store per species for FP32 fields. Every column of the output is written:
//   interior (1 <= i, j <= no_xy-2): the 7-point Lax-Wendroff update,
//     z-weights swapped for the negative species, minus alpha*dt*n+*n-;
//   outer ring, absorbing wall: the ring is carried with this step's
//     deposition added (the reference's deposit-then-carry, state.py:157-176);
//   outer ring, reflecting wall: the new value of the nearest interior column
//     (the reference's i-planes-then-j-planes mirror, state.py:151-154, which
//     maps corners to the diagonal interior column).
// The step's deposition is added to every value as it is read (gap layers
// only), the fused form of the reference's separate broadcast pass
// (solver_numba_parallel.py:222-277): each column reads one pair, its own
// G * density (added to its values) and the sum over its four lateral
// neighbours (added to the stencil's lateral sum). The z end planes
// k = 0 and k >= nzb-1 (and the row padding) are written as zero.
//
// Tallies over the scored set (interior, inside scoring_radius_sq, gap
// layers) follow _lax_wendroff_step_numba (solver_numba.py:204-211):
// recombined uses the pre-step densities, n+/n- the updated ones. The
// injected charge of the step is sum(G * density) over scored columns times
// no_z (solver_numba_parallel.py:271-276).
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_device.cuh"
#include "pic_flat.cuh"
#include "pic_internal.h"

namespace pic {

template <typename T, int BLOCK, typename I>
__global__ void __launch_bounds__(BLOCK) step_kernel(StepArgs<T> a) {
    Tally<T> t_rec, t_p, t_n, t_inj;
    const I stride = (I)gridDim.x * BLOCK, items = (I)a.items;
    for (I item = (I)blockIdx.x * BLOCK + threadIdx.x; item < items; item += stride)
        flat_item<T, I>(a, item, t_rec, t_p, t_n, t_inj);
    if (!a.tally) return;  // no tallies wanted (a recomputation): no reduction
    if constexpr (sizeof(T) == 4) {
        DF v[4] = {df_of(t_inj), df_of(t_rec), df_of(t_p), df_of(t_n)};
        finish_tally_df<BLOCK>(v, a.partials, a.counter, a.tally, a.injected_scale);
    } else {
        double v[4] = {t_inj.value(), t_rec.value(), t_p.value(), t_n.value()};
        finish_tally<BLOCK>(v, a.partials, a.counter, a.tally, a.injected_scale);
    }
}

template <typename T>
static int launch_step_t(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                         const void *dens, void *dens_zero, double *tally, void *ws, cudaStream_t st) {
    constexpr int BLOCK = 256;
    StepArgs<T> a;
    a.pos_in = (const T *)pos_in;
    a.neg_in = (const T *)neg_in;
    a.pos_out = (T *)pos_out;
    a.neg_out = (T *)neg_out;
    a.dens = (const pair_t<T> *)dens;
    a.dens_zero = (pair_t<T> *)dens_zero;
    a.tally = tally;
    Workspace w = workspace_layout(ws);
    a.partials = w.partials;
    a.counter = w.counter;
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
    int64_t blocks = (a.items + BLOCK - 1) / BLOCK;
    const int64_t cap = step_grid_cap(g->dtype == PIC_F64 ? 1 : 0);
    if (blocks > cap) blocks = cap;
    if (blocks > kMaxStepBlocks) blocks = kMaxStepBlocks;
    // (items + stride stays below 2^32 on the 32-bit path: items < 2^29)
    if (flat_index32(g->no_xy, g->kpitch))
        step_kernel<T, BLOCK, uint32_t><<<(unsigned)blocks, BLOCK, 0, st>>>(a);
    else
        step_kernel<T, BLOCK, int64_t><<<(unsigned)blocks, BLOCK, 0, st>>>(a);
    return check_launch("step_kernel");
}

int launch_step(const pic_grid *g_in, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                const void *dens, void *dens_zero, double *tally, void *ws, cudaStream_t st) {
    pic_grid r = *g_in;
    int rc = resolve_shape(&r);
    if (rc) return rc;
    const pic_grid *g = &r;
    if (g->variant == PIC_VARIANT_STREAM) {
        StreamShape sh{g->tile_rows, g->planes_per_item, g->stages, g->consumer_warps, g->ctas_per_sm, sm_count()};
        return launch_stream_step(g, sh, pos_in, neg_in, pos_out, neg_out, dens, dens_zero, tally, ws, st);
    }
    if (g->dtype == PIC_F64)
        return launch_step_t<double>(g, pos_in, neg_in, pos_out, neg_out, dens, dens_zero, tally, ws, st);
    return launch_step_t<float>(g, pos_in, neg_in, pos_out, neg_out, dens, dens_zero, tally, ws, st);
}

int step_occupancy(int dtype, int *blocks_per_sm) {
    cudaError_t e = dtype == PIC_F64
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, step_kernel<double, 256, uint32_t>, 256, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, step_kernel<float, 256, uint32_t>, 256, 0);
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaOccupancyMaxActiveBlocksPerMultiprocessor", e);
}

}  // namespace pic
