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
// The step's deposition (gaussian_factor * dens[i][j], gap layers only) is
// added to every value as it is read, the fused form of the reference's
// separate broadcast pass (solver_numba_parallel.py:222-277). The z end planes
// k = 0 and k >= nzb-1 (and the row padding) are written as zero.
//
// Tallies over the scored set (interior, inside scoring_radius_sq, gap
// layers) follow _lax_wendroff_step_numba (solver_numba.py:204-211):
// recombined uses the pre-step densities, n+/n- the updated ones. The
// injected charge of the step is sum(dens) over scored columns times
// gaussian_factor * no_z (solver_numba_parallel.py:271-276).
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_device.cuh"
#include "pic_internal.h"

namespace pic {

template <typename T>
struct StepArgs {
    const T *pos_in, *neg_in;
    T *pos_out, *neg_out;
    const T *dens;   // null: no deposition this step
    T *dens_zero;    // null: nothing to clear
    double *tally;
    double *partials;
    unsigned int *counter;
    int64_t n, kp, c4, items, dp;  // dp: density row pitch
    int nzb, nze, gap_end;  // gap = [nze, gap_end)
    int reflecting;
    T p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt, gfac;
    ScoreTest score;
    double injected_scale;
};

template <typename T>
__device__ __forceinline__ T dep_at(const StepArgs<T> &a, int64_t dcol) {
    return a.dens ? a.gfac * a.dens[dcol] : T(0);
}

template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) step_kernel(StepArgs<T> a) {
    Tally<T> t_rec, t_p, t_n, t_inj;
    const int64_t stride = (int64_t)gridDim.x * BLOCK;
    const int64_t n = a.n, kp = a.kp;
    for (int64_t item = (int64_t)blockIdx.x * BLOCK + threadIdx.x; item < a.items; item += stride) {
        const int64_t col = item / a.c4;
        const int c = (int)(item - col * a.c4);
        const int64_t i = col / n, j = col - i * n;
        const int k0 = 4 * c;
        if (c == 0 && a.dens_zero) a.dens_zero[i * a.dp + j] = T(0);

        // gap mask of the four outputs and of the two z-neighbours
        bool g[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) g[e] = (k0 + e >= a.nze) && (k0 + e < a.gap_end);
        const bool g_km = (k0 - 1 >= a.nze) && (k0 - 1 < a.gap_end);
        const bool g_kp = (k0 + 4 >= a.nze) && (k0 + 4 < a.gap_end);

        const int64_t ci = i < 1 ? 1 : (i > n - 2 ? n - 2 : i);
        const int64_t cj = j < 1 ? 1 : (j > n - 2 ? n - 2 : j);
        const bool ring = (ci != i) || (cj != j);
        const int64_t out_off = col * kp + k0;

        if (ring && !a.reflecting) {
            const T d = dep_at(a, i * a.dp + j);
            V4<T> P = load4(a.pos_in + out_off), N = load4(a.neg_in + out_off);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                P.v[e] += g[e] ? d : T(0);
                N.v[e] += g[e] ? d : T(0);
            }
            store4(a.pos_out + out_off, P);
            store4(a.neg_out + out_off, N);
            continue;
        }

        const int64_t ccol = ci * n + cj;
        const int64_t base = ccol * kp + k0;
        const int64_t di = n * kp;
        V4<T> P = load4(a.pos_in + base), N = load4(a.neg_in + base);
        V4<T> Pim = load4(a.pos_in + base - di), Pip = load4(a.pos_in + base + di);
        V4<T> Pjm = load4(a.pos_in + base - kp), Pjp = load4(a.pos_in + base + kp);
        V4<T> Nim = load4(a.neg_in + base - di), Nip = load4(a.neg_in + base + di);
        V4<T> Njm = load4(a.neg_in + base - kp), Njp = load4(a.neg_in + base + kp);
        T pkm = c > 0 ? a.pos_in[base - 1] : T(0);
        T nkm = c > 0 ? a.neg_in[base - 1] : T(0);
        T pkp = k0 + 4 < kp ? a.pos_in[base + 4] : T(0);
        T nkp = k0 + 4 < kp ? a.neg_in[base + 4] : T(0);

        const int64_t dcol = ci * a.dp + cj;
        if (a.dens) {
            const T dc = a.gfac * a.dens[dcol];
            const T dim = a.gfac * a.dens[dcol - a.dp], dip = a.gfac * a.dens[dcol + a.dp];
            const T djm = a.gfac * a.dens[dcol - 1], djp = a.gfac * a.dens[dcol + 1];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                if (g[e]) {
                    P.v[e] += dc; N.v[e] += dc;
                    Pim.v[e] += dim; Nim.v[e] += dim;
                    Pip.v[e] += dip; Nip.v[e] += dip;
                    Pjm.v[e] += djm; Njm.v[e] += djm;
                    Pjp.v[e] += djp; Njp.v[e] += djp;
                }
            }
            if (g_km) { pkm += dc; nkm += dc; }
            if (g_kp) { pkp += dc; nkp += dc; }
        }

        const bool scored_col = !ring && scored_column(a.score, ci, cj);
        V4<T> PO, NO;
        T rec_sum = 0, p_sum = 0, n_sum = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = k0 + e;
            const T p = P.v[e], nn = N.v[e];
            const T p_km1 = e > 0 ? P.v[e - 1] : pkm;
            const T p_kp1 = e < 3 ? P.v[e + 1] : pkp;
            const T n_km1 = e > 0 ? N.v[e - 1] : nkm;
            const T n_kp1 = e < 3 ? N.v[e + 1] : nkp;
            const T p_new = a.p_zm * p_km1 + a.p_zp * p_kp1 +
                            a.p_lat * ((Pjm.v[e] + Pjp.v[e]) + (Pim.v[e] + Pip.v[e])) + a.p_cen * p;
            const T n_new = a.n_zm * n_kp1 + a.n_zp * n_km1 +
                            a.n_lat * ((Njm.v[e] + Njp.v[e]) + (Nim.v[e] + Nip.v[e])) + a.n_cen * nn;
            const T rec = a.alpha_dt * p * nn;
            const bool valid = (k >= 1) && (k <= a.nzb - 2);
            const T po = valid ? p_new - rec : T(0);
            const T no = valid ? n_new - rec : T(0);
            PO.v[e] = po;
            NO.v[e] = no;
            if (scored_col && g[e]) {
                rec_sum += rec;
                p_sum += po;
                n_sum += no;
            }
        }
        store4(a.pos_out + out_off, PO);
        store4(a.neg_out + out_off, NO);
        if (scored_col) {
            t_rec.add(rec_sum);
            t_p.add(p_sum);
            t_n.add(n_sum);
            if (c == 0 && a.dens) t_inj.add(a.dens[dcol]);
        }
    }
    double v[4] = {t_inj.value(), t_rec.value(), t_p.value(), t_n.value()};
    finish_tally<BLOCK>(v, a.partials, a.counter, a.tally, a.injected_scale);
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
    a.dens = (const T *)dens;
    a.dens_zero = (T *)dens_zero;
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
    a.p_lat = (T)g->p_lat; a.p_zm = (T)g->p_zm; a.p_zp = (T)g->p_zp; a.p_cen = (T)g->p_cen;
    a.n_lat = (T)g->n_lat; a.n_zm = (T)g->n_zm; a.n_zp = (T)g->n_zp; a.n_cen = (T)g->n_cen;
    a.alpha_dt = (T)g->alpha_dt;
    a.gfac = (T)g->gaussian_factor;
    int rc = score_test(g, &a.score);
    if (rc) return rc;
    a.injected_scale = g->gaussian_factor * (double)g->no_z;
    int64_t blocks = (a.items + BLOCK - 1) / BLOCK;
    const int64_t cap = step_grid_cap(g->dtype == PIC_F64 ? 1 : 0);
    if (blocks > cap) blocks = cap;
    if (blocks > kMaxStepBlocks) blocks = kMaxStepBlocks;
    step_kernel<T, BLOCK><<<(unsigned)blocks, BLOCK, 0, st>>>(a);
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
                        ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, step_kernel<double, 256>, 256, 0)
                        : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, step_kernel<float, 256>, 256, 0);
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaOccupancyMaxActiveBlocksPerMultiprocessor", e);
}

}  // namespace pic
