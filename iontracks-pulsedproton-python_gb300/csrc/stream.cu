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

namespace pic {

struct StreamArgs {
    const float *pos_in, *neg_in;
    float *pos_out, *neg_out;
    const float *dens;  // null: no deposition this step
    float *dens_zero;   // null: nothing to clear
    double *tally, *partials;
    unsigned int *counter;
    int *status;
    int n, kp, c4, nzb, nze, gap_end, reflecting;
    int tj, li, jt, n_items, stages, consumer_warps;
    float p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt, gfac;
    ScoreTest score;
    double injected_scale;
};

__device__ __forceinline__ void item_geometry(const StreamArgs &a, int w, int &cj_lo, int &cj_hi, int &ci_lo,
                                              int &ci_hi) {
    const int u = w / a.jt, t = w - u * a.jt;
    cj_lo = 1 + t * a.tj;
    cj_hi = min(cj_lo + a.tj, a.n - 1);
    ci_lo = 1 + u * a.li;
    ci_hi = min(ci_lo + a.li, a.n - 1);
}

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ void add_dep(float4 &v, float d, const bool (&g)[4]) {
    v.x += g[0] ? d : 0.f;
    v.y += g[1] ? d : 0.f;
    v.z += g[2] ? d : 0.f;
    v.w += g[3] ? d : 0.f;
}

__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }

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

__global__ void __launch_bounds__(kStreamMaxThreads, 1) stream_step_kernel(StreamArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ volatile int abort_flag;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + a.stages;
    const int bar_bytes = (2 * a.stages * 8 + 127) / 128 * 128;
    float *stage0 = reinterpret_cast<float *>(smem_raw + bar_bytes);
    const int rows_max = a.tj + 2;
    const int spec = rows_max * a.kp;       // floats per species in a stage
    const int dens_off = 2 * spec;          // the plane's density at each staged row
    const int stage_floats = 2 * spec + ((rows_max + 3) & ~3);
    const int S = a.stages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = a.consumer_warps;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            // full: the producer's expect-tx arrival + the arrival after the
            // density row is staged; the bulk copies' bytes complete it.
            mbar_init(&full[s], 2);
            mbar_init(&empty[s], cw);
        }
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();

    Tally<float> t_rec, t_p, t_n, t_inj;

    if (warp == cw) {
        // ---------------- producer warp ----------------
        // lane 0 issues the bulk copies; every lane stages one density value
        // of the plane's rows; lane 0 then arrives a second time.
        long long g = 0;
        bool ok = true;
        for (int w = blockIdx.x; w < a.n_items && ok; w += gridDim.x) {
            int cj_lo, cj_hi, ci_lo, ci_hi;
            item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
            const int rows = cj_hi - cj_lo + 2;
            const uint32_t bytes = (uint32_t)(rows * a.kp * 4);
            for (int pl = ci_lo - 1; pl <= ci_hi; ++pl, ++g) {
                const int slot = (int)(g % S);
                if (g >= S && !mbar_wait(&empty[slot], (uint32_t)(((g / S) - 1) & 1), a.status, 1)) abort_flag = 1;
                __syncwarp();
                if (abort_flag) {
                    ok = false;
                    break;
                }
                float *dst = stage0 + (size_t)slot * stage_floats;
                const size_t src = ((size_t)pl * a.n + (cj_lo - 1)) * a.kp;
                if (lane == 0) {
                    mbar_arrive_expect_tx(&full[slot], 2 * bytes);
                    bulk_g2s(dst, a.pos_in + src, bytes, &full[slot]);
                    bulk_g2s(dst + spec, a.neg_in + src, bytes, &full[slot]);
                }
                for (int q = lane; q < rows; q += 32)
                    dst[dens_off + q] = a.dens ? __ldg(a.dens + (size_t)pl * a.n + (cj_lo - 1) + q) : 0.f;
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[slot]);
            }
        }
        if (!ok && lane == 0) {
            // drain: every copy still in flight must land before exit
            for (long long gg = g - S < 0 ? 0 : g - S; gg < g; ++gg)
                mbar_wait(&full[gg % S], (uint32_t)((gg / S) & 1), a.status, 2);
        }
    } else {
        // ---------------- consumers ----------------
        const int ctid = threadIdx.x;
        const int nct = cw * 32;
        const int n = a.n, kp = a.kp;
        long long g = 0;
        for (int w = blockIdx.x; w < a.n_items; w += gridDim.x) {
            int cj_lo, cj_hi, ci_lo, ci_hi;
            item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
            const int nplanes = ci_hi - ci_lo + 2;
            if (!mbar_wait(&full[g % S], (uint32_t)((g / S) & 1), a.status, 3) ||
                !mbar_wait(&full[(g + 1) % S], (uint32_t)(((g + 1) / S) & 1), a.status, 3))
                abort_flag = 1;
            const int rows_out = cj_hi - cj_lo;
            const int n_it = rows_out * a.c4;
            for (int q = 0; q < ci_hi - ci_lo && !abort_flag; ++q) {
                const long long gm = g + q, gc = gm + 1, gp = gm + 2;
                if (!mbar_wait(&full[gp % S], (uint32_t)((gp / S) & 1), a.status, 3)) {
                    abort_flag = 1;
                    break;
                }
                const float *Sm = stage0 + (size_t)(gm % S) * stage_floats;
                const float *Sc = stage0 + (size_t)(gc % S) * stage_floats;
                const float *Sp = stage0 + (size_t)(gp % S) * stage_floats;
                const int ci = ci_lo + q;
                for (int it = ctid; it < n_it; it += nct) {
                    const int r = it / a.c4;
                    const int c = it - r * a.c4;
                    const int cj = cj_lo + r;
                    const int k0 = 4 * c;
                    const int rs = r + 1;
                    bool gk[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) gk[e] = (k0 + e >= a.nze) && (k0 + e < a.gap_end);
                    const bool g_km = (k0 - 1 >= a.nze) && (k0 - 1 < a.gap_end);
                    const bool g_kp = (k0 + 4 >= a.nze) && (k0 + 4 < a.gap_end);
                    const int oc = rs * kp + k0;  // offset of the centre vector in a species block
                    float4 P = lds4(Sc + oc), N = lds4(Sc + spec + oc);
                    float4 Pjm = lds4(Sc + oc - kp), Njm = lds4(Sc + spec + oc - kp);
                    float4 Pjp = lds4(Sc + oc + kp), Njp = lds4(Sc + spec + oc + kp);
                    float4 Pim = lds4(Sm + oc), Nim = lds4(Sm + spec + oc);
                    float4 Pip = lds4(Sp + oc), Nip = lds4(Sp + spec + oc);
                    float pkm = c > 0 ? Sc[oc - 1] : 0.f, nkm = c > 0 ? Sc[spec + oc - 1] : 0.f;
                    float pkp = k0 + 4 < kp ? Sc[oc + 4] : 0.f, nkp = k0 + 4 < kp ? Sc[spec + oc + 4] : 0.f;
                    const int64_t ccol = (int64_t)ci * n + cj;
                    const float dens_c = Sc[dens_off + rs];
                    if (a.dens) {
                        const float dc = a.gfac * dens_c;
                        const float dim = a.gfac * Sm[dens_off + rs], dip = a.gfac * Sp[dens_off + rs];
                        const float djm = a.gfac * Sc[dens_off + rs - 1], djp = a.gfac * Sc[dens_off + rs + 1];
                        add_dep(P, dc, gk);
                        add_dep(N, dc, gk);
                        add_dep(Pjm, djm, gk);
                        add_dep(Njm, djm, gk);
                        add_dep(Pjp, djp, gk);
                        add_dep(Njp, djp, gk);
                        add_dep(Pim, dim, gk);
                        add_dep(Nim, dim, gk);
                        add_dep(Pip, dip, gk);
                        add_dep(Nip, dip, gk);
                        if (g_km) { pkm += dc; nkm += dc; }
                        if (g_kp) { pkp += dc; nkp += dc; }
                    }
                    const float pv[6] = {pkm, P.x, P.y, P.z, P.w, pkp};
                    const float nv[6] = {nkm, N.x, N.y, N.z, N.w, nkp};
                    const float pl4[4] = {(Pjm.x + Pjp.x) + (Pim.x + Pip.x), (Pjm.y + Pjp.y) + (Pim.y + Pip.y),
                                          (Pjm.z + Pjp.z) + (Pim.z + Pip.z), (Pjm.w + Pjp.w) + (Pim.w + Pip.w)};
                    const float nl4[4] = {(Njm.x + Njp.x) + (Nim.x + Nip.x), (Njm.y + Njp.y) + (Nim.y + Nip.y),
                                          (Njm.z + Njp.z) + (Nim.z + Nip.z), (Njm.w + Njp.w) + (Nim.w + Nip.w)};
                    const bool scored = scored_column(a.score, ci, cj);
                    float po[4], no[4];
                    float rec_sum = 0.f, p_sum = 0.f, n_sum = 0.f;
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int k = k0 + e;
                        const float p = pv[e + 1], nn = nv[e + 1];
                        const float p_new = a.p_zm * pv[e] + a.p_zp * pv[e + 2] + a.p_lat * pl4[e] + a.p_cen * p;
                        const float n_new = a.n_zm * nv[e + 2] + a.n_zp * nv[e] + a.n_lat * nl4[e] + a.n_cen * nn;
                        const float rec = a.alpha_dt * p * nn;
                        const bool valid = (k >= 1) && (k <= a.nzb - 2);
                        po[e] = valid ? p_new - rec : 0.f;
                        no[e] = valid ? n_new - rec : 0.f;
                        if (scored && gk[e]) {
                            rec_sum += rec;
                            p_sum += po[e];
                            n_sum += no[e];
                        }
                    }
                    const float4 PO = make_float4(po[0], po[1], po[2], po[3]);
                    const float4 NO = make_float4(no[0], no[1], no[2], no[3]);
                    st4(a.pos_out + ccol * kp + k0, PO);
                    st4(a.neg_out + ccol * kp + k0, NO);
                    if (scored) {
                        t_rec.add(rec_sum);
                        t_p.add(p_sum);
                        t_n.add(n_sum);
                        if (c == 0 && a.dens) t_inj.add(dens_c);
                    }
                    if (c == 0 && a.dens_zero) a.dens_zero[ccol] = 0.f;

                    // ring columns attached to this interior column
                    const bool lo_i = (ci == 1), hi_i = (ci == n - 2), lo_j = (cj == 1), hi_j = (cj == n - 2);
                    if (lo_i || hi_i || lo_j || hi_j) {
                        // up to three targets: (ri, cj), (ci, rj), (ri, rj)
                        for (int tgt = 0; tgt < 3; ++tgt) {
                            int ri = ci, rj = cj;
                            const float *S = Sc;
                            int row = rs;
                            if (tgt == 0) {
                                if (!(lo_i || hi_i)) continue;
                                ri = lo_i ? 0 : n - 1;
                                S = lo_i ? Sm : Sp;
                            } else if (tgt == 1) {
                                if (!(lo_j || hi_j)) continue;
                                rj = lo_j ? 0 : n - 1;
                                row = lo_j ? rs - 1 : rs + 1;
                            } else {
                                if (!((lo_i || hi_i) && (lo_j || hi_j))) continue;
                                ri = lo_i ? 0 : n - 1;
                                rj = lo_j ? 0 : n - 1;
                                S = lo_i ? Sm : Sp;
                                row = lo_j ? rs - 1 : rs + 1;
                            }
                            const int64_t rcol = (int64_t)ri * n + rj;
                            if (a.reflecting) {
                                st4(a.pos_out + rcol * kp + k0, PO);
                                st4(a.neg_out + rcol * kp + k0, NO);
                            } else {
                                float4 RP = lds4(S + row * kp + k0), RN = lds4(S + spec + row * kp + k0);
                                if (a.dens) {
                                    const float d = a.gfac * S[dens_off + row];
                                    add_dep(RP, d, gk);
                                    add_dep(RN, d, gk);
                                }
                                st4(a.pos_out + rcol * kp + k0, RP);
                                st4(a.neg_out + rcol * kp + k0, RN);
                            }
                            if (c == 0 && a.dens_zero) a.dens_zero[rcol] = 0.f;
                        }
                    }
                }
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[gm % S]);
            }
            if (abort_flag) break;
            __syncwarp();
            if (lane == 0) {
                mbar_arrive(&empty[(g + nplanes - 2) % S]);
                mbar_arrive(&empty[(g + nplanes - 1) % S]);
            }
            g += nplanes;
        }
    }
    double v[4] = {t_inj.value(), t_rec.value(), t_p.value(), t_n.value()};
    finish_tally_rt(v, a.partials, a.counter, a.tally, a.injected_scale);
}

int stream_smem_bytes(int tj, int kp, int stages) {
    return (2 * stages * 8 + 127) / 128 * 128 + stages * (2 * (tj + 2) * kp + ((tj + 2 + 3) & ~3)) * 4;
}

int launch_stream_step(const pic_grid *g, const StreamShape &sh, const void *pos_in, const void *neg_in,
                       void *pos_out, void *neg_out, const void *dens, void *dens_zero, double *tally, void *ws,
                       cudaStream_t st) {
    StreamArgs a;
    a.pos_in = (const float *)pos_in;
    a.neg_in = (const float *)neg_in;
    a.pos_out = (float *)pos_out;
    a.neg_out = (float *)neg_out;
    a.dens = (const float *)dens;
    a.dens_zero = (float *)dens_zero;
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
    a.tj = sh.tile_rows;
    a.li = sh.planes_per_item;
    a.jt = (a.n - 2 + a.tj - 1) / a.tj;
    const int ic = (a.n - 2 + a.li - 1) / a.li;
    a.n_items = a.jt * ic;
    a.stages = sh.stages;
    a.consumer_warps = sh.consumer_warps;
    a.p_lat = (float)g->p_lat; a.p_zm = (float)g->p_zm; a.p_zp = (float)g->p_zp; a.p_cen = (float)g->p_cen;
    a.n_lat = (float)g->n_lat; a.n_zm = (float)g->n_zm; a.n_zp = (float)g->n_zp; a.n_cen = (float)g->n_cen;
    a.alpha_dt = (float)g->alpha_dt;
    a.gfac = (float)g->gaussian_factor;
    int rc = score_test(g, &a.score);
    if (rc) return rc;
    a.injected_scale = g->gaussian_factor * (double)g->no_z;
    const int smem = stream_smem_bytes(a.tj, a.kp, a.stages);
    static int configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(stream_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(stream_step_kernel)", e);
        configured = smem;
    }
    int64_t blocks = (int64_t)sh.sm_count * sh.ctas_per_sm;
    if (blocks > a.n_items) blocks = a.n_items;
    if (blocks > kMaxStepBlocks) blocks = kMaxStepBlocks;
    stream_step_kernel<<<(unsigned)blocks, (a.consumer_warps + 1) * 32, smem, st>>>(a);
    return check_launch("stream_step_kernel");
}

}  // namespace pic
