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
    const float2 *dens;  // deposition pairs (G * density, G * neighbours'); null: none
    float2 *dens_zero;   // the next step's pairs, cleared here; null: nothing to clear
    double *tally, *partials;
    unsigned int *counter;
    int *status;
    int n, kp, c4, nzb, nze, gap_end, reflecting;
    int dp;  // deposition row pitch (multiple of 4 pairs)
    int tj, li, jt, n_items, stages, consumer_warps;
    float p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt, gfac;
    int two_mid;    // 2 * mid_xy
    uint32_t thr4;  // scored iff (2i - two_mid)^2 + (2j - two_mid)^2 <= thr4
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

template <int IPT, int MAXT>
__global__ void __launch_bounds__(MAXT, 1) stream_step_kernel(StreamArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ volatile int abort_flag;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + a.stages;
    const int bar_bytes = (2 * a.stages * 8 + 127) / 128 * 128;
    float *stage0 = reinterpret_cast<float *>(smem_raw + bar_bytes);
    const int rows_max = a.tj + 2;
    const int spec = rows_max * a.kp;       // floats per species in a stage
    const int dens_off = 2 * spec;          // the plane's deposition pairs (float offset)
    const int stage_floats = 2 * spec + 2 * ((a.tj + 8) & ~3);
    const bool has_dens = a.dens != nullptr;
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
        // Per plane: the tile's rows (plus j-halo) of both species, and the
        // plane's deposition pairs over the same rows, fetched from their
        // 32-byte-aligned cover [a0, a0 + 4 * ceil((off + rows) / 4)) of the
        // padded row.
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < a.n_items && ok; w += gridDim.x) {
                int cj_lo, cj_hi, ci_lo, ci_hi;
                item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
                const int rows = cj_hi - cj_lo + 2;
                const uint32_t bytes = (uint32_t)(rows * a.kp * 4);
                const int doff = (cj_lo - 1) & 3;
                const uint32_t dbytes = has_dens ? (uint32_t)(((doff + rows + 3) & ~3) * 8) : 0u;
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
                    float *dst = stage0 + (size_t)slot * stage_floats;
                    const size_t src = ((size_t)pl * a.n + (cj_lo - 1)) * a.kp;
                    mbar_arrive_expect_tx(&full[slot], 2 * bytes + dbytes);
                    bulk_g2s(dst, a.pos_in + src, bytes, &full[slot]);
                    bulk_g2s(dst + spec, a.neg_in + src, bytes, &full[slot]);
                    if (has_dens)
                        bulk_g2s(dst + dens_off, a.dens + (size_t)pl * a.dp + (cj_lo - 1 - doff), dbytes,
                                 &full[slot]);
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
        // The k-vectors of a row split into CORE vectors, whose four elements
        // all lie in the gap (always valid, always deposited into, scored when
        // the column is), and EDGE vectors (the k = 0 plane, the electrode
        // buffers, the z end plane and the row padding). Core vectors take a
        // mask-free path in packed FP32x2 arithmetic; edge vectors the general
        // masked one. Work slot s of a plane is core item s (row s / ncore,
        // vector c_lo + s % ncore) for s < n_core, then edge items; consumer
        // thread t owns slots t + k * nct, k < IPT, so consecutive lanes hold
        // consecutive core vectors of a row (their k-1 / k+4 neighbours are
        // read from shared memory).
        const int ctid = threadIdx.x;
        const int nct = cw * 32;
        const int n = a.n, kp = a.kp, c4 = a.c4;
        const int c_lo = (a.nze + 3) / 4, c_hi = a.gap_end / 4;  // core vectors: [c_lo, c_hi)
        const int ncore = c_hi > c_lo ? c_hi - c_lo : 0;
        const int nedge = c4 - ncore;
        const bool gap_below = 4 * c_lo - 1 >= a.nze;  // element before the first core vector
        const bool gap_above = 4 * c_hi < a.gap_end;   // element after the last core vector
        const int64_t plane_stride = (int64_t)n * kp;
        const float2 ZMp = make_float2(a.p_zm, a.p_zm), ZPp = make_float2(a.p_zp, a.p_zp);
        const float2 LATp = make_float2(a.p_lat, a.p_lat), CENp = make_float2(a.p_cen, a.p_cen);
        const float2 ZMn = make_float2(a.n_zm, a.n_zm), ZPn = make_float2(a.n_zp, a.n_zp);
        const float2 LATn = make_float2(a.n_lat, a.n_lat), CENn = make_float2(a.n_cen, a.n_cen);
        const float2 ADT = make_float2(a.alpha_dt, a.alpha_dt), NEG1 = make_float2(-1.f, -1.f);
        long long g = 0;
        for (int w = blockIdx.x; w < a.n_items; w += gridDim.x) {
            int cj_lo, cj_hi, ci_lo, ci_hi;
            item_geometry(a, w, cj_lo, cj_hi, ci_lo, ci_hi);
            const int nplanes = ci_hi - ci_lo + 2;
            const int rows_out = cj_hi - cj_lo;
            const int n_core = rows_out * ncore, n_all = rows_out * c4;
            const int dq = (cj_lo - 1) & 3;  // pair of staged row q: dq + q
            // per-slot constants: kind (0 dead, 1 core, 2 edge), row+1, vector
            int kind[IPT], rs_[IPT], c_[IPT];
            uint32_t dy2[IPT];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const int sl = ctid + k * nct;
                int r = 0, c = 0, kd = 0;
                if (sl < n_core) {
                    r = sl / ncore;
                    c = c_lo + (sl - r * ncore);
                    kd = 1;
                } else if (sl < n_all) {
                    const int e = sl - n_core;
                    r = e / nedge;
                    const int ei = e - r * nedge;
                    c = ei < c_lo ? ei : ncore + ei;  // edge vectors below, then above the core
                    kd = 2;
                }
                kind[k] = kd;
                rs_[k] = r + 1;
                c_[k] = c;
                const int dy = 2 * (cj_lo + r) - a.two_mid;
                dy2[k] = (uint32_t)(dy * dy);
            }
            // ring positions of loads g (plane ci-1), g+1 (ci), g+2 (ci+1),
            // advanced incrementally: slot index and the phase parity to wait on
            int sm_ = (int)(g % S), sc_ = sm_ + 1 == S ? 0 : sm_ + 1, sp_ = sc_ + 1 == S ? 0 : sc_ + 1;
            uint32_t pm_ = (uint32_t)((g / S) & 1), pc_ = sc_ == 0 ? pm_ ^ 1u : pm_, pp_ = sp_ == 0 ? pc_ ^ 1u : pc_;
            if (!mbar_wait(&full[sm_], pm_, a.status, 3) || !mbar_wait(&full[sc_], pc_, a.status, 3)) abort_flag = 1;
            for (int q = 0; q < ci_hi - ci_lo && !abort_flag; ++q) {
                if (!mbar_wait(&full[sp_], pp_, a.status, 3)) {
                    abort_flag = 1;
                    break;
                }
                const float *Sm = stage0 + (size_t)sm_ * stage_floats;
                const float *Sc = stage0 + (size_t)sc_ * stage_floats;
                const float *Sp = stage0 + (size_t)sp_ * stage_floats;
                const int ci = ci_lo + q;
                const int dx = 2 * ci - a.two_mid;
                const uint32_t dx2 = (uint32_t)(dx * dx);
                const int64_t pbase = (int64_t)ci * plane_stride;
                float *const pos_plane = a.pos_out + pbase;  // outputs of this plane; items add a 32-bit offset
                float *const neg_plane = a.neg_out + pbase;
                const bool edge_i = (ci == 1) || (ci == n - 2);
                float rec_acc = 0.f, p_acc = 0.f, n_acc = 0.f;
#pragma unroll
                for (int k = 0; k < IPT; ++k) {
                    const int kd = kind[k], rs = rs_[k], c = c_[k];
                    const int k0 = 4 * c;
                    const int o = rs * kp + k0;
                    // centre vectors and this column's densities
                    float4 P = lds4(Sc + o), N = lds4(Sc + spec + o);
                    const float2 dpair = has_dens ? reinterpret_cast<const float2 *>(Sc + dens_off)[dq + rs]
                                                  : make_float2(0.f, 0.f);
                    const float dens_c = dpair.x;  // G * density of this column
                    const float dcen = dens_c;
                    const float dlat = dpair.y;    // G * density of its four neighbours
                    if (kd == 1) {
                        P.x += dcen; P.y += dcen; P.z += dcen; P.w += dcen;
                        N.x += dcen; N.y += dcen; N.z += dcen; N.w += dcen;
                    }
                    if (kd == 0) continue;
                    const int cj = cj_lo + rs - 1;
                    const bool scored = (dx2 + dy2[k] <= a.thr4);
                    float4 PO, NO;
                    if (kd == 1) {
                        // ---- core vector: mask-free, packed FP32x2 ----
                        // k-1 / k+4 neighbours from shared memory (+ their
                        // deposition when they lie in the gap): uniform across the
                        // warp, where shuffles needed a divergent fallback at the
                        // warp's and the core's ends (measured 1.255 -> 1.201 ms a
                        // full-electrode step)
                        float pkm, nkm, pkp, nkp;
                        {
                            const float dm = (c > c_lo || gap_below) ? dcen : 0.f;
                            const float dp = (c < c_hi - 1 || gap_above) ? dcen : 0.f;
                            pkm = Sc[o - 1] + dm;
                            nkm = Sc[spec + o - 1] + dm;
                            pkp = Sc[o + 4] + dp;
                            nkp = Sc[spec + o + 4] + dp;
                        }
                        const float4 Pjm = lds4(Sc + o - kp), Pjp = lds4(Sc + o + kp);
                        const float4 Pim = lds4(Sm + o), Pip = lds4(Sp + o);
                        const float2 DL = make_float2(dlat, dlat);
                        const float2 Llo = __fadd2_rn(__fadd2_rn(__fadd2_rn(make_float2(Pjm.x, Pjm.y), make_float2(Pjp.x, Pjp.y)),
                                                                 __fadd2_rn(make_float2(Pim.x, Pim.y), make_float2(Pip.x, Pip.y))), DL);
                        const float2 Lhi = __fadd2_rn(__fadd2_rn(__fadd2_rn(make_float2(Pjm.z, Pjm.w), make_float2(Pjp.z, Pjp.w)),
                                                                 __fadd2_rn(make_float2(Pim.z, Pim.w), make_float2(Pip.z, Pip.w))), DL);
                        const float4 Njm = lds4(Sc + spec + o - kp), Njp = lds4(Sc + spec + o + kp);
                        const float4 Nim = lds4(Sm + spec + o), Nip = lds4(Sp + spec + o);
                        const float2 Mlo = __fadd2_rn(__fadd2_rn(__fadd2_rn(make_float2(Njm.x, Njm.y), make_float2(Njp.x, Njp.y)),
                                                                 __fadd2_rn(make_float2(Nim.x, Nim.y), make_float2(Nip.x, Nip.y))), DL);
                        const float2 Mhi = __fadd2_rn(__fadd2_rn(__fadd2_rn(make_float2(Njm.z, Njm.w), make_float2(Njp.z, Njp.w)),
                                                                 __fadd2_rn(make_float2(Nim.z, Nim.w), make_float2(Nip.z, Nip.w))), DL);
                        const float2 Plo = make_float2(P.x, P.y), Phi = make_float2(P.z, P.w);
                        const float2 Nlo = make_float2(N.x, N.y), Nhi = make_float2(N.z, N.w);
                        // positive: zm * n[k-1] + zp * n[k+1] + lat * L + cen * n
                        float2 plo = __ffma2_rn(CENp, Plo, __ffma2_rn(LATp, Llo, __ffma2_rn(ZPp, make_float2(P.y, P.z), __fmul2_rn(ZMp, make_float2(pkm, P.x)))));
                        float2 phi = __ffma2_rn(CENp, Phi, __ffma2_rn(LATp, Lhi, __ffma2_rn(ZPp, make_float2(P.w, pkp), __fmul2_rn(ZMp, make_float2(P.y, P.z)))));
                        // negative drifts the other way: zm on k+1, zp on k-1
                        float2 nlo = __ffma2_rn(CENn, Nlo, __ffma2_rn(LATn, Mlo, __ffma2_rn(ZPn, make_float2(nkm, N.x), __fmul2_rn(ZMn, make_float2(N.y, N.z)))));
                        float2 nhi = __ffma2_rn(CENn, Nhi, __ffma2_rn(LATn, Mhi, __ffma2_rn(ZPn, make_float2(N.y, N.z), __fmul2_rn(ZMn, make_float2(N.w, nkp)))));
                        const float2 rlo = __fmul2_rn(__fmul2_rn(ADT, Plo), Nlo);
                        const float2 rhi = __fmul2_rn(__fmul2_rn(ADT, Phi), Nhi);
                        plo = __ffma2_rn(rlo, NEG1, plo);
                        phi = __ffma2_rn(rhi, NEG1, phi);
                        nlo = __ffma2_rn(rlo, NEG1, nlo);
                        nhi = __ffma2_rn(rhi, NEG1, nhi);
                        PO = make_float4(plo.x, plo.y, phi.x, phi.y);
                        NO = make_float4(nlo.x, nlo.y, nhi.x, nhi.y);
                        if (scored) {
                            const float2 rs2 = __fadd2_rn(rlo, rhi), ps2 = __fadd2_rn(plo, phi), ns2 = __fadd2_rn(nlo, nhi);
                            rec_acc += rs2.x + rs2.y;
                            p_acc += ps2.x + ps2.y;
                            n_acc += ns2.x + ns2.y;
                        }
                    } else {
                        // ---- edge vector: per-element gap and validity masks ----
                        float gk[4];
                        bool valid[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int kk = k0 + e;
                            gk[e] = (kk >= a.nze && kk < a.gap_end) ? 1.f : 0.f;
                            valid[e] = kk >= 1 && kk <= a.nzb - 2;
                        }
                        P.x = fmaf(gk[0], dcen, P.x); P.y = fmaf(gk[1], dcen, P.y);
                        P.z = fmaf(gk[2], dcen, P.z); P.w = fmaf(gk[3], dcen, P.w);
                        N.x = fmaf(gk[0], dcen, N.x); N.y = fmaf(gk[1], dcen, N.y);
                        N.z = fmaf(gk[2], dcen, N.z); N.w = fmaf(gk[3], dcen, N.w);
                        const bool g_km = (k0 - 1 >= a.nze && k0 - 1 < a.gap_end);
                        const bool g_kp = (k0 + 4 >= a.nze && k0 + 4 < a.gap_end);
                        const float pkm = c > 0 ? Sc[o - 1] + (g_km ? dcen : 0.f) : 0.f;
                        const float nkm = c > 0 ? Sc[spec + o - 1] + (g_km ? dcen : 0.f) : 0.f;
                        const float pkp = c + 1 < c4 ? Sc[o + 4] + (g_kp ? dcen : 0.f) : 0.f;
                        const float nkp = c + 1 < c4 ? Sc[spec + o + 4] + (g_kp ? dcen : 0.f) : 0.f;
                        const float4 Pjm = lds4(Sc + o - kp), Pjp = lds4(Sc + o + kp);
                        const float4 Njm = lds4(Sc + spec + o - kp), Njp = lds4(Sc + spec + o + kp);
                        const float4 Pim = lds4(Sm + o), Pip = lds4(Sp + o);
                        const float4 Nim = lds4(Sm + spec + o), Nip = lds4(Sp + spec + o);
                        const float pv[6] = {pkm, P.x, P.y, P.z, P.w, pkp};
                        const float nv[6] = {nkm, N.x, N.y, N.z, N.w, nkp};
                        const float pl4[4] = {fmaf(gk[0], dlat, (Pjm.x + Pjp.x) + (Pim.x + Pip.x)),
                                              fmaf(gk[1], dlat, (Pjm.y + Pjp.y) + (Pim.y + Pip.y)),
                                              fmaf(gk[2], dlat, (Pjm.z + Pjp.z) + (Pim.z + Pip.z)),
                                              fmaf(gk[3], dlat, (Pjm.w + Pjp.w) + (Pim.w + Pip.w))};
                        const float nl4[4] = {fmaf(gk[0], dlat, (Njm.x + Njp.x) + (Nim.x + Nip.x)),
                                              fmaf(gk[1], dlat, (Njm.y + Njp.y) + (Nim.y + Nip.y)),
                                              fmaf(gk[2], dlat, (Njm.z + Njp.z) + (Nim.z + Nip.z)),
                                              fmaf(gk[3], dlat, (Njm.w + Njp.w) + (Nim.w + Nip.w))};
                        float po[4], no[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const float p = pv[e + 1], nn = nv[e + 1];
                            const float p_new = a.p_zm * pv[e] + a.p_zp * pv[e + 2] + a.p_lat * pl4[e] + a.p_cen * p;
                            const float n_new = a.n_zm * nv[e + 2] + a.n_zp * nv[e] + a.n_lat * nl4[e] + a.n_cen * nn;
                            const float rec = a.alpha_dt * p * nn;
                            po[e] = valid[e] ? p_new - rec : 0.f;
                            no[e] = valid[e] ? n_new - rec : 0.f;
                            if (scored && gk[e] != 0.f) {
                                rec_acc += rec;
                                p_acc += po[e];
                                n_acc += no[e];
                            }
                        }
                        PO = make_float4(po[0], po[1], po[2], po[3]);
                        NO = make_float4(no[0], no[1], no[2], no[3]);
                        if (c == 0) {
                            if (scored && has_dens) t_inj.add(dens_c);
                            if (a.dens_zero) a.dens_zero[(int64_t)ci * a.dp + cj] = make_float2(0.f, 0.f);
                        }
                    }
                    const int out = cj * kp + k0;
                    st4(pos_plane + out, PO);
                    st4(neg_plane + out, NO);

                    // ring columns attached to this interior column
                    const bool lo_j = (cj == 1), hi_j = (cj == n - 2);
                    if (edge_i || lo_j || hi_j) {
                        const bool lo_i = (ci == 1), hi_i = (ci == n - 2);
                        // up to three targets: (ri, cj), (ci, rj), (ri, rj)
                        for (int tgt = 0; tgt < 3; ++tgt) {
                            int ri = ci, rj = cj;
                            const float *Sr = Sc;
                            int row = rs;
                            if (tgt == 0) {
                                if (!(lo_i || hi_i)) continue;
                                ri = lo_i ? 0 : n - 1;
                                Sr = lo_i ? Sm : Sp;
                            } else if (tgt == 1) {
                                if (!(lo_j || hi_j)) continue;
                                rj = lo_j ? 0 : n - 1;
                                row = lo_j ? rs - 1 : rs + 1;
                            } else {
                                if (!((lo_i || hi_i) && (lo_j || hi_j))) continue;
                                ri = lo_i ? 0 : n - 1;
                                rj = lo_j ? 0 : n - 1;
                                Sr = lo_i ? Sm : Sp;
                                row = lo_j ? rs - 1 : rs + 1;
                            }
                            const int64_t rcol = (int64_t)ri * n + rj;
                            if (a.reflecting) {
                                st4(a.pos_out + rcol * kp + k0, PO);
                                st4(a.neg_out + rcol * kp + k0, NO);
                            } else {
                                float4 RP = lds4(Sr + row * kp + k0), RN = lds4(Sr + spec + row * kp + k0);
                                const float d = has_dens ? reinterpret_cast<const float2 *>(Sr + dens_off)[dq + row].x : 0.f;
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    const int kk = k0 + e;
                                    const float de = (kk >= a.nze && kk < a.gap_end) ? d : 0.f;
                                    (&RP.x)[e] += de;
                                    (&RN.x)[e] += de;
                                }
                                st4(a.pos_out + rcol * kp + k0, RP);
                                st4(a.neg_out + rcol * kp + k0, RN);
                            }
                            if (c == 0 && a.dens_zero) a.dens_zero[(int64_t)ri * a.dp + rj] = make_float2(0.f, 0.f);
                        }
                    }
                }
                t_rec.add(rec_acc);
                t_p.add(p_acc);
                t_n.add(n_acc);
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[sm_]);
                // advance the window by one load
                sm_ = sc_; pm_ = pc_;
                sc_ = sp_; pc_ = pp_;
                sp_ = sp_ + 1 == S ? 0 : sp_ + 1;
                pp_ = sp_ == 0 ? pp_ ^ 1u : pp_;
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
    return (2 * stages * 8 + 127) / 128 * 128 + stages * (2 * (tj + 2) * kp + 2 * ((tj + 8) & ~3)) * 4;
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
    a.p_lat = (float)g->p_lat; a.p_zm = (float)g->p_zm; a.p_zp = (float)g->p_zp; a.p_cen = (float)g->p_cen;
    a.n_lat = (float)g->n_lat; a.n_zm = (float)g->n_zm; a.n_zp = (float)g->n_zp; a.n_cen = (float)g->n_cen;
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
