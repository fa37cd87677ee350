// pic_stream.cuh -- the consumer side of the streaming step, shared by the
// single-grid kernel (stream.cu) and the batched one (batched_stream.cu).
//
// A work item is a tile of interior rows j = [cj_lo, cj_hi) with every k,
// over interior planes i = [ci_lo, ci_hi). A producer warp streams the planes
// ci_lo-1 .. ci_hi of the item (rows cj_lo-1 .. cj_hi of both species, one
// contiguous block per species and plane, plus the plane's deposition pairs
// over the same rows) into an S-stage shared-memory ring; the consumer warps
// compute plane ci from the stages holding ci-1, ci and ci+1, so every stencil
// neighbour is read from shared memory.
//
// The arithmetic is the reference's _lax_wendroff_step_numba
// (solver_numba.py:130-213) with the broadcast of the deposition
// (solver_numba_parallel.py:222-277) fused in, and state.py:113-176 for the
// ring columns, which the interior column next to them writes: reflecting
// copies the new interior value (corners take the diagonal interior column),
// absorbing carries the ring's own input plus this step's deposition.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_async.cuh"
#include "pic_device.cuh"

namespace pic {

// One grid's arguments of a streaming step (the single-grid kernel takes it
// as its parameter; the batched kernel builds one per grid and stages the
// current item's in shared memory).
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

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }

__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }

// Floats of one ring stage: both species' (tj + 2) rows of kp, then the
// plane's deposition pairs over a 32-byte-aligned cover of those rows.
__host__ __device__ __forceinline__ int stream_stage_floats(int tj, int kp) {
    return 2 * (tj + 2) * kp + 2 * ((tj + 8) & ~3);
}

// The producer's copies of one plane `pl` of an item with rows
// [cj_lo - 1, cj_hi] into ring stage `dst`: both species, then the pairs of
// the plane's 32-byte-aligned cover of those rows. Completes on `bar`.
__device__ __forceinline__ void stream_issue_plane(const StreamArgs &a, int pl, int cj_lo, int cj_hi, float *dst,
                                                   uint64_t *bar) {
    const int rows = cj_hi - cj_lo + 2;
    const uint32_t bytes = (uint32_t)(rows * a.kp * 4);
    const int doff = (cj_lo - 1) & 3;
    const bool has_dens = a.dens != nullptr;
    const uint32_t dbytes = has_dens ? (uint32_t)(((doff + rows + 3) & ~3) * 8) : 0u;
    const int spec = (a.tj + 2) * a.kp;
    const size_t src = ((size_t)pl * a.n + (cj_lo - 1)) * a.kp;
    mbar_arrive_expect_tx(bar, 2 * bytes + dbytes);
    bulk_g2s(dst, a.pos_in + src, bytes, bar);
    bulk_g2s(dst + spec, a.neg_in + src, bytes, bar);
    if (has_dens) bulk_g2s(dst + 2 * spec, a.dens + (size_t)pl * a.dp + (cj_lo - 1 - doff), dbytes, bar);
}

// Per-grid constants of the consumers, formed once per grid (the single-grid
// kernel forms them once per launch, outside its item loop).
struct StreamConsts {
    int spec, dens_off, c_lo, c_hi, ncore, nedge;
    bool has_dens, gap_below, gap_above;
    int64_t plane_stride;
    float2 ZMp, ZPp, LATp, CENp, ZMn, ZPn, LATn, CENn, ADT;
};

__device__ __forceinline__ StreamConsts stream_consts(const StreamArgs &a) {
    StreamConsts k;
    k.spec = (a.tj + 2) * a.kp;  // floats per species in a stage
    k.dens_off = 2 * k.spec;     // the plane's deposition pairs (float offset)
    k.has_dens = a.dens != nullptr;
    k.c_lo = (a.nze + 3) / 4;    // core vectors: [c_lo, c_hi)
    k.c_hi = a.gap_end / 4;
    k.ncore = k.c_hi > k.c_lo ? k.c_hi - k.c_lo : 0;
    k.nedge = a.c4 - k.ncore;
    k.gap_below = 4 * k.c_lo - 1 >= a.nze;  // element before the first core vector
    k.gap_above = 4 * k.c_hi < a.gap_end;   // element after the last core vector
    k.plane_stride = (int64_t)a.n * a.kp;
    k.ZMp = make_float2(a.p_zm, a.p_zm);
    k.ZPp = make_float2(a.p_zp, a.p_zp);
    k.LATp = make_float2(a.p_lat, a.p_lat);
    k.CENp = make_float2(a.p_cen, a.p_cen);
    k.ZMn = make_float2(a.n_zm, a.n_zm);
    k.ZPn = make_float2(a.n_zp, a.n_zp);
    k.LATn = make_float2(a.n_lat, a.n_lat);
    k.CENn = make_float2(a.n_cen, a.n_cen);
    k.ADT = make_float2(a.alpha_dt, a.alpha_dt);
    return k;
}

// Consumes one work item from the ring: its planes are loads g .. g + nplanes
// - 1 (nplanes = ci_hi - ci_lo + 2) of the ring of S stages of stage_floats
// floats at stage0; writes planes ci_lo .. ci_hi - 1 of the outputs and the
// ring columns next to them, adds the item's scored sums to the tallies, and
// releases every stage (g advances by nplanes). Consumer thread ctid of nct.
// Returns false if a bounded wait ran out (abort_flag is then set and the
// caller leaves).
//
// The k-vectors of a row split into CORE vectors, whose four elements all lie
// in the gap (always valid, always deposited into, scored when the column is),
// and EDGE vectors (the k = 0 plane, the electrode buffers, the z end plane
// and the row padding). Core vectors take a mask-free path in packed FP32x2
// arithmetic; edge vectors the general masked one. Work slot s of a plane is
// core item s (row s / ncore, vector c_lo + s % ncore) for s < n_core, then
// edge items; consumer thread t owns slots t + k * nct, k < IPT, so
// consecutive lanes hold consecutive core vectors of a row (their k-1 / k+4
// neighbours are read from shared memory).
template <int IPT>
__device__ __forceinline__ bool stream_consume_item(const StreamArgs &a, const StreamConsts &K, int cj_lo, int cj_hi,
                                                    int ci_lo, int ci_hi, const float *stage0, int stage_floats,
                                                    uint64_t *full, uint64_t *empty, int S, long long &g,
                                                    volatile int &abort_flag, int ctid, int nct, Tally<float> &t_rec,
                                                    Tally<float> &t_p, Tally<float> &t_n, Tally<float> &t_inj) {
    // Every argument the loops read, in registers: the batched kernel keeps
    // its grid's arguments in shared memory, and the output stores go through
    // generic pointers the compiler cannot prove apart from that copy, so
    // reading them here once keeps them from being reloaded after every store.
    const int n = a.n, kp = a.kp, c4 = a.c4;
    const int A_nze = a.nze, A_gap_end = a.gap_end, A_nzb = a.nzb, A_reflecting = a.reflecting, A_dp = a.dp;
    const int A_two_mid = a.two_mid;
    const uint32_t A_thr4 = a.thr4;
    float *const A_pos_out = a.pos_out;
    float *const A_neg_out = a.neg_out;
    float2 *const A_dens_zero = a.dens_zero;
    int *const A_status = a.status;
    const float A_p_zm = a.p_zm, A_p_zp = a.p_zp, A_p_lat = a.p_lat, A_p_cen = a.p_cen;
    const float A_n_zm = a.n_zm, A_n_zp = a.n_zp, A_n_lat = a.n_lat, A_n_cen = a.n_cen, A_alpha_dt = a.alpha_dt;
    const int lane = ctid & 31;
    const int spec = K.spec, dens_off = K.dens_off;
    const bool has_dens = K.has_dens;
    const int c_lo = K.c_lo, c_hi = K.c_hi, ncore = K.ncore, nedge = K.nedge;
    const bool gap_below = K.gap_below, gap_above = K.gap_above;
    const int64_t plane_stride = K.plane_stride;
    const float2 ZMp = K.ZMp, ZPp = K.ZPp, LATp = K.LATp, CENp = K.CENp;
    const float2 ZMn = K.ZMn, ZPn = K.ZPn, LATn = K.LATn, CENn = K.CENn;
    const float2 ADT = K.ADT, NEG1 = make_float2(-1.f, -1.f);

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
        const int dy = 2 * (cj_lo + r) - A_two_mid;
        dy2[k] = (uint32_t)(dy * dy);
    }
    // ring positions of loads g (plane ci-1), g+1 (ci), g+2 (ci+1),
    // advanced incrementally: slot index and the phase parity to wait on
    int sm_ = (int)(g % S), sc_ = sm_ + 1 == S ? 0 : sm_ + 1, sp_ = sc_ + 1 == S ? 0 : sc_ + 1;
    uint32_t pm_ = (uint32_t)((g / S) & 1), pc_ = sc_ == 0 ? pm_ ^ 1u : pm_, pp_ = sp_ == 0 ? pc_ ^ 1u : pc_;
    if (!mbar_wait(&full[sm_], pm_, A_status, 3) || !mbar_wait(&full[sc_], pc_, A_status, 3)) abort_flag = 1;
    for (int q = 0; q < ci_hi - ci_lo && !abort_flag; ++q) {
        if (!mbar_wait(&full[sp_], pp_, A_status, 3)) {
            abort_flag = 1;
            break;
        }
        const float *Sm = stage0 + (size_t)sm_ * stage_floats;
        const float *Sc = stage0 + (size_t)sc_ * stage_floats;
        const float *Sp = stage0 + (size_t)sp_ * stage_floats;
        const int ci = ci_lo + q;
        const int dx = 2 * ci - A_two_mid;
        const uint32_t dx2 = (uint32_t)(dx * dx);
        const int64_t pbase = (int64_t)ci * plane_stride;
        float *const pos_plane = A_pos_out + pbase;  // outputs of this plane; items add a 32-bit offset
        float *const neg_plane = A_neg_out + pbase;
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
            const bool scored = (dx2 + dy2[k] <= A_thr4);
            float4 PO, NO;
            if (kd == 1) {
                // ---- core vector: mask-free, packed FP32x2 ----
                // k-1 / k+4 neighbours from shared memory (+ their deposition
                // when they lie in the gap): uniform across the warp, where
                // shuffles needed a divergent fallback at the warp's and the
                // core's ends (measured 1.255 -> 1.201 ms a full-electrode step)
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
                    gk[e] = (kk >= A_nze && kk < A_gap_end) ? 1.f : 0.f;
                    valid[e] = kk >= 1 && kk <= A_nzb - 2;
                }
                P.x = fmaf(gk[0], dcen, P.x); P.y = fmaf(gk[1], dcen, P.y);
                P.z = fmaf(gk[2], dcen, P.z); P.w = fmaf(gk[3], dcen, P.w);
                N.x = fmaf(gk[0], dcen, N.x); N.y = fmaf(gk[1], dcen, N.y);
                N.z = fmaf(gk[2], dcen, N.z); N.w = fmaf(gk[3], dcen, N.w);
                const bool g_km = (k0 - 1 >= A_nze && k0 - 1 < A_gap_end);
                const bool g_kp = (k0 + 4 >= A_nze && k0 + 4 < A_gap_end);
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
                    const float p_new = A_p_zm * pv[e] + A_p_zp * pv[e + 2] + A_p_lat * pl4[e] + A_p_cen * p;
                    const float n_new = A_n_zm * nv[e + 2] + A_n_zp * nv[e] + A_n_lat * nl4[e] + A_n_cen * nn;
                    const float rec = A_alpha_dt * p * nn;
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
                    if (A_dens_zero) A_dens_zero[(int64_t)ci * A_dp + cj] = make_float2(0.f, 0.f);
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
                    if (A_reflecting) {
                        st4(A_pos_out + rcol * kp + k0, PO);
                        st4(A_neg_out + rcol * kp + k0, NO);
                    } else {
                        float4 RP = lds4(Sr + row * kp + k0), RN = lds4(Sr + spec + row * kp + k0);
                        const float d = has_dens ? reinterpret_cast<const float2 *>(Sr + dens_off)[dq + row].x : 0.f;
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const int kk = k0 + e;
                            const float de = (kk >= A_nze && kk < A_gap_end) ? d : 0.f;
                            (&RP.x)[e] += de;
                            (&RN.x)[e] += de;
                        }
                        st4(A_pos_out + rcol * kp + k0, RP);
                        st4(A_neg_out + rcol * kp + k0, RN);
                    }
                    if (c == 0 && A_dens_zero) A_dens_zero[(int64_t)ri * A_dp + rj] = make_float2(0.f, 0.f);
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
    if (abort_flag) return false;
    __syncwarp();
    if (lane == 0) {
        mbar_arrive(&empty[(g + nplanes - 2) % S]);
        mbar_arrive(&empty[(g + nplanes - 1) % S]);
    }
    g += nplanes;
    return true;
}

}  // namespace pic
