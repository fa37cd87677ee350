// adjoint_stream.cu -- the adjoint step (adjoint.cu states its equations) as
// a 2.5D streaming kernel for large float32 grids.
//
// The adjoint of a voxel reads lambda_{s+1} of both species and the pre-step
// state u~ of both species at the voxel and its six neighbours: four 7-point
// stencils, 24 bytes of compulsory traffic per voxel (read p, n, lambda+,
// lambda-; write lambda+, lambda-). Read through L1/L2 from a flat grid walk
// that is some 26 loads per four-voxel item, in dependent phases, and the
// flat kernel waits on them (31 % of DRAM peak on a 608 x 608 x 406 grid).
// Here, as in the forward streaming kernel (stream.cu), a producer warp
// copies whole (tile rows + j-halo) x k planes of the four arrays and the
// plane's deposition pairs into a shared-memory ring with bulk asynchronous
// copies (cp.async.bulk, completing on mbarriers), and consumer warps march
// along i computing plane ci from the stages of ci-1, ci, ci+1: every stencil
// neighbour comes from shared memory and each array crosses HBM once per step.
//
// Work item: TJ interior rows j = [cj_lo, cj_hi) x LI interior planes
// i = [ci_lo, ci_hi), all k. Outputs: lambda_s of the item's interior
// columns, and of the ring columns next to them -- lat * mu of the interior
// neighbour, plus (absorbing wall) the ring's own lambda_{s+1}; a corner has
// no interior neighbour and keeps only the carry. A reflecting wall's ring
// adjoint is folded into the interior columns first (adjoint_fold_kernel), as
// for the flat kernel. The arithmetic per voxel is the flat kernel's, term
// for term.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_adjoint.cuh"
#include "pic_async.cuh"
#include "pic_device.cuh"
#include "pic_internal.h"

namespace pic {

namespace {

constexpr int kAdjStreamStages = 4;
// consumer warps; full electrode, packed, 32-plane items: 12 warps 2.35 ms,
// 10: 2.42 ms, 15: 2.64 ms; 64-plane items: 12 warps 2.34 ms, 13: 2.60 ms,
// 14: 2.59 ms; with the derivative sums by parts: 11 warps 2.232 ms, 12: 2.244
// ms, 13: 2.451 ms, 14: 2.503 ms; with each slot's values formed once per
// item: 11 warps 2.146 ms, 10: 2.160 ms. Twelve warps in all (eleven and the
// producer) leave each SM sub-partition three warps and so 168 registers a
// thread; thirteen would cap it at 128.
constexpr int kAdjStreamWarps = 11;
// Planes per work item: a longer item restarts the ring (two planes of
// halo) less often -- 64 planes: 2.337 ms per full-electrode step, 32: 2.377
// ms, 96: 2.341 ms, 128: 2.434 ms; on 608 x 608 x 406 (6.6 items of 64
// planes per SM) 0.788 against 0.794 ms -- but leaves fewer items to balance
// over the SMs, so 64 is taken only where every SM still gets
// kAdjStreamMinItems.
constexpr int kAdjStreamPlanes = 64, kAdjStreamPlanesShort = 32, kAdjStreamMinItems = 6;
constexpr int kAdjStreamMaxIpt = 4;
// flags of a consumer slot (bits 0-3: in the gap, 4-7: valid k, 16-23: the
// index of its deposition pair in a stage)
constexpr uint32_t kSlotJm = 1u << 8, kSlotJp = 1u << 9, kSlotKm = 1u << 10, kSlotKp = 1u << 11,
                   kSlotRingJ = 1u << 12, kSlotLive = 1u << 13;
constexpr int kAdjStreamSmemMax = 220 * 1024;

struct AdjStreamArgs {
    const float *lp, *ln;    // lambda_{s+1} (reflecting: folded)
    const float *pos, *neg;  // u_s
    float *lp_out, *ln_out;  // lambda_s
    const float2 *dens;      // deposition pairs of step s (null: none)
    double *grad, *partials;
    unsigned int *counter;
    int *status;
    int accumulate;
    int n, kp, c4, nzb, nze, gap_end, reflecting, dp;
    int tj, li, jt, n_items, stages, consumer_warps;
    float p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, a, c_pos, c_neg;
    int two_mid;
    uint32_t thr4;
};

__device__ __forceinline__ float4 lds4(const float *p) { return *reinterpret_cast<const float4 *>(p); }
__device__ __forceinline__ void st4(float *p, float4 v) { *reinterpret_cast<float4 *>(p) = v; }
__device__ __forceinline__ float comp(const float4 &v, int e) { return (&v.x)[e]; }
__device__ __forceinline__ float2 lo2(const float4 &v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 &v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __fadd2_rn(a, make_float2(-b.x, -b.y)); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

int stage_floats(int tj, int kp) { return 4 * (tj + 2) * kp + 2 * ((tj + 8) & ~3); }

int smem_bytes(int tj, int kp, int stages) {
    return (2 * stages * 8 + 127) / 128 * 128 + stages * stage_floats(tj, kp) * 4;
}

template <int IPT>
__global__ void __launch_bounds__((kAdjStreamWarps + 1) * 32, 1) adjoint_stream_kernel(AdjStreamArgs a) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ volatile int abort_flag;
    __shared__ DF red[32][kAdjGrad];
    __shared__ bool last;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + a.stages;
    const int bar_bytes = (2 * a.stages * 8 + 127) / 128 * 128;
    float *stage0 = reinterpret_cast<float *>(smem_raw + bar_bytes);
    const int spec = (a.tj + 2) * a.kp;  // floats per array in a stage
    const int dens_off = 4 * spec;
    const int sfl = 4 * spec + 2 * ((a.tj + 8) & ~3);
    const bool has_dens = a.dens != nullptr;
    const int S = a.stages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = a.consumer_warps;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], cw);
        }
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();

    Tally<float> acc[kAdjGrad];

    if (warp == cw) {
        // ---- producer: lane 0 copies, per plane, the tile rows (+ j-halo)
        // of lambda+, lambda-, p, n and the plane's deposition pairs
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < a.n_items && ok; w += gridDim.x) {
                const int u = w / a.jt, t = w - u * a.jt;
                const int cj_lo = 1 + t * a.tj, cj_hi = min(cj_lo + a.tj, a.n - 1);
                const int ci_lo = 1 + u * a.li, ci_hi = min(ci_lo + a.li, a.n - 1);
                const int rows = cj_hi - cj_lo + 2;
                const uint32_t bytes = (uint32_t)(rows * a.kp * 4);
                const int doff = (cj_lo - 1) & 3;
                const uint32_t dbytes = has_dens ? (uint32_t)(((doff + rows + 3) & ~3) * 8) : 0u;
                for (int pl = ci_lo - 1; pl <= ci_hi; ++pl, ++g) {
                    const int slot = (int)(g % S);
                    if (g >= S && !mbar_wait(&empty[slot], (uint32_t)(((g / S) - 1) & 1), a.status, 11)) {
                        abort_flag = 1;
                        ok = false;
                        break;
                    }
                    if (abort_flag) {
                        ok = false;
                        break;
                    }
                    float *dst = stage0 + (size_t)slot * sfl;
                    const size_t src = ((size_t)pl * a.n + (cj_lo - 1)) * a.kp;
                    mbar_arrive_expect_tx(&full[slot], 4 * bytes + dbytes);
                    bulk_g2s(dst, a.lp + src, bytes, &full[slot]);
                    bulk_g2s(dst + spec, a.ln + src, bytes, &full[slot]);
                    bulk_g2s(dst + 2 * spec, a.pos + src, bytes, &full[slot]);
                    bulk_g2s(dst + 3 * spec, a.neg + src, bytes, &full[slot]);
                    if (has_dens)
                        bulk_g2s(dst + dens_off, a.dens + (size_t)pl * a.dp + (cj_lo - 1 - doff), dbytes,
                                 &full[slot]);
                }
            }
            if (!ok) {
                // every copy still in flight lands before the block exits
                for (long long gg = g - S < 0 ? 0 : g - S; gg < g; ++gg)
                    mbar_wait(&full[gg % S], (uint32_t)((gg / S) & 1), a.status, 12);
            }
        }
    } else {
        // ---- consumers: thread t owns work slots t + k * nct (k < IPT) of a
        // plane, slot s = row s / c4, k-vector s % c4
        const int ctid = threadIdx.x, nct = cw * 32;
        const int n = a.n, kp = a.kp, c4 = a.c4;
        const float2 PZM = make_float2(a.p_zm, a.p_zm), PZP = make_float2(a.p_zp, a.p_zp);
        const float2 PLT = make_float2(a.p_lat, a.p_lat), PCN = make_float2(a.p_cen, a.p_cen);
        const float2 NZM = make_float2(a.n_zm, a.n_zm), NZP = make_float2(a.n_zp, a.n_zp);
        const float2 NLT = make_float2(a.n_lat, a.n_lat), NCN = make_float2(a.n_cen, a.n_cen);
        const float2 AD = make_float2(a.a, a.a), CPOS = make_float2(a.c_pos, a.c_pos);
        const float2 CNEG = make_float2(a.c_neg, a.c_neg), HALF = make_float2(0.5f, 0.5f);
        const float2 M2 = make_float2(-2.f, -2.f), M6 = make_float2(-6.f, -6.f);
        long long g = 0;
        for (int w = blockIdx.x; w < a.n_items; w += gridDim.x) {
            const int u = w / a.jt, t = w - u * a.jt;
            const int cj_lo = 1 + t * a.tj, cj_hi = min(cj_lo + a.tj, a.n - 1);
            const int ci_lo = 1 + u * a.li, ci_hi = min(ci_lo + a.li, a.n - 1);
            const int nplanes = ci_hi - ci_lo + 2;
            const int n_all = (cj_hi - cj_lo) * c4;
            const int dq = (cj_lo - 1) & 3;  // pair of staged row q: dq + q
            // per slot, fixed over the item's planes: its offset in a stage
            // (staged row rs, k0: rs kp + k0; its output offset within a plane
            // is that plus (cj_lo - 1) kp), dy^2 of the scored test, and flags
            // (k gap / valid bits, lateral and k neighbours present, ring
            // rows, the pair index dq + rs). Formed once per item instead of
            // once per plane: 2.146 against 2.233 ms a full-electrode step.
            int so_[IPT];
            uint32_t dy2_[IPT], fl_[IPT];
            const int64_t oo_base = (int64_t)(cj_lo - 1) * kp;
#pragma unroll
            for (int kk = 0; kk < IPT; ++kk) {
                const int sl = ctid + kk * nct;
                const bool live = sl < n_all;
                const int r = live ? sl / c4 : 0, c = live ? sl - r * c4 : 0;
                const int rs = r + 1;  // staged row of this column
                const int cj = cj_lo + r;
                const int k0 = 4 * c;
                so_[kk] = rs * kp + k0;
                const int dy = 2 * cj - a.two_mid;
                dy2_[kk] = (uint32_t)(dy * dy);
                uint32_t f = live ? kSlotLive : 0u;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    if (k0 + e >= a.nze && k0 + e < a.gap_end) f |= 1u << e;
                    if (k0 + e >= 1 && k0 + e <= a.nzb - 2) f |= 16u << e;
                }
                if (cj - 1 >= 1) f |= kSlotJm;
                if (cj + 1 <= n - 2) f |= kSlotJp;
                if (k0 >= 1) f |= kSlotKm;
                if (k0 + 4 < kp) f |= kSlotKp;
                if (cj == 1 || cj == n - 2) f |= kSlotRingJ;
                fl_[kk] = f | ((uint32_t)(dq + rs) << 16);
            }
            int sm_ = (int)(g % S), sc_ = sm_ + 1 == S ? 0 : sm_ + 1, sp_ = sc_ + 1 == S ? 0 : sc_ + 1;
            uint32_t pm_ = (uint32_t)((g / S) & 1), pc_ = sc_ == 0 ? pm_ ^ 1u : pm_, pp_ = sp_ == 0 ? pc_ ^ 1u : pc_;
            if (!mbar_wait(&full[sm_], pm_, a.status, 13) || !mbar_wait(&full[sc_], pc_, a.status, 13)) abort_flag = 1;
            for (int q = 0; q < ci_hi - ci_lo && !abort_flag; ++q) {
                if (!mbar_wait(&full[sp_], pp_, a.status, 13)) {
                    abort_flag = 1;
                    break;
                }
                const float *Sm = stage0 + (size_t)sm_ * sfl;
                const float *Sc = stage0 + (size_t)sc_ * sfl;
                const float *Sp = stage0 + (size_t)sp_ * sfl;
                const int ci = ci_lo + q;
                const int dx = 2 * ci - a.two_mid;
                const uint32_t dx2 = (uint32_t)(dx * dx);
                const bool im_in = ci - 1 >= 1, ip_in = ci + 1 <= n - 2;  // i-neighbours interior
                float2 G0 = make_float2(0.f, 0.f), G1 = G0, G2 = G0, G3 = G0, G4 = G0;
#pragma unroll
                for (int kk = 0; kk < IPT; ++kk) {
                    const uint32_t fl = fl_[kk];
                    if (!(fl & kSlotLive)) break;
                    const int o = so_[kk];
                    bool g4[4], valid[4], sc[4];
                    const bool scored = dx2 + dy2_[kk] <= a.thr4;
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        g4[e] = (fl >> e) & 1u;
                        valid[e] = (fl >> (4 + e)) & 1u;
                        sc[e] = scored && g4[e];
                    }
                    const float2 dpr = has_dens ? reinterpret_cast<const float2 *>(Sc + dens_off)[fl >> 16]
                                                : make_float2(0.f, 0.f);
                    const float dc = dpr.x, dl = dpr.y;  // this column's deposition, its neighbours' sum
                    const bool jm_in = fl & kSlotJm, jp_in = fl & kSlotJp;

                    // mu = lambda_{s+1}: zero on the end planes and the padding as
                    // every adjoint step writes it; zero on ring columns by the
                    // interior tests of the neighbours. (Carrying planes ci - 1
                    // and ci over from the previous plane in registers instead
                    // measured slower: 2.26-2.32 against 2.16 ms, it spills.)
                    const float4 MP = lds4(Sc + o), MN = lds4(Sc + spec + o);
                    const float mp_km = (fl & kSlotKm) ? Sc[o - 1] : 0.f, mn_km = (fl & kSlotKm) ? Sc[spec + o - 1] : 0.f;
                    const float mp_kp = (fl & kSlotKp) ? Sc[o + 4] : 0.f, mn_kp = (fl & kSlotKp) ? Sc[spec + o + 4] : 0.f;
                    const float4 Z = make_float4(0.f, 0.f, 0.f, 0.f);
                    const float4 A0 = im_in ? lds4(Sm + o) : Z, B0 = im_in ? lds4(Sm + spec + o) : Z;
                    const float4 A1 = ip_in ? lds4(Sp + o) : Z, B1 = ip_in ? lds4(Sp + spec + o) : Z;
                    const float4 A2 = jm_in ? lds4(Sc + o - kp) : Z, B2 = jm_in ? lds4(Sc + spec + o - kp) : Z;
                    const float4 A3 = jp_in ? lds4(Sc + o + kp) : Z, B3 = jp_in ? lds4(Sc + spec + o + kp) : Z;
                    // lateral sums of mu in the order i-1, i+1, j-1, j+1
                    const float2 LPl = add2(add2(add2(lo2(A0), lo2(A1)), lo2(A2)), lo2(A3));
                    const float2 LPh = add2(add2(add2(hi2(A0), hi2(A1)), hi2(A2)), hi2(A3));
                    const float2 LNl = add2(add2(add2(lo2(B0), lo2(B1)), lo2(B2)), lo2(B3));
                    const float2 LNh = add2(add2(add2(hi2(B0), hi2(B1)), hi2(B2)), hi2(B3));
                    // centre state u~ (this step's deposition on gap layers)
                    const float2 DCl = make_float2(g4[0] ? dc : 0.f, g4[1] ? dc : 0.f);
                    const float2 DCh = make_float2(g4[2] ? dc : 0.f, g4[3] ? dc : 0.f);
                    const float4 P0 = lds4(Sc + 2 * spec + o), N0 = lds4(Sc + 3 * spec + o);
                    const float2 Pl = add2(lo2(P0), DCl), Ph = add2(hi2(P0), DCh);
                    const float2 Nl = add2(lo2(N0), DCl), Nh = add2(hi2(N0), DCh);
                    const float2 MPl = lo2(MP), MPh = hi2(MP), MNl = lo2(MN), MNh = hi2(MN);
                    // k+1 / k-1 neighbours of the four elements
                    const float2 mpu_l = make_float2(MP.y, MP.z), mpu_h = make_float2(MP.w, mp_kp);
                    const float2 mpd_l = make_float2(mp_km, MP.x), mpd_h = make_float2(MP.y, MP.z);
                    const float2 mnu_l = make_float2(MN.y, MN.z), mnu_h = make_float2(MN.w, mn_kp);
                    const float2 mnd_l = make_float2(mn_km, MN.x), mnd_h = make_float2(MN.y, MN.z);
                    const float2 Ssl = add2(MPl, MNl), Ssh = add2(MPh, MNh);  // mu+ + mu-
                    const float2 ANl = mul2(AD, Nl), ANh = mul2(AD, Nh), APl = mul2(AD, Pl), APh = mul2(AD, Ph);
                    // lambda+ = zm mu+[k+1] + zp mu+[k-1] + lat L+ + cen mu+ - a n~ (mu+ + mu-)
                    // lambda- = zm mu-[k-1] + zp mu-[k+1] + lat L- + cen mu- - a p~ (mu+ + mu-)
                    float2 lpl = fma2(PCN, MPl, fma2(PLT, LPl, fma2(PZP, mpd_l, mul2(PZM, mpu_l))));
                    float2 lph = fma2(PCN, MPh, fma2(PLT, LPh, fma2(PZP, mpd_h, mul2(PZM, mpu_h))));
                    float2 lnl = fma2(NCN, MNl, fma2(NLT, LNl, fma2(NZP, mnu_l, mul2(NZM, mnd_l))));
                    float2 lnh = fma2(NCN, MNh, fma2(NLT, LNh, fma2(NZP, mnu_h, mul2(NZM, mnd_h))));
                    lpl = fma2(neg2(ANl), Ssl, lpl);
                    lph = fma2(neg2(ANh), Ssh, lph);
                    lnl = fma2(neg2(APl), Ssl, lnl);
                    lnh = fma2(neg2(APh), Ssh, lnh);
                    // scored gap voxels: + a n~ (positive), + a p~ (negative)
                    lpl = add2(lpl, make_float2(sc[0] ? ANl.x : 0.f, sc[1] ? ANl.y : 0.f));
                    lph = add2(lph, make_float2(sc[2] ? ANh.x : 0.f, sc[3] ? ANh.y : 0.f));
                    lnl = add2(lnl, make_float2(sc[0] ? APl.x : 0.f, sc[1] ? APl.y : 0.f));
                    lnh = add2(lnh, make_float2(sc[2] ? APh.x : 0.f, sc[3] ? APh.y : 0.f));
                    // zero on the end planes and the padding
                    const float4 OP = make_float4(valid[0] ? lpl.x : 0.f, valid[1] ? lpl.y : 0.f,
                                                  valid[2] ? lph.x : 0.f, valid[3] ? lph.y : 0.f);
                    const float4 ON = make_float4(valid[0] ? lnl.x : 0.f, valid[1] ? lnl.y : 0.f,
                                                  valid[2] ? lnh.x : 0.f, valid[3] ? lnh.y : 0.f);
                    const int64_t out = (int64_t)ci * n * kp + oo_base + o;
                    st4(a.lp_out + out, OP);
                    st4(a.ln_out + out, ON);

                    // ring columns next to this interior column: (ri, cj),
                    // (ci, rj) get lat * mu + carry; the corner (ri, rj) the carry
                    // (mu and the carry are zero on the end planes and padding)
                    const bool lo_i = ci == 1, hi_i = ci == n - 2;
                    if (lo_i || hi_i || (fl & kSlotRingJ)) {
                        const int rs = (int)(fl >> 16) - dq;  // staged row of this column
                        const int cj = cj_lo - 1 + rs;
                        const int k0 = o - rs * kp;
                        const bool lo_j = cj == 1, hi_j = cj == n - 2;
                        for (int tgt = 0; tgt < 3; ++tgt) {
                            int ri = ci, rj = cj, row = rs;
                            const float *Sr = Sc;
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
                            float4 RP, RN;
                            const float lat_on = tgt < 2 ? 1.f : 0.f;
#pragma unroll
                            for (int e = 0; e < 4; ++e) {
                                (&RP.x)[e] = a.p_lat * (lat_on * comp(MP, e));
                                (&RN.x)[e] = a.n_lat * (lat_on * comp(MN, e));
                            }
                            if (!a.reflecting) {
                                const float4 CP = lds4(Sr + row * kp + k0), CN = lds4(Sr + spec + row * kp + k0);
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    (&RP.x)[e] += comp(CP, e);
                                    (&RN.x)[e] += comp(CN, e);
                                }
                            }
                            const int64_t rcol = (int64_t)ri * n + rj;
                            st4(a.lp_out + rcol * kp + k0, RP);
                            st4(a.ln_out + rcol * kp + k0, RN);
                            if (tgt < 2) {
                                // the ring column's u~ enters the lateral sum of this
                                // interior column: its share of dR/ds (summed by parts
                                // below, the ring columns are no centres of their own)
                                const float4 UP = lds4(Sr + 2 * spec + row * kp + k0);
                                const float4 UN = lds4(Sr + 3 * spec + row * kp + k0);
                                float gp = 0.f, gn = 0.f;
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    gp = fmaf(comp(UP, e), comp(MP, e), gp);
                                    gn = fmaf(comp(UN, e), comp(MN, e), gn);
                                }
                                G0.x += gp;
                                G2.x += gn;
                            }
                        }
                    }

                    // derivative sums, summed by parts: sum_v mu(v) D u(v) =
                    // sum_w u(w) D' mu(w) over the voxels w this column holds,
                    // with D' the transposed difference (the 7-point Laplacian is
                    // its own transpose; the z differences swap their ends). mu
                    // is zero off the interior columns and valid k, u is zero on
                    // the z end planes and padding, so the only terms beyond
                    // these columns' voxels are the ring columns' u in their
                    // interior neighbours' lateral sums, added with the ring
                    // writes above. The lateral neighbours enter as the raw state
                    // plus this column's pair of neighbour deposition (dl), a
                    // local term; the z neighbours and the centre carry their own
                    // column's deposition (u~). Every mu value needed is already
                    // loaded for lambda; no neighbour of the state is read.
                    const float2 DLl = make_float2(g4[0] ? dl : 0.f, g4[1] ? dl : 0.f);
                    const float2 DLh = make_float2(g4[2] ? dl : 0.f, g4[3] ? dl : 0.f);
                    const float2 zsp_l = add2(mpu_l, mpd_l), zsp_h = add2(mpu_h, mpd_h);
                    const float2 zsn_l = add2(mnu_l, mnd_l), zsn_h = add2(mnu_h, mnd_h);
                    // z neighbours and centre of the Laplacian of mu: z sum - 6 mu
                    const float2 plm_l = fma2(M6, MPl, zsp_l), plm_h = fma2(M6, MPh, zsp_h);
                    const float2 nlm_l = fma2(M6, MNl, zsn_l), nlm_h = fma2(M6, MNh, zsn_h);
                    // transposed Courant derivative: c (mu[w+z] + mu[w-z] - 2 mu[w]) plus
                    // (mu[w+z] - mu[w-z]) / 2 (positive) or its negative (negative,
                    // which drifts the other way)
                    const float2 pcm_l = fma2(CPOS, fma2(M2, MPl, zsp_l), mul2(HALF, sub2(mpu_l, mpd_l)));
                    const float2 pcm_h = fma2(CPOS, fma2(M2, MPh, zsp_h), mul2(HALF, sub2(mpu_h, mpd_h)));
                    const float2 ncm_l = fma2(CNEG, fma2(M2, MNl, zsn_l), mul2(HALF, sub2(mnd_l, mnu_l)));
                    const float2 ncm_h = fma2(CNEG, fma2(M2, MNh, zsn_h), mul2(HALF, sub2(mnd_h, mnu_h)));
                    const float2 pnl = mul2(Pl, Nl), pnh = mul2(Ph, Nh);
                    // dR/ds: raw u against the lateral sum of mu (by parts), u~
                    // against its z neighbours and centre, mu against dl (local)
                    G0 = fma2(lo2(P0), LPl, fma2(Pl, plm_l, fma2(MPl, DLl, G0)));
                    G0 = fma2(hi2(P0), LPh, fma2(Ph, plm_h, fma2(MPh, DLh, G0)));
                    G1 = fma2(Ph, pcm_h, fma2(Pl, pcm_l, G1));
                    G2 = fma2(lo2(N0), LNl, fma2(Nl, nlm_l, fma2(MNl, DLl, G2)));
                    G2 = fma2(hi2(N0), LNh, fma2(Nh, nlm_h, fma2(MNh, DLh, G2)));
                    G3 = fma2(Nh, ncm_h, fma2(Nl, ncm_l, G3));
                    G4 = fma2(neg2(Ssh), pnh, fma2(neg2(Ssl), pnl, G4));
                    G4 = add2(G4, make_float2(sc[0] ? pnl.x : 0.f, sc[1] ? pnl.y : 0.f));
                    G4 = add2(G4, make_float2(sc[2] ? pnh.x : 0.f, sc[3] ? pnh.y : 0.f));
                }
                // this plane's sums of the thread's items, into the compensated totals
                acc[0].add(G0.x + G0.y);
                acc[1].add(G1.x + G1.y);
                acc[2].add(G2.x + G2.y);
                acc[3].add(G3.x + G3.y);
                acc[4].add(G4.x + G4.y);
                __syncwarp();
                if (lane == 0) mbar_arrive(&empty[sm_]);
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

    // block sums of the five derivative sums (double-float)
    DF v[kAdjGrad];
    const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) v[q] = warp_sum(df_of(acc[q]));
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) red[warp][q] = v[q];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) v[q] = warp_sum(lane < nw ? red[lane][q] : DF{0.f, 0.f});
    }
    const bool failed = abort_flag != 0;
    if (a.accumulate) {
        // each block keeps its running sums in its own slot; a block whose
        // wait expired poisons its slot, so the sum over the sweep is NaN
        if (threadIdx.x == 0) {
#pragma unroll
            for (int q = 0; q < kAdjGrad; ++q)
                adj_accumulate(a.partials + (int64_t)kAdjGrad * blockIdx.x + q,
                               failed ? DF{__int_as_float(0x7fc00000), 0.f} : v[q]);
        }
        return;
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q)
            adj_store(a.partials + (int64_t)kAdjGrad * blockIdx.x + q,
                      failed ? DF{__int_as_float(0x7fc00000), 0.f} : v[q]);
        __threadfence();
        last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    DF s[kAdjGrad];
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) s[q] = DF{0.f, 0.f};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) adj_load_add(s[q], a.partials + (int64_t)kAdjGrad * b + q);
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) s[q] = warp_sum(s[q]);
    __syncthreads();
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) red[warp][q] = s[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        DF t[kAdjGrad];
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) t[q] = DF{0.f, 0.f};
        for (int w = 0; w < nw; ++w)
#pragma unroll
            for (int q = 0; q < kAdjGrad; ++q) t[q] = df_add(t[q], red[w][q]);
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) a.grad[q] = df_value(t[q]);
        *a.counter = 0u;
        __threadfence();
    }
}

template <int IPT>
int launch_ipt(const AdjStreamArgs &a, unsigned blocks, int smem, cudaStream_t st) {
    static int configured = 0;  // per instantiation: largest dynamic smem set so far
    if (smem > configured) {
        cudaError_t e =
            cudaFuncSetAttribute(adjoint_stream_kernel<IPT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(adjoint_stream_kernel)", e);
        configured = smem;
    }
    adjoint_stream_kernel<IPT><<<blocks, (kAdjStreamWarps + 1) * 32, 0 + smem, st>>>(a);
    return check_launch("adjoint_stream_kernel");
}

// Rows per tile: the most that fit kAdjStreamStages stages and at most
// kAdjStreamMaxIpt k-vectors per consumer thread (0: none fit).
int tile_rows(int n, int kp) {
    const int c4 = kp / 4, nct = kAdjStreamWarps * 32;
    int best = 0;
    for (int tj = 1; tj <= 16 && tj <= n - 2; ++tj) {
        if (smem_bytes(tj, kp, kAdjStreamStages) > kAdjStreamSmemMax) break;
        if ((tj * c4 + nct - 1) / nct > kAdjStreamMaxIpt) break;
        best = tj;
    }
    return best;
}

}  // namespace

bool adjoint_stream_eligible(const pic_grid *g) {
    if (g->dtype != PIC_F32 || g->no_xy < 4 || g->no_xy > 16383) return false;
    if (tile_rows((int)g->no_xy, (int)g->kpitch) < 1) return false;
    if (g->adjoint_variant == PIC_VARIANT_AUTO) return g->no_xy * g->no_xy * g->kpitch >= kAdjStreamMinCells;
    return g->adjoint_variant == PIC_VARIANT_STREAM;
}

int launch_adjoint_stream(const pic_grid *g, const void *pos, const void *neg, const void *dens, const void *lp_in,
                          const void *ln_in, void *lp_out, void *ln_out, double *grad, unsigned int *counter,
                          int *status, double *partials, int64_t max_blocks, cudaStream_t st, bool accumulate) {
    AdjStreamArgs a;
    a.lp = (const float *)lp_in;
    a.ln = (const float *)ln_in;
    a.pos = (const float *)pos;
    a.neg = (const float *)neg;
    a.lp_out = (float *)lp_out;
    a.ln_out = (float *)ln_out;
    a.dens = (const float2 *)dens;
    a.grad = grad;
    a.partials = partials;
    a.counter = counter;
    a.status = status;
    a.accumulate = accumulate ? 1 : 0;
    a.n = (int)g->no_xy;
    a.kp = (int)g->kpitch;
    a.c4 = a.kp / 4;
    a.nzb = (int)g->nzb;
    a.nze = (int)g->nze;
    a.gap_end = (int)(g->nze + g->no_z);
    a.reflecting = g->wall == PIC_WALL_REFLECTING;
    a.dp = (int)dens_pitch(g->no_xy);
    a.tj = tile_rows(a.n, a.kp);
    if (a.tj < 1) return set_error(PIC_E_CAPACITY, "adjoint stream variant: no tile fits shared memory");
    a.jt = (a.n - 2 + a.tj - 1) / a.tj;
    a.li = kAdjStreamPlanes;
    if ((int64_t)a.jt * ((a.n - 2 + a.li - 1) / a.li) < (int64_t)kAdjStreamMinItems * sm_count())
        a.li = kAdjStreamPlanesShort;
    a.n_items = a.jt * ((a.n - 2 + a.li - 1) / a.li);
    a.stages = kAdjStreamStages;
    a.consumer_warps = kAdjStreamWarps;
    a.p_lat = (float)g->p_lat; a.p_zm = (float)g->p_zm; a.p_zp = (float)g->p_zp;
    a.p_cen = centre_weight<float>(g->p_lat, g->p_zm, g->p_zp, g->p_cen);
    a.n_lat = (float)g->n_lat; a.n_zm = (float)g->n_zm; a.n_zp = (float)g->n_zp;
    a.n_cen = centre_weight<float>(g->n_lat, g->n_zm, g->n_zp, g->n_cen);
    a.a = (float)g->alpha_dt;
    a.c_pos = (float)(g->p_zm - g->p_zp);
    a.c_neg = (float)(g->n_zm - g->n_zp);
    ScoreTest sc;
    int rc = score_test(g, &sc);
    if (rc) return rc;
    a.two_mid = (int)sc.two_mid;
    // (2i - two_mid)^2 + (2j - two_mid)^2 < 2^31 for no_xy <= 16383
    a.thr4 = sc.thr4 < 0 ? 0u : (sc.thr4 > 0x7fffffffLL ? 0xffffffffu : (uint32_t)sc.thr4);
    const int smem = smem_bytes(a.tj, a.kp, a.stages);
    int64_t blocks = sm_count();
    if (blocks > a.n_items) blocks = a.n_items;
    if (blocks > max_blocks) blocks = max_blocks;  // one derivative slot per block
    if (blocks < 1) blocks = 1;
    const int ipt = (a.tj * a.c4 + kAdjStreamWarps * 32 - 1) / (kAdjStreamWarps * 32);
    switch (ipt) {
        case 1: return launch_ipt<1>(a, (unsigned)blocks, smem, st);
        case 2: return launch_ipt<2>(a, (unsigned)blocks, smem, st);
        case 3: return launch_ipt<3>(a, (unsigned)blocks, smem, st);
        case 4: return launch_ipt<4>(a, (unsigned)blocks, smem, st);
        default: return set_error(PIC_E_INVALID, "adjoint stream variant: too many k-vectors per thread");
    }
}

}  // namespace pic
