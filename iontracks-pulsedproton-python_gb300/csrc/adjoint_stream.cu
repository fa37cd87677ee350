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
constexpr int kAdjStreamWarps = 12;  // consumer warps (8: 2.74 ms, 15: 2.73 ms on the full electrode)
constexpr int kAdjStreamPlanes = 32;  // planes per work item
constexpr int kAdjStreamMaxIpt = 4;
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
        long long g = 0;
        for (int w = blockIdx.x; w < a.n_items; w += gridDim.x) {
            const int u = w / a.jt, t = w - u * a.jt;
            const int cj_lo = 1 + t * a.tj, cj_hi = min(cj_lo + a.tj, a.n - 1);
            const int ci_lo = 1 + u * a.li, ci_hi = min(ci_lo + a.li, a.n - 1);
            const int nplanes = ci_hi - ci_lo + 2;
            const int n_all = (cj_hi - cj_lo) * c4;
            const int dq = (cj_lo - 1) & 3;  // pair of staged row q: dq + q
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
#pragma unroll
                for (int kk = 0; kk < IPT; ++kk) {
                    const int sl = ctid + kk * nct;
                    if (sl >= n_all) break;
                    const int r = sl / c4, c = sl - r * c4;
                    const int rs = r + 1;  // staged row of this column
                    const int cj = cj_lo + r;
                    const int k0 = 4 * c;
                    const int o = rs * kp + k0;
                    bool g4[4], valid[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        g4[e] = (k0 + e >= a.nze) && (k0 + e < a.gap_end);
                        valid[e] = (k0 + e >= 1) && (k0 + e <= a.nzb - 2);
                    }
                    const int dy = 2 * cj - a.two_mid;
                    const bool scored = dx2 + (uint32_t)(dy * dy) <= a.thr4;
                    const float2 dpr = has_dens ? reinterpret_cast<const float2 *>(Sc + dens_off)[dq + rs]
                                                : make_float2(0.f, 0.f);
                    const float dc = dpr.x, dl = dpr.y;
                    const bool jm_in = cj - 1 >= 1, jp_in = cj + 1 <= n - 2;

                    // mu = lambda_{s+1} on interior columns and valid k
                    auto mu4 = [&](const float *p, bool in) {
                        float4 m = in ? lds4(p) : make_float4(0.f, 0.f, 0.f, 0.f);
                        m.x = valid[0] ? m.x : 0.f;
                        m.y = valid[1] ? m.y : 0.f;
                        m.z = valid[2] ? m.z : 0.f;
                        m.w = valid[3] ? m.w : 0.f;
                        return m;
                    };
                    const float4 MP = mu4(Sc + o, true), MN = mu4(Sc + spec + o, true);
                    const bool km_ok = k0 - 1 >= 1, kp_ok = k0 + 4 <= a.nzb - 2;
                    const float mp_km = km_ok ? Sc[o - 1] : 0.f, mp_kp = kp_ok ? Sc[o + 4] : 0.f;
                    const float mn_km = km_ok ? Sc[spec + o - 1] : 0.f, mn_kp = kp_ok ? Sc[spec + o + 4] : 0.f;
                    // lateral sums of mu, in the order i-1, i+1, j-1, j+1
                    float4 LP, LN;
                    {
                        const float4 A0 = mu4(Sm + o, im_in), B0 = mu4(Sm + spec + o, im_in);
                        const float4 A1 = mu4(Sp + o, ip_in), B1 = mu4(Sp + spec + o, ip_in);
                        const float4 A2 = mu4(Sc + o - kp, jm_in), B2 = mu4(Sc + spec + o - kp, jm_in);
                        const float4 A3 = mu4(Sc + o + kp, jp_in), B3 = mu4(Sc + spec + o + kp, jp_in);
                        LP.x = ((0.f + A0.x) + A1.x + A2.x) + A3.x; LN.x = ((0.f + B0.x) + B1.x + B2.x) + B3.x;
                        LP.y = ((0.f + A0.y) + A1.y + A2.y) + A3.y; LN.y = ((0.f + B0.y) + B1.y + B2.y) + B3.y;
                        LP.z = ((0.f + A0.z) + A1.z + A2.z) + A3.z; LN.z = ((0.f + B0.z) + B1.z + B2.z) + B3.z;
                        LP.w = ((0.f + A0.w) + A1.w + A2.w) + A3.w; LN.w = ((0.f + B0.w) + B1.w + B2.w) + B3.w;
                    }
                    // centre state u~ (this step's deposition on gap layers)
                    float4 P = lds4(Sc + 2 * spec + o), N = lds4(Sc + 3 * spec + o);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        (&P.x)[e] += g4[e] ? dc : 0.f;
                        (&N.x)[e] += g4[e] ? dc : 0.f;
                    }
                    float4 OP, ON;
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float mp = comp(MP, e), mn = comp(MN, e);
                        const float mp_up = e < 3 ? comp(MP, e + 1) : mp_kp, mp_dn = e > 0 ? comp(MP, e - 1) : mp_km;
                        const float mn_up = e < 3 ? comp(MN, e + 1) : mn_kp, mn_dn = e > 0 ? comp(MN, e - 1) : mn_km;
                        const float msum = mp + mn;
                        const bool sc = scored && g4[e];
                        float lp = a.p_zm * mp_up + a.p_zp * mp_dn + a.p_lat * comp(LP, e) + a.p_cen * mp -
                                   a.a * comp(N, e) * msum;
                        float ln = a.n_zm * mn_dn + a.n_zp * mn_up + a.n_lat * comp(LN, e) + a.n_cen * mn -
                                   a.a * comp(P, e) * msum;
                        if (sc) {
                            lp += a.a * comp(N, e);
                            ln += a.a * comp(P, e);
                        }
                        const bool pad = (k0 + e) >= a.nzb;
                        (&OP.x)[e] = pad ? 0.f : lp;
                        (&ON.x)[e] = pad ? 0.f : ln;
                    }
                    const int64_t col = (int64_t)ci * n + cj;
                    st4(a.lp_out + col * kp + k0, OP);
                    st4(a.ln_out + col * kp + k0, ON);

                    // ring columns next to this interior column: (ri, cj),
                    // (ci, rj) get lat * mu + carry; the corner (ri, rj) the carry
                    const bool lo_i = ci == 1, hi_i = ci == n - 2, lo_j = cj == 1, hi_j = cj == n - 2;
                    if (lo_i || hi_i || lo_j || hi_j) {
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
                                    const bool in_k = (k0 + e) < a.nzb;
                                    (&RP.x)[e] = (in_k ? (&RP.x)[e] : 0.f) + (in_k ? comp(CP, e) : 0.f);
                                    (&RN.x)[e] = (in_k ? (&RN.x)[e] : 0.f) + (in_k ? comp(CN, e) : 0.f);
                                }
                            } else {
#pragma unroll
                                for (int e = 0; e < 4; ++e) {
                                    const bool pad = (k0 + e) >= a.nzb;
                                    (&RP.x)[e] = pad ? 0.f : (&RP.x)[e];
                                    (&RN.x)[e] = pad ? 0.f : (&RN.x)[e];
                                }
                            }
                            const int64_t rcol = (int64_t)ri * n + rj;
                            st4(a.lp_out + rcol * kp + k0, RP);
                            st4(a.ln_out + rcol * kp + k0, RN);
                        }
                    }

                    // derivative sums of this column's outputs
                    const float pkm = k0 >= 1 ? Sc[2 * spec + o - 1] + ((k0 - 1 >= a.nze && k0 - 1 < a.gap_end) ? dc : 0.f) : 0.f;
                    const float nkm = k0 >= 1 ? Sc[3 * spec + o - 1] + ((k0 - 1 >= a.nze && k0 - 1 < a.gap_end) ? dc : 0.f) : 0.f;
                    const float pkp = k0 + 4 < kp ? Sc[2 * spec + o + 4] + ((k0 + 4 >= a.nze && k0 + 4 < a.gap_end) ? dc : 0.f) : 0.f;
                    const float nkp = k0 + 4 < kp ? Sc[3 * spec + o + 4] + ((k0 + 4 >= a.nze && k0 + 4 < a.gap_end) ? dc : 0.f) : 0.f;
                    float4 SP, SN;
                    {
                        const float4 A0 = lds4(Sm + 2 * spec + o), B0 = lds4(Sm + 3 * spec + o);
                        const float4 A1 = lds4(Sp + 2 * spec + o), B1 = lds4(Sp + 3 * spec + o);
                        const float4 A2 = lds4(Sc + 2 * spec + o - kp), B2 = lds4(Sc + 3 * spec + o - kp);
                        const float4 A3 = lds4(Sc + 2 * spec + o + kp), B3 = lds4(Sc + 3 * spec + o + kp);
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            (&SP.x)[e] = (((0.f + comp(A0, e)) + comp(A1, e)) + comp(A2, e)) + comp(A3, e);
                            (&SN.x)[e] = (((0.f + comp(B0, e)) + comp(B1, e)) + comp(B2, e)) + comp(B3, e);
                            (&SP.x)[e] += g4[e] ? dl : 0.f;
                            (&SN.x)[e] += g4[e] ? dl : 0.f;
                        }
                    }
                    float gs[kAdjGrad] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const float mp = comp(MP, e), mn = comp(MN, e);
                        const float p = comp(P, e), nn = comp(N, e);
                        const float p_dn = e > 0 ? comp(P, e - 1) : pkm, p_up = e < 3 ? comp(P, e + 1) : pkp;
                        const float n_dn = e > 0 ? comp(N, e - 1) : nkm, n_up = e < 3 ? comp(N, e + 1) : nkp;
                        const float pz2 = (p_dn + p_up) - 2.f * p, nz2 = (n_dn + n_up) - 2.f * nn;
                        const float plap = (comp(SP, e) - 4.f * p) + pz2, nlap = (comp(SN, e) - 4.f * nn) + nz2;
                        const float pc = 0.5f * (p_dn - p_up) + a.c_pos * pz2;
                        const float nc = 0.5f * (n_up - n_dn) + a.c_neg * nz2;
                        const float pn = p * nn;
                        gs[0] += mp * plap;
                        gs[1] += mp * pc;
                        gs[2] += mn * nlap;
                        gs[3] += mn * nc;
                        gs[4] += ((scored && g4[e]) ? pn : 0.f) - (mp + mn) * pn;
                    }
#pragma unroll
                    for (int qq = 0; qq < kAdjGrad; ++qq) acc[qq].add(gs[qq]);
                }
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
    a.li = kAdjStreamPlanes;
    a.jt = (a.n - 2 + a.tj - 1) / a.tj;
    a.n_items = a.jt * ((a.n - 2 + a.li - 1) / a.li);
    a.stages = kAdjStreamStages;
    a.consumer_warps = kAdjStreamWarps;
    a.p_lat = (float)g->p_lat; a.p_zm = (float)g->p_zm; a.p_zp = (float)g->p_zp; a.p_cen = (float)g->p_cen;
    a.n_lat = (float)g->n_lat; a.n_zm = (float)g->n_zm; a.n_zp = (float)g->n_zp; a.n_cen = (float)g->n_cen;
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
