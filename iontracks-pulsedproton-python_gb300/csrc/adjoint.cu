// adjoint.cu -- reverse-mode derivative of the recombined charge through the
// fused time step, and the two segment runners the checkpointed sweep uses.
//
// The forward step (step.cu; the reference's _lax_wendroff_step_numba,
// solver_numba.py:130-213, with the deposition broadcast fused in) maps the
// pre-step state u~ = u_s + deposition_s to u_{s+1}:
//   interior column, 1 <= k <= nzb-2:
//     P'[v] = zm+ p~[v-z] + zp+ p~[v+z] + lat+ sum_lat p~ + cen+ p~[v] - a p~[v] n~[v]
//     N'[v] = zm- n~[v+z] + zp- n~[v-z] + lat- sum_lat n~ + cen- n~[v] - a p~[v] n~[v]
//   z end planes and row padding: 0;
//   outer ring, absorbing: the ring's own u~ (carried);
//   outer ring, reflecting: the new value of the nearest interior column.
// and scores R_s = a * sum over the scored set of p~ n~ (a = alpha * dt).
//
// Given lambda_{s+1} = dR/du_{s+1} (R = total recombined charge of the run),
// one adjoint step forms lambda_s = dR/du_s and the step's contribution to
// dR/ds+, dR/dc+, dR/ds-, dR/dc-, dR/da, where s = D dt/h^2 and c = mu E dt/h
// are the diffusion and Courant numbers the weights are made of
// (lat = s, zm = s + c(c+1)/2, zp = s + c(c-1)/2, cen = 1 - c^2 - 6s). With
// mu = lambda_{s+1} on interior columns and valid k (zero elsewhere; a
// reflecting ring's lambda is first folded into the interior column it
// copies):
//   lambda+_s[w] = zm+ mu+[w+z] + zp+ mu+[w-z] + lat+ sum_lat mu+ + cen+ mu+[w]
//                  - a n~[w] (mu+[w] + mu-[w]) + [w scored] a n~[w]
//   lambda-_s[w] = zm- mu-[w-z] + zp- mu-[w+z] + lat- sum_lat mu- + cen- mu-[w]
//                  - a p~[w] (mu+[w] + mu-[w]) + [w scored] a p~[w]
//   (+ lambda_{s+1}[w] on an absorbing ring),
//   dR/ds+ += mu+[v] lap p~[v]   (the 7-point Laplacian: sum of the six
//             neighbours - 6 p~[v]),
//   dR/dc+ += mu+[v] ((p~[v-z] - p~[v+z]) / 2 + c+ (p~[v-z] + p~[v+z] - 2 p~[v])),
//   the same for the negative species with its z-swapped neighbours, and
//   dR/da += [v scored] p~ n~ - (mu+[v] + mu-[v]) p~ n~.
// The differences are formed per voxel before the products are summed: the
// per-weight sums they combine are large and nearly equal, and subtracting
// them after summation would cancel most of the float32 digits. The
// deposition is a constant of every step: it enters only through u~.
//
// lambda_s is written as zero on the z end planes (k = 0, nzb-1) and the row
// padding: u there is fixed at zero whatever the parameters, so its adjoint
// never enters a derivative (the stencil reads mu there as zero). Every
// adjoint step keeps the convention; lambda_{n_steps} = 0 starts it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "pic_adjoint.cuh"
#include "pic_device.cuh"
#include "pic_flat.cuh"
#include "pic_internal.h"

namespace pic {

template <typename T>
struct AdjArgs {
    const T *pos, *neg;   // u_s
    const pair_t<T> *dens;  // deposition pairs of step s (null: none)
    const T *lp, *ln;     // lambda_{s+1}
    T *lp_out, *ln_out;   // lambda_s
    double *grad;         // [kAdjGrad] of this step
    double *partials;     // [blocks][kAdjGrad] 8-byte slots
    unsigned int *counter;
    int accumulate;       // 1: add the block's sums into its slots (no per-step total)
    int64_t n, kp, c4, items, dp;
    int nzb, nze, gap_end, reflecting;
    T p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, a, gfac;
    T c_pos, c_neg;  // Courant numbers (zm - zp of each species)
    ScoreTest score;
    FastDiv div_c4, div_n;  // item -> column -> (i, j) on the 32-bit path
};

template <typename I>
__device__ __forceinline__ bool interior_col(I i, I j, I n) {
    return i >= 1 && j >= 1 && i <= n - 2 && j <= n - 2;
}

template <int BLOCK, typename A>
__device__ __forceinline__ void block_sum_n(A (&v)[kAdjGrad], A (*smem)[kAdjGrad]) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) v[q] = warp_sum(v[q]);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) smem[warp][q] = v[q];
    __syncthreads();
    if (warp == 0)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) v[q] = warp_sum(lane < BLOCK / 32 ? smem[lane][q] : A{});
    __syncthreads();
}

// u~ (with this step's deposition on gap layers) of four k at column offset
template <typename T, typename I>
__device__ __forceinline__ V4<T> state4(const T *f, I off, T d, const bool (&g)[4]) {
    V4<T> v = load4(f + off);
#pragma unroll
    for (int e = 0; e < 4; ++e) v.v[e] += g[e] ? d : T(0);
    return v;
}

template <typename T, int BLOCK, typename I>
__global__ void __launch_bounds__(BLOCK) adjoint_step_kernel(AdjArgs<T> a) {
    using R = typename AdjRed<T>::type;
    __shared__ R red[BLOCK / 32][kAdjGrad];
    __shared__ bool last;
    Tally<T> acc[kAdjGrad];
    const I n = (I)a.n, kp = (I)a.kp, c4 = (I)a.c4, dp = (I)a.dp, items = (I)a.items;
    const I stride = (I)gridDim.x * BLOCK;
    for (I item = (I)blockIdx.x * BLOCK + threadIdx.x; item < items; item += stride) {
        I col, i;
        if constexpr (sizeof(I) == 4) {
            col = fast_div(item, a.div_c4);
            i = fast_div(col, a.div_n);
        } else {
            col = item / c4;
            i = col / n;
        }
        const int c = (int)(item - col * c4);
        const I j = col - i * n;
        const int k0 = 4 * c;
        const I off = col * kp + k0;
        bool g[4], valid[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            g[e] = (k0 + e >= a.nze) && (k0 + e < a.gap_end);
            valid[e] = (k0 + e >= 1) && (k0 + e <= a.nzb - 2);
        }
        const bool interior = interior_col(i, j, n);
        const bool scored = interior && scored_col_t<I>(a.score, i, j);
        const pair_t<T> dpr = a.dens ? a.dens[i * dp + j] : pair_t<T>{T(0), T(0)};
        const T dc = dpr.x, dl = dpr.y;  // this column's deposition, its neighbours' sum

        // mu of this column (zero off the interior and on invalid k), with
        // its k-1 / k+4 neighbours
        auto mu4 = [&](const T *lam, I ci, I cj, I o) {
            V4<T> m;
            if (interior_col(ci, cj, n)) {
                m = load4(lam + o);
#pragma unroll
                for (int e = 0; e < 4; ++e) m.v[e] = valid[e] ? m.v[e] : T(0);
            } else {
#pragma unroll
                for (int e = 0; e < 4; ++e) m.v[e] = T(0);
            }
            return m;
        };
        auto mu1 = [&](const T *lam, int k) {
            return (interior && k >= 1 && k <= a.nzb - 2) ? lam[col * kp + k] : T(0);
        };
        const V4<T> MP = mu4(a.lp, i, j, off), MN = mu4(a.ln, i, j, off);
        const T mp_km = mu1(a.lp, k0 - 1), mp_kp = mu1(a.lp, k0 + 4);
        const T mn_km = mu1(a.ln, k0 - 1), mn_kp = mu1(a.ln, k0 + 4);
        // lateral sums of mu (neighbour columns; zero off the interior)
        V4<T> LP, LN;
#pragma unroll
        for (int e = 0; e < 4; ++e) LP.v[e] = LN.v[e] = T(0);
        {
            const I nb[4][2] = {{i - 1, j}, {i + 1, j}, {i, j - 1}, {i, j + 1}};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const I ni = nb[q][0], nj = nb[q][1];
                if (ni < n && nj < n) {  // unsigned wrap makes -1 large
                    const I o = (ni * n + nj) * kp + k0;
                    const V4<T> A = mu4(a.lp, ni, nj, o), B = mu4(a.ln, ni, nj, o);
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        LP.v[e] += A.v[e];
                        LN.v[e] += B.v[e];
                    }
                }
            }
        }
        // centre state u~
        const V4<T> P = state4(a.pos, off, dc, g), N = state4(a.neg, off, dc, g);
        V4<T> OP, ON;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const T mp = MP.v[e], mn = MN.v[e];
            const T mp_up = e < 3 ? MP.v[e + 1] : mp_kp, mp_dn = e > 0 ? MP.v[e - 1] : mp_km;
            const T mn_up = e < 3 ? MN.v[e + 1] : mn_kp, mn_dn = e > 0 ? MN.v[e - 1] : mn_km;
            const T msum = mp + mn;
            const bool sc = scored && g[e];
            T lp = a.p_zm * mp_up + a.p_zp * mp_dn + a.p_lat * LP.v[e] + a.p_cen * mp - a.a * N.v[e] * msum;
            T ln = a.n_zm * mn_dn + a.n_zp * mn_up + a.n_lat * LN.v[e] + a.n_cen * mn - a.a * P.v[e] * msum;
            if (sc) {
                lp += a.a * N.v[e];
                ln += a.a * P.v[e];
            }
            // zero on the end planes and the padding (see the header)
            OP.v[e] = valid[e] ? lp : T(0);
            ON.v[e] = valid[e] ? ln : T(0);
        }
        if (!interior && !a.reflecting) {  // absorbing ring: identity carry
            const V4<T> RP = load4(a.lp + off), RN = load4(a.ln + off);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                OP.v[e] += valid[e] ? RP.v[e] : T(0);
                ON.v[e] += valid[e] ? RN.v[e] : T(0);
            }
        }
        store4(a.lp_out + off, OP);
        store4(a.ln_out + off, ON);

        // coefficient gradients of the outputs of this item (interior only)
        if (interior) {
            T pkm = k0 >= 1 ? a.pos[off - 1] + ((k0 - 1 >= a.nze && k0 - 1 < a.gap_end) ? dc : T(0)) : T(0);
            T nkm = k0 >= 1 ? a.neg[off - 1] + ((k0 - 1 >= a.nze && k0 - 1 < a.gap_end) ? dc : T(0)) : T(0);
            T pkp = k0 + 4 < kp ? a.pos[off + 4] + ((k0 + 4 >= a.nze && k0 + 4 < a.gap_end) ? dc : T(0)) : T(0);
            T nkp = k0 + 4 < kp ? a.neg[off + 4] + ((k0 + 4 >= a.nze && k0 + 4 < a.gap_end) ? dc : T(0)) : T(0);
            V4<T> SP, SN;
#pragma unroll
            for (int e = 0; e < 4; ++e) SP.v[e] = SN.v[e] = T(0);
            const I di = n * kp;
            const I nbo[4] = {off - di, off + di, off - kp, off + kp};
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const V4<T> A = load4(a.pos + nbo[q]), B = load4(a.neg + nbo[q]);
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    SP.v[e] += A.v[e];
                    SN.v[e] += B.v[e];
                }
            }
#pragma unroll
            for (int e = 0; e < 4; ++e) {  // the neighbours' deposition, summed
                SP.v[e] += g[e] ? dl : T(0);
                SN.v[e] += g[e] ? dl : T(0);
            }
            T gs[kAdjGrad];
#pragma unroll
            for (int q = 0; q < kAdjGrad; ++q) gs[q] = T(0);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const T mp = MP.v[e], mn = MN.v[e];  // zero on invalid k
                const T p = P.v[e], nn = N.v[e];
                const T p_dn = e > 0 ? P.v[e - 1] : pkm, p_up = e < 3 ? P.v[e + 1] : pkp;
                const T n_dn = e > 0 ? N.v[e - 1] : nkm, n_up = e < 3 ? N.v[e + 1] : nkp;
                const T pz2 = (p_dn + p_up) - T(2) * p, nz2 = (n_dn + n_up) - T(2) * nn;
                const T plap = (SP.v[e] - T(4) * p) + pz2, nlap = (SN.v[e] - T(4) * nn) + nz2;
                // positive: zm on k-1, zp on k+1; negative: zm on k+1, zp on k-1
                const T pc = T(0.5) * (p_dn - p_up) + a.c_pos * pz2;
                const T nc = T(0.5) * (n_up - n_dn) + a.c_neg * nz2;
                const T pn = p * nn;
                gs[0] += mp * plap;
                gs[1] += mp * pc;
                gs[2] += mn * nlap;
                gs[3] += mn * nc;
                gs[4] += ((scored && g[e]) ? pn : T(0)) - (mp + mn) * pn;
            }
#pragma unroll
            for (int q = 0; q < kAdjGrad; ++q) acc[q].add(gs[q]);
        }
    }
    R v[kAdjGrad];
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) v[q] = adj_of(acc[q]);
    block_sum_n<BLOCK>(v, red);
    if (a.accumulate) {
        // the backward sweep needs only the sum over steps: each block keeps
        // its own running sums (same block, same slot, every step; launches
        // are ordered on the stream), reduced once at the end
        if (threadIdx.x == 0)
#pragma unroll
            for (int q = 0; q < kAdjGrad; ++q) adj_accumulate(a.partials + (int64_t)kAdjGrad * blockIdx.x + q, v[q]);
        return;
    }
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) adj_store(a.partials + (int64_t)kAdjGrad * blockIdx.x + q, v[q]);
        __threadfence();
        last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    R s[kAdjGrad];
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) s[q] = R{};
    for (int b = threadIdx.x; b < (int)gridDim.x; b += BLOCK)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) adj_load_add(s[q], a.partials + (int64_t)kAdjGrad * b + q);
    block_sum_n<BLOCK>(s, red);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) a.grad[q] = adj_value(s[q]);
        *a.counter = 0u;
        __threadfence();
    }
}

// Sum of the accumulated block slots of a backward sweep: grad[q] =
// sum over blocks of slot[b][q], in block order (one block).
template <typename T, int BLOCK>
__global__ void __launch_bounds__(BLOCK) adjoint_collect_kernel(const double *slots, int n_blocks, double *grad) {
    using R = typename AdjRed<T>::type;
    __shared__ R red[BLOCK / 32][kAdjGrad];
    R s[kAdjGrad];
#pragma unroll
    for (int q = 0; q < kAdjGrad; ++q) s[q] = R{};
    for (int b = threadIdx.x; b < n_blocks; b += BLOCK)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) adj_load_add(s[q], slots + (int64_t)kAdjGrad * b + q);
    block_sum_n<BLOCK>(s, red);
    if (threadIdx.x == 0)
#pragma unroll
        for (int q = 0; q < kAdjGrad; ++q) grad[q] = adj_value(s[q]);
}

// Reflecting wall: the ring's output is a copy of the nearest interior
// column's, so its adjoint is added to that column's (corners to the diagonal
// one). One thread per (interior edge column, k-vector); each column gathers
// the ring columns that copy it, so no two threads write the same value.
template <typename T>
__global__ void adjoint_fold_kernel(T *lp, T *ln, int64_t n, int64_t kp, int64_t n_edge) {
    const int64_t c4 = kp / 4;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n_edge * c4) return;
    const int64_t e = t / c4, k0 = 4 * (t - e * c4);
    // distinct interior edge columns: row 1 (all), row n-2 (if n-2 > 1), then
    // columns 1 and n-2 of the rows strictly between
    const int64_t m = n - 2;
    int64_t ci, cj;
    if (e < m) {
        ci = 1; cj = 1 + e;
    } else if (m > 1 && e < 2 * m) {
        ci = m; cj = 1 + (e - m);
    } else {
        const int64_t r = e - (m > 1 ? 2 * m : m);  // rows 2 .. m-1
        const int64_t inner = m > 2 ? m - 2 : 0;
        if (r < inner) {
            ci = 2 + r; cj = 1;
        } else {
            ci = 2 + (r - inner); cj = m;
        }
    }
    int64_t ri[3], rj[3];
    int ni = 0, nj = 0;
    ri[ni++] = ci;
    if (ci == 1) ri[ni++] = 0;
    if (ci == m) ri[ni++] = n - 1;
    rj[nj++] = cj;
    if (cj == 1) rj[nj++] = 0;
    if (cj == m) rj[nj++] = n - 1;
    V4<T> sp = load4(lp + (ci * n + cj) * kp + k0), sn = load4(ln + (ci * n + cj) * kp + k0);
    for (int x = 0; x < ni; ++x)
        for (int y = 0; y < nj; ++y) {
            if (x == 0 && y == 0) continue;
            const int64_t o = (ri[x] * n + rj[y]) * kp + k0;
            const V4<T> A = load4(lp + o), B = load4(ln + o);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                sp.v[q] += A.v[q];
                sn.v[q] += B.v[q];
            }
        }
    store4(lp + (ci * n + cj) * kp + k0, sp);
    store4(ln + (ci * n + cj) * kp + k0, sn);
}

// The adjoint workspace: [counter at 0 | status at 64 | .. 256 | slots].
static int64_t adj_counter_bytes() { return 256; }
static int64_t adj_status_offset() { return 64; }

int adjoint_workspace_bytes(int64_t *bytes) {
    *bytes = adj_counter_bytes() + (int64_t)kMaxStepBlocks * kAdjGrad * 8;
    return PIC_OK;
}

static int64_t adjoint_blocks(const pic_grid *g) {
    const int64_t items = g->no_xy * g->no_xy * (g->kpitch / 4);
    int64_t blocks = (items + 255) / 256;
    const int64_t cap = step_grid_cap(g->dtype == PIC_F64 ? 1 : 0);
    if (blocks > cap) blocks = cap;
    if (blocks > kMaxStepBlocks) blocks = kMaxStepBlocks;
    return blocks;
}

template <typename T>
static int launch_adjoint_t(const pic_grid *g, const void *pos, const void *neg, const void *dens, void *lp_in,
                            void *ln_in, void *lp_out, void *ln_out, double *grad, void *ws, cudaStream_t st,
                            bool accumulate) {
    constexpr int BLOCK = 256;
    const int64_t n = g->no_xy, kp = g->kpitch;
    if (g->wall == PIC_WALL_REFLECTING && n >= 3) {
        const int64_t m = n - 2;
        const int64_t n_edge = m + (m > 1 ? m : 0) + (m > 2 ? 2 * (m - 2) : 0);
        const int64_t threads = n_edge * (kp / 4);
        adjoint_fold_kernel<T><<<(unsigned)((threads + 255) / 256), 256, 0, st>>>((T *)lp_in, (T *)ln_in, n, kp,
                                                                                 n_edge);
        int rc = check_launch("adjoint_fold_kernel");
        if (rc) return rc;
    }
    if (sizeof(T) == 4 && adjoint_stream_eligible(g)) {
        char *w = static_cast<char *>(ws);
        return launch_adjoint_stream(g, pos, neg, dens, lp_in, ln_in, lp_out, ln_out, grad,
                                     reinterpret_cast<unsigned int *>(w), reinterpret_cast<int *>(w + adj_status_offset()),
                                     reinterpret_cast<double *>(w + adj_counter_bytes()), adjoint_blocks(g), st,
                                     accumulate);
    }
    AdjArgs<T> a;
    a.pos = (const T *)pos;
    a.neg = (const T *)neg;
    a.dens = (const pair_t<T> *)dens;
    a.lp = (const T *)lp_in;
    a.ln = (const T *)ln_in;
    a.lp_out = (T *)lp_out;
    a.ln_out = (T *)ln_out;
    a.grad = grad;
    a.accumulate = accumulate ? 1 : 0;
    a.counter = reinterpret_cast<unsigned int *>(ws);
    a.partials = reinterpret_cast<double *>(static_cast<char *>(ws) + adj_counter_bytes());
    a.n = n;
    a.kp = kp;
    a.c4 = kp / 4;
    a.items = n * n * (kp / 4);
    a.dp = dens_pitch(n);
    a.nzb = (int)g->nzb;
    a.nze = (int)g->nze;
    a.gap_end = (int)(g->nze + g->no_z);
    a.reflecting = g->wall == PIC_WALL_REFLECTING;
    a.p_lat = (T)g->p_lat; a.p_zm = (T)g->p_zm; a.p_zp = (T)g->p_zp;
    a.p_cen = centre_weight<T>(g->p_lat, g->p_zm, g->p_zp, g->p_cen);
    a.n_lat = (T)g->n_lat; a.n_zm = (T)g->n_zm; a.n_zp = (T)g->n_zp;
    a.n_cen = centre_weight<T>(g->n_lat, g->n_zm, g->n_zp, g->n_cen);
    a.a = (T)g->alpha_dt;
    a.gfac = (T)g->gaussian_factor;
    a.c_pos = (T)(g->p_zm - g->p_zp);
    a.c_neg = (T)(g->n_zm - g->n_zp);
    a.div_c4 = make_fastdiv(a.c4);
    a.div_n = make_fastdiv(a.n);
    int rc = score_test(g, &a.score);
    if (rc) return rc;
    const int64_t blocks = adjoint_blocks(g);
    if (flat_index32(n, kp))
        adjoint_step_kernel<T, BLOCK, uint32_t><<<(unsigned)blocks, BLOCK, 0, st>>>(a);
    else
        adjoint_step_kernel<T, BLOCK, int64_t><<<(unsigned)blocks, BLOCK, 0, st>>>(a);
    return check_launch("adjoint_step_kernel");
}

int launch_adjoint(const pic_grid *g, const void *pos, const void *neg, const void *dens, void *lp_in, void *ln_in,
                   void *lp_out, void *ln_out, double *grad, void *ws, cudaStream_t st, bool accumulate) {
    if (g->dtype == PIC_F64)
        return launch_adjoint_t<double>(g, pos, neg, dens, lp_in, ln_in, lp_out, ln_out, grad, ws, st, accumulate);
    return launch_adjoint_t<float>(g, pos, neg, dens, lp_in, ln_in, lp_out, ln_out, grad, ws, st, accumulate);
}

int adjoint_accumulate_begin(const pic_grid *g, void *ws, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(static_cast<char *>(ws) + adj_counter_bytes(), 0,
                                    (size_t)(adjoint_blocks(g) * kAdjGrad * 8), st);
    return e == cudaSuccess ? PIC_OK : set_cuda_error("cudaMemsetAsync(adjoint slots)", e);
}

int adjoint_accumulate_end(const pic_grid *g, void *ws, double *grad, cudaStream_t st) {
    const double *slots = reinterpret_cast<const double *>(static_cast<char *>(ws) + adj_counter_bytes());
    const int nb = (int)adjoint_blocks(g);
    if (g->dtype == PIC_F64)
        adjoint_collect_kernel<double, 256><<<1, 256, 0, st>>>(slots, nb, grad);
    else
        adjoint_collect_kernel<float, 256><<<1, 256, 0, st>>>(slots, nb, grad);
    return check_launch("adjoint_collect_kernel");
}

}  // namespace pic
