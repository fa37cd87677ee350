// pic_flat.cuh -- the flat form of the fused step: arguments and the
// per-item body, shared by the single-grid kernel (step.cu) and the
// batched multi-grid kernel (batched.cu). See step.cu for the semantics.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "pic_device.cuh"
#include "pic_internal.h"

namespace pic {

template <typename T>
struct StepArgs {
    const T *pos_in, *neg_in;
    T *pos_out, *neg_out;
    const pair_t<T> *dens;  // the step's deposition pairs (null: none)
    pair_t<T> *dens_zero;   // the next step's pairs, cleared here (null: none)
    double *tally;
    double *partials;
    unsigned int *counter;
    int64_t n, kp, c4, items, dp;  // dp: density row pitch
    int nzb, nze, gap_end;  // gap = [nze, gap_end)
    int reflecting;
    T p_lat, p_zm, p_zp, p_cen, n_lat, n_zm, n_zp, n_cen, alpha_dt, gfac;
    ScoreTest score;
    double injected_scale;  // no_z: the pairs carry G already
    FastDiv div_c4, div_n;  // item -> column -> (i, j) on the 32-bit path
};

// One element or one deposition pair: plain, or (COH) from L2 only.
template <bool COH, typename V>
__device__ __forceinline__ V ld1(const V *p) {
    if constexpr (COH) return __ldcg(p);
    else return *p;
}

template <typename T, bool COH = false>
__device__ __forceinline__ T dep_at(const StepArgs<T> &a, int64_t dcol) {
    return a.dens ? ld1<COH>(a.dens + dcol).x : T(0);
}

// Index type of a grid: 32-bit unsigned offsets when every element offset of
// the fields fits (no_xy^2 * kpitch < 2^31) and the scored test fits 32-bit
// arithmetic (no_xy <= 16383) -- every grid up to ~2 G cells; the item
// decode then costs two 32-bit divisions instead of two 64-bit ones.
inline bool flat_index32(int64_t n, int64_t kp) { return n <= 16383 && n * n * kp < ((int64_t)1 << 31); }

template <typename I>
__device__ __forceinline__ bool scored_col_t(const ScoreTest &t, I i, I j) {
    if constexpr (sizeof(I) == 4) {
        // |2i - two_mid| < 2^15 for no_xy <= 16383: the squares fit uint32
        const int dx = 2 * (int)i - (int)t.two_mid, dy = 2 * (int)j - (int)t.two_mid;
        const uint32_t r2 = (uint32_t)(dx * dx) + (uint32_t)(dy * dy);
        return t.thr4 >= 0 && (t.thr4 >= 0xffffffffLL || r2 <= (uint32_t)t.thr4);
    } else {
        return scored_column(t, (int64_t)i, (int64_t)j);
    }
}

// The fused step for one work item: four consecutive k of output column
// (i, j), decoded from the flat item index (k-vector fastest). Adds the
// item's scored contributions to the thread's running tallies. I is the index
// type (uint32_t when flat_index32 holds for the grid, else int64_t). COH:
// plain (coherent) vector loads instead of the read-only path, for a kernel
// that reads fields other blocks wrote earlier in the same launch.
template <typename T, typename I, bool COH = false>
__device__ __forceinline__ void flat_item(const StepArgs<T> &a, I item, Tally<T> &t_rec,
                                          Tally<T> &t_p, Tally<T> &t_n, Tally<T> &t_inj) {
    auto ld4 = [](const T *p) { return COH ? load4c(p) : load4(p); };
    const I n = (I)a.n, kp = (I)a.kp, c4 = (I)a.c4, dp = (I)a.dp;
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
    if (c == 0 && a.dens_zero) a.dens_zero[i * dp + j] = pair_t<T>{T(0), T(0)};

    // gap mask of the four outputs and of the two z-neighbours
    bool g[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) g[e] = (k0 + e >= a.nze) && (k0 + e < a.gap_end);
    const bool g_km = (k0 - 1 >= a.nze) && (k0 - 1 < a.gap_end);
    const bool g_kp = (k0 + 4 >= a.nze) && (k0 + 4 < a.gap_end);

    const I ci = i < 1 ? 1 : (i > n - 2 ? n - 2 : i);
    const I cj = j < 1 ? 1 : (j > n - 2 ? n - 2 : j);
    const bool ring = (ci != i) || (cj != j);
    const I out_off = col * kp + k0;

    if (ring && !a.reflecting) {
        const T d = dep_at<T, COH>(a, (int64_t)(i * dp + j));
        V4<T> P = ld4(a.pos_in + out_off), N = ld4(a.neg_in + out_off);
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            P.v[e] += g[e] ? d : T(0);
            N.v[e] += g[e] ? d : T(0);
        }
        store4(a.pos_out + out_off, P);
        store4(a.neg_out + out_off, N);
        return;
    }

    const I ccol = ci * n + cj;
    const I base = ccol * kp + k0;
    const I di = n * kp;
    V4<T> P = ld4(a.pos_in + base), N = ld4(a.neg_in + base);
    V4<T> Pim = ld4(a.pos_in + base - di), Pip = ld4(a.pos_in + base + di);
    V4<T> Pjm = ld4(a.pos_in + base - kp), Pjp = ld4(a.pos_in + base + kp);
    V4<T> Nim = ld4(a.neg_in + base - di), Nip = ld4(a.neg_in + base + di);
    V4<T> Njm = ld4(a.neg_in + base - kp), Njp = ld4(a.neg_in + base + kp);
    T pkm = c > 0 ? ld1<COH>(a.pos_in + base - 1) : T(0);
    T nkm = c > 0 ? ld1<COH>(a.neg_in + base - 1) : T(0);
    T pkp = k0 + 4 < kp ? ld1<COH>(a.pos_in + base + 4) : T(0);
    T nkp = k0 + 4 < kp ? ld1<COH>(a.neg_in + base + 4) : T(0);

    const I dcol = ci * dp + cj;
    // this column's deposition and its neighbours' (gap layers only): one
    // pair per column
    T dc = T(0), dl = T(0);
    if (a.dens) {
        const pair_t<T> d = ld1<COH>(a.dens + dcol);
        dc = d.x;
        dl = d.y;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            if (g[e]) {
                P.v[e] += dc;
                N.v[e] += dc;
            }
        }
        if (g_km) { pkm += dc; nkm += dc; }
        if (g_kp) { pkp += dc; nkp += dc; }
    }

    const bool scored_col = !ring && scored_col_t<I>(a.score, ci, cj);
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
        const T dle = g[e] ? dl : T(0);
        const T p_new = a.p_zm * p_km1 + a.p_zp * p_kp1 +
                        a.p_lat * (((Pjm.v[e] + Pjp.v[e]) + (Pim.v[e] + Pip.v[e])) + dle) + a.p_cen * p;
        const T n_new = a.n_zm * n_kp1 + a.n_zp * n_km1 +
                        a.n_lat * (((Njm.v[e] + Njp.v[e]) + (Nim.v[e] + Nip.v[e])) + dle) + a.n_cen * nn;
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
        if (c == 0 && a.dens) t_inj.add(dc);
    }
}

}  // namespace pic
