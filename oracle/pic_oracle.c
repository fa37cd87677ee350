/*
 * pic_oracle.c -- FP64 CPU restatement of the reference solver's hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker the GPU kernels are
 * compared against, and the timed CPU baseline of the benchmark. It is never
 * linked into, loaded by or called from the product library.
 *
 * It follows the reference's arithmetic term by term, in the same order, in
 * IEEE float64 with no contraction (build with -ffp-contract=off), so that:
 *   - oracle_insert_track           == _insert_track_numba
 *                                      (pulsed_ion_chamber/solver_numba.py:54-127)
 *   - oracle_lw_step (1 thread)     == _lax_wendroff_step_numba, bit for bit
 *                                      (pulsed_ion_chamber/solver_numba.py:130-213)
 *   - oracle_accumulate_density     == _precompute_track_gaussians + _build_row_index
 *                                      + _accumulate_track_density_numba_parallel
 *                                      (pulsed_ion_chamber/solver_numba_parallel.py:421-457,
 *                                       :140-180, :183-219)
 *   - oracle_broadcast              == _broadcast_density_numba_parallel
 *                                      (pulsed_ion_chamber/solver_numba_parallel.py:222-277)
 *   - oracle_copy_back / oracle_apply_lateral_boundary / oracle_carry_ring
 *                                   == solver_numba.py:345-348 and
 *                                      pulsed_ion_chamber/state.py:113-176
 * With OpenMP the sweep's three sums are formed per thread over contiguous
 * i-blocks and added in thread order: deterministic for a given thread count,
 * and equal to the serial order when one thread is used.
 *
 * Layout: C order [no_xy][no_xy][nzb], k fastest, float64.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IDX(i, j, k) (((int64_t)(i) * no_xy + (j)) * nzb + (k))

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* One track into both species; returns the scored injected charge. */
double oracle_insert_track(double *pos, double *neg, double x, double y, int64_t no_xy, int64_t nzb,
                           int64_t no_z, int64_t nze, double h2, double b2, double gaussian_factor,
                           double mid_xy, double scoring_radius_sq, double cutoff_voxels) {
    int64_t i_lo = (int64_t)ceil(x - cutoff_voxels);
    int64_t i_hi = (int64_t)floor(x + cutoff_voxels) + 1;
    int64_t j_lo = (int64_t)ceil(y - cutoff_voxels);
    int64_t j_hi = (int64_t)floor(y + cutoff_voxels) + 1;
    if (i_lo < 0) i_lo = 0;
    if (j_lo < 0) j_lo = 0;
    if (i_hi > no_xy) i_hi = no_xy;
    if (j_hi > no_xy) j_hi = no_xy;
    if (i_hi <= i_lo || j_hi <= j_lo) return 0.0;
    double *gi = (double *)malloc(sizeof(double) * (size_t)(i_hi - i_lo));
    double *gj = (double *)malloc(sizeof(double) * (size_t)(j_hi - j_lo));
    /* (i - x) ** 2 is evaluated by the reference as a power (libm pow when
     * the kernel runs as plain Python); libm's pow(d, 2.0) can differ from
     * d * d by one ulp, so the same call is made here, through a volatile
     * pointer because compilers fold pow(d, 2.0) into d * d. */
    double (*volatile libm_pow)(double, double) = pow;
    for (int64_t i = i_lo; i < i_hi; ++i) {
        double d = (double)i - x;
        gi[i - i_lo] = exp(-libm_pow(d, 2.0) * h2 / b2);
    }
    for (int64_t j = j_lo; j < j_hi; ++j) {
        double d = (double)j - y;
        gj[j - j_lo] = exp(-libm_pow(d, 2.0) * h2 / b2);
    }
    double inserted = 0.0;
    for (int64_t i = i_lo; i < i_hi; ++i) {
        double di = (double)i - mid_xy;
        double di_sq = di * di;
        double g_i = gi[i - i_lo];
        for (int64_t j = j_lo; j < j_hi; ++j) {
            double dens = gaussian_factor * g_i * gj[j - j_lo];
            double *pp = pos + IDX(i, j, 0);
            double *nn = neg + IDX(i, j, 0);
            for (int64_t k = nze; k < nze + no_z; ++k) {
                pp[k] += dens;
                nn[k] += dens;
            }
            double dj = (double)j - mid_xy;
            if (i >= 1 && i <= no_xy - 2 && j >= 1 && j <= no_xy - 2 && di_sq + dj * dj < scoring_radius_sq)
                inserted += dens * (double)no_z;
        }
    }
    free(gi);
    free(gj);
    return inserted;
}

/* Sum of one step's track Gaussians (dimensionless) into dens[no_xy][no_xy],
 * which the caller zeroes. Per row i, tracks are visited in ascending index
 * order and columns j ascending: the reference's row-index order. */
void oracle_accumulate_density(double *dens, const double *xs, const double *ys, int64_t n_tracks,
                               int64_t no_xy, double h2, double b2, double cutoff_voxels) {
    if (n_tracks <= 0) return;
    int64_t *lo_i = (int64_t *)malloc(sizeof(int64_t) * (size_t)n_tracks * 4);
    int64_t *hi_i = lo_i + n_tracks, *lo_j = hi_i + n_tracks, *hi_j = lo_j + n_tracks;
    const double h2b2 = h2 / b2;
    for (int64_t t = 0; t < n_tracks; ++t) {
        double a = ceil(xs[t] - cutoff_voxels), b = floor(xs[t] + cutoff_voxels) + 1.0;
        double c = ceil(ys[t] - cutoff_voxels), d = floor(ys[t] + cutoff_voxels) + 1.0;
        lo_i[t] = (int64_t)(a > 0.0 ? a : 0.0);
        hi_i[t] = (int64_t)(b < (double)no_xy ? b : (double)no_xy);
        lo_j[t] = (int64_t)(c > 0.0 ? c : 0.0);
        hi_j[t] = (int64_t)(d < (double)no_xy ? d : (double)no_xy);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < no_xy; ++i) {
        double *row = dens + i * no_xy;
        for (int64_t t = 0; t < n_tracks; ++t) {
            if (i < lo_i[t] || i >= hi_i[t]) continue;
            double di = (double)i - xs[t];
            double g_i = exp(-(di * di) * h2b2);
            for (int64_t j = lo_j[t]; j < hi_j[t]; ++j) {
                double dj = (double)j - ys[t];
                row[j] += g_i * exp(-(dj * dj) * h2b2);
            }
        }
    }
    free(lo_i);
}

/* G * dens into every gap layer of both species; returns scored injected. */
double oracle_broadcast(double *pos, double *neg, const double *dens, int64_t no_xy, int64_t nzb,
                        int64_t no_z, int64_t nze, double gaussian_factor, double mid_xy,
                        double scoring_radius_sq) {
    double inserted = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : inserted)
    for (int64_t i = 0; i < no_xy; ++i) {
        for (int64_t j = 0; j < no_xy; ++j) {
            double d = dens[i * no_xy + j];
            if (d == 0.0) continue;
            d *= gaussian_factor;
            double *pp = pos + IDX(i, j, 0);
            double *nn = neg + IDX(i, j, 0);
            for (int64_t k = nze; k < nze + no_z; ++k) {
                pp[k] += d;
                nn[k] += d;
            }
            double di = (double)i - mid_xy, dj = (double)j - mid_xy;
            if (i >= 1 && i <= no_xy - 2 && j >= 1 && j <= no_xy - 2 && di * di + dj * dj < scoring_radius_sq)
                inserted += d * (double)no_z;
        }
    }
    return inserted;
}

/* One Lax-Wendroff step over the interior; out = {recombined, sum p, sum n}. */
void oracle_lw_step(const double *pos, const double *neg, double *pos_next, double *neg_next, int64_t no_xy,
                    int64_t nzb, int64_t nze, int64_t no_z, double mid_xy, double scoring_radius_sq,
                    double p_lat, double p_zm, double p_zp, double p_cen, double n_lat, double n_zm,
                    double n_zp, double n_cen, double alpha_dt, double *out) {
    int nthreads = 1;
#ifdef _OPENMP
    nthreads = omp_get_max_threads();
#endif
    double *part = (double *)calloc((size_t)nthreads * 3, sizeof(double));
#pragma omp parallel num_threads(nthreads)
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double rec = 0.0, tp = 0.0, tn = 0.0;
#pragma omp for schedule(static)
        for (int64_t i = 1; i < no_xy - 1; ++i) {
            double di = (double)i - mid_xy;
            double di_sq = di * di;
            for (int64_t j = 1; j < no_xy - 1; ++j) {
                double dj = (double)j - mid_xy;
                int inside = di_sq + dj * dj < scoring_radius_sq;
                const double *P = pos + IDX(i, j, 0);
                const double *N = neg + IDX(i, j, 0);
                const double *Pjm = pos + IDX(i, j - 1, 0), *Pjp = pos + IDX(i, j + 1, 0);
                const double *Pim = pos + IDX(i - 1, j, 0), *Pip = pos + IDX(i + 1, j, 0);
                const double *Njm = neg + IDX(i, j - 1, 0), *Njp = neg + IDX(i, j + 1, 0);
                const double *Nim = neg + IDX(i - 1, j, 0), *Nip = neg + IDX(i + 1, j, 0);
                double *PO = pos_next + IDX(i, j, 0);
                double *NO = neg_next + IDX(i, j, 0);
                for (int64_t k = 1; k < nzb - 1; ++k) {
                    double p = P[k];
                    double n = N[k];
                    double p_new = p_zm * P[k - 1] + p_zp * P[k + 1] + p_lat * Pjm[k] + p_lat * Pjp[k] +
                                   p_lat * Pim[k] + p_lat * Pip[k] + p_cen * p;
                    double n_new = n_zm * N[k + 1] + n_zp * N[k - 1] + n_lat * Njm[k] + n_lat * Njp[k] +
                                   n_lat * Nim[k] + n_lat * Nip[k] + n_cen * n;
                    double recomb = alpha_dt * p * n;
                    double p_out = p_new - recomb;
                    double n_out = n_new - recomb;
                    PO[k] = p_out;
                    NO[k] = n_out;
                    if (inside && k >= nze && k < no_z + nze) {
                        rec += recomb;
                        tp += p_out;
                        tn += n_out;
                    }
                }
            }
        }
        part[3 * tid + 0] = rec;
        part[3 * tid + 1] = tp;
        part[3 * tid + 2] = tn;
    }
    double rec = 0.0, tp = 0.0, tn = 0.0;
    for (int t = 0; t < nthreads; ++t) {
        rec += part[3 * t + 0];
        tp += part[3 * t + 1];
        tn += part[3 * t + 2];
    }
    free(part);
    out[0] = rec;
    out[1] = tp;
    out[2] = tn;
}

/* cur[1:-1,1:-1,1:-1] = next[1:-1,1:-1,1:-1] */
void oracle_copy_back(double *cur, const double *next, int64_t no_xy, int64_t nzb) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 1; i < no_xy - 1; ++i)
        for (int64_t j = 1; j < no_xy - 1; ++j)
            memcpy(cur + IDX(i, j, 1), next + IDX(i, j, 1), sizeof(double) * (size_t)(nzb - 2));
}

/* Reflecting wall: mirror the four outer planes, i-planes first, then j. */
void oracle_apply_lateral_boundary(double *a, int64_t no_xy, int64_t nzb, int reflecting) {
    if (!reflecting) return;
    const size_t plane = sizeof(double) * (size_t)(no_xy * nzb);
    const size_t row = sizeof(double) * (size_t)nzb;
    memcpy(a + IDX(0, 0, 0), a + IDX(1, 0, 0), plane);
    memcpy(a + IDX(no_xy - 1, 0, 0), a + IDX(no_xy - 2, 0, 0), plane);
    for (int64_t i = 0; i < no_xy; ++i) {
        memcpy(a + IDX(i, 0, 0), a + IDX(i, 1, 0), row);
        memcpy(a + IDX(i, no_xy - 1, 0), a + IDX(i, no_xy - 2, 0), row);
    }
}

/* Absorbing wall across a buffer swap: dst's four outer planes = src's. */
void oracle_carry_ring(double *dst, const double *src, int64_t no_xy, int64_t nzb) {
    const size_t plane = sizeof(double) * (size_t)(no_xy * nzb);
    const size_t row = sizeof(double) * (size_t)nzb;
    memcpy(dst + IDX(0, 0, 0), src + IDX(0, 0, 0), plane);
    memcpy(dst + IDX(no_xy - 1, 0, 0), src + IDX(no_xy - 1, 0, 0), plane);
    for (int64_t i = 0; i < no_xy; ++i) {
        memcpy(dst + IDX(i, 0, 0), src + IDX(i, 0, 0), row);
        memcpy(dst + IDX(i, no_xy - 1, 0), src + IDX(i, no_xy - 1, 0), row);
    }
}
