// sampler.cu -- the rejection step of the track sampler, on the host.
//
// The reference draws track centres uniformly in the sampling disc by
// rejection from consecutive pairs of doubles of its NumPy generator
// (pulsed_ion_chamber/pulses.py:64-82 per track, :84-171 in blocks):
//   x = u[2a] * no_xy,  y = u[2a+1] * no_xy,
//   accepted when (x - mid)^2 + (y - mid)^2 <= radius^2.
// Two forms:
//   * sample_disc scans doubles the caller drew from its generator;
//   * sample_disc_pcg64 draws them itself from the generator's own state when
//     that generator is NumPy's PCG64 (the default_rng the reference seeds):
//     the permuted congruential generator of M. E. O'Neill, "PCG: A Family of
//     Simple Fast Space-Efficient Statistically Good Algorithms for Random
//     Number Generation" (2014), variant XSL-RR 128/64 -- a 128-bit LCG
//     state' = state * M + inc, output rotr64(hi(state') ^ lo(state'),
//     state' >> 122) -- and NumPy's double = (output >> 11) * 2^-53. It draws
//     exactly the doubles the scan consumes and returns the advanced state, so
//     the caller's generator continues from the same point as if it had drawn
//     them.
// Both stop at the wanted count. The arithmetic is the reference's, one
// rounding per operation: this file is compiled with -ffp-contract=off so that
// the sum of squares is never fused into an FMA (which NumPy does not do), on
// either host architecture.
#include <stdint.h>

#include <algorithm>
#include <memory>
#include <thread>
#include <vector>

#include "pic_internal.h"

namespace pic {

int sample_disc(const double *u, int64_t n_pairs, double scale, double mid, double radius_sq, int64_t n_wanted,
                double *xs, double *ys, int64_t *n_accepted, int64_t *n_pairs_used) {
    int64_t got = 0, a = 0;
    for (; a < n_pairs && got < n_wanted; ++a) {
        const double x = u[2 * a] * scale;
        const double y = u[2 * a + 1] * scale;
        const double dx = x - mid, dy = y - mid;
        const double dx2 = dx * dx, dy2 = dy * dy;
        if (dx2 + dy2 <= radius_sq) {
            xs[got] = x;
            ys[got] = y;
            ++got;
        }
    }
    *n_accepted = got;
    *n_pairs_used = a;
    return PIC_OK;
}

namespace {

typedef unsigned __int128 u128;

// PCG's default 128-bit LCG multiplier.
constexpr u128 kPcgMult = ((u128)2549297995355413924ULL << 64) | (u128)4865540595714422341ULL;

struct Pcg64 {
    u128 state, inc;
    inline uint64_t next() {
        state = state * kPcgMult + inc;
        const uint64_t x = (uint64_t)(state >> 64) ^ (uint64_t)state;
        const unsigned rot = (unsigned)(state >> 122);
        return (x >> rot) | (x << ((64u - rot) & 63u));
    }
    inline double next_double() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
};

// The state `delta` steps on: the LCG's map x -> M x + inc composed with
// itself delta times, by squaring (F. B. Brown, "Random number generation
// with arbitrary strides", Trans. Am. Nucl. Soc. 71, 1994): the maps of
// 1, 2, 4, ... steps are (M^k, inc (M^k - 1) / (M - 1)), doubled as
// (A, C) -> (A^2, (A + 1) C), and those of delta's set bits applied in turn.
inline u128 pcg_advance(u128 state, u128 inc, u128 delta) {
    u128 acc_mult = 1, acc_plus = 0, cur_mult = kPcgMult, cur_plus = inc;
    while (delta) {
        if (delta & 1) {
            acc_mult *= cur_mult;
            acc_plus = acc_plus * cur_mult + cur_plus;
        }
        cur_plus = (cur_mult + 1) * cur_plus;
        cur_mult *= cur_mult;
        delta >>= 1;
    }
    return acc_mult * state + acc_plus;
}

}  // namespace

int sample_disc_pcg64(uint64_t *st, double scale, double mid, double radius_sq, int64_t n_wanted, int64_t max_pairs,
                      double *xs, double *ys, int64_t *n_accepted, int64_t *n_draws) {
    Pcg64 r{((u128)st[0] << 64) | st[1], ((u128)st[2] << 64) | st[3]};
    int64_t got = 0, draws = 0;
    // Branch-free accept: every pair is written at the next free slot (in
    // bounds, since got < n_wanted inside the loop) and the slot is kept only
    // when accepted -- about a third of the pairs are rejected, at random.
    while (got < n_wanted && draws < 2 * max_pairs) {
        const double x = r.next_double() * scale;
        const double y = r.next_double() * scale;
        draws += 2;
        const double dx = x - mid, dy = y - mid;
        const double dx2 = dx * dx, dy2 = dy * dy;
        xs[got] = x;
        ys[got] = y;
        got += (dx2 + dy2 <= radius_sq) ? 1 : 0;
    }
    st[0] = (uint64_t)(r.state >> 64);
    st[1] = (uint64_t)r.state;
    *n_accepted = got;
    *n_draws = draws;
    return PIC_OK;
}

// Arrival counts of one pulse (pulsed_ion_chamber/pulses.py:39-61) from a
// PCG64 state: n uniforms u_k drawn as NumPy's random(n) draws them, their
// running sum S_k (left to right, as np.cumsum), arrival a_k = (S_k / S_{n-1})
// * duration (as the in-place divide and multiply), then per bin b the
// count of a_k in [edges[b], edges[b+1]) -- the last bin closed on the right --
// which is what np.histogram counts over explicit edges.
//
// The running sum is one chain of float64 additions in order (its rounding
// is the contract); the rest is not. The draws are split over the host's
// cores, each thread starting from the state advanced to its first draw
// (pcg_advance); the sum then runs once over them in place; and since a_k
// never decreases in k, bin b's count is the distance between the first
// index whose a_k reaches edges[b] and the first reaching edges[b + 1]
// (binary searches). Small pulses take one sequential pass instead.
namespace {

constexpr int64_t kArrivalThreadedMin = (int64_t)1 << 20;

void arrival_counts_serial(Pcg64 start, int64_t n, double duration, const double *edges, int64_t n_edges,
                           int64_t *counts, Pcg64 &end) {
    Pcg64 r = start;
    double last = 0.0;
    for (int64_t k = 0; k < n; ++k) last += r.next_double();
    const int64_t nb = n_edges - 1;
    for (int64_t q = 0; q < nb; ++q) counts[q] = 0;
    r = start;
    double s = 0.0;
    int64_t bin = 0;
    for (int64_t k = 0; k < n; ++k) {
        s += r.next_double();
        const double q = s / last;
        const double t = q * duration;
        if (t < edges[0]) continue;
        while (bin < nb - 1 && t >= edges[bin + 1]) ++bin;
        if (bin < nb - 1 || t <= edges[nb]) ++counts[bin];
    }
    end = r;
}

}  // namespace

int arrival_counts_pcg64(uint64_t *st, int64_t n, double duration, const double *edges, int64_t n_edges,
                         int64_t *counts) {
    const Pcg64 start{((u128)st[0] << 64) | st[1], ((u128)st[2] << 64) | st[3]};
    Pcg64 end = start;
    const int64_t nb = n_edges - 1;
    const unsigned hw = std::thread::hardware_concurrency();
    const int64_t threads = std::min<int64_t>(std::max<unsigned>(hw, 1u), 64);
    if (n < kArrivalThreadedMin || threads < 2) {
        arrival_counts_serial(start, n, duration, edges, n_edges, counts, end);
    } else {
        std::unique_ptr<double[]> S(new double[(size_t)n]);
        double *u = S.get();
        std::vector<std::thread> pool;
        for (int64_t j = 0; j < threads; ++j)
            pool.emplace_back([=] {
                const int64_t k0 = n * j / threads, k1 = n * (j + 1) / threads;
                Pcg64 r{pcg_advance(start.state, start.inc, (u128)k0), start.inc};
                for (int64_t k = k0; k < k1; ++k) u[k] = r.next_double();
            });
        for (auto &t : pool) t.join();
        double s = 0.0;
        for (int64_t k = 0; k < n; ++k) {
            s += u[k];
            u[k] = s;
        }
        const double last = u[n - 1];
        // first index whose arrival reaches e (strict: passes e)
        auto first_at = [&](double e, bool strict) {
            int64_t lo = 0, hi = n;
            while (lo < hi) {
                const int64_t mid = lo + (hi - lo) / 2;
                const double q = u[mid] / last;
                const double t = q * duration;
                if (strict ? t > e : t >= e) hi = mid; else lo = mid + 1;
            }
            return lo;
        };
        int64_t prev = first_at(edges[0], false);
        for (int64_t b = 0; b < nb; ++b) {
            const int64_t next = b + 1 < nb ? first_at(edges[b + 1], false) : first_at(edges[nb], true);
            counts[b] = next > prev ? next - prev : 0;
            prev = next > prev ? next : prev;
        }
        end.state = pcg_advance(start.state, start.inc, (u128)n);
    }
    st[0] = (uint64_t)(end.state >> 64);
    st[1] = (uint64_t)end.state;
    return PIC_OK;
}

}  // namespace pic
