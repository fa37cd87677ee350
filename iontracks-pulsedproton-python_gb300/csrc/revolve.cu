// revolve.cu -- gradients of long runs in bounded memory: binomial
// checkpointing of the fused step and its adjoint, with every recomputed step
// re-depositing its own tracks.
//
// The segment scheme of pic_adjoint_forward / pic_adjoint_backward stores a
// state every K steps, a buffer of K states and the 2D deposition of every
// step with tracks. On the 5 um full electrode (3.7 GB per float32 state,
// 985 801 steps, 26 620 of them with tracks at 9.2 MB of deposition each)
// that is terabytes. Here the memory is a fixed number of state slots, s, and
// the schedule is the binomial one of Griewank (A. Griewank, "Achieving
// logarithmic growth of temporal and spatial complexity in reverse automatic
// differentiation", Optimization Methods and Software 1, 1992; A. Griewank and
// A. Walther, "Algorithm 799: revolve", ACM TOMS 26, 2000), restated from the
// published recursion:
//
//   beta(s, t) = C(s + t, s) steps can be reversed from a stored start state
//   with s slots (the start's included) when no step is advanced more than t
//   times; the fewest forward steps that reversing l steps with s slots takes
//   is  t l - beta(s + 1, t - 1),  t the smallest with beta(s, t) >= l
//   (s = 1: l (l - 1) / 2, every step recomputed from the start).
//
// reverse(s0, l, slot b, s): the state of step s0 is in slot b and slots
// b+1 .. b+s-1 are free.
//   l = 1: the adjoint step of s0 straight from slot b;
//   s = 1: for j = l-1 .. 0, advance j steps from slot b, then the adjoint
//          step of s0 + j;
//   else:  advance m steps from slot b into slot b+1, reverse(s0 + m, l - m,
//          b+1, s-1), then reverse(s0, m, b, s), with m the split that
//          minimises m + cost(l - m, s - 1) + cost(m, s) (the cost is convex
//          in the split, so a bisection on its forward difference finds it).
// The top level's chain of right parts -- the "spine", states s0 of every
// level -- is what the forward solve stores as it passes it; the backward then
// reverses the deepest part first and each level's left part after it.
//
// The adjoint of step s needs u_s and the deposition of step s; a recomputed
// step deposits its tracks again into one scratch pair buffer (the deposition
// is a sum of float atomics, so a recomputed state may differ from the
// forward's in the last bit; the gradient does not notice). Everything is
// issued on one stream in order, so one scratch buffer serves every step.
#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "pic_internal.h"

namespace pic {

namespace {

constexpr int64_t kBetaCap = (int64_t)1 << 62;

// C(s + t, s), saturating at kBetaCap.
int64_t beta(int64_t s, int64_t t) {
    if (s < 0 || t < 0) return 0;
    const int64_t n = s + t, k = s < t ? s : t;
    __int128 r = 1;
    for (int64_t i = 1; i <= k; ++i) {
        r = r * (n - k + i) / i;  // C(n - k + i, i), exact
        if (r >= kBetaCap) return kBetaCap;
    }
    return (int64_t)r;
}

// Smallest t with beta(s, t) >= l (s >= 2, l >= 1).
int64_t reps(int64_t l, int64_t s) {
    int64_t t = 0;
    while (beta(s, t) < l) ++t;
    return t;
}

// Fewest forward steps to reverse l steps from a stored start with s slots.
int64_t cost(int64_t l, int64_t s) {
    if (l <= 1) return 0;
    if (s <= 1) return l * (l - 1) / 2;
    const int64_t t = reps(l, s);
    return t * l - beta(s + 1, t - 1);
}

// The split m in [1, l-1] minimising m + cost(l-m, s-1) + cost(m, s) (l >= 2, s >= 2).
int64_t split(int64_t l, int64_t s) {
    auto f = [&](int64_t m) { return m + cost(l - m, s - 1) + cost(m, s); };
    int64_t lo = 1, hi = l - 1;
    while (lo < hi) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (f(mid + 1) - f(mid) >= 0)
            hi = mid;
        else
            lo = mid + 1;
    }
    return lo;
}

struct Level {
    int64_t s0, l, slot, snaps;
};

// The spine: level q holds the state of step s0 in slot q.
std::vector<Level> spine(int64_t n_steps, int64_t n_slots) {
    std::vector<Level> out;
    if (n_steps <= 0) return out;
    Level v{0, n_steps, 0, n_slots};
    for (;;) {
        out.push_back(v);
        if (v.l == 1 || v.snaps == 1) return out;
        const int64_t m = split(v.l, v.snaps);
        v = Level{v.s0 + m, v.l - m, v.slot + 1, v.snaps - 1};
    }
}

// What the schedule does, independent of who carries it out.
struct Executor {
    // advance n >= 1 steps from slot b (state of step s0); the last result
    // goes to slot `to` when to >= 0, else it stays in the working buffers
    virtual int advance(int64_t s0, int64_t b, int64_t n, int64_t to) = 0;
    // the adjoint step of step s from slot b (from_slot) or from the working
    // buffer the last advance ended in
    virtual int adjoint(int64_t s, int64_t b, bool from_slot) = 0;
    virtual ~Executor() = default;
};

int reverse(Executor &x, int64_t s0, int64_t l, int64_t b, int64_t snaps) {
    int rc;
    if (l == 1) return x.adjoint(s0, b, true);
    if (snaps <= 1) {
        for (int64_t j = l - 1; j >= 0; --j) {
            if (j > 0 && (rc = x.advance(s0, b, j, -1))) return rc;
            if ((rc = x.adjoint(s0 + j, b, j == 0))) return rc;
        }
        return PIC_OK;
    }
    const int64_t m = split(l, snaps);
    if ((rc = x.advance(s0, b, m, b + 1))) return rc;
    if ((rc = reverse(x, s0 + m, l - m, b + 1, snaps - 1))) return rc;
    return reverse(x, s0, m, b, snaps);
}

int backward(Executor &x, int64_t n_steps, int64_t n_slots) {
    const std::vector<Level> sp = spine(n_steps, n_slots);
    if (sp.empty()) return PIC_OK;
    const Level &tail = sp.back();
    int rc = reverse(x, tail.s0, tail.l, tail.slot, tail.snaps);
    if (rc) return rc;
    for (int64_t q = (int64_t)sp.size() - 2; q >= 0; --q) {
        const Level &v = sp[q];
        if ((rc = reverse(x, v.s0, split(v.l, v.snaps), v.slot, v.snaps))) return rc;
    }
    return PIC_OK;
}

// Records the schedule: (kind, a, b, c) per event, kind 1 = advance (s0, n,
// slot to or -1), kind 2 = adjoint (s, slot or -1); slot contents are checked.
struct TraceExecutor : Executor {
    std::vector<int64_t> slot_step;  // step whose state each slot holds (-1: none)
    int64_t work_step = -1;          // step of the working buffers' state
    int64_t *events;
    int64_t cap, n = 0;
    int64_t advanced = 0;
    TraceExecutor(int64_t n_slots, int64_t *ev, int64_t c) : slot_step(n_slots, -1), events(ev), cap(c) {}
    void record(int64_t k, int64_t a, int64_t b, int64_t c) {
        if (events && n < cap) {
            events[4 * n] = k;
            events[4 * n + 1] = a;
            events[4 * n + 2] = b;
            events[4 * n + 3] = c;
        }
        ++n;
    }
    int advance(int64_t s0, int64_t b, int64_t cnt, int64_t to) override {
        if (b < 0 || b >= (int64_t)slot_step.size() || slot_step[b] != s0)
            return set_error(PIC_E_INVALID, "revolve schedule: advance from a slot that does not hold its step");
        if (to >= (int64_t)slot_step.size()) return set_error(PIC_E_INVALID, "revolve schedule: slot out of range");
        advanced += cnt;
        // an advance into a slot leaves the working buffers holding no step
        // the schedule may name
        if (to >= 0) {
            slot_step[to] = s0 + cnt;
            work_step = -1;
        } else {
            work_step = s0 + cnt;
        }
        record(1, s0, cnt, to);
        return PIC_OK;
    }
    int adjoint(int64_t s, int64_t b, bool from_slot) override {
        const int64_t have = from_slot ? (b >= 0 && b < (int64_t)slot_step.size() ? slot_step[b] : -2) : work_step;
        if (have != s) return set_error(PIC_E_INVALID, "revolve schedule: adjoint step without its state");
        record(2, s, from_slot ? b : -1, 0);
        return PIC_OK;
    }
};

struct DeviceExecutor : Executor {
    const pic_grid *g;
    cudaStream_t st;
    int64_t es, stride, dslot;
    char *SP, *SN;          // slots
    void *W[2][2];          // [buffer][species] working states
    int w_last = 0;         // working buffer of the last advance's result
    const double *xs, *ys;
    const int64_t *off;
    void *dens;             // one step's deposition pairs (scratch)
    void *ws;               // step workspace
    int64_t ws_bytes;
    void *lam[2][2];        // [buffer][species]
    int cur = 0;            // lambda_{s+1} is in lam[cur]
    void *adj_ws;

    void *slot_pos(int64_t b) const { return SP + b * stride * es; }
    void *slot_neg(int64_t b) const { return SN + b * stride * es; }

    int deposit(int64_t s, const void **d) {
        const int64_t m = off[s + 1] - off[s];
        *d = nullptr;
        if (m <= 0) return PIC_OK;
        cudaError_t e = cudaMemsetAsync(dens, 0, (size_t)(dslot * es), st);
        if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(deposition scratch)", e);
        int rc = launch_deposit(g, xs + off[s], ys + off[s], m, dens, nullptr, st, ws, ws_bytes);
        if (rc) return rc;
        *d = dens;
        return PIC_OK;
    }
    int advance(int64_t s0, int64_t b, int64_t n, int64_t to) override {
        const void *ip = slot_pos(b), *in = slot_neg(b);
        int w = 0;
        for (int64_t q = 0; q < n; ++q) {
            const void *d;
            int rc = deposit(s0 + q, &d);
            if (rc) return rc;
            void *pp, *pn;
            if (q == n - 1 && to >= 0) {
                pp = slot_pos(to);
                pn = slot_neg(to);
            } else {
                pp = W[w][0];
                pn = W[w][1];
                w_last = w;
                w ^= 1;
            }
            if ((rc = launch_step(g, ip, in, pp, pn, d, nullptr, nullptr, ws, st))) return rc;
            ip = pp;
            in = pn;
        }
        return PIC_OK;
    }
    int adjoint(int64_t s, int64_t b, bool from_slot) override {
        const void *d;
        int rc = deposit(s, &d);
        if (rc) return rc;
        const void *p = from_slot ? slot_pos(b) : W[w_last][0];
        const void *n = from_slot ? slot_neg(b) : W[w_last][1];
        rc = launch_adjoint(g, p, n, d, lam[cur][0], lam[cur][1], lam[cur ^ 1][0], lam[cur ^ 1][1], nullptr, adj_ws,
                            st, true);
        cur ^= 1;
        return rc;
    }
};

}  // namespace

int revolve_plan(int64_t n_steps, int64_t n_slots, int64_t *recompute_steps, int64_t *spine_levels) {
    if (n_steps < 0 || n_slots < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and n_slots >= 1");
    const std::vector<Level> sp = spine(n_steps, n_slots);
    // the forward solve passes the spine once; the rest is recomputation
    const int64_t total = cost(n_steps, n_slots);
    if (total >= kBetaCap / 2) return set_error(PIC_E_CAPACITY, "revolve schedule: too many steps for the slots");
    if (recompute_steps) *recompute_steps = total - (sp.empty() ? 0 : sp.back().s0);
    if (spine_levels) *spine_levels = (int64_t)sp.size();
    return PIC_OK;
}

int revolve_spine(int64_t n_steps, int64_t n_slots, int64_t *steps, int64_t cap, int64_t *n_levels) {
    if (n_steps < 0 || n_slots < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and n_slots >= 1");
    const std::vector<Level> sp = spine(n_steps, n_slots);
    for (int64_t q = 0; q < (int64_t)sp.size() && q < cap; ++q) steps[q] = sp[q].s0;
    *n_levels = (int64_t)sp.size();
    return PIC_OK;
}

int revolve_trace(int64_t n_steps, int64_t n_slots, int64_t *events, int64_t cap, int64_t *n_events,
                  int64_t *advanced) {
    if (n_steps < 0 || n_slots < 1) return set_error(PIC_E_INVALID, "n_steps must be >= 0 and n_slots >= 1");
    TraceExecutor x(n_slots, events, cap);
    for (const Level &v : spine(n_steps, n_slots)) x.slot_step[v.slot] = v.s0;  // stored by the forward
    int rc = backward(x, n_steps, n_slots);
    if (rc) return rc;
    *n_events = x.n;
    *advanced = x.advanced;
    return PIC_OK;
}

int revolve_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                    const double *xs, const double *ys, const int64_t *off, void *dens, uint32_t *counts,
                    double *tally, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots, void *ws,
                    int64_t ws_bytes, cudaStream_t st) {
    const int64_t es = g->dtype == PIC_F64 ? 8 : 4;
    const int64_t field = g->no_xy * g->no_xy * g->kpitch;
    const int64_t dslot = 2 * g->no_xy * dens_pitch(g->no_xy);
    const std::vector<Level> sp = spine(n_steps, n_slots);
    void *pos[2] = {pos0, pos1}, *neg[2] = {neg0, neg1};
    size_t q = 0;
    for (int64_t s = 0; s < n_steps; ++s) {
        const int b = (int)(s & 1);
        if (q < sp.size() && sp[q].s0 == s) {
            char *dp = static_cast<char *>(slots_pos) + sp[q].slot * state_stride * es;
            char *dn = static_cast<char *>(slots_neg) + sp[q].slot * state_stride * es;
            cudaError_t e = cudaMemcpyAsync(dp, pos[b], (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
            if (e == cudaSuccess) e = cudaMemcpyAsync(dn, neg[b], (size_t)(field * es), cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemcpyAsync(checkpoint)", e);
            ++q;
        }
        const int64_t m = off[s + 1] - off[s];
        const void *d = nullptr;
        if (m > 0) {
            cudaError_t e = cudaMemsetAsync(dens, 0, (size_t)(dslot * es), st);
            if (e != cudaSuccess) return set_cuda_error("cudaMemsetAsync(deposition scratch)", e);
            int rc = launch_deposit(g, xs + off[s], ys + off[s], m, dens, counts, st, ws, ws_bytes);
            if (rc) return rc;
            d = dens;
        }
        int rc = launch_step(g, pos[b], neg[b], pos[b ^ 1], neg[b ^ 1], d, nullptr, tally + 4 * s, ws, st);
        if (rc) return rc;
    }
    return PIC_OK;
}

int revolve_backward(const pic_grid *g, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots,
                     int64_t n_steps, const double *xs, const double *ys, const int64_t *off, void *dens,
                     void *work_pos0, void *work_neg0, void *work_pos1, void *work_neg1, void *lam_pos0,
                     void *lam_neg0, void *lam_pos1, void *lam_neg1, double *grad, void *ws, int64_t ws_bytes,
                     void *adj_ws, cudaStream_t st) {
    DeviceExecutor x;
    x.g = g;
    x.st = st;
    x.es = g->dtype == PIC_F64 ? 8 : 4;
    x.stride = state_stride;
    x.dslot = 2 * g->no_xy * dens_pitch(g->no_xy);
    x.SP = static_cast<char *>(slots_pos);
    x.SN = static_cast<char *>(slots_neg);
    x.W[0][0] = work_pos0;
    x.W[0][1] = work_neg0;
    x.W[1][0] = work_pos1;
    x.W[1][1] = work_neg1;
    x.xs = xs;
    x.ys = ys;
    x.off = off;
    x.dens = dens;
    x.ws = ws;
    x.ws_bytes = ws_bytes;
    x.lam[0][0] = lam_pos0;
    x.lam[0][1] = lam_neg0;
    x.lam[1][0] = lam_pos1;
    x.lam[1][1] = lam_neg1;
    x.adj_ws = adj_ws;
    int rc = adjoint_accumulate_begin(g, adj_ws, st);
    if (rc) return rc;
    if ((rc = backward(x, n_steps, n_slots))) return rc;
    return adjoint_accumulate_end(g, adj_ws, grad, st);
}

}  // namespace pic
