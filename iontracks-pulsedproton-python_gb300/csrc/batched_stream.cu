// batched_stream.cu -- the streaming step over many grids at once.
//
// The flat batched step (batched.cu) reads every stencil neighbour through
// L1/L2; on the big phases of a sweep (a gigabyte of fields, far more than
// L2) its neighbour planes miss L2 and it moves ~1.4x the compulsory bytes at
// about half of the HBM peak. This kernel runs the single-grid streaming
// step's copy ring (pic_stream.cuh) over a table of work items drawn from
// every active grid: an item is (grid, a tile of interior rows with every k,
// a range of interior planes), and a CTA's producer warp takes items from a
// device-wide queue (one atomic per item) and streams their planes into the
// ring while the consumer warps compute them with the grid's own coefficients
// (staged per warp in shared memory).
//
// Per-grid geometry: each grid has its own tile height, chosen on the host so
// that a tile's k-vectors fit the consumer threads (rows x kpitch/4 <= IPT x
// 32 x consumer warps) and a stage of any grid fits the launch's stage size.
//
// Tallies: every consumer warp writes its sums over an item into its own slot
// (item, warp) and counts itself in on the item's grid; the warp that
// completes a grid sums that grid's slots in a fixed order (double-float
// arithmetic) and writes the grid's tally row. No barrier spans warps inside
// the item loop, so an expired bounded wait in one warp cannot leave another
// waiting; results are deterministic for a given item table and launch shape
// whichever CTA takes which item.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "pic_async.cuh"
#include "pic_device.cuh"
#include "pic_internal.h"
#include "pic_stream.cuh"

namespace pic {

namespace {

constexpr int kQueue = 8;  // items the producer may run ahead of the consumers (entries of item_q)
constexpr int kBsWarps = 15;
constexpr int kBsMaxThreads = (kBsWarps + 1) * 32;

// One grid of a batched streaming launch: its step arguments with the field,
// deposition and status pointers left null (set per item from the launch's
// packed buffers), and its offsets in those buffers.
struct BsGrid {
    StreamArgs a;
    int64_t field_off, dens_off, tally_off;
    int32_t item0, n_items;  // its items in the launch's table
};

struct BsHeader {
    unsigned int next;   // next item of the current step (device-wide queue)
    unsigned int done;   // CTAs finished with the current step
    int status;          // 0, or the code of a bounded wait that ran out / a refused item
};

struct BsArgs {
    const BsGrid *grids;
    const int4 *items;  // grid, cj_lo, ci_lo, ci_hi
    int n_items;
    const float *pos_in, *neg_in;
    float *pos_out, *neg_out;
    const float2 *dens;
    float2 *dens_zero;
    double *tally;
    int64_t step;
    BsHeader *hdr;
    unsigned int *grid_ctr;
    float2 *part;  // [n_items][consumer_warps][4] double-float partials
    int stages, consumer_warps, stage_floats;
};

// Workspace: [header | per-grid counters | grid table | item table | partials],
// each part padded to 256 bytes.
int64_t pad256(int64_t b) { return (b + 255) / 256 * 256; }
int64_t off_ctr() { return 256; }
int64_t off_grids(int32_t n_cfgs) { return off_ctr() + pad256((int64_t)n_cfgs * 4); }
int64_t off_items(int32_t n_cfgs) { return off_grids(n_cfgs) + pad256((int64_t)n_cfgs * (int64_t)sizeof(BsGrid)); }
int64_t off_part(int32_t n_cfgs, int32_t n_items) { return off_items(n_cfgs) + pad256((int64_t)n_items * 16); }

__device__ __forceinline__ void copy_args(StreamArgs &dst, const StreamArgs &src, int lane) {
    const uint32_t *s = reinterpret_cast<const uint32_t *>(&src);
    uint32_t *d = reinterpret_cast<uint32_t *>(&dst);
    for (int w = lane; w < (int)(sizeof(StreamArgs) / 4); w += 32) d[w] = s[w];
}

template <int IPT>
__global__ void __launch_bounds__(kBsMaxThreads, 1) batched_stream_kernel(BsArgs b) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    __shared__ volatile int abort_flag;
    __shared__ int item_q[kQueue];
    __shared__ StreamArgs wargs[kBsWarps];  // per consumer warp: its current item's grid
    uint64_t *full = reinterpret_cast<uint64_t *>(smem_raw);
    uint64_t *empty = full + b.stages;
    const int bar_bytes = (2 * b.stages * 8 + 127) / 128 * 128;
    float *stage0 = reinterpret_cast<float *>(smem_raw + bar_bytes);
    const int S = b.stages;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cw = b.consumer_warps;
    int *status = &b.hdr->status;

    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], cw);
        }
        mbar_fence_init();
        abort_flag = 0;
    }
    __syncthreads();

    if (warp == cw) {
        // ---------------- producer: lane 0 takes items and issues their copies ----------------
        if (lane == 0) {
            long long g = 0;
            bool ok = true;
            for (int k = 0; ok; ++k) {
                int w = (int)atomicAdd(&b.hdr->next, 1u);
                int4 it = make_int4(0, 0, 0, 0);
                const BsGrid *G = nullptr;
                // refuse (skip, with a status) an item outside its grid or one
                // whose tile does not fit the consumers or a stage
                while (w < b.n_items) {
                    it = b.items[w];
                    G = b.grids + it.x;
                    const StreamArgs &a = G->a;
                    const bool fits = it.y >= 1 && it.y <= a.n - 2 && it.z >= 1 && it.z < it.w && it.w <= a.n - 1 &&
                                      a.tj * a.c4 <= IPT * 32 * cw && stream_stage_floats(a.tj, a.kp) <= b.stage_floats;
                    if (fits) break;
                    atomicExch(status, 7);
                    w = (int)atomicAdd(&b.hdr->next, 1u);
                }
                const bool done = w >= b.n_items;
                int slot = (int)(g % S);
                if (g >= S && !mbar_wait(&empty[slot], (uint32_t)(((g / S) - 1) & 1), status, 1)) {
                    abort_flag = 1;
                    ok = false;
                    break;
                }
                if (abort_flag) {
                    ok = false;
                    break;
                }
                item_q[k % kQueue] = done ? -1 : w;
                if (done) {
                    mbar_arrive(&full[slot]);  // the end mark: a phase without bytes
                    break;
                }
                StreamArgs a = G->a;
                a.pos_in = b.pos_in + G->field_off;
                a.neg_in = b.neg_in + G->field_off;
                a.dens = b.dens + G->dens_off;
                const int cj_lo = it.y, cj_hi = min(it.y + a.tj, a.n - 1);
                for (int pl = it.z - 1; pl <= it.w; ++pl, ++g) {
                    slot = (int)(g % S);
                    if (pl > it.z - 1 && g >= S &&
                        !mbar_wait(&empty[slot], (uint32_t)(((g / S) - 1) & 1), status, 1)) {
                        abort_flag = 1;
                        ok = false;
                        break;
                    }
                    if (abort_flag) {
                        ok = false;
                        break;
                    }
                    stream_issue_plane(a, pl, cj_lo, cj_hi, stage0 + (size_t)slot * b.stage_floats, &full[slot]);
                }
            }
            if (!ok) {
                for (long long gg = g - S < 0 ? 0 : g - S; gg < g; ++gg)
                    mbar_wait(&full[gg % S], (uint32_t)((gg / S) & 1), status, 2);
            }
        }
    } else {
        // ---------------- consumers: one item after another, per warp ----------------
        StreamArgs &a = wargs[warp];
        long long g = 0;
        for (int k = 0;; ++k) {
            // the item's first plane, or the end mark, tells which item comes next
            if (!mbar_wait(&full[g % S], (uint32_t)((g / S) & 1), status, 3)) {
                abort_flag = 1;
                break;
            }
            if (abort_flag) break;
            const int w = item_q[k % kQueue];
            if (w < 0) break;
            const int4 it = b.items[w];
            const BsGrid *G = b.grids + it.x;
            copy_args(a, G->a, lane);
            __syncwarp();
            if (lane == 0) {
                a.pos_in = b.pos_in + G->field_off;
                a.neg_in = b.neg_in + G->field_off;
                a.pos_out = b.pos_out + G->field_off;
                a.neg_out = b.neg_out + G->field_off;
                a.dens = b.dens + G->dens_off;
                a.dens_zero = b.dens_zero ? b.dens_zero + G->dens_off : nullptr;
                a.status = status;
            }
            __syncwarp();
            Tally<float> t_rec, t_p, t_n, t_inj;
            const int cj_lo = it.y, cj_hi = min(it.y + a.tj, a.n - 1);
            const StreamConsts K = stream_consts(a);
            if (!stream_consume_item<IPT>(a, K, cj_lo, cj_hi, it.z, it.w, stage0, b.stage_floats, full, empty, S, g,
                                          abort_flag, threadIdx.x, cw * 32, t_rec, t_p, t_n, t_inj))
                break;
            // this warp's sums over the item into its slot; the warp that
            // completes the grid sums the grid's slots
            DF v[4] = {df_of(t_inj), df_of(t_rec), df_of(t_p), df_of(t_n)};
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = warp_sum(v[q]);
            const int c = it.x;
            unsigned int prev = 0;
            if (lane == 0) {
                float2 *slot = b.part + ((int64_t)w * cw + warp) * 4;
#pragma unroll
                for (int q = 0; q < 4; ++q) slot[q] = make_float2(v[q].hi, v[q].lo);
                __threadfence();
                prev = atomicAdd(b.grid_ctr + c, 1u);
            }
            prev = __shfl_sync(0xffffffffu, prev, 0);
            const unsigned int total = (unsigned int)(G->n_items * cw);
            if (prev == total - 1u) {
                __threadfence();
                DF acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
                const float2 *p0 = b.part + (int64_t)G->item0 * cw * 4;
                for (unsigned int s = lane; s < total; s += 32)
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const float2 p = __ldcg(p0 + (int64_t)s * 4 + q);
                        acc[q] = df_add(acc[q], DF{p.x, p.y});
                    }
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[q] = warp_sum(acc[q]);
                if (lane == 0) {
                    double *t = b.tally + 4 * (G->tally_off + b.step);
                    t[0] = df_value(acc[0]) * a.injected_scale;
                    t[1] = df_value(acc[1]);
                    t[2] = df_value(acc[2]);
                    t[3] = df_value(acc[3]);
                    b.grid_ctr[c] = 0u;
                    __threadfence();
                }
            }
        }
    }
    // the last CTA to finish resets the queue for the next step: every CTA has
    // taken its last ticket by now
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&b.hdr->done, 1u) == gridDim.x - 1) {
            b.hdr->next = 0u;
            b.hdr->done = 0u;
            __threadfence();
        }
    }
}

template <int IPT>
int launch_bs(const BsArgs &b, unsigned blocks, int threads, int smem, cudaStream_t st) {
    static int configured = 0;
    if (smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(batched_stream_kernel<IPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             smem);
        if (e != cudaSuccess) return set_cuda_error("cudaFuncSetAttribute(batched_stream_kernel)", e);
        configured = smem;
    }
    batched_stream_kernel<IPT><<<blocks, threads, smem, st>>>(b);
    return check_launch("batched_stream_kernel");
}

// Static shared memory of the kernel: item queue, per-warp arguments, flags.
constexpr int kBsStaticSmem = (int)(kQueue * 4 + kBsWarps * sizeof(StreamArgs) + 64);

int smem_for(int stages, int stage_floats) { return (2 * stages * 8 + 127) / 128 * 128 + stages * stage_floats * 4; }

}  // namespace

int batched_stream_workspace_bytes(int32_t n_cfgs, int32_t n_items, int32_t consumer_warps, int64_t *bytes) {
    if (n_cfgs < 1 || n_items < 1 || consumer_warps < 1 || consumer_warps > kBsWarps)
        return set_error(PIC_E_INVALID, "n_cfgs, n_items >= 1 and consumer_warps in 1 .. 15");
    *bytes = off_part(n_cfgs, n_items) + (int64_t)n_items * consumer_warps * 4 * 8;
    return PIC_OK;
}

int batched_stream_prepare(const pic_batch_cfg *cfgs, int32_t n_cfgs, const int32_t *items, int32_t n_items,
                           const int32_t *tile_rows, int32_t consumer_warps, void *ws, int64_t ws_bytes,
                           cudaStream_t st, pic_batch_stream *out) {
    int64_t need = 0;
    int rc = batched_stream_workspace_bytes(n_cfgs, n_items, consumer_warps, &need);
    if (rc) return rc;
    if (!cfgs || !items || !tile_rows || !ws || !out) return set_error(PIC_E_INVALID, "null pointer argument");
    if (ws_bytes < need) return set_error(PIC_E_INVALID, "workspace too small (pic_batched_stream_workspace_bytes)");
    if (reinterpret_cast<uintptr_t>(ws) % 256) return set_error(PIC_E_INVALID, "workspace must be 256-byte aligned");
    const int nct = consumer_warps * 32;
    std::vector<BsGrid> grids(n_cfgs);
    int max_stage = 0, ipt = 1;
    for (int c = 0; c < n_cfgs; ++c) {
        const pic_grid &g = cfgs[c].grid;
        if (g.dtype != PIC_F32) return set_error(PIC_E_INVALID, "the batched streaming step takes float32 grids only");
        if (g.no_xy < 4 || g.no_xy > 16383) return set_error(PIC_E_INVALID, "batched streaming step: no_xy in 4 .. 16383");
        if (g.kpitch != pic_kpitch(g.nzb) || g.nze < 1 || g.no_z < 1 || g.nze + g.no_z > g.nzb - 1)
            return set_error(PIC_E_INVALID, "batched streaming step: inconsistent k geometry of grid " + std::to_string(c));
        const int tj = tile_rows[c];
        const int c4 = (int)(g.kpitch / 4);
        if (tj < 1 || tj > g.no_xy - 2) return set_error(PIC_E_INVALID, "tile_rows must be in 1 .. no_xy - 2");
        const int need_ipt = (tj * c4 + nct - 1) / nct;
        ipt = std::max(ipt, need_ipt);
        max_stage = std::max(max_stage, stream_stage_floats(tj, (int)g.kpitch));
        StreamArgs &a = grids[c].a;
        a = StreamArgs{};
        a.n = (int)g.no_xy;
        a.kp = (int)g.kpitch;
        a.c4 = c4;
        a.nzb = (int)g.nzb;
        a.nze = (int)g.nze;
        a.gap_end = (int)(g.nze + g.no_z);
        a.reflecting = g.wall == PIC_WALL_REFLECTING;
        a.dp = (int)dens_pitch(g.no_xy);
        a.tj = tj;
        a.consumer_warps = consumer_warps;
        a.p_lat = (float)g.p_lat; a.p_zm = (float)g.p_zm; a.p_zp = (float)g.p_zp;
        a.p_cen = centre_weight<float>(g.p_lat, g.p_zm, g.p_zp, g.p_cen);
        a.n_lat = (float)g.n_lat; a.n_zm = (float)g.n_zm; a.n_zp = (float)g.n_zp;
        a.n_cen = centre_weight<float>(g.n_lat, g.n_zm, g.n_zp, g.n_cen);
        a.alpha_dt = (float)g.alpha_dt;
        a.gfac = (float)g.gaussian_factor;
        ScoreTest sc;
        if ((rc = score_test(&g, &sc))) return rc;
        a.two_mid = (int)sc.two_mid;
        a.thr4 = sc.thr4 < 0 ? 0u : (sc.thr4 > 0x7fffffffLL ? 0xffffffffu : (uint32_t)sc.thr4);
        a.injected_scale = (double)g.no_z;
        grids[c].field_off = cfgs[c].field_off;
        grids[c].dens_off = cfgs[c].dens_off;
        grids[c].tally_off = cfgs[c].tally_off;
        grids[c].item0 = 0;
        grids[c].n_items = 0;
    }
    if (ipt > 3) return set_error(PIC_E_INVALID, "tile_rows x kpitch/4 exceed 3 k-vectors per consumer thread");
    // items: grouped by grid, each inside its grid
    std::vector<int> seen(n_cfgs, 0);
    int prev = -1;
    for (int w = 0; w < n_items; ++w) {
        const int c = items[4 * w], cj = items[4 * w + 1], i0 = items[4 * w + 2], i1 = items[4 * w + 3];
        if (c < 0 || c >= n_cfgs) return set_error(PIC_E_INVALID, "item " + std::to_string(w) + ": grid out of range");
        const int64_t n = cfgs[c].grid.no_xy;
        if (cj < 1 || cj > n - 2 || i0 < 1 || i0 >= i1 || i1 > n - 1)
            return set_error(PIC_E_INVALID, "item " + std::to_string(w) + ": rows or planes outside its grid");
        if (c != prev) {
            if (seen[c]) return set_error(PIC_E_INVALID, "items must be grouped by grid");
            seen[c] = 1;
            grids[c].item0 = w;
            prev = c;
        }
        grids[c].n_items++;
    }
    const int stages_fit = (kStreamMaxSmem - kBsStaticSmem - 2048 - 256) / (max_stage * 4);
    const int stages = std::min(16, stages_fit);
    if (stages < 4) return set_error(PIC_E_CAPACITY, "batched streaming step: fewer than 4 ring stages fit");
    char *base = static_cast<char *>(ws);
    cudaError_t e = cudaMemsetAsync(base, 0, (size_t)off_grids(n_cfgs), st);  // header and grid counters
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + off_grids(n_cfgs), grids.data(), grids.size() * sizeof(BsGrid),
                            cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(base + off_items(n_cfgs), items, (size_t)n_items * 16, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the host tables may go once this returns
    if (e != cudaSuccess) return set_cuda_error("pic_batched_stream_prepare upload", e);
    out->n_cfgs = n_cfgs;
    out->n_items = n_items;
    out->consumer_warps = consumer_warps;
    out->stages = stages;
    out->stage_floats = max_stage;
    out->ipt = ipt;
    out->workspace = ws;
    out->workspace_bytes = ws_bytes;
    return PIC_OK;
}

int batched_stream_step(const BatchLaunch &L, const pic_batch_stream &B, int bi, int bo, int64_t step,
                        const void *dens, void *dens_zero, cudaStream_t st) {
    char *base = static_cast<char *>(B.workspace);
    BsArgs b;
    b.grids = reinterpret_cast<const BsGrid *>(base + off_grids(B.n_cfgs));
    b.items = reinterpret_cast<const int4 *>(base + off_items(B.n_cfgs));
    b.n_items = B.n_items;
    b.pos_in = (const float *)L.pos[bi];
    b.neg_in = (const float *)L.neg[bi];
    b.pos_out = (float *)L.pos[bo];
    b.neg_out = (float *)L.neg[bo];
    b.dens = (const float2 *)dens;
    b.dens_zero = (float2 *)dens_zero;
    b.tally = L.tally;
    b.step = step;
    b.hdr = reinterpret_cast<BsHeader *>(base);
    b.grid_ctr = reinterpret_cast<unsigned int *>(base + off_ctr());
    b.part = reinterpret_cast<float2 *>(base + off_part(B.n_cfgs, B.n_items));
    b.stages = B.stages;
    b.consumer_warps = B.consumer_warps;
    b.stage_floats = B.stage_floats;
    const int smem = smem_for(B.stages, B.stage_floats);
    unsigned blocks = (unsigned)std::min<int64_t>(sm_count(), B.n_items);
    const int threads = (B.consumer_warps + 1) * 32;
    return B.ipt <= 2 ? launch_bs<2>(b, blocks, threads, smem, st) : launch_bs<3>(b, blocks, threads, smem, st);
}

int batched_stream_status(const pic_batch_stream &B, int32_t reset, cudaStream_t st, int32_t *status) {
    BsHeader *h = static_cast<BsHeader *>(B.workspace);
    int v = 0;
    cudaError_t e = cudaMemcpyAsync(&v, &h->status, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return set_cuda_error("reading the batched streaming status word", e);
    *status = v;
    if (reset && v != 0) {
        // an aborted step can leave the queue and the grid counters mid-count
        e = cudaMemsetAsync(B.workspace, 0, (size_t)off_grids(B.n_cfgs), st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return set_cuda_error("resetting the batched streaming workspace", e);
    }
    return PIC_OK;
}

}  // namespace pic
