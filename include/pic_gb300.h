/*
 * pic_gb300.h -- C ABI of the GB300 (sm_103a) hot path of the pulsed-proton
 * ion-chamber recombination solver.
 *
 * Plain pointers and sizes only. Every device pointer is a CUDA device
 * address owned by the caller (the Python host allocates with PyTorch and
 * passes Tensor.data_ptr()); streams are cudaStream_t passed as uintptr_t
 * (0 = legacy default stream). Every entry point returns PIC_OK (0) or a
 * negative PIC_E_* code; pic_last_error() then describes the failure (the
 * message is per host thread). No C++ exception crosses this boundary.
 *
 * Field layout in HBM: one array per species and buffer,
 *     field[i][j][k],  0 <= i, j < no_xy,  0 <= k < kpitch,
 * k fastest, kpitch = pic_kpitch(nzb) >= nzb (rows start 32-byte aligned).
 * Elements k >= nzb - 1 and k == 0 are the z end planes plus padding and are
 * kept at zero. Fields are float32 (PIC_F32) or float64 (PIC_F64, the
 * validation build). A step's deposition follows the field type and is laid
 * out as pairs dens[i][j] = {G * density, G * (sum of the density of the four
 * lateral neighbours)}, 0 <= j < pic_dens_pitch(no_xy) (rows padded to 4
 * pairs so each starts 32-byte aligned; G = gaussian_factor). Per-step tallies
 * are always float64: tally[s] = {injected, recombined, sum n+, sum n-} over
 * the scored voxels.
 */
#ifndef PIC_GB300_H
#define PIC_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PIC_OK 0
#define PIC_E_INVALID (-1)  /* bad argument: size, alignment, null pointer */
#define PIC_E_CUDA (-2)     /* a CUDA runtime call failed */
#define PIC_E_DEVICE (-3)   /* no usable sm_103 device */
#define PIC_E_CAPACITY (-4) /* a size beyond what the entry point supports */

#define PIC_F32 0
#define PIC_F64 1

#define PIC_WALL_ABSORBING 0
#define PIC_WALL_REFLECTING 1

/* One grid and the scalars its kernels need. Mirrors the attributes of the
 * reference's SimulationConfig that its kernels take as arguments
 * (pulsed_ion_chamber/solver_numba.py:54-68, :130-151). */
typedef struct pic_grid {
    int64_t no_xy;          /* lateral size (both axes)                      */
    int64_t nzb;            /* no_z_with_buffer: k extent incl. electrodes   */
    int64_t kpitch;         /* allocated k extent, pic_kpitch(nzb)           */
    int64_t no_z;           /* gap layers                                    */
    int64_t nze;            /* no_z_electrode: first gap layer               */
    double mid_xy;          /* grid centre (float; odd no_xy gives .5)       */
    double scoring_radius_sq;
    double p_lat, p_zm, p_zp, p_cen; /* positive-species LW weights          */
    double n_lat, n_zm, n_zp, n_cen; /* negative species, applied z-swapped  */
    double alpha_dt;        /* recombination alpha * dt                      */
    double gaussian_factor; /* N0 / (pi b^2), track peak density             */
    double h2_over_b2;      /* voxel area / track radius^2                   */
    double cutoff_voxels;   /* deposition half-width                         */
    int32_t wall;           /* PIC_WALL_*                                    */
    int32_t dtype;          /* PIC_F32 or PIC_F64                            */
    /* Launch shape of the fused step (0 = chosen by the library). */
    int32_t variant;         /* PIC_VARIANT_*                                */
    int32_t tile_rows;       /* stream variant: interior j rows per tile     */
    int32_t planes_per_item; /* stream variant: i planes per work item       */
    int32_t stages;          /* stream variant: shared-memory ring stages    */
    int32_t consumer_warps;  /* stream variant: compute warps per CTA        */
    int32_t ctas_per_sm;     /* stream variant: resident CTAs per SM         */
    int32_t steps_per_launch; /* flat variant: 0 or 1 = one launch per step
                              * (two with tracks); K in 2 .. 256 = up to K
                              * steps per cooperative launch (device-wide
                              * barriers between the phases of a step), for
                              * latency-bound small grids */
    /* Adjoint step kernel (pic_adjoint_*, pic_revolve_backward): a
     * PIC_VARIANT_* of its own, so tuning the step's shape leaves it alone.
     * AUTO: STREAM for float32 grids with no_xy >= 4 and no_xy^2 * kpitch >=
     * 2^24 cells, FLAT otherwise; STREAM on a float64 grid is refused. */
    int32_t adjoint_variant;
    /* Deposition form (PIC_DEPOSIT_*). */
    int32_t deposit_variant;
} pic_grid;

/* Deposition forms. TRACKS: one to eight warps per track, each cell's pair
 * added with a vector atomic (any call). BINNED: a binning launch lists each
 * track in the 62 x 62-cell tiles its box meets, then one block per tile sums
 * its tracks' separable Gaussians as outer products in ascending track order
 * and stores each cell once (no atomics on the pairs; two runs give identical
 * pairs). pic_run_segment deposits up to 8 of its steps (65536 tracks) per
 * pair of launches, into pair buffers in the workspace; its dens0/dens1 then
 * end as the per-step forms leave them (the last step's pairs if it
 * deposited, the other buffer zero). It needs the track lists of the step workspace, so only the calls
 * that take one use it (pic_run_segment, the graph capture, the gradient
 * drivers), for no_xy <= 4096 and cutoff_voxels < 31.5 (truncation boxes of
 * at most 64 cells); elsewhere BINNED is refused. AUTO: BINNED
 * where it can run: for the steps of a segment (pic_run_segment,
 * pic_adjoint_forward) unless a few tiles would each gather more than ~1024
 * of a step's tracks; for one step alone (the checkpointed gradient) where
 * the grid has at least two tiles per SM (no_xy >= 1055 on 152 SMs);
 * otherwise TRACKS, or on small grids
 * whose steps bring many tracks a scan-tile form (every block scans the
 * step's tracks; one vector atomic per cell and block). */
#define PIC_DEPOSIT_AUTO 0
#define PIC_DEPOSIT_TRACKS 1
#define PIC_DEPOSIT_BINNED 2

/* Fused-step kernels. FLAT: one thread per four k of a column, neighbours
 * through L1/L2, any grid and either field type. STREAM: float32 only; whole
 * (j-tile x k-row) planes staged in shared memory by bulk asynchronous copies
 * while the CTA marches along i, for grids with no_xy >= 16. AUTO picks
 * STREAM for float32 grids with no_xy >= 64 and no_xy^2 * kpitch >= 1e8 cells,
 * FLAT otherwise; planes_per_item 0 gives about 12 work items per SM,
 * consumer_warps 0 gives 13, tile_rows 0 about three k-vectors a consumer
 * thread, stages 0 as many as shared memory holds. */
#define PIC_VARIANT_AUTO 0
#define PIC_VARIANT_FLAT 1
#define PIC_VARIANT_STREAM 2

/* Description of the last failure on this host thread ("" if none). */
const char *pic_last_error(void);

/* ABI version (bumped on any signature or struct change). */
int pic_abi_version(void);

/* k pitch for a given no_z_with_buffer: nzb rounded up to 8 elements. */
int64_t pic_kpitch(int64_t nzb);

/* Row pitch of the deposition pairs: no_xy rounded up to 4 pairs. */
int64_t pic_dens_pitch(int64_t no_xy);

/* Checks that a CUDA device of compute capability 10.3 is current; fills the
 * SM count and the device's total memory. */
int pic_device_info(int32_t *sm_count, int64_t *total_bytes, int32_t *cc_major, int32_t *cc_minor);

/* Bytes of device scratch the fused step needs for this grid (per-block
 * tally partials, a completion counter, a status word and, where the
 * binned deposition can run, for each of 8 steps its per-tile track lists
 * and deposition pairs, and the boxes and Gaussian factors of up to 65536
 * tracks: about 150 MB for a 1068 x 1068 float32 grid). The caller allocates it once, zero-filled, and passes it
 * to pic_step / pic_run_segment; every call leaves its counters at zero again.
 * A workspace of the fixed part alone (ABI 5's size) is still accepted: the
 * deposition then runs without the binned form. */
int pic_step_workspace_bytes(const pic_grid *g, int64_t *bytes);

/* Reads (and with reset != 0 clears) the status word a kernel sets in the
 * workspace when a bounded wait gave up: 0 = ok, > 0 = the wait that
 * expired. Synchronises the stream first. */
int pic_workspace_status(void *workspace, int32_t reset, uintptr_t stream, int32_t *status);

/* The launch shape the library would use for this grid when the shape
 * fields are 0: fills variant .. ctas_per_sm of *resolved. */
int pic_resolve_shape(const pic_grid *g, pic_grid *resolved);

/*
 * pic_deposit -- sum one step's track Gaussians into the deposition pairs.
 *
 * With g_i = exp(-(i-x_t)^2 h2/b2) on each track's truncated stencil box
 * [ceil(x-cut), floor(x+cut)] clipped to the grid (0 outside it), and the
 * same g_j in y: dens[i][j].x += G sum_t g_i g_j and
 * dens[i][j].y += G sum_t ((g_{i-1} + g_{i+1}) g_j + g_i (g_{j-1} + g_{j+1})),
 * i.e. the density and its four lateral neighbours' sum, both times
 * G = gaussian_factor; counts[int(x)][int(y)] += 1 per track. dens must be
 * zero on entry for a fresh step (pic_step zeroes the next step's buffer).
 *
 * Replaces: _insert_track_numba's per-track stencil (solver_numba.py:84-98),
 * _precompute_track_gaussians + _build_row_index +
 * _accumulate_track_density_numba_parallel (solver_numba_parallel.py:421-457,
 * :140-180, :183-219), _accumulate_kernel (solver_cuda.py:291-323) and
 * Diagnostics.count_tracks (state.py:71-84).
 */
int pic_deposit(const pic_grid *g, const double *xs, const double *ys, int64_t n_tracks, void *dens,
                uint32_t *counts, uintptr_t stream);

/*
 * pic_step -- one fused time step: deposition broadcast, Lax-Wendroff sweep,
 * recombination sink, lateral wall and the step's tallies.
 *
 * Reads pos_in/neg_in (+ the deposition in every gap layer when dens is
 * non-null: a column's own density on its values, its neighbours' sum on the
 * stencil's lateral sum), writes every column of pos_out/neg_out: the interior by the
 * 7-point Lax-Wendroff stencil minus alpha*dt*n+*n-, the outer ring carried
 * with the step's deposition (absorbing) or mirrored from the new interior
 * (reflecting). Writes tally[0..3] = {injected, recombined, sum n+, sum n-}
 * over the scored voxels. If dens_zero is non-null it is zero-filled (the
 * buffer the next step's pic_deposit accumulates into).
 *
 * Replaces: _broadcast_density_numba_parallel (solver_numba_parallel.py:222-277),
 * _lax_wendroff_step_numba(_parallel) (solver_numba.py:130-213,
 * solver_numba_parallel.py:280-418), apply_lateral_boundary /
 * carry_lateral_ring and the swap (state.py:113-176,
 * solver_numba_parallel.py:686-695), _sweep_kernel + _broadcast_kernel + the
 * masked injected sum (solver_cuda.py:176-289, :325-354, :812).
 */
int pic_step(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
             const void *dens, void *dens_zero, double *tally, void *workspace, int64_t workspace_bytes,
             uintptr_t stream);

/*
 * pic_step_noalloc -- one whole time step, allocating nothing: this step's
 * n_tracks track centres deposited (as pic_deposit, counts updated), then the
 * fused step (as pic_step) from pos_in/neg_in into pos_out/neg_out, tallies
 * into tally[0..3]. The 2D density and the tally workspace live in a static
 * device array inside the library, so a caller that cannot allocate device
 * memory -- a binding that only holds buffers owned by another runtime, or
 * code running where cudaMalloc is not allowed -- passes only its inputs and
 * outputs.
 *
 * No counterpart in the reference (whose drivers allocate their own arrays).
 * Limit: the deposition pairs must fit the 16 MiB static scratch -- no_xy <=
 * 1448 for float32 fields, <= 1024 for float64 -- else PIC_E_CAPACITY. Every
 * GPU that loads the library holds the array (16 MiB plus the tally workspace)
 * until exit. All calls share it: calls that overlap on the GPU race, so
 * serialise them. Each call looks up the array's device address on the
 * current device (so it stays right after a device reset); the first call on
 * a device also loads the library's device code there: make it before any
 * stream capture.
 */
int pic_step_noalloc(const pic_grid *g, const void *pos_in, const void *neg_in, void *pos_out, void *neg_out,
                     const double *xs, const double *ys, int64_t n_tracks, uint32_t *counts, double *tally,
                     uintptr_t stream);

/*
 * pic_step_noalloc_status -- the status word of pic_step_noalloc's static
 * workspace: 0, or the code of a bounded wait of the streaming step that ran
 * out (the fields of that step are then wrong). Waits for `stream` first.
 * With reset != 0 it also clears the word and the tally completion counter.
 * Allocates nothing. No counterpart in the reference; it exists because the
 * caller of pic_step_noalloc never sees the workspace that pic_workspace_status
 * would need.
 */
int pic_step_noalloc_status(int32_t reset, uintptr_t stream, int32_t *status);

/*
 * pic_sample_disc -- the rejection step of the host track sampler (no GPU).
 * Replaces the block loop of CylinderSampler.sample
 * (pulsed_ion_chamber/pulses.py:84-171; per track :64-82): pair a of the
 * caller's uniforms u[0 .. 2*n_pairs) gives x = u[2a] * scale,
 * y = u[2a+1] * scale, accepted when (x-mid)^2 + (y-mid)^2 <= radius_sq, in
 * float64 with one rounding per operation (bit-identical to the reference's
 * NumPy expression). Scans pairs in order until n_wanted centres are accepted
 * or the pairs run out; writes the centres to xs/ys and sets *n_accepted and
 * *n_pairs_used (pairs consumed, including the last accepted one).
 */
int pic_sample_disc(const double *u, int64_t n_pairs, double scale, double mid, double radius_sq, int64_t n_wanted,
                    double *xs, double *ys, int64_t *n_accepted, int64_t *n_pairs_used);

/*
 * pic_sample_disc_pcg64 -- the same scan, drawing the uniforms itself from a
 * NumPy PCG64 generator's state (the reference seeds np.random.default_rng,
 * a PCG64): state[4] = {state_hi, state_lo, inc_hi, inc_lo} as in
 * bit_generator.state. Each uniform is one PCG64 XSL-RR 128/64 output
 * converted as NumPy's random() does ((out >> 11) * 2^-53), so the centres are
 * bit-identical to drawing with the generator and scanning as above. Stops at
 * n_wanted accepted centres or after max_pairs pairs; advances state[0..1]
 * past exactly the *n_draws uniforms it consumed (the caller writes the state
 * back to its generator). No counterpart in the reference as a function: it
 * fuses the reference's draw (pulses.py:84-171) and scan.
 */
int pic_sample_disc_pcg64(uint64_t *state, double scale, double mid, double radius_sq, int64_t n_wanted,
                          int64_t max_pairs, double *xs, double *ys, int64_t *n_accepted, int64_t *n_draws);

/*
 * pic_arrival_counts_pcg64 -- tracks arriving in each time step of one pulse
 * (host, no GPU), replacing pulse_arrival_counts (pulsed_ion_chamber/pulses.py:
 * 39-61) for a NumPy PCG64 generator: n uniforms drawn as random(n) draws
 * them, arrival = cumsum / cumsum[-1] * duration, then counts[b] = the
 * arrivals in [edges[b], edges[b+1]) (the last bin closed), as np.histogram
 * over the n_edges edges; bit-identical. Advances state[0..1] past the n
 * draws.
 */
int pic_arrival_counts_pcg64(uint64_t *state, int64_t n, double duration, const double *edges, int64_t n_edges,
                             int64_t *counts);

/*
 * Adjoint of the fused step (no counterpart in the reference, which has no
 * derivatives): reverse-mode derivatives of R, the run's total recombined
 * charge, for k_s = I / (I - R).
 *
 * pic_adjoint_step -- one step backwards. Given the state u_s that step s
 * read (pos/neg), its deposition pairs (dens, or NULL when the step deposited
 * nothing) and lambda_{s+1} = dR/du_{s+1} (lam_*_in), writes
 * lambda_s = dR/du_s (lam_*_out) and grad[0..4] = this step's contribution to
 * dR/ds+, dR/dc+, dR/ds-, dR/dc-, dR/d(alpha_dt), where s = D dt / h^2 and
 * c = mu E dt / h are each species' diffusion and Courant numbers (the
 * descriptor's weights are lat = s, zm = s + c(c+1)/2, zp = s + c(c-1)/2,
 * cen = 1 - c^2 - 6s), at fixed dt. Reflecting wall: lam_*_in
 * is modified (the ring's adjoint is folded into the interior columns it
 * copies). lambda is zero on the z end planes (k = 0, nzb-1) and the row
 * padding: lam_*_out is written so, and lam_*_in must be so (u there is fixed
 * at zero; lambda_{n_steps} = 0 and every step keep it). Workspace:
 * pic_adjoint_workspace_bytes, zeroed once.
 */
int pic_adjoint_workspace_bytes(const pic_grid *g, int64_t *bytes);
int pic_adjoint_step(const pic_grid *g, const void *pos, const void *neg, const void *dens, void *lam_pos_in,
                     void *lam_neg_in, void *lam_pos_out, void *lam_neg_out, double *grad, void *workspace,
                     int64_t workspace_bytes, uintptr_t stream);

/*
 * pic_adjoint_forward -- the forward pass of a checkpointed gradient:
 * n_steps steps over the field pair (state s in (pos0, neg0) for even s,
 * (pos1, neg1) for odd s; state 0 in pair 0 on entry), tallies into
 * tally[4*s ..], the track histogram into counts. Before step
 * c * ckpt_every it copies the state into checkpoint c
 * (ckpt_pos/neg + c * state_stride elements; state_stride >= no_xy^2 *
 * kpitch, a multiple of 8). Every step with tracks keeps its deposition: the
 * d-th such step deposits into slot d of dens_keep
 * ([n_dep][no_xy][pic_dens_pitch] pairs, cleared here first), which the backward
 * pass reads instead of depositing again. Workspace as pic_step.
 */
int pic_adjoint_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                        const double *xs, const double *ys, const int64_t *track_offsets, void *dens_keep,
                        uint32_t *counts, double *tally, void *ckpt_pos, void *ckpt_neg, int64_t ckpt_every,
                        int64_t state_stride, void *workspace, int64_t workspace_bytes, uintptr_t stream);

/*
 * pic_adjoint_backward -- the reverse sweep: for each checkpoint segment from
 * the last, recompute the segment's states from its checkpoint into
 * states_pos/neg (ckpt_every states, state_stride apart; kept densities, no
 * deposition, no tallies), then run the adjoint
 * steps over them backwards. lambda starts at zero in buffer 0 of
 * (lam_*0, lam_*1) (both zeroed by the caller); lambda_0 ends in buffer
 * n_steps & 1. grad[0..4] receives dR/d(s+, c+, s-, c-, alpha_dt) summed
 * over all steps (each step's terms as pic_adjoint_step's). Workspaces: the
 * step's (pic_step_workspace_bytes) and the adjoint's
 * (pic_adjoint_workspace_bytes), each zeroed once.
 */
int pic_adjoint_backward(const pic_grid *g, const void *ckpt_pos, const void *ckpt_neg, int64_t state_stride,
                         int64_t n_steps, int64_t ckpt_every, const int64_t *track_offsets, const void *dens_keep,
                         void *states_pos, void *states_neg, void *lam_pos0, void *lam_neg0, void *lam_pos1,
                         void *lam_neg1, double *grad, void *workspace,
                         int64_t workspace_bytes, void *adj_workspace, int64_t adj_workspace_bytes, uintptr_t stream);

/*
 * Binomial checkpointing (no counterpart in the reference, which has no
 * adjoint): the gradient of a run too long for pic_adjoint_forward/_backward's
 * kept densities and checkpoint segments, in a fixed number of state slots.
 * The schedule is the binomial one of Griewank ("revolve", ACM TOMS 26, 2000):
 * with n_slots slots (the initial state's included), n_steps steps are
 * reversed with the fewest recomputed steps; no deposition is kept, a
 * recomputed step deposits its tracks again into the one scratch pair buffer
 * `dens` ([no_xy][pic_dens_pitch] pairs, 16-byte aligned).
 *
 * pic_revolve_plan -- no device work: *recompute_steps = the steps the
 * backward pass recomputes, *spine_levels = the states the forward stores.
 * pic_revolve_spine -- the steps whose states the forward stores, slot q
 * holding steps[q] (up to cap entries; *n_levels = how many).
 * pic_revolve_trace -- no device work: runs the backward schedule against a
 * bookkeeping of the slots, failing if any step's adjoint would run without
 * its state; events[4*e ..] = (1, s0, n, slot or -1) for "advance n steps
 * from step s0" and (2, s, slot or -1, 0) for "adjoint step s" (up to cap
 * events; *n_events = how many); *advanced = recomputed steps.
 *
 * pic_revolve_forward -- the forward pass: as pic_adjoint_forward (state s in
 * pair s & 1, tallies into tally[4*s ..], histogram into counts), storing the
 * spine states into slots_pos/neg + slot * state_stride elements.
 * pic_revolve_backward -- the reverse sweep from those slots (same n_steps,
 * n_slots, tracks): work_* are two scratch field pairs (e.g. the forward's),
 * lambda as pic_adjoint_backward (zeroed by the caller, starts in buffer 0,
 * lambda_0 ends in buffer n_steps & 1), grad[0..4] = dR/d(s+, c+, s-, c-,
 * alpha_dt) summed over all steps.
 */
int pic_revolve_plan(int64_t n_steps, int64_t n_slots, int64_t *recompute_steps, int64_t *spine_levels);
int pic_revolve_spine(int64_t n_steps, int64_t n_slots, int64_t *steps, int64_t cap, int64_t *n_levels);
int pic_revolve_trace(int64_t n_steps, int64_t n_slots, int64_t *events, int64_t cap, int64_t *n_events,
                      int64_t *advanced);
int pic_revolve_forward(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t n_steps,
                        const double *xs, const double *ys, const int64_t *track_offsets, void *dens,
                        uint32_t *counts, double *tally, void *slots_pos, void *slots_neg, int64_t state_stride,
                        int64_t n_slots, void *workspace, int64_t workspace_bytes, uintptr_t stream);
int pic_revolve_backward(const pic_grid *g, void *slots_pos, void *slots_neg, int64_t state_stride, int64_t n_slots,
                         int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                         void *dens, void *work_pos0, void *work_neg0, void *work_pos1, void *work_neg1,
                         void *lam_pos0, void *lam_neg0, void *lam_pos1, void *lam_neg1, double *grad,
                         void *workspace, int64_t workspace_bytes, void *adj_workspace, int64_t adj_workspace_bytes,
                         uintptr_t stream);

/*
 * pic_selftest_waits -- no counterpart in the reference: runs the kernels'
 * two bounded waits against partners that never come, with short limits --
 * the device-wide barrier of the persistent and multi-step kernels with one
 * block that never arrives, and an mbarrier of the streaming kernels that
 * nothing arrives on -- and returns the status codes they leave (5 for the
 * barrier, 91 for the mbarrier: an expired wait). Neither faults or hangs;
 * the context stays usable.
 */
int pic_selftest_waits(int32_t *barrier_status, int32_t *mbarrier_status, uintptr_t stream);

/*
 * pic_capture_begin / pic_capture_end -- record every launch the library
 * issues on `stream` between the two calls (made from this host thread) into
 * a CUDA graph, instantiated and returned in *graph_out (replay with
 * pic_graph_launch, free with pic_graph_destroy). `stream` must be a stream
 * the caller created, not the default stream. Nothing runs while capturing:
 * host-side checks still happen, device work only at replay. Used to replay a
 * whole adjoint pass (pic_adjoint_forward / _backward) as one graph. No
 * counterpart in the reference.
 */
int pic_capture_begin(uintptr_t stream);
int pic_capture_end(uintptr_t stream, uintptr_t *graph_out);

/*
 * pic_run_segment -- n_steps consecutive time steps on the device.
 *
 * Step s (0-based within the segment) reads fields[(parity + s) & 1] and
 * writes fields[(parity + s + 1) & 1], where fields[b] = (pos_b, neg_b).
 * Its tracks are xs/ys[track_offsets[s] .. track_offsets[s+1]) (host array of
 * n_steps + 1 offsets into the device track arrays). Tallies go to
 * tally[4*s .. 4*s+3] (device). dens0/dens1 alternate as the density buffer;
 * both must be zero on the first call of a run.
 *
 * Replaces the per-step loop of run_simulation_numba_parallel /
 * run_simulation_cuda (solver_numba_parallel.py:600-707,
 * solver_cuda.py:791-872), without the per-step host synchronisation.
 */
int pic_run_segment(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                    int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                    void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                    void *workspace, int64_t workspace_bytes, uintptr_t stream);

/*
 * CUDA-graph form of pic_run_segment: the same launches captured once and
 * replayed. The graph bakes in every pointer and the track offsets, so a
 * replay is only valid with the same buffers; pic_graph_launch replays it on
 * a stream. Used to replay a pulse's step sequence (every pulse has the same
 * per-step track counts) and fixed-length idle segments.
 */
int pic_graph_create(const pic_grid *g, void *pos0, void *neg0, void *pos1, void *neg1, int64_t parity,
                     int64_t n_steps, const double *xs, const double *ys, const int64_t *track_offsets,
                     void *dens0, void *dens1, int64_t dens_parity, uint32_t *counts, double *tally,
                     void *workspace, int64_t workspace_bytes, uintptr_t stream, uintptr_t *graph_out);
int pic_graph_launch(uintptr_t graph, uintptr_t stream);
int pic_graph_destroy(uintptr_t graph);

/* Kernel launches this library has issued in this process: every launch of
 * every entry point, and for each replay of a graph (pic_graph_launch) the
 * launches captured into it (those do not count when captured). Host-only;
 * no counterpart in the reference: the figure a benchmark reports as its
 * kernel count. */
int64_t pic_kernel_launches(void);

/*
 * Batched runs: many independent grids advanced together.
 *
 * Each grid occupies its own block of packed device buffers, described by a
 * pic_batch_cfg entry (its pic_grid scalars -- launch-shape fields ignored --
 * and its offsets). One global step advances every active grid by one of its
 * own time steps, with two launches for the whole batch: a deposition over
 * the step's tracks of all grids (a task list gives each grid's tracks; each
 * 64 x 64 tile of a grid's deposition sums the tracks that reach it) and the
 * flat fused step over a work table that gives each block
 * one grid and a contiguous range of that grid's items (a grid's blocks are
 * consecutive; its last block to finish writes its tallies). Grids that have
 * finished are left out of the work table and task list of later steps.
 *
 * Replaces running the reference's driver once per configuration
 * (run_simulation_numba, solver_numba.py:237-370) for a parameter sweep.
 */
typedef struct pic_batch_cfg {
    int64_t field_off;  /* element offset of the grid's [no_xy][no_xy][kpitch] fields    */
    int64_t dens_off;   /* pair offset of its [no_xy][dens_pitch] deposition pairs     */
    int64_t counts_off; /* offset of its [no_xy][no_xy] track histogram                */
    int64_t tally_off;  /* row offset of its [steps][4] tallies                         */
    pic_grid grid;      /* the grid's scalars (dtype must match the batch)             */
} pic_batch_cfg;

typedef struct pic_batch_launch {
    const pic_batch_cfg *cfgs;             /* device, n_cfgs entries                         */
    int32_t n_cfgs;
    int32_t dtype;                         /* PIC_F32 or PIC_F64, for every grid             */
    const int32_t *blk_cfg;                /* device, per block: its grid                    */
    const int64_t *blk_item0, *blk_item1;  /* device, per block: its item range              */
    int32_t n_blocks;
    int32_t index32;                       /* 1: every grid has no_xy <= 16383 and          */
                                           /*  no_xy^2 * kpitch < 2^31 (32-bit offsets, the  */
                                           /*  faster decode); 0: 64-bit offsets (any grid)  */
    const int32_t *cfg_blk0, *cfg_nblk;    /* device, per grid: first block, block count     */
    void *pos[2], *neg[2];                 /* device, packed fields of time levels 0 and 1   */
    void *dens[2];                         /* device, packed deposition pairs, by step parity */
    const double *xs, *ys;                 /* device, packed track centres                   */
    const int32_t *task_cfg;               /* device, per task (grid, tracks of one step):   */
    const int64_t *task_first;             /*   grid, first track, and the step's tracks     */
    const int64_t *task_prefix;            /*   before the task                              */
    const int64_t *step_task_off;          /* host, n_steps + 1: the steps' task ranges      */
    const int64_t *step_tracks;            /* host, n_steps: tracks deposited in each step   */
    const int64_t *step_blocks;            /* host, n_steps: blocks of each step's           */
                                           /*  deposition, the sum over its tasks of         */
                                           /*  ceil(no_xy/64)^2 x min(32, max(1, ceil(tracks */
                                           /*  of the task / 32)))                           */
    int64_t first_step, n_steps;           /* global steps [first_step, first_step+n_steps)  */
    uint32_t *counts;                      /* device, packed track histograms                */
    double *tally;                         /* device, packed [rows][4] tallies               */
    void *workspace;                       /* device, pic_batched_workspace_bytes, zeroed    */
    int64_t workspace_bytes;
    /* The binned deposition (every grid's tracks listed per 62 x 62-cell
     * tile, summed by one block per tile in a fixed order, each cell stored
     * once), up to 8 global steps per pair of launches, each step's pairs in
     * a buffer of the deposition workspace (pic_batched_segment; the
     * streaming step deposits one global step at a time into dens). With
     * dep_workspace null: the tile form (step_blocks). Needs n_cfgs <= 1024
     * and every grid's cutoff_voxels < 31.5 (boxes of at most 64 cells). */
    void *dep_workspace;                   /* device, pic_batched_deposit_bytes, zeroed once */
    int64_t dep_workspace_bytes;
    int64_t dep_max_tracks;                /* the most tracks of 8 consecutive global steps  */
    int64_t dep_dens_bytes;                /* bytes of one packed pair buffer (dens[0])      */
    int32_t dep_total_tiles;               /* sum over the grids of ceil(no_xy / 62)^2       */
    int32_t dep_max_tiles;                 /* the largest of those                           */
} pic_batch_launch;

/* Workspace of a batched launch with n_blocks blocks and n_cfgs grids. */
int pic_batched_workspace_bytes(int32_t n_blocks, int32_t n_cfgs, int64_t *bytes);

/* Workspace of the binned batched deposition: for each of 8 steps a slot
 * per grid, the per-tile track counts and lists of total_tiles tiles and a
 * packed pair buffer of dens_bytes; the boxes and factors of max_tracks
 * tracks in the field type (dtype). */
int pic_batched_deposit_bytes(int32_t n_cfgs, int32_t total_tiles, int64_t max_tracks, int64_t dens_bytes,
                              int32_t dtype, int64_t *bytes);

/* Runs global steps [first_step, first_step + n_steps) of a batch. Step s
 * reads time level s & 1 and density buffer s & 1, writes level (s+1) & 1
 * and clears density buffer (s+1) & 1; both density buffers must be zero
 * before step 0. */
int pic_batched_segment(const pic_batch_launch *launch, uintptr_t stream);

/* The same launches captured into a CUDA graph (replay with
 * pic_graph_launch, free with pic_graph_destroy). */
int pic_batched_graph_create(const pic_batch_launch *launch, uintptr_t stream, uintptr_t *graph_out);

/* The same global steps in ONE persistent launch (a cooperative launch, one
 * block per resident slot): per step the deposition of every grid's tracks
 * and the fused step over the work table, separated by device-wide barriers
 * whose waits are bounded. step_task_off_dev / step_tracks_dev are device
 * copies of the step tables indexed by GLOBAL step (launch->step_task_off /
 * step_tracks, the host copies for this chunk, are still required: they are
 * validated). After the run, pic_batched_status reads the status word: 0, or
 * 5 when a barrier wait gave up after its bounded polls (the results are then
 * invalid). The workspace is pic_batched_workspace_bytes, zeroed once. */
int pic_batched_persistent(const pic_batch_launch *launch, const int64_t *step_task_off_dev,
                           const int64_t *step_tracks_dev, uintptr_t stream);
int pic_batched_status(const pic_batch_launch *launch, uintptr_t stream, int32_t *status);

/*
 * The streaming batched step: the same global steps as pic_batched_segment,
 * with the fused step of every active grid run by the streaming kernel (whole
 * (row-tile x k) planes staged in a shared-memory ring by bulk asynchronous
 * copies) over a table of work items from all grids, which the CTAs take from
 * a device-wide queue. float32 batches only. Replaces, like
 * pic_batched_segment, running the reference's driver once per configuration
 * (solver_numba_parallel.py:526-723) for a parameter sweep.
 *
 * An item is four int32: grid c, the first interior row cj_lo of its tile
 * (rows cj_lo .. min(cj_lo + tile_rows[c], no_xy - 1) - 1), and its interior
 * planes [ci_lo, ci_hi); every interior row and plane of every active grid
 * must be covered exactly once, and the items of a grid must be consecutive
 * in the table (grids without items are not stepped). tile_rows[c] x
 * kpitch/4 must be <= 3 x 32 x consumer_warps.
 *
 * pic_batched_stream_prepare validates the host tables (cfgs_host is the host
 * copy of launch->cfgs), uploads them into the workspace
 * (pic_batched_stream_workspace_bytes, 256-byte aligned; clears its counters)
 * and fills *out, the launch shape the segment calls take. It waits for the
 * upload, so the host tables may be released when it returns. Call it again
 * whenever the item table changes (a grid finished).
 * pic_batched_stream_segment runs global steps [first_step, first_step +
 * n_steps) of `launch` (its task tables and buffers; its flat work table and
 * workspace are not used) with the prepared tables. The deposition is the
 * one pic_batched_segment runs: binned, up to 8 global steps per launch pair,
 * when launch->dep_workspace is set, else the tile form.
 * pic_batched_stream_status reads the workspace's status word: 0, 1-3 when a
 * bounded wait of the copy ring ran out, 7 when an item was refused on the
 * device; with reset != 0 a non-zero word is cleared together with the queue
 * and grid counters the aborted step left behind.
 */
typedef struct pic_batch_stream {
    int32_t n_cfgs, n_items;
    int32_t consumer_warps; /* compute warps per CTA (1 .. 15)               */
    int32_t stages;         /* ring stages that fit the largest stage        */
    int32_t stage_floats;   /* floats of one stage (the largest grid's)      */
    int32_t ipt;            /* k-vectors per consumer thread (1 .. 3)        */
    void *workspace;
    int64_t workspace_bytes;
} pic_batch_stream;

int pic_batched_stream_workspace_bytes(int32_t n_cfgs, int32_t n_items, int32_t consumer_warps, int64_t *bytes);
int pic_batched_stream_prepare(const pic_batch_cfg *cfgs_host, int32_t n_cfgs, const int32_t *items_host,
                               int32_t n_items, const int32_t *tile_rows_host, int32_t consumer_warps,
                               void *workspace, int64_t workspace_bytes, uintptr_t stream, pic_batch_stream *out);
int pic_batched_stream_segment(const pic_batch_launch *launch, const pic_batch_stream *bs, uintptr_t stream);
int pic_batched_stream_status(const pic_batch_stream *bs, int32_t reset, uintptr_t stream, int32_t *status);

#ifdef __cplusplus
}
#endif

#endif /* PIC_GB300_H */
