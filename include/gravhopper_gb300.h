/*
 * gravhopper_gb300.h -- C ABI of the GB300 gravity engine (libgravhopper_gb300.so).
 *
 * Plain pointers and sizes only.  Units: code units G=1, length kpc, mass Msun for
 * forces (as gravhopper/_jbgrav.c:137-139); the leapfrog entry points take positions
 * in kpc, velocities in km/s and times in Myr (gravhopper/gravhopper.py:146-151).
 * Arrays of vectors are (N,3) C-contiguous float64, masses (N) float64.
 *
 * Every function returns GH_OK (0) or an error code; gh_last_error() gives the
 * message of the calling thread's last failure.
 *
 * "host" entry points take host pointers, copy to the device, compute and copy back
 * before returning.  "_dev" entry points take device pointers and a cudaStream_t
 * (passed as void*, NULL = legacy default stream) and are stream-ordered: they return
 * once the work is enqueued.  The library keeps one grow-only device workspace per
 * device; calls that use it must not run concurrently on different streams.
 */
#ifndef GRAVHOPPER_GB300_H
#define GRAVHOPPER_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GH_VERSION 100

/* status codes */
#define GH_OK 0
#define GH_ERR_ARG 1       /* invalid argument: negative size, NULL buffer, unknown enum */
#define GH_ERR_SHAPE 2     /* inconsistent shapes (host mirrors raise RuntimeError) */
#define GH_ERR_OOM 3       /* device allocation failed */
#define GH_ERR_DEPTH 4     /* octree deeper than supported: coincident particles */
#define GH_ERR_TIMEOUT 5   /* a bounded device-side wait gave up */
#define GH_ERR_CUDA 6      /* CUDA runtime error */
#define GH_ERR_NO_DEVICE 7 /* no usable CUDA device */

/* precision of the direct-sum pair arithmetic */
#define GH_PREC_FP64 0  /* FP64 throughout, bit-exact with the reference's operation order */
#define GH_PREC_MIXED 1 /* FP32 pairs, compensated per-particle accumulation, FP64 state */

/* force algorithm, as Simulation.params['algorithm'] (gravhopper/gravhopper.py:255-274) */
#define GH_ALGO_DIRECT 0
#define GH_ALGO_TREE 1

/* ---- library ------------------------------------------------------------------ */
const char* gh_last_error(void);
int gh_version(void);
/* Number of kernels this library has launched since load (all threads). */
int64_t gh_launch_count(void);
/* Enables (1) or disables (0) NVTX ranges around the library's calls, leapfrog steps,
 * tree builds and walks, for NVTX-aware profilers (no counterpart in the reference). */
int gh_trace(int enable);

/* ---- host-buffer drop-ins for the reference module gravhopper._jbgrav --------- */

/* Replaces _jbgrav.direct_summation(pos, mass, eps), gravhopper/_jbgrav.c:68-193.
 * pos (np,3), mass (np) -> out (np,3) in code units.  FP64, bit-exact. */
int gh_direct_summation(const double* pos, const double* mass, int64_t np, double eps,
                        double* out);

/* Replaces _jbgrav.direct_summation_position(pos, mass, force_pos, eps),
 * gravhopper/_jbgrav.c:200-353.  force_pos (nf,3) -> out (nf,3).  A target that
 * coincides with a particle when eps == 0 gets no term from it (r^2+eps^2 == 0). */
int gh_direct_summation_position(const double* pos, const double* mass, int64_t np,
                                 const double* force_pos, int64_t nf, double eps, double* out);

/* Replaces _jbgrav.tree_force(pos, mass, eps, theta), gravhopper/_jbgrav.c:564-630 and
 * treeforce_workhorse :737-806.  Barnes-Hut octree with the reference's cells,
 * centres and opening test (leaf, or size/|center - x| < theta); monopoles; FP64.
 * Returns GH_ERR_DEPTH for particles that share position to 126 octree levels
 * (the reference recurses without bound on coincident particles). */
int gh_tree_force(const double* pos, const double* mass, int64_t np, double eps, double theta,
                  double* out);

/* Replaces _jbgrav.tree_force_position(pos, mass, force_pos, eps, theta),
 * gravhopper/_jbgrav.c:634-727.  np == 0 gives zeros. */
int gh_tree_force_position(const double* pos, const double* mass, int64_t np, const double* force_pos,
                           int64_t nf, double eps, double theta, double* out);

/* Direct sum with a precision choice (GH_PREC_*).  force_pos == NULL: targets are
 * the particles themselves and the self term is skipped (direct_summation). */
int gh_direct_host(const double* pos, const double* mass, int64_t np, const double* force_pos,
                   int64_t nf, double eps, int precision, double* out);

/* ---- device-pointer, stream-ordered ------------------------------------------- */

/* Direct-sum acceleration (code units) into acc (nf,3), or (np,3) when
 * force_pos == NULL (self term skipped). */
int gh_direct_dev(const double* pos, const double* mass, int64_t np, const double* force_pos,
                  int64_t nf, double eps, int precision, double* acc, void* stream);

/* Barnes-Hut acceleration (code units) into acc (nf,3), or (np,3) when force_pos == NULL.
 * Opening decisions are the reference's in both precisions; GH_PREC_MIXED evaluates the
 * accepted cells' monopoles in FP32 on hi/lo split coordinates with compensated sums. */
int gh_tree_dev(const double* pos, const double* mass, int64_t np, const double* force_pos, int64_t nf,
                double eps, double theta, int precision, double* acc, void* stream);

/* Advances (pos, vel) in place by nsteps drift-kick-drift leapfrog steps
 * (Simulation.perform_timestep, gravhopper/gravhopper.py:405-416): pos [kpc],
 * vel [km/s], mass [Msun], dt [Myr], eps [kpc].  algorithm GH_ALGO_DIRECT uses
 * `precision`; GH_ALGO_TREE uses `theta` and `precision` (the walk's interactions).  When hist_pos/hist_vel are
 * non-NULL, the state after every hist_stride-th step is written to consecutive
 * (np,3) slots of them (nsteps/hist_stride slots). */
int gh_run_dkd(double* pos, double* vel, const double* mass, int64_t np, int64_t nsteps,
               double dt, double eps, int algorithm, int precision, double theta,
               double* hist_pos, double* hist_vel, int64_t hist_stride, void* stream);

/* The leapfrog step of gh_run_dkd in two launches, for runs whose acceleration has a
 * part computed outside this library (the external forces of
 * Simulation.calculate_extra_acceleration, gravhopper/gravhopper.py:462-473).
 * gh_dkd_drift: pos_half = pos + ((0.5 vel) dt) F, F = km Myr/s in kpc (the first
 * drift of Simulation.perform_timestep, gravhopper.py:405-416); all device (np,3)
 * buffers, pos_half may be pos.  gh_dkd_kick_drift: vel += ((acc ACC) + acc_ext) dt,
 * then pos_out = pos_half + ((0.5 vel) dt) F, with acc the N-body acceleration in code
 * units (as gh_direct_dev and gh_tree_dev give it; NULL for none, as for np <= 1,
 * gravhopper.py:457-458), ACC = G Msun/kpc^2 in km/s/Myr (jbgrav.py:40-48), and
 * acc_ext the external acceleration in km/s/Myr (NULL for none): the reference's
 * nbody + extra (gravhopper.py:459).  No FMA contraction, as in gh_run_dkd. */
int gh_dkd_drift(const double* pos, const double* vel, int64_t np, double dt, double* pos_half, void* stream);
int gh_dkd_kick_drift(const double* pos_half, double* vel, const double* acc, const double* acc_ext, int64_t np,
                      double dt, double* pos_out, void* stream);

/* Mixed-precision direct-sum self-force (as gh_direct_dev with force_pos == NULL and
 * GH_PREC_MIXED) that allocates no device memory.  No counterpart in the reference:
 * it is for callers that cannot let a library allocate, such as an application
 * that owns all device memory through its own pool, or a stepping loop that must not
 * call cudaMalloc/cudaFree because those can synchronise the device.  The caller
 * passes device inputs pos (np,3), mass (np) and the output acc (np,3); all scratch
 * lives in one fixed ~16 MiB array in this library's device memory, held by every GPU
 * that loads the library until the process exits.  np above 65536 is rejected with
 * GH_ERR_ARG.  Each call made outside stream capture looks up that array's device
 * address on the current device; a call during capture reuses the last one, so make
 * the first call on a device before any stream capture.  The persistent grid is capped
 * at 304 CTAs (two per SM of a 152-SM GB300) by the array's partial-sum space.  Every
 * call shares the array and finds the previous call's contents in it: calls that
 * overlap on the GPU (different streams, or threads) race and must not be issued. */
int gh_direct_mixed_noalloc(const double* pos, const double* mass, int64_t np, double eps, double* acc,
                            void* stream);

/* Selects the tile shape of the mixed-precision direct kernel (0 .. gh_direct_num_shapes()-1)
 * for all later calls in this process; -1 (the default) picks the shape by problem size.
 * No counterpart in the reference. */
int gh_direct_set_shape(int shape);
int gh_direct_num_shapes(void);

/* Installs an autotuned shape rule for the mixed-precision direct kernel (no
 * counterpart in the reference): from n_min particles on (the rule with the largest
 * n_min <= N applies), calls of kind fused_step (0 a force, 1 a fused leapfrog step)
 * use tile shape `shape`; shape -1 clears that kind's rules.  Sizes below every rule
 * keep the built-in table.  gh_direct_set_shape(k >= 0) overrides the rules. */
int gh_direct_tune(int64_t n_min, int fused_step, int shape);

/* The tile shape a call of N particles of kind fused_step would use now (-1 on bad
 * arguments); no device work. */
int gh_direct_shape_for(int64_t n, int fused_step);

/* Selects the FP64 direct kernel for all later calls in this process: 0 one thread
 * per target, 1 CTA-wide pair terms summed in order per target (for few targets),
 * -1 (the default) by target count.  Both give the reference's bits.  No counterpart
 * in the reference. */
int gh_direct_set_fp64_form(int form);

/* ---- adjoint and diagnostics of the direct sum (no counterpart in the reference) ---- */

/* Vector-Jacobian product of the direct-sum self-acceleration a(x, m) (code units):
 * given the cotangent cot (np,3) of a, writes grad_pos (np,3) = sum_i cot_i . da_i/dx
 * (the softened tidal tensor contracted with cot) and, when grad_mass is non-NULL,
 * grad_mass (np) = sum_i cot_i . da_i/dm.  precision GH_PREC_FP64 or GH_PREC_MIXED. */
int gh_direct_vjp_dev(const double* pos, const double* mass, int64_t np, double eps, const double* cot,
                      int precision, double* grad_pos, double* grad_mass, void* stream);

/* Reverse-mode pass through nsteps direct-sum drift-kick-drift steps that start from
 * the state (x0, v0) (device buffers; same units as gh_run_dkd).  Recomputes the
 * nsteps states from (x0, v0), then back-propagates: on entry (xbar, vbar) hold the
 * cotangents of the state after the last step, on return those of (x0, v0); mbar,
 * when non-NULL, is incremented by the mass gradient.  One checkpoint segment of a
 * differentiable rollout. */
/* The same for a whole checkpointed rollout: ckpt_x, ckpt_v (nseg,np,3) hold the state
 * at the start of each segment, seg_steps (host array, nseg entries) the segments'
 * step counts.  The segments are taken in reverse; each one's states are recomputed
 * on a second stream while the following segment back-propagates on `stream`. */
int gh_dkd_backward_chain_dev(const double* ckpt_x, const double* ckpt_v, const int64_t* seg_steps, int64_t nseg,
                              const double* mass, int64_t np, double dt, double eps, int precision, double* xbar,
                              double* vbar, double* mbar, void* stream);

int gh_dkd_backward_dev(const double* x0, const double* v0, const double* mass, int64_t np, int64_t nsteps,
                        double dt, double eps, int precision, double* xbar, double* vbar, double* mbar,
                        void* stream);

/* Per-particle softened potential phi (np) = -sum_{j != k} m_j / sqrt(r^2 + eps^2), code
 * units (G=1), FP64.  Potential energy = 0.5 * G * sum_k m_k phi_k. */
int gh_potential_dev(const double* pos, const double* mass, int64_t np, double eps, double* phi, void* stream);

/* ---- batched ensembles (no counterpart in the reference) ------------------------- */

/* Advances nsys independent systems by nsteps drift-kick-drift steps each, mixed
 * precision, in one persistent launch per step with the step loop replayed from a
 * CUDA graph when use_graph != 0.  pos/vel/mass: device buffers holding the systems
 * back to back; offsets (host, nsys+1, offsets[0] = 0), eps and dt (host, nsys) give
 * each system's range, softening [kpc] and time step [Myr].  tile_config selects one
 * of gh_ensemble_num_configs() tile shapes (-1: default); the Python autotuner
 * picks it by timing. */
int gh_ensemble_run(double* pos, double* vel, const double* mass, const int64_t* offsets, int64_t nsys,
                    const double* eps, const double* dt, int64_t nsteps, int tile_config, int use_graph,
                    void* stream);
int gh_ensemble_num_configs(void);

/* ---- diagnostics -------------------------------------------------------------- */

/* Measures the current device's FMA-pipe throughput with dependent-chain kernels
 * (no counterpart in the reference): FP32 (packed f32x2) and FP64 FMA lane-operations
 * per second; either pointer may be NULL.  Used as roofline denominators. */
int gh_measure_fma_peaks(double* fp32_lane_ops_per_s, double* fp64_lane_ops_per_s, void* stream);

/* Measures the pairs per second that the mixed direct sum's pair arithmetic reaches on
 * the current device with every operand in registers (12 FMA-pipe instructions and one
 * MUFU rsqrt per pair; with equal_mass != 0 the loop that systems of equal masses run,
 * 11 FMA-pipe instructions; 4 targets per thread, one 512-thread CTA per SM, no memory
 * in the loop): the ceiling of that instruction mix, against which the kernel's pairs
 * per second are compared (no counterpart in the reference). */
int gh_measure_pair_mix(int equal_mass, double* pairs_per_s, void* stream);

/* Enables (1) or disables (0) CUDA-event timing of every force-kernel launch (direct
 * FP64, direct mixed, tree walk) on the stream it is launched on (no counterpart in
 * the reference). */
int gh_kernel_timing(int enable);

/* Synchronises on and sums the recorded launch durations since the last collect:
 * total milliseconds and number of timed launches; clears the record. */
int gh_kernel_timing_collect(double* total_ms, int64_t* launches);

/* Measures the current device's L2 read bandwidth (bytes/s) with 16-byte L1-bypassing
 * loads over a 32 MiB buffer read 64 times (no counterpart in the reference).  The
 * roofline denominator of the tree walk, whose cell records stay in L2. */
int gh_measure_l2_read(double* bytes_per_s, void* stream);

/* Self-check of the integer-pipe softened inverse cube RN(RN(1/s)/RN(sqrt(s))) used
 * by the FP64 direct sum (no counterpart in the reference, whose C code evaluates
 * 1.0/s/sqrt(s) with the FPU, gravhopper/_jbgrav.c:159-166): n seeded inputs on the
 * current device compared bit for bit with the native IEEE operations, half of them
 * also through the integer-pipe squared distance s = dx^2 + dy^2 + dz^2 + eps^2.
 * Writes the number of differing results and of in-range inputs that took the
 * native path. */
int gh_check_inv_cube(int64_t n, uint64_t seed, long long* wrong_fallback, void* stream);

/* Builds the octree of (pos, mass) (device buffers) and checks its invariants (no
 * counterpart in the reference, whose pointer tree has none to check): out holds 9
 * entries, out[0] the number of cells, out[1] the leaves (np when the tree is whole),
 * then violations: out[2] skip indices out of range, out[3] children that do not tile
 * their cell's subtree, out[4] cells with more than 8 child cells, out[5] cell masses
 * that are not the sum of their children's (1e-12 relative), out[6] children whose
 * centre of mass lies outside their cell, out[7] walk records that do not match the
 * FP64 cells, out[8] a root whose subtree is not the whole preorder.  Synchronises. */
int gh_tree_validate(const double* pos, const double* mass, int64_t np, double eps, int64_t* out, void* stream);

/* Enables (1) or disables (0) the tree-walk counters (no counterpart in the
 * reference, which counts nothing).  While enabled every walk adds, over its warps,
 * the cell steps (one 48-byte cell record read per warp step), the cells visited by
 * each target (what a per-target walk would read), the target-cell interactions, the
 * exact FP64 opening tests and the interactions with leaves. */
int gh_tree_stats(int enable);

/* Synchronises the device and returns the counters accumulated since the last read,
 * then clears them (out holds 7 entries): out[0] walks, out[1] warp cell steps,
 * out[2] target cell visits, out[3] interactions, out[4] exact opening tests,
 * out[5] interactions with leaves, out[6] warp steps at cells with a single child
 * cell (the uncompressed octree's chains). */
int gh_tree_stats_read(int64_t* out);

/* ---- fault injection for tests (no counterpart in the reference) ----------------- */

/* Kinds of host-side fault that gh_debug_inject can make the library meet. */
#define GH_INJECT_ALLOC 1     /* a device workspace allocation runs out of memory */
#define GH_INJECT_TREE_WAIT 2 /* a tree build finds its radix sort's bounded wait given up */

/* Makes the next `count` occurrences of `fault` fail on the host as if the device had
 * reported them (0 clears it): GH_INJECT_ALLOC fails workspace reservations with
 * GH_ERR_OOM (the reserved buffer is released, as after a failed growth);
 * GH_INJECT_TREE_WAIT makes tree builds return GH_ERR_TIMEOUT after their sort.  Every
 * later call works normally.  For testing the error paths; no GPU fault is involved. */
int gh_debug_inject(int fault, int64_t count);

/* Runs one pass of the tree build's radix sort over two tiles of keys in which tile 0
 * is never published, so tile 1's bounded look-back wait gives up after wait_ns
 * nanoseconds (GPU global timer) and sets the sort's error flag.  Returns GH_ERR_TIMEOUT
 * when the wait gave up, as it must; *waited_ns, when non-NULL, receives the host time
 * the call took.  Tests the bound without a hang. */
int gh_debug_sort_stall(int64_t wait_ns, int64_t* waited_ns);

#ifdef __cplusplus
}
#endif

#endif /* GRAVHOPPER_GB300_H */
