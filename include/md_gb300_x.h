/*
 * md_gb300_x.h -- what libxmd_x adds to the MD-Lab C ABI: status codes,
 * stream and CUDA-graph control, and explicit release of device state.
 *
 * These have no counterpart in MD-Lab's headers: the reference's OpenCL
 * back end keeps one global queue (md_util_x.c:16-83) and never frees.
 */
#ifndef MD_GB300_X_H
#define MD_GB300_X_H

#include "md_pimd_x.h"

#ifdef __cplusplus
extern "C" {
#endif

/* status codes returned (negated) by every int entry point */
#define MD_GB_OK 0
#define MD_GB_ERR_NO_DEVICE (-1001)   /* no CUDA device / driver */
#define MD_GB_ERR_CUDA (-1002)        /* a CUDA call failed; see md_gb300_last_error_x */
#define MD_GB_ERR_ALLOC (-1003)       /* device or host allocation failed */
#define MD_GB_ERR_UNSUPPORTED (-1004) /* potential / shape this library has no kernel for */
#define MD_GB_ERR_ARG (-1005)         /* invalid argument (NULL, N < 1, P < 2, ...) */
#define MD_GB_ERR_CAPTURE (-1006)     /* operation not allowed while capturing a graph */

/* text of the last failure on this thread ("" if none) */
const char *md_gb300_last_error_x(void);

/* compile-time shape of this library variant */
void md_gb300_variant_x(int *dimension, int *nhc_length);

/* number of CUDA devices (0 when none is usable) */
int md_gb300_device_count_x(void);

/* kernels launched by this library so far (all threads) */
unsigned long long md_gb300_launch_count_x(void);

/* select the CUDA device (one per process); call before any device work */
int md_gb300_set_device_x(int device);

/* all work is ordered on one CUDA stream; by default a non-blocking stream
   created by the library.  Set another (a cudaStream_t) before the first
   device call, or NULL to restore the library's own stream. */
int md_gb300_set_stream_x(void *cuda_stream);
void *md_gb300_get_stream_x(void);
int md_gb300_synchronize_x(void);

/* CUDA graphs: every md_* device call made between begin and end is
   recorded instead of executed; md_gb300_graph_launch_x replays the whole
   sequence count times.  Potential parameters and time steps are frozen
   into the graph.  Device state must already exist (make one ordinary call
   first); host <-> device synchronisation is refused while capturing. */
typedef struct md_gb300_graph md_gb300_graph_t_x;
int md_gb300_capture_begin_x(void);
int md_gb300_capture_end_x(md_gb300_graph_t_x **graph);
int md_gb300_graph_launch_x(md_gb300_graph_t_x *graph, int count);
/* One step of several independent systems as one graph.  The library calls
   step(i, ctx) for i = 0 .. n-1 while capturing, each call's md_* work
   recorded on its own branch stream forked from and joined to the library
   stream; replaying the graph advances every system with one launch, and
   the GPU runs the independent branches concurrently.  step sets whatever
   md_set_* parameters its system needs (they are frozen into the graph) and
   returns 0, or an error code that ends the capture.  Each system's device
   state must exist already (one ordinary step first). */
typedef int (*md_gb300_system_step_fn_x)(int system, void *ctx);
int md_gb300_capture_ensemble_x(int n, md_gb300_system_step_fn_x step, void *ctx, md_gb300_graph_t_x **graph);
/* The same ensemble step as ONE persistent kernel launch (captured into a
   graph): the step's stages are nine phases, each holding that stage's work
   of every system of a group of blocks spread over the group, separated by
   the group's barriers
   (a cooperative launch of exactly the blocks that fit; a barrier wait that
   runs out, about a second, ends the kernel instead of hanging and is
   reported by md_gb300_ensemble_status_x).  While planning, step(i, ctx)'s
   calls do not launch; each records its call and the md_set_* parameters
   of the moment.  Every system's calls must be the reference driver's step,
   in this order: md_update_nhc_VV3_1_x, md_reset_force_x,
   md_pimd_fast_fill_ENk_x, md_pimd_fill_VB_x, md_pimd_fast_fill_force_VB_x,
   optionally md_pimd_calc_trap_force_x and md_pimd_calc_pair_force_x,
   md_update_nhc_VV3_2_x, optionally md_periodic_boundary_x; pair forces in
   MD_GB_PRECISION_MIXED (FP32) with equal bead masses, one-DOF thermostat
   chains of length 4 or 8, P >= 2, N <= 2048, no learned model attached.
   Other calls are refused (MD_GB_ERR_UNSUPPORTED).  The results equal those
   of the per-system calls.  The grid is the shape that
   md_gb300_autotune_ensemble_x chose for this ensemble's shapes, else 2
   blocks per SM in 4 groups. */
int md_gb300_capture_ensemble_persistent_x(int n, md_gb300_system_step_fn_x step, void *ctx,
                                           md_gb300_graph_t_x **graph);
/* 0 when every launch of a persistent ensemble graph so far completed its
   barriers; MD_GB_ERR_CUDA when a barrier wait ran out.  Synchronises. */
int md_gb300_ensemble_status_x(md_gb300_graph_t_x *graph);
/* The last launch's phase durations in microseconds (up to n of them: the
   thermostat's first half and force reset; springs, cycle-energy increments,
   pair tiles and structure factors; prefix sums and force tables; cycle
   energies and reciprocal forces; recursion weights, block inverses and the
   pair sums; the two solves; G; the end-bead exchange forces; the second
   half step), as one block saw them, then that block's own time in the
   second phase for its springs, cycle-energy increments, pair tiles and
   structure factors, then each group's step time; returns the number of
   values (13 + groups).  Synchronises. */
int md_gb300_ensemble_phase_times_x(md_gb300_graph_t_x *graph, double *us, int n);
/* Times the persistent step at each grid shape: 2 or 3 blocks per SM (the
   latter with the kernel compiled for three) and the blocks split into 1,
   2, 4, 8, 16 or 32 groups, each stepping its share of the systems (spread by
   estimated cost) with its own barriers, so that the groups' phases drift
   apart and one group's FP64 thermostat overlaps another's FP32 sums.
   The fastest shape is then rebalanced up to three times: each system's
   estimated cost is scaled by its group's measured time over the group's
   estimate, and the systems are spread again.  Each trial runs `repeats` + 1
   launches, so the systems advance by those steps.  The fastest shape and
   balance are recorded for this ensemble's shapes; *blocks_per_sm, *groups
   and *ms (may be NULL) receive the shape and its time per step. */
int md_gb300_autotune_ensemble_x(int n, md_gb300_system_step_fn_x step, void *ctx, int repeats, int *blocks_per_sm,
                                 int *groups, double *ms);
/* kernel nodes in a captured graph (kernels launched per replay) */
int md_gb300_graph_kernel_count_x(md_gb300_graph_t_x *graph);
void md_gb300_graph_free_x(md_gb300_graph_t_x *graph);

/* live per-kernel timing: while on, every kernel launched outside graph
   capture is bracketed by CUDA events on the library stream.  The report
   (written to buf, NUL-terminated) is "kernel total_ms launches;..." and
   clears the record; returns the report length. */
int md_gb300_profile_x(int on);
int md_gb300_profile_report_x(char *buf, int len);

/* measured FP64 fused-multiply-add throughput of the current GPU, TFLOP/s:
   the roofline denominator of the FP64 kernels (-1 on failure) */
double md_gb300_fp64_peak_x(void);
/* the same for FP32 fused multiply-add (the FP32 kernels' denominator) */
double md_gb300_fp32_peak_x(void);

/* Pair forces for callers that cannot allocate device memory.  No
   counterpart in MD-Lab.  Every other compute call here allocates its device
   copies and scratch on first use; some callers cannot allow that: a host
   application whose own allocator has reserved the GPU's memory up front
   (a framework's caching allocator, a fixed-footprint service), or a plugin
   that must not change the process's device-memory footprint.  This call
   takes the caller's device buffers and stream and allocates nothing: the
   per-tile partial sums use a fixed 4 MiB array inside the library, which
   every GPU that loads the library keeps until the process exits.

   pf     md_gaussian_force_x, md_periodic_gaussian_force_x,
          md_coulomb_force_x or md_coulomb_periodic_force_x (parameters from
          the usual globals); Ewald is not available here
   x, m   device arrays, bead slices major: x[(j*D + d)*ld + l], m[j*ld + l]
          for particle l < N, bead j < P, dimension d < D
   f      device array laid out like x; receives += the pair forces of each
          bead slice with the reference's convention (F/(m P), m of the
          higher-index particle; md_pimd_x.c:1650-1675)
   ld     leading dimension, ld >= N
   L      host array of D box lengths (needed by the periodic kinds)
   stream cudaStream_t to run on (NULL: the legacy default stream)

   Limit: ceil(N/32) * P * D * ld <= 524288 doubles (for example N = 256,
   P = 64 in 3D); larger configurations are refused with MD_GB_ERR_ARG.
   The arithmetic is always FP64 (the MD_GB_PRECISION_FP64 kernel), whatever
   md_gb300_set_precision_x selected for the other calls.
   The first call on each device looks up the array's device address with
   that device current.  All calls share the array, so calls that overlap
   on the GPU (different streams, or several host threads) race; nothing in
   the array needs clearing between calls.  A launch error left pending by
   the caller's own earlier work is reported as MD_GB_ERR_CUDA before this
   call launches anything. */
int md_gb300_pair_force_noalloc_x(md_pair_force_t_x pf, const double *x, const double *m, double *f, int N, int P,
                                  int ld, const double *L, void *stream);

/* Arithmetic of the pair forces (md_pimd_calc_pair_force_x), including
   both Ewald parts.  MD_GB_PRECISION_FP64 (default) reproduces MD-Lab to
   1e-10: every term is FP64 except two groups of small ones, evaluated on
   the FP32 pipe: the real-space Ewald images at alpha R >= 4 (each below
   5.2e-7 of the pair strength over R^2; added to the FP64 sum per pair),
   and the reciprocal wave-vector columns (nx, ny) whose every vector has a
   force weight |G| c(n) below 1e-7 of the largest (FP32 structure factors,
   tables and compensated column sums).  Against
   MD_GB_PRECISION_FP64_STRICT, which evaluates those in FP64 too, the
   forces of the 512-electron, 64-bead electron gas (Ewald |n| <= 10) differ
   by 2.4e-16 of the largest and by at most 6.8e-12 of any bead's own.
   MD_GB_PRECISION_MIXED evaluates pair and real-space Ewald forces in
   FP32: each lane adds at most 32 FP32 pair terms (one 32 x 32 tile), and
   the tile partials are added in FP64; the reciprocal sum builds its
   structure factors from FP32 phase products, summed in FP32 over 16
   particles at a time and those partial sums in double-float (two-sum),
   then FP32 force tables and compensated (Kahan) column sums per particle.
   Positions, the exchange recursion, springs, the thermostat and every
   estimator stay FP64.  The force error against the FP64 form, measured as
   max |f32 - f64| / max |f64| over all beads of the 512-electron, 64-bead
   electron gas (Ewald |n| <= 10), is 1.1e-5 and set mainly by the FP32
   rounding of the pair separations; the library's tests bound it by 5e-5
   there and on the smaller systems they run. */
/* Tile shape of the FP32 pair kernel (the mixed form) for pimd's system
   shape, chosen by timing: warps of 32 x 32 pair tiles per thread block, 1,
   2, 4 or 8 (small systems in an ensemble spread better over the SMs with
   small blocks).  The choice is kept for this potential kind, D, N and P
   and used by md_pimd_calc_pair_force_x; the forces do not depend on it.
   *warps and *ms (may be NULL) receive the choice and its time per call. */
int md_gb300_autotune_pair_x(md_pimd_t_x *pimd, md_pair_force_t_x pf, int repeats, int *warps, double *ms);
/* set that choice directly (a tuning table kept by the caller) */
int md_gb300_set_pair_tile_x(md_pair_force_t_x pf, int N, int P, int warps);
/* The FP64 form's launch shapes for pimd's system shape, chosen by timing:
   the tile kernels' thread blocks per SM (1 or 2, *blocks_per_sm) and, for
   md_coulomb_3d_ewald_force_x, the structure-factor kernel's layout
   (*sk_layout: 1 = 16 columns x 16 particle groups per block, 2 = 8 x 32,
   3 = 64 columns, one thread each; 0 for the other potentials).  The choices
   are kept for this potential kind, N, P (and n_sum) and used by the FP64
   force calls; the forces agree to rounding whatever the choice.  *ms: the
   time of one force call's tiles plus reciprocal sum with the choices. */
int md_gb300_autotune_fp64_x(md_pimd_t_x *pimd, md_pair_force_t_x pf, int repeats, int *blocks_per_sm,
                             int *sk_layout, double *ms);

/* Which kernel solves the exchange recursions (V_B and the backward tmpV,
   md_pimd_fill_VB_x and the force call): MD_GB_SOLVE_BLOCK runs one thread
   block per direction, MD_GB_SOLVE_CLUSTER one cluster of eight blocks per
   direction (distributed shared memory), MD_GB_SOLVE_AUTO (default) picks
   per N: a choice recorded by md_gb300_autotune_solve_x, else the cluster
   from N = 129 on.  All paths give the same values to rounding.  Forcing
   the cluster where none of its size fits makes the recursion calls fail
   with MD_GB_ERR_CUDA.  md_gb300_get_solve_path_x(N) returns the path that
   N uses (N < 1: the forced setting). */
#define MD_GB_SOLVE_AUTO 0
#define MD_GB_SOLVE_BLOCK 1
#define MD_GB_SOLVE_CLUSTER 2
int md_gb300_set_solve_path_x(int path);
int md_gb300_get_solve_path_x(int N);
/* Times both solve kernels on pimd's current cycle energies (scratch
   outputs; pimd's V_B and tmpV are untouched) and records the faster one
   for pimd's N; *path and *ms (may be NULL) receive it and its time. */
int md_gb300_autotune_solve_x(md_pimd_t_x *pimd, int repeats, int *path, double *ms);
/* Host copies of the backward recursion tmpV[0..N] and the connection
   probabilities G[(l-1)*N + (j-1)] (md_pimd_x.c:2588-2673) left by the last
   md_pimd_fast_fill_force_VB_x (either may be NULL); synchronises. */
int md_gb300_exchange_tables_x(md_pimd_t_x *pimd, double *tmpV, double *G);

#define MD_GB_PRECISION_FP64 0
#define MD_GB_PRECISION_MIXED 1
#define MD_GB_PRECISION_FP64_STRICT 2
int md_gb300_set_precision_x(int mode);
int md_gb300_get_precision_x(void);

/* ---- learned Ewald residual (no counterpart in MD-Lab) ----
   A network of 64 -> 128 -> 128 -> 4 units (tanh, BF16 weights and
   activations, FP32 accumulation on the tcgen05 tensor cores) predicts, per
   bead slice and particle, the difference between the converged Ewald
   reciprocal sum (n_sum from md_set_coulomb_*) and a truncated one
   (n_sum_cheap): an energy and the coefficients of three vector features
   that give the force.  Inputs are 64 descriptors per particle: 32 Gaussian
   radial functions (centres 0.5 .. L/2) of the particle's minimum-image
   neighbours within half the box, and |S(k)| of its bead slice on the 32
   lowest reciprocal-lattice shells (the root mean square of |S(k)|/sqrt(N)
   over each shell).  A model belongs to one system shape (N, P, box, Ewald
   alpha and strength) and lives on the GPU. */
typedef struct md_gb300_ewald_model md_gb300_ewald_model_t_x;
int md_gb300_ewald_model_nparam_x(void);
/* capacity: configurations (all bead slices of the system) kept for training */
int md_gb300_ewald_model_create_x(md_gb300_ewald_model_t_x **model, md_pimd_t_x *pimd, int nsum_cheap,
                                  long capacity, unsigned seed);
void md_gb300_ewald_model_free_x(md_gb300_ewald_model_t_x *model);
/* add pimd's current configuration to the training set (descriptors and the
   FP64 converged-minus-truncated forces and per-particle energies); the first
   call also fixes the normalisation of inputs and outputs */
int md_gb300_ewald_model_collect_x(md_gb300_ewald_model_t_x *model, md_pimd_t_x *pimd);
/* steps Adam steps on random batches of batch_tiles x 128 rows; *loss: the
   last batch's loss (may be NULL) */
int md_gb300_ewald_model_train_x(md_gb300_ewald_model_t_x *model, int steps, int batch_tiles, double lr,
                                 double *loss);
/* From now on md_pimd_calc_pair_force_x / md_pimd_calc_pair_energy_x with
   md_coulomb_3d_ewald_* on pimd use the truncated sum plus the network.
   Every judge_every-th force call outside graph capture (0: never) computes
   the converged sum instead and judges the network on that configuration;
   when the force error (rms |dF| / rms |F_reciprocal|) is above force_tol or
   the energy error per particle above energy_tol, the network is dropped
   and later calls use the converged sum.  model NULL detaches. */
int md_gb300_ewald_model_attach_x(md_pimd_t_x *pimd, md_gb300_ewald_model_t_x *model, int judge_every,
                                  double force_tol, double energy_tol);
/* errors on pimd's current configuration: out[0] force error and out[1]
   energy error per particle (Ha) of truncated sum + network, out[2], out[3]
   the same for the truncated sum alone.  A judgement (this call, or the
   attached model's own cadence) evaluates eight consecutive bead slices
   (all of them when P <= 8), the next eight at the next judgement, so that
   every slice is judged in turn at an eighth of the cost of all 64. */
int md_gb300_ewald_model_judge_x(md_gb300_ewald_model_t_x *model, md_pimd_t_x *pimd, double out[4]);
int md_gb300_ewald_model_status_x(md_gb300_ewald_model_t_x *model, long *configurations, int *judged,
                                  int *reverted, double last[4]);
/* FP32 master parameters (md_gb300_ewald_model_nparam_x floats: W1[128][64],
   b1, W2[128][128], b2, W3[4][128], b3); set != 0 uploads */
int md_gb300_ewald_model_params_x(md_gb300_ewald_model_t_x *model, float *params, int set);
/* the tensor-core kernels on host data: outputs Y[rows][4] of inputs
   X[rows][64] (rounded to BF16); gradient of the training loss for rows
   with vector features and weight V[rows][12] and targets T[rows][4] */
int md_gb300_mlp_forward_x(md_gb300_ewald_model_t_x *model, const float *X, int rows, float *Y);
int md_gb300_mlp_grad_x(md_gb300_ewald_model_t_x *model, const float *X, const float *V, const float *T, int rows,
                        double we, double wf, float *grad, float *loss);
/* raw descriptors F[N*P][64] and vector features V[N*P][12] of pimd's
   current configuration (row j*N + l), and the descriptor definition: the
   cut-off rc, the radial basis basis[64][32] (the 32 Gaussians at the
   centres of 64 histogram bins on [0, rc)), and the centres and widths of
   the vector features' radial bumps */
int md_gb300_ewald_model_features_x(md_gb300_ewald_model_t_x *model, md_pimd_t_x *pimd, float *F, float *V);
int md_gb300_ewald_model_desc_info_x(md_gb300_ewald_model_t_x *model, double *rc, float *basis, double vmu[3],
                                     double vsig[3]);
/* tensor-core layout self-test: max errors of a 128 x 128 product for
   K-major operands and the two readings of MN-major descriptors */
int md_gb300_tc_selftest_x(double err[5]);
/* Bounded waits of the tensor-core kernels.  Every wait on an mbarrier
   phase (bulk copies, MMA completion) gives up after `cycles` SM clock
   cycles (default 2^32, about two seconds); the kernel then waits once more,
   bounded the same way, for its own copies in flight, frees its tensor
   memory, records an error status and returns, and the call that launched
   it reports MD_GB_ERR_CUDA.  The self-test arms a barrier for 16 bytes that
   nothing delivers (no copy is issued), waits with the limit `cycles` and
   returns the recorded status in *status (4: the wait ran out) and the
   cycles the wait took in *waited (may be NULL); the device stays usable. */
int md_gb300_set_wait_limit_x(long long cycles);
long long md_gb300_get_wait_limit_x(void);
int md_gb300_wait_selftest_x(long long cycles, int *status, long long *waited);

/* Text checkpoints (md_fprint_particle_pos_x / _vel_x / _force_x,
   md_fprint_nhcs_x, md_fprint_sim_box_x):
   on != 0 writes "%.17g" instead of the reference's lossy "%f", so that a
   resumed run continues bit for bit; the reference reads both. */
int md_gb300_set_text_exact_x(int on);

/* release the device copies (and, for *_free_*, the host structs) */
int md_gb300_release_simulation_x(md_simulation_t_x *sim);
void md_gb300_free_simulation_x(md_simulation_t_x *sim);
void md_gb300_free_pimd_x(md_pimd_t_x *pimd);
void md_gb300_free_stats_x(md_stats_t_x *stats);

#ifdef __cplusplus
}
#endif
#endif
