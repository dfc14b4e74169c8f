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
   The first call on each device looks up the array's device address with
   that device current.  All calls share the array, so calls that overlap
   on the GPU (different streams, or several host threads) race; nothing in
   the array needs clearing between calls. */
int md_gb300_pair_force_noalloc_x(md_pair_force_t_x pf, const double *x, const double *m, double *f, int N, int P,
                                  int ld, const double *L, void *stream);

/* Arithmetic of the pair forces (md_pimd_calc_pair_force_x), including
   both Ewald parts.  MD_GB_PRECISION_FP64 (default) reproduces MD-Lab to
   1e-10.  MD_GB_PRECISION_MIXED evaluates pair and real-space Ewald forces in
   FP32 with compensated (Kahan) accumulation and the reciprocal sum with FP32
   phase products accumulated in double-float; positions, the exchange
   recursion, springs, the thermostat and every estimator stay FP64.  The
   force error against the FP64 form is about 1e-6 of the force scale. */
#define MD_GB_PRECISION_FP64 0
#define MD_GB_PRECISION_MIXED 1
int md_gb300_set_precision_x(int mode);
int md_gb300_get_precision_x(void);

/* release the device copies (and, for *_free_*, the host structs) */
int md_gb300_release_simulation_x(md_simulation_t_x *sim);
void md_gb300_free_simulation_x(md_simulation_t_x *sim);
void md_gb300_free_pimd_x(md_pimd_t_x *pimd);
void md_gb300_free_stats_x(md_stats_t_x *stats);

#ifdef __cplusplus
}
#endif
#endif
