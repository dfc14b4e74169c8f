/*
 * md_statistics_x.h -- block-averaging accumulator and pair/trap energies of
 * the MD-Lab C ABI, as implemented by libxmd_x (GB300).
 *
 * Replaces MD-Lab md_statistics_x.h:1-100 for the estimators of the
 * path-integral step.  Estimator calls accumulate into es[N-1] on the
 * device; md_stats_sync_host_x copies the running value back into
 * es[N-1] and drops the device copy (the reference's OpenCL semantics,
 * md_statistics_x.c:163-201).  Energy functions select device kernels by
 * pointer identity, like the force functions.
 */
#ifndef MD_STATISTICS_X_H
#define MD_STATISTICS_X_H

#include "md_particle_x.h"
#include "md_simulation_x.h"

#ifdef __cplusplus
extern "C" {
#endif

/* md_statistics_x.h:7 */
#define MD_MAX_STATS_COUNT 10000

/* md_statistics_x.h:9-25 without the OpenCL members */
typedef struct {
  int N;
  int count;
  md_num_t_x e;
  md_num_t_x *es;
  md_num_t_x T;
  md_num_t_x *Ts;
  int points;
  md_num_t_x *fx;
  md_num_t_x **fxs;
} md_stats_t_x;

/* md_statistics_x.h:28-34: one wave vector per distinct |q| of the cubic
   grid q0, q0 + qincre, ... <= qmax in each component, sorted by |q| */
typedef struct {
  int N;
  md_num_t_x *qs;
  md_num_t_x *qis;
} md_sk_sphere_t_x;

md_sk_sphere_t_x *md_alloc_sk_sphere_3d_x(md_num_t_x q0, md_num_t_x qincre, md_num_t_x qmax);

/* md_statistics_x.h:40 */
md_stats_t_x *md_stats_sync_host_x(md_stats_t_x *stats);

/* md_statistics_x.h:42-43 */
typedef md_num_t_x (*md_pair_energy_t_x)(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);
typedef md_num_t_x (*md_trap_energy_t_x)(md_num_t_x *p1, md_num_t_x *L, md_num_t_x m);

/* md_statistics_x.h:45-47 */
md_stats_t_x *md_alloc_stats_x(int points);
md_stats_t_x *md_update_stats_x(md_stats_t_x *stats);
md_stats_t_x *md_finalize_stats_x(md_stats_t_x *stats);

/* energies with device kernels: md_statistics_x.h:49-56 */
md_num_t_x md_harmonic_trap_energy_x(md_num_t_x *p1, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_neg_harmonic_trap_energy_x(md_num_t_x *p1, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_harmonic_trap_energy_2_x(md_num_t_x *p1, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_gaussian_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_periodic_gaussian_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_coulomb_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_coulomb_periodic_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);
md_num_t_x md_coulomb_3d_ewald_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L, md_num_t_x m);

#ifdef __cplusplus
}
#endif
#endif
