/*
 * md_pimd_x.h -- the path-integral (PIMD) step for fictitious identical
 * particles: exchange recursion, bead forces and estimators.  MD-Lab C ABI
 * as implemented by the GB300 library libxmd_x.
 *
 * Replaces MD-Lab md_pimd_x.h:1-233 for the force-and-integrate step.
 * Every compute entry point below is asynchronous on the library's CUDA
 * stream, exactly like the reference's OpenCL queue: results become visible
 * on the host through md_pimd_sync_host_x / md_simulation_sync_host_x /
 * md_stats_sync_host_x.  Functions return 0 on success and a negative
 * MD_GB_ERR_* code (md_gb300_x.h) on failure; nothing falls back to the CPU.
 */
#ifndef MD_PIMD_X_H
#define MD_PIMD_X_H

#include <stdio.h>

#include "md_particle_x.h"
#include "md_simulation_x.h"
#include "md_statistics_x.h"
#include "md_util_x.h"

#ifdef __cplusplus
extern "C" {
#endif

/* bead (l, j) of a ring polymer, both 1-based: md_pimd_x.h:10 */
#define MD_PIMD_INDEX_X(l, j, P) (((l)-1) * (P) + (j)-1)

/* md_pimd_x.h:12-106 without the OpenCL members */
typedef struct {
  md_simulation_t_x *sim;
  int N, P;
  int ENk_count;       /* N(N+1)/2 */
  md_num_t_x **ENk;    /* ENk[l-1][k-1]: spring energy of the cycle over l-k+1..l */
  md_num_t_x **ENk2;   /* virial cross terms, same shape */
  md_num_t_x **ENk3;
  md_num_t_x *VBN;     /* [N+1] exchange potentials V_B^(n) */
  md_num_t_x vi;       /* statistics parameter xi */
  md_num_t_x omegaP;   /* sqrt(P)/(beta hbar) */
  md_num_t_x beta;
  int pcount_in, pcount_ex;
  md_index_pair_t_x *pair_in;
  md_index_pair_t_x *pair_ex;
  int *Eindices;
  md_num_t_x *minE;
  int cut_Pj;
  md_num_t_x *Eint;
  md_num_t_x *Evir;
  int mc_par;
  int pbc;
  int *pbW;
  int worm_index;
  md_num_t_x worm_pos[MD_DIMENSION_X];
  int old_worm_index;
  md_num_t_x old_worm_pos[MD_DIMENSION_X];
} md_pimd_t_x;

/* md_pimd_x.h:114-120 */
md_pimd_t_x *md_pimd_sync_host_x(md_pimd_t_x *pimd, int read_only);
md_pimd_t_x *md_alloc_pimd_x(md_simulation_t_x *sim, int N, int P, md_num_t_x vi, md_num_t_x T);
void md_pimd_change_temperature_x(md_pimd_t_x *pimd, md_num_t_x T);
int md_pimd_next_index_x(int l, int j, int N2, int k, int P);
int md_pimd_prev_index_x(int l, int j, int N2, int k, int P);
int md_pimd_init_particle_uniform_pos_x(md_pimd_t_x *pimd, md_num_t_x *center, md_num_t_x *L, md_num_t_x fluc);

/* exchange: md_pimd_x.h:121-140.  The cubic-scaling entry points
   (md_pimd_fill_ENk_x, md_pimd_fill_force_VB_x) run the quadratic kernels,
   which compute the same quantities (they agree with the reference's cubic
   output to rounding). */
md_num_t_x md_pimd_ENk_x(md_pimd_t_x *pimd, int N2, int k, int image);
int md_pimd_fill_ENk_x(md_pimd_t_x *pimd, int image);
int md_pimd_fprint_ENk_x(FILE *out, md_pimd_t_x *pimd);
md_num_t_x md_pimd_xexp_x(md_num_t_x k, md_num_t_x E, md_num_t_x EE, md_num_t_x beta, md_num_t_x vi);
md_num_t_x md_pimd_xminE_x(md_pimd_t_x *pimd, int N2);
int md_pimd_fill_VB_x(md_pimd_t_x *pimd);
int md_pimd_fprint_VBN_x(FILE *out, md_pimd_t_x *pimd);
int md_pimd_fill_force_VB_x(md_pimd_t_x *pimd, int image);
int md_pimd_fast_fill_ENk_x(md_pimd_t_x *pimd, int image);
md_num_t_x md_pimd_fast_xminE_x(md_pimd_t_x *pimd, int u, md_num_t_x *V);
md_num_t_x md_pimd_fast_xexp_x(md_num_t_x l, md_num_t_x k, md_num_t_x E, md_num_t_x EE, md_num_t_x beta, md_num_t_x vi);
int md_pimd_fast_fill_force_VB_x(md_pimd_t_x *pimd, int image);

/* external bead forces and energies: md_pimd_x.h:130-134 */
int md_pimd_calc_VBN_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats);
int md_pimd_calc_trap_force_x(md_pimd_t_x *pimd, md_trap_force_t_x tf);
int md_pimd_calc_trap_energy_x(md_pimd_t_x *pimd, md_trap_energy_t_x te, md_stats_t_x *stats);
int md_pimd_calc_pair_force_x(md_pimd_t_x *pimd, md_pair_force_t_x pf);
int md_pimd_calc_pair_energy_x(md_pimd_t_x *pimd, md_pair_energy_t_x pe, md_stats_t_x *stats);

/* two species with the same P, e.g. the two spins of an unpolarised
   electron gas: md_pimd_x.h:146-147 (md_pimd_x.c:3282-3481, :3483-3632).
   Cross pairs only (each species' own pairs come from
   md_pimd_calc_pair_force_x), pimd's box; -1 when P differs, as in the
   reference.  The Ewald callback needs both species in one box and equal
   bead masses within each species.  FP64 in every precision mode. */
int md_pimd_calc_pair_force_2_x(md_pimd_t_x *pimd, md_pimd_t_x *pimd2, md_pair_force_t_x pf);
int md_pimd_calc_pair_energy_2_x(md_pimd_t_x *pimd, md_pimd_t_x *pimd2, md_pair_energy_t_x pe, md_stats_t_x *stats);

/* virial estimator: md_pimd_x.h:157-162 */
int md_pimd_fill_ENk2_x(md_pimd_t_x *pimd, int image);
int md_pimd_fprint_ENk2_x(FILE *out, md_pimd_t_x *pimd);
int md_pimd_calc_vi_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int image);
int md_pimd_fast_fill_ENk2_x(md_pimd_t_x *pimd, int image);

/* estimators and observables outside the step: md_pimd_x.h:143, :155-156,
   :160.  The virial about the box centre (md_pimd_x.c:3898) and the centroid
   virial (:3924) sum over beads on the GPU; md_pimd_polymer_periodic_
   boundary_x shifts whole ring polymers by their first bead's image count
   (:4350); md_pimd_calc_pair_correlation_x bins the distances from bead 1 to
   bead pi on the GPU (each in the reference's bin) and adds 1/norm per count
   to stats->fxs[stats->N - 1] on the host (:2974). */
int md_pimd_calc_pair_correlation_x(md_pimd_t_x *pimd, md_stats_t_x *stats, md_num_t_x rmax, md_num_t_x norm, int pi,
                                    int image);
int md_pimd_calc_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats);
int md_pimd_calc_centroid_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int fc);
int md_pimd_polymer_periodic_boundary_x(md_pimd_t_x *pimd);

/* accumulator arithmetic: md_pimd_x.h:163-170, scalar (es) and
   function-valued (fxs, the _f forms) */
int md_reset_stats_x(md_stats_t_x *stats, md_num_t_x e);
int md_reset_stats_f_x(md_stats_t_x *stats, md_num_t_x e);
int md_stats_add_to_x(md_stats_t_x *stats, md_stats_t_x *stats2);
int md_stats_add_to_f_x(md_stats_t_x *stats, md_stats_t_x *stats2);
int md_stats_copy_to_x(md_stats_t_x *stats, md_stats_t_x *stats2);
int md_stats_copy_to_f_x(md_stats_t_x *stats, md_stats_t_x *stats2);
int md_stats_mult_to_x(md_stats_t_x *stats, md_stats_t_x *stats2);
int md_stats_mult_to_f_x(md_stats_t_x *stats, md_stats_t_x *stats2);

/* xi -> xi' reweighting with sign, e.g. bosons to fermions:
   md_pimd_x.h:171-172 (md_pimd_calc_vi_sign_x: the signed recursion runs on
   the GPU, es[0] of both accumulators is scaled on the host as in the
   reference; md_pimd_xminE2_x on the synced host tables) */
md_num_t_x md_pimd_xminE2_x(md_pimd_t_x *pimd, int N2, md_num_t_x *VBN2, md_num_t_x vi2);
int md_pimd_calc_vi_sign_x(md_pimd_t_x *pimd, md_stats_t_x *e_s, md_stats_t_x *s_s, md_num_t_x vi2);
/* md_pimd_x.h:190 (md_pimd_x.c:5404-5448): static structure factor between
   bead 1 and bead pi for the first min(sk_sphere->N, stats->points) wave
   vectors, added to stats->fxs[stats->N - 1][j]; the sums run on the GPU */
int md_pimd_calc_sphere_Sk_structure_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int pi, md_sk_sphere_t_x *sk_sphere);

#ifdef __cplusplus
}
#endif
#endif
