/*
 * md_simulation_x.h -- potentials, parameters and the Nose-Hoover-chain
 * integrator of the MD-Lab C ABI, as implemented by libxmd_x (GB300).
 *
 * Replaces MD-Lab md_simulation_x.h:1-89 for the path-integral step.
 * Potentials are chosen by function-pointer identity, as in the reference's
 * OpenCL build (md_simulation_x.c:8-67): passing one of the functions below
 * to md_pimd_calc_pair_force_x / md_pimd_calc_trap_force_x selects the
 * matching CUDA kernel; any other pointer is rejected with
 * MD_GB_ERR_UNSUPPORTED (there is no CPU fallback).  The functions keep
 * their CPU bodies, so a driver may still call them on host data.
 * Parameters are the reference's globals, read at each device call.
 */
#ifndef MD_SIMULATION_X_H
#define MD_SIMULATION_X_H

#include "md_particle_x.h"

#ifdef __cplusplus
extern "C" {
#endif

/* parameter globals: md_simulation_x.h:16-24 */
extern md_num_t_x md_trap_frequency_x;
extern md_num_t_x md_trap_center_x[MD_DIMENSION_X];
extern md_num_t_x md_trap_frequency_2_x[MD_DIMENSION_X];
extern md_num_t_x md_gaussian_strength_x;
extern md_num_t_x md_gaussian_range_x;
extern md_num_t_x md_coulomb_strength_x;
extern md_num_t_x md_coulomb_truc_x;   /* Ewald splitting parameter alpha */
extern int md_coulomb_n_sum_x;         /* Ewald image / reciprocal cube |n_i| <= n */

/* md_simulation_x.h:38-39 */
typedef void (*md_pair_force_t_x)(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
typedef void (*md_trap_force_t_x)(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);

/* geometry: md_simulation_x.h:41-44 */
md_num_t_x md_minimum_image_x(md_num_t_x a, md_num_t_x L);
md_num_t_x md_minimum_image_distance_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L);
md_num_t_x md_distance_x(md_num_t_x *p1, md_num_t_x *p2);

/* traps and pair potentials with device kernels: md_simulation_x.h:46-64 */
void md_harmonic_trap_force_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_neg_harmonic_trap_force_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_set_harmonic_trap_frequency_x(md_num_t_x f);
void md_set_harmonic_trap_center_x(md_num_t_x *center);
void md_set_harmonic_trap_frequency_2_x(md_num_t_x *f);
void md_harmonic_trap_force_2_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_gaussian_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_periodic_gaussian_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_set_gaussian_force_strength_x(md_num_t_x g);
void md_set_guassian_force_range_x(md_num_t_x s); /* sic: the reference's name */
void md_coulomb_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_coulomb_periodic_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);
void md_set_coulomb_force_strength_x(md_num_t_x g);
void md_set_coulomb_truc_x(md_num_t_x k);
void md_set_coulomb_n_sum_x(int n);
md_num_t_x md_calc_3d_ueg_madelung_x(md_num_t_x *L);
void md_coulomb_3d_ewald_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L, md_num_t_x m);

/* integrator: md_simulation_x.h:76-86 */
int md_reset_force_x(md_simulation_t_x *sim);
void md_calc_nhc_force_x(md_simulation_t_x *sim, int f0, int f2, int i, md_num_t_x *res);
int md_update_nhc_VV3_1_x(md_simulation_t_x *sim, md_num_t_x h);
int md_update_nhc_VV3_2_x(md_simulation_t_x *sim, md_num_t_x h);
int md_periodic_boundary_x(md_simulation_t_x *sim);
int md_periodic_image_count_x(md_num_t_x x, md_num_t_x L);
int md_simulation_rescale_velocity_x(md_simulation_t_x *sim, md_num_t_x T);

#ifdef __cplusplus
}
#endif
#endif
