/*
 * md_util_x.h -- set-up, allocation, initial conditions, random numbers and
 * text checkpoints of the MD-Lab C ABI, as implemented by libxmd_x (GB300).
 *
 * Replaces MD-Lab md_util_x.h:1-150 for the path-integral step.  All of
 * these run on the host.  md_alloc_simulation_x allocates the particle and
 * chain arrays in page-locked memory when a GPU is present, so that the
 * host <-> device copies of md_simulation_sync_host_x run at full speed.
 * Random numbers reproduce the reference bit for bit (glibc rand() and the
 * same Box-Muller pairing, md_util_x.c:671-693).
 */
#ifndef MD_UTIL_X_H
#define MD_UTIL_X_H

#include <stdio.h>

#include "md_particle_x.h"

#ifdef __cplusplus
extern "C" {
#endif

/* md_util_x.h:7-8 */
extern int md_pimd_mode_x;
void md_set_pimd_mode_x(int pimd_mode);

/* md_util_x.h:10-26 */
#define MD_MAX_NAME_LENGTH_X 1024
typedef char md_name_t_x[MD_MAX_NAME_LENGTH_X + 1];
typedef struct {
  int N;
  md_name_t_x *names;
  md_num_t_x *values;
} md_attr_pair_t_x;
md_attr_pair_t_x *md_alloc_attr_pair_x(void);
md_attr_pair_t_x *md_read_attr_pair_x(FILE *in, md_attr_pair_t_x *attr);
md_num_t_x md_get_attr_value_x(md_attr_pair_t_x *attr, const char *name, int *found);

#define MD_MIN_X(a, b) (((a) < (b)) ? (a) : (b))

/* md_util_x.h:62-70.  gpu_count selects nothing: the library uses the
   current CUDA device.  cl_path is ignored (kernels are compiled ahead of
   time for sm_103a). */
typedef struct {
  int cpu_count;
  int gpu_count;
  int acc_count;
  unsigned int seed;
  const char *cl_path;
} md_init_config_x;
int md_init_setup_x(FILE *out, void *config);

/* md_util_x.h:78-98 */
md_simulation_t_x *md_simulation_sync_host_x(md_simulation_t_x *sim, int read_only);
md_simulation_t_x *md_alloc_simulation_x(int N, int f, int fc, int box_type);
simulation_box_t_x *md_alloc_box_x(int box_type);
int md_init_particle_face_center_3d_lattice_pos_x(md_simulation_t_x *sim, md_num_t_x *center, md_num_t_x *length, md_num_t_x fluc, md_num_t_x eps);
int md_init_maxwell_vel_x(md_simulation_t_x *sim, md_num_t_x T);
int md_init_particle_mass_x(md_simulation_t_x *sim, md_num_t_x m, int start, int end);
int md_init_nhc_x(md_simulation_t_x *sim, md_num_t_x Q, int start, int end, md_num_t_x fp);
int md_init_nd_rect_box_x(simulation_box_t_x *box, md_num_t_x *L);
int md_fprint_particle_pos_x(FILE *out, md_simulation_t_x *sim);
int md_fprint_particle_vel_x(FILE *out, md_simulation_t_x *sim);
int md_fprint_particle_force_x(FILE *out, md_simulation_t_x *sim);
int md_fprint_nhcs_x(FILE *out, md_simulation_t_x *sim);
int md_fprint_sim_box_x(FILE *out, simulation_box_t_x *box);
void md_set_seed_x(unsigned int seed);
md_num_t_x md_random_uniform_x(md_num_t_x a, md_num_t_x b);
md_num_t_x md_random_gaussian_x(void);
md_num_t_x md_get_quick_Q_x(md_num_t_x T, md_num_t_x omega);
int md_fread_particle_pos_x(FILE *in, md_simulation_t_x *sim);
int md_fread_particle_vel_x(FILE *in, md_simulation_t_x *sim);
int md_fread_nhcs_x(FILE *in, md_simulation_t_x *sim);

/* md_util_x.h:148 */
int md_simulation_copy_to_x(md_simulation_t_x *sim, md_simulation_t_x *sim2);

#ifdef __cplusplus
}
#endif
#endif
