/*
 * md_particle_x.h -- value types of the MD-Lab C ABI (single-threaded
 * "_nocl" layout), as implemented by the GB300 library libxmd_x.
 *
 * Replaces MD-Lab md_particle_x.h:1-108.  The structs below must keep the
 * reference's field order and types byte for byte: drivers written against
 * the reference read and write them directly.  Differences:
 *   - MD_DIMENSION_X / MD_NHC_LENGTH_X are #ifndef-guarded, so a library
 *     variant is chosen with -D at build time (the reference hard-codes
 *     3 and 8 at md_particle_x.h:3-4);
 *   - there are no OpenCL members (the _nocl layout); device state lives in
 *     the library, keyed by the struct's address, and never in the struct.
 */
#ifndef MD_PARTICLE_X_H
#define MD_PARTICLE_X_H

#ifndef MD_DIMENSION_X
#define MD_DIMENSION_X 3
#endif
#ifndef MD_NHC_LENGTH_X
#define MD_NHC_LENGTH_X 8
#endif
#define MD_kB_X 1.0
#define MD_hBar_X 1.0

#include <math.h>

#ifndef M_PI
#define M_PI 3.141592653589793
#endif

#ifdef __GNUC__
#define MD_UNUSED_X(x) UNUSED_##x __attribute__((__unused__))
#else
#define MD_UNUSED_X(x) UNUSED_##x
#endif

/* md_particle_x.h:32-35: double precision on the host side */
typedef double md_num_t_x;

/* one bead: mass, position, velocity, force (stored as acceleration F/m);
   md_particle_x.h:37-42 */
typedef struct {
  md_num_t_x m;
  md_num_t_x x[MD_DIMENSION_X];
  md_num_t_x v[MD_DIMENSION_X];
  md_num_t_x f[MD_DIMENSION_X];
} md_particle_t_x;

/* one Nose-Hoover chain acting on f degrees of freedom; md_particle_x.h:44-49 */
typedef struct {
  int f;
  md_num_t_x theta[MD_NHC_LENGTH_X];
  md_num_t_x vtheta[MD_NHC_LENGTH_X];
  md_num_t_x Q[MD_NHC_LENGTH_X];
} md_nhc_t_x;

/* md_particle_x.h:51 */
enum { MD_ND_RECT_BOX_X };

/* md_particle_x.h:53-56 */
typedef struct {
  int type;
  void *box;
} simulation_box_t_x;

/* md_particle_x.h:58-60 */
typedef struct {
  md_num_t_x L[MD_DIMENSION_X];
} nd_rect_t_x;

/* md_particle_x.h:62-64 */
typedef struct {
  int i, j;
} md_index_pair_t_x;

/* md_particle_x.h:66-106 without the MD_USE_OPENCL_X members */
typedef struct {
  int N;                       /* beads (N*P for a path-integral run) */
  md_particle_t_x *particles;  /* [N], bead (l,j) at (l-1)*P + j-1 */
  int fc;                      /* thermostatted DOFs: D*N - constraints */
  int Nf;                      /* number of chains */
  int *fs;                     /* [Nf] DOFs per chain */
  int *f0s;                    /* [Nf] first DOF of each chain */
  md_nhc_t_x *nhcs;            /* [Nf] */
  simulation_box_t_x *box;
  md_num_t_x T;                /* thermostat temperature */
  int pcount_in, pcount_ex;
  md_index_pair_t_x *pair_in;  /* classical-MD pair lists (unused in PIMD mode) */
  md_index_pair_t_x *pair_ex;
} md_simulation_t_x;

#endif
