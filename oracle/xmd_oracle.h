/*
 * xmd_oracle.h -- CPU restatement of MD-Lab's single-threaded (_nocl) PIMD
 * force-and-integrate step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the test-suite,
 * __graft_entry__.smoke() and the CPU-baseline leg of bench.py call it to
 * produce the values the CUDA library must reproduce.  The product library
 * (libxmd_x) never links or calls it.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's
 * own _nocl build (compiled from its sources by oracle/Makefile into
 * oracle/_ref/), and tests/test_oracle_golden.py checks every function here
 * against them.
 *
 * Unlike the reference, the dimension D and the chain length L are run-time
 * values, so one oracle build serves every library variant.  Arrays are
 * plain C arrays in the reference's own (bead-major) order:
 *   bead b = (l-1)*P + (j-1)  for particle l = 1..N, bead j = 1..P
 *   x[b*D + d], v[b*D + d], f[b*D + d], m[b]
 *   chain c: theta[c*L + i], vtheta[c*L + i], Q[c*L + i], cf[c] (its f)
 *   ENk triangle: ENk[l*(l-1)/2 + (k-1)] for l = 1..N, k = 1..l
 */
#ifndef XMD_ORACLE_H
#define XMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int D;           /* spatial dimension */
  int L;           /* Nose-Hoover chain length (even) */
  int nb;          /* number of beads (the reference's sim->N) */
  double *m;       /* [nb] */
  double *x;       /* [nb*D] */
  double *v;       /* [nb*D] */
  double *f;       /* [nb*D] forces stored as accelerations */
  int nf;          /* number of chains (sim->Nf) */
  int *cf;         /* [nf] DOFs per chain (nhcs[i].f) */
  double *theta;   /* [nf*L] */
  double *vtheta;  /* [nf*L] */
  double *Q;       /* [nf*L] */
  double T;        /* thermostat temperature (sim->T) */
  double box[3];   /* rectangular box lengths */
} orc_sim_t;

/* potentials, selected by kind (the reference selects by function pointer) */
enum {
  ORC_TRAP_HARMONIC = 1,      /* md_harmonic_trap_force_x:   -w^2 (x-c)      */
  ORC_TRAP_HARMONIC_2 = 2,    /* md_harmonic_trap_force_2_x: -w_d^2 (x_d-c_d)*/
  ORC_TRAP_NEG_HARMONIC = 3   /* md_neg_harmonic_trap_force_x: +w^2 (x-c)    */
};
enum {
  ORC_PAIR_GAUSSIAN = 1,          /* md_gaussian_force_x            */
  ORC_PAIR_PERIODIC_GAUSSIAN = 2, /* md_periodic_gaussian_force_x   */
  ORC_PAIR_COULOMB = 3,           /* md_coulomb_force_x             */
  ORC_PAIR_PERIODIC_COULOMB = 4,  /* md_coulomb_periodic_force_x    */
  ORC_PAIR_EWALD = 5              /* md_coulomb_3d_ewald_force_x    */
};

typedef struct {
  double trap_w;          /* md_trap_frequency_x */
  double trap_w2[3];      /* md_trap_frequency_2_x */
  double trap_c[3];       /* md_trap_center_x */
  double gauss_g;         /* md_gaussian_strength_x */
  double gauss_s;         /* md_gaussian_range_x */
  double coul_s;          /* md_coulomb_strength_x */
  double coul_alpha;      /* md_coulomb_truc_x */
  int coul_nsum;          /* md_coulomb_n_sum_x */
} orc_params_t;

/* ---- ring-polymer geometry ---- */
double orc_minimum_image(double a, double L);
int orc_periodic_image_count(double x, double L);

/* ---- integrator (md_simulation_x.c) ---- */
void orc_reset_force(orc_sim_t *s);
int orc_nhc_vv3_1(orc_sim_t *s, double h);
int orc_nhc_vv3_2(orc_sim_t *s, double h);
void orc_periodic_boundary(orc_sim_t *s);

/* ---- exchange (md_pimd_x.c) ---- */
int orc_fast_fill_ENk(const orc_sim_t *s, int N, int P, double omegaP, int image,
                      double *ENk, double *Eint);
int orc_fill_ENk_cubic(const orc_sim_t *s, int N, int P, double omegaP, int image,
                       double *ENk);
int orc_fill_VB(int N, double beta, double vi, const double *ENk, double *VBN);
int orc_fast_force_VB(orc_sim_t *s, int N, int P, double beta, double vi,
                      double omegaP, int image, const double *ENk,
                      const double *VBN, double *G_out, double *tmpV_out);
int orc_force_VB_cubic(orc_sim_t *s, int N, int P, double beta, double vi,
                       double omegaP, int image, const double *ENk,
                       const double *VBN);

/* ---- external forces ---- */
int orc_trap_force(orc_sim_t *s, int N, int P, int kind, const orc_params_t *p);
int orc_pair_force(orc_sim_t *s, int N, int P, int kind, const orc_params_t *p);
void orc_pair_force_one(int kind, const orc_params_t *p, int D, const double *p1,
                        const double *p2, double *f, const double *L, double m);
/* two species with the same P: cross pairs only (md_pimd_calc_pair_force_2_x) */
int orc_pair_force_2(orc_sim_t *a, int Na, orc_sim_t *b, int Nb, int P, int kind,
                     const orc_params_t *p);

/* ---- estimators ---- */
double orc_vbn_energy(int D, int N, int P, double beta, double vi,
                      const double *ENk, const double *VBN);
int orc_fast_fill_ENk2(const orc_sim_t *s, int N, int P, double omegaP,
                       int image, double *ENk2);
int orc_fill_ENk2_cubic(const orc_sim_t *s, int N, int P, double omegaP,
                        int image, double *ENk2);
double orc_vi_virial_energy(const orc_sim_t *s, int N, int P, double beta,
                            double vi, int image, const double *ENk,
                            const double *ENk2, const double *VBN);
double orc_trap_energy(const orc_sim_t *s, int N, int P, int kind,
                       const orc_params_t *p);
double orc_pair_energy(const orc_sim_t *s, int N, int P, int kind,
                       const orc_params_t *p);
double orc_pair_energy_one(int kind, const orc_params_t *p, int D,
                           const double *p1, const double *p2, const double *L);
double orc_pair_energy_2(const orc_sim_t *a, int Na, const orc_sim_t *b, int Nb,
                         int P, int kind, const orc_params_t *p);
double orc_madelung(const double *L, const orc_params_t *p);
double orc_virial_energy(const orc_sim_t *s, int N, int P);
double orc_centroid_virial_energy(const orc_sim_t *s, int N, int P, double beta, int fc);
void orc_polymer_periodic_boundary(orc_sim_t *s, int N, int P);
void orc_pair_correlation(const orc_sim_t *s, int N, int P, int points, double rmax, double norm, int pi,
                          int image, double *out);
double orc_vi_sign(int N, double beta, double vi, double vi2, const double *ENk,
                   const double *VBN);

/* ---- one MD step in the order a driver calls the reference ---- */
typedef struct {
  int N, P;
  double beta, vi, omegaP;
  int image;          /* minimum image in the spring terms */
  int trap_kind;      /* 0 = none */
  int pair_kind;      /* 0 = none */
  int pbc;            /* wrap positions into the box after the step */
  orc_params_t prm;
} orc_step_cfg_t;

/* ENk [N(N+1)/2], Eint [N], VBN [N+1] are caller-provided work arrays */
int orc_step(orc_sim_t *s, const orc_step_cfg_t *c, double h, double *ENk,
             double *Eint, double *VBN);

/* ---- initial conditions from glibc rand(), as md_util_x.c:671-836 ---- */
void orc_set_seed(unsigned int seed);
double orc_random_uniform(double a, double b);
double orc_random_gaussian(void);

#ifdef __cplusplus
}
#endif
#endif
