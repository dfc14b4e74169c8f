/*
 * make_golden.c -- writes golden vectors by running MD-Lab's own _nocl build
 * through its public API (md_pimd_x.h / md_simulation_x.h).
 *
 * Compiled by tests/golden/make_golden.sh once per (dimension, chain length)
 * variant against oracle/_ref/src_d<D>l<L>/ (the reference headers) and
 * linked with oracle/_ref/libxmd_x_d<D>l<L>.so.  Output: one binary fixture
 * per scenario, a sequence of records
 *     char name[32]; int64 count; double data[count];
 * read by tests/golden/fixtures.py.
 *
 * The driver follows the per-step call order of the reference's PIMD
 * application (md_update_nhc_VV3_1_x ... md_update_nhc_VV3_2_x,
 * md_periodic_boundary_x) and records the state after each stage.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "md_pimd_x.h"
#include "md_simulation_x.h"
#include "md_statistics_x.h"
#include "md_util_x.h"

#define D MD_DIMENSION_X
#define LC MD_NHC_LENGTH_X

static FILE *g_out;

static void rec(const char *name, const double *a, long n) {
  char nm[32];
  memset(nm, 0, sizeof nm);
  strncpy(nm, name, 31);
  long long c = n;
  fwrite(nm, 1, 32, g_out);
  fwrite(&c, sizeof c, 1, g_out);
  fwrite(a, sizeof(double), (size_t)n, g_out);
}

static void rec1(const char *name, double v) { rec(name, &v, 1); }

static void rec_field(const char *prefix, md_simulation_t_x *sim, char which) {
  long n = (long)sim->N * D;
  double *buf = malloc(sizeof(double) * n);
  for (int b = 0; b < sim->N; ++b)
    for (int d = 0; d < D; ++d) {
      md_particle_t_x *p = &sim->particles[b];
      buf[b * D + d] = which == 'x' ? p->x[d] : which == 'v' ? p->v[d] : p->f[d];
    }
  char nm[64];
  snprintf(nm, sizeof nm, "%s%c", prefix, which);
  rec(nm, buf, n);
  free(buf);
}

static void rec_chains(const char *prefix, md_simulation_t_x *sim) {
  long n = (long)sim->Nf * LC;
  double *th = malloc(sizeof(double) * n), *vt = malloc(sizeof(double) * n), *q = malloc(sizeof(double) * n);
  double *cf = malloc(sizeof(double) * sim->Nf);
  for (int i = 0; i < sim->Nf; ++i) {
    cf[i] = sim->nhcs[i].f;
    for (int j = 0; j < LC; ++j) {
      th[i * LC + j] = sim->nhcs[i].theta[j];
      vt[i * LC + j] = sim->nhcs[i].vtheta[j];
      q[i * LC + j] = sim->nhcs[i].Q[j];
    }
  }
  char nm[64];
  snprintf(nm, sizeof nm, "%stheta", prefix);
  rec(nm, th, n);
  snprintf(nm, sizeof nm, "%svtheta", prefix);
  rec(nm, vt, n);
  snprintf(nm, sizeof nm, "%sQ", prefix);
  rec(nm, q, n);
  snprintf(nm, sizeof nm, "%scf", prefix);
  rec(nm, cf, sim->Nf);
  free(th);
  free(vt);
  free(q);
  free(cf);
}

static void rec_state(const char *prefix, md_simulation_t_x *sim) {
  rec_field(prefix, sim, 'x');
  rec_field(prefix, sim, 'v');
  rec_field(prefix, sim, 'f');
  rec_chains(prefix, sim);
}

typedef struct {
  int N, P, f, fc, steps, nsum, ueg, image, pbc, seed, every;
  double vi, beta, g, s, dt, rs, theta, alpha_L, box;
} scen_t;

static md_stats_t_x *g_st;

static double take(void) {
  double e = g_st->es[g_st->N - 1];
  g_st->es[g_st->N - 1] = 0;
  return e;
}

static void estimators(const char *prefix, md_pimd_t_x *pimd, const scen_t *c) {
  char nm[64];
  md_pimd_calc_VBN_energy_x(pimd, g_st);
  snprintf(nm, sizeof nm, "%se_prim_exch", prefix);
  rec1(nm, take());
  md_pimd_fast_fill_ENk2_x(pimd, c->image);
  snprintf(nm, sizeof nm, "%sENk2", prefix);
  rec(nm, pimd->ENk2[0], pimd->ENk_count);
  md_pimd_calc_vi_virial_energy_x(pimd, g_st, c->image);
  snprintf(nm, sizeof nm, "%se_vir_exch", prefix);
  rec1(nm, take());
  if (!c->ueg) {
    md_pimd_calc_trap_energy_x(pimd, md_harmonic_trap_energy_x, g_st);
    snprintf(nm, sizeof nm, "%se_trap", prefix);
    rec1(nm, take());
    md_pimd_calc_pair_energy_x(pimd, md_gaussian_energy_x, g_st);
  } else {
    md_pimd_calc_pair_energy_x(pimd, md_coulomb_3d_ewald_energy_x, g_st);
  }
  snprintf(nm, sizeof nm, "%se_pair", prefix);
  rec1(nm, take());
}

static void forces(md_pimd_t_x *pimd, const scen_t *c, int record) {
  md_simulation_t_x *sim = pimd->sim;
  md_reset_force_x(sim);
  md_pimd_fast_fill_ENk_x(pimd, c->image);
  if (record) {
    rec("ENk", pimd->ENk[0], pimd->ENk_count);
    rec("Eint", pimd->Eint, pimd->N);
  }
  md_pimd_fill_VB_x(pimd);
  if (record) rec("VBN", pimd->VBN, pimd->N + 1);
  md_pimd_fast_fill_force_VB_x(pimd, c->image);
  if (record) rec_field("f_exch/", sim, 'f');
  if (!c->ueg) {
    md_pimd_calc_trap_force_x(pimd, md_harmonic_trap_force_x);
    if (record) rec_field("f_trap/", sim, 'f');
    md_pimd_calc_pair_force_x(pimd, md_gaussian_force_x);
  } else {
    md_pimd_calc_pair_force_x(pimd, md_coulomb_3d_ewald_force_x);
  }
  if (record) rec_field("f_pair/", sim, 'f');
}

static void run(const scen_t *c) {
  md_set_pimd_mode_x(1);
  md_set_seed_x((unsigned)c->seed);
  int nb = c->N * c->P;
  md_simulation_t_x *sim = md_alloc_simulation_x(nb, c->f, c->fc, MD_ND_RECT_BOX_X);
  double T, Lb;
  if (c->ueg) {
    /* spin-polarised electron gas: n = 3/(4 pi rs^3), T_F = (6 pi^2 n)^(2/3)/2 */
    Lb = cbrt(4.0 * M_PI * c->N / 3.0) * c->rs;
    double n = c->N / (Lb * Lb * Lb);
    double TF = 0.5 * pow(6.0 * M_PI * M_PI * n, 2.0 / 3.0);
    T = c->theta * TF;
  } else {
    Lb = c->box;
    T = 1.0 / c->beta;
  }
  double Lv[D];
  for (int d = 0; d < D; ++d) Lv[d] = Lb;
  md_init_nd_rect_box_x(sim->box, Lv);
  md_pimd_t_x *pimd = md_alloc_pimd_x(sim, c->N, c->P, c->vi, T);
  md_init_particle_mass_x(sim, 1.0, 0, nb);
  if (c->ueg) {
    double center[D];
    for (int d = 0; d < D; ++d) center[d] = Lb / 2;
    md_pimd_init_particle_uniform_pos_x(pimd, center, Lv, 0.05 * c->rs);
  } else {
    for (int b = 0; b < nb; ++b)
      for (int d = 0; d < D; ++d) sim->particles[b].x[d] = md_random_gaussian_x();
  }
  md_init_maxwell_vel_x(sim, T);
  double Q = md_get_quick_Q_x(T, pimd->omegaP);
  md_init_nhc_x(sim, Q, 0, sim->Nf, 0);
  for (int b = 0; b < nb; ++b)
    for (int d = 0; d < D; ++d) sim->particles[b].f[d] = 0;
  double zero[D];
  for (int d = 0; d < D; ++d) zero[d] = 0;
  md_set_harmonic_trap_frequency_x(1.0);
  md_set_harmonic_trap_center_x(zero);
  md_set_gaussian_force_strength_x(c->g);
  md_set_guassian_force_range_x(c->s);
  md_set_coulomb_force_strength_x(1.0);
  md_set_coulomb_truc_x(c->alpha_L / Lb);
  md_set_coulomb_n_sum_x(c->nsum);

  double hdr[] = {D, LC, c->N, c->P, c->f, c->fc, c->vi, pimd->beta, pimd->omegaP, T, Lb, c->dt,
                  c->image, c->pbc, c->ueg, c->g, c->s, c->alpha_L / Lb, c->nsum, c->steps, c->every};
  rec("hdr", hdr, sizeof hdr / sizeof hdr[0]);
  {
    double *m = malloc(sizeof(double) * nb);
    for (int b = 0; b < nb; ++b) m[b] = sim->particles[b].m;
    rec("m", m, nb);
    free(m);
  }
  rec_state("init/", sim);
  if (c->ueg) rec1("madelung", md_calc_3d_ueg_madelung_x(Lv));

  /* step 1, every stage recorded */
  md_update_nhc_VV3_1_x(sim, c->dt);
  rec_state("s1/", sim);
  forces(pimd, c, 1);
  /* estimators at the positions the forces were computed for */
  estimators("s1/", pimd, c);
  {
    md_stats_t_x *es = md_alloc_stats_x(1), *ss = md_alloc_stats_x(1);
    es->es[0] = 1;
    ss->es[0] = 1;
    md_pimd_calc_vi_sign_x(pimd, es, ss, -1.0);
    rec1("s1/sign_m1", es->es[0]);
  }
#if MD_DIMENSION_X == 3
  {
    /* spherical S(k) between bead 1 and bead P/2+1 at these positions */
    md_sk_sphere_t_x *sk = md_alloc_sk_sphere_3d_x(0.0, 0.5, 2.0);
    md_stats_t_x *st = md_alloc_stats_x(sk->N);
    md_pimd_calc_sphere_Sk_structure_x(pimd, st, c->P / 2 + 1, sk);
    rec("sk/qs", sk->qs, sk->N);
    rec("sk/qis", sk->qis, 3L * sk->N);
    rec("sk/res", st->fxs[st->N - 1], sk->N);
  }
#endif
  md_update_nhc_VV3_2_x(sim, c->dt);
  rec_state("s2/", sim);
  if (c->pbc) {
    md_periodic_boundary_x(sim);
    rec_field("s3/", sim, 'x');
  }

  /* trajectory */
  int every = c->every > 0 ? c->every : 100;
  for (int st = 2; st <= c->steps; ++st) {
    md_update_nhc_VV3_1_x(sim, c->dt);
    forces(pimd, c, 0);
    if (st % every == 0) {
      char nm[32];
      snprintf(nm, sizeof nm, "t%d/", st);
      estimators(nm, pimd, c);
    }
    md_update_nhc_VV3_2_x(sim, c->dt);
    if (c->pbc) md_periodic_boundary_x(sim);
  }
  if (c->steps >= 2) rec_state("final/", sim);
}

/* positions-only check of the cubic paths (md_pimd_fill_ENk_x,
   md_pimd_fill_force_VB_x, md_pimd_fill_ENk2_x) on the init state */
static void run_cubic(const scen_t *c) {
  md_set_pimd_mode_x(1);
  md_set_seed_x((unsigned)c->seed);
  int nb = c->N * c->P;
  md_simulation_t_x *sim = md_alloc_simulation_x(nb, c->f, c->fc, MD_ND_RECT_BOX_X);
  double Lv[D];
  for (int d = 0; d < D; ++d) Lv[d] = c->box;
  md_init_nd_rect_box_x(sim->box, Lv);
  md_pimd_t_x *pimd = md_alloc_pimd_x(sim, c->N, c->P, c->vi, 1.0 / c->beta);
  md_init_particle_mass_x(sim, 1.0, 0, nb);
  for (int b = 0; b < nb; ++b)
    for (int d = 0; d < D; ++d) {
      sim->particles[b].x[d] = md_random_gaussian_x();
      sim->particles[b].f[d] = 0;
    }
  double hdr[] = {D, LC, c->N, c->P, c->vi, pimd->beta, pimd->omegaP, c->image, c->box};
  rec("hdr", hdr, sizeof hdr / sizeof hdr[0]);
  rec_field("init/", sim, 'x');
  md_pimd_fill_ENk_x(pimd, c->image);
  rec("ENk_cubic", pimd->ENk[0], pimd->ENk_count);
  md_pimd_fill_VB_x(pimd);
  rec("VBN_cubic", pimd->VBN, pimd->N + 1);
  md_pimd_fill_force_VB_x(pimd, c->image);
  rec_field("f_cubic/", sim, 'f');
  md_reset_force_x(sim);
  md_pimd_fast_fill_ENk_x(pimd, c->image);
  rec("ENk_fast", pimd->ENk[0], pimd->ENk_count);
  md_pimd_fill_VB_x(pimd);
  md_pimd_fast_fill_force_VB_x(pimd, c->image);
  rec_field("f_fast/", sim, 'f');
  md_pimd_fill_ENk2_x(pimd, c->image);
  rec("ENk2_cubic", pimd->ENk2[0], pimd->ENk_count);
}

static void run_rng(void) {
  double u[32], g[32];
  md_set_seed_x(1234);
  for (int i = 0; i < 32; ++i) u[i] = md_random_uniform_x(-1.0, 2.0);
  for (int i = 0; i < 32; ++i) g[i] = md_random_gaussian_x();
  rec("uniform", u, 32);
  rec("gaussian", g, 32);
  md_set_seed_x(7);
  for (int i = 0; i < 31; ++i) g[i] = md_random_gaussian_x();
  rec("gaussian_seed7_odd", g, 31);
}

/* isolated pair callbacks at random separations (D=3 only for Ewald) */
static void run_pairs(void) {
  md_set_seed_x(99);
  const int npair = 24;
  double L[D];
  for (int d = 0; d < D; ++d) L[d] = 3.3 + 0.2 * d;
  rec("L", L, D);
  double *p = malloc(sizeof(double) * npair * 2 * D);
  for (int i = 0; i < npair * 2 * D; ++i) p[i] = md_random_uniform_x(-0.2, L[i % D] + 0.2);
  rec("pos", p, npair * 2 * D);
  double ff[64 * D], ee[64];
  md_set_gaussian_force_strength_x(0.75 * M_PI);
  md_set_guassian_force_range_x(0.5);
  md_set_coulomb_force_strength_x(1.3);
  struct {
    const char *nm;
    md_pair_force_t_x pf;
    md_pair_energy_t_x pe;
  } kinds[] = {{"gauss", md_gaussian_force_x, md_gaussian_energy_x},
               {"pgauss", md_periodic_gaussian_force_x, md_periodic_gaussian_energy_x},
               {"coul", md_coulomb_force_x, md_coulomb_energy_x},
               {"pcoul", md_coulomb_periodic_force_x, md_coulomb_periodic_energy_x}};
  for (int k = 0; k < 4; ++k) {
    for (int i = 0; i < npair; ++i) {
      double f[D];
      for (int d = 0; d < D; ++d) f[d] = 0;
      kinds[k].pf(&p[2 * i * D], &p[(2 * i + 1) * D], f, L, 1.7);
      for (int d = 0; d < D; ++d) ff[i * D + d] = f[d];
      ee[i] = kinds[k].pe(&p[2 * i * D], &p[(2 * i + 1) * D], L, 1.7);
    }
    char nm[32];
    snprintf(nm, sizeof nm, "%s/f", kinds[k].nm);
    rec(nm, ff, npair * D);
    snprintf(nm, sizeof nm, "%s/e", kinds[k].nm);
    rec(nm, ee, npair);
  }
#if MD_DIMENSION_X == 3
  int nsums[] = {1, 2, 3};
  double als[] = {5.6, 3.0};
  for (int a = 0; a < 2; ++a)
    for (int n = 0; n < 3; ++n) {
      md_set_coulomb_truc_x(als[a] / L[0]);
      md_set_coulomb_n_sum_x(nsums[n]);
      for (int i = 0; i < npair; ++i) {
        double f[D] = {0, 0, 0};
        md_coulomb_3d_ewald_force_x(&p[2 * i * D], &p[(2 * i + 1) * D], f, L, 1.7);
        for (int d = 0; d < D; ++d) ff[i * D + d] = f[d];
        ee[i] = md_coulomb_3d_ewald_energy_x(&p[2 * i * D], &p[(2 * i + 1) * D], L, 1.7);
      }
      char nm[32];
      snprintf(nm, sizeof nm, "ewald_a%d_n%d/f", a, nsums[n]);
      rec(nm, ff, npair * D);
      snprintf(nm, sizeof nm, "ewald_a%d_n%d/e", a, nsums[n]);
      rec(nm, ee, npair);
      snprintf(nm, sizeof nm, "ewald_a%d_n%d/mad", a, nsums[n]);
      rec1(nm, md_calc_3d_ueg_madelung_x(L));
    }
#endif
  free(p);
}

/* two species with the same P (md_pimd_calc_pair_force_2_x,
   md_pimd_calc_pair_energy_2_x): a spin-unpolarised electron gas, N up and
   Nb down electrons in one box with Ewald everywhere (ueg=1), or two trapped
   species with Gaussian interactions (ueg=0).  Species b has mass mb.
   Records both initial states, the cross forces and cross energy alone, the
   forces of a full two-species force call, and a short trajectory in which
   each species has its own exchange and pair forces plus the cross term. */
static md_pair_force_t_x g_pf2;
static md_pair_energy_t_x g_pe2;

static void forces2(md_pimd_t_x *pa, md_pimd_t_x *pb, const scen_t *c) {
  md_pimd_t_x *ps[2] = {pa, pb};
  for (int s = 0; s < 2; ++s) {
    md_reset_force_x(ps[s]->sim);
    md_pimd_fast_fill_ENk_x(ps[s], c->image);
    md_pimd_fill_VB_x(ps[s]);
    md_pimd_fast_fill_force_VB_x(ps[s], c->image);
    if (!c->ueg) md_pimd_calc_trap_force_x(ps[s], md_harmonic_trap_force_x);
    md_pimd_calc_pair_force_x(ps[s], g_pf2);
  }
  md_pimd_calc_pair_force_2_x(pa, pb, g_pf2);
}

static void run_two(const scen_t *c, int Nb, double mb) {
  md_set_pimd_mode_x(1);
  md_set_seed_x((unsigned)c->seed);
  const int Na = c->N, P = c->P;
  md_simulation_t_x *sa = md_alloc_simulation_x(Na * P, c->f, c->fc, MD_ND_RECT_BOX_X);
  md_simulation_t_x *sb = md_alloc_simulation_x(Nb * P, c->f, c->fc, MD_ND_RECT_BOX_X);
  double T, Lb;
  if (c->ueg) {
    /* unpolarised gas: n = (Na + Nb)/L^3 = 3/(4 pi rs^3), T_F = (3 pi^2 n)^(2/3)/2 */
    Lb = cbrt(4.0 * M_PI * (Na + Nb) / 3.0) * c->rs;
    double n = (Na + Nb) / (Lb * Lb * Lb);
    T = c->theta * 0.5 * pow(3.0 * M_PI * M_PI * n, 2.0 / 3.0);
    g_pf2 = md_coulomb_3d_ewald_force_x;
    g_pe2 = md_coulomb_3d_ewald_energy_x;
  } else {
    Lb = c->box;
    T = 1.0 / c->beta;
    g_pf2 = md_gaussian_force_x;
    g_pe2 = md_gaussian_energy_x;
  }
  double Lv[D], center[D], zero[D];
  for (int d = 0; d < D; ++d) {
    Lv[d] = Lb;
    center[d] = Lb / 2;
    zero[d] = 0;
  }
  md_init_nd_rect_box_x(sa->box, Lv);
  md_init_nd_rect_box_x(sb->box, Lv);
  md_pimd_t_x *pa = md_alloc_pimd_x(sa, Na, P, c->vi, T);
  md_pimd_t_x *pb = md_alloc_pimd_x(sb, Nb, P, c->vi, T);
  md_init_particle_mass_x(sa, 1.0, 0, Na * P);
  md_init_particle_mass_x(sb, mb, 0, Nb * P);
  md_simulation_t_x *ss[2] = {sa, sb};
  md_pimd_t_x *ps[2] = {pa, pb};
  for (int s = 0; s < 2; ++s) {
    if (c->ueg)
      md_pimd_init_particle_uniform_pos_x(ps[s], center, Lv, 0.05 * c->rs);
    else
      for (int b = 0; b < ss[s]->N; ++b)
        for (int d = 0; d < D; ++d) ss[s]->particles[b].x[d] = md_random_gaussian_x();
    md_init_maxwell_vel_x(ss[s], T);
    md_init_nhc_x(ss[s], md_get_quick_Q_x(T, ps[s]->omegaP), 0, ss[s]->Nf, 0);
    for (int b = 0; b < ss[s]->N; ++b)
      for (int d = 0; d < D; ++d) ss[s]->particles[b].f[d] = 0;
  }
  md_set_harmonic_trap_frequency_x(1.0);
  md_set_harmonic_trap_center_x(zero);
  md_set_gaussian_force_strength_x(c->g);
  md_set_guassian_force_range_x(c->s);
  md_set_coulomb_force_strength_x(1.0);
  md_set_coulomb_truc_x(c->alpha_L / Lb);
  md_set_coulomb_n_sum_x(c->nsum);
  double hdr[] = {D, LC, Na, Nb, P, c->vi, pa->beta, pa->omegaP, T, Lb, c->dt, c->image, c->pbc, c->ueg,
                  c->g, c->s, c->alpha_L / Lb, c->nsum, c->steps, mb};
  rec("hdr", hdr, sizeof hdr / sizeof hdr[0]);
  rec_state("a/init/", sa);
  rec_state("b/init/", sb);
  /* the cross term alone */
  md_reset_force_x(sa);
  md_reset_force_x(sb);
  md_pimd_calc_pair_force_2_x(pa, pb, g_pf2);
  rec_field("a/cross/", sa, 'f');
  rec_field("b/cross/", sb, 'f');
  md_pimd_calc_pair_energy_2_x(pa, pb, g_pe2, g_st);
  rec1("cross/e", take());
  /* a full force call, then a trajectory starting from those forces */
  forces2(pa, pb, c);
  rec_field("a/all/", sa, 'f');
  rec_field("b/all/", sb, 'f');
  for (int st = 1; st <= c->steps; ++st) {
    md_update_nhc_VV3_1_x(sa, c->dt);
    md_update_nhc_VV3_1_x(sb, c->dt);
    forces2(pa, pb, c);
    md_update_nhc_VV3_2_x(sa, c->dt);
    md_update_nhc_VV3_2_x(sb, c->dt);
    if (c->pbc) {
      md_periodic_boundary_x(sa);
      md_periodic_boundary_x(sb);
    }
  }
  rec_state("a/final/", sa);
  rec_state("b/final/", sb);
  md_pimd_calc_pair_energy_2_x(pa, pb, g_pe2, g_st);
  rec1("final/cross_e", take());
}

/* observables and accumulator helpers outside the step: the plain and
   centroid virial estimators (md_pimd_x.c:3898, :3924), g(r) between bead 1
   and bead P/2+1 (md_pimd_x.c:2974) with and without the minimum image, the
   whole-polymer periodic wrap (md_pimd_x.c:4350) and the function-valued
   accumulator arithmetic (md_pimd_x.c:4566-4650).  The trajectory before
   them runs without the per-step wrap, so beads leave the box. */
static void rec_stats_f(const char *name, md_stats_t_x *st) { rec(name, st->fxs[st->N - 1], st->points); }

static void run_obs(const scen_t *c) {
  scen_t c2 = *c;
  c2.pbc = 0;
  md_set_pimd_mode_x(1);
  md_set_seed_x((unsigned)c->seed);
  int nb = c->N * c->P;
  md_simulation_t_x *sim = md_alloc_simulation_x(nb, c->f, c->fc, MD_ND_RECT_BOX_X);
  double T, Lb;
  if (c->ueg) {
    Lb = cbrt(4.0 * M_PI * c->N / 3.0) * c->rs;
    double n = c->N / (Lb * Lb * Lb);
    T = c->theta * 0.5 * pow(6.0 * M_PI * M_PI * n, 2.0 / 3.0);
  } else {
    Lb = c->box;
    T = 1.0 / c->beta;
  }
  double Lv[D], center[D], zero[D];
  for (int d = 0; d < D; ++d) {
    Lv[d] = Lb;
    center[d] = Lb / 2;
    zero[d] = 0;
  }
  md_init_nd_rect_box_x(sim->box, Lv);
  md_pimd_t_x *pimd = md_alloc_pimd_x(sim, c->N, c->P, c->vi, T);
  md_init_particle_mass_x(sim, 1.0, 0, nb);
  if (c->ueg)
    md_pimd_init_particle_uniform_pos_x(pimd, center, Lv, 0.05 * c->rs);
  else
    for (int b = 0; b < nb; ++b)
      for (int d = 0; d < D; ++d) sim->particles[b].x[d] = md_random_gaussian_x();
  md_init_maxwell_vel_x(sim, T);
  md_init_nhc_x(sim, md_get_quick_Q_x(T, pimd->omegaP), 0, sim->Nf, 0);
  for (int b = 0; b < nb; ++b)
    for (int d = 0; d < D; ++d) sim->particles[b].f[d] = 0;
  md_set_harmonic_trap_frequency_x(1.0);
  md_set_harmonic_trap_center_x(zero);
  md_set_gaussian_force_strength_x(c->g);
  md_set_guassian_force_range_x(c->s);
  md_set_coulomb_force_strength_x(1.0);
  md_set_coulomb_truc_x(c->alpha_L / Lb);
  md_set_coulomb_n_sum_x(c->nsum);
  double hdr[] = {D, LC, c->N, c->P, c->f, c->fc, c->vi, pimd->beta, pimd->omegaP, T, Lb, c->dt,
                  c->image, 0, c->ueg, c->g, c->s, c->alpha_L / Lb, c->nsum, c->steps, c->every};
  rec("hdr", hdr, sizeof hdr / sizeof hdr[0]);
  {
    double *m = malloc(sizeof(double) * nb);
    for (int b = 0; b < nb; ++b) m[b] = sim->particles[b].m;
    rec("m", m, nb);
    free(m);
  }
  for (int st = 1; st <= c->steps; ++st) {
    md_update_nhc_VV3_1_x(sim, c->dt);
    forces(pimd, &c2, 0);
    md_update_nhc_VV3_2_x(sim, c->dt);
  }
  forces(pimd, &c2, 0);
  rec_field("obs/", sim, 'x');
  rec_field("obs/", sim, 'f');
  md_pimd_calc_virial_energy_x(pimd, g_st);
  rec1("obs/e_virial", take());
  md_pimd_calc_centroid_virial_energy_x(pimd, g_st, 0);
  rec1("obs/e_centroid_fc0", take());
  md_pimd_calc_centroid_virial_energy_x(pimd, g_st, 3);
  rec1("obs/e_centroid_fc3", take());
  const int pts = 40;
  const double norm = 0.5 * c->N * (c->N - 1);
  for (int img = 0; img <= 1; ++img) {
    md_stats_t_x *st = md_alloc_stats_x(pts);
    st->fxs[0][3] = 0.25;  /* the call adds to what is there */
    md_pimd_calc_pair_correlation_x(pimd, st, Lb / 2, norm, c->P / 2 + 1, img);
    rec_stats_f(img ? "gr/image" : "gr/plain", st);
  }
  double grp[] = {pts, Lb / 2, norm, c->P / 2 + 1};
  rec("gr/params", grp, 4);
  md_pimd_polymer_periodic_boundary_x(pimd);
  rec_field("pbc/", sim, 'x');
  /* accumulator arithmetic on fxs */
  md_stats_t_x *a = md_alloc_stats_x(5), *b = md_alloc_stats_x(5), *q = md_alloc_stats_x(4);
  for (int i = 0; i < 5; ++i) b->fxs[0][i] = i + 0.5;
  b->es[0] = 1.5;
  md_reset_stats_f_x(a, 2.0);
  rec_stats_f("acc/reset", a);
  md_stats_add_to_f_x(a, b);
  rec_stats_f("acc/add", a);
  md_stats_mult_to_f_x(a, b);
  rec_stats_f("acc/mult", a);
  rec1("acc/add_mismatch_rc", md_stats_add_to_f_x(a, q));
  rec1("acc/copy_mismatch_rc", md_stats_copy_to_f_x(a, q));
  md_stats_copy_to_f_x(a, b);
  rec_stats_f("acc/copy", a);
}

static int geti(int argc, char **argv, const char *k, int dflt) {
  size_t n = strlen(k);
  for (int i = 3; i < argc; ++i)
    if (!strncmp(argv[i], k, n) && argv[i][n] == '=') return atoi(argv[i] + n + 1);
  return dflt;
}
static double getd(int argc, char **argv, const char *k, double dflt) {
  size_t n = strlen(k);
  for (int i = 3; i < argc; ++i)
    if (!strncmp(argv[i], k, n) && argv[i][n] == '=') return atof(argv[i] + n + 1);
  return dflt;
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s scenario out.bin [key=value ...]\n", argv[0]);
    return 2;
  }
  g_out = fopen(argv[2], "wb");
  if (!g_out) return 1;
  g_st = md_alloc_stats_x(1);
  scen_t c;
  c.N = geti(argc, argv, "N", 8);
  c.P = geti(argc, argv, "P", 8);
  c.f = geti(argc, argv, "f", 1);
  c.fc = geti(argc, argv, "fc", 0);
  c.steps = geti(argc, argv, "steps", 1);
  c.every = geti(argc, argv, "every", 100);
  c.nsum = geti(argc, argv, "nsum", 2);
  c.ueg = geti(argc, argv, "ueg", 0);
  c.image = geti(argc, argv, "image", 0);
  c.pbc = geti(argc, argv, "pbc", 0);
  c.seed = geti(argc, argv, "seed", 11);
  c.vi = getd(argc, argv, "vi", 1.0);
  c.beta = getd(argc, argv, "beta", 4.0);
  c.g = getd(argc, argv, "g", 0.75 * M_PI);
  c.s = getd(argc, argv, "s", 0.5);
  c.dt = getd(argc, argv, "dt", 0.005);
  c.rs = getd(argc, argv, "rs", 2.0);
  c.theta = getd(argc, argv, "theta", 0.5);
  c.alpha_L = getd(argc, argv, "alphaL", 5.6);
  c.box = getd(argc, argv, "box", 10.0);
  if (!strcmp(argv[1], "pimd"))
    run(&c);
  else if (!strcmp(argv[1], "cubic"))
    run_cubic(&c);
  else if (!strcmp(argv[1], "rng"))
    run_rng();
  else if (!strcmp(argv[1], "pairs"))
    run_pairs();
  else if (!strcmp(argv[1], "obs"))
    run_obs(&c);
  else if (!strcmp(argv[1], "two"))
    run_two(&c, geti(argc, argv, "Nb", 4), getd(argc, argv, "mb", 1.0));
  else
    return 2;
  fclose(g_out);
  return 0;
}
