/*
 * xmd_run.c -- a path-integral MD driver for libxmd_x, reading MD-Lab's
 * "key value" input files (md_read_attr_pair_x, md_util_x.c:95-119).
 *
 * MD-Lab ships sample inputs for its "Fast PIMD test" as plain key/value
 * text (N, P, T, omega, vi, g, s: particles, beads, temperature, trap
 * frequency, statistics parameter xi, Gaussian strength and range) but not
 * the main.c that reads them.  This driver reads the same keys, builds the
 * system through the MD-Lab C ABI (md_alloc_*, md_init_*, md_set_*), runs
 * the reference's per-step call sequence on the GPU library, and samples
 * the primitive and virial energy estimators.  Built once per library
 * variant (bin/xmd_run_d<D>l<L>, dimension D, chain length L).
 *
 *   xmd_run_d2l4 input.txt [--parse-only]
 *
 * Keys (missing ones take the defaults in brackets):
 *   N [500] P [72] T [1/6] omega [1] vi [1] g [0] s [0.5]   MD-Lab's names
 *   dt [0.01]  equil [1000]  steps [1000]  every [10]  seed [1]
 *   blocks [10]  batch of the block averages of the estimators
 *   ueg [0]: 1 = periodic electron gas (3D variants): box from rs [1],
 *            Ewald alpha = alphaL [5.6] / L, reciprocal cube nsum [8];
 *            T from theta [0.5] x the spin-polarised Fermi temperature
 *            when the input gives no T
 *   precision [0]: 1 = FP32 pair forces, 2 = every term in FP64
 *            (md_gb300_set_precision_x)
 * Output: "param key value" lines, then "sample step E_primitive
 * E_virial" every `every` steps after equilibration, and one line
 * "result E_primitive mean err E_virial mean err samples n blocks b
 * seconds t" (err: standard error of the block means).
 * Exit status 0, or 1 with a message on stderr.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "md_gb300_x.h"
#include "md_pimd_x.h"

#define D MD_DIMENSION_X

static md_attr_pair_t_x *g_attr;

static double key(const char *name, double dflt) {
  int found = 0;
  const double v = md_get_attr_value_x(g_attr, name, &found);
  return found ? v : dflt;
}

static int check(int rc, const char *what) {
  if (rc != 0) {
    fprintf(stderr, "xmd_run: %s failed (%d): %s\n", what, rc, md_gb300_last_error_x());
    exit(1);
  }
  return rc;
}

/* the value the last estimator call added to st (read on the host) */
static double take(md_stats_t_x *st) {
  st = md_stats_sync_host_x(st);
  if (!st) {
    fprintf(stderr, "xmd_run: accumulator read failed: %s\n", md_gb300_last_error_x());
    exit(1);
  }
  const double e = st->es[0];
  st->es[0] = 0;
  return e;
}

static double now(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return t.tv_sec + 1e-9 * t.tv_nsec;
}

static void mean_err(const double *v, int n, int blocks, double *mean, double *err) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += v[i];
  *mean = n ? s / n : 0;
  *err = 0;
  if (blocks < 2 || n < blocks) return;
  const int per = n / blocks;
  double bm[4096], sum = 0, sq = 0;
  if (blocks > 4096) blocks = 4096;
  for (int b = 0; b < blocks; ++b) {
    double t = 0;
    for (int i = 0; i < per; ++i) t += v[b * per + i];
    bm[b] = t / per;
    sum += bm[b];
  }
  const double m = sum / blocks;
  for (int b = 0; b < blocks; ++b) sq += (bm[b] - m) * (bm[b] - m);
  *err = sqrt(sq / (blocks - 1) / blocks);
}

int main(int argc, char **argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s input.txt [--parse-only]\n", argv[0]);
    return 1;
  }
  FILE *in = fopen(argv[1], "r");
  if (!in) {
    fprintf(stderr, "xmd_run: cannot open %s\n", argv[1]);
    return 1;
  }
  g_attr = md_read_attr_pair_x(in, NULL);
  fclose(in);
  if (!g_attr) {
    fprintf(stderr, "xmd_run: %s is not a list of \"key value\" pairs\n", argv[1]);
    return 1;
  }
  const int N = (int)key("N", 500), P = (int)key("P", 72);
  const int ueg = (int)key("ueg", 0);
  const double rs = key("rs", 1.0);
  double box = key("L", 10.0);
  if (ueg) box = cbrt(4.0 * M_PI * N / 3.0) * rs;
  double T = key("T", 1.0 / 6.0);
  if (ueg) {
    int found = 0;
    md_get_attr_value_x(g_attr, "T", &found);
    if (!found) T = key("theta", 0.5) * 0.5 * pow(6.0 * M_PI * M_PI * N / (box * box * box), 2.0 / 3.0);
  }
  const double omega = key("omega", 1.0), vi = key("vi", 1.0), g = key("g", 0.0), s = key("s", 0.5);
  const double dt = key("dt", 0.01), alphaL = key("alphaL", 5.6);
  const int equil = (int)key("equil", 1000), steps = (int)key("steps", 1000), every = (int)key("every", 10);
  const int seed = (int)key("seed", 1), blocks = (int)key("blocks", 10), nsum = (int)key("nsum", 8);
  const int precision = (int)key("precision", 0);
  printf("param N %d\nparam P %d\nparam D %d\nparam T %.17g\nparam omega %.17g\nparam vi %.17g\n", N, P, D, T, omega,
         vi);
  printf("param g %.17g\nparam s %.17g\nparam dt %.17g\nparam equil %d\nparam steps %d\nparam every %d\n", g, s, dt,
         equil, steps, every);
  printf("param seed %d\nparam ueg %d\nparam L %.17g\nparam nsum %d\nparam precision %d\n", seed, ueg, box, nsum,
         precision);
  if (N < 1 || P < 2 || every < 1 || T <= 0 || (ueg && D != 3)) {
    fprintf(stderr, "xmd_run: invalid parameters (N >= 1, P >= 2, every >= 1, T > 0; ueg needs D = 3)\n");
    return 1;
  }
  if (argc > 2 && !strcmp(argv[2], "--parse-only")) return 0;

  /* the system, through the MD-Lab C ABI */
  md_set_pimd_mode_x(1);
  md_set_seed_x((unsigned)seed);
  md_simulation_t_x *sim = md_alloc_simulation_x(N * P, 1, 0, MD_ND_RECT_BOX_X);
  if (!sim) return check(-1, "md_alloc_simulation_x");
  double Lv[D], c[D], zero[D];
  for (int d = 0; d < D; ++d) {
    Lv[d] = box;
    c[d] = ueg ? box / 2 : 0.0;
    zero[d] = 0.0;
  }
  check(md_init_nd_rect_box_x(sim->box, Lv), "md_init_nd_rect_box_x");
  md_pimd_t_x *pimd = md_alloc_pimd_x(sim, N, P, vi, T);
  if (!pimd) return check(-1, "md_alloc_pimd_x");
  check(md_init_particle_mass_x(sim, 1.0, 0, N * P), "md_init_particle_mass_x");
  if (ueg) {
    check(md_pimd_init_particle_uniform_pos_x(pimd, c, Lv, 0.05 * rs), "md_pimd_init_particle_uniform_pos_x");
  } else {
    for (int b = 0; b < N * P; ++b)
      for (int d = 0; d < D; ++d) sim->particles[b].x[d] = md_random_gaussian_x() / sqrt(omega);
  }
  check(md_init_maxwell_vel_x(sim, T), "md_init_maxwell_vel_x");
  check(md_init_nhc_x(sim, md_get_quick_Q_x(T, pimd->omegaP), 0, sim->Nf, 0.0), "md_init_nhc_x");
  md_set_harmonic_trap_frequency_x(omega);
  md_set_harmonic_trap_center_x(zero);
  md_set_gaussian_force_strength_x(g);
  md_set_guassian_force_range_x(s);
  md_set_coulomb_force_strength_x(1.0);
  md_set_coulomb_truc_x(alphaL / box);
  md_set_coulomb_n_sum_x(nsum);
  check(md_gb300_set_precision_x(precision), "md_gb300_set_precision_x");
  const int image = ueg ? 1 : 0;
  md_trap_force_t_x tf = ueg ? NULL : md_harmonic_trap_force_x;
  md_pair_force_t_x pf = ueg ? md_coulomb_3d_ewald_force_x : (g != 0.0 ? md_gaussian_force_x : NULL);
  md_pair_energy_t_x pe = ueg ? md_coulomb_3d_ewald_energy_x : (g != 0.0 ? md_gaussian_energy_x : NULL);
  md_stats_t_x *st = md_alloc_stats_x(1);
  const int nsamp = steps / every;
  double *eprim = (double *)calloc(nsamp > 0 ? nsamp : 1, sizeof(double));
  double *evir = (double *)calloc(nsamp > 0 ? nsamp : 1, sizeof(double));
  if (!st || !eprim || !evir) return check(-1, "allocation");

  /* the reference's per-step call sequence */
  const double t0 = now();
  int ns = 0;
  for (int it = 1; it <= equil + steps; ++it) {
    check(md_update_nhc_VV3_1_x(sim, dt), "md_update_nhc_VV3_1_x");
    check(md_reset_force_x(sim), "md_reset_force_x");
    check(md_pimd_fast_fill_ENk_x(pimd, image), "md_pimd_fast_fill_ENk_x");
    check(md_pimd_fill_VB_x(pimd), "md_pimd_fill_VB_x");
    check(md_pimd_fast_fill_force_VB_x(pimd, image), "md_pimd_fast_fill_force_VB_x");
    if (tf) check(md_pimd_calc_trap_force_x(pimd, tf), "md_pimd_calc_trap_force_x");
    if (pf) check(md_pimd_calc_pair_force_x(pimd, pf), "md_pimd_calc_pair_force_x");
    check(md_update_nhc_VV3_2_x(sim, dt), "md_update_nhc_VV3_2_x");
    if (ueg) check(md_periodic_boundary_x(sim), "md_periodic_boundary_x");
    if (it > equil && (it - equil) % every == 0 && ns < nsamp) {
      /* estimators at the positions of the step's forces: the potential
         part (trap, pairs) is common to both */
      double pot = 0;
      if (!ueg) {
        check(md_pimd_calc_trap_energy_x(pimd, md_harmonic_trap_energy_x, st), "md_pimd_calc_trap_energy_x");
        pot += take(st);
      }
      if (pe) {
        check(md_pimd_calc_pair_energy_x(pimd, pe, st), "md_pimd_calc_pair_energy_x");
        pot += take(st);
      }
      check(md_pimd_calc_VBN_energy_x(pimd, st), "md_pimd_calc_VBN_energy_x");
      eprim[ns] = take(st) + pot;
      check(md_pimd_fast_fill_ENk2_x(pimd, image), "md_pimd_fast_fill_ENk2_x");
      check(md_pimd_calc_vi_virial_energy_x(pimd, st, image), "md_pimd_calc_vi_virial_energy_x");
      evir[ns] = take(st) + pot;
      printf("sample %d %.17g %.17g\n", it, eprim[ns], evir[ns]);
      ++ns;
    }
  }
  check(md_gb300_synchronize_x(), "md_gb300_synchronize_x");
  const double secs = now() - t0;
  double mp, ep, mv, ev;
  mean_err(eprim, ns, blocks, &mp, &ep);
  mean_err(evir, ns, blocks, &mv, &ev);
  printf("result E_primitive %.17g %.6g E_virial %.17g %.6g samples %d blocks %d seconds %.3f\n", mp, ep, mv, ev, ns,
         blocks, secs);
  free(eprim);
  free(evir);
  md_gb300_free_stats_x(st);
  md_gb300_free_pimd_x(pimd);
  md_gb300_free_simulation_x(sim);
  return 0;
}
