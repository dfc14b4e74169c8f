// xmd_host.cpp -- host side of the MD-Lab C ABI in libxmd_x: parameters,
// potentials (CPU bodies, kept so drivers can call them on host data),
// allocation, initial conditions, random numbers, text checkpoints and the
// block-averaging accumulator.
//
// Counterparts: md_simulation_x.c:70-419 (geometry, potentials, setters),
// md_util_x.c:84-1011 and :1634-1653 (set-up, allocation, initial
// conditions, RNG, text I/O), md_statistics_x.c:203-396 (accumulator and
// energies), md_pimd_x.c:330-567 (path-integral allocation and indices).
// Random numbers must match the reference bit for bit, so they come from
// the same glibc rand() stream through the same Box-Muller pairing.
#include <cmath>
#include <vector>
#include <array>
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "xmd_internal.h"

using xmd::host_alloc;
using xmd::host_free;

static const int D = MD_DIMENSION_X;
static const int LC = MD_NHC_LENGTH_X;

extern "C" {

// ------------------------------------------------------------------
// parameters (md_simulation_x.c:124-221)
// ------------------------------------------------------------------
md_num_t_x md_trap_frequency_x;
md_num_t_x md_trap_center_x[MD_DIMENSION_X];
md_num_t_x md_trap_frequency_2_x[MD_DIMENSION_X];
md_num_t_x md_gaussian_strength_x;
md_num_t_x md_gaussian_range_x;
md_num_t_x md_coulomb_strength_x;
md_num_t_x md_coulomb_truc_x;
int md_coulomb_n_sum_x;
int md_pimd_mode_x = 0;

void md_set_pimd_mode_x(int pimd_mode) { md_pimd_mode_x = pimd_mode; }
void md_set_harmonic_trap_frequency_x(md_num_t_x f) { md_trap_frequency_x = f; }
void md_set_harmonic_trap_center_x(md_num_t_x *c) {
  for (int d = 0; d < D; ++d) md_trap_center_x[d] = c[d];
}
void md_set_harmonic_trap_frequency_2_x(md_num_t_x *f) {
  for (int d = 0; d < D; ++d) md_trap_frequency_2_x[d] = f[d];
}
void md_set_gaussian_force_strength_x(md_num_t_x g) { md_gaussian_strength_x = g; }
void md_set_guassian_force_range_x(md_num_t_x s) { md_gaussian_range_x = s; }
void md_set_coulomb_force_strength_x(md_num_t_x g) { md_coulomb_strength_x = g; }
void md_set_coulomb_truc_x(md_num_t_x k) { md_coulomb_truc_x = k; }
void md_set_coulomb_n_sum_x(int n) { md_coulomb_n_sum_x = n; }

// ------------------------------------------------------------------
// geometry (md_simulation_x.c:70-114, :858-865)
// ------------------------------------------------------------------
int md_periodic_image_count_x(md_num_t_x x, md_num_t_x L) {
  const int c = (int)(fabs(x) / L);
  return x > L ? -c : (x < 0 ? c + 1 : 0);
}

md_num_t_x md_minimum_image_x(md_num_t_x a, md_num_t_x L) {
  const double s = a + L / 2;
  return s + L * md_periodic_image_count_x(s, L) - L / 2;
}

md_num_t_x md_distance_x(md_num_t_x *p1, md_num_t_x *p2) {
  double s = 0;
  for (int d = 0; d < D; ++d) s += (p1[d] - p2[d]) * (p1[d] - p2[d]);
  return sqrt(s);
}

md_num_t_x md_minimum_image_distance_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L) {
  double s = 0;
  for (int d = 0; d < D; ++d) {
    const double t = md_minimum_image_x(p1[d] - p2[d], L[d]);
    s += t * t;
  }
  return sqrt(s);
}

// ------------------------------------------------------------------
// potentials: forces (md_simulation_x.c:127-293), stored as F/m
// ------------------------------------------------------------------
void md_harmonic_trap_force_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *MD_UNUSED_X(L),
                              md_num_t_x MD_UNUSED_X(m)) {
  const double w2 = md_trap_frequency_x * md_trap_frequency_x;
  for (int d = 0; d < D; ++d) f[d] += -w2 * (p1[d] - md_trap_center_x[d]);
}

void md_neg_harmonic_trap_force_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *MD_UNUSED_X(L),
                                  md_num_t_x MD_UNUSED_X(m)) {
  const double w2 = md_trap_frequency_x * md_trap_frequency_x;
  for (int d = 0; d < D; ++d) f[d] -= -w2 * (p1[d] - md_trap_center_x[d]);
}

void md_harmonic_trap_force_2_x(md_num_t_x *p1, md_num_t_x *f, md_num_t_x *MD_UNUSED_X(L),
                                md_num_t_x MD_UNUSED_X(m)) {
  for (int d = 0; d < D; ++d)
    f[d] += -md_trap_frequency_2_x[d] * md_trap_frequency_2_x[d] * (p1[d] - md_trap_center_x[d]);
}

static void gauss_force(double *dx, double r, double *f, double m) {
  const double s2 = md_gaussian_range_x * md_gaussian_range_x;
  const double amp = (md_gaussian_strength_x / (M_PI * s2)) * exp(-r * r / s2);
  for (int d = 0; d < D; ++d) f[d] += amp * (2 * dx[d]) / s2 / m;
}

void md_gaussian_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *MD_UNUSED_X(L),
                         md_num_t_x m) {
  double dx[MD_DIMENSION_X];
  for (int d = 0; d < D; ++d) dx[d] = p1[d] - p2[d];
  gauss_force(dx, md_distance_x(p1, p2), f, m);
}

void md_periodic_gaussian_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L,
                                  md_num_t_x m) {
  double dx[MD_DIMENSION_X];
  for (int d = 0; d < D; ++d) dx[d] = md_minimum_image_x(p1[d] - p2[d], L[d]);
  gauss_force(dx, md_minimum_image_distance_x(p1, p2, L), f, m);
}

void md_coulomb_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *MD_UNUSED_X(L),
                        md_num_t_x m) {
  const double k = md_coulomb_strength_x / pow(md_distance_x(p1, p2), 3);
  for (int d = 0; d < D; ++d) f[d] += k * (p1[d] - p2[d]) / m;
}

void md_coulomb_periodic_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L,
                                 md_num_t_x m) {
  const double k = md_coulomb_strength_x / pow(md_minimum_image_distance_x(p1, p2, L), 3);
  for (int d = 0; d < D; ++d) f[d] += k * md_minimum_image_x(p1[d] - p2[d], L[d]) / m;
}

// Ewald: reciprocal sum over the cube |n_i| <= n (n != 0) plus real-space
// images over the same cube; md_simulation_x.c:259-293 (3D only)
void md_coulomb_3d_ewald_force_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *f, md_num_t_x *L,
                                 md_num_t_x m) {
  if (D != 3) return;
  const int n = md_coulomb_n_sum_x;
  const double a = md_coulomb_truc_x, qs = md_coulomb_strength_x;
  const double vol = L[0] * L[1] * L[2];
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (!i && !j && !k) continue;
        const double g[3] = {i / L[0], j / L[1], k / L[2]};
        const double G = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        const double ph = 2 * M_PI * (g[0] * (p1[0] - p2[0]) + g[1] * (p1[1] - p2[1]) + g[2] * (p1[2] - p2[2]));
        const double w = qs * sin(ph) * pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (vol * M_PI);
        for (int d = 0; d < 3; ++d) f[d] += 2 * M_PI * g[d] * w / m;
      }
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        const double r[3] = {p1[0] - (p2[0] + i * L[0]), p1[1] - (p2[1] + j * L[1]), p1[2] - (p2[2] + k * L[2])};
        const double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        const double w = qs * 2 * a * exp(-a * a * R * R) / (sqrt(M_PI) * R * R) + qs * erfc(a * R) / (R * R * R);
        for (int d = 0; d < 3; ++d) f[d] += r[d] * w / m;
      }
}

// self / background constant of the Ewald sum: md_simulation_x.c:223-257
md_num_t_x md_calc_3d_ueg_madelung_x(md_num_t_x *L) {
  if (D != 3) return 0;
  const int n = md_coulomb_n_sum_x;
  const double a = md_coulomb_truc_x, vol = L[0] * L[1] * L[2];
  double res = 0;
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (!i && !j && !k) continue;
        const double g[3] = {i / L[0], j / L[1], k / L[2]};
        const double G = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        res += pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (vol * M_PI);
      }
  res -= M_PI / (a * a * vol);
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (!i && !j && !k) continue;
        const double r[3] = {i * L[0], j * L[1], k * L[2]};
        const double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        res += erfc(a * R) / R;
      }
  res -= 2 * a * pow(M_PI, -0.5);
  return md_coulomb_strength_x * res;
}

// ------------------------------------------------------------------
// potentials: energies (md_statistics_x.c:322-396)
// ------------------------------------------------------------------
md_num_t_x md_harmonic_trap_energy_x(md_num_t_x *p1, md_num_t_x *MD_UNUSED_X(L), md_num_t_x m) {
  const double r = md_distance_x(p1, md_trap_center_x);
  return 0.5 * m * md_trap_frequency_x * md_trap_frequency_x * r * r;
}

md_num_t_x md_neg_harmonic_trap_energy_x(md_num_t_x *p1, md_num_t_x *L, md_num_t_x m) {
  return -md_harmonic_trap_energy_x(p1, L, m);
}

md_num_t_x md_harmonic_trap_energy_2_x(md_num_t_x *p1, md_num_t_x *MD_UNUSED_X(L), md_num_t_x m) {
  double e = 0;
  for (int d = 0; d < D; ++d)
    e += 0.5 * m * md_trap_frequency_2_x[d] * md_trap_frequency_2_x[d] * (p1[d] - md_trap_center_x[d]) *
         (p1[d] - md_trap_center_x[d]);
  return e;
}

static double gauss_energy(double r) {
  const double s2 = md_gaussian_range_x * md_gaussian_range_x;
  return (md_gaussian_strength_x / (M_PI * s2)) * exp(-r * r / s2);
}

md_num_t_x md_gaussian_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *MD_UNUSED_X(L),
                                md_num_t_x MD_UNUSED_X(m)) {
  return gauss_energy(md_distance_x(p1, p2));
}

md_num_t_x md_periodic_gaussian_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L,
                                         md_num_t_x MD_UNUSED_X(m)) {
  return gauss_energy(md_minimum_image_distance_x(p1, p2, L));
}

md_num_t_x md_coulomb_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *MD_UNUSED_X(L),
                               md_num_t_x MD_UNUSED_X(m)) {
  return md_coulomb_strength_x / md_distance_x(p1, p2);
}

md_num_t_x md_coulomb_periodic_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L,
                                        md_num_t_x MD_UNUSED_X(m)) {
  return md_coulomb_strength_x / md_minimum_image_distance_x(p1, p2, L);
}

md_num_t_x md_coulomb_3d_ewald_energy_x(md_num_t_x *p1, md_num_t_x *p2, md_num_t_x *L,
                                        md_num_t_x MD_UNUSED_X(m)) {
  if (D != 3) return 0;
  const int n = md_coulomb_n_sum_x;
  const double a = md_coulomb_truc_x, vol = L[0] * L[1] * L[2];
  double res = 0;
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (!i && !j && !k) continue;
        const double g[3] = {i / L[0], j / L[1], k / L[2]};
        const double G = sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
        const double ph = 2 * M_PI * (g[0] * (p1[0] - p2[0]) + g[1] * (p1[1] - p2[1]) + g[2] * (p1[2] - p2[2]));
        res += cos(ph) * pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (vol * M_PI);
      }
  res -= M_PI / (a * a * vol);
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        const double r[3] = {p1[0] - (p2[0] + i * L[0]), p1[1] - (p2[1] + j * L[1]), p1[2] - (p2[2] + k * L[2])};
        const double R = sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
        res += erfc(a * R) / R;
      }
  return md_coulomb_strength_x * res;
}

// ------------------------------------------------------------------
// key/value input (md_util_x.c:84-134)
// ------------------------------------------------------------------
md_attr_pair_t_x *md_alloc_attr_pair_x(void) {
  md_attr_pair_t_x *a = (md_attr_pair_t_x *)calloc(1, sizeof(md_attr_pair_t_x));
  return a;
}

md_attr_pair_t_x *md_read_attr_pair_x(FILE *in, md_attr_pair_t_x *attr) {
  md_attr_pair_t_x *a = attr ? attr : md_alloc_attr_pair_x();
  if (!a) return NULL;
  char key[MD_MAX_NAME_LENGTH_X + 1];
  char fmt[32];
  snprintf(fmt, sizeof fmt, "%%%ds", MD_MAX_NAME_LENGTH_X);
  while (fscanf(in, fmt, key) == 1 && key[0]) {
    double v;
    if (fscanf(in, "%lf", &v) != 1) return NULL;
    md_name_t_x *names = (md_name_t_x *)realloc(a->names, sizeof(md_name_t_x) * (a->N + 1));
    md_num_t_x *vals = (md_num_t_x *)realloc(a->values, sizeof(md_num_t_x) * (a->N + 1));
    if (!names || !vals) return NULL;
    a->names = names;
    a->values = vals;
    strcpy(a->names[a->N], key);
    a->values[a->N] = v;
    a->N++;
    key[0] = '\0';
  }
  return a;
}

md_num_t_x md_get_attr_value_x(md_attr_pair_t_x *attr, const char *name, int *found) {
  if (found) *found = 0;
  for (int i = 0; i < attr->N; ++i)
    if (!strcmp(name, attr->names[i])) {
      if (found) *found = 1;
      return attr->values[i];
    }
  return 0;
}

// ------------------------------------------------------------------
// random numbers (md_util_x.c:671-693)
// ------------------------------------------------------------------
static double g_gauss_spare;
static int g_gauss_has = 0;

void md_set_seed_x(unsigned int seed) { srand(seed); }

md_num_t_x md_random_uniform_x(md_num_t_x a, md_num_t_x b) {
  const double u = ((double)rand()) / RAND_MAX;
  return a + (b - a) * u;
}

md_num_t_x md_random_gaussian_x(void) {
  if (g_gauss_has) {
    g_gauss_has = 0;
    return g_gauss_spare;
  }
  const double rad = sqrt(-2 * log(md_random_uniform_x(0, 1)));
  const double ang = 2 * M_PI * md_random_uniform_x(0, 1);
  g_gauss_spare = rad * sin(ang);
  g_gauss_has = 1;
  return rad * cos(ang);
}

md_num_t_x md_get_quick_Q_x(md_num_t_x T, md_num_t_x omega) { return T * MD_kB_X / (omega * omega); }

// md_util_x.c:348-356: seeds the generator; there is no run-time kernel
// build.  A missing GPU is reported, because every compute call needs one.
int md_init_setup_x(FILE *out, void *config) {
  md_init_config_x *c = (md_init_config_x *)config;
  if (c) md_set_seed_x(c->seed);
  const int rc = xmd::ensure_device();
  if (out) {
    if (rc == 0) {
      int dev = 0;
      cudaDeviceProp p;
      cudaGetDevice(&dev);
      cudaGetDeviceProperties(&p, dev);
      fprintf(out, "libxmd_x: %s, %d SMs, sm_%d%d\n", p.name, p.multiProcessorCount, p.major, p.minor);
    }
    fprintf(out, "Initialization completed\n");
  }
  return rc;
}

// ------------------------------------------------------------------
// allocation and initial conditions (md_util_x.c:553-836)
// ------------------------------------------------------------------
simulation_box_t_x *md_alloc_box_x(int box_type) {
  if (box_type != MD_ND_RECT_BOX_X) return NULL;
  simulation_box_t_x *b = (simulation_box_t_x *)calloc(1, sizeof(simulation_box_t_x));
  if (!b) return NULL;
  b->type = box_type;
  b->box = calloc(1, sizeof(nd_rect_t_x));
  if (!b->box) {
    free(b);
    return NULL;
  }
  return b;
}

md_simulation_t_x *md_alloc_simulation_x(int N, int f, int fc, int box_type) {
  if (N < 1 || f < 1) return NULL;
  md_simulation_t_x *s = (md_simulation_t_x *)calloc(1, sizeof(md_simulation_t_x));
  if (!s) return NULL;
  s->N = N;
  s->particles = (md_particle_t_x *)host_alloc(sizeof(md_particle_t_x) * (size_t)N);
  const int ndof = D * N - fc;
  s->fc = ndof;
  s->Nf = ndof / f + (ndof % f != 0);
  s->fs = (int *)malloc(sizeof(int) * (s->Nf > 0 ? s->Nf : 1));
  s->f0s = (int *)malloc(sizeof(int) * (s->Nf > 0 ? s->Nf : 1));
  s->nhcs = (md_nhc_t_x *)host_alloc(sizeof(md_nhc_t_x) * (size_t)(s->Nf > 0 ? s->Nf : 1));
  s->box = md_alloc_box_x(box_type);
  if (!s->particles || !s->fs || !s->f0s || !s->nhcs || !s->box) {
    md_gb300_free_simulation_x(s);
    return NULL;
  }
  for (int i = 0, f0 = 0; i < s->Nf; ++i) {
    s->fs[i] = (i + 1) * f > ndof ? ndof - i * f : f;
    s->f0s[i] = f0;
    f0 += s->fs[i];
  }
  s->pcount_in = N * (N + 1) / 2;
  s->pcount_ex = N * (N - 1) / 2;
  if (!md_pimd_mode_x) {
    s->pair_in = (md_index_pair_t_x *)malloc(sizeof(md_index_pair_t_x) * (size_t)s->pcount_in);
    s->pair_ex = (md_index_pair_t_x *)malloc(sizeof(md_index_pair_t_x) * (size_t)(s->pcount_ex > 0 ? s->pcount_ex : 1));
    if (!s->pair_in || !s->pair_ex) {
      md_gb300_free_simulation_x(s);
      return NULL;
    }
    int a = 0, b = 0;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j <= i; ++j) {
        s->pair_in[a++] = {i, j};
        if (j < i) s->pair_ex[b++] = {i, j};
      }
  }
  return s;
}

void md_gb300_free_simulation_x(md_simulation_t_x *s) {
  if (!s) return;
  xmd::forget(s);
  host_free(s->particles);
  host_free(s->nhcs);
  free(s->fs);
  free(s->f0s);
  free(s->pair_in);
  free(s->pair_ex);
  if (s->box) free(s->box->box);
  free(s->box);
  free(s);
}

int md_init_nd_rect_box_x(simulation_box_t_x *box, md_num_t_x *L) {
  if (box->type != MD_ND_RECT_BOX_X) return -1;
  nd_rect_t_x *r = (nd_rect_t_x *)box->box;
  for (int d = 0; d < D; ++d) r->L[d] = L[d];
  return 0;
}

md_simulation_t_x *md_simulation_sync_host_x(md_simulation_t_x *sim, int read_only) {
  return xmd::sim_to_host(sim, read_only != 0) == 0 ? sim : NULL;
}

int md_init_particle_mass_x(md_simulation_t_x *sim, md_num_t_x m, int start, int end) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  for (int i = start; i < end; ++i) sim->particles[i].m = m;
  return 0;
}

// Maxwell-Boltzmann velocities with the mean momentum per particle removed:
// md_util_x.c:695-716
int md_init_maxwell_vel_x(md_simulation_t_x *sim, md_num_t_x T) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  double mom[MD_DIMENSION_X] = {0};
  for (int i = 0; i < sim->N; ++i)
    for (int d = 0; d < D; ++d) {
      md_particle_t_x *p = &sim->particles[i];
      p->v[d] = md_random_gaussian_x() * sqrt(MD_kB_X * T / p->m);
      mom[d] += p->m * p->v[d];
    }
  for (int d = 0; d < D; ++d) mom[d] /= sim->N;
  for (int i = 0; i < sim->N; ++i)
    for (int d = 0; d < D; ++d) sim->particles[i].v[d] -= mom[d] / sim->particles[i].m;
  return 0;
}

// fcc lattice in four interleaved sub-lattices: md_util_x.c:728-803
int md_init_particle_face_center_3d_lattice_pos_x(md_simulation_t_x *sim, md_num_t_x *center,
                                                   md_num_t_x *length, md_num_t_x fluc,
                                                   md_num_t_x eps) {
  if (D != 3) return -1;
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  const double side = pow(sim->N / 4.0, 1.0 / D);
  int M = (int)side;
  if (side - M != 0) ++M;
  int count = 0;
  // sub-lattice s shifts every axis but (s-1) by half a cell (s = 0: none)
  for (int s = 0; s < 4; ++s)
    for (int i = 0; i < M; ++i)
      for (int j = 0; j < M; ++j)
        for (int k = 0; k < M; ++k) {
          if (count >= sim->N) break;
          const int cell[3] = {i, j, k};
          for (int d = 0; d < D; ++d) {
            double x = center[d] - length[d] / 2.0 + cell[d] * length[d] / M;
            if (s > 0 && d != s - 1) x += length[d] / M / 2.0;
            sim->particles[count].x[d] = x + eps + md_random_uniform_x(-fluc, fluc);
          }
          ++count;
        }
  return 0;
}

// md_util_x.c:805-825
int md_init_nhc_x(md_simulation_t_x *sim, md_num_t_x Q, int start, int end, md_num_t_x fp) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  for (int i = start; i < end; ++i) {
    md_nhc_t_x *c = &sim->nhcs[i];
    c->f = sim->fs[i];
    for (int j = 0; j < LC; ++j) {
      c->theta[j] = 0;
      c->vtheta[j] = 1;
      c->Q[j] = Q;
    }
    c->Q[0] = (fp == 0.0) ? c->f * Q : fp * Q;
  }
  return 0;
}

int md_simulation_copy_to_x(md_simulation_t_x *sim, md_simulation_t_x *sim2) {
  if (sim->N != sim2->N || sim->Nf != sim2->Nf) return -1;
  if (!md_simulation_sync_host_x(sim, 0) || !md_simulation_sync_host_x(sim2, 1)) return -1;
  for (int i = 0; i < sim->N; ++i) {
    memcpy(sim->particles[i].x, sim2->particles[i].x, sizeof(sim->particles[i].x));
    memcpy(sim->particles[i].v, sim2->particles[i].v, sizeof(sim->particles[i].v));
    sim->particles[i].m = sim2->particles[i].m;
  }
  for (int i = 0; i < sim->Nf; ++i) sim->nhcs[i] = sim2->nhcs[i];
  return 0;
}

// host evaluation of one chain's thermostat forces: md_simulation_x.c:599-613
void md_calc_nhc_force_x(md_simulation_t_x *sim, int f0, int f2, int i, md_num_t_x *res) {
  double kin = 0;
  for (int j = 0; j < f2; ++j) {
    const int dof = f0 + j;
    const md_particle_t_x *p = &sim->particles[dof / D];
    kin += p->m * p->v[dof % D] * p->v[dof % D];
  }
  const md_nhc_t_x *c = &sim->nhcs[i];
  res[0] = (kin - c->f * MD_kB_X * sim->T) / c->Q[0];
  for (int j = 1; j < LC; ++j) res[j] = (c->Q[j - 1] * c->vtheta[j - 1] * c->vtheta[j - 1] - MD_kB_X * sim->T) / c->Q[j];
}

// md_simulation_x.c:888-899 (host, after a sync)
int md_simulation_rescale_velocity_x(md_simulation_t_x *sim, md_num_t_x T) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  double kin = 0;
  for (int i = 0; i < sim->N; ++i)
    for (int d = 0; d < D; ++d) kin += sim->particles[i].m * sim->particles[i].v[d] * sim->particles[i].v[d];
  const double lam = sqrt(sim->fc * MD_kB_X * T / kin);
  for (int i = 0; i < sim->N; ++i)
    for (int d = 0; d < D; ++d) sim->particles[i].v[d] *= lam;
  return 0;
}

// number format of the text checkpoints: the reference's "%f " (6 decimals,
// lossy) by default; "%.17g " (md_gb300_set_text_exact_x(1)) round-trips
// every double exactly and is still read by the reference's fscanf("%lf")
static const char *g_text_fmt = "%f ";

extern "C" int md_gb300_set_text_exact_x(int on) {
  g_text_fmt = on ? "%.17g " : "%f ";
  return 0;
}

// ------------------------------------------------------------------
// text checkpoints (md_util_x.c:838-1011), same format
// ------------------------------------------------------------------
static int print_field(FILE *out, md_simulation_t_x *sim, char tag) {
  fprintf(out, "%c %d %d\n", tag, sim->N, D);
  if (!(sim = md_simulation_sync_host_x(sim, 1))) return -1;
  for (int i = 0; i < sim->N; ++i) {
    const md_particle_t_x *p = &sim->particles[i];
    const double *v = tag == 'x' ? p->x : tag == 'v' ? p->v : p->f;
    for (int d = 0; d < D; ++d) fprintf(out, g_text_fmt, v[d]);
    fprintf(out, "\n");
  }
  return ferror(out);
}

int md_fprint_particle_pos_x(FILE *out, md_simulation_t_x *sim) { return print_field(out, sim, 'x'); }
int md_fprint_particle_vel_x(FILE *out, md_simulation_t_x *sim) { return print_field(out, sim, 'v'); }
int md_fprint_particle_force_x(FILE *out, md_simulation_t_x *sim) { return print_field(out, sim, 'f'); }

int md_fprint_nhcs_x(FILE *out, md_simulation_t_x *sim) {
  fprintf(out, "nhc %d %d\n", sim->Nf, LC);
  if (!(sim = md_simulation_sync_host_x(sim, 1))) return -1;
  for (int i = 0; i < sim->Nf; ++i) {
    const md_nhc_t_x *c = &sim->nhcs[i];
    fprintf(out, "%d\n", c->f);
    const double *rows[3] = {c->theta, c->vtheta, c->Q};
    for (int r = 0; r < 3; ++r) {
      for (int j = 0; j < LC; ++j) fprintf(out, g_text_fmt, rows[r][j]);
      fprintf(out, "\n");
    }
  }
  return ferror(out);
}

int md_fprint_sim_box_x(FILE *out, simulation_box_t_x *box) {
  fprintf(out, "box %d %d\n", box->type, D);
  if (box->type == MD_ND_RECT_BOX_X) {
    const nd_rect_t_x *r = (const nd_rect_t_x *)box->box;
    for (int d = 0; d < D; ++d) fprintf(out, g_text_fmt, r->L[d]);
    fprintf(out, "\n");
  }
  return ferror(out);
}

static int read_header(FILE *in, int expect_n, int expect_d) {
  char tag[32];
  int n, d;
  if (fscanf(in, "%31s", tag) != 1 || fscanf(in, "%d", &n) != 1 || n != expect_n) return -1;
  if (fscanf(in, "%d", &d) != 1 || d != expect_d) return -1;
  return 0;
}

static int read_field(FILE *in, md_simulation_t_x *sim, char tag) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  if (read_header(in, sim->N, D)) return -1;
  for (int i = 0; i < sim->N; ++i)
    for (int d = 0; d < D; ++d) {
      double v;
      if (fscanf(in, "%lf", &v) != 1) return -1;
      (tag == 'x' ? sim->particles[i].x : sim->particles[i].v)[d] = v;
    }
  return ferror(in);
}

int md_fread_particle_pos_x(FILE *in, md_simulation_t_x *sim) { return read_field(in, sim, 'x'); }
int md_fread_particle_vel_x(FILE *in, md_simulation_t_x *sim) { return read_field(in, sim, 'v'); }

int md_fread_nhcs_x(FILE *in, md_simulation_t_x *sim) {
  if (!(sim = md_simulation_sync_host_x(sim, 0))) return -1;
  if (read_header(in, sim->Nf, LC)) return -1;
  for (int i = 0; i < sim->Nf; ++i) {
    md_nhc_t_x *c = &sim->nhcs[i];
    if (fscanf(in, "%d", &c->f) != 1) return -1;
    double *rows[3] = {c->theta, c->vtheta, c->Q};
    for (int r = 0; r < 3; ++r)
      for (int j = 0; j < LC; ++j)
        if (fscanf(in, "%lf", &rows[r][j]) != 1) return -1;
  }
  return ferror(in);
}

// ------------------------------------------------------------------
// block-averaging accumulator (md_statistics_x.c:203-315,
// md_pimd_x.c:4558-4650)
// ------------------------------------------------------------------
md_stats_t_x *md_stats_sync_host_x(md_stats_t_x *stats) {
  return xmd::stats_to_host(stats) == 0 ? stats : NULL;
}

// md_statistics_x.c:104-161: wave vectors on the cube q0, q0 + qincre, ...
// <= qmax per component (loop order x, y, z), one per distinct |q| (first
// found within 1e-4), skipping |q| < 1e-4; ascending |q|
md_sk_sphere_t_x *md_alloc_sk_sphere_3d_x(md_num_t_x q0, md_num_t_x qincre, md_num_t_x qmax) {
  if (D != 3 || !(qincre > 0)) return NULL;
  std::vector<std::array<double, 4>> v;  // |q|, qx, qy, qz
  for (double qx = q0; qx <= qmax; qx += qincre)
    for (double qy = q0; qy <= qmax; qy += qincre)
      for (double qz = q0; qz <= qmax; qz += qincre) {
        const double q = sqrt(qx * qx + qy * qy + qz * qz);
        if (fabs(q) < 1e-4) continue;
        bool found = false;
        for (const auto &e : v)
          if (fabs(e[0] - q) < 1e-4) {
            found = true;
            break;
          }
        if (!found) v.push_back({q, qx, qy, qz});
      }
  std::stable_sort(v.begin(), v.end(), [](const std::array<double, 4> &a, const std::array<double, 4> &b) {
    return a[0] < b[0];
  });
  md_sk_sphere_t_x *r = (md_sk_sphere_t_x *)calloc(1, sizeof(md_sk_sphere_t_x));
  if (!r) return NULL;
  r->N = (int)v.size();
  r->qs = (md_num_t_x *)malloc(sizeof(md_num_t_x) * (v.empty() ? 1 : v.size()));
  r->qis = (md_num_t_x *)malloc(sizeof(md_num_t_x) * 3 * (v.empty() ? 1 : v.size()));
  if (!r->qs || !r->qis) {
    free(r->qs);
    free(r->qis);
    free(r);
    return NULL;
  }
  for (size_t i = 0; i < v.size(); ++i) {
    r->qs[i] = v[i][0];
    for (int d = 0; d < 3; ++d) r->qis[3 * i + d] = v[i][1 + d];
  }
  return r;
}

md_stats_t_x *md_alloc_stats_x(int points) {
  md_stats_t_x *s = (md_stats_t_x *)calloc(1, sizeof(md_stats_t_x));
  if (!s) return NULL;
  s->N = 1;
  s->es = (md_num_t_x *)calloc(1, sizeof(md_num_t_x));
  s->Ts = (md_num_t_x *)calloc(1, sizeof(md_num_t_x));
  s->points = points;
  s->fx = (md_num_t_x *)calloc(points > 0 ? points : 1, sizeof(md_num_t_x));
  s->fxs = (md_num_t_x **)calloc(1, sizeof(md_num_t_x *));
  if (s->fxs) s->fxs[0] = (md_num_t_x *)calloc(points > 0 ? points : 1, sizeof(md_num_t_x));
  if (!s->es || !s->Ts || !s->fx || !s->fxs || !s->fxs[0]) {
    md_gb300_free_stats_x(s);
    return NULL;
  }
  return s;
}

void md_gb300_free_stats_x(md_stats_t_x *s) {
  if (!s) return;
  xmd::forget(s);
  if (s->fxs)
    for (int i = 0; i < s->N; ++i) free(s->fxs[i]);
  free(s->fxs);
  free(s->fx);
  free(s->es);
  free(s->Ts);
  free(s);
}

md_stats_t_x *md_update_stats_x(md_stats_t_x *s) {
  s->count++;
  if (s->count < MD_MAX_STATS_COUNT) return s;
  if (!(s = md_stats_sync_host_x(s))) return NULL;
  s->es[s->N - 1] /= MD_MAX_STATS_COUNT;
  s->Ts[s->N - 1] /= MD_MAX_STATS_COUNT;
  for (int i = 0; i < s->points; ++i) s->fxs[s->N - 1][i] /= MD_MAX_STATS_COUNT;
  s->N++;
  s->count = 0;
  md_num_t_x *es = (md_num_t_x *)realloc(s->es, sizeof(md_num_t_x) * s->N);
  md_num_t_x *Ts = (md_num_t_x *)realloc(s->Ts, sizeof(md_num_t_x) * s->N);
  md_num_t_x **fxs = (md_num_t_x **)realloc(s->fxs, sizeof(md_num_t_x *) * s->N);
  if (!es || !Ts || !fxs) return NULL;
  s->es = es;
  s->Ts = Ts;
  s->fxs = fxs;
  s->es[s->N - 1] = 0;
  s->Ts[s->N - 1] = 0;
  s->fxs[s->N - 1] = (md_num_t_x *)calloc(s->points > 0 ? s->points : 1, sizeof(md_num_t_x));
  return s->fxs[s->N - 1] ? s : NULL;
}

md_stats_t_x *md_finalize_stats_x(md_stats_t_x *s) {
  if (!(s = md_stats_sync_host_x(s))) return NULL;
  s->e = 0;
  s->T = 0;
  for (int i = 0; i < s->points; ++i) s->fx[i] = 0;
  if (s->count != 0) {
    s->es[s->N - 1] /= s->count;
    s->Ts[s->N - 1] /= s->count;
    for (int i = 0; i < s->points; ++i) s->fxs[s->N - 1][i] /= s->count;
  } else {
    s->N--;
  }
  for (int b = 0; b < s->N; ++b) {
    s->e += s->es[b];
    s->T += s->Ts[b];
    for (int i = 0; i < s->points; ++i) s->fx[i] += s->fxs[b][i];
  }
  s->e /= s->N;
  s->T /= s->N;
  for (int i = 0; i < s->points; ++i) s->fx[i] /= s->N;
  return s;
}

int md_reset_stats_x(md_stats_t_x *s, md_num_t_x e) {
  if (!(s = md_stats_sync_host_x(s))) return -1;
  s->es[0] = e;
  return 0;
}

int md_stats_add_to_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  s->es[s->N - 1] += s2->es[0];
  return 0;
}

int md_stats_copy_to_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  s->es[0] = s2->es[0];
  return 0;
}

int md_stats_mult_to_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  s->es[0] *= s2->es[0];
  return 0;
}

// the same four on the function-valued accumulator fxs (S(k) and other
// observables with `points` values): md_pimd_x.c:4566-4650.  add and copy
// need equal point counts; mult scales by the scalar es[0] of the second
int md_reset_stats_f_x(md_stats_t_x *s, md_num_t_x e) {
  if (!(s = md_stats_sync_host_x(s))) return -1;
  for (int i = 0; i < s->points; ++i) s->fxs[0][i] = e;
  return 0;
}

int md_stats_add_to_f_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!s || !s2 || s->points != s2->points) return -1;
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  for (int i = 0; i < s->points; ++i) s->fxs[s->N - 1][i] += s2->fxs[0][i];
  return 0;
}

int md_stats_copy_to_f_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!s || !s2 || s->points != s2->points) return -1;
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  for (int i = 0; i < s->points; ++i) s->fxs[0][i] = s2->fxs[0][i];
  return 0;
}

int md_stats_mult_to_f_x(md_stats_t_x *s, md_stats_t_x *s2) {
  if (!(s = md_stats_sync_host_x(s)) || !(s2 = md_stats_sync_host_x(s2))) return -1;
  for (int i = 0; i < s->points; ++i) s->fxs[0][i] *= s2->es[0];
  return 0;
}

}  // extern "C"
