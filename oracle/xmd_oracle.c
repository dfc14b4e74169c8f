/*
 * xmd_oracle.c -- CPU restatement of MD-Lab's _nocl PIMD step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  Only tests/, smoke() and the
 * CPU-baseline leg of bench.py use it; the CUDA product never links it.
 *
 * Each function restates the reference's single-threaded branch (the #else
 * of MD_USE_OPENCL_X) in plain C with the same loop order and the same
 * floating-point expressions, so that its results agree with the reference
 * build to rounding.  It is compiled with -ffp-contract=off so that x86 and
 * aarch64 hosts produce the same bits.  Citations are file:line inside the
 * MD-Lab source tree.
 */
#include "xmd_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.141592653589793
#endif

#define ORC_KB 1.0     /* MD_kB_X, md_particle_x.h:5 */
#define ORC_HBAR 1.0   /* MD_hBar_X, md_particle_x.h:6 */

/* bead index of particle l (1-based), bead j (1-based): md_pimd_x.h:10 */
static inline int bidx(int l, int j, int P) { return (l - 1) * P + j - 1; }
/* row start of the ENk triangle for particle count n (1-based) */
static inline int tri(int n) { return n * (n - 1) / 2; }

/* md_simulation_x.c:858-865 */
int orc_periodic_image_count(double x, double L) {
  int c = (int)(fabs(x) / L);
  if (x > L) return -c;
  if (x < 0) return c + 1;
  return 0;
}

/* md_simulation_x.c:70-81: shift into [0,L) around +L/2 and back */
double orc_minimum_image(double a, double L) {
  a += L / 2;
  a += L * orc_periodic_image_count(a, L);
  return a - L / 2;
}

static double dist(int D, const double *a, const double *b) {
  double s = 0;
  for (int i = 0; i < D; ++i) {
    double t = a[i] - b[i];
    s += t * t;
  }
  return sqrt(s);
}

static double mi_dist(int D, const double *a, const double *b, const double *L) {
  double s = 0;
  for (int i = 0; i < D; ++i) {
    double t = orc_minimum_image(a[i] - b[i], L[i]);
    s += t * t;
  }
  return sqrt(s);
}

static double spring_d(const orc_sim_t *s, int b1, int b2, int image) {
  const double *p1 = s->x + (size_t)b1 * s->D, *p2 = s->x + (size_t)b2 * s->D;
  return image ? mi_dist(s->D, p1, p2, s->box) : dist(s->D, p1, p2);
}

/* ------------------------------------------------------------------ */
/* integrator                                                           */
/* ------------------------------------------------------------------ */

/* md_simulation_x.c:421-472 (CPU branch :465-470) */
void orc_reset_force(orc_sim_t *s) {
  memset(s->f, 0, sizeof(double) * (size_t)s->nb * s->D);
}

/* md_simulation_x.c:599-613: thermostat forces of chain i over its DOFs */
static void chain_force(const orc_sim_t *s, int f0, int f2, int i, double *res) {
  const int L = s->L;
  double sum = 0;
  for (int j = 0; j < f2; ++j) {
    int dof = f0 + j;
    int b = dof / s->D;
    sum += s->m[b] * s->v[dof] * s->v[dof];
  }
  res[0] = (sum - s->cf[i] * ORC_KB * s->T) / s->Q[i * L];
  for (int j = 1; j < L; ++j)
    res[j] = (s->Q[i * L + j - 1] * s->vtheta[i * L + j - 1] * s->vtheta[i * L + j - 1] -
              ORC_KB * s->T) / s->Q[i * L + j];
}

/* kick of one chain's DOFs by the thermostat: md_simulation_x.c:674-678 */
static void chain_kick(orc_sim_t *s, int f0, int f2, double h, double vt0) {
  for (int j = 0; j < f2; ++j) {
    int dof = f0 + j;
    s->v[dof] = s->v[dof] * exp(-0.5 * h * vt0) + 0.5 * h * s->f[dof] * exp(-0.25 * h * vt0);
  }
}

/* odd chain members: md_simulation_x.c:682-683 */
static void chain_odd_v(orc_sim_t *s, int i, double h, const double *nhf) {
  const int L = s->L, M2 = L / 2;
  double *vt = s->vtheta + (size_t)i * L;
  for (int j = 1; j <= M2; ++j) {
    double nxt = (j == M2) ? 0 : vt[2 * j];
    vt[2 * j - 1] = vt[2 * j - 1] * exp(-0.5 * h * nxt) + 0.5 * h * nhf[2 * j - 1] * exp(-0.25 * h * nxt);
  }
}

/* md_simulation_x.c:615-708 (CPU branch :660-706) */
int orc_nhc_vv3_1(orc_sim_t *s, double h) {
  const int L = s->L, M2 = L / 2;
  double nhf[64];
  if (L > 64 || (L & 1)) return -1;
  int f0 = 0;
  for (int i = 0; i < s->nf; ++i) {
    int f = s->cf[i];
    int f2 = (i == s->nf - 1) ? s->D * s->nb - f0 : f;
    double *th = s->theta + (size_t)i * L, *vt = s->vtheta + (size_t)i * L;
    chain_force(s, f0, f2, i, nhf);
    chain_kick(s, f0, f2, h, vt[0]);
    for (int j = 1; j <= M2; ++j) th[2 * j - 2] = th[2 * j - 2] + h * vt[2 * j - 2] / 2;
    chain_odd_v(s, i, h, nhf);
    for (int j = 0; j < f2; ++j) s->x[f0 + j] = s->x[f0 + j] + h * s->v[f0 + j];
    for (int j = 1; j <= M2; ++j) th[2 * j - 1] = th[2 * j - 1] + h * vt[2 * j - 1];
    chain_force(s, f0, f2, i, nhf);
    for (int j = 1; j <= M2; ++j)
      vt[2 * j - 2] = vt[2 * j - 2] * exp(-h * vt[2 * j - 1]) + h * nhf[2 * j - 2] * exp(-0.5 * h * vt[2 * j - 1]);
    f0 += f;
  }
  return 0;
}

/* md_simulation_x.c:710-792 (CPU branch :757-790) */
int orc_nhc_vv3_2(orc_sim_t *s, double h) {
  const int L = s->L, M2 = L / 2;
  double nhf[64];
  if (L > 64 || (L & 1)) return -1;
  int f0 = 0;
  for (int i = 0; i < s->nf; ++i) {
    int f = s->cf[i];
    int f2 = (i == s->nf - 1) ? s->D * s->nb - f0 : f;
    double *th = s->theta + (size_t)i * L, *vt = s->vtheta + (size_t)i * L;
    chain_kick(s, f0, f2, h, vt[0]);
    for (int j = 1; j <= M2; ++j) th[2 * j - 2] = th[2 * j - 2] + h * vt[2 * j - 2] / 2;
    chain_force(s, f0, f2, i, nhf);
    chain_odd_v(s, i, h, nhf);
    f0 += f;
  }
  return 0;
}

/* md_simulation_x.c:794-856 (CPU branch :846-853) */
void orc_periodic_boundary(orc_sim_t *s) {
  for (int b = 0; b < s->nb; ++b)
    for (int d = 0; d < s->D; ++d) {
      double *x = &s->x[(size_t)b * s->D + d];
      if (*x < 0)
        *x += s->box[d];
      else if (*x > s->box[d])
        *x -= s->box[d];
    }
}

/* ------------------------------------------------------------------ */
/* exchange                                                             */
/* ------------------------------------------------------------------ */

/* next / previous bead on the cycle closing particles N2-k+1..N2:
   md_pimd_x.c:521-549 */
static int next_bead(int l, int j, int N2, int k, int P) {
  if (j == P) return (l == N2) ? bidx(N2 - k + 1, 1, P) : bidx(l + 1, 1, P);
  return bidx(l, j + 1, P);
}
static int prev_bead(int l, int j, int N2, int k, int P) {
  if (j == 1) return (l == N2 - k + 1) ? bidx(N2, P, P) : bidx(l - 1, P, P);
  return bidx(l, j - 1, P);
}

/* md_pimd_x.c:569-591 and :593-665 (CPU branch :658-663) */
int orc_fill_ENk_cubic(const orc_sim_t *s, int N, int P, double omegaP, int image, double *ENk) {
  for (int N2 = 1; N2 <= N; ++N2)
    for (int k = 1; k <= N2; ++k) {
      double res = 0;
      for (int l = N2 - k + 1; l <= N2; ++l)
        for (int j = 1; j <= P; ++j) {
          int b = bidx(l, j, P), b2 = next_bead(l, j, N2, k, P);
          double d = spring_d(s, b, b2, image);
          res += 0.5 * s->m[b] * omegaP * omegaP * d * d;
        }
      ENk[tri(N2) + k - 1] = res;
    }
  return 0;
}

/* md_pimd_x.c:1969-2210 (CPU branch :2086-2207), default path: no worm,
   no cut bead, no winding bookkeeping */
int orc_fast_fill_ENk(const orc_sim_t *s, int N, int P, double omegaP, int image, double *ENk,
                      double *Eint) {
  const double w2 = omegaP * omegaP;
  for (int l = 1; l <= N; ++l) {
    double res = 0;
    for (int j = 1; j < P; ++j) {
      int b = bidx(l, j, P), b2 = bidx(l, j + 1, P);
      double d = spring_d(s, b, b2, image);
      res += 0.5 * s->m[b] * w2 * d * d;
    }
    Eint[l - 1] = res;
    int b = bidx(l, P, P), b2 = bidx(l, 1, P);
    double d = spring_d(s, b, b2, image);
    ENk[tri(l)] = res + 0.5 * s->m[b] * w2 * d * d;
  }
  for (int l = 1; l <= N; ++l)
    for (int k = 2; k <= l; ++k) {
      double e = ENk[tri(l) + k - 2] + Eint[l - k];
      /* drop the spring P(l) -> 1(l-k+2) that closed the shorter cycle */
      int b = bidx(l, P, P), b2 = bidx(l - k + 2, 1, P);
      double d = spring_d(s, b, b2, image);
      e -= 0.5 * s->m[b] * w2 * d * d;
      /* link P(l-k+1) -> 1(l-k+2) */
      b = bidx(l - k + 1, P, P);
      b2 = bidx(l - k + 2, 1, P);
      d = spring_d(s, b, b2, image);
      e += 0.5 * s->m[b] * w2 * d * d;
      /* close the new cycle P(l) -> 1(l-k+1) */
      b = bidx(l, P, P);
      b2 = bidx(l - k + 1, 1, P);
      d = spring_d(s, b, b2, image);
      e += 0.5 * s->m[b] * w2 * d * d;
      ENk[tri(l) + k - 1] = e;
    }
  return 0;
}

/* md_pimd_x.c:681-686 */
static double xexp(double k, double E, double EE, double beta, double vi) {
  if (vi == 0.0) return exp(-beta * E + EE);
  return exp((k - 1) * log(vi) - beta * E + EE);
}

/* md_pimd_x.c:688-808 (CPU branch :796-806) */
static double xminE(int N2, double beta, double vi, const double *ENk, const double *VBN) {
  if (vi == 0.0) return beta * (ENk[tri(N2)] + VBN[N2 - 1]);
  double res = 1e10;
  for (int k = 1; k <= N2; ++k) {
    double t = -(k - 1) * log(vi) + beta * (ENk[tri(N2) + k - 1] + VBN[N2 - k]);
    if (t < res) res = t;
  }
  return res;
}

/* md_pimd_x.c:814-953 (CPU branch :934-950), no worm */
int orc_fill_VB(int N, double beta, double vi, const double *ENk, double *VBN) {
  VBN[0] = 0.0;
  for (int N2 = 1; N2 <= N; ++N2) {
    double sum = 0;
    double m = xminE(N2, beta, vi, ENk, VBN);
    for (int k = 1; k <= N2; ++k) {
      if (vi == 0 && k - 1 != 0) continue;
      sum += xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
    }
    VBN[N2] = (m - log(sum) + log(N2)) / beta;
  }
  return 0;
}

/* md_pimd_x.c:2213-2335 (CPU branch :2321-2333) */
static double fast_xminE(int N, int u, double beta, double vi, const double *ENk, const double *V) {
  if (vi == 0.0) return log(u) + beta * (ENk[tri(u)] + V[u]);
  double res = 1e10;
  for (int l = u; l <= N; ++l) {
    int k = l - u + 1;
    double t = -(k - 1) * log(vi) + log(l) + beta * (ENk[tri(l) + k - 1] + V[l]);
    if (t < res) res = t;
  }
  return res;
}

/* md_pimd_x.c:2337-2342 */
static double fast_xexp(double l, double k, double E, double EE, double beta, double vi) {
  if (vi == 0.0) return exp(-beta * E + EE - log(l));
  return exp((k - 1) * log(vi) - beta * E + EE - log(l));
}

/* md_pimd_x.c:2344-2367: gradient of the two springs at bead b */
static void spring_grad(const orc_sim_t *s, double w2, int b, int bn, int bp, int image, double *g) {
  const int D = s->D;
  for (int i = 0; i < D; ++i) {
    double a = s->x[(size_t)b * D + i] - s->x[(size_t)bn * D + i];
    double c = s->x[(size_t)b * D + i] - s->x[(size_t)bp * D + i];
    if (image) {
      a = orc_minimum_image(a, s->box[i]);
      c = orc_minimum_image(c, s->box[i]);
    }
    g[i] = 0;
    g[i] += s->m[b] * w2 * a;
    g[i] += s->m[b] * w2 * c;
  }
}

/* md_pimd_x.c:2369-2721 (CPU branch :2648-2719) */
int orc_fast_force_VB(orc_sim_t *s, int N, int P, double beta, double vi, double omegaP,
                      int image, const double *ENk, const double *VBN, double *G_out,
                      double *tmpV_out) {
  const int D = s->D;
  const double w2 = omegaP * omegaP;
  double *tmpV = (double *)malloc(sizeof(double) * (N + 1));
  double *G = (double *)malloc(sizeof(double) * (size_t)N * N);
  if (!tmpV || !G) {
    free(tmpV);
    free(G);
    return -1;
  }
  tmpV[N] = 0;
  for (int u = N; u >= 1; --u) {
    double sum = 0;
    double m = fast_xminE(N, u, beta, vi, ENk, tmpV);
    for (int l = u; l <= N; ++l) {
      int k = l - u + 1;
      if (vi == 0 && k - 1 != 0) continue;
      sum += fast_xexp(l, k, ENk[tri(l) + k - 1] + tmpV[l], m, beta, vi);
    }
    tmpV[u - 1] = (m - log(sum)) / beta;
  }
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= N; ++j) {
      double g;
      if (j > l + 1)
        g = 0;
      else if (j == l + 1)
        g = 1 - exp(-beta * (VBN[l] + tmpV[l] - VBN[N]));
      else if (vi == 0 && l - j != 0)
        g = 0;
      else if (vi == 0)
        g = exp(-beta * (VBN[j - 1] + ENk[tri(l) + l - j] + tmpV[l] - VBN[N])) / l;
      else
        g = exp(-beta * (VBN[j - 1] + ENk[tri(l) + l - j] + tmpV[l] - VBN[N]) + (l - j) * log(vi)) / l;
      G[(size_t)(l - 1) * N + (j - 1)] = g;
    }
  double grad[8];
  /* interior beads */
  for (int l = 1; l <= N; ++l)
    for (int j = 2; j < P; ++j) {
      int b = bidx(l, j, P);
      spring_grad(s, w2, b, bidx(l, j + 1, P), bidx(l, j - 1, P), image, grad);
      for (int i = 0; i < D; ++i) s->f[(size_t)b * D + i] += -grad[i] / s->m[b];
    }
  /* bead 1 of l, preceded by bead P of j with weight G[j][l] */
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= N; ++j) {
      int b = bidx(l, 1, P);
      spring_grad(s, w2, b, bidx(l, 2, P), bidx(j, P, P), image, grad);
      for (int i = 0; i < D; ++i)
        s->f[(size_t)b * D + i] += -G[(size_t)(j - 1) * N + (l - 1)] * grad[i] / s->m[b];
    }
  /* bead P of l, followed by bead 1 of j with weight G[l][j] */
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= N; ++j) {
      int b = bidx(l, P, P);
      spring_grad(s, w2, b, bidx(l, P - 1, P), bidx(j, 1, P), image, grad);
      for (int i = 0; i < D; ++i)
        s->f[(size_t)b * D + i] += -G[(size_t)(l - 1) * N + (j - 1)] * grad[i] / s->m[b];
    }
  if (G_out) memcpy(G_out, G, sizeof(double) * (size_t)N * N);
  if (tmpV_out) memcpy(tmpV_out, tmpV, sizeof(double) * (N + 1));
  free(tmpV);
  free(G);
  return 0;
}

/* cubic derivative recursion, md_pimd_x.c:967-995 and :997-1109 (CPU
   branch :1070-1106); used only to cross-check the quadratic path */
int orc_force_VB_cubic(orc_sim_t *s, int N, int P, double beta, double vi, double omegaP,
                       int image, const double *ENk, const double *VBN) {
  const int D = s->D;
  const double w2 = omegaP * omegaP;
  double *res = (double *)malloc(sizeof(double) * D * (N + 1));
  double *grad = (double *)malloc(sizeof(double) * D * N);
  if (!res || !grad) {
    free(res);
    free(grad);
    return -1;
  }
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= P; ++j) {
      for (int i = 0; i < D; ++i) res[i] = 0;
      for (int N2 = 1; N2 <= N; ++N2) {
        double sum2 = 0;
        double m = xminE(N2, beta, vi, ENk, VBN);
        for (int k = 1; k <= N2; ++k) {
          if (vi == 0 && k - 1 != 0) continue;
          sum2 += xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
        }
        for (int k = 1; k <= N2; ++k) {
          double *g = &grad[D * (k - 1)];
          if (!(l >= N2 - k + 1 && l <= N2)) {
            for (int i = 0; i < D; ++i) g[i] = 0;
            continue;
          }
          int b = bidx(l, j, P);
          spring_grad(s, w2, b, next_bead(l, j, N2, k, P), prev_bead(l, j, N2, k, P), image, g);
        }
        for (int i = 0; i < D; ++i) {
          double sum = 0;
          for (int k = 1; k <= N2; ++k) {
            if (vi == 0 && k - 1 != 0) continue;
            sum += (grad[D * (k - 1) + i] + res[D * (N2 - k) + i]) *
                   xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
          }
          res[D * N2 + i] = sum / sum2;
        }
      }
      int b = bidx(l, j, P);
      for (int i = 0; i < D; ++i) s->f[(size_t)b * D + i] += -res[D * N + i] / s->m[b];
    }
  free(res);
  free(grad);
  return 0;
}

/* ------------------------------------------------------------------ */
/* external potentials                                                  */
/* ------------------------------------------------------------------ */

/* md_simulation_x.c:127-131, :133-137, :155-159 (m is ignored, as there) */
static void trap_force_one(int kind, const orc_params_t *p, int D, const double *x, double *f) {
  for (int i = 0; i < D; ++i) {
    if (kind == ORC_TRAP_HARMONIC)
      f[i] += -p->trap_w * p->trap_w * (x[i] - p->trap_c[i]);
    else if (kind == ORC_TRAP_NEG_HARMONIC)
      f[i] -= -p->trap_w * p->trap_w * (x[i] - p->trap_c[i]);
    else
      f[i] += -p->trap_w2[i] * p->trap_w2[i] * (x[i] - p->trap_c[i]);
  }
}

/* md_pimd_x.c:1297-1391 (CPU branch :1370-1389) */
int orc_trap_force(orc_sim_t *s, int N, int P, int kind, const orc_params_t *p) {
  const int D = s->D;
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= P; ++j) {
      int b = bidx(l, j, P);
      double f[8] = {0};
      trap_force_one(kind, p, D, s->x + (size_t)b * D, f);
      for (int i = 0; i < D; ++i) s->f[(size_t)b * D + i] += f[i] / P;
    }
  return 0;
}

/* md_simulation_x.c:259-293 */
static void ewald_force_one(const orc_params_t *p, const double *p1, const double *p2, double *f,
                            const double *L, double m) {
  const double V = L[0] * L[1] * L[2];
  const double a = p->coul_alpha, sc = p->coul_s;
  const int n = p->coul_nsum;
  const double origin[3] = {0, 0, 0};
  double g[3], r[3];
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (i == 0 && j == 0 && k == 0) continue;
        g[0] = i / L[0];
        g[1] = j / L[1];
        g[2] = k / L[2];
        double G = dist(3, g, origin);
        double dot = 2 * M_PI * (g[0] * (p1[0] - p2[0]) + g[1] * (p1[1] - p2[1]) + g[2] * (p1[2] - p2[2]));
        double mult = sc * sin(dot) * pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (V * M_PI);
        for (int d = 0; d < 3; ++d) f[d] += 2 * M_PI * g[d] * mult / m;
      }
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        r[0] = p2[0] + i * L[0];
        r[1] = p2[1] + j * L[1];
        r[2] = p2[2] + k * L[2];
        double R = dist(3, p1, r);
        double mult = sc * 2 * a * exp(-a * a * R * R) / (sqrt(M_PI) * R * R);
        mult += sc * erfc(a * R) / (R * R * R);
        for (int d = 0; d < 3; ++d) f[d] += (p1[d] - r[d]) * mult / m;
      }
}

/* one pair force, as the reference's pair-force callbacks
   (md_simulation_x.c:166-172, :174-180, :188-194, :196-202, :259-293) */
void orc_pair_force_one(int kind, const orc_params_t *p, int D, const double *p1,
                        const double *p2, double *f, const double *L, double m) {
  if (kind == ORC_PAIR_GAUSSIAN || kind == ORC_PAIR_PERIODIC_GAUSSIAN) {
    const double s = p->gauss_s;
    double d = (kind == ORC_PAIR_GAUSSIAN) ? dist(D, p1, p2) : mi_dist(D, p1, p2, L);
    double mult = (p->gauss_g / (M_PI * s * s)) * exp(-d * d / (s * s));
    for (int i = 0; i < D; ++i) {
      double dx = p1[i] - p2[i];
      if (kind == ORC_PAIR_PERIODIC_GAUSSIAN) dx = orc_minimum_image(dx, L[i]);
      f[i] += mult * (2 * dx) / (s * s) / m;
    }
  } else if (kind == ORC_PAIR_COULOMB || kind == ORC_PAIR_PERIODIC_COULOMB) {
    double d = (kind == ORC_PAIR_COULOMB) ? dist(D, p1, p2) : mi_dist(D, p1, p2, L);
    double mult = p->coul_s / pow(d, 3);
    for (int i = 0; i < D; ++i) {
      double dx = p1[i] - p2[i];
      if (kind == ORC_PAIR_PERIODIC_COULOMB) dx = orc_minimum_image(dx, L[i]);
      f[i] += mult * dx / m;
    }
  } else if (kind == ORC_PAIR_EWALD) {
    if (D == 3) ewald_force_one(p, p1, p2, f, L, m);
  }
}

/* md_pimd_x.c:1527-1677 (CPU branch :1650-1675): per bead slice, pairs
   l2 < l, the force divided by m of particle l, Newton's third law */
int orc_pair_force(orc_sim_t *s, int N, int P, int kind, const orc_params_t *p) {
  const int D = s->D;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= N; ++l)
      for (int l2 = 1; l2 < l; ++l2) {
        int b = bidx(l, j, P), b2 = bidx(l2, j, P);
        double f[8] = {0};
        orc_pair_force_one(kind, p, D, s->x + (size_t)b * D, s->x + (size_t)b2 * D, f, s->box, s->m[b]);
        for (int i = 0; i < D; ++i) {
          s->f[(size_t)b * D + i] += f[i] / P;
          s->f[(size_t)b2 * D + i] -= f[i] / P;
        }
      }
  return 0;
}

/* two species, md_pimd_x.c:3444-3467 (the CPU branch of
   md_pimd_calc_pair_force_2_x): in every bead slice each bead of species a
   meets each bead of species b once; the callback gets a's mass and a's box,
   f_a += F/P and f_b -= m_a F/(P m_b) */
int orc_pair_force_2(orc_sim_t *a, int Na, orc_sim_t *b, int Nb, int P, int kind, const orc_params_t *p) {
  const int D = a->D;
  if (b->D != D) return -1;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= Na; ++l)
      for (int l2 = 1; l2 <= Nb; ++l2) {
        int ia = bidx(l, j, P), ib = bidx(l2, j, P);
        double f[8] = {0};
        orc_pair_force_one(kind, p, D, a->x + (size_t)ia * D, b->x + (size_t)ib * D, f, a->box, a->m[ia]);
        for (int i = 0; i < D; ++i) {
          a->f[(size_t)ia * D + i] += f[i] / P;
          b->f[(size_t)ib * D + i] -= a->m[ia] * f[i] / P / b->m[ib];
        }
      }
  return 0;
}

/* ------------------------------------------------------------------ */
/* estimators                                                           */
/* ------------------------------------------------------------------ */

/* primitive exchange estimator: md_pimd_x.c:1111-1295 (CPU :1267-1293) */
double orc_vbn_energy(int D, int N, int P, double beta, double vi, const double *ENk,
                      const double *VBN) {
  double *res = (double *)malloc(sizeof(double) * (N + 1));
  if (!res) return NAN;
  res[0] = 0;
  for (int N2 = 1; N2 <= N; ++N2) {
    double sum2 = 0, sum = 0;
    double m = xminE(N2, beta, vi, ENk, VBN);
    for (int k = 1; k <= N2; ++k) {
      if (vi == 0 && k - 1 != 0) continue;
      sum2 += xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
    }
    for (int k = 1; k <= N2; ++k) {
      if (vi == 0 && k - 1 != 0) continue;
      sum += (res[N2 - k] - ENk[tri(N2) + k - 1]) * xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
    }
    res[N2] = sum / sum2;
  }
  double e = 0;
  e += res[N];
  e += D * N * P / (2 * beta);
  free(res);
  return e;
}

/* md_pimd_x.c:4376-4421 (default path: no winding bookkeeping) */
static double enk2_term(const orc_sim_t *s, double w2, int b, int b2, int b3, int image) {
  const int D = s->D;
  double res = 0;
  for (int i = 0; i < D; ++i) {
    double d = s->x[(size_t)b * D + i] - s->x[(size_t)b2 * D + i];
    double d2 = s->x[(size_t)b * D + i] - s->x[(size_t)b3 * D + i];
    if (image) {
      d = orc_minimum_image(d, s->box[i]);
      d2 = orc_minimum_image(d2, s->box[i]);
    }
    res += 0.5 * s->m[b] * w2 * d * d2;
  }
  return res;
}

/* md_pimd_x.c:4423-4556 (CPU branch :4521-4553) */
int orc_fast_fill_ENk2(const orc_sim_t *s, int N, int P, double omegaP, int image, double *ENk2) {
  const double w2 = omegaP * omegaP;
  for (int l = 1; l <= N; ++l)
    ENk2[tri(l)] = enk2_term(s, w2, bidx(l, 1, P), bidx(l, P, P), bidx(l, 1, P), image);
  for (int l = 1; l <= N; ++l)
    for (int k = 2; k <= l; ++k) {
      double e = ENk2[tri(l) + k - 2] -
                 enk2_term(s, w2, bidx(l, 1, P), bidx(l - k + 2, P, P), bidx(l - k + 2, 1, P), image);
      e += enk2_term(s, w2, bidx(l - k + 1, 1, P), bidx(l - k + 2, P, P), bidx(l - k + 2, 1, P), image);
      e += enk2_term(s, w2, bidx(l, 1, P), bidx(l - k + 1, P, P), bidx(l - k + 1, 1, P), image);
      ENk2[tri(l) + k - 1] = e;
    }
  return 0;
}

/* md_pimd_x.c:3959-3987 and :3989-4056 (CPU branch :4049-4054) */
int orc_fill_ENk2_cubic(const orc_sim_t *s, int N, int P, double omegaP, int image, double *ENk2) {
  const double w2 = omegaP * omegaP;
  for (int N2 = 1; N2 <= N; ++N2)
    for (int k = 1; k <= N2; ++k) {
      double res = 0;
      for (int l = N2 - k + 1; l <= N2; ++l) {
        int b = next_bead(l, P, N2, k, P);
        int b2 = bidx(l, P, P), b3 = bidx(l, 1, P);
        const int D = s->D;
        for (int i = 0; i < D; ++i) {
          double d = s->x[(size_t)b * D + i] - s->x[(size_t)b2 * D + i];
          double d2 = s->x[(size_t)b * D + i] - s->x[(size_t)b3 * D + i];
          if (image) {
            d = orc_minimum_image(d, s->box[i]);
            d2 = orc_minimum_image(d2, s->box[i]);
          }
          res += 0.5 * s->m[b] * w2 * d * d2;
        }
      }
      ENk2[tri(N2) + k - 1] = res;
    }
  return 0;
}

/* virial exchange estimator: md_pimd_x.c:4072-4348 (CPU :4288-4346),
   default path (no winding bookkeeping) */
double orc_vi_virial_energy(const orc_sim_t *s, int N, int P, double beta, double vi, int image,
                            const double *ENk, const double *ENk2, const double *VBN) {
  const int D = s->D;
  double *res = (double *)malloc(sizeof(double) * (N + 1));
  if (!res) return NAN;
  res[0] = 0;
  for (int N2 = 1; N2 <= N; ++N2) {
    double sum2 = 0, sum = 0;
    double m = xminE(N2, beta, vi, ENk, VBN);
    for (int k = 1; k <= N2; ++k) {
      if (vi == 0 && k - 1 != 0) continue;
      sum2 += xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
    }
    for (int k = 1; k <= N2; ++k) {
      if (vi == 0 && k - 1 != 0) continue;
      sum += (res[N2 - k] - ENk2[tri(N2) + k - 1]) * xexp(k, ENk[tri(N2) + k - 1] + VBN[N2 - k], m, beta, vi);
    }
    res[N2] = sum / sum2;
  }
  double e = 0;
  e += res[N];
  e += D * N / (2 * beta);
  free(res);
  double res2 = 0;
  for (int j = 2; j <= P; ++j)
    for (int l = 1; l <= N; ++l) {
      int b = bidx(l, j, P), b2 = bidx(l, 1, P);
      for (int i = 0; i < D; ++i) {
        double dx = s->x[(size_t)b * D + i] - s->x[(size_t)b2 * D + i];
        if (image) dx = orc_minimum_image(dx, s->box[i]);
        res2 += -dx * s->f[(size_t)b * D + i] * s->m[b];
      }
    }
  e += res2 / 2.0;
  return e;
}

/* md_statistics_x.c:322-325 (harmonic), :327-330 (negative), :332-338 */
static double trap_energy_one(int kind, const orc_params_t *p, int D, const double *x, double m) {
  if (kind == ORC_TRAP_HARMONIC || kind == ORC_TRAP_NEG_HARMONIC) {
    double d = dist(D, x, p->trap_c);
    double e = 0.5 * m * p->trap_w * p->trap_w * d * d;
    return kind == ORC_TRAP_HARMONIC ? e : -e;
  }
  double r = 0;
  for (int i = 0; i < D; ++i)
    r += 0.5 * m * p->trap_w2[i] * p->trap_w2[i] * (x[i] - p->trap_c[i]) * (x[i] - p->trap_c[i]);
  return r;
}

/* md_pimd_x.c:1393-1525 (CPU branch :1510-1523) */
double orc_trap_energy(const orc_sim_t *s, int N, int P, int kind, const orc_params_t *p) {
  double e = 0;
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= P; ++j) {
      int b = bidx(l, j, P);
      e += trap_energy_one(kind, p, s->D, s->x + (size_t)b * s->D, s->m[b]) / P;
    }
  return e;
}

/* md_statistics_x.c:364-396 */
static double ewald_energy_one(const orc_params_t *p, const double *p1, const double *p2,
                               const double *L) {
  const double V = L[0] * L[1] * L[2];
  const double a = p->coul_alpha;
  const int n = p->coul_nsum;
  const double origin[3] = {0, 0, 0};
  double g[3], r[3], res = 0;
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (i == 0 && j == 0 && k == 0) continue;
        g[0] = i / L[0];
        g[1] = j / L[1];
        g[2] = k / L[2];
        double G = dist(3, g, origin);
        double dot = 2 * M_PI * (g[0] * (p1[0] - p2[0]) + g[1] * (p1[1] - p2[1]) + g[2] * (p1[2] - p2[2]));
        res += cos(dot) * pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (V * M_PI);
      }
  res -= M_PI / (a * a * V);
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        r[0] = p2[0] + i * L[0];
        r[1] = p2[1] + j * L[1];
        r[2] = p2[2] + k * L[2];
        double R = dist(3, p1, r);
        res += erfc(a * R) / R;
      }
  return p->coul_s * res;
}

/* md_statistics_x.c:340-362, :364-396 */
double orc_pair_energy_one(int kind, const orc_params_t *p, int D, const double *p1,
                           const double *p2, const double *L) {
  if (kind == ORC_PAIR_GAUSSIAN || kind == ORC_PAIR_PERIODIC_GAUSSIAN) {
    const double s = p->gauss_s;
    double d = (kind == ORC_PAIR_GAUSSIAN) ? dist(D, p1, p2) : mi_dist(D, p1, p2, L);
    return (p->gauss_g / (M_PI * s * s)) * exp(-d * d / (s * s));
  }
  if (kind == ORC_PAIR_COULOMB) return p->coul_s / dist(D, p1, p2);
  if (kind == ORC_PAIR_PERIODIC_COULOMB) return p->coul_s / mi_dist(D, p1, p2, L);
  if (kind == ORC_PAIR_EWALD) return D == 3 ? ewald_energy_one(p, p1, p2, L) : 0;
  return 0;
}

/* md_pimd_x.c:1679-1824 (CPU branch :1805-1822) */
double orc_pair_energy(const orc_sim_t *s, int N, int P, int kind, const orc_params_t *p) {
  double e = 0;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= N; ++l)
      for (int l2 = 1; l2 < l; ++l2) {
        int b = bidx(l, j, P), b2 = bidx(l2, j, P);
        e += orc_pair_energy_one(kind, p, s->D, s->x + (size_t)b * s->D, s->x + (size_t)b2 * s->D, s->box) / P;
      }
  return e;
}

/* two species, md_pimd_x.c:3606-3627 (the CPU branch of
   md_pimd_calc_pair_energy_2_x): sum over slices and all (a, b) pairs of
   V/P with a's box */
double orc_pair_energy_2(const orc_sim_t *a, int Na, const orc_sim_t *b, int Nb, int P, int kind,
                         const orc_params_t *p) {
  double e = 0;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= Na; ++l)
      for (int l2 = 1; l2 <= Nb; ++l2) {
        int ia = bidx(l, j, P), ib = bidx(l2, j, P);
        e += orc_pair_energy_one(kind, p, a->D, a->x + (size_t)ia * a->D, b->x + (size_t)ib * b->D, a->box) / P;
      }
  return e;
}

/* md_simulation_x.c:223-257 */
/* md_pimd_x.c:3898-3922: -(1/2) sum over beads of (x - L/2) . f m, f the
   stored accelerations, L the box */
double orc_virial_energy(const orc_sim_t *s, int N, int P) {
  double res = 0;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= N; ++l) {
      const int b = bidx(l, j, P);
      for (int i = 0; i < s->D; ++i)
        res += -(s->x[(size_t)b * s->D + i] - s->box[i] / 2) * s->f[(size_t)b * s->D + i] * s->m[b];
    }
  return res / 2.0;
}

/* md_pimd_x.c:3923-3955: the same about each particle's centroid, plus
   (D N - fc/P) / (2 beta) */
double orc_centroid_virial_energy(const orc_sim_t *s, int N, int P, double beta, int fc) {
  const int D = s->D;
  double *c = (double *)malloc(sizeof(double) * D * N);
  if (!c) return NAN;
  for (int l = 1; l <= N; ++l) {
    for (int i = 0; i < D; ++i) c[D * (l - 1) + i] = 0;
    for (int j = 1; j <= P; ++j)
      for (int i = 0; i < D; ++i) c[D * (l - 1) + i] += s->x[(size_t)bidx(l, j, P) * D + i] / P;
  }
  double res = 0;
  for (int j = 1; j <= P; ++j)
    for (int l = 1; l <= N; ++l) {
      const int b = bidx(l, j, P);
      for (int i = 0; i < D; ++i)
        res += -(s->x[(size_t)b * D + i] - c[D * (l - 1) + i]) * s->f[(size_t)b * D + i] * s->m[b];
    }
  free(c);
  return res / 2.0 + (D * N - fc / (double)P) / (2 * beta);
}

/* md_pimd_x.c:4350-4374: each ring polymer shifted by the image count of
   its first bead */
void orc_polymer_periodic_boundary(orc_sim_t *s, int N, int P) {
  const int D = s->D;
  int cnt[3];
  for (int l = 1; l <= N; ++l) {
    const int b1 = bidx(l, 1, P);
    for (int i = 0; i < D; ++i) cnt[i] = orc_periodic_image_count(s->x[(size_t)b1 * D + i], s->box[i]);
    for (int j = 1; j <= P; ++j)
      for (int i = 0; i < D; ++i) s->x[(size_t)bidx(l, j, P) * D + i] += cnt[i] * s->box[i];
  }
}

/* md_pimd_x.c:2974, CPU branch :3081-3108 (md_pimd_calc_pair_correlation_x):
   distances from bead 1 of l to bead pi of every other particle, minimum
   image when `image`, histogram of `points` bins over [0, rmax), each count
   adding 1/norm to out (distances at rmax and beyond are dropped) */
void orc_pair_correlation(const orc_sim_t *s, int N, int P, int points, double rmax, double norm, int pi,
                          int image, double *out) {
  const int D = s->D;
  const double incre = rmax / points;
  for (int l = 1; l <= N; ++l)
    for (int j = 1; j <= N; ++j) {
      if (l == j) continue;
      const double *p1 = &s->x[(size_t)bidx(l, 1, P) * D];
      const double *p2 = &s->x[(size_t)bidx(j, pi, P) * D];
      double r;
      if (image) {
        double d = 0;
        for (int i = 0; i < D; ++i) {
          const double t = orc_minimum_image(p1[i] - p2[i], s->box[i]);
          d += t * t;
        }
        r = sqrt(d);
      } else {
        r = dist(D, p1, p2);
      }
      const int k = (int)(r / incre);
      if (k >= points) continue;
      out[k] += 1.0 / norm;
    }
}

double orc_madelung(const double *L, const orc_params_t *p) {
  const double V = L[0] * L[1] * L[2];
  const double a = p->coul_alpha;
  const int n = p->coul_nsum;
  const double origin[3] = {0, 0, 0};
  double g[3], r[3], res = 0;
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (i == 0 && j == 0 && k == 0) continue;
        g[0] = i / L[0];
        g[1] = j / L[1];
        g[2] = k / L[2];
        double G = dist(3, g, origin);
        res += pow(G, -2) * exp(-M_PI * M_PI * G * G / (a * a)) / (V * M_PI);
      }
  res -= M_PI / (a * a * V);
  for (int i = -n; i <= n; ++i)
    for (int j = -n; j <= n; ++j)
      for (int k = -n; k <= n; ++k) {
        if (i == 0 && j == 0 && k == 0) continue;
        r[0] = i * L[0];
        r[1] = j * L[1];
        r[2] = k * L[2];
        double R = dist(3, r, origin);
        res += erfc(a * R) / R;
      }
  res -= 2 * a * pow(M_PI, -0.5);
  return p->coul_s * res;
}

/* signed reweighting factor xi -> xi2: md_pimd_x.c:4652-4706; returns s */
double orc_vi_sign(int N, double beta, double vi, double vi2, const double *ENk, const double *VBN) {
  (void)vi;
  double *V2 = (double *)malloc(sizeof(double) * (N + 1));
  double *sg = (double *)malloc(sizeof(double) * (N + 1));
  if (!V2 || !sg) {
    free(V2);
    free(sg);
    return NAN;
  }
  V2[0] = 0;
  sg[0] = 1;
  double sv = vi2 < 0 ? -1 : 1, a2 = fabs(vi2);
  for (int N2 = 1; N2 <= N; ++N2) {
    double sum = 0;
    double m = xminE(N2, beta, a2, ENk, V2);
    for (int k = 1; k <= N2; ++k) {
      if (vi2 == 0 && k - 1 != 0) continue;
      sum += sg[N2 - k] * pow(sv, k - 1) * xexp(k, ENk[tri(N2) + k - 1] + V2[N2 - k], m, beta, a2);
    }
    sg[N2] = sum >= 0 ? 1 : -1;
    V2[N2] = (m - log(fabs(sum)) + log(N2)) / beta;
  }
  double r = sg[N] * exp(-beta * V2[N] + beta * VBN[N]);
  free(V2);
  free(sg);
  return r;
}

/* ------------------------------------------------------------------ */
/* one step                                                             */
/* ------------------------------------------------------------------ */

int orc_step(orc_sim_t *s, const orc_step_cfg_t *c, double h, double *ENk, double *Eint,
             double *VBN) {
  if (orc_nhc_vv3_1(s, h)) return -1;
  orc_reset_force(s);
  orc_fast_fill_ENk(s, c->N, c->P, c->omegaP, c->image, ENk, Eint);
  orc_fill_VB(c->N, c->beta, c->vi, ENk, VBN);
  if (orc_fast_force_VB(s, c->N, c->P, c->beta, c->vi, c->omegaP, c->image, ENk, VBN, NULL, NULL))
    return -1;
  if (c->trap_kind) orc_trap_force(s, c->N, c->P, c->trap_kind, &c->prm);
  if (c->pair_kind) orc_pair_force(s, c->N, c->P, c->pair_kind, &c->prm);
  if (orc_nhc_vv3_2(s, h)) return -1;
  if (c->pbc) orc_periodic_boundary(s);
  return 0;
}

/* ------------------------------------------------------------------ */
/* random numbers: md_util_x.c:671-693                                  */
/* ------------------------------------------------------------------ */

static double g_second;
static int g_has;

void orc_set_seed(unsigned int seed) { srand(seed); }

double orc_random_uniform(double a, double b) {
  double r = ((double)rand()) / RAND_MAX;
  return a + (b - a) * r;
}

double orc_random_gaussian(void) {
  if (g_has) {
    g_has = 0;
    return g_second;
  }
  g_has = 1;
  double r = sqrt(-2 * log(orc_random_uniform(0, 1)));
  double ang = 2 * M_PI * orc_random_uniform(0, 1);
  g_second = r * sin(ang);
  return r * cos(ang);
}
