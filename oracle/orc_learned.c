/*
 * orc_learned.c -- CPU restatement of the learned Ewald residual's parts
 * (descriptors, the 64-128-128-4 network, its loss and gradients), and of
 * MD-Lab's spherical static structure factor (orc_sk_sphere,
 * orc_sk_structure).
 *
 * TEST INFRASTRUCTURE ONLY, like the rest of oracle/.  MD-Lab has no learned
 * part, so there is no reference code to follow: this file states the
 * definitions the GPU kernels implement, in double precision, with optional
 * rounding to BF16 at exactly the points where the GPU stores BF16 values,
 * so that a GPU result can be compared element by element.  The gradients
 * are in turn checked against finite differences of orc_mlp_loss.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define ORC_IN 64
#define ORC_H 128
#define ORC_OUT 4
#define ORC_W1 0
#define ORC_B1 (ORC_W1 + ORC_H * ORC_IN)
#define ORC_W2 (ORC_B1 + ORC_H)
#define ORC_B2 (ORC_W2 + ORC_H * ORC_H)
#define ORC_W3 (ORC_B2 + ORC_H)
#define ORC_B3 (ORC_W3 + ORC_OUT * ORC_H)
#define ORC_NPARAM (ORC_B3 + ORC_OUT)

int orc_mlp_nparam(void) { return ORC_NPARAM; }

/* round to the nearest BF16 value, ties to even (through float) */
double orc_bf16(double v) {
  float f = (float)v;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  memcpy(&f, &u, 4);
  return f;
}
static double rnd(double v, int on) { return on ? orc_bf16(v) : v; }

/*
 * Descriptors of the N particles of one bead slice (positions AoS
 * x[l*3 + d], box L[3]), 64 per particle:
 *
 * F[0..31]: every minimum-image partner c != l with r < rc deposits
 *   fc(r) = (1 - r^2/rc^2)^2 into a histogram of nb bins of width h = rc/nb
 *   by linear weights between bin centres (b + 1/2) h: t = r/h - 1/2,
 *   b0 = floor(t), w = t - b0; bin b0 gets fc (1 - w), bin b0 + 1 gets fc w;
 *   below the first centre (b0 < 0) or from the last centre on
 *   (b0 >= nb - 1) all of fc goes to the end bin.  F[f] = sum_b hist[b]
 *   basis[b][f] (basis[nb][32]: Gaussians in r).
 * F[32..63]: for the 32 lowest shells |n|^2 of the reciprocal lattice
 *   (k = 2 pi n / L), sqrt(sum over the shell's half-space vectors of
 *   |S(k)|^2 / (N count)), S(k) = sum_l exp(i k . x_l); the same for every
 *   particle of the slice.
 * Vector features Vv[3m + d] = sum_c fc(r) exp(-(r - mu_m)^2 / (2 s_m^2))
 *   (x_l - x_c)_d / r.
 */
#define ORC_SHELLS 32

/* the ORC_SHELLS lowest positive sums of three squares */
static void lowest_shells(int *sh) {
  int n = 0;
  for (int n2 = 1; n < ORC_SHELLS; ++n2) {
    int ok = 0;
    for (int a = 0; a * a <= n2 && !ok; ++a)
      for (int b = 0; a * a + b * b <= n2 && !ok; ++b) {
        const int c2 = n2 - a * a - b * b, c = (int)lround(sqrt((double)c2));
        if (c * c == c2) ok = 1;
      }
    if (ok) sh[n++] = n2;
  }
}

void orc_desc_features(int N, const double *x, const double *L, double rc, int nb, const double *basis,
                       const double *vmu, const double *vsig, double *F, double *Vv) {
  const double h = rc / nb;
  double hist[1024];
  for (int l = 0; l < N; ++l) {
    for (int b = 0; b < nb; ++b) hist[b] = 0;
    for (int i = 0; i < 9; ++i) Vv[l * 9 + i] = 0;
    for (int c = 0; c < N; ++c) {
      if (c == l) continue;
      double d[3], r2 = 0;
      for (int k = 0; k < 3; ++k) {
        d[k] = x[l * 3 + k] - x[c * 3 + k];
        d[k] -= L[k] * rint(d[k] / L[k]);
        r2 += d[k] * d[k];
      }
      if (!(r2 < rc * rc)) continue;
      const double r = sqrt(r2), u = 1 - r2 / (rc * rc), fc = u * u;
      const double t = r / h - 0.5;
      int b0 = (int)floor(t);
      double w = t - b0;
      if (b0 < 0) {
        b0 = 0;
        w = 0;
      }
      if (b0 >= nb - 1) {
        b0 = nb - 1;
        w = 0;
      }
      hist[b0] += fc * (1 - w);
      if (w > 0) hist[b0 + 1] += fc * w;
      for (int m = 0; m < 3; ++m) {
        const double q = fc * exp(-(r - vmu[m]) * (r - vmu[m]) / (2 * vsig[m] * vsig[m])) / r;
        for (int k = 0; k < 3; ++k) Vv[l * 9 + 3 * m + k] += q * d[k];
      }
    }
    for (int f = 0; f < 32; ++f) {
      double s = 0;
      for (int b = 0; b < nb; ++b) s += hist[b] * basis[b * 32 + f];
      F[l * ORC_IN + f] = s;
    }
  }
  /* structure-factor shells */
  int sh[ORC_SHELLS];
  lowest_shells(sh);
  const int nmax = (int)floor(sqrt((double)sh[ORC_SHELLS - 1]));
  double acc[ORC_SHELLS];
  int cnt[ORC_SHELLS];
  for (int i = 0; i < ORC_SHELLS; ++i) acc[i] = 0, cnt[i] = 0;
  for (int a = 0; a <= nmax; ++a)
    for (int b = -nmax; b <= nmax; ++b)
      for (int c = -nmax; c <= nmax; ++c) {
        if (!(a > 0 || (a == 0 && b > 0) || (a == 0 && b == 0 && c > 0))) continue;
        const int n2 = a * a + b * b + c * c;
        int s2 = -1;
        for (int i = 0; i < ORC_SHELLS; ++i)
          if (sh[i] == n2) s2 = i;
        if (s2 < 0) continue;
        double sr = 0, si = 0;
        for (int l = 0; l < N; ++l) {
          const double ph = 2 * M_PI * (a * x[l * 3] / L[0] + b * x[l * 3 + 1] / L[1] + c * x[l * 3 + 2] / L[2]);
          sr += cos(ph);
          si += sin(ph);
        }
        acc[s2] += sr * sr + si * si;
        cnt[s2] += 1;
      }
  for (int i = 0; i < ORC_SHELLS; ++i) {
    const double v = sqrt(acc[i] / ((double)N * cnt[i]));
    for (int l = 0; l < N; ++l) F[l * ORC_IN + 32 + i] = v;
  }
}

/*
 * Forward pass of rows inputs X[r][64]:  h1 = tanh(W1 x + b1),
 * h2 = tanh(W2 h1 + b2), y = W3 h2 + b3.  p holds the parameters in the order
 * W1[128][64], b1, W2[128][128], b2, W3[4][128], b3.  With bf != 0 the
 * weights, inputs and activations are rounded to BF16 (the tensor-core
 * operands); sums and biases stay in double.  H1/H2 (optional) receive the
 * activations as used by the next layer.
 */
void orc_mlp_forward(int rows, const double *X, const double *p, int bf, double *Y, double *H1, double *H2) {
  double h1[ORC_H], h2[ORC_H];
  for (int r = 0; r < rows; ++r) {
    for (int o = 0; o < ORC_H; ++o) {
      double z = 0;
      for (int i = 0; i < ORC_IN; ++i) z += rnd(X[r * ORC_IN + i], bf) * rnd(p[ORC_W1 + o * ORC_IN + i], bf);
      h1[o] = rnd(tanh(z + p[ORC_B1 + o]), bf);
    }
    for (int o = 0; o < ORC_H; ++o) {
      double z = 0;
      for (int i = 0; i < ORC_H; ++i) z += h1[i] * rnd(p[ORC_W2 + o * ORC_H + i], bf);
      h2[o] = rnd(tanh(z + p[ORC_B2 + o]), bf);
    }
    for (int o = 0; o < ORC_OUT; ++o) {
      double z = 0;
      for (int i = 0; i < ORC_H; ++i) z += h2[i] * rnd(p[ORC_W3 + o * ORC_H + i], bf);
      Y[r * ORC_OUT + o] = z + p[ORC_B3 + o];
    }
    if (H1) memcpy(H1 + (size_t)r * ORC_H, h1, sizeof h1);
    if (H2) memcpy(H2 + (size_t)r * ORC_H, h2, sizeof h2);
  }
}

/*
 * Loss of a batch: per row with weight w = V[r][9],
 *   we (y0 - t0)^2 + wf |y1 v1 + y2 v2 + y3 v3 - (t1, t2, t3)|^2,
 * v_m = V[r][3m .. 3m+2]; both sums scaled by inv_rows.  loss[0], loss[1]:
 * the two terms (unscaled by inv_rows, as the GPU accumulates them).
 */
static void out_grad(const double *y, const double *v, const double *t, double we, double wf, double inv_rows,
                     double *dy, double *le, double *lf) {
  const double w = v[9], de = y[0] - t[0];
  double dF[3];
  for (int k = 0; k < 3; ++k) dF[k] = y[1] * v[k] + y[2] * v[3 + k] + y[3] * v[6 + k] - t[1 + k];
  *le = we * de * de * w;
  *lf = wf * (dF[0] * dF[0] + dF[1] * dF[1] + dF[2] * dF[2]) * w;
  dy[0] = 2 * we * de * w * inv_rows;
  for (int m = 0; m < 3; ++m)
    dy[1 + m] = 2 * wf * (dF[0] * v[3 * m] + dF[1] * v[3 * m + 1] + dF[2] * v[3 * m + 2]) * w * inv_rows;
}

double orc_mlp_loss(int rows, const double *X, const double *V, const double *T, const double *p, double we,
                    double wf, double inv_rows, int bf) {
  double y[ORC_OUT], dy[ORC_OUT], s = 0;
  for (int r = 0; r < rows; ++r) {
    double le, lf;
    orc_mlp_forward(1, X + (size_t)r * ORC_IN, p, bf, y, 0, 0);
    out_grad(y, V + (size_t)r * 12, T + (size_t)r * 4, we, wf, inv_rows, dy, &le, &lf);
    s += (le + lf) * inv_rows;
  }
  return s;
}

/*
 * Gradient of orc_mlp_loss with respect to p (grad[ORC_NPARAM], overwritten)
 * and the two loss terms.  With bf != 0 the rounding follows the GPU kernel:
 * the output gradient enters dW3 as BF16 and dH2 in full precision; dZ2 and
 * dZ1 enter the tensor-core products (dW2, dH1, dW1) as BF16 and the bias
 * sums in full precision; tanh' uses the BF16 activations.
 */
void orc_mlp_grad(int rows, const double *X, const double *V, const double *T, const double *p, double we,
                  double wf, double inv_rows, int bf, double *grad, double *loss) {
  double h1[ORC_H], h2[ORC_H], y[ORC_OUT], dy[ORC_OUT], dz2[ORC_H], dz1[ORC_H];
  memset(grad, 0, sizeof(double) * ORC_NPARAM);
  loss[0] = loss[1] = 0;
  for (int r = 0; r < rows; ++r) {
    const double *x = X + (size_t)r * ORC_IN;
    double le, lf;
    orc_mlp_forward(1, x, p, bf, y, h1, h2);
    out_grad(y, V + (size_t)r * 12, T + (size_t)r * 4, we, wf, inv_rows, dy, &le, &lf);
    loss[0] += le;
    loss[1] += lf;
    for (int o = 0; o < ORC_OUT; ++o) {
      grad[ORC_B3 + o] += dy[o];
      for (int c = 0; c < ORC_H; ++c) grad[ORC_W3 + o * ORC_H + c] += rnd(dy[o], bf) * h2[c];
    }
    for (int c = 0; c < ORC_H; ++c) {
      double dh = 0;
      for (int o = 0; o < ORC_OUT; ++o) dh += dy[o] * rnd(p[ORC_W3 + o * ORC_H + c], bf);
      dz2[c] = dh * (1 - h2[c] * h2[c]);
      grad[ORC_B2 + c] += dz2[c];
    }
    for (int i = 0; i < ORC_H; ++i) {
      double dh = 0;
      for (int o = 0; o < ORC_H; ++o) dh += rnd(dz2[o], bf) * rnd(p[ORC_W2 + o * ORC_H + i], bf);
      dz1[i] = dh * (1 - h1[i] * h1[i]);
      grad[ORC_B1 + i] += dz1[i];
    }
    for (int o = 0; o < ORC_H; ++o) {
      const double a = rnd(dz2[o], bf), b = rnd(dz1[o], bf);
      for (int i = 0; i < ORC_H; ++i) grad[ORC_W2 + o * ORC_H + i] += a * h1[i];
      for (int i = 0; i < ORC_IN; ++i) grad[ORC_W1 + o * ORC_IN + i] += b * rnd(x[i], bf);
    }
  }
}

/*
 * md_statistics_x.c:104-161 (md_alloc_sk_sphere_3d_x): wave vectors of the
 * cube q0, q0 + qincre, ... <= qmax (loop order x, y, z), one per distinct |q|
 * (first found within 1e-4), |q| >= 1e-4, then the reference's exchange sort
 * by |q|.  qs[n], qis[3n] must hold max entries; returns the count.
 */
int orc_sk_sphere(double q0, double qincre, double qmax, int max, double *qs, double *qis) {
  int n = 0;
  for (double qx = q0; qx <= qmax; qx += qincre)
    for (double qy = q0; qy <= qmax; qy += qincre)
      for (double qz = q0; qz <= qmax; qz += qincre) {
        const double q = sqrt(qx * qx + qy * qy + qz * qz);
        if (fabs(q) < 1e-4) continue;
        int found = 0;
        for (int i = 0; i < n && !found; ++i)
          if (fabs(qs[i] - q) < 1e-4) found = 1;
        if (found || n >= max) continue;
        qs[n] = q;
        qis[3 * n] = qx;
        qis[3 * n + 1] = qy;
        qis[3 * n + 2] = qz;
        ++n;
      }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < i; ++j)
      if (qs[j] > qs[i]) {
        double t = qs[i];
        qs[i] = qs[j];
        qs[j] = t;
        for (int k = 0; k < 3; ++k) {
          t = qis[3 * i + k];
          qis[3 * i + k] = qis[3 * j + k];
          qis[3 * j + k] = t;
        }
      }
  return n;
}

/*
 * md_pimd_x.c:5404-5448: for wave vector j, with a = bead 1 and b = bead
 * (pi-1) mod P + 1 of every particle (positions x[(l*P + bead)*3 + d],
 * bead 0-based), res[j] = (sum cos q.x_a)(sum cos q.x_b)/N +
 * (sum sin q.x_a)(sum sin q.x_b)/N, sums in particle order.
 */
void orc_sk_structure(int N, int P, const double *x, int pi, int nq, const double *qis, double *res) {
  const int jb = (pi - 1) % P;
  for (int j = 0; j < nq; ++j) {
    double out = 0, sum = 0, sum2 = 0;
    for (int l = 0; l < N; ++l) {
      double t = 0;
      for (int d = 0; d < 3; ++d) t += qis[3 * j + d] * x[((size_t)l * P) * 3 + d];
      sum += cos(t);
    }
    for (int l = 0; l < N; ++l) {
      double t = 0;
      for (int d = 0; d < 3; ++d) t += qis[3 * j + d] * x[((size_t)l * P + jb) * 3 + d];
      sum2 += cos(t);
    }
    out += sum * sum2 / N;
    sum = sum2 = 0;
    for (int l = 0; l < N; ++l) {
      double t = 0;
      for (int d = 0; d < 3; ++d) t += qis[3 * j + d] * x[((size_t)l * P) * 3 + d];
      sum += sin(t);
    }
    for (int l = 0; l < N; ++l) {
      double t = 0;
      for (int d = 0; d < 3; ++d) t += qis[3 * j + d] * x[((size_t)l * P + jb) * 3 + d];
      sum2 += sin(t);
    }
    out += sum * sum2 / N;
    res[j] = out;
  }
}
