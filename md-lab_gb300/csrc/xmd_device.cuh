// xmd_device.cuh -- device helpers shared by the kernels of xmd_kernels.cu
// and the persistent ensemble kernel (xmd_ensemble.cu): minimum image, warp
// and block reductions, the thermostat chain update, cycle springs, the
// extended-range arithmetic of the exchange recursions, the exchange spring
// gradients, trap forces, and the FP32 pair and phase arithmetic of the
// mixed form.  Everything here is inline device code or a constant.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <cstddef>
#include <cstdint>

#include "xmd_ewald_tables.h"
#include "xmd_kernels.cuh"

namespace xk {

#define FULL 0xffffffffu

__device__ inline size_t dtri(int n) { return (size_t)n * (n - 1) / 2; }

// Nearest image of a difference a in a box of side L: md_simulation_x.c:70-81
// with md_periodic_image_count_x (:858-865) shift a + L/2 into [0, L] by
// whole boxes and subtract L/2 again; a - L rint(a/L) is the same image in
// three FP64 operations instead of eight (ties at exactly L/2 aside, the
// results differ in the last bits only).
__device__ inline double min_image(double a, double L, double invL) { return fma(-L, rint(a * invL), a); }

__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
__device__ inline double warp_min(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    double t = __shfl_xor_sync(FULL, v, o);
    v = t < v ? t : v;
  }
  return v;
}

// block-wide reductions; buf needs 33 doubles and must not be reused by the
// caller until one more __syncthreads() has passed.
__device__ inline double block_sum(double v, double *buf) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_sum(v);
  if (lane == 0) buf[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < nw ? buf[lane] : 0.0;
    t = warp_sum(t);
    if (lane == 0) buf[32] = t;
  }
  __syncthreads();
  return buf[32];
}
__device__ inline double block_min(double v, double init, double *buf) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  v = warp_min(v);
  if (lane == 0) buf[w] = v;
  __syncthreads();
  if (w == 0) {
    double t = lane < nw ? buf[lane] : init;
    t = warp_min(t);
    if (lane == 0) buf[32] = t < init ? t : init;
  }
  __syncthreads();
  return buf[32];
}

// Thermostat update of one chain.  v[], F[], mass[] are the chain's DOFs
// (ndof of them, counted as cfv DOFs in the kinetic term); half = 1 is
// md_update_nhc_VV3_1_x (kick, chain, drift, chain), half = 2 is
// md_update_nhc_VV3_2_x (kick, chain).
template <int L>
struct ChainState {
  double th[L], vt[L], Q[L];
  double iQ[L];  // 1/Q (one-DOF chains): multiplications instead of FP64 divisions
};

// md_simulation_x.c:599-613; INV: divide by multiplying with the stored 1/Q
// (a double division is a multi-instruction sequence on the slow FP64 pipe)
template <int L, bool INV = false>
__device__ inline void chain_forces(const ChainState<L> &c, double kin, double cfv, double kT,
                                    double *nhf) {
  nhf[0] = INV ? (kin - cfv * kT) * c.iQ[0] : (kin - cfv * kT) / c.Q[0];
#pragma unroll
  for (int j = 1; j < L; ++j) {
    const double num = c.Q[j - 1] * c.vt[j - 1] * c.vt[j - 1] - kT;
    nhf[j] = INV ? num * c.iQ[j] : num / c.Q[j];
  }
}


// exp(x) for the thermostat factors exp(-h v_eta / 4) and exp(-h v_eta / 2):
// for |x| < 1/4, the usual case with a small step, its Taylor series through
// x^12/12! by Horner's rule (the first omitted term is below 3e-18
// relative, a fortieth of the FP64 rounding unit: twelve FMAs instead of a
// general exponential's range reduction and longer polynomial), otherwise
// exp().  The range test reads the bit pattern, off the FP64 pipe.
__device__ inline double nhc_exp(double x) {
  if ((__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFLL) < 0x3FD0000000000000LL) {  // |x| < 2^-2
    double p = 1.0 / 479001600.0;
    p = fma(p, x, 1.0 / 39916800.0);
    p = fma(p, x, 1.0 / 3628800.0);
    p = fma(p, x, 1.0 / 362880.0);
    p = fma(p, x, 1.0 / 40320.0);
    p = fma(p, x, 1.0 / 5040.0);
    p = fma(p, x, 1.0 / 720.0);
    p = fma(p, x, 1.0 / 120.0);
    p = fma(p, x, 1.0 / 24.0);
    p = fma(p, x, 1.0 / 6.0);
    p = fma(p, x, 0.5);
    p = fma(p, x, 1.0);
    return fma(p, x, 1.0);
  }
  return exp(x);
}

template <int L>
__device__ inline void chain_odd(ChainState<L> &c, double h, const double *nhf) {
  constexpr int M2 = L / 2;
  // exp(-h x / 2) is taken as exp(-h x / 4)^2 (one FP64 exp instead of two,
  // equal to rounding); the last member has no successor, both factors are 1
#pragma unroll
  for (int j = 1; j <= M2; ++j) {
    if (j == M2) {
      c.vt[2 * j - 1] = c.vt[2 * j - 1] + 0.5 * h * nhf[2 * j - 1];
    } else {
      const double e = nhc_exp(-0.25 * h * c.vt[2 * j]);
      c.vt[2 * j - 1] = c.vt[2 * j - 1] * (e * e) + 0.5 * h * nhf[2 * j - 1] * e;
    }
  }
}

template <int D>
__device__ inline double spring2(Geo g, const double *x, int ja, int la, int jb, int lb,
                                 int image) {
  double s = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    double t = x[sidx(ja, d, la, D, g.Ns)] - x[sidx(jb, d, lb, D, g.Ns)];
    if (image) t = min_image(t, g.box[d], g.inv_box[d]);
    s += t * t;
  }
  return s;
}

// spring between bead P of particle a and bead 1 of particle b (0-based),
// weighted by the mass of the bead-P end as in the reference.
template <int D>
__device__ inline double link(Geo g, const double *x, const double *m, double w2, int a, int b,
                              int image) {
  const int jP = g.P - 1;
  return 0.5 * m[(size_t)jP * g.Ns + a] * w2 * spring2<D>(g, x, jP, a, 0, b, image);
}

// exclusive prefix sums out[c] = in[0] + ... + in[c-1] (c = 0..n) by the
// block, in a fixed order (contiguous runs per thread, then the run totals
// scanned over the block): every block that calls it gets the same numbers
__device__ inline void block_exclusive_prefix(const double *__restrict__ in, int n, double *out) {
  __shared__ double wsum[32];
  const int per = (n + blockDim.x - 1) / blockDim.x;
  const int a = min(n, (int)threadIdx.x * per), b = min(n, a + per);
  double run = 0.0;
  for (int c = a; c < b; ++c) run += in[c];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double inc = run;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double t = __shfl_up_sync(FULL, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) wsum[w] = inc;
  __syncthreads();
  if (w == 0) {
    double v = lane < (int)(blockDim.x >> 5) ? wsum[lane] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double t = __shfl_up_sync(FULL, v, o);
      if (lane >= o) v += t;
    }
    wsum[lane] = v;
  }
  __syncthreads();
  double pre = (w > 0 ? wsum[w - 1] : 0.0) + (inc - run);
  for (int c = a; c < b; ++c) {
    out[c] = pre;
    pre += in[c];
  }
  if (threadIdx.x == blockDim.x - 1) out[n] = pre;
}

// One DOF of the fast-chain thermostat step (slot s = (j D + d) Ns + l,
// l < N): md_update_nhc_VV3_1_x (half 1) or _VV3_2_x (half 2) for the DOF
// and its own chain.
template <int D, int L>
__device__ inline void nhc_slot(const Geo &g, int half, size_t s, int l, double *__restrict__ x,
                                double *__restrict__ v, double *__restrict__ f, const double *__restrict__ fex,
                                const double *__restrict__ m, double *__restrict__ th, double *__restrict__ vt,
                                const double *__restrict__ Q, const double *__restrict__ iQ, double kT, double h) {
  const size_t S = g.slots();
  const int j = (int)(s / ((size_t)D * g.Ns));
  constexpr int M2 = L / 2;
  ChainState<L> c;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    c.th[i] = th[i * S + s];
    c.vt[i] = vt[i * S + s];
    c.Q[i] = Q[i * S + s];
    c.iQ[i] = iQ[i * S + s];
  }
  const double mass = m[(size_t)j * g.Ns + l];
  double vv = v[s];
  double F = f[s];
  if (fex) {  // the pending exchange forces, as add_into would add them
    F += fex[s];
    f[s] = F;
  }
  double nhf[L];
  if (half == 1) chain_forces<L, true>(c, mass * vv * vv, 1.0, kT, nhf);
  // thermostatted half kick: md_simulation_x.c:674-678
  const double ek = nhc_exp(-0.25 * h * c.vt[0]);
  vv = vv * (ek * ek) + 0.5 * h * F * ek;
#pragma unroll
  for (int k = 1; k <= M2; ++k) c.th[2 * k - 2] = c.th[2 * k - 2] + h * c.vt[2 * k - 2] / 2;
  if (half == 2) chain_forces<L, true>(c, mass * vv * vv, 1.0, kT, nhf);
  chain_odd<L>(c, h, nhf);
  if (half == 1) {
    x[s] = x[s] + h * vv;  // drift: md_simulation_x.c:684-689
#pragma unroll
    for (int k = 1; k <= M2; ++k) c.th[2 * k - 1] = c.th[2 * k - 1] + h * c.vt[2 * k - 1];
    chain_forces<L, true>(c, mass * vv * vv, 1.0, kT, nhf);
#pragma unroll
    for (int k = 1; k <= M2; ++k)
      {
        const double e = nhc_exp(-0.5 * h * c.vt[2 * k - 1]);
        c.vt[2 * k - 2] = c.vt[2 * k - 2] * (e * e) + h * nhf[2 * k - 2] * e;
      }
  }
  v[s] = vv;
#pragma unroll
  for (int i = 0; i < L; ++i) {
    th[i * S + s] = c.th[i];
    vt[i * S + s] = c.vt[i];
  }
}



// ln 2 split so that e * LN2_HI is exact for |e| < 2^21 (32 significant bits)
constexpr double LN2_HI = 0.6931471803691238, LN2_LO = 1.9082149292705877e-10;
constexpr double LOG2E = 1.4426950408889634;

struct Ext {
  double m;  // mantissa (0 or a normal number of moderate size)
  int e;     // value = m * 2^e
};

// exp(x) in extended range for any finite x: 2^e * exp(r), |r| <= ln2/2
__device__ inline Ext ext_exp(double x) {
  const double q = rint(x * LOG2E);
  double r = fma(-q, LN2_HI, x);
  r = fma(-q, LN2_LO, r);
  // exp(r) for |r| <= ln2/2 by its Taylor series through r^13/13! (Horner):
  // the first omitted term is below 5e-18 relative; thirteen FMAs, where a
  // general exponential would reduce the argument a second time
  double p = 1.0 / 6227020800.0;
  p = fma(p, r, 1.0 / 479001600.0);
  p = fma(p, r, 1.0 / 39916800.0);
  p = fma(p, r, 1.0 / 3628800.0);
  p = fma(p, r, 1.0 / 362880.0);
  p = fma(p, r, 1.0 / 40320.0);
  p = fma(p, r, 1.0 / 5040.0);
  p = fma(p, r, 1.0 / 720.0);
  p = fma(p, r, 1.0 / 120.0);
  p = fma(p, r, 1.0 / 24.0);
  p = fma(p, r, 1.0 / 6.0);
  p = fma(p, r, 0.5);
  p = fma(p, r, 1.0);
  return {fma(p, r, 1.0), (int)q};
}

// exp(x) through ext_exp, the power of two put into the exponent field by
// integer arithmetic; results near or beyond the ends of the normal range
// (|x| > 700) are left to exp()
__device__ inline double exp_fast(double x) {
  const Ext w = ext_exp(x);
  if (w.e <= -1020 || w.e >= 1020) return exp(x);
  return __longlong_as_double(__double_as_longlong(w.m) + ((long long)w.e << 52));
}

// m * 2^d for d <= 0 (0 once the result would drop below the subnormals)
__device__ inline double scale_down(double m, int d) {
  if (d >= -1022) return m * __longlong_as_double((long long)(d + 1023) << 52);
  if (d < -1100) return 0.0;
  return m * 0x1p-1022 * __longlong_as_double((long long)(d + 1022 + 1023) << 52);
}

// acc += t in extended range
__device__ inline void ext_add(double &am, int &ae, double tm, int te) {
  if (tm == 0.0) return;
  if (am == 0.0) {
    am = tm;
    ae = te;
  } else if (te > ae) {
    am = scale_down(am, ae - te) + tm;
    ae = te;
  } else {
    am += scale_down(tm, te - ae);
  }
}

__device__ inline void ext_norm(double &m, int &e) {
  if (m == 0.0) return;
  int k;
  m = frexp(m, &k);
  e += k;
}

// packed lower triangle: row i (1..N), column j (0..i-1) at tri(i) + j
__device__ inline size_t moff(int i, int j) { return (size_t)i * (i - 1) / 2 + j; }

// Both weight triangles in one launch: block (row, direction), threads
// along the row.  Forward row n: M_{n,j} = exp(-beta ENk[n][n-j] + (n-j-1)
// ln xi - ln n); backward row i <-> u = N-i+1, column j <-> l = N-j:
// exp(-beta ENk[l][i-j] + (i-j-1) ln xi - ln l).  ln xi and the table
// lnn[l] = ln l come from the host.
// sgn = -1 gives the weights of a negative xi' (|xi'| in vi and lnvi): the
// mantissa of every term with odd k - 1 changes sign.
// both = 1 (first = 0, both directions): the two triangles hold the same
// numbers, M_{l,l-k} = M'_{N-l+k,N-l}, so block l takes row l of ENk and
// writes each weight into both (one exponential per entry).
__device__ inline void weights_row(int N, double beta, double vi, double lnvi, const double *__restrict__ ENk,
                                   const double *__restrict__ lnn, double *__restrict__ Mf, int *__restrict__ Ef,
                                   double *__restrict__ Mb, int *__restrict__ Eb, int first, int sgn, int both,
                                   int row, int dir, int t0, int nt) {
  double *Mm = dir ? Mb : Mf;
  int *Me = dir ? Eb : Ef;
  for (int j = t0; j < row; j += nt) {
    const int k = row - j;
    const int l = dir ? N - j : row;
    Ext w{0.0, 0};
    if (vi != 0.0 || k == 1) w = ext_exp(-beta * ENk[dtri(l) + k - 1] + (k - 1) * lnvi - lnn[l]);
    if (sgn < 0 && ((k - 1) & 1)) w.m = -w.m;
    Mm[moff(row, j)] = w.m;
    Me[moff(row, j)] = w.e;
    if (both) {
      Mb[moff(N - row + k, N - row)] = w.m;
      Eb[moff(N - row + k, N - row)] = w.e;
    }
  }
}

// X_0 = 1, X_i = sum_{j<i} M_{i,j} X_j (i = 1..N); out_i = -ln(X_i)/beta written
// to out[i] (forward) or out[N-i] (backward).  One block, 16 warps.
constexpr int TS_WARPS = 16, TS_CHUNK = 32;

// v * 2^d for a non-negative double v and d <= 0, by integer arithmetic on
// the exponent field (the FP64 pipe is the scarce resource); results below
// the normal range are flushed to 0 (they are below 2^-1021 of the sum
// they enter)
__device__ inline double scale2(double v, int d) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7ff);
  const long long r = b + ((long long)d << 52);
  return __longlong_as_double((ex == 0 || ex + d <= 0) ? 0LL : r);  // selects, no branch
}

// normalise a non-negative extended value to a mantissa in [0.5, 1)
__device__ inline void norm2(double &m, int &e) {
  const long long b = __double_as_longlong(m);
  const int ex = (int)((b >> 52) & 0x7ff);
  const bool z = ex == 0;  // zero (values here are never subnormal) stays zero
  e = z ? e : e + ex - 1022;
  m = __longlong_as_double(z ? 0LL : ((b & ~(0x7ffLL << 52)) | (1022LL << 52)));
}

// Block b solves direction first + b (0 forward, 1 backward) with the
// weights (Mm[dir], Me[dir]) into out[dir]: launched with two blocks, the
// forward and backward recursions run side by side on two SMs.
struct TriJob {
  const double *Mm[2];
  const int *Me[2];
  double *out[2];
  double *sign;  // optional: sign of X_i (signed weights), forward direction only
  double *Bm[2];  // inverses of the 32 x 32 diagonal blocks (unsigned weights):
  int *Be[2];     // [chunk][32][32] mantissas and exponents
  double *Xm[2];  // optional: the unknowns X_0..X_N in extended range (unsigned
  int *Xe[2];     // solves), kept for the connection probabilities
};

// Extended-range dot product of row i of the weights with the unknowns over
// columns [j0, j1), reduced over the warp: (am, E) with value am 2^E.  One
// pass: each lane keeps a running (am, E) and rescales when a larger term
// exponent arrives; loads are issued four columns per lane at a time.  Zero
// weights (xi = 0 beyond k = 1) are skipped by their bit pattern.  E is
// EXT_NONE while a lane has no term.
constexpr int EXT_NONE = -2147483647;

// Warp sums of extended-range terms are taken in 64-bit fixed point on the
// integer pipe: a warp-wide FP64 add holds GB300's FP64 pipe for many cycles,
// and a five-level reduction of doubles cost more than the dot products
// around it.  fx(v, d, FB): v * 2^d (d <= 0) as a signed integer with FB
// fractional bits, built from the bit pattern (truncated); the caller keeps
// 32 |v| 2^FB below 2^63.
__device__ inline long long fx(double v, int d, int FB) {
  const long long b = __double_as_longlong(v);
  const int ex = (int)((b >> 52) & 0x7ff);
  const long long sig = (b & 0xFFFFFFFFFFFFFLL) | (1LL << 52);
  const int sh = ex - 1075 + FB + d;
  const long long q = sh >= 0 ? (sig << sh) : (sh > -63 ? (sig >> -sh) : 0LL);
  return ex == 0 ? 0LL : (b < 0 ? -q : q);
}
// q * 2^-FB as a double (truncated to 53 bits), by integer arithmetic
__device__ inline double fx_to_double(long long q, int FB) {
  if (q == 0) return 0.0;
  const bool neg = q < 0;
  const unsigned long long u = neg ? (unsigned long long)(-q) : (unsigned long long)q;
  const int top = 63 - __clzll((long long)u);
  const unsigned long long m = top > 52 ? (u >> (top - 52)) : (u << (52 - top));
  const long long bits = ((long long)(neg ? 1 : 0) << 63) | ((long long)(top - FB + 1023) << 52) |
                         (long long)(m & 0xFFFFFFFFFFFFFULL);
  return __longlong_as_double(bits);
}
__device__ inline long long warp_sum_ll(long long q) {
#pragma unroll
  for (int o = 16; o; o >>= 1) q += __shfl_xor_sync(FULL, q, o);
  return q;
}
// warp sum of arbitrary finite doubles on the integer pipe: every lane's
// value in 57-bit fixed point relative to the largest lane's binade, summed
// exactly, rounded once (truncation) to 53 bits; the result reaches every lane
__device__ inline double warp_sum_fx(double v) {
  const int ex = (int)((__double_as_longlong(v) >> 52) & 0x7ff);
  int em = ex;
#pragma unroll
  for (int o = 16; o; o >>= 1) em = max(em, __shfl_xor_sync(FULL, em, o));
  if (em == 0) return 0.0;  // all zero (subnormals do not occur in these sums)
  const long long q = warp_sum_ll(fx(v, 1022 - em, 57));
  if (q == 0) return 0.0;
  const double r = fx_to_double(q, 57);  // value 2^(1022 - em) too large
  return __longlong_as_double(__double_as_longlong(r) + ((long long)(em - 1022) << 52));
}

constexpr int XD_SLOTS = 4;  // columns per lane per pass (loads in flight against L2 latency)
__device__ inline void ext_dot(const double *__restrict__ mr, const int *__restrict__ er, const double *Xm,
                               const int *Xe, int j0, int j1, int lane, double &am_out, int &E_out) {
  double am = 0.0;
  int E = EXT_NONE;
  for (int jb = j0 + lane; jb - lane < j1; jb += 32 * XD_SLOTS) {
    double mv[XD_SLOTS], xv[XD_SLOTS];
    int ev[XD_SLOTS], xe[XD_SLOTS];
#pragma unroll
    for (int u = 0; u < XD_SLOTS; ++u) {
      const int j = jb + 32 * u;
      const bool ok = j < j1;
      mv[u] = ok ? mr[j] : 0.0;
      ev[u] = ok ? er[j] : 0;
      xv[u] = ok ? Xm[j] : 0.0;
      xe[u] = ok ? Xe[j] : 0;
    }
#pragma unroll
    for (int u = 0; u < XD_SLOTS; ++u) {
      if (jb - lane + 32 * u >= j1) break;  // warp-uniform: no lane has this slot
      const bool nz = __double_as_longlong(mv[u]) != 0;
      const int te = ev[u] + xe[u];
      const int ne = (nz && (E == EXT_NONE || te > E)) ? te : E;
      const double a2 = scale2(am, E == EXT_NONE ? 0 : E - ne);
      const double t2 = fma(mv[u], scale2(xv[u], nz ? te - ne : 0), a2);
      am = nz ? t2 : am;
      E = ne;
    }
  }
  // each lane's sum normalised to a mantissa below 1, so that 57 fractional
  // bits keep the 32-lane sum below 2^62 and resolve it to 2^-51 of itself
  if (E != EXT_NONE) norm2(am, E);
  if (__double_as_longlong(am) == 0) E = EXT_NONE;
  int Em = E;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const int oe = __shfl_xor_sync(FULL, Em, o);
    Em = (Em == EXT_NONE || (oe != EXT_NONE && oe > Em)) ? oe : Em;
  }
  const long long q = warp_sum_ll(E == EXT_NONE ? 0LL : fx(am, E - Em, 57));
  am_out = fx_to_double(q, 57);
  E_out = Em;
}

// (pm, pe) += (am, E), both non-negative extended-range values; normalised
__device__ inline void ext_acc(double &pm, int &pe, double am, int E) {
  if (__double_as_longlong(am) != 0 && E != EXT_NONE) {
    if (__double_as_longlong(pm) == 0) {
      pm = am;
      pe = E;
    } else {
      const int mx = pe > E ? pe : E;
      pm = scale2(pm, pe - mx) + scale2(am, E - mx);
      pe = mx;
    }
  }
  norm2(pm, pe);
}

// The chunks of TS_CHUNK rows are solved in order by warp 0.  Row i's sum
// over the unknowns of earlier chunks is split: the part over all but the
// previous chunk is computed by warps 1.. while warp 0 is still solving that
// previous chunk (so it costs no time on the sequential path); the previous
// chunk's 32 columns are added by all warps between the two solves.  The
// weights the sequential steps need (the chunk's own triangle and the
// 32 x 32 block of the previous chunk's columns) are staged in shared memory
// by warps 1.. one chunk ahead, so the sequential path reads no global memory.
constexpr int TS_LD = TS_CHUNK + 1;  // padded row of the staged blocks

// (sum, E) of the warp's non-negative extended terms (pm, pe), nz marking
// lanes with a term; E = EXT_NONE when none has
__device__ inline void ext_warp_sum(bool nz, double pm, int pe, double &sum, int &E) {
  if (nz) norm2(pm, pe);  // mantissa below 1 (see ext_dot)
  int Em = nz ? pe : EXT_NONE;
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    const int oe = __shfl_xor_sync(FULL, Em, o);
    Em = (Em == EXT_NONE || (oe != EXT_NONE && oe > Em)) ? oe : Em;
  }
  sum = fx_to_double(warp_sum_ll(nz ? fx(pm, pe - Em, 57) : 0LL), 57);
  E = Em;
}

// B_c column s for every chunk c: grid (chunks x 4 column groups, directions),
// 8 warps per block, warp w of group g takes column s = 8 g + w.  Lane t
// holds B[t][s]; step r adds row r: B[r][s] = sum_{s<=t<r} A[r][t] B[t][s].
// weight M_{i,j} of direction dir (0 forward, 1 backward) from ENk, the same
// expression k_weights evaluates (so the same number)
__device__ inline Ext weight_at(int N, double beta, double vi, double lnvi, const double *__restrict__ ENk,
                                const double *__restrict__ lnn, int dir, int i, int j) {
  const int k = i - j, l = dir ? N - j : i;
  Ext w{0.0, 0};
  if (vi != 0.0 || k == 1) w = ext_exp(-beta * ENk[dtri(l) + k - 1] + (k - 1) * lnvi - lnn[l]);
  return w;
}

// Column s of B(c) for direction dir, one warp; the chunk's block
// A[r][t] = M_{i0+r, i0+t} (t < r) is staged in Am/Ae.
__device__ inline void block_inv_column(int N, const TriJob &job, int dir, int c, int s,
                                        const double (*Am)[TS_LD], const int (*Ae)[TS_LD]) {
  const int lane = threadIdx.x & 31;
  const int i0 = 1 + c * TS_CHUNK;
  double bm = lane == s ? 0.5 : 0.0;  // B[s][s] = 1 = 0.5 * 2^1
  int be = lane == s ? 1 : 0;
  for (int r = s + 1; r < TS_CHUNK && i0 + r <= N; ++r) {
    const bool in = lane >= s && lane < r;
    const double am = in ? Am[r][lane] : 0.0;
    const int ae = in ? Ae[r][lane] : 0;
    const bool nz = in && __double_as_longlong(am) != 0 && __double_as_longlong(bm) != 0;
    double sm;
    int se;
    ext_warp_sum(nz, am * bm, ae + be, sm, se);
    if (lane == r) {
      bm = se == EXT_NONE ? 0.0 : sm;
      be = se == EXT_NONE ? 0 : se;
      norm2(bm, be);
    }
  }
  double *Bm = job.Bm[dir] + (size_t)c * TS_CHUNK * TS_CHUNK;
  int *Be = job.Be[dir] + (size_t)c * TS_CHUNK * TS_CHUNK;
  Bm[lane * TS_CHUNK + s] = lane >= s ? bm : 0.0;
  Be[lane * TS_CHUNK + s] = lane >= s ? be : 0;
}

// m 2^e for 0 <= m < 4 (a product of normalised mantissas) and e <= 1021:
// one multiplication by a power of two built from its bit pattern, a second
// one below the normal range (results under 2^-1074 round to zero)
__device__ inline double ext_val(double m, int e) {
  if (e < -1021) {
    if (e < -1130) return 0.0;
    m *= 0x1p-200;
    e += 200;
  }
  return m * __longlong_as_double((long long)(e + 1023) << 52);
}

// gradient of the two springs at bead (ja, la) towards (jn, ln) and (jp, lp):
// m w2 (x - x_n) + m w2 (x - x_p), md_pimd_x.c:2344-2367
template <int D>
__device__ inline void grad2(Geo g, const double *x, double mw2, int ja, int la, int jn, int ln,
                             int jp, int lp, int image, double *gr) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const double xa = x[sidx(ja, d, la, D, g.Ns)];
    double a = xa - x[sidx(jn, d, ln, D, g.Ns)];
    double c = xa - x[sidx(jp, d, lp, D, g.Ns)];
    if (image) {
      a = min_image(a, g.box[d], g.inv_box[d]);
      c = min_image(c, g.box[d], g.inv_box[d]);
    }
    gr[d] = mw2 * a + mw2 * c;
  }
}

constexpr int EX_TY = 8;

__device__ inline double trap_f(const TrapPrm &p, int d, double xv) {
  if (p.kind == TRAP_HARMONIC) return -p.w * p.w * (xv - p.c[d]);
  if (p.kind == TRAP_NEG_HARMONIC) return -(-p.w * p.w * (xv - p.c[d]));
  return -p.w2[d] * p.w2[d] * (xv - p.c[d]);
}

// a column's nx and its largest kept |nz| share the int4's x field
__host__ __device__ inline int col_nx(const int4 &c) { return c.x & 255; }
__host__ __device__ inline int col_nz(const int4 &c) { return c.x >> 8; }

struct Kahan {
  float s = 0.f, c = 0.f;
  __device__ inline void add(float v) {
    const float y = v - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ inline double value() const { return (double)s - (double)c; }
};

// double-float accumulator: hi + lo with error-free TwoSum per addition
struct DF {
  float hi = 0.f, lo = 0.f;
  __device__ inline void add(float v) {
    const float s = hi + v;
    const float bp = s - hi;
    const float e = (hi - (s - bp)) + (v - bp);
    hi = s;
    lo += e;
  }
  __device__ inline double value() const { return (double)hi + (double)lo; }
};

// Real-space images farther than EW32_XCUT / alpha are left out of the FP32
// form: there h(x) = erfc(x) + 2x exp(-x^2)/sqrt(pi) < 1e-5, and for the
// electron gas at alpha L = 5.6 the dropped images change the largest force
// component by 4e-8 of itself (against 2e-12 at 4.6 and the FP32 form's own
// 6e-6 from rounding the positions), while the images per pair fall from
// 2.32 to 1.11.
constexpr float EW32_XCUT = 3.6f;

// h(alpha R) / R^3 in FP32 without tables: h(x) = exp(-x^2) (2x/sqrt(pi) +
// erfcx(x)), erfcx(x) ~ t P(t), t = 1/(1 + x/2) (fit in xmd_ewald_tables.h,
// relative error 2e-8 on [0, 4.7]); 1/R from rsqrt, exp from ex2
__device__ __forceinline__ float ew_h32(float R2, float alpha) {
  const float cc[EW32_DEG + 1] = EW32_ERFCX_INIT;
  const float ri = rsqrtf(R2);
  const float x = alpha * (R2 * ri);
  const float t = __fdividef(1.f, fmaf((float)EW32_C, x, 1.f));
  float q = cc[EW32_DEG];
#pragma unroll
  for (int k = EW32_DEG - 1; k >= 0; --k) q = fmaf(q, t, cc[k]);
  const float e = __expf(-x * x);
  return e * fmaf(x, 1.1283791670955126f, q * t) * (ri * ri * ri);
}

// constants of the FP32 pair kernel, prepared on the host so that the
// kernel issues no FP64 instruction (on GB300 the FP64 pipe is 58x slower
// and also serves conversions and divisions of doubles)
struct P32 {
  float L[3], iL[3];
  float igs2, gpre;  // Gaussian: 1/s^2 and (g / (pi s^2)) (2 / s^2)
  float qs;          // Coulomb / Ewald strength
  float alpha, rc2;  // Ewald: splitting, FP32 cut-off squared
  int kmax;          // Ewald: 0 = 8-image search, else |k_d| <= kmax
  int nsum;          // Ewald: the reference's image cube |n_d| <= nsum
  int uniform;       // all beads of the system have one mass (1/m = im0)
  float im0;
};

// the FP32 pair kernel's constants for a system and potential (host)
P32 make_p32(const Geo &g, const PairPrm &p);

template <int D, int KIND>
__device__ inline void pair_eval32(const P32 &q, const float *dx, float *F) {
  if (KIND == PAIR_GAUSSIAN || KIND == PAIR_PERIODIC_GAUSSIAN) {
    float t[D], r2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      t[d] = dx[d];
      if (KIND == PAIR_PERIODIC_GAUSSIAN) t[d] = t[d] - q.L[d] * rintf(t[d] * q.iL[d]);
      r2 = fmaf(t[d], t[d], r2);
    }
    const float mult = q.gpre * __expf(-r2 * q.igs2);
#pragma unroll
    for (int d = 0; d < D; ++d) F[d] = mult * t[d];
  } else if (KIND == PAIR_COULOMB || KIND == PAIR_PERIODIC_COULOMB) {
    float t[D], r2 = 0.f;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      t[d] = dx[d];
      if (KIND == PAIR_PERIODIC_COULOMB) t[d] = t[d] - q.L[d] * rintf(t[d] * q.iL[d]);
      r2 = fmaf(t[d], t[d], r2);
    }
    const float ri = rsqrtf(r2);
    const float mult = q.qs * ri * ri * ri;
#pragma unroll
    for (int d = 0; d < D; ++d) F[d] = mult * t[d];
  } else if (KIND == PAIR_EWALD_REAL) {
    // Minimum image m = dx - r L (r = rint(dx/L)); images t = m - k L.
    // Images beyond rc32 (alpha rc32 <= EW32_XCUT) are left out.  When rc32
    // is at most the smallest box length only the 8 images with k_d in
    // {0, sign(m_d)} can lie inside it (any other has a component of length
    // >= L); otherwise all 27 with |k_d| <= kmax are tried.  The reference's
    // cube |r_d + k_d| <= nsum matters only for nsum < 2.
    float m[3], sg[3], r[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      r[d] = rintf(dx[d] * q.iL[d]);
      m[d] = fmaf(-r[d], q.L[d], dx[d]);
      sg[d] = m[d] < 0.f ? -1.f : 1.f;
    }
    const float ns = (float)q.nsum;
    float F0 = 0.f, F1 = 0.f, F2 = 0.f;
    if (q.kmax == 0) {
      // With a_d = |m_d| the shifted component has length L_d - a_d, so an
      // image's squared distance is |m|^2 plus dl_d = L_d (L_d - 2 a_d) for
      // each shifted axis: the 8 candidates are tested with a few adds.  The
      // accepted ones (2.3 per pair on average at alpha L = 5.6) are then
      // evaluated lowest bit first, so the warp runs as many rounds as its
      // busiest lane has images instead of one round per candidate.
      const float R0 = fmaf(m[2], m[2], fmaf(m[1], m[1], m[0] * m[0]));
      float dl[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) dl[d] = q.L[d] * fmaf(-2.f, fabsf(m[d]), q.L[d]);
      unsigned mask = 0u;
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const float R2 = R0 + ((c & 1) ? dl[0] : 0.f) + ((c & 2) ? dl[1] : 0.f) + ((c & 4) ? dl[2] : 0.f);
        bool ok = R2 < q.rc2;
        if (q.nsum < 2)
          ok = ok && fabsf(r[0] + ((c & 1) ? sg[0] : 0.f)) <= ns && fabsf(r[1] + ((c & 2) ? sg[1] : 0.f)) <= ns &&
               fabsf(r[2] + ((c & 4) ? sg[2] : 0.f)) <= ns;
        mask |= ok ? 1u << c : 0u;
      }
      while (mask) {
        const int c = __ffs(mask) - 1;
        mask &= mask - 1;
        const float t0 = (c & 1) ? fmaf(-sg[0], q.L[0], m[0]) : m[0];
        const float t1 = (c & 2) ? fmaf(-sg[1], q.L[1], m[1]) : m[1];
        const float t2 = (c & 4) ? fmaf(-sg[2], q.L[2], m[2]) : m[2];
        const float R2 = fmaf(t2, t2, fmaf(t1, t1, t0 * t0));
        const float mult = ew_h32(R2, q.alpha);
        F0 = fmaf(t0, mult, F0);
        F1 = fmaf(t1, mult, F1);
        F2 = fmaf(t2, mult, F2);
      }
    } else {
      for (int k0 = -q.kmax; k0 <= q.kmax; ++k0) {
        const float f0 = (float)k0;
        if (fabsf(r[0] + f0) > ns) continue;
        const float t0 = fmaf(-f0, q.L[0], m[0]);
        for (int k1 = -q.kmax; k1 <= q.kmax; ++k1) {
          const float f1 = (float)k1;
          if (fabsf(r[1] + f1) > ns) continue;
          const float t1 = fmaf(-f1, q.L[1], m[1]);
          for (int k2 = -q.kmax; k2 <= q.kmax; ++k2) {
            const float f2 = (float)k2;
            if (fabsf(r[2] + f2) > ns) continue;
            const float t2 = fmaf(-f2, q.L[2], m[2]);
            const float R2 = fmaf(t2, t2, fmaf(t1, t1, t0 * t0));
            if (R2 >= q.rc2) continue;
            const float mult = ew_h32(R2, q.alpha);
            F0 = fmaf(t0, mult, F0);
            F1 = fmaf(t1, mult, F1);
            F2 = fmaf(t2, mult, F2);
          }
        }
      }
    }
    F[0] = q.qs * F0;
    if (D > 1) F[1] = q.qs * F1;
    if (D > 2) F[2] = q.qs * F2;
  }
}

__device__ inline float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}


// the solve's job for weight scratch rs_f / rs_b (rec_scratch_doubles(N)
// each) and outputs VBN / tmpV (host)
TriJob tri_job(int N, double *rs_f, double *rs_b, double *VBN, double *tmpV);

// The block solve of direction `backward` by the calling thread block (any
// whole number of warps; rows of a chunk go round-robin over the warps, each
// row's sums inside one warp, so the result does not depend on the count).
// sh: (8 + 4) (N + 1 + 2 TS_CHUNK + 2 TS_CHUNK TS_LD) bytes of shared memory.
__device__ inline void tri_solve_b_dev(int N, double beta, const TriJob &job, int backward, double *sh) {
  const double *__restrict__ Mm = job.Mm[backward];
  const int *__restrict__ Me = job.Me[backward];
  const double *__restrict__ Bgm = job.Bm[backward];
  const int *__restrict__ Bge = job.Be[backward];
  double *__restrict__ out = job.out[backward];
  double *Um = sh;                          // [TS_CHUNK][TS_LD] next chunk vs the chunk before it
  double *Bsm = Um + TS_CHUNK * TS_LD;      // [TS_CHUNK][TS_LD] the chunk's B block
  double *Pm = Bsm + TS_CHUNK * TS_LD;      // [TS_CHUNK] sums over the unknowns before the previous chunk
  double *Rm = Pm + TS_CHUNK;               // [TS_CHUNK] right-hand sides of the chunk
  double *Xm = Rm + TS_CHUNK;               // N+1
  int *Ue = (int *)(Xm + N + 1);            // [TS_CHUNK][TS_LD]
  int *Bse = Ue + TS_CHUNK * TS_LD;         // [TS_CHUNK][TS_LD]
  int *Pe = Bse + TS_CHUNK * TS_LD;         // [TS_CHUNK]
  int *Re = Pe + TS_CHUNK;                  // [TS_CHUNK]
  int *Xe = Re + TS_CHUNK;                  // N+1
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // stage chunk n0's B block and its rows' weights against columns c0..c0+31
  auto stage = [&](int n0, int c0) {
    const int cc = (n0 - 1) / TS_CHUNK;
    for (int q = threadIdx.x; q < 2 * TS_CHUNK * TS_CHUNK; q += blockDim.x) {
      const int which = q / (TS_CHUNK * TS_CHUNK), rs = q % (TS_CHUNK * TS_CHUNK);
      const int r = rs / TS_CHUNK, k = rs % TS_CHUNK, i = n0 + r;
      const size_t o = (size_t)r * TS_LD + k;
      if (which == 0) {
        const bool in = i <= N && c0 >= 0;
        Um[o] = in ? Mm[moff(i, c0 + k)] : 0.0;
        Ue[o] = in ? Me[moff(i, c0 + k)] : 0;
      } else {
        Bsm[o] = i <= N ? Bgm[(size_t)cc * TS_CHUNK * TS_CHUNK + rs] : 0.0;
        Bse[o] = i <= N ? Bge[(size_t)cc * TS_CHUNK * TS_CHUNK + rs] : 0;
      }
    }
  };
  if (threadIdx.x == 0) {
    Xm[0] = 0.5;
    Xe[0] = 1;
  }
  stage(1, -1);
  __syncthreads();
  // chunk 0: its rows against column 0 (X_0 = 1)
  for (int r = w; r < TS_CHUNK; r += nw) {
    const int i = 1 + r;
    double am = 0.0;
    int E = 0;
    if (i <= N) ext_dot(Mm + moff(i, 0), Me + moff(i, 0), Xm, Xe, 0, 1, lane, am, E);
    if (lane == 0) {
      double pm = 0.0;
      int pe = 0;
      if (i <= N) ext_acc(pm, pe, am, E);
      Pm[r] = pm;
      Pe[r] = pe;
    }
  }
  __syncthreads();
  for (int i0 = 1, c = 0; i0 <= N; i0 += TS_CHUNK, ++c) {
    // U: right-hand sides
    for (int r = w; r < TS_CHUNK; r += nw) {
      if (i0 + r > N) continue;  // warp-uniform
      double pm = Pm[r];
      int pe = Pe[r];
      if (c > 0) {
        const int col = i0 - TS_CHUNK + lane;
        const size_t o = (size_t)r * TS_LD + lane;
        const double mv = Um[o];
        const bool nz = __double_as_longlong(mv) != 0 && __double_as_longlong(Xm[col]) != 0;
        double sm;
        int se;
        ext_warp_sum(nz, mv * Xm[col], Ue[o] + Xe[col], sm, se);
        if (lane == 0 && se != EXT_NONE) ext_acc(pm, pe, sm, se);
      }
      if (lane == 0) {
        norm2(pm, pe);
        Rm[r] = pm;
        Re[r] = pe;
      }
    }
    __syncthreads();
    // B: the chunk's unknowns
    for (int r = w; r < TS_CHUNK; r += nw) {
      const int i = i0 + r;
      if (i > N) continue;  // warp-uniform
      const size_t o = (size_t)r * TS_LD + lane;
      const double bv = Bsm[o], rv = Rm[lane];
      const bool nz = lane <= r && __double_as_longlong(bv) != 0 && __double_as_longlong(rv) != 0;
      double sm;
      int se;
      ext_warp_sum(nz, bv * rv, Bse[o] + Re[lane], sm, se);
      if (lane == 0) {
        double xm = se == EXT_NONE ? 0.0 : sm;
        int xe = se == EXT_NONE ? 0 : se;
        norm2(xm, xe);
        Xm[i] = xm;
        Xe[i] = xe;
      }
    }
    __syncthreads();
    // next chunk: its weights against this chunk, its B block, and its rows'
    // sums over the unknowns before this chunk
    const int n0 = i0 + TS_CHUNK;
    if (n0 <= N) {
      stage(n0, i0);
      for (int r = w; r < TS_CHUNK; r += nw) {
        const int i = n0 + r;
        if (i > N) break;  // warp-uniform; later rows are out of range too
        double am;
        int E;
        ext_dot(Mm + moff(i, 0), Me + moff(i, 0), Xm, Xe, 0, i0, lane, am, E);
        if (lane == 0) {
          double pm = 0.0;
          int pe = 0;
          ext_acc(pm, pe, am, E);
          Pm[r] = pm;
          Pe[r] = pe;
        }
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x + 1; i <= N; i += blockDim.x) {
    const double lnx = log(fabs(Xm[i])) + Xe[i] * LN2_HI + Xe[i] * LN2_LO;
    out[backward ? N - i : i] = -lnx / beta;
  }
  if (threadIdx.x == 0) out[backward ? N : 0] = 0.0;
  if (job.Xm[backward])
    for (int i = threadIdx.x; i <= N; i += blockDim.x) {
      job.Xm[backward][i] = Xm[i];
      job.Xe[backward][i] = Xe[i];
    }
}


// particle l's interior springs, E_l^(1) and the increment gl[l]: one warp
template <int D>
__device__ inline void eint_particle(const Geo &g, const double *__restrict__ x, const double *__restrict__ m,
                                     double w2, int image, double *Eint, double *ENk, double *gl, int l, int lane) {
  double res = 0;
  for (int j = lane; j + 1 < g.P; j += 32)
    res += 0.5 * m[(size_t)j * g.Ns + l] * w2 * spring2<D>(g, x, j, l, j + 1, l, image);
  res = warp_sum(res);
  // lane 0: the closing spring of l (E_l^(1)); lane 1: the link to l+1 (the
  // increment of the prefix sums), both in one pass
  if (lane < 2) {
    const int b = lane == 0 ? l : (l + 1 < g.N ? l + 1 : l);
    const double lk = link<D>(g, x, m, w2, l, b, image);
    if (lane == 0) {
      Eint[l] = res;
      ENk[dtri(l + 1)] = res + lk;
    } else if (l + 1 < g.N) {
      gl[l] = res + lk;
    }
  }
}

// E_l^(k) (1-based row l, cycle length k >= 2) from the prefix sums G
template <int D>
__device__ inline void enk_entry(const Geo &g, const double *__restrict__ x, const double *__restrict__ m, double w2,
                                 int image, const double *__restrict__ Eint, const double *G, double *__restrict__ ENk,
                                 int l, int k) {
  ENk[dtri(l) + k - 1] = Eint[l - 1] + ((G[l - 1] - G[l - k]) + link<D>(g, x, m, w2, l - 1, l - k, image));
}

// the ring springs' force on interior bead j (1..P-2) of particle l, as the
// acceleration the step stores in f: the reference divides the gradient
// m w2 (2x - x_n - x_p) (md_pimd_x.c:2344-2367) by the bead's mass m, which
// cancels, so w2 (x - x_n) + w2 (x - x_p) is taken directly (equal to
// rounding; no FP64 division, the GPU's slowest FP64 operation)
template <int D>
__device__ inline void spring_interior_bead(const Geo &g, const double *__restrict__ x,
                                            const double *__restrict__ m, double w2, int image,
                                            double *__restrict__ f, int j, int l) {
  (void)m;
  double gr[D];
  grad2<D>(g, x, w2, j, l, j + 1, l, j - 1, l, image, gr);
#pragma unroll
  for (int d = 0; d < D; ++d) f[sidx(j, d, l, D, g.Ns)] += -gr[d];
}

// X'_{N-l} / X_N of row l (1-based) of G, as a mantissa q and an exponent qe
__device__ inline void g_ext_row(int N, const double *__restrict__ Xfm, const int *__restrict__ Xfe,
                                 const double *__restrict__ Xbm, const int *__restrict__ Xbe, int l, double &q,
                                 int &qe) {
  q = Xbm[N - l] / Xfm[N];
  qe = Xbe[N - l] - Xfe[N];
}

// G[l][j] (1-based) from the extended-range weights and unknowns, the row's
// factor (q, qe) from g_ext_row
__device__ inline void g_ext_elem(int N, const double *__restrict__ Mm, const int *__restrict__ Me,
                                  const double *__restrict__ Xfm, const int *__restrict__ Xfe, double q, int qe,
                                  double *__restrict__ G, int l, int j) {
  double gv;
  if (j > l + 1) {
    gv = 0;
  } else if (j == l + 1) {
    gv = 1 - ext_val(Xfm[l] * q, Xfe[l] + qe);
  } else {
    const size_t o = moff(l, j - 1);
    const double w = Mm[o];
    gv = w == 0.0 ? 0.0 : ext_val(w * Xfm[j - 1] * q, Me[o] + Xfe[j - 1] + qe);
  }
  G[(size_t)(l - 1) * N + (j - 1)] = gv;
}

// FP32 phase factors e^{2 pi i n x/L}, n = 0..ns, of slot t (D = 3 layout)
__device__ inline void phase32_slot(const Geo &g, int ns, const double *__restrict__ x, float2 *__restrict__ ph32,
                                    size_t t) {
  const int l = (int)(t % g.Ns);
  const int jd = (int)(t / g.Ns);  // j*3 + d
  const int d = jd % 3;
  float s1 = 0.f, c1 = 1.f;
  if (l < g.N) {
    double u = x[t] * g.inv_box[d];
    u -= rint(u);  // in [-1/2, 1/2]
    sincospif((float)(2.0 * u), &s1, &c1);
  }
  float re = 1.f, im = 0.f;
  float2 *o = ph32 + (size_t)jd * (ns + 1) * g.Ns + l;
  o[0] = make_float2(1.f, 0.f);
  for (int n = 1; n <= ns; ++n) {
    const float r2 = fmaf(re, c1, -im * s1), i2 = fmaf(re, s1, im * c1);
    re = r2;
    im = i2;
    o[(size_t)n * g.Ns] = make_float2(re, im);
  }
}

// entry n (0..ns) of column ci's FP32 force table of slice j, in FP32
// from the FP32 structure factors S and coefficients coef32
__device__ inline void recip_table32_entry(const int4 *__restrict__ cols, int ncol, const float2 *__restrict__ S,
                                           const float *__restrict__ coef32, int nk, float2 *__restrict__ T, int ns,
                                           int j, int ci, int n) {
  const int NT = 4 * ns + 1;
  const int4 c = cols[ci];
  auto W = [&](int nz) {
    if (nz < c.z) return make_float2(0.f, 0.f);
    const int k = c.w + (nz - c.z);
    const float2 s = S[(size_t)j * nk + k];
    return make_float2(coef32[k] * s.x, -coef32[k] * s.y);
  };
  float2 *o = T + ((size_t)j * ncol + ci) * NT;
  if (n == 0) {
    o[0] = W(0);
  } else {
    const float2 wp = W(n), wm = W(-n);
    const float Ar = wp.x + wm.x, Ai = wp.y + wm.y, Br = wp.x - wm.x, Bi = wp.y - wm.y;
    const float fn = (float)n;
    o[4 * n - 3] = make_float2(Ar, Ai);
    o[4 * n - 2] = make_float2(Br, Bi);
    o[4 * n - 1] = make_float2(fn * Ar, fn * Ai);
    o[4 * n] = make_float2(fn * Br, fn * Bi);
  }
}

// tile job wi (slice wi / jobs, tile pair I <= J) of the FP32 pair forces,
// one warp: per-tile sums into out (see k_pair_tiles32)
template <int D, int KIND>
__device__ inline void pair_tile32_job(const Geo &g, const P32 &q, const float *__restrict__ x,
                                       const float *__restrict__ im, float *__restrict__ out, int T, int jobs, int wi,
                                       int lane) {
  const int j = wi / jobs;
  int job = wi % jobs, I = 0;
  while (job >= T - I) {
    job -= T - I;
    ++I;
  }
  const int J = I + job;
  const int a = I * 32 + lane, b0 = J * 32 + lane;
  const bool va = a < g.N, vb = b0 < g.N;
  float xa[D], xb[D], fa[D], fb[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    xa[d] = va ? x[sidx(j, d, a, D, g.Ns)] : 0.f;
    xb[d] = vb ? x[sidx(j, d, b0, D, g.Ns)] : 0.f;
    fa[d] = fb[d] = 0.f;
  }
  const int src = (lane + 1) & 31;
  if (q.uniform) {
    for (int s = 0; s < 32; ++s) {
      const int bi = J * 32 + ((lane + s) & 31);
      if (va && bi < g.N && (I != J || a > bi)) {
        float dx[D], F[D];
#pragma unroll
        for (int d = 0; d < D; ++d) dx[d] = xa[d] - xb[d];
        pair_eval32<D, KIND>(q, dx, F);
#pragma unroll
        for (int d = 0; d < D; ++d) {
          fa[d] += F[d];
          fb[d] -= F[d];
        }
      }
#pragma unroll
      for (int d = 0; d < D; ++d) {
        xb[d] = __shfl_sync(FULL, xb[d], src);
        fb[d] = __shfl_sync(FULL, fb[d], src);
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      fa[d] *= q.im0;
      fb[d] *= q.im0;
    }
  } else {
    const float ima = va ? im[(size_t)j * g.Ns + a] : 1.f;
    float imb = vb ? im[(size_t)j * g.Ns + b0] : 1.f;
    for (int s = 0; s < 32; ++s) {
      const int bi = J * 32 + ((lane + s) & 31);
      if (va && bi < g.N && (I != J || a > bi)) {
        float dx[D], F[D];
#pragma unroll
        for (int d = 0; d < D; ++d) dx[d] = xa[d] - xb[d];
        pair_eval32<D, KIND>(q, dx, F);
        // the reference divides by the mass of the higher-index particle
        const float inv = a > bi ? ima : imb;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          fa[d] = fmaf(F[d], inv, fa[d]);
          fb[d] = fmaf(-F[d], inv, fb[d]);
        }
      }
#pragma unroll
      for (int d = 0; d < D; ++d) {
        xb[d] = __shfl_sync(FULL, xb[d], src);
        fb[d] = __shfl_sync(FULL, fb[d], src);
      }
      imb = __shfl_sync(FULL, imb, src);
    }
  }
  if (I == J) {
    if (va) {
#pragma unroll
      for (int d = 0; d < D; ++d) out[(((size_t)I * g.P + j) * D + d) * g.Ns + a] = fa[d] + fb[d];
    }
  } else {
    if (va) {
#pragma unroll
      for (int d = 0; d < D; ++d) out[(((size_t)J * g.P + j) * D + d) * g.Ns + a] = fa[d];
    }
    if (vb) {
#pragma unroll
      for (int d = 0; d < D; ++d) out[(((size_t)I * g.P + j) * D + d) * g.Ns + b0] = fb[d];
    }
  }
}

// the exchange spring forces on the end beads of particles bx*32 .. +31
// from partners js*EX_TY + ty + k nsplit EX_TY: one 32 x EX_TY thread
// block (tx, ty), red: EX_TY * 2D * 32 doubles of shared memory
template <int D>
__device__ inline void exch_ends_block(const Geo &g, const double *__restrict__ x, const double *__restrict__ m,
                                       double w2, int image, const double *__restrict__ G,
                                       double *__restrict__ scratch, int nsplit, int bx, int js, int tx, int ty,
                                       double *red) {
  const int l = bx * 32 + tx;
  const int N = g.N, jP = g.P - 1;
  double a1[D], aP[D];
#pragma unroll
  for (int d = 0; d < D; ++d) a1[d] = aP[d] = 0;
  if (l < N) {
    const double m1 = m[l], mP = m[(size_t)jP * g.Ns + l];
    // The reference adds G-weighted gradients of both springs at the end
    // bead for every partner q; the spring inside the ring (bead 1 -> 2,
    // bead P -> P-1) does not depend on q, so it is weighted once by the sum
    // of the weights and only the partner spring is evaluated per q (equal
    // to rounding).
    double x1[D], xP[D], s1 = 0.0, sP = 0.0;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      x1[d] = x[sidx(0, d, l, D, g.Ns)];
      xP[d] = x[sidx(jP, d, l, D, g.Ns)];
    }
    // partner q runs over this block's part of 0..N-1
    for (int q = js * EX_TY + ty; q < N; q += nsplit * EX_TY) {
      // bead 1 of l, previous bead = bead P of q, weight G[q][l]
      const double g1 = G[(size_t)q * N + l];
      if (g1 != 0.0) {
        s1 += g1;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double c = x1[d] - x[sidx(jP, d, q, D, g.Ns)];
          if (image) c = min_image(c, g.box[d], g.inv_box[d]);
          a1[d] = fma(g1, c, a1[d]);
        }
      }
      // bead P of l, next bead = bead 1 of q, weight G[l][q]
      const double gP = G[(size_t)l * N + q];
      if (gP != 0.0) {
        sP += gP;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          double c = xP[d] - x[sidx(0, d, q, D, g.Ns)];
          if (image) c = min_image(c, g.box[d], g.inv_box[d]);
          aP[d] = fma(gP, c, aP[d]);
        }
      }
    }
    const double k1 = m1 * w2, kP = mP * w2;
#pragma unroll
    for (int d = 0; d < D; ++d) {
      double a = x1[d] - x[sidx(1, d, l, D, g.Ns)];
      double b = xP[d] - x[sidx(jP - 1, d, l, D, g.Ns)];
      if (image) {
        a = min_image(a, g.box[d], g.inv_box[d]);
        b = min_image(b, g.box[d], g.inv_box[d]);
      }
      a1[d] = k1 * (s1 * a + a1[d]);
      aP[d] = kP * (sP * b + aP[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    red[(ty * 2 * D + d) * 32 + tx] = a1[d];
    red[(ty * 2 * D + D + d) * 32 + tx] = aP[d];
  }
  __syncthreads();
  if (ty == 0 && l < N) {
#pragma unroll
    for (int q = 0; q < 2 * D; ++q) {
      double s = 0;
      for (int y = 0; y < EX_TY; ++y) s += red[(y * 2 * D + q) * 32 + tx];
      scratch[((size_t)js * 2 * D + q) * g.Ns + l] = s;
    }
  }
}

// ---- FP32 structure factors (mixed form) --------------------------------
// An item is one kept wave-vector column (nx, ny) and SK_NG harmonics
// nz = n0+1 .. n0+SK_NG (and nz = 0 when n0 = 0) of one bead slice.  The
// particles' phase products are summed in FP32 over SK_PB particles at a
// time, and each partial sum is added into double-float accumulators: the FP32
// partial of at most 16 unit-size terms carries an error of ~1e-7 of a
// term, the size of the FP32 phase factors' own rounding, at a sixth of
// the arithmetic of a double-float addition per particle.
constexpr int SK_NG = 4;   // harmonics per item
constexpr int SK_PB = 16;  // particles per FP32 partial sum

struct SkAcc {
  DF s0r, s0i, P[SK_NG][2], Q[SK_NG][2];
};

// the item's sums over the staged particles 0 .. cnt-1 of a chunk (sp:
// [3][ns+1][stride] phase factors; stride padded so that rows fall in
// different banks): thread g of gr sharing the item takes particles
// b + g, b + g + gr, ... (SK_PB of them) of each block b of SK_PB * gr
// consecutive particles, blocks b0, b0 + SK_PB gr, ... (one thread: every
// block of SK_PB particles in order)
__device__ inline void sk_item_blocks(SkAcc &A, const float2 *__restrict__ sp, int stride, int ns, int ax, int ay,
                                      bool cy, int n0, int cnt, int g, int gr) {
  for (int b = 0; b < cnt; b += SK_PB * gr) {
    float s0r = 0.f, s0i = 0.f, p[SK_NG][2], q[SK_NG][2];
#pragma unroll
    for (int u = 0; u < SK_NG; ++u) p[u][0] = p[u][1] = q[u][0] = q[u][1] = 0.f;
    for (int k = 0; k < SK_PB; ++k) {
      const int l = b + g + k * gr;
      if (l >= cnt) break;
      float2 ey = sp[((ns + 1) + ay) * stride + l];
      if (cy) ey.y = -ey.y;
      const float2 exy = cmulf(sp[ax * stride + l], ey);
      s0r += exy.x;
      s0i += exy.y;
#pragma unroll
      for (int u = 0; u < SK_NG; ++u) {
        const int n = n0 + u + 1;
        if (n > ns) break;
        const float2 ez = sp[(2 * (ns + 1) + n) * stride + l];
        p[u][0] = fmaf(exy.x, ez.x, p[u][0]);
        p[u][1] = fmaf(exy.y, ez.x, p[u][1]);
        q[u][0] = fmaf(exy.x, ez.y, q[u][0]);
        q[u][1] = fmaf(exy.y, ez.y, q[u][1]);
      }
    }
    if (n0 == 0) {
      A.s0r.add(s0r);
      A.s0i.add(s0i);
    }
#pragma unroll
    for (int u = 0; u < SK_NG; ++u) {
      if (n0 + u + 1 > ns) break;
      A.P[u][0].add(p[u][0]);
      A.P[u][1].add(p[u][1]);
      A.Q[u][0].add(q[u][0]);
      A.Q[u][1].add(q[u][1]);
    }
  }
}

// a + b and a - b of two double-float values, rounded to FP32 (TwoSum of
// the high parts, the low parts added to its error)
__device__ inline float df_sum(const DF &a, const DF &b) {
  const float s = a.hi + b.hi, bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (b.hi - bp);
  return s + ((e + a.lo) + b.lo);
}
__device__ inline float df_diff(const DF &a, const DF &b) {
  const float s = a.hi - b.hi, bp = s - a.hi;
  const float e = (a.hi - (s - bp)) + (-b.hi - bp);
  return s + ((e + a.lo) - b.lo);
}

// S(k) of the item's wave vectors in FP32 (the FP32 force tables are all
// that reads it): Sj is the slice's row S + j nk
__device__ inline void sk_item_store(const SkAcc &A, float2 *Sj, int4 c, int ns, int n0) {
  float2 *o = Sj + c.w - c.z;
  if (n0 == 0 && c.z <= 0) o[0] = make_float2(A.s0r.hi + A.s0r.lo, A.s0i.hi + A.s0i.lo);
#pragma unroll
  for (int u = 0; u < SK_NG; ++u) {
    const int n = n0 + u + 1;
    if (n > ns) break;
    const DF &Pr = A.P[u][0], &Pi = A.P[u][1], &Qr = A.Q[u][0], &Qi = A.Q[u][1];
    o[n] = make_float2(df_diff(Pr, Qi), df_sum(Pi, Qr));
    if (c.z < 0) o[-n] = make_float2(df_sum(Pr, Qi), df_diff(Pi, Qr));
  }
}

constexpr int RF_PB = 128;  // particles per block of the FP32 reciprocal forces (two threads each)

// One particle's reciprocal force sums over cc kept columns (k_recip_force32's
// arithmetic): cols and the columns' FP32 force tables sT (4 ns + 1 entries
// each) in shared memory, the particle's x and y phase factors at
// pxy[(d (ns+1) + n) * stride + li] (shared), its z factors in ez[1..ns]
template <int NSM>
__device__ inline void recip_cols32(Kahan &Fx, Kahan &Fy, Kahan &Fz, const int4 *__restrict__ cols, int cc,
                                    const float2 *__restrict__ sT, int ns, const float2 *__restrict__ pxy, int stride,
                                    int li, const float2 *ez) {
  const int NT = 4 * ns + 1;
  for (int ci = 0; ci < cc; ++ci) {
    const int4 c = cols[ci];
    const int nzc = col_nz(c);
    float2 ey = pxy[((ns + 1) + (c.y < 0 ? -c.y : c.y)) * stride + li];
    if (c.y < 0) ey.y = -ey.y;
    const float2 exy = cmulf(pxy[col_nx(c) * stride + li], ey);
    const float2 *t = sT + ci * NT;
    float Ur = t[0].x, Ui = t[0].y, Vr = 0.f, Vi = 0.f;
#pragma unroll
    for (int n = 1; n <= NSM; ++n) {
      if (n > ns || n > nzc) break;
      const float2 A = t[4 * n - 3], B = t[4 * n - 2], nA = t[4 * n - 1], nB = t[4 * n];
      const float cz = ez[n].x, sz = ez[n].y;
      Ur = fmaf(cz, A.x, fmaf(-sz, B.y, Ur));
      Ui = fmaf(cz, A.y, fmaf(sz, B.x, Ui));
      Vr = fmaf(cz, nB.x, fmaf(-sz, nA.y, Vr));
      Vi = fmaf(cz, nB.y, fmaf(sz, nA.x, Vi));
    }
    const float Tm = fmaf(exy.x, Ui, exy.y * Ur);
    const float Zm = fmaf(exy.x, Vi, exy.y * Vr);
    Fx.add((float)col_nx(c) * Tm);
    Fy.add((float)c.y * Tm);
    Fz.add(Zm);
  }
}

}  // namespace xk

