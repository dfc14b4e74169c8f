// xmd_ensemble.cu -- the persistent ensemble step: independent ring-polymer
// systems of uneven N and P advanced by one kernel launch per step.
//
// The fictitious-particle method needs many (xi, beta) systems to
// extrapolate to xi = -1; each is small (N <= 128 beads per slice in the
// benchmark ensemble) and one system's step is a chain of a dozen dependent
// stages, so as separate kernels the systems leave most of the GPU idle
// between launches.  Here one launch runs every stage of every system:
// clusters of thread blocks take the systems of a list the host balanced
// by estimated cost (longest first, each to the least loaded cluster), and
// a cluster runs its systems one after the other.  Inside a system the
// stages are separated by cluster barriers (barrier.cluster, with the
// release / acquire ordering of the cluster's memory operations); there is
// no wait on another cluster, so no spin loop exists anywhere.
//
// Every stage uses the arithmetic of the per-system kernels through the same
// device functions (xmd_device.cuh), in the same summation orders: the
// thermostat half steps, the cycle energies, the weights and block inverses
// of the exchange recursions and their block solve, the cycle probabilities
// G, the exchange spring forces, the FP32 pair tiles and their FP64
// finishing sums, and the FP32 Ewald reciprocal sums (structure factors
// per column in double-float, force tables, Kahan-compensated forces).
// The forces add up in the order of the per-system calls (trap, reciprocal,
// real space; the exchange forces with the second half step), so one
// persistent step reproduces one step of the per-system calls.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "xmd_device.cuh"
#include "xmd_kernels.cuh"

namespace xk {

namespace cg = cooperative_groups;

constexpr int ENS_T = 256;                // threads per block
constexpr int ENS_W = ENS_T / 32;         // warps per block (the EX_TY rows of the end-bead block)
constexpr size_t ENS_SMEM = 64 * 1024;    // dynamic shared memory per block
constexpr int ENS_SKC = 128;              // particles per staged chunk of phase factors
constexpr int ENS_NG = 4;                 // harmonics n per structure-factor item
constexpr int ENS_NSMAX = 11;             // largest Ewald n_sum
static_assert(ENS_W == EX_TY, "the end-bead block is 32 x EX_TY threads");

struct EnsSys {
  EnsSysDesc d;
  TriJob job;
  P32 q;
  int T, jobs, nsplit;
  int ewald;  // reciprocal sums present (D = 3)
  int ns, ncol, nk;
  const int4 *cols;
  const double *coef;
  float2 *ph32, *T32;
  double2 *S;
  float *part, *x32;
  double lnvi, rscale, pscale;
};

// one FP32 pair tile job of the system's potential kind
template <int D>
__device__ inline void ens_pair_job(const EnsSys &E, int wi, int lane) {
  const Geo &g = E.d.g;
  switch (E.d.pair_kind) {
    case PAIR_GAUSSIAN:
      pair_tile32_job<D, PAIR_GAUSSIAN>(g, E.q, E.x32, nullptr, E.part, E.T, E.jobs, wi, lane);
      break;
    case PAIR_PERIODIC_GAUSSIAN:
      pair_tile32_job<D, PAIR_PERIODIC_GAUSSIAN>(g, E.q, E.x32, nullptr, E.part, E.T, E.jobs, wi, lane);
      break;
    case PAIR_COULOMB:
      pair_tile32_job<D, PAIR_COULOMB>(g, E.q, E.x32, nullptr, E.part, E.T, E.jobs, wi, lane);
      break;
    case PAIR_PERIODIC_COULOMB:
      pair_tile32_job<D, PAIR_PERIODIC_COULOMB>(g, E.q, E.x32, nullptr, E.part, E.T, E.jobs, wi, lane);
      break;
    default:
      if constexpr (D == 3) pair_tile32_job<3, PAIR_EWALD_REAL>(g, E.q, E.x32, nullptr, E.part, E.T, E.jobs, wi, lane);
      break;
  }
}

// Structure factors of bead slice j by the calling block.  Items are (kept
// column, group of ENS_NG harmonics); each thread sums its item over the
// slice's particles in order, as k_sk32 does per column, with the particles'
// phase factors staged in shared memory ENS_SKC at a time.
__device__ inline void ens_sk_slice(const EnsSys &E, int j, float2 *sp) {
  const Geo &g = E.d.g;
  const int ns = E.ns, N = g.N, tid = threadIdx.x;
  const int ngr = (ns + ENS_NG - 1) / ENS_NG;
  const int items = E.ncol * ngr;
  const float2 *base = E.ph32 + (size_t)j * 3 * (ns + 1) * g.Ns;
  const int rows = 3 * (ns + 1);
  for (int b0 = 0; b0 < items; b0 += ENS_T) {
    const int item = b0 + tid;
    const bool live = item < items;
    const int ci = live ? item / ngr : 0, gi = live ? item % ngr : 0;
    const int4 c = live ? E.cols[ci] : make_int4(0, 0, 1, 0);
    const int ax = col_nx(c), ay = c.y < 0 ? -c.y : c.y;
    const bool cy = c.y < 0;
    const int n0 = gi * ENS_NG;
    DF s0r, s0i, Pa[ENS_NG][2], Qa[ENS_NG][2];
    for (int l0 = 0; l0 < N; l0 += ENS_SKC) {
      const int cnt = N - l0 < ENS_SKC ? N - l0 : ENS_SKC;
      __syncthreads();
      for (int q = tid; q < rows * ENS_SKC; q += ENS_T) {
        const int l = q % ENS_SKC, row = q / ENS_SKC;
        sp[q] = l < cnt ? base[(size_t)row * g.Ns + l0 + l] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      if (!live) continue;
      for (int l = 0; l < cnt; ++l) {
        float2 ey = sp[((ns + 1) + ay) * ENS_SKC + l];
        if (cy) ey.y = -ey.y;
        const float2 exy = cmulf(sp[ax * ENS_SKC + l], ey);
        if (gi == 0) {
          s0r.add(exy.x);
          s0i.add(exy.y);
        }
#pragma unroll
        for (int u = 0; u < ENS_NG; ++u) {
          const int n = n0 + u + 1;
          if (n > ns) break;
          const float2 ez = sp[(2 * (ns + 1) + n) * ENS_SKC + l];
          Pa[u][0].add(exy.x * ez.x);
          Pa[u][1].add(exy.y * ez.x);
          Qa[u][0].add(exy.x * ez.y);
          Qa[u][1].add(exy.y * ez.y);
        }
      }
    }
    if (!live) continue;
    double2 *o = E.S + (size_t)j * E.nk + c.w - c.z;
    if (gi == 0 && c.z <= 0) o[0] = make_double2(s0r.value(), s0i.value());
#pragma unroll
    for (int u = 0; u < ENS_NG; ++u) {
      const int n = n0 + u + 1;
      if (n > ns) break;
      const double Pr = Pa[u][0].value(), Pi = Pa[u][1].value();
      const double Qr = Qa[u][0].value(), Qi = Qa[u][1].value();
      o[n] = make_double2(Pr - Qi, Pi + Qr);
      if (c.z < 0) o[-n] = make_double2(Pr + Qi, Pi - Qr);
    }
  }
}

// Reciprocal forces on the particles of bead slice j by the calling block,
// as k_recip_force32 computes them (the same column order and compensated
// sums), the slice's force tables staged in shared memory as many columns
// at a time as fit.
__device__ inline void ens_recip_slice(const EnsSys &E, int j, float2 *sT) {
  const Geo &g = E.d.g;
  const int ns = E.ns, NT = 4 * ns + 1, ncol = E.ncol, N = g.N, tid = threadIdx.x;
  const int ccap = (int)(ENS_SMEM / (sizeof(float2) * NT));
  const float2 *Tj = E.T32 + (size_t)j * ncol * NT;
  for (int lb = 0; lb < N; lb += ENS_T) {
    const int l = lb + tid;
    const bool live = l < N;
    const float2 *pj = E.ph32 + (size_t)j * 3 * (ns + 1) * g.Ns + (live ? l : 0);
    float2 ez[ENS_NSMAX + 1];
#pragma unroll
    for (int n = 1; n <= ENS_NSMAX; ++n)
      ez[n] = (live && n <= ns) ? pj[((size_t)2 * (ns + 1) + n) * g.Ns] : make_float2(0.f, 0.f);
    Kahan Fx, Fy, Fz;
    for (int c0 = 0; c0 < ncol; c0 += ccap) {
      const int cc = ncol - c0 < ccap ? ncol - c0 : ccap;
      __syncthreads();
      for (int q = tid; q < cc * NT; q += ENS_T) sT[q] = Tj[(size_t)c0 * NT + q];
      __syncthreads();
      if (!live) continue;
      for (int ci = 0; ci < cc; ++ci) {
        const int4 c = E.cols[c0 + ci];
        const int nzc = col_nz(c);
        float2 ey = pj[((size_t)(ns + 1) + (c.y < 0 ? -c.y : c.y)) * g.Ns];
        if (c.y < 0) ey.y = -ey.y;
        const float2 exy = cmulf(pj[(size_t)col_nx(c) * g.Ns], ey);
        const float2 *t = sT + ci * NT;
        float Ur = t[0].x, Ui = t[0].y, Vr = 0.f, Vi = 0.f;
#pragma unroll
        for (int n = 1; n <= ENS_NSMAX; ++n) {
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
    if (live) {
      double *f = E.d.f;
      f[sidx(j, 0, l, 3, g.Ns)] += E.rscale * Fx.value() * g.inv_box[0];
      f[sidx(j, 1, l, 3, g.Ns)] += E.rscale * Fy.value() * g.inv_box[1];
      f[sidx(j, 2, l, 3, g.Ns)] += E.rscale * Fz.value() * g.inv_box[2];
    }
  }
}

// The step of every system in the clusters' lists.  Grid: clusters of CL
// blocks of ENS_T threads; cluster k runs systems list[off[k] .. off[k+1]).
template <int D, int L>
__global__ void __launch_bounds__(ENS_T, 2) k_ensemble_step(const EnsSys *__restrict__ sys,
                                                            const int *__restrict__ list,
                                                            const int *__restrict__ off) {
  cg::cluster_group cl = cg::this_cluster();
  const int CL = (int)cl.num_blocks();
  const int cr = (int)cl.block_rank();
  const int cid = blockIdx.x / CL;
  extern __shared__ __align__(16) unsigned char ens_sh[];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const int gt = cr * ENS_T + tid, GT = CL * ENS_T;
  const int gw = cr * ENS_W + w, GW = CL * ENS_W;
  for (int it = off[cid]; it < off[cid + 1]; ++it) {
    const EnsSys &E = sys[list[it]];
    const EnsSysDesc &d = E.d;
    const Geo g = d.g;
    const size_t Sn = g.slots();
    const int N = g.N, P = g.P;

    // A: first half step (md_update_nhc_VV3_1_x); the forces restart from
    // the trap's (md_reset_force_x, md_pimd_calc_trap_force_x); FP32
    // positions and phase factors of the new positions
    for (size_t s = gt; s < Sn; s += GT) {
      const int l = (int)(s % g.Ns);
      if (l >= N) continue;
      nhc_slot<D, L>(g, 1, s, l, d.x, d.v, d.f, nullptr, d.m, d.th, d.vt, d.Q, d.iQ, d.kT, d.h);
      const double xn = d.x[s];
      double f0 = 0.0;
      if (d.trap_kind) f0 += trap_f(d.tp, (int)((s / g.Ns) % D), xn) / P;
      d.f[s] = f0;
      d.fex[s] = 0.0;
      if (d.pair_kind) E.x32[s] = (float)xn;
      if constexpr (D == 3)
        if (E.ewald) phase32_slot(g, E.ns, d.x, E.ph32, s);
    }
    cl.sync();

    // B: E_l^(1) and the prefix-sum increments (md_pimd_fast_fill_ENk_x),
    // interior ring springs into fex, FP32 pair tiles, structure factors
    for (int l = gw; l < N; l += GW) eint_particle<D>(g, d.x, d.m, d.w2, d.image, d.Eint, d.ENk, d.gl, l, lane);
    if (P > 2) {
      const size_t n2 = (size_t)(P - 2) * g.Ns;
      for (size_t t = gt; t < n2; t += GT) {
        const int l = (int)(t % g.Ns), j = (int)(t / g.Ns) + 1;
        if (l < N) spring_interior_bead<D>(g, d.x, d.m, d.w2, d.image, d.fex, j, l);
      }
    }
    if (d.pair_kind) {
      const int nj = E.jobs * P;
      for (int wi = gw; wi < nj; wi += GW) ens_pair_job<D>(E, wi, lane);
    }
    if constexpr (D == 3)
      if (E.ewald)
        for (int j = cr; j < P; j += CL) ens_sk_slice(E, j, (float2 *)ens_sh);
    cl.sync();

    // C: the remaining cycle energies E_l^(k), k >= 2, from each block's own
    // prefix sums; the FP32 force tables of the reciprocal sum
    if (N >= 2) {
      double *Gs = (double *)ens_sh;
      block_exclusive_prefix(d.gl, N - 1, Gs);
      __syncthreads();
      const size_t ne = (size_t)N * (N - 1) / 2;
      for (size_t q = gt; q < ne; q += GT) {
        // rows r = l - 1 = 1 .. N-1 hold r entries each, r (r - 1) / 2 before row r
        int r = (int)((1.f + sqrtf(1.f + 8.f * (float)q)) * 0.5f);
        while ((size_t)r * (r - 1) / 2 > q) --r;
        while ((size_t)r * (r + 1) / 2 <= q) ++r;
        const int k = 2 + (int)(q - (size_t)r * (r - 1) / 2);
        enk_entry<D>(g, d.x, d.m, d.w2, d.image, d.Eint, Gs, d.ENk, r + 1, k);
      }
    }
    if constexpr (D == 3)
      if (E.ewald) {
        const int per = E.ns + 1;
        const size_t nt = (size_t)P * E.ncol * per;
        for (size_t q = gt; q < nt; q += GT) {
          const int n = (int)(q % per);
          const size_t r = q / per;
          recip_table32_entry(E.cols, E.ncol, E.S, E.coef, E.nk, E.T32, E.ns, (int)(r / E.ncol), (int)(r % E.ncol),
                              n);
        }
      }
    cl.sync();

    // D: weight rows of both recursions and the diagonal-block inverses
    // (md_pimd_fill_VB_x); reciprocal forces
    for (int row = gw + 1; row <= N; row += GW)
      weights_row(N, d.beta, d.vi, E.lnvi, d.ENk, d.lnn, (double *)E.job.Mm[0], (int *)E.job.Me[0],
                  (double *)E.job.Mm[1], (int *)E.job.Me[1], 0, 1, 1, row, 0, lane, 32);
    {
      const int nch = (N + TS_CHUNK - 1) / TS_CHUNK;
      double(*Am)[TS_LD] = (double(*)[TS_LD])ens_sh;
      int(*Ae)[TS_LD] = (int(*)[TS_LD])(ens_sh + sizeof(double) * TS_CHUNK * TS_LD);
      for (int tk = cr; tk < 2 * nch; tk += CL) {
        const int dir = tk / nch, c = tk % nch, i0 = 1 + c * TS_CHUNK;
        __syncthreads();
        for (int e = tid; e < TS_CHUNK * TS_CHUNK; e += ENS_T) {
          const int r = e / TS_CHUNK, t = e % TS_CHUNK;
          Ext wv{0.0, 0};
          if (t < r && i0 + r <= N) wv = weight_at(N, d.beta, d.vi, E.lnvi, d.ENk, d.lnn, dir, i0 + r, i0 + t);
          Am[r][t] = wv.m;
          Ae[r][t] = wv.e;
        }
        __syncthreads();
        for (int sc = w; sc < TS_CHUNK; sc += ENS_W) block_inv_column(N, E.job, dir, c, sc, Am, Ae);
      }
    }
    if constexpr (D == 3)
      if (E.ewald)
        for (int j = cr; j < P; j += CL) ens_recip_slice(E, j, (float2 *)ens_sh);
    cl.sync();

    // E: the forward (V_B) and backward (tmpV) solves on blocks 0 and 1 (block
    // 0 alone: one after the other); the pair tiles' partial sums into f on
    // the other blocks
    if (cr == 0) tri_solve_b_dev(N, d.beta, E.job, 0, (double *)ens_sh);
    if (cr == (CL > 1 ? 1 : 0)) {
      if (CL == 1) __syncthreads();
      tri_solve_b_dev(N, d.beta, E.job, 1, (double *)ens_sh);
    }
    if (d.pair_kind) {
      const int b0 = CL > 2 ? 2 : 0, nb = CL > 2 ? CL - 2 : CL;
      if (cr >= b0)
        for (size_t s = (size_t)(cr - b0) * ENS_T + tid; s < Sn; s += (size_t)nb * ENS_T) {
          if ((int)(s % g.Ns) >= N) continue;
          double acc = 0;
          for (int t = 0; t < E.T; ++t) acc += (double)E.part[(size_t)t * Sn + s];
          d.f[s] += acc * E.pscale;
        }
    }
    cl.sync();

    // F: cycle probabilities G from the extended-range numbers
    // (md_pimd_fast_fill_force_VB_x)
    for (size_t q = gt; q < (size_t)N * N; q += GT)
      g_ext_elem(N, E.job.Mm[0], E.job.Me[0], E.job.Xm[0], E.job.Xe[0], E.job.Xm[1], E.job.Xe[1], d.G,
                 (int)(q / N) + 1, (int)(q % N) + 1);
    cl.sync();

    // G: G-weighted springs of the end beads, partial sums per partner split
    {
      const int tiles = (N + 31) / 32, ntask = tiles * E.nsplit;
      for (int tk = cr; tk < ntask; tk += CL) {
        exch_ends_block<D>(g, d.x, d.m, d.w2, d.image, d.G, d.xscr, E.nsplit, tk % tiles, tk / tiles, lane, w,
                           (double *)ens_sh);
        __syncthreads();
      }
    }
    cl.sync();

    // H: the end beads' exchange forces into fex, the second half step with
    // f + fex (md_update_nhc_VV3_2_x), the periodic wrap
    for (size_t s = gt; s < Sn; s += GT) {
      const int l = (int)(s % g.Ns);
      if (l >= N) continue;
      const int jd = (int)(s / g.Ns), j = jd / D, dd = jd % D;
      if (j == 0 || j == P - 1) {
        const int qq = (j == P - 1 ? D : 0) + dd;
        double sum = 0;
        for (int js = 0; js < E.nsplit; ++js) sum += d.xscr[((size_t)js * 2 * D + qq) * g.Ns + l];
        d.fex[s] += -sum / d.m[(size_t)j * g.Ns + l];
      }
      nhc_slot<D, L>(g, 2, s, l, d.x, d.v, d.f, d.fex, d.m, d.th, d.vt, d.Q, d.iQ, d.kT, d.h);
      if (d.wrap) {
        const double Lb = g.box[dd];
        double a = d.x[s];
        if (a < 0)
          a += Lb;
        else if (a > Lb)
          a -= Lb;
        d.x[s] = a;
      }
    }
  }
}

// ---- host side ----------------------------------------------------------

using EnsFn = void (*)(const EnsSys *, const int *, const int *);

static EnsFn ens_kernel(int D, int L) {
  switch (D * 16 + L) {
    case 1 * 16 + 4: return k_ensemble_step<1, 4>;
    case 1 * 16 + 8: return k_ensemble_step<1, 8>;
    case 2 * 16 + 4: return k_ensemble_step<2, 4>;
    case 2 * 16 + 8: return k_ensemble_step<2, 8>;
    case 3 * 16 + 4: return k_ensemble_step<3, 4>;
    case 3 * 16 + 8: return k_ensemble_step<3, 8>;
    default: return nullptr;
  }
}

static cudaError_t ens_opt_in(EnsFn fn) {
  static std::mutex mu;
  static std::vector<EnsFn> done;
  std::lock_guard<std::mutex> lk(mu);
  if (std::find(done.begin(), done.end(), fn) != done.end()) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ENS_SMEM);
  if (e != cudaSuccess) return e;
  done.push_back(fn);
  return cudaSuccess;
}

static void ens_config(int cluster, int clusters, cudaStream_t st, cudaLaunchConfig_t &cfg,
                       cudaLaunchAttribute &attr) {
  memset(&cfg, 0, sizeof(cfg));
  memset(&attr, 0, sizeof(attr));
  cfg.gridDim = dim3((unsigned)(cluster * clusters), 1, 1);
  cfg.blockDim = dim3(ENS_T, 1, 1);
  cfg.dynamicSmemBytes = ENS_SMEM;
  cfg.stream = st;
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = (unsigned)cluster;
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
}

int ensemble_resident_clusters(int D, int L, int cluster) {
  if (cluster != 1 && cluster != 2 && cluster != 4 && cluster != 8) return 0;
  EnsFn fn = ens_kernel(D, L);
  if (!fn || ens_opt_in(fn) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr;
  ens_config(cluster, 1, nullptr, cfg, attr);
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// estimated cost of one system's step (arbitrary units: pair-image
// evaluations, structure-factor products, recursion entries, barriers)
static double ens_cost(const EnsSys &E) {
  const Geo &g = E.d.g;
  double c = 2.0e4 + 40.0 * (double)g.N * g.N + 60.0 * (double)g.P * g.N;
  if (E.d.pair_kind) c += (double)E.jobs * 1024.0 * g.P * (E.d.pair_kind == PAIR_EWALD_REAL ? 3.0 : 1.0);
  if (E.ewald) c += 1.2 * (double)g.P * g.N * E.ncol * (E.ns + 1);
  return c;
}

cudaError_t ensemble_prepare(const EnsSysDesc *sd, int n, int D, int L, int cluster, EnsLaunch &out) {
  if (n < 1 || !ens_kernel(D, L)) return cudaErrorInvalidValue;
  const int resident = ensemble_resident_clusters(D, L, cluster);
  if (resident < 1) return cudaErrorInvalidConfiguration;
  std::vector<EnsSys> sys(n);
  for (int i = 0; i < n; ++i) {
    EnsSys &E = sys[i];
    memset(&E, 0, sizeof(E));
    E.d = sd[i];
    const Geo &g = E.d.g;
    if (g.D != D || g.N < 1 || g.N > ENS_MAX_N || g.P < 2) return cudaErrorInvalidValue;
    E.job = tri_job(g.N, E.d.rs_f, E.d.rs_b, E.d.VBN, E.d.tmpV);
    E.nsplit = (int)(exch_scratch_doubles(g) / ((size_t)2 * g.D * g.Ns));
    E.T = (g.N + 31) / 32;
    E.jobs = E.T * (E.T + 1) / 2;
    if (E.d.pair_kind) E.q = make_p32(g, E.d.pp);
    E.ewald = E.d.pair_kind == PAIR_EWALD_REAL && D == 3;
    if (E.ewald) {
      const Recip &r = E.d.rc;
      if (r.nsum < 1 || r.nsum > ENS_NSMAX) return cudaErrorInvalidValue;
      E.ns = r.nsum;
      E.ncol = r.ncol;
      E.nk = r.nk;
      E.cols = (const int4 *)r.kvec;
      E.coef = r.coef;
      E.ph32 = (float2 *)(r.phase + recip_phase_doubles(g, r.nsum));
      E.T32 = (float2 *)r.T;
      E.S = (double2 *)r.S;
      E.rscale = 4 * M_PI * E.d.inv_mP;
    }
    E.lnvi = E.d.vi != 0.0 ? log(E.d.vi) : 0.0;
    E.pscale = 1.0 / g.P;
  }
  // longest first, each to the least loaded of the resident clusters
  const int K = n < resident ? n : resident;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) cost[i] = ens_cost(sys[i]);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  std::vector<std::vector<int>> lists(K);
  std::vector<double> load(K, 0.0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lists[k].push_back(i);
    load[k] += cost[i];
  }
  std::vector<int> flat, off(K + 1, 0);
  for (int k = 0; k < K; ++k) {
    flat.insert(flat.end(), lists[k].begin(), lists[k].end());
    off[k + 1] = (int)flat.size();
  }
  // the FP32 pair scratch (tile partials, then the FP32 positions) of every
  // system lives in the plan itself, so that no later call can move it
  const size_t head = (sizeof(EnsSys) * n + sizeof(int) * (flat.size() + off.size()) + 255) & ~(size_t)255;
  std::vector<size_t> at(n, 0);
  size_t bytes = head;
  for (int i = 0; i < n; ++i) {
    if (!sys[i].d.pair_kind) continue;
    at[i] = bytes;
    bytes += (sizeof(float) * ((size_t)sys[i].T + 1) * sys[i].d.g.slots() + 255) & ~(size_t)255;
  }
  void *plan = nullptr;
  cudaError_t e = cudaMalloc(&plan, bytes);
  if (e != cudaSuccess) return e;
  for (int i = 0; i < n; ++i) {
    if (!sys[i].d.pair_kind) continue;
    sys[i].part = (float *)((unsigned char *)plan + at[i]);
    sys[i].x32 = sys[i].part + (size_t)sys[i].T * sys[i].d.g.slots();
  }
  std::vector<unsigned char> host(head);
  memcpy(host.data(), sys.data(), sizeof(EnsSys) * n);
  memcpy(host.data() + sizeof(EnsSys) * n, flat.data(), sizeof(int) * flat.size());
  memcpy(host.data() + sizeof(EnsSys) * n + sizeof(int) * flat.size(), off.data(), sizeof(int) * off.size());
  e = cudaMemcpy(plan, host.data(), head, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(plan);
    return e;
  }
  ensemble_free(out);
  out.plan = plan;
  out.D = D;
  out.L = L;
  out.cluster = cluster;
  out.clusters = K;
  out.nsys = n;
  out.smem = ENS_SMEM;
  return cudaSuccess;
}

cudaError_t ensemble_launch(const EnsLaunch &e, cudaStream_t st) {
  EnsFn fn = ens_kernel(e.D, e.L);
  if (!fn || !e.plan) return cudaErrorInvalidValue;
  cudaError_t oe = ens_opt_in(fn);
  if (oe != cudaSuccess) return oe;
  const EnsSys *sys = (const EnsSys *)e.plan;
  const int *list = (const int *)(sys + e.nsys);
  const int *off = list + e.nsys;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr;
  ens_config(e.cluster, e.clusters, st, cfg, attr);
  {
    XK_PROF("ensemble_step");
    oe = cudaLaunchKernelEx(&cfg, fn, sys, list, off);
  }
  if (oe != cudaSuccess) return oe;
  return XK_LAUNCHED();
}

void ensemble_free(EnsLaunch &e) {
  if (e.plan) cudaFree(e.plan);
  e = EnsLaunch{};
}

}  // namespace xk
