// xmd_ensemble.cu -- the persistent ensemble step: independent ring-polymer
// systems of uneven N and P advanced by one kernel launch per step.
//
// The fictitious-particle method needs many (xi, beta) systems to
// extrapolate to xi = -1; each is small (N <= 128 beads per slice in the
// benchmark ensemble) and one system's step is a chain of a dozen dependent
// stages, so as separate kernels the systems keep the GPU's launch path
// busy with about a thousand small kernels a step.  Here one launch runs
// every stage of every system: the step is nine phases, each phase holds the
// work of ALL systems for that stage (spread over every thread, warp or
// block of the grid, round-robin over the systems' tasks), and the phases
// are separated by grid barriers.  The grid is exactly the blocks that fit
// (a cooperative launch), and each barrier wait is bounded.
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

constexpr int ENS_T = 256;                // threads per block
constexpr int ENS_W = ENS_T / 32;         // warps per block (the EX_TY rows of the end-bead block)
constexpr size_t ENS_SMEM = 64 * 1024;    // dynamic shared memory per block
constexpr int ENS_SKC = 128;              // particles per staged chunk of phase factors
constexpr int ENS_NSMAX = 11;             // largest Ewald n_sum
constexpr long long ENS_WAIT_LIMIT = 1LL << 31;  // clock cycles a grid-barrier wait may take (~1 s)
static_assert(ENS_W == EX_TY, "the end-bead block is 32 x EX_TY threads");
static_assert(ENS_SKC % SK_PB == 0, "staged chunks hold whole particle blocks");

struct EnsSys {
  EnsSysDesc d;
  TriJob job;
  P32 q;
  int T, jobs, nsplit;
  int ewald;  // reciprocal sums present (D = 3)
  int ns, ncol, nk;
  const int4 *cols;
  const float *coef32;
  float2 *ph32, *T32;
  float2 *S;
  float *part, *x32;
  double lnvi, rscale, pscale;
  int rot[16];  // per task kind: (the kind's tasks before this system) mod (workers of that kind)
};

// task kinds of the step's phases (threads, warps or blocks, as noted)
enum {
  R_A,       // thread: first half step per slot
  R_B_SPR,   // thread: interior springs
  R_B_EINT,  // warp: E_l^(1) per particle (the pair tiles continue its numbering)
  R_B_PAIR,  // warp: FP32 pair tile jobs
  R_B_SK,    // block: structure factors per slice
  R_C_PRE,   // block: prefix sums per system
  R_C_TAB,   // thread: force-table entries
  R_D_ENK,   // thread: cycle energies E_l^(k), k >= 2
  R_D_REC,   // block: reciprocal forces per slice
  R_E_W,     // warp: weight rows
  R_E_PS,    // thread: pair sums per slot
  R_E_INV,   // block: diagonal-block inverses
  R_F,       // block: solves
  R_G,       // thread: G entries
  R_H,       // block: end-bead exchange forces
  R_I,       // thread: second half step per slot
  ENS_NROT
};
static_assert(ENS_NROT == 16, "EnsSys::rot holds every task kind");

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

// Structure factors of bead slice j by the calling block: one thread per
// item (kept column, SK_NG harmonics), every particle block in order, as
// k_sk32 with one thread per item computes them; the particles' phase
// factors staged in shared memory ENS_SKC at a time.
__device__ inline void ens_sk_slice(const EnsSys &E, int j, float2 *sp) {
  const Geo &g = E.d.g;
  const int ns = E.ns, N = g.N, tid = threadIdx.x;
  const int ngr = (ns + SK_NG - 1) / SK_NG;
  const int items = E.ncol * ngr;
  const float2 *base = E.ph32 + (size_t)j * 3 * (ns + 1) * g.Ns;
  const int rows = 3 * (ns + 1);
  for (int b0 = 0; b0 < items; b0 += ENS_T) {
    const int item = b0 + tid;
    const bool live = item < items;
    const int ci = live ? item / ngr : 0, n0 = live ? (item % ngr) * SK_NG : 0;
    const int4 c = live ? E.cols[ci] : make_int4(0, 0, 1, 0);
    const int ax = col_nx(c), ay = c.y < 0 ? -c.y : c.y;
    const bool cy = c.y < 0;
    SkAcc A;
    for (int l0 = 0; l0 < N; l0 += ENS_SKC) {
      const int cnt = N - l0 < ENS_SKC ? N - l0 : ENS_SKC;
      __syncthreads();
      for (int q = tid; q < rows * ENS_SKC; q += ENS_T) {
        const int l = q % ENS_SKC, row = q / ENS_SKC;
        sp[row * (ENS_SKC + 1) + l] = l < cnt ? base[(size_t)row * g.Ns + l0 + l] : make_float2(0.f, 0.f);
      }
      __syncthreads();
      if (live) sk_item_blocks(A, sp, ENS_SKC + 1, ns, ax, ay, cy, n0, cnt, 0, 1);
    }
    if (live) sk_item_store(A, E.S + (size_t)j * E.nk, c, ns, n0);
  }
}

// Reciprocal forces on the particles of bead slice j by the calling block,
// as k_recip_force32 computes them (two threads per particle, each summing
// its half of the columns in order with recip_cols32, the halves added in
// double), 128 particles at a time; the columns, the particles' x and y
// phase factors and as many columns' force tables as fit are staged in
// shared memory.
__device__ inline void ens_recip_slice(const EnsSys &E, int j, unsigned char *sh) {
  const Geo &g = E.d.g;
  const int ns = E.ns, NT = 4 * ns + 1, ncol = E.ncol, N = g.N, tid = threadIdx.x;
  int4 *sc = (int4 *)sh;
  float2 *pxy = (float2 *)(sc + ncol);
  float2 *sT = pxy + 2 * (ns + 1) * 128;
  const int ccap = (int)((ENS_SMEM - sizeof(int4) * ncol - sizeof(float2) * 2 * (ns + 1) * 128) / (sizeof(float2) * NT));
  const float2 *Tj = E.T32 + (size_t)j * ncol * NT;
  const float2 *pj = E.ph32 + (size_t)j * 3 * (ns + 1) * g.Ns;
  const int li = tid >> 1, h = tid & 1;
  const int half = (ncol + 1) / 2, ca = h ? half : 0, cb = h ? ncol : half;
  __syncthreads();
  for (int q = tid; q < ncol; q += ENS_T) sc[q] = E.cols[q];
  for (int lb = 0; lb < N; lb += 128) {
    const int l = lb + li;
    const bool live = l < N;
    __syncthreads();
    for (int q = tid; q < 2 * (ns + 1) * 128; q += ENS_T) {
      const int r = q / 128, lq = q % 128;
      pxy[q] = lb + lq < N ? pj[(size_t)r * g.Ns + lb + lq] : make_float2(0.f, 0.f);
    }
    float2 ez[ENS_NSMAX + 1];
#pragma unroll
    for (int n = 1; n <= ENS_NSMAX; ++n)
      ez[n] = (live && n <= ns) ? pj[((size_t)2 * (ns + 1) + n) * g.Ns + l] : make_float2(0.f, 0.f);
    Kahan Fx, Fy, Fz;
    for (int c0 = 0; c0 < ncol; c0 += ccap) {
      const int cc = ncol - c0 < ccap ? ncol - c0 : ccap;
      __syncthreads();
      for (int q = tid; q < cc * NT; q += ENS_T) sT[q] = Tj[(size_t)c0 * NT + q];
      __syncthreads();
      const int a = ca > c0 ? ca : c0, b = cb < c0 + cc ? cb : c0 + cc;
      if (live && a < b) recip_cols32<ENS_NSMAX>(Fx, Fy, Fz, sc + a, b - a, sT + (size_t)(a - c0) * NT, ns, pxy, 128, li, ez);
    }
    double fx = Fx.value(), fy = Fy.value(), fz = Fz.value();
    fx += __shfl_xor_sync(FULL, fx, 1);
    fy += __shfl_xor_sync(FULL, fy, 1);
    fz += __shfl_xor_sync(FULL, fz, 1);
    if (live && !h) {
      double *f = E.d.f;
      f[sidx(j, 0, l, 3, g.Ns)] += E.rscale * fx * g.inv_box[0];
      f[sidx(j, 1, l, 3, g.Ns)] += E.rscale * fy * g.inv_box[1];
      f[sidx(j, 2, l, 3, g.Ns)] += E.rscale * fz * g.inv_box[2];
    }
  }
}

// ---- grid barrier ----------------------------------------------------------
// The phases of the step are separated by a barrier over the whole grid
// (every block is resident: the grid is the number of blocks that fit, and
// the launch is cooperative).  Block b's thread 0 arrives with an atomic
// increment; the last arrival resets the count and advances the generation
// the others wait on.  A wait gives up after `limit` clock cycles: it sets
// err, and every later barrier of any launch returns at once, so a broken
// grid ends instead of hanging; the host reads err as the step's status.
struct EnsBar {
  unsigned int count, gen;
  int err;
  int pad;
  unsigned long long stamp[ENS_PHASES + 1];  // block 0's %globaltimer at the start and after each phase
  unsigned long long sub[4];  // block 0 inside phase B: after its springs, E_l^(1), pair tiles, structure factors
  unsigned long long t0, t1;  // the group's first block: start and end of the step
};

// block 0's own time inside a phase (its threads synchronised first)
__device__ inline void ens_sub(EnsBar *b, int k) {
  if (blockIdx.x == 0) {
    __syncthreads();
    if (threadIdx.x == 0) {
      unsigned long long t;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
      b->sub[k] = t;
    }
  }
}

__device__ inline void ens_stamp(EnsBar *b, int k) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    b->stamp[k] = t;
  }
}

__device__ inline void ens_grid_sync(EnsBar *b, unsigned int nblocks, long long limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int *genp = &b->gen;
    volatile int *errp = &b->err;
    const unsigned int my = *genp;
    __threadfence();
    if (atomicAdd(&b->count, 1u) + 1u == nblocks) {
      atomicExch(&b->count, 0u);
      __threadfence();
      atomicAdd(&b->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*genp == my && !*errp) {
        if (clock64() - t0 > limit) {
          atomicExch(&b->err, 1);
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
}

// the first of a system's tasks that worker `me` (of `stride`) takes, the
// tasks of all systems numbered in turn and dealt round-robin; rot is the
// number of the kind's tasks before this system, modulo stride
__device__ inline long long ens_first(long long me, int rot, long long stride) {
  return me >= rot ? me - rot : me - rot + stride;
}

// One step of every system.  Each phase's work of ALL systems is spread over
// the whole grid (threads, warps or blocks, round-robin over the tasks of the
// systems in turn); the phases are separated by grid barriers.
template <int D, int L, int MINB>
__global__ void __launch_bounds__(ENS_T, MINB) k_ensemble_step(const EnsSys *__restrict__ sys,
                                                               const int *__restrict__ goff, int K, EnsBar *bars,
                                                               long long limit) {
  extern __shared__ __align__(16) unsigned char ens_sh[];
  // K groups of blocks (block b in group b mod K), each stepping its own
  // systems sys[goff[k] .. goff[k+1]) with its own barriers: the groups'
  // phases drift apart, so one group's FP64 thermostat runs beside another
  // group's FP32 sums on the same SMs
  const int grp = blockIdx.x % K;
  EnsBar *bar = bars + grp;
  if (*(volatile int *)&bar->err) return;  // an earlier step's barrier gave up
  const unsigned int G = gridDim.x / K;
  const int i0 = goff[grp], i1 = goff[grp + 1];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const long long rank = blockIdx.x / K;
  const long long GT = (long long)G * ENS_T, GW = (long long)G * ENS_W;
  const long long gt = rank * ENS_T + tid, gw = rank * ENS_W + w;
  const long long gb = rank;
  ens_stamp(bar, 0);
  if (rank == 0 && tid == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    bar->t0 = t;
  }

  // A: first half step (md_update_nhc_VV3_1_x); the forces restart from the
  // trap's (md_reset_force_x, md_pimd_calc_trap_force_x); FP32 positions and
  // phase factors of the new positions
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const EnsSysDesc &d = E.d;
      const Geo g = d.g;
      const long long n = (long long)g.slots();
      for (long long q = ens_first(gt, sys[i].rot[R_A], GT); q < n; q += GT) {
        const size_t s = (size_t)q;
        const int l = (int)(s % g.Ns);
        if (l >= g.N) continue;
        nhc_slot<D, L>(g, 1, s, l, d.x, d.v, d.f, nullptr, d.m, d.th, d.vt, d.Q, d.iQ, d.kT, d.h);
        const double xn = d.x[s];
        double f0 = 0.0;
        if (d.trap_kind) f0 += trap_f(d.tp, (int)((s / g.Ns) % D), xn) * E.pscale;
        d.f[s] = f0;
        d.fex[s] = 0.0;
        if (d.pair_kind) E.x32[s] = (float)xn;
        if constexpr (D == 3)
          if (E.ewald) phase32_slot(g, E.ns, d.x, E.ph32, s);
      }
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 1);

  // B: interior ring springs into fex; E_l^(1) and the prefix-sum increments
  // (md_pimd_fast_fill_ENk_x); FP32 pair tiles; structure factors
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSysDesc &d = sys[i].d;
      const Geo g = d.g;
      const long long n = g.P > 2 ? (long long)(g.P - 2) * g.Ns : 0;
      for (long long t = ens_first(gt, sys[i].rot[R_B_SPR], GT); t < n; t += GT) {
        const int l = (int)(t % g.Ns), j = (int)(t / g.Ns) + 1;
        if (l < g.N) spring_interior_bead<D>(g, d.x, d.m, d.w2, d.image, d.fex, j, l);
      }
    }
  }
  ens_sub(bar, 0);
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSysDesc &d = sys[i].d;
      const Geo g = d.g;
      for (long long l = ens_first(gw, sys[i].rot[R_B_EINT], GW); l < g.N; l += GW)
        eint_particle<D>(g, d.x, d.m, d.w2, d.image, d.Eint, d.ENk, d.gl, (int)l, lane);
    }
    ens_sub(bar, 1);
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      if (!E.d.pair_kind) continue;
      const long long n = (long long)E.jobs * E.d.g.P;
      for (long long wi = ens_first(gw, sys[i].rot[R_B_PAIR], GW); wi < n; wi += GW) ens_pair_job<D>(E, (int)wi, lane);
    }
  }
  ens_sub(bar, 2);
  if constexpr (D == 3) {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      if (!E.ewald) continue;
      for (long long j = ens_first(gb, sys[i].rot[R_B_SK], G); j < E.d.g.P; j += G) ens_sk_slice(E, (int)j, (float2 *)ens_sh);
    }
  }
  ens_sub(bar, 3);
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 2);

  // C: prefix sums of the increments (a block per system, the block size of
  // k_enk_direct's own scan, into gl[N ..]); the FP32 force tables
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSysDesc &d = sys[i].d;
      if (d.g.N < 2) continue;
      if (ens_first(gb, sys[i].rot[R_C_PRE], G) == 0) {
        block_exclusive_prefix(d.gl, d.g.N - 1, d.gl + d.g.N);
        __syncthreads();  // its scratch is reused by the block's next system
      }
    }
  }
  if constexpr (D == 3) {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      if (!E.ewald) continue;
      const int per = E.ns + 1;
      const long long n = (long long)E.d.g.P * E.ncol * per;
      for (long long q = ens_first(gt, sys[i].rot[R_C_TAB], GT); q < n; q += GT) {
        const long long r = q / per;
        recip_table32_entry(E.cols, E.ncol, E.S, E.coef32, E.nk, E.T32, E.ns, (int)(r / E.ncol), (int)(r % E.ncol),
                            (int)(q % per));
      }
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 3);

  // D: the cycle energies E_l^(k), k >= 2; reciprocal forces
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSysDesc &d = sys[i].d;
      const Geo g = d.g;
      const long long n = (long long)g.N * (g.N - 1) / 2;
      for (long long q = ens_first(gt, sys[i].rot[R_D_ENK], GT); q < n; q += GT) {
        // rows r = l - 1 = 1 .. N-1 hold r entries each, r (r - 1) / 2 before row r
        int r = (int)((1.f + sqrtf(1.f + 8.f * (float)q)) * 0.5f);
        while ((long long)r * (r - 1) / 2 > q) --r;
        while ((long long)r * (r + 1) / 2 <= q) ++r;
        const int k = 2 + (int)(q - (long long)r * (r - 1) / 2);
        enk_entry<D>(g, d.x, d.m, d.w2, d.image, d.Eint, d.gl + g.N, d.ENk, r + 1, k);
      }
    }
  }
  if constexpr (D == 3) {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      if (!E.ewald) continue;
      for (long long j = ens_first(gb, sys[i].rot[R_D_REC], G); j < E.d.g.P; j += G) ens_recip_slice(E, (int)j, ens_sh);
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 4);

  // E: weight rows of both recursions and the diagonal-block inverses
  // (md_pimd_fill_VB_x); the pair tiles' partial sums into f
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const EnsSysDesc &d = E.d;
      const int N = d.g.N;
      for (long long r = ens_first(gw, sys[i].rot[R_E_W], GW); r < N; r += GW)
        weights_row(N, d.beta, d.vi, E.lnvi, d.ENk, d.lnn, (double *)E.job.Mm[0], (int *)E.job.Me[0],
                    (double *)E.job.Mm[1], (int *)E.job.Me[1], 0, 1, 1, (int)r + 1, 0, lane, 32);
    }
  }
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      if (!E.d.pair_kind) continue;
      const Geo g = E.d.g;
      const long long n = (long long)g.slots();
      for (long long q = ens_first(gt, sys[i].rot[R_E_PS], GT); q < n; q += GT) {
        const size_t s = (size_t)q;
        if ((int)(s % g.Ns) >= g.N) continue;
        double acc = 0;
        for (int t = 0; t < E.T; ++t) acc += (double)E.part[(size_t)t * n + s];
        E.d.f[s] += acc * E.pscale;
      }
    }
  }
  {
    double(*Am)[TS_LD] = (double(*)[TS_LD])ens_sh;
    int(*Ae)[TS_LD] = (int(*)[TS_LD])(ens_sh + sizeof(double) * TS_CHUNK * TS_LD);
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const EnsSysDesc &d = E.d;
      const int N = d.g.N, nch = (N + TS_CHUNK - 1) / TS_CHUNK;
      for (long long tk = ens_first(gb, sys[i].rot[R_E_INV], G); tk < 2 * nch; tk += G) {
        const int dir = (int)tk / nch, c = (int)tk % nch, i0 = 1 + c * TS_CHUNK;
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
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 5);

  // F: the forward (V_B) and backward (tmpV) block solves, a block each
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      for (long long dir = ens_first(gb, sys[i].rot[R_F], G); dir < 2; dir += G) {
        __syncthreads();
        tri_solve_b_dev(E.d.g.N, E.d.beta, E.job, (int)dir, (double *)ens_sh);
      }
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 6);

  // G: cycle probabilities G from the extended-range numbers
  // (md_pimd_fast_fill_force_VB_x)
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const int N = E.d.g.N;
      const long long n = (long long)N * N;
      for (long long q = ens_first(gt, sys[i].rot[R_G], GT); q < n; q += GT) {
        const int l = (int)(q / N) + 1;
        double qf;
        int qe;
        g_ext_row(N, E.job.Xm[0], E.job.Xe[0], E.job.Xm[1], E.job.Xe[1], l, qf, qe);
        g_ext_elem(N, E.job.Mm[0], E.job.Me[0], E.job.Xm[0], E.job.Xe[0], qf, qe, E.d.G, l, (int)(q % N) + 1);
      }
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 7);

  // H: G-weighted springs of the end beads, partial sums per partner split
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const EnsSysDesc &d = E.d;
      const Geo g = d.g;
      const int tiles = (g.N + 31) / 32;
      const long long n = (long long)tiles * E.nsplit;
      for (long long tk = ens_first(gb, sys[i].rot[R_H], G); tk < n; tk += G) {
        exch_ends_block<D>(g, d.x, d.m, d.w2, d.image, d.G, d.xscr, E.nsplit, (int)(tk % tiles), (int)(tk / tiles),
                           lane, w, (double *)ens_sh);
        __syncthreads();
      }
    }
  }
  ens_grid_sync(bar, G, limit);
  ens_stamp(bar, 8);

  // I: the end beads' exchange forces into fex, the second half step with
  // f + fex (md_update_nhc_VV3_2_x), the periodic wrap
  {
    for (int i = i0; i < i1; ++i) {
      const EnsSys &E = sys[i];
      const EnsSysDesc &d = E.d;
      const Geo g = d.g;
      const long long n = (long long)g.slots();
      for (long long q = ens_first(gt, sys[i].rot[R_I], GT); q < n; q += GT) {
        const size_t s = (size_t)q;
        const int l = (int)(s % g.Ns);
        if (l >= g.N) continue;
        const int jd = (int)(s / g.Ns), j = jd / D, dd = jd % D;
        if (j == 0 || j == g.P - 1) {
          const int qq = (j == g.P - 1 ? D : 0) + dd;
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
  __syncthreads();
  ens_stamp(bar, ENS_PHASES);
  if (rank == 0 && tid == 0) {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    bar->t1 = t;
  }
}

// ---- host side ----------------------------------------------------------

using EnsFn = void (*)(const EnsSys *, const int *, int, EnsBar *, long long);

// the kernel compiled for 2 blocks per SM (128 registers) or 3 (80
// registers, some spilled to local memory)
static EnsFn ens_kernel(int D, int L, int bps) {
  const bool three = bps >= 3;
  switch (D * 16 + L) {
    case 1 * 16 + 4: return three ? k_ensemble_step<1, 4, 3> : k_ensemble_step<1, 4, 2>;
    case 1 * 16 + 8: return three ? k_ensemble_step<1, 8, 3> : k_ensemble_step<1, 8, 2>;
    case 2 * 16 + 4: return three ? k_ensemble_step<2, 4, 3> : k_ensemble_step<2, 4, 2>;
    case 2 * 16 + 8: return three ? k_ensemble_step<2, 8, 3> : k_ensemble_step<2, 8, 2>;
    case 3 * 16 + 4: return three ? k_ensemble_step<3, 4, 3> : k_ensemble_step<3, 4, 2>;
    case 3 * 16 + 8: return three ? k_ensemble_step<3, 8, 3> : k_ensemble_step<3, 8, 2>;
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

int ensemble_max_blocks_per_sm(int D, int L) {
  int best = 0;
  for (int bps : {2, 3}) {
    EnsFn fn = ens_kernel(D, L, bps);
    if (!fn || ens_opt_in(fn) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, ENS_T, ENS_SMEM) != cudaSuccess) {
      cudaGetLastError();
      continue;
    }
    if (n > best) best = n > 3 ? 3 : n;
  }
  return best;
}

static int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// estimated cost of a system's step in microseconds of one group of the
// benchmark's grid, for spreading the systems over the groups: a fixed part
// per system (its latency-bound tasks: prefix scan, solves, barriers' share)
// and the work that grows with the system (fitted to measured group times of
// the 64-system ensemble: the Ewald sums dominate, then the pair tiles)
static double ens_cost(const EnsSys &E) {
  const Geo &g = E.d.g;
  const double N = g.N, P = g.P, slots = (double)g.slots();
  double c = 30.0 + 1.0e-3 * slots + 1.0e-3 * N * N;
  if (E.d.pair_kind && !E.ewald) c += 1.2e-4 * (double)E.jobs * P * 1024.0;
  if (E.ewald) c += 4.0e-5 * P * N * E.ncol * (E.ns + 1);
  return c;
}

cudaError_t ensemble_prepare(const EnsSysDesc *sd, int n, int D, int L, int blocks_per_sm, int groups,
                             EnsLaunch &out, const double *costs) {
  if (n < 1 || !ens_kernel(D, L, 2) || groups < 1 || groups > ENS_MAX_GROUPS) return cudaErrorInvalidValue;
  const int fit = ensemble_max_blocks_per_sm(D, L);
  if (fit < 1 || blocks_per_sm < 1) return cudaErrorInvalidConfiguration;
  if (blocks_per_sm > fit) blocks_per_sm = fit;
  const int K = groups < n ? groups : n;
  const int blocks = (blocks_per_sm * sm_count()) / K * K;
  const long long Gk = blocks / K;
  std::vector<EnsSys> all(n);
  for (int i = 0; i < n; ++i) {
    EnsSys &E = all[i];
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
      E.coef32 = (const float *)(r.coef + r.nk);
      E.ph32 = (float2 *)(r.phase + recip_phase_doubles(g, r.nsum));
      E.T32 = (float2 *)r.T;
      E.S = (float2 *)r.S;
      E.rscale = 4 * M_PI * E.d.inv_mP;
    }
    E.lnvi = E.d.vi != 0.0 ? log(E.d.vi) : 0.0;
    E.pscale = 1.0 / g.P;
  }
  // longest first, each to the least loaded group; each group's systems
  // contiguous, its largest first (the round-robin of each phase then starts
  // with the longest tasks)
  std::vector<int> order(n);
  std::vector<double> cost(n);
  for (int i = 0; i < n; ++i) {
    order[i] = i;
    cost[i] = costs ? costs[i] : ens_cost(all[i]);
  }
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return cost[x] > cost[y]; });
  std::vector<std::vector<int>> lists(K);
  std::vector<double> load(K, 0.0);
  for (int i : order) {
    const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    lists[k].push_back(i);
    load[k] += cost[i];
  }
  std::vector<EnsSys> sys;
  std::vector<int> goff(K + 1, 0);
  for (int k = 0; k < K; ++k) {
    for (int i : lists[k]) sys.push_back(all[i]);
    goff[k + 1] = (int)sys.size();
  }
  // each kind's tasks numbered over the group's systems in this order (as
  // the kernel's loops number them); rot = tasks before the system, mod the
  // group's workers of that kind
  for (int k = 0; k < K; ++k) {
    const long long stride[ENS_NROT] = {Gk * ENS_T, Gk * ENS_T, Gk * ENS_W, Gk * ENS_W, Gk, Gk, Gk * ENS_T, Gk * ENS_T,
                                        Gk, Gk * ENS_W, Gk * ENS_T, Gk, Gk, Gk * ENS_T, Gk, Gk * ENS_T};
    long long base[ENS_NROT] = {};
    for (int pass = 0; pass < 2; ++pass)  // the pair tiles continue E_l^(1)'s numbering
      for (int i = goff[k]; i < goff[k + 1]; ++i) {
        EnsSys &E = sys[i];
        const Geo &g = E.d.g;
        const long long slots = (long long)g.slots(), N = g.N, P = g.P;
        long long cnt[ENS_NROT] = {};
        cnt[R_A] = slots;
        cnt[R_B_SPR] = P > 2 ? (P - 2) * g.Ns : 0;
        cnt[R_B_EINT] = N;
        cnt[R_B_PAIR] = E.d.pair_kind ? (long long)E.jobs * P : 0;
        cnt[R_B_SK] = E.ewald ? P : 0;
        cnt[R_C_PRE] = N >= 2 ? 1 : 0;
        cnt[R_C_TAB] = E.ewald ? P * E.ncol * (E.ns + 1) : 0;
        cnt[R_D_ENK] = N * (N - 1) / 2;
        cnt[R_D_REC] = E.ewald ? P : 0;
        cnt[R_E_W] = N;
        cnt[R_E_PS] = E.d.pair_kind ? slots : 0;
        cnt[R_E_INV] = 2 * ((N + TS_CHUNK - 1) / TS_CHUNK);
        cnt[R_F] = 2;
        cnt[R_G] = N * N;
        cnt[R_H] = (long long)((g.N + 31) / 32) * E.nsplit;
        cnt[R_I] = slots;
        for (int q = 0; q < ENS_NROT; ++q) {
          if ((q == R_B_PAIR) != (pass == 1)) continue;
          if (pass == 1 && i == goff[k]) base[R_B_PAIR] = base[R_B_EINT];
          E.rot[q] = (int)(base[q] % stride[q]);
          base[q] += cnt[q];
        }
      }
  }
  // the systems, the group offsets, the groups' barriers, then the FP32 pair
  // scratch of every system (tile partials, FP32 positions), kept in the
  // plan so that no later call can move it
  const size_t goff_at = (sizeof(EnsSys) * n + 255) & ~(size_t)255;
  const size_t bar_at = (goff_at + sizeof(int) * (K + 1) + 255) & ~(size_t)255;
  const size_t head = bar_at + ((sizeof(EnsBar) * K + 255) & ~(size_t)255);
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
  std::vector<unsigned char> host(head, 0);
  memcpy(host.data(), sys.data(), sizeof(EnsSys) * n);
  memcpy(host.data() + goff_at, goff.data(), sizeof(int) * (K + 1));
  e = cudaMemcpy(plan, host.data(), head, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(plan);
    return e;
  }
  ensemble_free(out);
  out.cost = cost;
  out.group_of.assign(n, 0);
  for (int k = 0; k < K; ++k)
    for (int i : lists[k]) out.group_of[i] = k;
  out.load = load;
  out.plan = plan;
  out.goff = (unsigned char *)plan + goff_at;
  out.bar = (unsigned char *)plan + bar_at;
  out.D = D;
  out.L = L;
  out.blocks = blocks;
  out.bps = blocks_per_sm;
  out.groups = K;
  out.nsys = n;
  out.smem = ENS_SMEM;
  return cudaSuccess;
}

cudaError_t ensemble_launch(const EnsLaunch &e, cudaStream_t st) {
  EnsFn fn = ens_kernel(e.D, e.L, e.bps);
  if (!fn || !e.plan) return cudaErrorInvalidValue;
  cudaError_t oe = ens_opt_in(fn);
  if (oe != cudaSuccess) return oe;
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr;
  memset(&cfg, 0, sizeof(cfg));
  memset(&attr, 0, sizeof(attr));
  cfg.gridDim = dim3((unsigned)e.blocks, 1, 1);
  cfg.blockDim = dim3(ENS_T, 1, 1);
  cfg.dynamicSmemBytes = ENS_SMEM;
  cfg.stream = st;
  attr.id = cudaLaunchAttributeCooperative;  // every block resident: the grid barrier needs it
  attr.val.cooperative = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  {
    XK_PROF("ensemble_step");
    oe = cudaLaunchKernelEx(&cfg, fn, (const EnsSys *)e.plan, (const int *)e.goff, e.groups, (EnsBar *)e.bar,
                            ENS_WAIT_LIMIT);
  }
  if (oe != cudaSuccess) return oe;
  return XK_LAUNCHED();
}

cudaError_t ensemble_status(const EnsLaunch &e, int *failed, double *phase_us) {
  std::vector<EnsBar> b(e.groups);
  cudaError_t r = cudaMemcpy(b.data(), e.bar, sizeof(EnsBar) * e.groups, cudaMemcpyDeviceToHost);
  if (r != cudaSuccess) return r;
  *failed = 0;
  for (const EnsBar &x : b) *failed |= x.err;
  if (phase_us) {
    for (int k = 0; k < ENS_PHASES; ++k) phase_us[k] = (double)(b[0].stamp[k + 1] - b[0].stamp[k]) * 1e-3;
    unsigned long long prev = b[0].stamp[1];
    for (int k = 0; k < 4; ++k) {
      phase_us[ENS_PHASES + k] = (double)(b[0].sub[k] - prev) * 1e-3;
      prev = b[0].sub[k];
    }
    for (int k = 0; k < ENS_MAX_GROUPS; ++k)
      phase_us[ENS_PHASES + 4 + k] = k < e.groups ? (double)(b[k].t1 - b[k].t0) * 1e-3 : 0.0;
  }
  return r;
}

void ensemble_free(EnsLaunch &e) {
  if (e.plan) cudaFree(e.plan);
  e.plan = e.goff = e.bar = nullptr;
  e.D = e.L = e.blocks = e.bps = e.groups = e.nsys = 0;
  e.smem = 0;
}

}  // namespace xk
