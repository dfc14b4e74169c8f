// xmd_step.cpp -- device entry points of the MD-Lab C ABI in libxmd_x: the
// integrator, the exchange recursion, bead forces and estimators.
//
// Each function validates its arguments, makes sure the state is on the
// device (xmd_runtime.cpp) and enqueues the kernels of xmd_kernels.cu on
// the library stream.  Reference counterparts are cited per function
// (MD-Lab file:line); the OpenCL branch of each is what these replace.
#include <cmath>
#include <vector>
#include <cstdlib>
#include <cstring>

#include "xmd_internal.h"

using namespace xmd;

static const int D = MD_DIMENSION_X;

// Ewald real-space images are summed while alpha*R < EWALD_XCUT (energies)
// or EWALD_XCUT_FORCE (FP64 forces); the reference sums the same images
// over its whole cube.  Beyond 5.8 an image's energy term erfc(aR)/R is below
// 2e-16 of erfc at contact (energies add every pair's images with one sign,
// so their tail is kept long).  A force term is h(x) a^2/x^2 with x = aR and
// h(x) = erfc(x) + 2x exp(-x^2)/sqrt(pi); h(5.2) = 1.1e-11, so an image
// beyond 5.2 adds less than 4e-13 a^2 to a bead's force, and the few hundred
// such images of a bead, pointing every way, change it by well under 1e-11
// of the largest force: 28% fewer images than at 5.8, the same 1e-10 parity.
static const double EWALD_XCUT = 5.8;
static const double EWALD_XCUT_FORCE = 5.2;

namespace xmd {

xk::TrapPrm trap_params(int kind) {
  xk::TrapPrm p{};
  p.kind = kind;
  p.w = md_trap_frequency_x;
  for (int d = 0; d < 3; ++d) {
    p.w2[d] = d < D ? md_trap_frequency_2_x[d] : 0;
    p.c[d] = d < D ? md_trap_center_x[d] : 0;
  }
  return p;
}

int trap_kind_of(const void *fn, bool energy) {
  if (!energy) {
    if (fn == (const void *)&md_harmonic_trap_force_x) return xk::TRAP_HARMONIC;
    if (fn == (const void *)&md_harmonic_trap_force_2_x) return xk::TRAP_HARMONIC_2;
    if (fn == (const void *)&md_neg_harmonic_trap_force_x) return xk::TRAP_NEG_HARMONIC;
  } else {
    if (fn == (const void *)&md_harmonic_trap_energy_x) return xk::TRAP_HARMONIC;
    if (fn == (const void *)&md_harmonic_trap_energy_2_x) return xk::TRAP_HARMONIC_2;
    if (fn == (const void *)&md_neg_harmonic_trap_energy_x) return xk::TRAP_NEG_HARMONIC;
  }
  return 0;
}

int pair_kind_of(const void *fn, bool energy) {
  if (!energy) {
    if (fn == (const void *)&md_gaussian_force_x) return xk::PAIR_GAUSSIAN;
    if (fn == (const void *)&md_periodic_gaussian_force_x) return xk::PAIR_PERIODIC_GAUSSIAN;
    if (fn == (const void *)&md_coulomb_force_x) return xk::PAIR_COULOMB;
    if (fn == (const void *)&md_coulomb_periodic_force_x) return xk::PAIR_PERIODIC_COULOMB;
    if (fn == (const void *)&md_coulomb_3d_ewald_force_x) return xk::PAIR_EWALD_REAL;
  } else {
    if (fn == (const void *)&md_gaussian_energy_x) return xk::PAIR_GAUSSIAN;
    if (fn == (const void *)&md_periodic_gaussian_energy_x) return xk::PAIR_PERIODIC_GAUSSIAN;
    if (fn == (const void *)&md_coulomb_energy_x) return xk::PAIR_COULOMB;
    if (fn == (const void *)&md_coulomb_periodic_energy_x) return xk::PAIR_PERIODIC_COULOMB;
    if (fn == (const void *)&md_coulomb_3d_ewald_energy_x) return xk::PAIR_EWALD_REAL;
  }
  return 0;
}

}  // namespace xmd

static xk::Chains chains_of(SimDev *sd) {
  xk::Chains c{};
  c.fast = sd->fast_chains;
  c.L = sd->L;
  c.nf = sd->nf;
  c.th = sd->th.as<double>();
  c.vt = sd->vt.as<double>();
  c.Q = sd->Q.as<double>();
  c.iQ = sd->iQ.as<double>();
  c.cf = sd->cf.as<int>();
  c.c0 = sd->c0.as<int>();
  c.c2 = sd->c2.as<int>();
  return c;
}

// features of the reference's PIMC / worm code paths that this step does not
// implement: refuse rather than compute something else
static int check_plain(md_pimd_t_x *p) {
  if (p->worm_index > 0 || p->cut_Pj != -1 || p->pbc)
    return fail(MD_GB_ERR_UNSUPPORTED, "worm, cut-bead and winding bookkeeping are not supported");
  return 0;
}

int xmd::check_image(const SimDev *sd, int image) {
  if (image && (sd->geo.box[0] <= 0 || (D > 1 && sd->geo.box[1] <= 0) || (D > 2 && sd->geo.box[2] <= 0)))
    return fail(MD_GB_ERR_ARG, "minimum image requested without a positive box");
  return 0;
}

double *xmd::scratch_for(SimDev *sd, size_t doubles, int *rc) {
  double *p = nullptr;
  *rc = scratch(sd, doubles, &p);
  return p;
}

size_t xmd::general_scratch(const xk::Geo &g) {
  size_t n = xk::pair_scratch_doubles(g);
  const size_t e = xk::exch_scratch_doubles(g);
  if (e > n) n = e;
  if (n < 4096) n = 4096;
  if (n < (size_t)g.P) n = g.P;
  return n;
}

extern "C" {

// ------------------------------------------------------------------
// integrator: md_simulation_x.c:421-472, :615-792, :794-856
// ------------------------------------------------------------------
int md_reset_force_x(md_simulation_t_x *sim) {
  if (ens_recording()) return ens_record(ENS_RESET, sim, nullptr, 0, 0, nullptr);
  SimDev *sd;
  XMD_TRY(sim_device(sim, &sd));
  XMD_CUDA(xk::zero(sd->f.as<double>(), sd->geo.slots(), stream()));
  return 0;
}

static int nhc(md_simulation_t_x *sim, md_num_t_x h, int half) {
  if (ens_recording()) return ens_record(half == 1 ? ENS_NHC1 : ENS_NHC2, sim, nullptr, h, 0, nullptr);
  SimDev *sd;
  const double *fex;  // exchange forces still to be added to f, if any
  XMD_TRY(sim_device_fex(sim, &sd, &fex));
  if (sd->nf < 1 || sd->L % 2 || sd->L > 8) {
    if (fex) XMD_CUDA(xk::add_into(sd->f.as<double>(), fex, sd->geo.slots(), stream()));
    if (sd->nf < 1) return 0;
    return fail(MD_GB_ERR_UNSUPPORTED, "chain length %d (even, <= 8 supported)", sd->L);
  }
  XMD_CUDA(xk::nhc_vv3(sd->geo, half, chains_of(sd), sd->x.as<double>(), sd->v.as<double>(),
                       sd->f.as<double>(), sd->m.as<double>(), MD_kB_X * sim->T, h, stream(), fex));
  return 0;
}

int md_update_nhc_VV3_1_x(md_simulation_t_x *sim, md_num_t_x h) { return nhc(sim, h, 1); }
int md_update_nhc_VV3_2_x(md_simulation_t_x *sim, md_num_t_x h) { return nhc(sim, h, 2); }

int md_periodic_boundary_x(md_simulation_t_x *sim) {
  if (!sim || !sim->box || sim->box->type != MD_ND_RECT_BOX_X) return 0;
  if (ens_recording()) return ens_record(ENS_WRAP, sim, nullptr, 0, 0, nullptr);
  SimDev *sd;
  XMD_TRY(sim_device(sim, &sd));
  XMD_CUDA(xk::wrap_box(sd->geo, sd->x.as<double>(), stream()));
  return 0;
}

// ------------------------------------------------------------------
// path-integral state: md_pimd_x.c:330-567
// ------------------------------------------------------------------
md_pimd_t_x *md_alloc_pimd_x(md_simulation_t_x *sim, int N, int P, md_num_t_x vi, md_num_t_x T) {
  if (!sim || N < 1 || P < 1) return NULL;
  md_pimd_t_x *p = (md_pimd_t_x *)calloc(1, sizeof(md_pimd_t_x));
  if (!p) return NULL;
  p->sim = sim;
  p->N = N;
  p->P = P;
  p->vi = vi;
  sim->T = T;
  p->beta = 1.0 / (MD_kB_X * T);
  p->omegaP = sqrt((double)P) / (p->beta * MD_hBar_X);
  const size_t nt = xk::ntri(N);
  p->ENk_count = (int)nt;
  p->VBN = (md_num_t_x *)calloc(N + 1, sizeof(md_num_t_x));
  p->minE = (md_num_t_x *)calloc(N + 1, sizeof(md_num_t_x));
  p->Eint = (md_num_t_x *)calloc(N, sizeof(md_num_t_x));
  p->Evir = (md_num_t_x *)calloc(N + 1, sizeof(md_num_t_x));
  md_num_t_x ***tabs[3] = {&p->ENk, &p->ENk2, &p->ENk3};
  for (int t = 0; t < 3; ++t) {
    *tabs[t] = (md_num_t_x **)malloc(sizeof(md_num_t_x *) * N);
    if (!*tabs[t]) {
      md_gb300_free_pimd_x(p);
      return NULL;
    }
    (*tabs[t])[0] = (md_num_t_x *)calloc(nt, sizeof(md_num_t_x));
    if (!(*tabs[t])[0]) {
      md_gb300_free_pimd_x(p);
      return NULL;
    }
    for (int l = 2; l <= N; ++l) (*tabs[t])[l - 1] = (*tabs[t])[0] + xk::tri(l);
  }
  p->pcount_in = (int)nt;
  p->pcount_ex = N * (N - 1) / 2;
  p->pair_in = (md_index_pair_t_x *)malloc(sizeof(md_index_pair_t_x) * nt);
  p->pair_ex = (md_index_pair_t_x *)malloc(sizeof(md_index_pair_t_x) * (p->pcount_ex > 0 ? p->pcount_ex : 1));
  p->Eindices = (int *)malloc(sizeof(int) * (size_t)N * N);
  p->pbW = (int *)calloc((size_t)N * P * D, sizeof(int));
  if (!p->VBN || !p->minE || !p->Eint || !p->Evir || !p->pair_in || !p->pair_ex || !p->Eindices || !p->pbW) {
    md_gb300_free_pimd_x(p);
    return NULL;
  }
  int a = 0, b = 0;
  for (int i = 0; i < N; ++i)
    for (int j = 0; j <= i; ++j) {
      p->pair_in[a] = {i, j};
      p->Eindices[i * N + j] = a++;
      if (j < i) p->pair_ex[b++] = {i, j};
    }
  p->cut_Pj = -1;
  p->mc_par = -1;
  p->pbc = 0;
  p->worm_index = -1;
  p->old_worm_index = -1;
  layout_hint(sim, N, P);
  return p;
}

void md_gb300_free_pimd_x(md_pimd_t_x *p) {
  if (!p) return;
  forget(p);
  md_num_t_x **tabs[3] = {p->ENk, p->ENk2, p->ENk3};
  for (int t = 0; t < 3; ++t)
    if (tabs[t]) {
      free(tabs[t][0]);
      free(tabs[t]);
    }
  free(p->VBN);
  free(p->minE);
  free(p->Eint);
  free(p->Evir);
  free(p->pair_in);
  free(p->pair_ex);
  free(p->Eindices);
  free(p->pbW);
  free(p);
}

md_pimd_t_x *md_pimd_sync_host_x(md_pimd_t_x *pimd, int read_only) {
  return pimd_to_host(pimd, read_only != 0) == 0 ? pimd : NULL;
}

void md_pimd_change_temperature_x(md_pimd_t_x *p, md_num_t_x T) {
  p->sim->T = T;
  p->beta = 1.0 / (MD_kB_X * T);
  p->omegaP = sqrt((double)p->P) / (p->beta * MD_hBar_X);
}

// neighbours on the cycle closing particles N2-k+1..N2: md_pimd_x.c:521-549
int md_pimd_next_index_x(int l, int j, int N2, int k, int P) {
  if (j != P) return MD_PIMD_INDEX_X(l, j + 1, P);
  return MD_PIMD_INDEX_X(l == N2 ? N2 - k + 1 : l + 1, 1, P);
}

int md_pimd_prev_index_x(int l, int j, int N2, int k, int P) {
  if (j != 1) return MD_PIMD_INDEX_X(l, j - 1, P);
  return MD_PIMD_INDEX_X(l == N2 - k + 1 ? N2 : l - 1, P, P);
}

// md_pimd_x.c:551-567
int md_pimd_init_particle_uniform_pos_x(md_pimd_t_x *p, md_num_t_x *center, md_num_t_x *L, md_num_t_x fluc) {
  if (!md_simulation_sync_host_x(p->sim, 0)) return -1;
  for (int l = 0; l < p->N; ++l) {
    double c[MD_DIMENSION_X];
    for (int d = 0; d < D; ++d) c[d] = md_random_uniform_x(center[d] - L[d] / 2, center[d] + L[d] / 2);
    for (int j = 0; j < p->P; ++j)
      for (int d = 0; d < D; ++d)
        p->sim->particles[MD_PIMD_INDEX_X(l + 1, j + 1, p->P)].x[d] = c[d] + fluc * (md_random_uniform_x(0, 2) - 1);
  }
  return 0;
}

// ------------------------------------------------------------------
// exchange: md_pimd_x.c:593-665, :814-953, :997-1109, :1969-2210, :2369-2721
// ------------------------------------------------------------------
int md_pimd_fast_fill_ENk_x(md_pimd_t_x *pimd, int image) {
  if (ens_recording()) return ens_record(ENS_ENK, nullptr, pimd, 0, image, nullptr);
  // on the library stream: on the side stream its many small blocks would
  // compete with the structure-factor kernels that start the pair forces,
  // which costs more than the overlap gains
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(check_image(sd, image));
  XMD_CUDA(xk::fill_enk(sd->geo, sd->x.as<double>(), sd->m.as<double>(), pimd->omegaP * pimd->omegaP, image,
                        pd->Eint.as<double>(), pd->ENk.as<double>(), pd->linkt.as<double>(), stream()));
  pd->tmpv_fresh = false;
  pd->g_fresh = false;
  return 0;
}

int md_pimd_fill_ENk_x(md_pimd_t_x *pimd, int image) { return md_pimd_fast_fill_ENk_x(pimd, image); }

int md_pimd_fill_VB_x(md_pimd_t_x *pimd) {
  if (ens_recording()) return ens_record(ENS_VB, nullptr, pimd, 0, 0, nullptr);
  NoJoin nj;  // the exchange chain starts on the side stream here
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  // the backward recursion (tmpV of the exchange forces) needs only ENk as
  // well: both run now, side by side, and the force call reuses tmpV while
  // ENk, beta and vi are unchanged
  // Both run on the side stream, which overlaps whatever the driver queues
  // next that does not read them (the pair and trap forces).
  double *rs = pd->rec.as<double>();
  cudaStream_t s2;
  XMD_TRY(side_begin(&s2));
  XMD_CUDA(xk::fill_vb_tv(pimd->N, pimd->beta, pimd->vi, pd->ENk.as<double>(), pd->lnn.as<double>(),
                          pd->VBN.as<double>(), pd->tmpV.as<double>(), rs, rs + xk::rec_scratch_doubles(pimd->N), s2));
  XMD_TRY(side_end(nullptr));
  pd->tmpv_fresh = true;
  pd->tmpv_beta = pimd->beta;
  pd->tmpv_vi = pimd->vi;
  pd->g_fresh = false;
  return 0;
}

int md_pimd_fast_fill_force_VB_x(md_pimd_t_x *pimd, int image) {
  if (ens_recording()) return ens_record(ENS_FVB, nullptr, pimd, 0, image, nullptr);
  // continues the side stream after md_pimd_fill_VB_x (no join): G and the
  // exchange spring forces are computed there, into sd->fex, which the next
  // join adds to f
  NoJoin nj;
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(check_image(sd, image));
  if (pimd->P < 2) return fail(MD_GB_ERR_ARG, "the exchange spring force needs P >= 2 beads");
  const size_t nx = xk::exch_scratch_doubles(sd->geo);
  if (sd->fex.bytes < sd->geo.slots() * sizeof(double) || sd->xscr.bytes < nx * sizeof(double)) {
    if (capturing()) return fail(MD_GB_ERR_CAPTURE, "exchange buffers are not allocated yet");
    XMD_TRY(reserve(sd->fex, sd->geo.slots() * sizeof(double)));
    XMD_TRY(reserve(sd->xscr, nx * sizeof(double)));
  }
  double *scr = sd->xscr.as<double>();
  cudaStream_t st;
  XMD_TRY(side_begin(&st));
  const int N = pimd->N;
  if (pd->tmpv_fresh && pd->tmpv_beta == pimd->beta && pd->tmpv_vi == pimd->vi) {
    // both recursions of the current ENk are in pd->rec: G from their
    // extended-range numbers
    double *rs = pd->rec.as<double>();
    XMD_CUDA(xk::fill_g_ext(N, rs, rs + xk::rec_scratch_doubles(N), pd->G.as<double>(), st));
  } else {
    XMD_CUDA(xk::back_vb(N, pimd->beta, pimd->vi, pd->ENk.as<double>(), pd->lnn.as<double>(),
                         pd->tmpV.as<double>(), pd->rec.as<double>(), st));
    XMD_CUDA(xk::fill_g(N, pimd->beta, pimd->vi, pd->ENk.as<double>(), pd->VBN.as<double>(),
                        pd->tmpV.as<double>(), pd->lnn.as<double>(), pd->G.as<double>(), st));
  }
  XMD_CUDA(cudaMemsetAsync(sd->fex.p, 0, sd->geo.slots() * sizeof(double), st));
  XMD_CUDA(xk::exch_force(sd->geo, sd->x.as<double>(), sd->m.as<double>(), pimd->omegaP * pimd->omegaP, image,
                          pd->G.as<double>(), sd->fex.as<double>(), scr, st));
  XMD_TRY(side_end(sd));
  pd->g_fresh = true;
  pd->g_beta = pimd->beta;
  pd->g_vi = pimd->vi;
  return 0;
}

int md_pimd_fill_force_VB_x(md_pimd_t_x *pimd, int image) { return md_pimd_fast_fill_force_VB_x(pimd, image); }

// ------------------------------------------------------------------
// external forces: md_pimd_x.c:1297-1391, :1527-1677
// ------------------------------------------------------------------
int md_pimd_calc_trap_force_x(md_pimd_t_x *pimd, md_trap_force_t_x tf) {
  if (ens_recording()) return ens_record(ENS_TRAP, nullptr, pimd, 0, 0, (const void *)tf);
  NoJoin nj;  // adds to f only: may overlap the side stream's exchange work
  const int kind = trap_kind_of((const void *)tf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "trap force function has no device kernel");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_CUDA(xk::trap_force(sd->geo, trap_params(kind), sd->x.as<double>(), sd->f.as<double>(), stream()));
  return 0;
}

}  // extern "C"

int xmd::ewald_tables(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd) {
  const int ns = md_coulomb_n_sum_x;
  const double a = md_coulomb_truc_x, qs = md_coulomb_strength_x;
  if (ns < 1 || ns > 11) return fail(MD_GB_ERR_UNSUPPORTED, "Ewald n_sum %d (1..11 supported)", ns);
  if (!(a > 0)) return fail(MD_GB_ERR_ARG, "Ewald alpha must be positive");
  const xk::Geo &g = sd->geo;
  if (pd->rc_nsum == ns && pd->rc_alpha == a && pd->rc_qs == qs && pd->rc_box[0] == g.box[0] &&
      pd->rc_box[1] == g.box[1] && pd->rc_box[2] == g.box[2] && pd->rc_phase.p)
    return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "Ewald tables change while capturing a graph");
  const int nk = xk::recip_count(ns);
  XMD_TRY(reserve(pd->rc_coef, xk::recip_coef_bytes(nk)));
  XMD_TRY(reserve(pd->rc_cols, sizeof(int) * xk::recip_cols_ints(ns)));
  // FP64 phases, then their FP32 copy for the mixed form
  XMD_TRY(reserve(pd->rc_phase, sizeof(double) * xk::recip_phase_doubles(g, ns) * 3 / 2));
  // FP64 structure factors, then the FP32 ones of the FP64 form's split
  XMD_TRY(reserve(pd->rc_S, sizeof(double) * 3 * (size_t)nk * g.P));
  XMD_TRY(reserve(pd->rc_T, sizeof(double) * xk::recip_table_doubles(g, ns)));
  xk::Recip r{};
  r.coef = pd->rc_coef.as<double>();
  r.kvec = pd->rc_cols.as<int>();
  r.S = pd->rc_S.as<double>();
  r.S32 = r.S + 2 * (size_t)nk * g.P;
  XMD_CUDA(xk::recip_setup(g, ns, a, qs, r, stream()));
  pd->rc_ncol = r.ncol;
  pd->rc_tsz = r.tsz;
  pd->rc_ncol_in = r.ncol_in;
  pd->rc_ncol_out = r.ncol_out;
  pd->rc_tsz_in = r.tsz_in;
  pd->rc_s32_off = 2 * (size_t)nk * g.P;
  pd->rc_nsum = ns;
  pd->rc_alpha = a;
  pd->rc_qs = qs;
  pd->rc_nk = nk;
  pd->rc_csum = r.csum;
  for (int d = 0; d < 3; ++d) pd->rc_box[d] = g.box[d];
  (void)pimd;
  return 0;
}

// library-wide arithmetic of the pair and Ewald forces (md_gb300_x.h)
static int g_precision = MD_GB_PRECISION_FP64;

xk::Recip xmd::recip_of(PimdDev *pd) {
  xk::Recip r{};
  r.nsum = pd->rc_nsum;
  r.nk = pd->rc_nk;
  r.ncol = pd->rc_ncol;
  r.tsz = pd->rc_tsz;
  r.ncol_in = pd->rc_ncol_in;
  r.ncol_out = pd->rc_ncol_out;
  r.tsz_in = pd->rc_tsz_in;
  r.S32 = pd->rc_S.as<double>() + pd->rc_s32_off;
  r.coef = pd->rc_coef.as<double>();
  r.kvec = pd->rc_cols.as<int>();
  r.phase = pd->rc_phase.as<double>();
  r.S = pd->rc_S.as<double>();
  r.T = pd->rc_T.as<double>();
  r.csum = pd->rc_csum;
  return r;
}

xk::PairPrm xmd::pair_params(int kind) {
  xk::PairPrm p{};
  p.kind = kind;
  p.g = md_gaussian_strength_x;
  p.s = md_gaussian_range_x;
  p.qs = md_coulomb_strength_x;
  p.alpha = md_coulomb_truc_x;
  p.nsum = md_coulomb_n_sum_x;
  p.rcut = p.alpha > 0 ? EWALD_XCUT / p.alpha : 0;
  p.xsplit = g_precision == MD_GB_PRECISION_FP64_STRICT ? 0.0 : xk::EWALD_XSPLIT;
  return p;
}

// image shifts around the minimum image that can fall inside rcut:
// |m - k L| < rcut with |m| <= L/2 needs |k| < 1/2 + rcut/L
void xmd::ewald_shifts(xk::PairPrm &p, const xk::Geo &g) {
  for (int d = 0; d < 3; ++d) {
    p.kmax[d] = 0;
    if (g.box[d] > 0) p.kmax[d] = (int)ceil(0.5 + p.rcut / g.box[d]) - 1;
    if (p.kmax[d] < 0) p.kmax[d] = 0;
  }
}

xk::PairPrm xmd::force_params(int kind, const SimDev *sd) {
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sd->geo);  // the alpha L limit is the energies' (the longer cut-off)
  prm.inv_mass = sd->uniform_mass ? 1.0 / sd->mass0 : 0.0;
  if (kind == xk::PAIR_EWALD_REAL && prm.alpha > 0) prm.rcut = EWALD_XCUT_FORCE / prm.alpha;
  return prm;
}

extern "C" {

int md_pimd_calc_pair_force_x(md_pimd_t_x *pimd, md_pair_force_t_x pf) {
  if (ens_recording()) return ens_record(ENS_PAIR, nullptr, pimd, 0, 0, (const void *)pf);
  NoJoin nj;  // adds to f only: may overlap the side stream's exchange work
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair force function has no device kernel");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  if (kind == xk::PAIR_EWALD_REAL && D != 3) return 0;  // the reference's Ewald is 3D only
  if (kind == xk::PAIR_PERIODIC_GAUSSIAN || kind == xk::PAIR_PERIODIC_COULOMB || kind == xk::PAIR_EWALD_REAL)
    XMD_TRY(check_image(sd, 1));
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  cudaStream_t st = stream();
  xk::PairPrm prm = force_params(kind, sd);
  const bool mixed = g_precision == MD_GB_PRECISION_MIXED;
  int learned = 0;
  if (kind == xk::PAIR_EWALD_REAL) {
    if (prm.kmax[0] > 1 || prm.kmax[1] > 1 || prm.kmax[2] > 1)
      return fail(MD_GB_ERR_UNSUPPORTED, "Ewald alpha*L below %.1f (images beyond the neighbouring boxes)",
                  2 * EWALD_XCUT / 3);
    if (!sd->uniform_mass) return fail(MD_GB_ERR_UNSUPPORTED, "structure-factor Ewald needs equal bead masses");
    XMD_TRY(ewald_tables(pimd, sd, pd));
    learned = learned_mode(pimd, true);
    if (learned == 1) return learned_pair_force(pimd, sd, pd, prm, scr);
    const double inv_mP = 1.0 / (sd->mass0 * pimd->P);
    if (mixed)
      XMD_CUDA(xk::recip_force32(sd->geo, recip_of(pd), sd->x.as<double>(), inv_mP, sd->f.as<double>(), st));
    else
      XMD_CUDA(xk::recip_force(sd->geo, recip_of(pd), sd->x.as<double>(), inv_mP, sd->f.as<double>(), st,
                               g_precision != MD_GB_PRECISION_FP64_STRICT));
  }
  if (mixed)
    XMD_CUDA(xk::pair_force32(sd->geo, prm, sd->x.as<double>(), sd->m.as<double>(), sd->f.as<double>(), scr, st));
  else
    XMD_CUDA(xk::pair_force(sd->geo, prm, sd->x.as<double>(), sd->m.as<double>(), sd->f.as<double>(), scr, st));
  if (learned == 2) XMD_TRY(learned_judge_step(pimd, sd, pd));
  return 0;
}

// Two species (md_pimd_x.c:3282-3481, :3483-3632): the cross pairs between
// pimd and pimd2, with pimd's box.  Both species stay on the device; the
// cross call adds to both f arrays only (NoJoin, like the one-species call).
// The Ewald callback needs both species in one box (the reciprocal sums use
// each species' structure factors with one set of coefficients) and equal
// bead masses within each species.  Always FP64, in every precision mode.
static int two_species(md_pimd_t_x *pimd, md_pimd_t_x *pimd2, int kind, SimDev **sa, PimdDev **pa, SimDev **sb,
                       PimdDev **pb) {
  XMD_TRY(pimd_device(pimd, sa, pa));
  XMD_TRY(pimd_device(pimd2, sb, pb));
  if (kind == xk::PAIR_PERIODIC_GAUSSIAN || kind == xk::PAIR_PERIODIC_COULOMB || kind == xk::PAIR_EWALD_REAL)
    XMD_TRY(check_image(*sa, 1));
  if (kind == xk::PAIR_EWALD_REAL) {
    for (int d = 0; d < 3; ++d)
      if ((*sa)->geo.box[d] != (*sb)->geo.box[d])
        return fail(MD_GB_ERR_UNSUPPORTED, "Ewald between species in different boxes");
    xk::PairPrm prm = pair_params(kind);
    ewald_shifts(prm, (*sa)->geo);
    if (prm.kmax[0] > 1 || prm.kmax[1] > 1 || prm.kmax[2] > 1)
      return fail(MD_GB_ERR_UNSUPPORTED, "Ewald alpha*L below %.1f (images beyond the neighbouring boxes)",
                  2 * EWALD_XCUT / 3);
    XMD_TRY(ewald_tables(pimd, *sa, *pa));
    XMD_TRY(ewald_tables(pimd2, *sb, *pb));
  }
  return 0;
}

int md_pimd_calc_pair_force_2_x(md_pimd_t_x *pimd, md_pimd_t_x *pimd2, md_pair_force_t_x pf) {
  if (!pimd || !pimd2) return fail(MD_GB_ERR_ARG, "NULL simulation");
  if (pimd->P != pimd2->P) return -1;  // md_pimd_x.c:3283-3284
  NoJoin nj;
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair force function has no device kernel");
  if (kind == xk::PAIR_EWALD_REAL && D != 3) return 0;  // the reference's Ewald is 3D only
  SimDev *sa, *sb;
  PimdDev *pa, *pb;
  XMD_TRY(two_species(pimd, pimd2, kind, &sa, &pa, &sb, &pb));
  int rc;
  double *scr = scratch_for(sa, xk::pair2_scratch_doubles(sa->geo, sb->geo), &rc);
  if (rc) return rc;
  cudaStream_t st = stream();
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sa->geo);
  if (kind == xk::PAIR_EWALD_REAL && prm.alpha > 0) prm.rcut = EWALD_XCUT_FORCE / prm.alpha;
  if (kind == xk::PAIR_EWALD_REAL) {
    if (!sa->uniform_mass || !sb->uniform_mass)
      return fail(MD_GB_ERR_UNSUPPORTED, "structure-factor Ewald needs equal bead masses within each species");
    XMD_CUDA(xk::recip_force_2(sa->geo, recip_of(pa), sa->x.as<double>(), 1.0 / (sa->mass0 * pimd->P),
                               sa->f.as<double>(), sb->geo, recip_of(pb), sb->x.as<double>(),
                               1.0 / (sb->mass0 * pimd2->P), sb->f.as<double>(), st));
  }
  XMD_CUDA(xk::pair_force_2(sa->geo, sb->geo, prm, sa->x.as<double>(), sa->m.as<double>(), sb->x.as<double>(),
                            sb->m.as<double>(), sa->f.as<double>(), sb->f.as<double>(), scr, st));
  return 0;
}

int md_pimd_calc_pair_energy_2_x(md_pimd_t_x *pimd, md_pimd_t_x *pimd2, md_pair_energy_t_x pe,
                                 md_stats_t_x *stats) {
  if (!pimd || !pimd2) return fail(MD_GB_ERR_ARG, "NULL simulation");
  if (pimd->P != pimd2->P) return -1;  // md_pimd_x.c:3484-3485
  const int kind = pair_kind_of((const void *)pe, true);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair energy function has no device kernel");
  if (kind == xk::PAIR_EWALD_REAL && D != 3) return 0;
  SimDev *sa, *sb;
  PimdDev *pa, *pb;
  double *acc;
  XMD_TRY(two_species(pimd, pimd2, kind, &sa, &pa, &sb, &pb));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  size_t need = xk::pair2_scratch_doubles(sa->geo, sb->geo);
  if (need < (size_t)pimd->P) need = pimd->P;
  double *scr = scratch_for(sa, need, &rc);
  if (rc) return rc;
  cudaStream_t st = stream();
  if (kind == xk::PAIR_EWALD_REAL)
    XMD_CUDA(xk::recip_energy_2(sa->geo, recip_of(pa), sa->x.as<double>(), sb->geo, recip_of(pb),
                                sb->x.as<double>(), acc, scr, st));
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sa->geo);
  XMD_CUDA(xk::pair_energy_2(sa->geo, sb->geo, prm, sa->x.as<double>(), sb->x.as<double>(), acc, scr, st));
  return 0;
}

int md_gb300_set_pair_tile_x(md_pair_force_t_x pf, int N, int P, int warps) {
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair force function has no device kernel");
  if (warps != 1 && warps != 2 && warps != 4 && warps != 8) return fail(MD_GB_ERR_ARG, "warps must be 1, 2, 4 or 8");
  if (N < 1 || P < 1) return fail(MD_GB_ERR_ARG, "invalid system shape");
  xk::set_pair32_warps(kind, D, N, P, warps);
  return 0;
}

// Tile-shape autotuner of the FP32 pair kernel (md_gb300_x.h): times each
// shape on this system's own positions into a scratch force array.
int md_gb300_autotune_pair_x(md_pimd_t_x *pimd, md_pair_force_t_x pf, int repeats, int *warps, double *ms) {
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair force function has no device kernel");
  if (repeats < 1) return fail(MD_GB_ERR_ARG, "repeats must be positive");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "autotuning times kernels; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  if (kind == xk::PAIR_EWALD_REAL && D != 3) return fail(MD_GB_ERR_UNSUPPORTED, "Ewald is 3D only");
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sd->geo);
  prm.inv_mass = sd->uniform_mass ? 1.0 / sd->mass0 : 0.0;
  const xk::Geo &g = sd->geo;
  DevBuf ftmp;
  XMD_TRY(reserve(ftmp, g.slots() * sizeof(double)));
  cudaStream_t st = stream();
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const int cand[4] = {1, 2, 4, 8};
  int best_w = 8;
  double best = INFINITY;
  for (int ci = 0; ci < 4 && e == cudaSuccess; ++ci) {
    xk::set_pair32_warps(kind, D, g.N, g.P, cand[ci]);
    e = xk::pair_force32(g, prm, sd->x.as<double>(), sd->m.as<double>(), ftmp.as<double>(), scr, st);
    if (e == cudaSuccess) e = cudaEventRecord(a, st);
    for (int r = 0; r < repeats && e == cudaSuccess; ++r)
      e = xk::pair_force32(g, prm, sd->x.as<double>(), sd->m.as<double>(), ftmp.as<double>(), scr, st);
    if (e == cudaSuccess) e = cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    if (e == cudaSuccess && t / repeats < best) {
      best = t / repeats;
      best_w = cand[ci];
    }
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  release(ftmp);
  xk::set_pair32_warps(kind, D, g.N, g.P, best_w);
  if (e != cudaSuccess) return cuda_fail(e, "pair-kernel autotuning");
  if (warps) *warps = best_w;
  if (ms) *ms = best;
  return 0;
}

// FP64 autotuner (md_gb300_x.h): the tile kernels' blocks per SM and, for
// Ewald, the structure-factor layout, each timed on this system's positions
// into a scratch force array; the choices are recorded for this shape.
int md_gb300_autotune_fp64_x(md_pimd_t_x *pimd, md_pair_force_t_x pf, int repeats, int *blocks_per_sm,
                             int *sk_layout, double *ms) {
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair force function has no device kernel");
  if (repeats < 1) return fail(MD_GB_ERR_ARG, "repeats must be positive");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "autotuning times kernels; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  const bool ewald = kind == xk::PAIR_EWALD_REAL;
  if (ewald && D != 3) return fail(MD_GB_ERR_UNSUPPORTED, "Ewald is 3D only");
  if (ewald && !sd->uniform_mass) return fail(MD_GB_ERR_UNSUPPORTED, "structure-factor Ewald needs equal bead masses");
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sd->geo);
  if (ewald) {
    if (prm.kmax[0] > 1 || prm.kmax[1] > 1 || prm.kmax[2] > 1)
      return fail(MD_GB_ERR_UNSUPPORTED, "Ewald alpha*L below %.1f (images beyond the neighbouring boxes)",
                  2 * EWALD_XCUT / 3);
    prm.rcut = EWALD_XCUT_FORCE / prm.alpha;
    XMD_TRY(ewald_tables(pimd, sd, pd));
  }
  const xk::Geo &g = sd->geo;
  DevBuf ftmp;
  XMD_TRY(reserve(ftmp, g.slots() * sizeof(double)));
  cudaStream_t st = stream();
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  // mean time of one call of fn after one untimed call
  auto timeit = [&](auto fn, double &out) {
    if (e == cudaSuccess) e = fn();
    if (e == cudaSuccess) e = cudaEventRecord(a, st);
    for (int r = 0; r < repeats && e == cudaSuccess; ++r) e = fn();
    if (e == cudaSuccess) e = cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    out = t / repeats;
  };
  auto tiles = [&]() { return xk::pair_force(g, prm, sd->x.as<double>(), sd->m.as<double>(), ftmp.as<double>(), scr, st); };
  int best_bps = 0;
  double best_t = INFINITY, best_r = 0;
  for (int bps = 1; bps <= 2 && e == cudaSuccess; ++bps) {
    xk::set_tuning(xk::TUNE_PAIR64_BPS, kind, D, g.N, g.P, bps);
    double t = 0;
    timeit(tiles, t);
    if (e == cudaSuccess && t < best_t) {
      best_t = t;
      best_bps = bps;
    }
  }
  if (best_bps) xk::set_tuning(xk::TUNE_PAIR64_BPS, kind, D, g.N, g.P, best_bps);
  int best_lay = 0;
  if (ewald && e == cudaSuccess) {
    const double inv_mP = 1.0 / (sd->mass0 * pimd->P);
    auto recip = [&]() {
    return xk::recip_force(g, recip_of(pd), sd->x.as<double>(), inv_mP, ftmp.as<double>(), st,
                           g_precision != MD_GB_PRECISION_FP64_STRICT);
  };
    best_r = INFINITY;
    const int lays[3] = {xk::SK_16x16, xk::SK_8x32, xk::SK_64x1};
    for (int i = 0; i < 3 && e == cudaSuccess; ++i) {
      xk::set_tuning(xk::TUNE_SK_LAYOUT, md_coulomb_n_sum_x, 3, g.N, g.P, lays[i]);
      double t = 0;
      timeit(recip, t);
      if (e == cudaSuccess && t < best_r) {
        best_r = t;
        best_lay = lays[i];
      }
    }
    if (best_lay) xk::set_tuning(xk::TUNE_SK_LAYOUT, md_coulomb_n_sum_x, 3, g.N, g.P, best_lay);
  }
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  release(ftmp);
  if (e != cudaSuccess) return cuda_fail(e, "FP64 autotuning");
  if (blocks_per_sm) *blocks_per_sm = best_bps;
  if (sk_layout) *sk_layout = best_lay;
  if (ms) *ms = best_t + best_r;
  return 0;
}

int md_gb300_set_precision_x(int mode) {
  if (mode != MD_GB_PRECISION_FP64 && mode != MD_GB_PRECISION_MIXED && mode != MD_GB_PRECISION_FP64_STRICT)
    return fail(MD_GB_ERR_ARG, "unknown precision mode %d", mode);
  g_precision = mode;
  return 0;
}

int md_gb300_get_precision_x(void) { return g_precision; }

int md_gb300_set_solve_path_x(int path) {
  if (path != MD_GB_SOLVE_AUTO && path != MD_GB_SOLVE_BLOCK && path != MD_GB_SOLVE_CLUSTER)
    return fail(MD_GB_ERR_ARG, "unknown recursion solve path %d", path);
  xk::set_solve_path(path);
  return 0;
}

int md_gb300_get_solve_path_x(int N) { return N < 1 ? xk::solve_path() : xk::solve_choice(N); }

// Solve autotuner (md_gb300_x.h): both recursions of pimd's current ENk,
// timed with each solve kernel into scratch outputs; pimd's own V_B, tmpV
// and weights are not touched.
int md_gb300_autotune_solve_x(md_pimd_t_x *pimd, int repeats, int *path, double *ms) {
  if (repeats < 1) return fail(MD_GB_ERR_ARG, "repeats must be positive");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "autotuning times kernels; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  const int N = pimd->N;
  const size_t nrs = xk::rec_scratch_doubles(N);
  DevBuf tmp;
  XMD_TRY(reserve(tmp, (2 * nrs + 2 * (size_t)(N + 1)) * sizeof(double)));
  double *rs = tmp.as<double>(), *vb = rs + 2 * nrs, *tv = vb + N + 1;
  cudaStream_t st = stream();
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaMemsetAsync(tmp.p, 0, tmp.bytes, st);
  if (e == cudaSuccess) e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  const int saved = xk::solve_path();
  const int cand[2] = {MD_GB_SOLVE_BLOCK, MD_GB_SOLVE_CLUSTER};
  int best_p = xk::solve_choice(N);
  double best = INFINITY;
  for (int ci = 0; ci < 2 && e == cudaSuccess; ++ci) {
    xk::set_solve_path(cand[ci]);
    e = xk::fill_vb_tv(N, pimd->beta, pimd->vi, pd->ENk.as<double>(), pd->lnn.as<double>(), vb, tv, rs, rs + nrs,
                       st);
    if (e == cudaErrorInvalidConfiguration) {  // no cluster of this size fits: not a candidate
      cudaGetLastError();
      e = cudaSuccess;
      continue;
    }
    if (e == cudaSuccess) e = cudaEventRecord(a, st);
    for (int r = 0; r < repeats && e == cudaSuccess; ++r)
      e = xk::fill_vb_tv(N, pimd->beta, pimd->vi, pd->ENk.as<double>(), pd->lnn.as<double>(), vb, tv, rs, rs + nrs,
                         st);
    if (e == cudaSuccess) e = cudaEventRecord(b, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(b);
    float t = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, a, b);
    if (e == cudaSuccess && t / repeats < best) {
      best = t / repeats;
      best_p = cand[ci];
    }
  }
  xk::set_solve_path(saved);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  release(tmp);
  if (e != cudaSuccess) return cuda_fail(e, "recursion-solve autotuning");
  xk::set_solve_choice(N, best_p);
  if (path) *path = best_p;
  if (ms) *ms = best;
  return 0;
}

// tmpV (backward recursion, N+1) and G (connection probabilities, N x N,
// G[(l-1)*N + (j-1)]) of the last exchange force call, copied to the host
int md_gb300_exchange_tables_x(md_pimd_t_x *pimd, double *tmpV, double *G) {
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "host copy while capturing a graph");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  const int N = pimd->N;
  cudaStream_t st = stream();
  if (tmpV) XMD_CUDA(cudaMemcpyAsync(tmpV, pd->tmpV.p, (size_t)(N + 1) * 8, cudaMemcpyDeviceToHost, st));
  if (G) XMD_CUDA(cudaMemcpyAsync(G, pd->G.p, (size_t)N * N * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  return 0;
}

// Pair forces for callers that cannot allocate device memory (md_gb300_x.h).
// Everything here works on the caller's device pointers and stream; the
// per-tile partial sums go to a fixed array inside the library.  This
// function calls no allocator: not cudaMalloc, not the stream-ordered
// allocator, and it creates no stream or event.
int md_gb300_pair_force_noalloc_x(md_pair_force_t_x pf, const double *x, const double *m, double *f, int N, int P,
                                  int ld, const double *L, void *stream) {
  const int kind = pair_kind_of((const void *)pf, false);
  if (!kind || kind == xk::PAIR_EWALD_REAL)
    return fail(MD_GB_ERR_UNSUPPORTED, "no-allocation pair forces: Gaussian and Coulomb kinds only");
  if (!x || !m || !f || N < 1 || P < 1 || ld < N)
    return fail(MD_GB_ERR_ARG, "no-allocation pair forces: invalid pointers or sizes (N=%d P=%d ld=%d)", N, P, ld);
  const bool periodic = kind == xk::PAIR_PERIODIC_GAUSSIAN || kind == xk::PAIR_PERIODIC_COULOMB;
  if (periodic && !L) return fail(MD_GB_ERR_ARG, "no-allocation pair forces: periodic kind needs the box");
  if (!device_present()) return fail(MD_GB_ERR_NO_DEVICE, "no CUDA device is available");
  xk::Geo g{};
  g.D = D;
  g.N = N;
  g.P = P;
  g.Ns = ld;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = (L && d < D) ? L[d] : 0.0;
    g.inv_box[d] = g.box[d] > 0 ? 1.0 / g.box[d] : 0.0;
  }
  if (periodic)
    for (int d = 0; d < D; ++d)
      if (!(g.box[d] > 0)) return fail(MD_GB_ERR_ARG, "no-allocation pair forces: box lengths must be positive");
  const size_t need = xk::pair_force_noalloc_need(g);
  if (need > xk::NOALLOC_SCRATCH_DOUBLES)
    return fail(MD_GB_ERR_ARG,
                "no-allocation pair forces: N=%d, P=%d, ld=%d needs %zu doubles of scratch, more than the fixed %zu "
                "(ceil(N/32) * P * D * ld must not exceed it)",
                N, P, ld, need, (size_t)xk::NOALLOC_SCRATCH_DOUBLES);
  // a launch error left by the caller's earlier work is theirs: report it
  // as such before this call launches anything (its own launch status is
  // read with cudaGetLastError, which would otherwise return that error)
  const cudaError_t pending = cudaGetLastError();
  if (pending != cudaSuccess) return cuda_fail(pending, "error pending from earlier work, before the no-allocation call");
  XMD_CUDA(xk::pair_force_noalloc(g, pair_params(kind), x, m, f, (cudaStream_t)stream));
  return 0;
}

// ------------------------------------------------------------------
// estimators: md_pimd_x.c:1111-1295, :1393-1525, :1679-1824,
// :3989-4056, :4072-4348, :4423-4556
// ------------------------------------------------------------------
// G of the last exchange force call when it belongs to the stored ENk,
// VBN and the current beta and xi, else null (the estimators then solve the
// reference's recursion)
static const double *cycle_probs(const md_pimd_t_x *pimd, PimdDev *pd) {
  return pd->g_fresh && pd->g_beta == pimd->beta && pd->g_vi == pimd->vi ? pd->G.as<double>() : nullptr;
}

int md_pimd_calc_VBN_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats) {
  SimDev *sd;
  PimdDev *pd;
  double *acc;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  double *scr = scratch_for(sd, xk::vbn_scratch_doubles(pimd->N), &rc);
  if (rc) return rc;
  const double add = D * pimd->N * pimd->P / (2 * pimd->beta);
  XMD_CUDA(xk::vbn_energy(pimd->N, pimd->beta, pimd->vi, add, pd->ENk.as<double>(), pd->VBN.as<double>(), nullptr,
                          acc, scr, stream(), cycle_probs(pimd, pd)));
  return 0;
}

int md_pimd_fast_fill_ENk2_x(md_pimd_t_x *pimd, int image) {
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(check_image(sd, image));
  XMD_CUDA(xk::fill_enk2(sd->geo, sd->x.as<double>(), sd->m.as<double>(), pimd->omegaP * pimd->omegaP, image,
                         pd->ENk2.as<double>(), stream()));
  return 0;
}

// the cubic entry point fills a different table than the fast one (only
// the virial estimator built on either agrees): md_pimd_x.c:3959-4056
int md_pimd_fill_ENk2_x(md_pimd_t_x *pimd, int image) {
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(check_image(sd, image));
  XMD_CUDA(xk::fill_enk2_cubic(sd->geo, sd->x.as<double>(), sd->m.as<double>(), pimd->omegaP * pimd->omegaP,
                               image, pd->ENk2.as<double>(), stream()));
  return 0;
}

int md_pimd_calc_vi_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int image) {
  SimDev *sd;
  PimdDev *pd;
  double *acc;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  XMD_TRY(check_image(sd, image));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  size_t need = general_scratch(sd->geo);
  if (need < xk::vbn_scratch_doubles(pimd->N)) need = xk::vbn_scratch_doubles(pimd->N);
  double *scr = scratch_for(sd, need, &rc);
  if (rc) return rc;
  cudaStream_t st = stream();
  const double add = D * pimd->N / (2 * pimd->beta);
  XMD_CUDA(xk::vbn_energy(pimd->N, pimd->beta, pimd->vi, add, pd->ENk.as<double>(), pd->VBN.as<double>(),
                          pd->ENk2.as<double>(), acc, scr, st, cycle_probs(pimd, pd)));
  XMD_CUDA(xk::force_virial(sd->geo, sd->x.as<double>(), sd->f.as<double>(), sd->m.as<double>(), image, acc, scr, st));
  return 0;
}

// md_pimd_x.c:3898-3922 and :3923-3955: the virial about the box centre and
// the centroid virial (plus (D N - fc/P) / (2 beta)), from the stored forces
static int virial_about(md_pimd_t_x *pimd, md_stats_t_x *stats, int mode, double add) {
  SimDev *sd;
  PimdDev *pd;
  double *acc;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  XMD_CUDA(xk::virial_about(sd->geo, sd->x.as<double>(), sd->f.as<double>(), sd->m.as<double>(), mode, add, acc, scr,
                            stream()));
  return 0;
}

int md_pimd_calc_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats) {
  if (!pimd || !pimd->sim || !pimd->sim->box || pimd->sim->box->type != MD_ND_RECT_BOX_X)
    return fail(MD_GB_ERR_ARG, "the virial about the box centre needs a rectangular box");
  return virial_about(pimd, stats, 0, 0.0);
}

int md_pimd_calc_centroid_virial_energy_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int fc) {
  if (!pimd) return fail(MD_GB_ERR_ARG, "NULL path-integral state");
  return virial_about(pimd, stats, 1, (D * pimd->N - fc / (double)pimd->P) / (2 * pimd->beta));
}

// md_pimd_x.c:4350-4374
int md_pimd_polymer_periodic_boundary_x(md_pimd_t_x *pimd) {
  if (!pimd || !pimd->sim || !pimd->sim->box || pimd->sim->box->type != MD_ND_RECT_BOX_X)
    return fail(MD_GB_ERR_ARG, "the polymer wrap needs a rectangular box");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_CUDA(xk::polymer_wrap(sd->geo, sd->x.as<double>(), stream()));
  return 0;
}

// md_pimd_x.c:2974-3109: g(r) between bead 1 and bead pi.  The distances
// are binned on the GPU (integer counts, each distance in the reference's
// bin); the counts then add 1/norm to stats->fxs[stats->N - 1] on the host,
// one addition per count as the reference does, so the sums are the
// reference's to the bit.
int md_pimd_calc_pair_correlation_x(md_pimd_t_x *pimd, md_stats_t_x *stats, md_num_t_x rmax, md_num_t_x norm, int pi,
                                    int image) {
  if (!stats || !stats->fxs) return fail(MD_GB_ERR_ARG, "NULL accumulator");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "reads a result back; not while capturing");
  if (stats->points < 1) return 0;
  if (!(rmax > 0)) return fail(MD_GB_ERR_ARG, "rmax must be positive");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_image(sd, image));
  if (pi < 1 || pi > pimd->P) return fail(MD_GB_ERR_ARG, "bead index pi must be in 1..P");
  const int pts = stats->points;
  XMD_TRY(reserve(pd->sk_buf, sizeof(unsigned int) * (size_t)pts));
  cudaStream_t st = stream();
  std::vector<unsigned int> cnt(pts);
  XMD_CUDA(xk::pair_hist(sd->geo, sd->x.as<double>(), pi - 1, pts, rmax, image, pd->sk_buf.as<unsigned int>(), st));
  XMD_CUDA(cudaMemcpyAsync(cnt.data(), pd->sk_buf.p, sizeof(unsigned int) * pts, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (!md_stats_sync_host_x(stats)) return -1;
  const double w = 1.0 / norm;
  for (int k = 0; k < pts; ++k) {
    double v = stats->fxs[stats->N - 1][k];
    for (unsigned int c = 0; c < cnt[k]; ++c) v += w;
    stats->fxs[stats->N - 1][k] = v;
  }
  return 0;
}

int md_pimd_calc_trap_energy_x(md_pimd_t_x *pimd, md_trap_energy_t_x te, md_stats_t_x *stats) {
  const int kind = trap_kind_of((const void *)te, true);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "trap energy function has no device kernel");
  SimDev *sd;
  PimdDev *pd;
  double *acc;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  XMD_CUDA(xk::trap_energy(sd->geo, trap_params(kind), sd->x.as<double>(), sd->m.as<double>(), acc, scr, stream()));
  return 0;
}

int md_pimd_calc_pair_energy_x(md_pimd_t_x *pimd, md_pair_energy_t_x pe, md_stats_t_x *stats) {
  const int kind = pair_kind_of((const void *)pe, true);
  if (!kind) return fail(MD_GB_ERR_UNSUPPORTED, "pair energy function has no device kernel");
  SimDev *sd;
  PimdDev *pd;
  double *acc;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  if (kind == xk::PAIR_EWALD_REAL && D != 3) return 0;
  if (kind == xk::PAIR_PERIODIC_GAUSSIAN || kind == xk::PAIR_PERIODIC_COULOMB || kind == xk::PAIR_EWALD_REAL)
    XMD_TRY(check_image(sd, 1));
  XMD_TRY(stats_device(stats, &acc));
  int rc;
  double *scr = scratch_for(sd, general_scratch(sd->geo), &rc);
  if (rc) return rc;
  cudaStream_t st = stream();
  if (kind == xk::PAIR_EWALD_REAL) {
    XMD_TRY(ewald_tables(pimd, sd, pd));
    if (learned_mode(pimd, false) == 1) {
      XMD_TRY(learned_recip_energy(pimd, sd, acc, scr));
    } else {
      XMD_CUDA(xk::recip_energy(sd->geo, recip_of(pd), sd->x.as<double>(), acc, scr, st));
    }
  }
  xk::PairPrm prm = pair_params(kind);
  ewald_shifts(prm, sd->geo);
  if (kind == xk::PAIR_EWALD_REAL && (prm.kmax[0] > 1 || prm.kmax[1] > 1 || prm.kmax[2] > 1))
    return fail(MD_GB_ERR_UNSUPPORTED, "Ewald alpha*L below %.1f (images beyond the neighbouring boxes)",
                2 * EWALD_XCUT / 3);
  XMD_CUDA(xk::pair_energy(sd->geo, prm, sd->x.as<double>(), acc, scr, st));
  return 0;
}

// ------------------------------------------------------------------
// host-side helpers on synchronised data (md_pimd_x.c:569-591, :667-812,
// :955-965, :2213-2342, :4058-4070, :4652-4706)
// ------------------------------------------------------------------
md_num_t_x md_pimd_ENk_x(md_pimd_t_x *pimd, int N2, int k, int image) {
  md_simulation_t_x *sim = md_simulation_sync_host_x(pimd->sim, 1);
  if (!sim) return NAN;
  const double *L = sim->box && sim->box->box ? ((nd_rect_t_x *)sim->box->box)->L : nullptr;
  double e = 0;
  for (int l = N2 - k + 1; l <= N2; ++l)
    for (int j = 1; j <= pimd->P; ++j) {
      const md_particle_t_x *a = &sim->particles[MD_PIMD_INDEX_X(l, j, pimd->P)];
      const md_particle_t_x *b = &sim->particles[md_pimd_next_index_x(l, j, N2, k, pimd->P)];
      const double r = image ? md_minimum_image_distance_x((double *)a->x, (double *)b->x, (double *)L)
                             : md_distance_x((double *)a->x, (double *)b->x);
      e += 0.5 * a->m * pimd->omegaP * pimd->omegaP * r * r;
    }
  return e;
}

static int print_tri(FILE *out, const char *tag, md_pimd_t_x *pimd, md_num_t_x **tab) {
  if (!md_pimd_sync_host_x(pimd, 1)) return -1;
  fprintf(out, "%s %d\n", tag, pimd->N);
  for (int l = 1; l <= pimd->N; ++l) {
    for (int k = 1; k <= l; ++k) fprintf(out, "%f ", tab[l - 1][k - 1]);
    fprintf(out, "\n");
  }
  return ferror(out);
}

int md_pimd_fprint_ENk_x(FILE *out, md_pimd_t_x *pimd) { return print_tri(out, "ENk", pimd, pimd->ENk); }
int md_pimd_fprint_ENk2_x(FILE *out, md_pimd_t_x *pimd) { return print_tri(out, "ENk2", pimd, pimd->ENk2); }

int md_pimd_fprint_VBN_x(FILE *out, md_pimd_t_x *pimd) {
  if (!md_pimd_sync_host_x(pimd, 1)) return -1;
  fprintf(out, "VBN %d\n", pimd->N);
  for (int i = 0; i <= pimd->N; ++i) fprintf(out, "%f ", pimd->VBN[i]);
  fprintf(out, "\n");
  return ferror(out);
}

md_num_t_x md_pimd_xexp_x(md_num_t_x k, md_num_t_x E, md_num_t_x EE, md_num_t_x beta, md_num_t_x vi) {
  return vi == 0.0 ? exp(-beta * E + EE) : exp((k - 1) * log(vi) - beta * E + EE);
}

md_num_t_x md_pimd_fast_xexp_x(md_num_t_x l, md_num_t_x k, md_num_t_x E, md_num_t_x EE, md_num_t_x beta,
                               md_num_t_x vi) {
  return vi == 0.0 ? exp(-beta * E + EE - log(l)) : exp((k - 1) * log(vi) - beta * E + EE - log(l));
}

// log-sum-exp shift over the cycles ending at particle N2 for a given
// xi and V_B table (also used for the xi' reweighting)
static double min_shift(md_pimd_t_x *p, int N2, const double *V, double vi) {
  if (vi == 0.0) return p->beta * (p->ENk[N2 - 1][0] + V[N2 - 1]);
  double m = 1e10;
  for (int k = 1; k <= N2; ++k) {
    const double t = -(k - 1) * log(vi) + p->beta * (p->ENk[N2 - 1][k - 1] + V[N2 - k]);
    if (t < m) m = t;
  }
  return m;
}

md_num_t_x md_pimd_xminE_x(md_pimd_t_x *pimd, int N2) {
  if (!md_pimd_sync_host_x(pimd, 1)) return NAN;
  return min_shift(pimd, N2, pimd->VBN, pimd->vi);
}

md_num_t_x md_pimd_xminE2_x(md_pimd_t_x *pimd, int N2, md_num_t_x *VBN2, md_num_t_x vi2) {
  if (!md_pimd_sync_host_x(pimd, 1)) return NAN;
  return min_shift(pimd, N2, VBN2, vi2);
}

md_num_t_x md_pimd_fast_xminE_x(md_pimd_t_x *pimd, int u, md_num_t_x *V) {
  if (!md_pimd_sync_host_x(pimd, 1)) return NAN;
  if (pimd->vi == 0.0) return log(u) + pimd->beta * (pimd->ENk[u - 1][0] + V[u]);
  double m = 1e10;
  for (int l = u; l <= pimd->N; ++l) {
    const int k = l - u + 1;
    const double t = -(k - 1) * log(pimd->vi) + log(l) + pimd->beta * (pimd->ENk[l - 1][k - 1] + V[l]);
    if (t < m) m = t;
  }
  return m;
}

// md_pimd_x.c:5404-5448: S(q) between bead 1 and bead pi of every particle
// for the first min(sk->N, stats->points) wave vectors, added to
// stats->fxs[stats->N - 1][j]; the sums over particles run on the GPU
int md_pimd_calc_sphere_Sk_structure_x(md_pimd_t_x *pimd, md_stats_t_x *stats, int pi, md_sk_sphere_t_x *sk) {
  if (!stats || !sk || !stats->fxs) return fail(MD_GB_ERR_ARG, "NULL argument");
  if (D != 3) return fail(MD_GB_ERR_UNSUPPORTED, "the spherical S(k) is 3D only");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "reads a result back; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  const int n = sk->N < stats->points ? sk->N : stats->points;
  if (n <= 0) return 0;
  if (pi < 1) return fail(MD_GB_ERR_ARG, "bead index pi must be >= 1");
  const int jb = (pi - 1) % pimd->P;
  XMD_TRY(reserve(pd->sk_buf, sizeof(double) * 4 * (size_t)n));
  cudaStream_t st = stream();
  double *qd = pd->sk_buf.as<double>(), *out = qd + 3 * (size_t)n;
  std::vector<double> res(n);
  XMD_CUDA(cudaMemcpyAsync(qd, sk->qis, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, st));
  XMD_CUDA(xk::sk_structure(sd->geo, sd->x.as<double>(), 0, jb, qd, n, out, st));
  XMD_CUDA(cudaMemcpyAsync(res.data(), out, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (!md_stats_sync_host_x(stats)) return -1;
  for (int j = 0; j < n; ++j) stats->fxs[stats->N - 1][j] += res[j];
  return 0;
}

// signed V_B for xi' (possibly negative) on the current ENk, on the GPU:
// the same extended-range solve as V_B with the terms of odd k-1 negated
// for xi' < 0 (md_pimd_x.c:4665-4706).  Both accumulators' es[0] are then
// multiplied by sign * exp(-beta (V'_N - V_N)), on the host as in the
// reference.
int md_pimd_calc_vi_sign_x(md_pimd_t_x *pimd, md_stats_t_x *e_s, md_stats_t_x *s_s, md_num_t_x vi2) {
  if (!e_s || !s_s) return fail(MD_GB_ERR_ARG, "NULL accumulator");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "reads a result back; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(check_plain(pimd));
  const int N = pimd->N;
  // its own weight scratch behind V2 and the signs: the recursions' scratch
  // (pd->rec) holds the weights and unknowns the next force call reads
  const size_t need = sizeof(double) * (2 * (size_t)(N + 1) + xk::rec_scratch_doubles(N));
  cudaStream_t st = stream();
  if (pd->vsign.bytes < need) {
    XMD_TRY(reserve(pd->vsign, need));
    XMD_CUDA(cudaMemsetAsync(pd->vsign.p, 0, need, st));
  }
  double *V2 = pd->vsign.as<double>(), *sg = V2 + (N + 1);
  XMD_CUDA(xk::fill_vb_signed(N, pimd->beta, vi2, pd->ENk.as<double>(), pd->lnn.as<double>(), V2, sg,
                              V2 + 2 * (N + 1), st));
  double r[3];
  XMD_CUDA(cudaMemcpyAsync(&r[0], V2 + N, 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(&r[1], sg + N, 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(&r[2], pd->VBN.as<double>() + N, 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (!md_stats_sync_host_x(e_s) || !md_stats_sync_host_x(s_s)) return -1;
  const double s = r[1] * exp(-pimd->beta * r[0] + pimd->beta * r[2]);
  e_s->es[0] *= s;
  s_s->es[0] *= s;
  return 0;
}

}  // extern "C"
