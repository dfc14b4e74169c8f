// xmd_learned_api.cpp -- md_gb300_ewald_model_*_x: the learned residual of a
// truncated Ewald reciprocal sum (no counterpart in MD-Lab).
//
// A model belongs to one system shape (N, P, box, Ewald alpha and strength).
// collect() adds the current configuration of every bead slice to a data set
// held in HBM: descriptors of each particle and the difference between the
// converged reciprocal sum (the n_sum set with md_set_coulomb_*) and the
// truncated one (n_sum_cheap), for forces and per-particle energies, both in
// FP64.  train() runs Adam steps of the tensor-core training kernel on random
// batches of that set.  attach() makes md_pimd_calc_pair_force_x /
// md_pimd_calc_pair_energy_x with md_coulomb_3d_ewald_* use the truncated
// sum plus the network; every judge_every-th force call (outside graph
// capture) computes the converged sum instead, measures the network's error
// on that configuration and drops the network for good when the error is
// above the tolerances.
#include <cmath>
#include <cstring>
#include <iterator>
#include <map>
#include <random>
#include <vector>

#include "xmd_internal.h"
#include "xmd_learned.cuh"

using namespace xmd;

static const int D = MD_DIMENSION_X;

struct md_gb300_ewald_model {
  int N = 0, P = 0, Ns = 0, nsum_cheap = 3;
  double box[3] = {0, 0, 0}, alpha = 0, qs = 0;
  int rows_cfg = 0;  // rows of one configuration, padded to a tile
  long cap_cfg = 0, ncollected = 0;
  DevBuf par, grad, m1, m2, w1, w2, w3, w3f, lossacc, err;
  DevBuf basis, fmean, fistd;
  DevBuf dkv, dsn, dsh;  // descriptor wave vectors, shell normalisation, per-slice shell features
  DevBuf dsx, dsv, dst;
  DevBuf lx, lv, ly, raw;
  DevBuf fa, fb, ea, eb, fp, ep, jacc;
  DevBuf rc_coef, rc_cols, rc_phase, rc_S, rc_T;
  xk::Recip cheap{};
  xk::DescPrm dp{};
  xk::ResidPrm rp{0.f, 1.f, 1.f};
  bool normalized = false;
  int adam_t = 0;
  uint32_t seed = 1;
  double vsig[3] = {0, 0, 0};
  // attachment and judging
  int judge_every = 0;
  double ftol = 0, etol = 0;
  long calls = 0;
  int judged = 0;
  bool reverted = false;
  double last[4] = {NAN, NAN, NAN, NAN};
  // the network's branch of a learned force call (descriptors and forward
  // pass need only positions, so they run beside the truncated Ewald sums)
  cudaStream_t ms = nullptr;
  cudaEvent_t mfork = nullptr, mdone = nullptr;
};

typedef md_gb300_ewald_model Model;
static std::map<const void *, Model *> g_attached;

static xk::MlpDev dev_view(Model *M) {
  xk::MlpDev w{};
  w.w1img = M->w1.as<uint8_t>();
  w.w2img = M->w2.as<uint8_t>();
  w.w3img = M->w3.as<uint8_t>();
  w.b1 = M->par.as<float>() + xk::MLP_B1;
  w.b2 = M->par.as<float>() + xk::MLP_B2;
  w.b3 = M->par.as<float>() + xk::MLP_B3;
  w.w3f = M->w3f.as<float>();
  return w;
}

static int tiles_of(int rows) { return (rows + xk::MLP_TILE - 1) / xk::MLP_TILE; }

// The weight-gradient products read activation images "MN-major", with the
// stride between core matrices along M/N in the descriptor's stride field
// and the stride along K in its leading field (mdesc<0>).  The tensor-core
// self-test confirms that reading once per process before the first
// training step; a GPU that disagrees fails loudly instead of training on
// wrong gradients.
static int mn_variant(int *out) {
  static int checked = 0;
  if (!checked) {
    double e[5];
    XMD_CUDA(xk::tc_selftest(e, stream()));
    const double tol = 1e-3;
    if (!(e[0] < tol)) return fail(MD_GB_ERR_CUDA, "tensor-core self-test: K-major product off by %g", e[0]);
    if (!(e[1] < tol && e[3] < tol))
      return fail(MD_GB_ERR_CUDA, "tensor-core self-test: MN-major operands off by %g / %g", e[1], e[3]);
    checked = 1;
  }
  *out = 0;
  return 0;
}

// 32 lowest |n|^2 > 0 of the reciprocal lattice (sums of three squares)
static std::vector<int> lowest_shells(int count) {
  std::vector<int> s;
  for (int n2 = 1; (int)s.size() < count; ++n2) {
    bool ok = false;
    for (int a = 0; a * a <= n2 && !ok; ++a)
      for (int b = 0; a * a + b * b <= n2 && !ok; ++b) {
        const int c2 = n2 - a * a - b * b, c = (int)lround(sqrt((double)c2));
        if (c * c == c2) ok = true;
      }
    if (ok) s.push_back(n2);
  }
  return s;
}

// histogram -> radial features: 32 Gaussians in r (centres 0.5 .. rc,
// width their spacing) evaluated at the bin centres
static void make_basis(double rc, std::vector<float> &B) {
  B.assign((size_t)xk::DESC_BINS * 32, 0.f);
  const double h = rc / xk::DESC_BINS, sp = (rc - 0.5) / 31.0;
  for (int b = 0; b < xk::DESC_BINS; ++b) {
    const double r = (b + 0.5) * h;
    for (int f = 0; f < 32; ++f) {
      const double mu = 0.5 + f * sp;
      B[(size_t)b * 32 + f] = (float)exp(-(r - mu) * (r - mu) / (2 * sp * sp));
    }
  }
}

// half-space wave vectors n (nx > 0; or nx = 0, ny > 0; or nx = ny = 0,
// nz > 0) of the DESC_SHELLS lowest shells |n|^2, as (nx, ny, nz, shell),
// and the number of vectors per shell
static void shell_vectors(std::vector<int> &kv, std::vector<int> &count, int &nmax) {
  const std::vector<int> sh = lowest_shells(xk::DESC_SHELLS);
  const int top = sh.back();
  nmax = (int)floor(sqrt((double)top));
  count.assign(xk::DESC_SHELLS, 0);
  kv.clear();
  for (int a = 0; a <= nmax; ++a)
    for (int b = -nmax; b <= nmax; ++b)
      for (int c = -nmax; c <= nmax; ++c) {
        if (!(a > 0 || (a == 0 && b > 0) || (a == 0 && b == 0 && c > 0))) continue;
        const int n2 = a * a + b * b + c * c;
        for (int s2 = 0; s2 < xk::DESC_SHELLS; ++s2)
          if (sh[s2] == n2) {
            kv.insert(kv.end(), {a, b, c, s2});
            count[s2]++;
          }
      }
}

static int geometry_matches(Model *M, SimDev *sd) {
  const xk::Geo &g = sd->geo;
  if (g.N != M->N || g.P != M->P || g.Ns != M->Ns || g.box[0] != M->box[0] || g.box[1] != M->box[1] ||
      g.box[2] != M->box[2])
    return fail(MD_GB_ERR_ARG, "system shape differs from the one the model was made for");
  if (md_coulomb_truc_x != M->alpha || md_coulomb_strength_x != M->qs)
    return fail(MD_GB_ERR_ARG, "Ewald alpha or strength differs from the model's");
  return 0;
}

static int zero(DevBuf &b) {
  XMD_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, stream()));
  return 0;
}

// converged and truncated reciprocal forces (raw, FP64) and per-particle
// energies of the bead slices g covers (x: the first of them) into fa/ea
// and fb/eb
static int both_sums(Model *M, md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd, const xk::Geo &g, const double *x) {
  XMD_TRY(ewald_tables(pimd, sd, pd));
  XMD_TRY(zero(M->fa));
  XMD_TRY(zero(M->fb));
  XMD_CUDA(xk::recip_force_energy(g, recip_of(pd), x, 1.0, M->fa.as<double>(), M->ea.as<double>(), stream()));
  XMD_CUDA(xk::recip_force_energy(g, M->cheap, x, 1.0, M->fb.as<double>(), M->eb.as<double>(), stream()));
  return 0;
}
static int both_sums(Model *M, md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd) {
  return both_sums(M, pimd, sd, pd, sd->geo, sd->x.as<double>());
}

// descriptors and network output of the bead slices g covers (live buffers)
static int predict(Model *M, const xk::Geo &g, const double *x, cudaStream_t st) {
  XMD_CUDA(xk::desc_build(g, M->dp, x, M->lx.as<uint8_t>(), M->lv.as<float>(), nullptr, st));
  XMD_CUDA(xk::mlp_forward(dev_view(M), M->lx.as<uint8_t>(), tiles_of(g.N * g.P), M->ly.as<float4>(),
                           M->err.as<int>(), st));
  return 0;
}
static int predict(Model *M, SimDev *sd, cudaStream_t st) { return predict(M, sd->geo, sd->x.as<double>(), st); }

// normalisation of inputs and outputs from the first configuration
static int normalise(Model *M, SimDev *sd) {
  cudaStream_t st = stream();
  const int rows = M->N * M->P;
  XMD_CUDA(xk::desc_build(sd->geo, M->dp, sd->x.as<double>(), M->lx.as<uint8_t>(), M->lv.as<float>(),
                          M->raw.as<float>(), st));
  std::vector<float> F((size_t)rows * 64), V((size_t)rows * xk::DESC_VSTRIDE);
  const size_t ns = sd->geo.slots(), ne = (size_t)M->P * M->Ns;
  std::vector<double> fa(ns), fb(ns), ea(ne), eb(ne);
  XMD_CUDA(cudaMemcpyAsync(F.data(), M->raw.p, F.size() * 4, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(V.data(), M->lv.p, V.size() * 4, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(fa.data(), M->fa.p, ns * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(fb.data(), M->fb.p, ns * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(ea.data(), M->ea.p, ne * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(eb.data(), M->eb.p, ne * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  std::vector<float> mean(64), istd(64);
  for (int f = 0; f < 64; ++f) {
    double s = 0, s2 = 0;
    for (int r = 0; r < rows; ++r) {
      s += F[(size_t)r * 64 + f];
      s2 += (double)F[(size_t)r * 64 + f] * F[(size_t)r * 64 + f];
    }
    const double m = s / rows, var = fmax(s2 / rows - m * m, 0.0), sd_ = sqrt(var);
    mean[f] = (float)m;
    istd[f] = (float)(1.0 / fmax(sd_, 1e-6 * (fabs(m) + 1.0)));
  }
  for (int m = 0; m < 3; ++m) {
    double s2 = 0;
    for (int r = 0; r < rows; ++r)
      for (int d = 0; d < 3; ++d) s2 += (double)V[(size_t)r * xk::DESC_VSTRIDE + 3 * m + d] * V[(size_t)r * xk::DESC_VSTRIDE + 3 * m + d];
    const double rms = sqrt(s2 / rows);
    M->dp.vscale[m] = (float)(rms > 0 ? 1.0 / rms : 1.0);
  }
  double es = 0, es2 = 0, fs2 = 0;
  for (int j = 0; j < M->P; ++j)
    for (int l = 0; l < M->N; ++l) {
      const double e = ea[(size_t)j * M->Ns + l] - eb[(size_t)j * M->Ns + l];
      es += e;
      es2 += e * e;
      for (int d = 0; d < 3; ++d) {
        const size_t q = xk::sidx(j, d, l, 3, M->Ns);
        fs2 += (fa[q] - fb[q]) * (fa[q] - fb[q]);
      }
    }
  const double em = es / rows, esd = sqrt(fmax(es2 / rows - em * em, 0.0)), frms = sqrt(fs2 / (3.0 * rows));
  M->rp.e_mean = (float)em;
  M->rp.e_scale = (float)(esd > 0 ? esd : 1.0);
  M->rp.f_scale = (float)(frms > 0 ? frms : 1.0);
  XMD_CUDA(cudaMemcpyAsync(M->fmean.p, mean.data(), 64 * 4, cudaMemcpyHostToDevice, st));
  XMD_CUDA(cudaMemcpyAsync(M->fistd.p, istd.data(), 64 * 4, cudaMemcpyHostToDevice, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  M->normalized = true;
  return 0;
}

// A judgement evaluates the converged and truncated FP64 reciprocal sums and
// the network on JUDGE_SLICES consecutive bead slices, a different block each
// time (every slice is judged in turn): the errors are averages over
// N x JUDGE_SLICES particle-slices, at a fraction of the cost of all of them.
constexpr int JUDGE_SLICES = 8;

static int judge_now(Model *M, md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd, double out[4]) {
  if (!M->normalized) return fail(MD_GB_ERR_ARG, "the model has no data yet");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "judging reads results back; not while capturing");
  cudaStream_t st = stream();
  xk::Geo g = sd->geo;
  const int pj = M->P < JUDGE_SLICES ? M->P : JUDGE_SLICES;
  int j0 = (int)(((long)M->judged * pj) % M->P);
  if (j0 + pj > M->P) j0 = M->P - pj;
  g.P = pj;
  const double *x = sd->x.as<double>() + (size_t)j0 * 3 * g.Ns;
  XMD_TRY(both_sums(M, pimd, sd, pd, g, x));
  XMD_TRY(predict(M, g, x, stream()));
  XMD_CUDA(xk::resid_apply(g, M->rp, M->ly.as<float4>(), M->lv.as<float>(), 1.0, nullptr, M->fp.as<double>(),
                           M->ep.as<double>(), st));
  XMD_TRY(zero(M->jacc));
  XMD_CUDA(xk::resid_judge(g, M->fp.as<double>(), M->fa.as<double>(), M->fb.as<double>(), M->ep.as<double>(),
                           M->ea.as<double>(), M->eb.as<double>(), M->jacc.as<double>(), st));
  std::vector<double> acc(3 + 2 * (size_t)pj);
  int kerr = 0;
  XMD_CUDA(cudaMemcpyAsync(acc.data(), M->jacc.p, acc.size() * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(&kerr, M->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (kerr) return fail(MD_GB_ERR_CUDA, "tensor-core kernel reported error %d (wait timed out)", kerr);
  double em = 0, et = 0;
  for (int j = 0; j < pj; ++j) {
    em += acc[3 + j];
    et += acc[3 + pj + j];
  }
  const double norm = acc[1] > 0 ? acc[1] : 1.0, np = (double)M->N * pj;
  out[0] = sqrt(acc[0] / norm);
  out[1] = fabs(em) / np;
  out[2] = sqrt(acc[2] / norm);
  out[3] = fabs(et) / np;
  for (int i = 0; i < 4; ++i) M->last[i] = out[i];
  M->judged += 1;
  return 0;
}

namespace xmd {

static Model *attached(const void *pimd) {
  auto it = g_attached.find(pimd);
  return it == g_attached.end() ? nullptr : it->second;
}

int learned_mode(md_pimd_t_x *pimd, bool count_call) {
  Model *M = attached(pimd);
  if (!M || M->reverted || !M->normalized) return 0;
  if (count_call && M->judge_every > 0 && !capturing())
    if (++M->calls % M->judge_every == 0) return 2;
  return 1;
}

int learned_pair_force(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd, const xk::PairPrm &prm, double *scr) {
  Model *M = attached(pimd);
  XMD_TRY(geometry_matches(M, sd));
  (void)pd;
  cudaStream_t st = stream();
  const double inv_mP = 1.0 / (sd->mass0 * pimd->P);
  const double *x = sd->x.as<double>();
  double *f = sd->f.as<double>();
  // fork: the network's branch on its own stream, joined before its
  // forces are added (graph capture records the fork and the join)
  if (!M->ms) {
    XMD_CUDA(cudaStreamCreateWithFlags(&M->ms, cudaStreamNonBlocking));
    XMD_CUDA(cudaEventCreateWithFlags(&M->mfork, cudaEventDisableTiming));
    XMD_CUDA(cudaEventCreateWithFlags(&M->mdone, cudaEventDisableTiming));
  }
  XMD_CUDA(cudaEventRecord(M->mfork, st));
  XMD_CUDA(cudaStreamWaitEvent(M->ms, M->mfork, 0));
  XMD_TRY(predict(M, sd, M->ms));
  XMD_CUDA(cudaEventRecord(M->mdone, M->ms));
  // timing each kernel alone: the network's branch is joined at once
  if (xk::profiling() && !capturing()) XMD_CUDA(cudaStreamWaitEvent(st, M->mdone, 0));
  if (md_gb300_get_precision_x() == MD_GB_PRECISION_MIXED) {
    XMD_CUDA(xk::recip_force32(sd->geo, M->cheap, x, inv_mP, f, st));
    XMD_CUDA(xk::pair_force32(sd->geo, prm, x, sd->m.as<double>(), f, scr, st));
  } else {
    XMD_CUDA(xk::recip_force(sd->geo, M->cheap, x, inv_mP, f, st));
    XMD_CUDA(xk::pair_force(sd->geo, prm, x, sd->m.as<double>(), f, scr, st));
  }
  XMD_CUDA(cudaStreamWaitEvent(st, M->mdone, 0));
  XMD_CUDA(xk::resid_apply(sd->geo, M->rp, M->ly.as<float4>(), M->lv.as<float>(), inv_mP, f, nullptr, nullptr, st));
  return 0;
}

int learned_judge_step(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd) {
  Model *M = attached(pimd);
  double out[4];
  XMD_TRY(judge_now(M, pimd, sd, pd, out));
  if (!(out[0] <= M->ftol) || !(out[1] <= M->etol)) M->reverted = true;
  return 0;
}

int learned_recip_energy(md_pimd_t_x *pimd, SimDev *sd, double *acc, double *scr) {
  Model *M = attached(pimd);
  XMD_TRY(geometry_matches(M, sd));
  cudaStream_t st = stream();
  XMD_CUDA(xk::recip_energy(sd->geo, M->cheap, sd->x.as<double>(), acc, scr, st));
  XMD_TRY(predict(M, sd, stream()));
  XMD_CUDA(xk::resid_apply(sd->geo, M->rp, M->ly.as<float4>(), M->lv.as<float>(), 0.0, nullptr, M->fp.as<double>(),
                           M->ep.as<double>(), st));
  XMD_CUDA(xk::sum_particles(sd->geo, M->ep.as<double>(), 1.0 / M->P, acc, st));
  return 0;
}

}  // namespace xmd

// ------------------------------------------------------------------
// public entry points (md_gb300_x.h)
// ------------------------------------------------------------------
extern "C" {

int md_gb300_ewald_model_nparam_x(void) { return xk::MLP_NPARAM; }

int md_gb300_tc_selftest_x(double err[5]) {
  XMD_TRY(ensure_device());
  if (!err) return fail(MD_GB_ERR_ARG, "NULL error array");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "self-test while capturing");
  XMD_CUDA(xk::tc_selftest(err, stream()));
  return 0;
}

int md_gb300_set_wait_limit_x(long long cycles) {
  if (cycles < 1) return fail(MD_GB_ERR_ARG, "wait limit must be positive");
  xk::set_wait_limit(cycles);
  return 0;
}

long long md_gb300_get_wait_limit_x(void) { return xk::wait_limit(); }

int md_gb300_wait_selftest_x(long long cycles, int *status, long long *waited) {
  XMD_TRY(ensure_device());
  if (!status || cycles < 1) return fail(MD_GB_ERR_ARG, "wait self-test: NULL status or non-positive limit");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "self-test while capturing");
  long long w = 0;
  XMD_CUDA(xk::wait_probe(cycles, status, &w, stream()));
  if (waited) *waited = w;
  return 0;
}

void md_gb300_ewald_model_free_x(md_gb300_ewald_model_t_x *M) {
  if (!M) return;
  for (auto it = g_attached.begin(); it != g_attached.end();)
    it = it->second == M ? g_attached.erase(it) : std::next(it);
  DevBuf *bufs[] = {&M->par,  &M->grad, &M->m1,   &M->m2,    &M->w1,      &M->w2,   &M->w3,   &M->w3f,  &M->lossacc,
                    &M->err,  &M->basis, &M->fmean, &M->fistd, &M->dsx,   &M->dsv,  &M->dst,  &M->lx,   &M->lv,
                    &M->ly,   &M->raw,  &M->fa,   &M->fb,    &M->ea,      &M->eb,   &M->fp,   &M->ep,   &M->jacc,
                    &M->rc_coef, &M->rc_cols, &M->rc_phase, &M->rc_S, &M->rc_T, &M->dkv, &M->dsn, &M->dsh};
  for (DevBuf *b : bufs) release(*b);
  if (M->ms) {
    cudaStreamSynchronize(M->ms);
    cudaStreamDestroy(M->ms);
    cudaEventDestroy(M->mfork);
    cudaEventDestroy(M->mdone);
  }
  delete M;
}

int md_gb300_ewald_model_create_x(md_gb300_ewald_model_t_x **out, md_pimd_t_x *pimd, int nsum_cheap,
                                  long capacity_cfg, unsigned seed) {
  if (!out || !pimd) return fail(MD_GB_ERR_ARG, "NULL argument");
  *out = nullptr;
  if (D != 3) return fail(MD_GB_ERR_UNSUPPORTED, "the learned Ewald residual is 3D only");
  if (nsum_cheap < 1 || nsum_cheap > 11) return fail(MD_GB_ERR_ARG, "n_sum_cheap %d (1..11)", nsum_cheap);
  if (capacity_cfg < 1) return fail(MD_GB_ERR_ARG, "capacity must hold at least one configuration");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "model creation allocates; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  const xk::Geo &g = sd->geo;
  for (int d = 0; d < 3; ++d)
    if (!(g.box[d] > 0)) return fail(MD_GB_ERR_ARG, "the learned residual needs a periodic box");
  if (!(md_coulomb_truc_x > 0)) return fail(MD_GB_ERR_ARG, "set the Ewald parameters first");
  if (nsum_cheap >= md_coulomb_n_sum_x)
    return fail(MD_GB_ERR_ARG, "n_sum_cheap %d is not below the converged n_sum %d", nsum_cheap, md_coulomb_n_sum_x);
  if (!sd->uniform_mass) return fail(MD_GB_ERR_UNSUPPORTED, "structure-factor Ewald needs equal bead masses");
  Model *M = new Model();
  M->N = g.N;
  M->P = g.P;
  M->Ns = g.Ns;
  for (int d = 0; d < 3; ++d) M->box[d] = g.box[d];
  M->alpha = md_coulomb_truc_x;
  M->qs = md_coulomb_strength_x;
  M->nsum_cheap = nsum_cheap;
  M->rows_cfg = tiles_of(g.N * g.P) * xk::MLP_TILE;
  M->cap_cfg = capacity_cfg;
  M->seed = seed ? seed : 1u;
  const size_t rows = M->rows_cfg, tile_bytes = xk::MLP_TILE_BYTES;
  const size_t slots = g.slots(), ne = (size_t)g.P * g.Ns;
  int rc = 0;
  auto res = [&](DevBuf &b, size_t bytes) {
    if (!rc) rc = reserve(b, bytes);
    if (!rc && cudaMemsetAsync(b.p, 0, bytes, stream()) != cudaSuccess) rc = fail(MD_GB_ERR_CUDA, "memset");
  };
  res(M->par, 4 * xk::MLP_NPARAM);
  res(M->grad, 4 * xk::MLP_NPARAM);
  res(M->m1, 4 * xk::MLP_NPARAM);
  res(M->m2, 4 * xk::MLP_NPARAM);
  res(M->w1, 16384);
  res(M->w2, 32768);
  res(M->w3, 4096);
  res(M->w3f, 4 * 512);
  res(M->lossacc, 16);
  res(M->err, 16);
  res(M->basis, 4 * xk::DESC_BINS * 32);
  std::vector<int> kvh, kcount;
  int kmax = 0;
  shell_vectors(kvh, kcount, kmax);
  res(M->dkv, sizeof(int) * kvh.size());
  res(M->dsn, 4 * xk::DESC_SHELLS);
  res(M->dsh, 4 * (size_t)xk::DESC_SHELLS * g.P);
  res(M->fmean, 4 * 64);
  res(M->fistd, 4 * 64);
  res(M->dsx, (size_t)capacity_cfg * (rows / xk::MLP_TILE) * tile_bytes);
  res(M->dsv, (size_t)capacity_cfg * rows * xk::DESC_VSTRIDE * 4);
  res(M->dst, (size_t)capacity_cfg * rows * 16);
  res(M->lx, (rows / xk::MLP_TILE) * tile_bytes);
  res(M->lv, rows * xk::DESC_VSTRIDE * 4);
  res(M->ly, rows * 16);
  res(M->raw, rows * 64 * 4);
  res(M->fa, slots * 8);
  res(M->fb, slots * 8);
  res(M->fp, slots * 8);
  res(M->ea, ne * 8);
  res(M->eb, ne * 8);
  res(M->ep, ne * 8);
  res(M->jacc, (3 + 2 * (size_t)g.P) * 8);
  const int nk = xk::recip_count(nsum_cheap);
  res(M->rc_coef, xk::recip_coef_bytes(nk));
  res(M->rc_cols, sizeof(int) * xk::recip_cols_ints(nsum_cheap));
  res(M->rc_phase, 8 * xk::recip_phase_doubles(g, nsum_cheap) * 3 / 2);
  res(M->rc_S, 16 * (size_t)nk * g.P);
  res(M->rc_T, 8 * xk::recip_table_doubles(g, nsum_cheap));
  if (rc) {
    md_gb300_ewald_model_free_x(M);
    return rc;
  }
  M->cheap.coef = M->rc_coef.as<double>();
  M->cheap.kvec = M->rc_cols.as<int>();
  M->cheap.phase = M->rc_phase.as<double>();
  M->cheap.S = M->rc_S.as<double>();
  M->cheap.T = M->rc_T.as<double>();
  M->cheap.S32 = nullptr;  // no split: the truncated sums are all FP64 or all FP32
  cudaError_t e = xk::recip_setup(g, nsum_cheap, M->alpha, M->qs, M->cheap, stream());
  if (e != cudaSuccess) {
    md_gb300_ewald_model_free_x(M);
    return cuda_fail(e, "truncated Ewald tables");
  }
  // descriptors
  const double rcut = 0.5 * fmin(g.box[0], fmin(g.box[1], g.box[2]));
  std::vector<float> B;
  make_basis(rcut, B);
  std::vector<float> sn(xk::DESC_SHELLS);
  for (int i = 0; i < xk::DESC_SHELLS; ++i) sn[i] = (float)(1.0 / ((double)g.N * kcount[i]));
  M->dp.kvec = M->dkv.as<int4>();
  M->dp.nkvec = (int)(kvh.size() / 4);
  M->dp.nmax = kmax;
  M->dp.shell_norm = M->dsn.as<float>();
  M->dp.shell = M->dsh.as<float>();
  M->dp.rc = (float)rcut;
  M->dp.inv_h = (float)(xk::DESC_BINS / rcut);
  for (int d = 0; d < 3; ++d) {
    M->dp.box[d] = (float)g.box[d];
    M->dp.inv_box[d] = (float)(1.0 / g.box[d]);
    M->dp.vmu[d] = (float)(0.25 * (d + 1) * rcut);
    M->vsig[d] = 0.15 * rcut;
    M->dp.vinv2s2[d] = (float)(1.0 / (2 * M->vsig[d] * M->vsig[d]));
    M->dp.vscale[d] = 1.f;
  }
  {
    const double a = 1.0 / (2 * M->vsig[0] * M->vsig[0]), D = 0.25 * rcut, L2E = 1.4426950408889634;
    M->dp.qa = (float)(a * L2E);
    M->dp.qc1 = (float)(2 * a * D * L2E);
    M->dp.qc0 = (float)(-a * D * D * L2E);
    M->dp.qk = (float)exp(-2 * a * D * D);
  }
  M->dp.basis = M->basis.as<float>();
  M->dp.fmean = M->fmean.as<float>();
  M->dp.fistd = M->fistd.as<float>();
  // parameters: uniform Glorot initialisation, zero biases, small last layer
  std::vector<float> p(xk::MLP_NPARAM, 0.f);
  std::mt19937 rng(M->seed);
  auto fill = [&](int off, int fan_in, int fan_out, int n, double gain) {
    const double a = gain * sqrt(6.0 / (fan_in + fan_out));
    std::uniform_real_distribution<double> u(-a, a);
    for (int i = 0; i < n; ++i) p[off + i] = (float)u(rng);
  };
  fill(xk::MLP_W1, 64, 128, 128 * 64, 1.0);
  fill(xk::MLP_W2, 128, 128, 128 * 128, 1.0);
  fill(xk::MLP_W3, 128, 4, 4 * 128, 0.1);
  cudaStream_t st = stream();
  if ((e = cudaMemcpyAsync(M->basis.p, B.data(), B.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(M->dkv.p, kvh.data(), kvh.size() * sizeof(int), cudaMemcpyHostToDevice, st)) !=
          cudaSuccess ||
      (e = cudaMemcpyAsync(M->dsn.p, sn.data(), sn.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(M->par.p, p.data(), p.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
      (e = xk::mlp_pack(M->par.as<float>(), M->w1.as<uint8_t>(), M->w2.as<uint8_t>(), M->w3.as<uint8_t>(),
                        M->w3f.as<float>(), st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    md_gb300_ewald_model_free_x(M);
    return cuda_fail(e, "model initialisation");
  }
  *out = M;
  return 0;
}

int md_gb300_ewald_model_collect_x(md_gb300_ewald_model_t_x *M, md_pimd_t_x *pimd) {
  if (!M || !pimd) return fail(MD_GB_ERR_ARG, "NULL argument");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "collecting reads results back; not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(geometry_matches(M, sd));
  XMD_TRY(both_sums(M, pimd, sd, pd));
  if (!M->normalized) XMD_TRY(normalise(M, sd));
  const long slot = M->ncollected % M->cap_cfg;
  const size_t rows = M->rows_cfg;
  cudaStream_t st = stream();
  XMD_CUDA(xk::desc_build(sd->geo, M->dp, sd->x.as<double>(),
                          M->dsx.as<uint8_t>() + (size_t)slot * (rows / xk::MLP_TILE) * xk::MLP_TILE_BYTES,
                          M->dsv.as<float>() + (size_t)slot * rows * xk::DESC_VSTRIDE, nullptr, st));
  XMD_CUDA(xk::resid_targets(sd->geo, M->rp, M->fa.as<double>(), M->fb.as<double>(), M->ea.as<double>(),
                             M->eb.as<double>(), M->dst.as<float4>() + (size_t)slot * rows, st));
  M->ncollected += 1;
  return 0;
}

int md_gb300_ewald_model_train_x(md_gb300_ewald_model_t_x *M, int steps, int batch_tiles, double lr, double *loss) {
  if (!M || steps < 1 || batch_tiles < 1 || !(lr > 0)) return fail(MD_GB_ERR_ARG, "invalid training arguments");
  if (!M->ncollected) return fail(MD_GB_ERR_ARG, "the model has no data yet");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "training while capturing");
  int mnv;
  XMD_TRY(mn_variant(&mnv));
  cudaStream_t st = stream();
  const long cfgs = M->ncollected < M->cap_cfg ? M->ncollected : M->cap_cfg;
  const int ntiles = (int)(cfgs * (M->rows_cfg / xk::MLP_TILE));
  xk::MlpLoss L{1.f, 1.f, (float)(1.0 / ((double)batch_tiles * xk::MLP_TILE))};
  const xk::MlpDev w = dev_view(M);
  for (int s = 0; s < steps; ++s) {
    if (s == steps - 1) XMD_CUDA(cudaMemsetAsync(M->lossacc.p, 0, 8, st));
    M->adam_t += 1;
    const uint32_t sd = M->seed * 2654435761u + (uint32_t)M->adam_t * 40503u + 1u;
    XMD_CUDA(xk::mlp_train_grad(w, M->dsx.as<uint8_t>(), M->dsv.as<float>(), M->dst.as<float4>(), ntiles,
                                batch_tiles, sd ? sd : 1u, L, M->grad.as<float>(), M->lossacc.as<float>(), mnv,
                                M->err.as<int>(), st));
    xk::AdamPrm a{(float)lr, 0.9f, 0.999f, 1e-8f, (float)(1.0 / (1.0 - pow(0.9, M->adam_t))),
                  (float)(1.0 / (1.0 - pow(0.999, M->adam_t)))};
    XMD_CUDA(xk::mlp_adam(M->par.as<float>(), M->grad.as<float>(), M->m1.as<float>(), M->m2.as<float>(), a,
                          M->w1.as<uint8_t>(), M->w2.as<uint8_t>(), M->w3.as<uint8_t>(), M->w3f.as<float>(), st));
  }
  float la[2] = {0, 0};
  int kerr = 0;
  XMD_CUDA(cudaMemcpyAsync(la, M->lossacc.p, 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(&kerr, M->err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (kerr) return fail(MD_GB_ERR_CUDA, "tensor-core kernel reported error %d (wait timed out)", kerr);
  if (loss) *loss = (la[0] + la[1]) * L.inv_rows;
  return 0;
}

int md_gb300_ewald_model_attach_x(md_pimd_t_x *pimd, md_gb300_ewald_model_t_x *M, int judge_every, double force_tol,
                                  double energy_tol) {
  if (!pimd) return fail(MD_GB_ERR_ARG, "NULL path-integral state");
  if (!M) {
    g_attached.erase(pimd);
    return 0;
  }
  if (!M->normalized) return fail(MD_GB_ERR_ARG, "the model has no data yet");
  if (judge_every < 0) return fail(MD_GB_ERR_ARG, "judge interval must be >= 0");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(geometry_matches(M, sd));
  M->judge_every = judge_every;
  M->ftol = force_tol;
  M->etol = energy_tol;
  M->calls = 0;
  M->reverted = false;
  g_attached[pimd] = M;
  return 0;
}

int md_gb300_ewald_model_judge_x(md_gb300_ewald_model_t_x *M, md_pimd_t_x *pimd, double out[4]) {
  if (!M || !pimd || !out) return fail(MD_GB_ERR_ARG, "NULL argument");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(geometry_matches(M, sd));
  return judge_now(M, pimd, sd, pd, out);
}

int md_gb300_ewald_model_status_x(md_gb300_ewald_model_t_x *M, long *configurations, int *judged, int *reverted,
                                  double last[4]) {
  if (!M) return fail(MD_GB_ERR_ARG, "NULL model");
  if (configurations) *configurations = M->ncollected < M->cap_cfg ? M->ncollected : M->cap_cfg;
  if (judged) *judged = M->judged;
  if (reverted) *reverted = M->reverted ? 1 : 0;
  if (last)
    for (int i = 0; i < 4; ++i) last[i] = M->last[i];
  return 0;
}

int md_gb300_ewald_model_params_x(md_gb300_ewald_model_t_x *M, float *p, int set) {
  if (!M || !p) return fail(MD_GB_ERR_ARG, "NULL argument");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "parameter copy while capturing");
  cudaStream_t st = stream();
  if (set) {
    XMD_CUDA(cudaMemcpyAsync(M->par.p, p, 4 * xk::MLP_NPARAM, cudaMemcpyHostToDevice, st));
    XMD_CUDA(xk::mlp_pack(M->par.as<float>(), M->w1.as<uint8_t>(), M->w2.as<uint8_t>(), M->w3.as<uint8_t>(),
                          M->w3f.as<float>(), st));
  } else {
    XMD_CUDA(cudaMemcpyAsync(p, M->par.p, 4 * xk::MLP_NPARAM, cudaMemcpyDeviceToHost, st));
  }
  XMD_CUDA(cudaStreamSynchronize(st));
  return 0;
}

// X [rows][64] -> tile images (BF16), zero rows up to a whole tile
static std::vector<uint8_t> host_images(const float *X, int rows) {
  const int nt = tiles_of(rows);
  std::vector<uint8_t> img((size_t)nt * xk::MLP_TILE_BYTES, 0);
  for (int r = 0; r < rows; ++r)
    for (int k = 0; k < 64; ++k) {
      float f = X[(size_t)r * 64 + k];
      uint32_t u;
      memcpy(&u, &f, 4);
      if ((u & 0x7f800000u) != 0x7f800000u) u += 0x7fffu + ((u >> 16) & 1u);
      const uint16_t h = (uint16_t)(u >> 16);
      memcpy(&img[(size_t)(r / xk::MLP_TILE) * xk::MLP_TILE_BYTES + xk::kmaj_off(r % xk::MLP_TILE, k, 64)], &h, 2);
    }
  return img;
}

int md_gb300_mlp_forward_x(md_gb300_ewald_model_t_x *M, const float *X, int rows, float *Y) {
  if (!M || !X || !Y || rows < 1) return fail(MD_GB_ERR_ARG, "invalid arguments");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "not while capturing");
  const std::vector<uint8_t> img = host_images(X, rows);
  const int nt = tiles_of(rows);
  DevBuf dx, dy;
  int rc = reserve(dx, img.size());
  if (!rc) rc = reserve(dy, (size_t)nt * xk::MLP_TILE * 16);
  cudaStream_t st = stream();
  cudaError_t e = cudaSuccess;
  if (!rc) {
    if ((e = cudaMemcpyAsync(dx.p, img.data(), img.size(), cudaMemcpyHostToDevice, st)) == cudaSuccess &&
        (e = xk::mlp_forward(dev_view(M), dx.as<uint8_t>(), nt, dy.as<float4>(), M->err.as<int>(), st)) ==
            cudaSuccess &&
        (e = cudaMemcpyAsync(Y, dy.p, (size_t)rows * 16, cudaMemcpyDeviceToHost, st)) == cudaSuccess)
      e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) rc = cuda_fail(e, "network forward");
  }
  release(dx);
  release(dy);
  return rc;
}

int md_gb300_mlp_grad_x(md_gb300_ewald_model_t_x *M, const float *X, const float *V, const float *T, int rows,
                        double we, double wf, float *grad, float *loss) {
  if (!M || !X || !V || !T || !grad || rows < 1) return fail(MD_GB_ERR_ARG, "invalid arguments");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "not while capturing");
  int mnv;
  XMD_TRY(mn_variant(&mnv));
  const std::vector<uint8_t> img = host_images(X, rows);
  const int nt = tiles_of(rows);
  const size_t rp = (size_t)nt * xk::MLP_TILE;
  DevBuf dx, dv, dt;
  int rc = reserve(dx, img.size());
  if (!rc) rc = reserve(dv, rp * xk::DESC_VSTRIDE * 4);
  if (!rc) rc = reserve(dt, rp * 16);
  cudaStream_t st = stream();
  cudaError_t e = cudaSuccess;
  if (!rc) {
    xk::MlpLoss L{(float)we, (float)wf, (float)(1.0 / rows)};
    int kerr = 0;
    if ((e = cudaMemsetAsync(dv.p, 0, rp * xk::DESC_VSTRIDE * 4, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(dt.p, 0, rp * 16, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(dx.p, img.data(), img.size(), cudaMemcpyHostToDevice, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(dv.p, V, (size_t)rows * xk::DESC_VSTRIDE * 4, cudaMemcpyHostToDevice, st)) ==
            cudaSuccess &&
        (e = cudaMemcpyAsync(dt.p, T, (size_t)rows * 16, cudaMemcpyHostToDevice, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(M->grad.p, 0, 4 * xk::MLP_NPARAM, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(M->lossacc.p, 0, 8, st)) == cudaSuccess &&
        (e = xk::mlp_train_grad(dev_view(M), dx.as<uint8_t>(), dv.as<float>(), dt.as<float4>(), nt, nt, 0u, L,
                                M->grad.as<float>(), M->lossacc.as<float>(), mnv, M->err.as<int>(), st)) ==
            cudaSuccess &&
        (e = cudaMemcpyAsync(grad, M->grad.p, 4 * xk::MLP_NPARAM, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (!loss || (e = cudaMemcpyAsync(loss, M->lossacc.p, 8, cudaMemcpyDeviceToHost, st)) == cudaSuccess) &&
        (e = cudaMemcpyAsync(&kerr, M->err.p, sizeof(int), cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemsetAsync(M->grad.p, 0, 4 * xk::MLP_NPARAM, st)) == cudaSuccess)
      e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
      rc = cuda_fail(e, "network gradient");
    else if (kerr)
      rc = fail(MD_GB_ERR_CUDA, "tensor-core kernel reported error %d", kerr);
  }
  release(dx);
  release(dv);
  release(dt);
  return rc;
}

int md_gb300_ewald_model_features_x(md_gb300_ewald_model_t_x *M, md_pimd_t_x *pimd, float *F, float *V) {
  if (!M || !pimd || !F || !V) return fail(MD_GB_ERR_ARG, "NULL argument");
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "not while capturing");
  SimDev *sd;
  PimdDev *pd;
  XMD_TRY(pimd_device(pimd, &sd, &pd));
  XMD_TRY(geometry_matches(M, sd));
  cudaStream_t st = stream();
  const size_t rows = (size_t)M->N * M->P;
  XMD_CUDA(xk::desc_build(sd->geo, M->dp, sd->x.as<double>(), M->lx.as<uint8_t>(), M->lv.as<float>(),
                          M->raw.as<float>(), st));
  XMD_CUDA(cudaMemcpyAsync(F, M->raw.p, rows * 64 * 4, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(V, M->lv.p, rows * xk::DESC_VSTRIDE * 4, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  return 0;
}

int md_gb300_ewald_model_desc_info_x(md_gb300_ewald_model_t_x *M, double *rc, float *basis, double vmu[3],
                                     double vsig[3]) {
  if (!M) return fail(MD_GB_ERR_ARG, "NULL model");
  if (rc) *rc = M->dp.rc;
  for (int d = 0; d < 3; ++d) {
    if (vmu) vmu[d] = M->dp.vmu[d];
    if (vsig) vsig[d] = M->vsig[d];
  }
  if (basis) {
    XMD_CUDA(cudaMemcpy(basis, M->basis.p, 4 * xk::DESC_BINS * 32, cudaMemcpyDeviceToHost));
  }
  return 0;
}

}  // extern "C"
