// xmd_runtime.cpp -- CUDA runtime layer of libxmd_x: errors, the stream,
// graph capture, and the device copies behind the MD-Lab structs.
//
// Replaces the reference's OpenCL glue (md_util_x.c:18-83 queue handling,
// :359-551 context transfer and host sync; md_pimd_x.c:9-326;
// md_statistics_x.c:72-201).  One CUDA stream orders all work, as the one
// OpenCL queue does; host <-> device copies use page-locked host memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "xmd_internal.h"

namespace xmd {

static thread_local std::string t_err;
static std::mutex g_mu;

int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  t_err = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(MD_GB_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

// ------------------------------------------------------------------
// device and stream
// ------------------------------------------------------------------
static int g_dev_state = 0;  // 0 unknown, 1 present, -1 absent
static cudaStream_t g_own = nullptr, g_user = nullptr;
static bool g_user_set = false;

bool device_present() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_dev_state == 0) {
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    g_dev_state = (e == cudaSuccess && n > 0) ? 1 : -1;
    if (g_dev_state < 0) cudaGetLastError();
  }
  return g_dev_state > 0;
}

int ensure_device() {
  if (!device_present()) return fail(MD_GB_ERR_NO_DEVICE, "no CUDA device is available");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_own) {
    // a middle priority: above the learned model's descriptor stream (the
    // default, lowest), below the exchange chain's side stream (highest)
    int lo = 0, hi = 0;
    cudaError_t e = cudaDeviceGetStreamPriorityRange(&lo, &hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&g_own, cudaStreamNonBlocking, (lo + hi) / 2);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreateWithPriority");
  }
  return 0;
}

cudaStream_t stream() { return g_user_set ? g_user : g_own; }

bool capturing() {
  cudaStreamCaptureStatus s = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream(), &s) != cudaSuccess) return false;
  return s != cudaStreamCaptureStatusNone;
}

// ------------------------------------------------------------------
// side stream: the exchange chain (recursions, G, exchange spring forces)
// runs on a second stream forked from the library stream, so that it
// overlaps the pair forces queued after it.  Every access to device state
// (sim_device, pimd_device, the host synchronisations, ...) first joins it;
// the pair- and trap-force entry points do not (NoJoin), and the exchange
// forces land in a separate array that the join adds to f.
// ------------------------------------------------------------------
struct Side {
  cudaStream_t s = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  bool pending = false;
  std::vector<SimDev *> fex;  // simulations whose exchange forces wait to be added to f
};
static std::unordered_map<cudaStream_t, Side> g_side;  // by library stream
static thread_local int t_nojoin = 0;

NoJoin::NoJoin() { ++t_nojoin; }
NoJoin::~NoJoin() { --t_nojoin; }

int side_begin(cudaStream_t *out) {
  Side &sd = g_side[stream()];
  if (!sd.s) {
    // highest priority: the exchange chain is latency-bound and should get
    // SMs as soon as any free up
    int lo = 0, hi = 0;
    XMD_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    XMD_CUDA(cudaStreamCreateWithPriority(&sd.s, cudaStreamNonBlocking, hi));
    XMD_CUDA(cudaEventCreateWithFlags(&sd.fork, cudaEventDisableTiming));
    XMD_CUDA(cudaEventCreateWithFlags(&sd.done, cudaEventDisableTiming));
  }
  XMD_CUDA(cudaEventRecord(sd.fork, stream()));
  XMD_CUDA(cudaStreamWaitEvent(sd.s, sd.fork, 0));
  *out = sd.s;
  return 0;
}

int side_end(SimDev *fex) {
  Side &sd = g_side[stream()];
  XMD_CUDA(cudaEventRecord(sd.done, sd.s));
  // timing each kernel alone: the library stream waits for the side chain now
  if (xk::profiling() && !capturing()) XMD_CUDA(cudaStreamWaitEvent(stream(), sd.done, 0));
  sd.pending = true;
  if (fex && std::find(sd.fex.begin(), sd.fex.end(), fex) == sd.fex.end()) sd.fex.push_back(fex);
  return 0;
}

// join; mine's exchange forces are not added but handed back in *fex (the
// caller's next kernel adds them on its way)
static int join_side_taking(SimDev *mine, const double **fex) {
  if (t_nojoin) return 0;
  auto it = g_side.find(stream());
  if (it == g_side.end() || !it->second.pending) return 0;
  Side &sd = it->second;
  sd.pending = false;
  XMD_CUDA(cudaStreamWaitEvent(stream(), sd.done, 0));
  std::vector<SimDev *> add;
  add.swap(sd.fex);
  for (SimDev *d : add) {
    if (d == mine && fex)
      *fex = d->fex.as<double>();
    else
      XMD_CUDA(xk::add_into(d->f.as<double>(), d->fex.as<double>(), d->geo.slots(), stream()));
  }
  return 0;
}
int join_side() { return join_side_taking(nullptr, nullptr); }

int reserve(DevBuf &b, size_t bytes) {
  if (bytes <= b.bytes && b.p) return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "device allocation requested while capturing a graph");
  if (b.p) {
    cudaFreeAsync(b.p, stream());
    b.p = nullptr;
    b.bytes = 0;
  }
  if (bytes == 0) bytes = 8;
  cudaError_t e = cudaMallocAsync(&b.p, bytes, stream());
  if (e != cudaSuccess) {
    b.p = nullptr;
    return fail(MD_GB_ERR_ALLOC, "cudaMallocAsync(%zu bytes): %s", bytes, cudaGetErrorString(e));
  }
  b.bytes = bytes;
  return 0;
}

void release(DevBuf &b) {
  if (b.p) cudaFreeAsync(b.p, stream());
  b.p = nullptr;
  b.bytes = 0;
}

static std::unordered_set<void *> g_pinned;

void *host_alloc(size_t bytes) {
  if (bytes == 0) bytes = 1;
  void *p = nullptr;
  if (device_present() && cudaMallocHost(&p, bytes) == cudaSuccess) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_pinned.insert(p);
    memset(p, 0, bytes);
    return p;
  }
  cudaGetLastError();
  p = calloc(1, bytes);
  return p;
}

void host_free(void *p) {
  if (!p) return;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_pinned.find(p);
    if (it != g_pinned.end()) {
      g_pinned.erase(it);
      cudaFreeHost(p);
      return;
    }
  }
  free(p);
}

// a page-locked array this library allocated (md_alloc_*): kernels read and
// write it directly over the CPU-GPU link, with no staging copy
static bool lib_pinned(const void *p) {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_pinned.count(const_cast<void *>(p)) != 0;
}

// ------------------------------------------------------------------
// side tables
// ------------------------------------------------------------------
struct Layout {
  int N, P;
};
static std::unordered_map<const void *, Layout> g_layout;
static std::unordered_map<const void *, SimDev *> g_sim;
static std::unordered_map<const void *, PimdDev *> g_pimd;
static std::unordered_map<const void *, StatsDev *> g_stats;

template <class T>
static T *lookup(std::unordered_map<const void *, T *> &m, const void *k, bool create) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = m.find(k);
  if (it != m.end()) return it->second;
  if (!create) return nullptr;
  T *t = new T();
  m[k] = t;
  return t;
}

static void free_sim(SimDev *d) {
  // side-stream work of this simulation finishes first; its pending forces
  // are dropped with it
  for (auto &kv : g_side)
    if (kv.second.s && kv.second.pending) {
      cudaStreamSynchronize(kv.second.s);
      auto &v = kv.second.fex;
      v.erase(std::remove(v.begin(), v.end(), d), v.end());
    }
  for (DevBuf *b : {&d->x, &d->v, &d->f, &d->m, &d->th, &d->vt, &d->Q, &d->iQ, &d->cf, &d->c0, &d->c2,
                    &d->stage, &d->cstage, &d->upflags, &d->scratch, &d->fex, &d->xscr})
    release(*b);
}

static void free_pimd(PimdDev *d) {
  for (DevBuf *b : {&d->ENk, &d->ENk2, &d->Eint, &d->VBN, &d->tmpV, &d->G, &d->linkt, &d->lnn, &d->vsign, &d->sk_buf, &d->rec, &d->rc_coef,
                    &d->rc_cols, &d->rc_phase, &d->rc_S, &d->rc_T})
    release(*b);
}

void forget(const void *key) {
  SimDev *s = nullptr;
  PimdDev *p = nullptr;
  StatsDev *t = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_layout.erase(key);
    auto a = g_sim.find(key);
    if (a != g_sim.end()) {
      s = a->second;
      g_sim.erase(a);
    }
    auto b = g_pimd.find(key);
    if (b != g_pimd.end()) {
      p = b->second;
      g_pimd.erase(b);
    }
    auto c = g_stats.find(key);
    if (c != g_stats.end()) {
      t = c->second;
      g_stats.erase(c);
    }
  }
  if (s) {
    free_sim(s);
    delete s;
  }
  if (p) {
    free_pimd(p);
    delete p;
  }
  if (t) {
    release(t->acc);
    delete t;
  }
}

void layout_hint(md_simulation_t_x *sim, int N, int P) {
  SimDev *d = lookup(g_sim, sim, false);
  if (d && d->valid && (d->geo.N != N || d->geo.P != P)) sim_to_host(sim, false);
  std::lock_guard<std::mutex> lk(g_mu);
  g_layout[sim] = {N, P};
}

static xk::Geo make_geo(md_simulation_t_x *sim) {
  xk::Geo g{};
  g.D = MD_DIMENSION_X;
  Layout lay{sim->N, 1};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_layout.find(sim);
    if (it != g_layout.end() && it->second.N * it->second.P == sim->N) lay = it->second;
  }
  g.N = lay.N;
  g.P = lay.P;
  g.Ns = xk::pad_n(lay.N);
  for (int d = 0; d < 3; ++d) {
    g.box[d] = 0;
    g.inv_box[d] = 0;
  }
  if (sim->box && sim->box->type == MD_ND_RECT_BOX_X && sim->box->box) {
    const nd_rect_t_x *r = (const nd_rect_t_x *)sim->box->box;
    for (int d = 0; d < MD_DIMENSION_X; ++d) {
      g.box[d] = r->L[d];
      g.inv_box[d] = r->L[d] != 0 ? 1.0 / r->L[d] : 0.0;
    }
  }
  return g;
}

// ------------------------------------------------------------------
// simulation
// ------------------------------------------------------------------
int sim_device(md_simulation_t_x *sim, SimDev **out) {
  if (!sim || !sim->particles || sim->N < 1) return fail(MD_GB_ERR_ARG, "invalid simulation");
  if (ens_recording()) XMD_TRY(ens_refuse());
  XMD_TRY(ensure_device());
  XMD_TRY(join_side());
  SimDev *d = lookup(g_sim, sim, true);
  *out = d;
  // the box may change between calls (md_init_nd_rect_box_x)
  if (d->valid) {
    xk::Geo g = make_geo(sim);
    for (int q = 0; q < 3; ++q) {
      d->geo.box[q] = g.box[q];
      d->geo.inv_box[q] = g.inv_box[q];
    }
    return 0;
  }
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "simulation state is not on the device yet");
  cudaStream_t st = stream();
  d->geo = make_geo(sim);
  const xk::Geo &g = d->geo;
  const size_t S = g.slots();
  const int D = MD_DIMENSION_X, L = MD_NHC_LENGTH_X;
  XMD_TRY(reserve(d->x, S * 8));
  XMD_TRY(reserve(d->v, S * 8));
  XMD_TRY(reserve(d->f, S * 8));
  XMD_TRY(reserve(d->m, (size_t)g.P * g.Ns * 8));
  // padding lanes stay zero so that slice-wide kernels read defined values
  // (no kernel writes them: once per layout and allocation)
  const bool same_layout = d->zx == d->x.p && d->zN == g.N && d->zNs == g.Ns && d->zP == g.P;
  if (!same_layout) {
    XMD_CUDA(cudaMemsetAsync(d->x.p, 0, S * 8, st));
    XMD_CUDA(cudaMemsetAsync(d->v.p, 0, S * 8, st));
    XMD_CUDA(cudaMemsetAsync(d->f.p, 0, S * 8, st));
    XMD_CUDA(cudaMemsetAsync(d->m.p, 0, (size_t)g.P * g.Ns * 8, st));
    d->zth = nullptr;
  }
  // Whether all masses are equal and all chains have one DOF is checked on
  // the device while the records are converted (walking 13 MB of records on
  // one host core took longer than the copies): the chain records are
  // converted in the one-DOF layout when their count says so, and only if a
  // record then shows f != 1 are they converted again in the grouped layout.
  d->nf = sim->Nf;
  d->L = L;
  const int nchain = sim->nhcs ? sim->Nf : 0;
  const size_t pbytes = sizeof(md_particle_t_x) * (size_t)sim->N;
  const size_t cbytes = sizeof(md_nhc_t_x) * (size_t)nchain;
  XMD_TRY(reserve(d->upflags, 2 * sizeof(int)));
  XMD_CUDA(cudaMemsetAsync(d->upflags.p, 0xff, 2 * sizeof(int), st));
  // the library's own page-locked arrays are read in place; others go up
  // to device stages first
  const bool direct = lib_pinned(sim->particles) && (!cbytes || lib_pinned(sim->nhcs));
  const unsigned char *prec = (const unsigned char *)sim->particles, *crec = (const unsigned char *)sim->nhcs;
  if (!direct) {
    XMD_TRY(reserve(d->stage, pbytes));
    if (cbytes) XMD_TRY(reserve(d->cstage, cbytes));
    XMD_CUDA(cudaMemcpyAsync(d->stage.p, sim->particles, pbytes, cudaMemcpyHostToDevice, st));
    if (cbytes) XMD_CUDA(cudaMemcpyAsync(d->cstage.p, sim->nhcs, cbytes, cudaMemcpyHostToDevice, st));
    prec = d->stage.as<unsigned char>();
    crec = d->cstage.as<unsigned char>();
  }
  XMD_CUDA(xk::aos_to_soa(g, (const double *)prec, d->x.as<double>(), d->v.as<double>(), d->f.as<double>(),
                          d->m.as<double>(), st, d->upflags.as<int>()));
  const bool try_fast = nchain > 0 && sim->Nf == D * sim->N;
  bool fresh_chains = true;
  if (try_fast) {
    XMD_TRY(reserve(d->th, S * L * 8));
    XMD_TRY(reserve(d->vt, S * L * 8));
    XMD_TRY(reserve(d->Q, S * L * 8));
    XMD_TRY(reserve(d->iQ, S * L * 8));
    fresh_chains = !(same_layout && d->zth == d->th.p);
    if (fresh_chains) {
      // padding slots stay zero (their 1/Q is 0, nothing divides by them)
      XMD_CUDA(cudaMemsetAsync(d->th.p, 0, S * L * 8, st));
      XMD_CUDA(cudaMemsetAsync(d->vt.p, 0, S * L * 8, st));
      XMD_CUDA(cudaMemsetAsync(d->Q.p, 0, S * L * 8, st));
      XMD_CUDA(cudaMemsetAsync(d->iQ.p, 0, S * L * 8, st));
    }
    XMD_CUDA(xk::chains_to_dev(g, L, sim->Nf, true, crec, sizeof(md_nhc_t_x), d->th.as<double>(),
                               d->vt.as<double>(), d->Q.as<double>(), d->iQ.as<double>(), fresh_chains, st,
                               d->upflags.as<int>() + 1));
  }
  int flags[2] = {0, 0};
  XMD_CUDA(cudaMemcpyAsync(flags, d->upflags.p, sizeof flags, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  d->uniform_mass = flags[0] != 0;
  d->mass0 = sim->particles[0].m;
  const bool fast = try_fast && flags[1] != 0;
  d->fast_chains = fast;
  if (sim->nhcs && sim->Nf > 0 && !fast) {
    // grouped chains: first DOF and DOF count as the reference's loop
    // (md_simulation_x.c:664-668) computes them
    const size_t cs = (size_t)sim->Nf;
    XMD_TRY(reserve(d->th, cs * L * 8));
    XMD_TRY(reserve(d->vt, cs * L * 8));
    XMD_TRY(reserve(d->Q, cs * L * 8));
    std::vector<int> cf(sim->Nf), c0(sim->Nf), c2(sim->Nf);
    int f0 = 0;
    for (int i = 0; i < sim->Nf; ++i) {
      cf[i] = sim->nhcs[i].f;
      c0[i] = f0;
      c2[i] = (i == sim->Nf - 1) ? D * sim->N - f0 : cf[i];
      if (f0 < 0 || c2[i] < 0 || f0 + c2[i] > D * sim->N)
        return fail(MD_GB_ERR_ARG, "chain %d covers DOFs outside the simulation", i);
      f0 += cf[i];
    }
    XMD_TRY(reserve(d->cf, sizeof(int) * sim->Nf));
    XMD_TRY(reserve(d->c0, sizeof(int) * sim->Nf));
    XMD_TRY(reserve(d->c2, sizeof(int) * sim->Nf));
    XMD_CUDA(cudaMemcpyAsync(d->cf.p, cf.data(), sizeof(int) * sim->Nf, cudaMemcpyHostToDevice, st));
    XMD_CUDA(cudaMemcpyAsync(d->c0.p, c0.data(), sizeof(int) * sim->Nf, cudaMemcpyHostToDevice, st));
    XMD_CUDA(cudaMemcpyAsync(d->c2.p, c2.data(), sizeof(int) * sim->Nf, cudaMemcpyHostToDevice, st));
    XMD_CUDA(xk::chains_to_dev(g, L, sim->Nf, false, crec, sizeof(md_nhc_t_x), d->th.as<double>(),
                               d->vt.as<double>(), d->Q.as<double>(), nullptr, true, st));
    XMD_CUDA(cudaStreamSynchronize(st));  // the vectors above go out of scope
  }
  d->zth = fast ? d->th.p : nullptr;
  d->zx = d->x.p;
  d->zN = g.N;
  d->zNs = g.Ns;
  d->zP = g.P;
  d->valid = true;
  return 0;
}

int sim_device_fex(md_simulation_t_x *sim, SimDev **out, const double **fex) {
  *fex = nullptr;
  if (sim && device_present() && g_own) {
    SimDev *d = lookup(g_sim, sim, false);
    if (d && d->valid) XMD_TRY(join_side_taking(d, fex));
  }
  return sim_device(sim, out);
}

int sim_to_host(md_simulation_t_x *sim, bool keep) {
  if (device_present() && g_own) XMD_TRY(join_side());
  if (!sim) return fail(MD_GB_ERR_ARG, "NULL simulation");
  SimDev *d = lookup(g_sim, sim, false);
  if (!d || !d->valid) return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "host synchronisation while capturing a graph");
  cudaStream_t st = stream();
  const xk::Geo &g = d->geo;
  const size_t pbytes = sizeof(md_particle_t_x) * (size_t)sim->N;
  // the library's own page-locked arrays are written in place by the
  // kernels; others come down through device stages
  if (lib_pinned(sim->particles)) {
    XMD_CUDA(xk::soa_to_aos(g, (double *)sim->particles, d->x.as<double>(), d->v.as<double>(), d->f.as<double>(),
                            d->m.as<double>(), st));
  } else {
    XMD_TRY(reserve(d->stage, pbytes));
    XMD_CUDA(xk::soa_to_aos(g, d->stage.as<double>(), d->x.as<double>(), d->v.as<double>(), d->f.as<double>(),
                            d->m.as<double>(), st));
    XMD_CUDA(cudaMemcpyAsync(sim->particles, d->stage.p, pbytes, cudaMemcpyDeviceToHost, st));
  }
  if (sim->nhcs && sim->Nf > 0) {
    // whole chain records (f as uploaded)
    const size_t cbytes = sizeof(md_nhc_t_x) * (size_t)sim->Nf;
    const bool direct = lib_pinned(sim->nhcs);
    if (!direct) XMD_TRY(reserve(d->cstage, cbytes));
    unsigned char *crec = direct ? (unsigned char *)sim->nhcs : d->cstage.as<unsigned char>();
    XMD_CUDA(xk::chains_to_host(g, d->L, sim->Nf, d->fast_chains, crec, sizeof(md_nhc_t_x), d->th.as<double>(),
                                d->vt.as<double>(), d->Q.as<double>(), d->cf.as<int>(), st));
    if (!direct) XMD_CUDA(cudaMemcpyAsync(sim->nhcs, d->cstage.p, cbytes, cudaMemcpyDeviceToHost, st));
  }
  XMD_CUDA(cudaStreamSynchronize(st));
  if (!keep) d->valid = false;
  return 0;
}

int scratch(SimDev *sd, size_t doubles, double **out) {
  XMD_TRY(reserve(sd->scratch, doubles * 8));
  *out = sd->scratch.as<double>();
  return 0;
}

// ------------------------------------------------------------------
// path-integral state
// ------------------------------------------------------------------
int pimd_device(md_pimd_t_x *pimd, SimDev **sd, PimdDev **pd) {
  if (!pimd || !pimd->sim) return fail(MD_GB_ERR_ARG, "invalid path-integral state");
  if (ens_recording()) XMD_TRY(ens_refuse());
  if (pimd->N < 1 || pimd->P < 1 || pimd->N * pimd->P != pimd->sim->N)
    return fail(MD_GB_ERR_ARG, "N*P (%d*%d) does not match the simulation's %d beads", pimd->N,
                pimd->P, pimd->sim->N);
  layout_hint(pimd->sim, pimd->N, pimd->P);
  XMD_TRY(sim_device(pimd->sim, sd));
  PimdDev *d = lookup(g_pimd, pimd, true);
  *pd = d;
  if (d->valid) return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "exchange state is not on the device yet");
  const int N = pimd->N;
  const size_t nt = xk::ntri(N);
  XMD_TRY(reserve(d->ENk, nt * 8));
  XMD_TRY(reserve(d->ENk2, nt * 8));
  XMD_TRY(reserve(d->Eint, (size_t)N * 8));
  XMD_TRY(reserve(d->VBN, (size_t)(N + 1) * 8));
  XMD_TRY(reserve(d->tmpV, (size_t)(N + 1) * 8));
  XMD_TRY(reserve(d->G, (size_t)N * N * 8));
  XMD_TRY(reserve(d->linkt, (size_t)2 * N * 8));
  {
    // ln l, then 1/l, for l = 0..N (entries 0 unused), host values
    std::vector<double> ln(2 * (size_t)(N + 1), 0.0);
    for (int l = 1; l <= N; ++l) {
      ln[l] = log((double)l);
      ln[N + 1 + l] = 1.0 / l;
    }
    XMD_TRY(reserve(d->lnn, 2 * (size_t)(N + 1) * 8));
    XMD_CUDA(cudaMemcpyAsync(d->lnn.p, ln.data(), 2 * (size_t)(N + 1) * 8, cudaMemcpyHostToDevice, stream()));
    XMD_CUDA(cudaStreamSynchronize(stream()));
  }
  XMD_TRY(reserve(d->rec, 2 * xk::rec_scratch_doubles(N) * 8));
  XMD_CUDA(cudaMemsetAsync(d->rec.p, 0, 2 * xk::rec_scratch_doubles(N) * 8, stream()));
  d->tmpv_fresh = false;
  d->g_fresh = false;
  XMD_CUDA(cudaMemsetAsync(d->tmpV.p, 0, (size_t)(N + 1) * 8, stream()));
  cudaStream_t st = stream();
  XMD_CUDA(cudaMemcpyAsync(d->ENk.p, pimd->ENk[0], nt * 8, cudaMemcpyHostToDevice, st));
  XMD_CUDA(cudaMemcpyAsync(d->ENk2.p, pimd->ENk2[0], nt * 8, cudaMemcpyHostToDevice, st));
  XMD_CUDA(cudaMemcpyAsync(d->Eint.p, pimd->Eint, (size_t)N * 8, cudaMemcpyHostToDevice, st));
  XMD_CUDA(cudaMemcpyAsync(d->VBN.p, pimd->VBN, (size_t)(N + 1) * 8, cudaMemcpyHostToDevice, st));
  d->valid = true;
  return 0;
}

int pimd_to_host(md_pimd_t_x *pimd, bool keep) {
  if (device_present() && g_own) XMD_TRY(join_side());
  if (!pimd) return fail(MD_GB_ERR_ARG, "NULL path-integral state");
  PimdDev *d = lookup(g_pimd, pimd, false);
  if (!d || !d->valid) return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "host synchronisation while capturing a graph");
  cudaStream_t st = stream();
  const int N = pimd->N;
  const size_t nt = xk::ntri(N);
  XMD_CUDA(cudaMemcpyAsync(pimd->ENk[0], d->ENk.p, nt * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(pimd->ENk2[0], d->ENk2.p, nt * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(pimd->Eint, d->Eint.p, (size_t)N * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaMemcpyAsync(pimd->VBN, d->VBN.p, (size_t)(N + 1) * 8, cudaMemcpyDeviceToHost, st));
  XMD_CUDA(cudaStreamSynchronize(st));
  if (!keep) d->valid = false;
  return 0;
}

// ------------------------------------------------------------------
// accumulators
// ------------------------------------------------------------------
int stats_device(md_stats_t_x *s, double **acc) {
  if (device_present() && g_own) XMD_TRY(join_side());
  if (!s || !s->es || s->N < 1) return fail(MD_GB_ERR_ARG, "invalid statistics accumulator");
  XMD_TRY(ensure_device());
  StatsDev *d = lookup(g_stats, s, true);
  if (!d->valid) {
    if (capturing()) return fail(MD_GB_ERR_CAPTURE, "accumulator is not on the device yet");
    XMD_TRY(reserve(d->acc, 8));
    // the host value travels as a kernel argument: no copy from host memory
    // in flight, so no synchronisation
    XMD_CUDA(xk::set_value(d->acc.as<double>(), s->es[s->N - 1], stream()));
    d->valid = true;
  }
  *acc = d->acc.as<double>();
  return 0;
}

int stats_to_host(md_stats_t_x *s) {
  if (device_present() && g_own) XMD_TRY(join_side());
  if (!s) return fail(MD_GB_ERR_ARG, "NULL accumulator");
  StatsDev *d = lookup(g_stats, s, false);
  if (!d || !d->valid) return 0;
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "host synchronisation while capturing a graph");
  XMD_CUDA(cudaMemcpyAsync(&s->es[s->N - 1], d->acc.p, 8, cudaMemcpyDeviceToHost, stream()));
  XMD_CUDA(cudaStreamSynchronize(stream()));
  d->valid = false;
  return 0;
}

}  // namespace xmd

// ------------------------------------------------------------------
// public additions (md_gb300_x.h)
// ------------------------------------------------------------------
using namespace xmd;

struct md_gb300_graph {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
  void (*release)(void *) = nullptr;  // frees what the graph's kernels read (owned)
  void *owned = nullptr;
  int kind = 0;  // what owned is (capture_single's caller)
};

namespace xmd {

void *graph_owned(md_gb300_graph_t_x *g, int kind) { return g && g->kind == kind ? g->owned : nullptr; }

int capture_single(cudaError_t (*launch)(void *), void *ctx, void (*release)(void *), int kind,
                   md_gb300_graph_t_x **out) {
  if (capturing()) {
    release(ctx);
    return fail(MD_GB_ERR_CAPTURE, "already capturing");
  }
  cudaError_t e = cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal);
  cudaGraph_t g = nullptr;
  if (e == cudaSuccess) {
    e = launch(ctx);
    const cudaError_t ee = cudaStreamEndCapture(stream(), &g);
    if (e == cudaSuccess) e = ee;
  }
  md_gb300_graph *gr = nullptr;
  if (e == cudaSuccess) {
    gr = new md_gb300_graph();
    gr->g = g;
    e = cudaGraphInstantiate(&gr->e, g, cudaGraphInstantiateFlagUseNodePriority);
  }
  if (e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    delete gr;
    release(ctx);
    cudaGetLastError();
    return cuda_fail(e, "single-launch capture");
  }
  gr->release = release;
  gr->owned = ctx;
  gr->kind = kind;
  *out = gr;
  return 0;
}

}  // namespace xmd

extern "C" {

const char *md_gb300_last_error_x(void) { return t_err.c_str(); }

void md_gb300_variant_x(int *dimension, int *nhc_length) {
  if (dimension) *dimension = MD_DIMENSION_X;
  if (nhc_length) *nhc_length = MD_NHC_LENGTH_X;
}

int md_gb300_device_count_x(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

unsigned long long md_gb300_launch_count_x(void) { return xk::launch_count(); }

int md_gb300_set_device_x(int dev) {
  if (!device_present()) return fail(MD_GB_ERR_NO_DEVICE, "no CUDA device is available");
  if (g_own) return fail(MD_GB_ERR_ARG, "the device must be chosen before the first device call");
  XMD_CUDA(cudaSetDevice(dev));
  return 0;
}

int md_gb300_set_stream_x(void *s) {
  XMD_TRY(ensure_device());
  g_user = (cudaStream_t)s;
  g_user_set = s != nullptr;
  return 0;
}

void *md_gb300_get_stream_x(void) {
  if (ensure_device() != 0) return nullptr;
  return (void *)stream();
}

int md_gb300_synchronize_x(void) {
  XMD_TRY(ensure_device());
  XMD_TRY(join_side());
  XMD_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

int md_gb300_capture_begin_x(void) {
  XMD_TRY(ensure_device());
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "already capturing");
  XMD_TRY(join_side());  // no side-stream work from before the capture stays open
  XMD_CUDA(cudaStreamBeginCapture(stream(), cudaStreamCaptureModeThreadLocal));
  return 0;
}

int md_gb300_capture_end_x(md_gb300_graph_t_x **out) {
  if (!out) return fail(MD_GB_ERR_ARG, "NULL graph pointer");
  XMD_TRY(ensure_device());
  XMD_TRY(join_side());  // side-stream work must rejoin before the capture ends
  md_gb300_graph *gr = new md_gb300_graph();
  cudaError_t e = cudaStreamEndCapture(stream(), &gr->g);
  if (e != cudaSuccess) {
    delete gr;
    return cuda_fail(e, "cudaStreamEndCapture");
  }
  e = cudaGraphInstantiate(&gr->e, gr->g, cudaGraphInstantiateFlagUseNodePriority);
  if (e != cudaSuccess) {
    cudaGraphDestroy(gr->g);
    delete gr;
    return cuda_fail(e, "cudaGraphInstantiate");
  }
  *out = gr;
  return 0;
}

// Branch streams of ensemble captures (created on first use, kept).
static std::vector<cudaStream_t> g_branches;

int md_gb300_capture_ensemble_x(int n, md_gb300_system_step_fn_x step, void *ctx, md_gb300_graph_t_x **out) {
  if (n < 1 || !step || !out) return fail(MD_GB_ERR_ARG, "invalid ensemble capture arguments");
  XMD_TRY(ensure_device());
  if (capturing()) return fail(MD_GB_ERR_CAPTURE, "already capturing");
  XMD_TRY(join_side());
  while ((int)g_branches.size() < n) {
    cudaStream_t b;
    XMD_CUDA(cudaStreamCreateWithFlags(&b, cudaStreamNonBlocking));
    g_branches.push_back(b);
  }
  const cudaStream_t main = stream();
  const cudaStream_t saved_user = g_user;
  const bool saved_set = g_user_set;
  std::vector<cudaEvent_t> ev(n + 1, nullptr);
  for (auto &e : ev) XMD_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  int rc = 0;
  cudaError_t ce = cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal);
  if (ce == cudaSuccess) ce = cudaEventRecord(ev[n], main);
  // every system's calls go to its own branch, forked from and joined to
  // the library stream: independent chains of nodes in one graph
  for (int i = 0; i < n && ce == cudaSuccess && !rc; ++i) {
    ce = cudaStreamWaitEvent(g_branches[i], ev[n], 0);
    if (ce != cudaSuccess) break;
    g_user = g_branches[i];
    g_user_set = true;
    rc = step(i, ctx);
    if (!rc) rc = join_side();
    g_user = saved_user;
    g_user_set = saved_set;
    if (!rc) ce = cudaEventRecord(ev[i], g_branches[i]);
  }
  g_user = saved_user;
  g_user_set = saved_set;
  for (int i = 0; i < n && ce == cudaSuccess && !rc; ++i) ce = cudaStreamWaitEvent(main, ev[i], 0);
  cudaGraph_t g = nullptr;
  const cudaError_t ee = cudaStreamEndCapture(main, &g);
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc || ce != cudaSuccess || ee != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    if (rc) return rc;
    return cuda_fail(ce != cudaSuccess ? ce : ee, "ensemble capture");
  }
  md_gb300_graph *gr = new md_gb300_graph();
  gr->g = g;
  const cudaError_t ie = cudaGraphInstantiate(&gr->e, gr->g, cudaGraphInstantiateFlagUseNodePriority);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(gr->g);
    delete gr;
    return cuda_fail(ie, "cudaGraphInstantiate");
  }
  *out = gr;
  return 0;
}

int md_gb300_graph_launch_x(md_gb300_graph_t_x *gr, int count) {
  if (!gr || count < 0) return fail(MD_GB_ERR_ARG, "invalid graph launch");
  XMD_TRY(join_side());
  for (int i = 0; i < count; ++i) XMD_CUDA(cudaGraphLaunch(gr->e, stream()));
  return 0;
}

int md_gb300_graph_kernel_count_x(md_gb300_graph_t_x *gr) {
  if (!gr) return fail(MD_GB_ERR_ARG, "NULL graph");
  size_t n = 0;
  XMD_CUDA(cudaGraphGetNodes(gr->g, nullptr, &n));
  std::vector<cudaGraphNode_t> nodes(n);
  XMD_CUDA(cudaGraphGetNodes(gr->g, nodes.data(), &n));
  int k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

void md_gb300_graph_free_x(md_gb300_graph_t_x *gr) {
  if (!gr) return;
  if (gr->e) cudaGraphExecDestroy(gr->e);
  if (gr->g) cudaGraphDestroy(gr->g);
  if (gr->release) gr->release(gr->owned);
  delete gr;
}

int md_gb300_profile_x(int on) {
  XMD_TRY(ensure_device());
  xk::profile_enable(on != 0);
  return 0;
}

int md_gb300_profile_report_x(char *buf, int len) {
  if (!buf || len < 1) return fail(MD_GB_ERR_ARG, "invalid report buffer");
  const std::string r = xk::profile_report();
  snprintf(buf, (size_t)len, "%s", r.c_str());
  return (int)r.size();
}

double md_gb300_fp64_peak_x(void) {
  if (ensure_device() != 0) return -1;
  return xk::fp64_peak_tflops(stream());
}

double md_gb300_fp32_peak_x(void) {
  if (ensure_device() != 0) return -1;
  return xk::fp32_peak_tflops(stream());
}

int md_gb300_release_simulation_x(md_simulation_t_x *sim) {
  if (!sim) return fail(MD_GB_ERR_ARG, "NULL simulation");
  XMD_TRY(sim_to_host(sim, false));
  forget(sim);
  return 0;
}

}  // extern "C"
