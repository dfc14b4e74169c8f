// xmd_internal.h -- device state behind the MD-Lab structs.
//
// The public structs keep the reference's exact layout, so device state is
// held in side tables keyed by the struct's address.  Ownership follows the
// reference's OpenCL back end (md_util_x.c:359-551, md_pimd_x.c:9-326): a
// device copy is created on the first device call and is authoritative until
// a *_sync_host_x(..., 0) hands authority back to the host; the next device
// call then uploads again.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "md_gb300_x.h"
#include "xmd_kernels.cuh"

namespace xmd {

// ---- errors ----
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
#define XMD_CUDA(call)                                   \
  do {                                                   \
    cudaError_t xmd_e_ = (call);                         \
    if (xmd_e_ != cudaSuccess) return ::xmd::cuda_fail(xmd_e_, #call); \
  } while (0)
#define XMD_TRY(call)                \
  do {                               \
    int xmd_r_ = (call);             \
    if (xmd_r_ != 0) return xmd_r_;  \
  } while (0)

// ---- runtime ----
int ensure_device();       // MD_GB_ERR_NO_DEVICE when CUDA has no device
bool device_present();     // without setting an error
cudaStream_t stream();
bool capturing();
struct SimDev;
// side stream of the exchange chain (xmd_runtime.cpp): fork from the library
// stream, mark its work (with the simulation whose exchange forces wait in
// fex) for the next join; join_side makes the library stream wait and adds
// fex to f.  NoJoin suppresses the join for the calls that may overlap.
int side_begin(cudaStream_t *side);
int side_end(SimDev *fex);
int join_side();
struct NoJoin {
  NoJoin();
  ~NoJoin();
};

struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  template <class T>
  T *as() const { return (T *)p; }
};
int reserve(DevBuf &b, size_t bytes);  // grows, never shrinks
void release(DevBuf &b);

// pinned host allocations made by md_alloc_* (freed with cudaFreeHost)
void *host_alloc(size_t bytes);
void host_free(void *p);

struct SimDev {
  bool valid = false;  // device copy authoritative
  // the layout whose padding lanes were last zeroed (re-uploads of the same
  // layout into the same buffers skip the memsets)
  const void *zx = nullptr, *zth = nullptr;
  int zN = -1, zNs = -1, zP = -1;
  xk::Geo geo{};
  int nf = 0, L = 0;
  bool fast_chains = true;
  bool uniform_mass = true;
  double mass0 = 1.0;
  DevBuf x, v, f, m;
  DevBuf th, vt, Q;
  DevBuf iQ;       // 1/Q of one-DOF chains
  DevBuf cf, c0, c2;
  DevBuf stage;    // AoS records on the device
  DevBuf cstage;   // chain records on their way to and from the host
  DevBuf upflags;  // results of the upload checks (equal masses, one-DOF chains)
  DevBuf scratch;  // partial sums of pair / exchange / reduction kernels
  DevBuf fex;      // exchange spring forces computed on the side stream
  DevBuf xscr;     // partial sums of the exchange forces (side stream)
};

struct PimdDev {
  bool valid = false;  // ENk / ENk2 / VBN / Eint on the device authoritative
  DevBuf ENk, ENk2, Eint, VBN, tmpV, G;
  DevBuf linkt;  // 2N doubles: ENk increments and their prefix sums (scratch of the ENk fill)
  DevBuf lnn;    // ln l for l = 0..N, then 1/l for l = 0..N (entries 0 unused), host values
  DevBuf vsign;  // V_B and signs of md_pimd_calc_vi_sign_x
  DevBuf sk_buf; // wave vectors and results of md_pimd_calc_sphere_Sk_structure_x
  DevBuf rec;  // weights of the forward and backward recursions (two halves)
  // tmpV (backward recursion) computed by the last md_pimd_fill_VB_x from
  // the current ENk with these beta and vi
  bool tmpv_fresh = false;
  double tmpv_beta = 0, tmpv_vi = 0;
  // G (the cycle probabilities) belongs to the stored ENk, VBN and tmpV at
  // g_beta, g_vi: the estimators then need no recursion of their own
  bool g_fresh = false;
  double g_beta = 0, g_vi = 0;
  // Ewald reciprocal tables, rebuilt when the parameters change
  DevBuf rc_coef, rc_cols, rc_phase, rc_S, rc_T;
  int rc_nsum = -1;
  double rc_alpha = 0, rc_qs = 0, rc_box[3] = {0, 0, 0};
  int rc_nk = 0;
  int rc_ncol = 0;  // kept wave-vector columns
  int rc_tsz = 0;   // entries of their compact force tables
  int rc_ncol_in = 0, rc_ncol_out = 0, rc_tsz_in = 0;  // the FP64 forces' split (xk::Recip)
  size_t rc_s32_off = 0;  // doubles of rc_S before the split's FP32 structure factors
  double rc_csum = 0;
};

struct StatsDev {
  bool valid = false;
  DevBuf acc;
};

// layout of a simulation: N particles x P beads (set by md_alloc_pimd_x)
void layout_hint(md_simulation_t_x *sim, int N, int P);
void forget(const void *key);

// device copies, created on demand
int sim_device(md_simulation_t_x *sim, SimDev **out);
// sim_device, with sim's pending exchange forces handed back in *fex (null
// if none) instead of added to f: the caller's kernel adds them
int sim_device_fex(md_simulation_t_x *sim, SimDev **out, const double **fex);
int sim_to_host(md_simulation_t_x *sim, bool keep);
int pimd_device(md_pimd_t_x *pimd, SimDev **sd, PimdDev **pd);
int pimd_to_host(md_pimd_t_x *pimd, bool keep);
int stats_device(md_stats_t_x *st, double **acc);
int stats_to_host(md_stats_t_x *st);
int scratch(SimDev *sd, size_t doubles, double **out);

// shared by the step and the learned residual (xmd_step.cpp)
int check_image(const SimDev *sd, int image);
double *scratch_for(SimDev *sd, size_t doubles, int *rc);
size_t general_scratch(const xk::Geo &g);
int ewald_tables(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd);
xk::Recip recip_of(PimdDev *pd);
xk::PairPrm pair_params(int kind);
// the parameters md_pimd_calc_pair_force_x uses for kind on this system
// (image shifts, inverse mass, the Ewald forces' cut-off)
xk::PairPrm force_params(int kind, const SimDev *sd);
void ewald_shifts(xk::PairPrm &p, const xk::Geo &g);

// learned Ewald residual (xmd_learned_api.cpp).  learned_mode: 0 = plain
// Ewald, 1 = truncated sum + network, 2 = plain Ewald then judge the network
// (force calls count towards the judging interval when count_call is set)
int learned_mode(md_pimd_t_x *pimd, bool count_call);
int learned_pair_force(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd, const xk::PairPrm &prm, double *scr);
int learned_judge_step(md_pimd_t_x *pimd, SimDev *sd, PimdDev *pd);
// reciprocal part of the energy in learned mode (truncated sum + network), added to *acc
int learned_recip_energy(md_pimd_t_x *pimd, SimDev *sd, double *acc, double *scr);

// persistent ensemble planning (xmd_ensemble_api.cpp): while it runs, the
// step's entry points record their call for the current system instead of
// launching (ens_record returns their status), and the device state of any
// other call is refused.
enum EnsOp { ENS_NHC1 = 1, ENS_RESET, ENS_ENK, ENS_VB, ENS_FVB, ENS_TRAP, ENS_PAIR, ENS_NHC2, ENS_WRAP };
bool ens_recording();
int ens_record(int op, md_simulation_t_x *sim, md_pimd_t_x *pimd, double dt, int arg, const void *fn);
int ens_refuse();  // the error of a device call that is not part of the step
// a graph of the one launch that launch(ctx) queues on the library stream;
// release(ctx) runs when the graph is freed (or the capture fails)
int capture_single(cudaError_t (*launch)(void *), void *ctx, void (*release)(void *), int kind,
                   md_gb300_graph_t_x **out);
// what a graph from capture_single owns, if it was made with this kind
void *graph_owned(md_gb300_graph_t_x *g, int kind);
constexpr int GRAPH_ENSEMBLE = 1;

// read the current potential parameter globals
xk::TrapPrm trap_params(int kind);
int pair_kind_of(const void *fn, bool energy);
int trap_kind_of(const void *fn, bool energy);

}  // namespace xmd
