// xmd_kernels.cuh -- launch interface of the sm_103a kernels behind libxmd_x.
//
// Every function enqueues work on `st` and returns the launch status.  All
// pointers are device pointers.  Bead data is kept slice-major ("SoA"):
//     x[(j*D + d)*Ns + l]   particle l = 0..N-1, bead j = 0..P-1, dim d
// with Ns = N rounded up to a multiple of 4, so that every bead slice starts
// on a 32-byte boundary and a slice's coordinates are contiguous.  Masses
// are m[j*Ns + l].  Thermostat chains with one DOF each ("fast" chains) are
// stored in the same slot order, member i of the chain at slot s being
// th[i*S + s] with S = P*D*Ns.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#ifdef __CUDACC__
#define XK_HD __host__ __device__
#else
#define XK_HD
#endif

namespace xk {

struct Geo {
  int D, N, P, Ns;
  double box[3];
  double inv_box[3];
  XK_HD size_t slots() const { return (size_t)P * D * Ns; }
};
// slot of coordinate d of particle l in bead slice j
XK_HD inline size_t sidx(int j, int d, int l, int D, int Ns) { return ((size_t)j * D + d) * Ns + l; }

inline int pad_n(int N) { return (N + 3) & ~3; }
inline size_t tri(int n) { return (size_t)n * (n - 1) / 2; }  // row start, 1-based n
inline size_t ntri(int n) { return (size_t)n * (n + 1) / 2; }

// count of kernels launched by this library (for launch accounting)
uint64_t launch_count();
// counts one launch and returns cudaGetLastError()
cudaError_t launched();
#define XK_LAUNCHED() ::xk::launched()
// RAII bracket around one launch for the live per-kernel timing; inert
// unless profiling is on and the stream is not being captured into a graph
struct Prof {
  const char *name;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  Prof(const char *n, cudaStream_t s);
  ~Prof();
};
#define XK_PROF(name) ::xk::Prof xk_prof_(name, st)

// live per-kernel timing with CUDA events; report is "name total_ms launches;..."
void profile_enable(bool on);
// whether the live per-kernel timing is on (the library then joins its
// forked streams at once, so that each kernel is timed alone)
bool profiling();
std::string profile_report();
// measured FP64 FMA throughput of this GPU in TFLOP/s (-1 on failure)
double fp64_peak_tflops(cudaStream_t st);
double fp32_peak_tflops(cudaStream_t st);

// ---- layout conversion (host AoS records <-> device SoA) ----
// mass_flag (optional, nonzero before) := 0 unless every record has the
// first one's mass (bit pattern)
cudaError_t aos_to_soa(const Geo &g, const double *aos, double *x, double *v, double *f,
                       double *m, cudaStream_t st, int *mass_flag = nullptr);
cudaError_t soa_to_aos(const Geo &g, double *aos, const double *x, const double *v,
                       const double *f, const double *m, cudaStream_t st);
// chains: host records {int f; double theta[L], vtheta[L], Q[L]} of rec_bytes each
// iQ (optional): 1/Q, updated where Q changes (everywhere with all_iq)
cudaError_t chains_to_dev(const Geo &g, int L, int nf, bool fast, const unsigned char *rec,
                          size_t rec_bytes, double *th, double *vt, double *Q, double *iQ, bool all_iq,
                          cudaStream_t st, int *f_flag = nullptr);  // f_flag := 0 unless every f is 1
// whole records back, f included: 1 for one-DOF chains, cf[c] for grouped ones
cudaError_t chains_to_host(const Geo &g, int L, int nf, bool fast, unsigned char *rec,
                           size_t rec_bytes, const double *th, const double *vt,
                           const double *Q, const int *cf, cudaStream_t st);

// ---- integrator ----
struct Chains {
  bool fast;            // one DOF per chain, chains in slot order
  int L, nf;            // chain length, number of chains
  double *th, *vt, *Q;  // [L][S] (fast) or [L][nf] (grouped)
  const double *iQ;     // fast: 1/Q, same layout
  const int *cf;        // grouped: nhcs[i].f
  const int *c0;        // grouped: first DOF (reference numbering)
  const int *c2;        // grouped: number of DOFs updated
  int ndof;             // D * beads
};
// fex (optional): exchange forces still to be added to f, added (and f
// updated) by the half step itself
cudaError_t nhc_vv3(const Geo &g, int half, const Chains &c, double *x, double *v,
                    double *f, const double *m, double kT, double h, cudaStream_t st,
                    const double *fex = nullptr);
cudaError_t wrap_box(const Geo &g, double *x, cudaStream_t st);
cudaError_t zero(double *p, size_t n, cudaStream_t st);
// *p = v in stream order (a value from the host without a host buffer)
cudaError_t set_value(double *p, double v, cudaStream_t st);

// ---- exchange ----
// gl: scratch of 2N doubles (the row increments and their prefix sums)
cudaError_t fill_enk(const Geo &g, const double *x, const double *m, double w2, int image,
                     double *Eint, double *ENk, double *gl, cudaStream_t st);
cudaError_t fill_enk2(const Geo &g, const double *x, const double *m, double w2, int image,
                      double *ENk2, cudaStream_t st);
// the cubic path's table (md_pimd_fill_ENk2_x), a different quantity
cudaError_t fill_enk2_cubic(const Geo &g, const double *x, const double *m, double w2, int image,
                            double *ENk2, cudaStream_t st);
// V_B^(n) (forward) and tmpV (backward) recursions, solved as extended-
// range triangular systems.  rs: rec_scratch_doubles(N) doubles of scratch.
size_t rec_scratch_doubles(int N);
// lnn[l] = ln l for l = 1..N (host values); rs: weight scratch of
// rec_scratch_doubles(N) doubles per direction
cudaError_t fill_vb(int N, double beta, double vi, const double *ENk, const double *lnn, double *VBN, double *rs,
                    cudaStream_t st);
cudaError_t back_vb(int N, double beta, double vi, const double *ENk, const double *lnn, double *tmpV, double *rs,
                    cudaStream_t st);
// both at once (the two recursions need only ENk): V_B into VBN and the
// backward tmpV, on two SMs; rs_f and rs_b are separate weight scratch
cudaError_t fill_vb_tv(int N, double beta, double vi, const double *ENk, const double *lnn, double *VBN,
                       double *tmpV, double *rs_f, double *rs_b, cudaStream_t st);
// V_B for a signed xi' (md_pimd_calc_vi_sign_x): V2[n] = -ln|Z'_n|/beta and
// sign[n] = sign of Z'_n, n = 0..N
// which kernel solves the unsigned recursions (both give the same unknowns
// to rounding): SOLVE_AUTO chooses by N (a recorded choice, else the cluster
// from five 32-row chunks on); the others force one for every N
enum SolvePath { SOLVE_AUTO = 0, SOLVE_BLOCK = 1, SOLVE_CLUSTER = 2 };
void set_solve_path(int path);
int solve_path();
// record the path for one N (the solve autotuner) and read the path used for N
void set_solve_choice(int N, int path);
int solve_choice(int N);
cudaError_t fill_vb_signed(int N, double beta, double vi2, const double *ENk, const double *lnn, double *V2,
                           double *sign, double *rs, cudaStream_t st);
// lnn: the host table of ln l then 1/l (2 (N+1) doubles)
cudaError_t fill_g(int N, double beta, double vi, const double *ENk, const double *VBN,
                   const double *tmpV, const double *lnn, double *G, cudaStream_t st);
// G from the extended-range weights and unknowns that fill_vb_tv left in
// its scratch (rs_f, rs_b): valid only while that call's ENk, beta and xi
// are current; a few ulps where fill_g loses up to beta V_B^(N) ulps
cudaError_t fill_g_ext(int N, const double *rs_f, const double *rs_b, double *G, cudaStream_t st);
// scratch: at least exch_scratch_doubles(g) doubles
size_t exch_scratch_doubles(const Geo &g);
cudaError_t exch_force(const Geo &g, const double *x, const double *m, double w2, int image,
                       const double *G, double *f, double *scratch, cudaStream_t st);

// ---- external forces ----
enum TrapKind { TRAP_HARMONIC = 1, TRAP_HARMONIC_2 = 2, TRAP_NEG_HARMONIC = 3 };
struct TrapPrm {
  int kind;
  double w;
  double w2[3];
  double c[3];
};
cudaError_t trap_force(const Geo &g, const TrapPrm &p, const double *x, double *f,
                       cudaStream_t st);
// energy sum over beads of V(x)/P, added to *acc
cudaError_t trap_energy(const Geo &g, const TrapPrm &p, const double *x, const double *m,
                        double *acc, double *scratch, cudaStream_t st);

enum PairKind {
  PAIR_GAUSSIAN = 1,
  PAIR_PERIODIC_GAUSSIAN = 2,
  PAIR_COULOMB = 3,
  PAIR_PERIODIC_COULOMB = 4,
  PAIR_EWALD_REAL = 5
};
struct PairPrm {
  int kind;
  double g, s;          // Gaussian strength / range
  double qs;            // Coulomb strength
  double alpha;         // Ewald splitting
  int nsum;             // Ewald image cube
  double rcut;          // Ewald real-space cut-off radius
  int kmax[3];          // Ewald: image shifts |k| <= kmax around the minimum image
  double inv_mass;      // > 0: every bead has this inverse mass (FP32 kernel shortcut)
  double xsplit;        // Ewald forces of the FP64 kernels: images with alpha R >= xsplit are
                        // evaluated on the FP32 pipe (0: every image in FP64)
  // set by the FP64 force launchers from the fields above and the box
  double rc2;           // rcut^2
  float alphaf;         // alpha
  float xs2f;           // (xsplit / alpha)^2, or FLT_MAX with xsplit = 0
  float rcf2;           // rcut^2
  float rcf2_cull;      // rcut^2 (1 + 1e-4): the FP32 culling's margin
  float boxf[3], iboxf[3];  // box lengths and their inverses
};
// alpha R at and beyond which the FP64 kernels evaluate real-space Ewald
// images on the FP32 pipe (every image there has h(alpha R) < 5.2e-7, and
// the sum of their sizes over all partners is 4 pi rho / alpha times the
// integral of h from 4 on, 6.3e-8 pi rho / alpha; the FP32 evaluation's own
// relative error is below 1e-5 there)
constexpr double EWALD_XSPLIT = 4.0;
size_t pair_scratch_doubles(const Geo &g);
cudaError_t pair_force(const Geo &g, const PairPrm &p, const double *x, const double *m,
                       double *f, double *scratch, cudaStream_t st);
// choices of the FP64 autotuner, per (what, kind, D, N, P); tuning() is 0
// where none was recorded (the built-in rule applies).  TUNE_PAIR64_BPS: the
// FP64 tile kernels' blocks per SM (kind = PairKind).  TUNE_SK_LAYOUT: the
// structure-factor kernel's layout (kind = n_sum, D = 3).
enum { TUNE_PAIR64_BPS = 0, TUNE_SK_LAYOUT = 1 };
enum { SK_16x16 = 1, SK_8x32 = 2, SK_64x1 = 3 };
void set_tuning(int what, int kind, int D, int N, int P, int v);
int tuning(int what, int kind, int D, int N, int P);
cudaError_t pair_energy(const Geo &g, const PairPrm &p, const double *x, double *acc,
                        double *scratch, cudaStream_t st);

// Pair forces (not Ewald) with the per-tile partials in a fixed array of
// NOALLOC_SCRATCH_DOUBLES doubles inside the library (4 MiB): no allocation.
// Returns cudaErrorInvalidValue when the configuration needs more than that
// (pair_force_noalloc_need), cudaErrorNotSupported for Ewald.
constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)1 << 19;
size_t pair_force_noalloc_need(const Geo &g);
cudaError_t pair_force_noalloc(const Geo &g, const PairPrm &p, const double *x, const double *m,
                               double *f, cudaStream_t st);

// two species with the same P and box (md_pimd_x.c:3282-3632): cross pairs
// only, every bead of species a with every bead of species b in its slice;
// f_a += F/(m_a P), f_b -= F/(m_b P), with a's box.  scratch: at least
// pair2_scratch_doubles(ga, gb) doubles.
size_t pair2_scratch_doubles(const Geo &ga, const Geo &gb);
cudaError_t pair_force_2(const Geo &ga, const Geo &gb, const PairPrm &p, const double *xa, const double *ma,
                         const double *xb, const double *mb, double *fa, double *fb, double *scratch,
                         cudaStream_t st);
// sum over slices and cross pairs of V/P (plus -pi/(alpha^2 V) per pair for Ewald), added to *acc
cudaError_t pair_energy_2(const Geo &ga, const Geo &gb, const PairPrm &p, const double *xa, const double *xb,
                          double *acc, double *scratch, cudaStream_t st);

// Ewald reciprocal space through structure factors (D = 3)
// Wave vectors whose force weight |G| c(n) is below RECIP_KEEP of the
// largest are left out (c(n) = 0 and no column work): each is below the
// resolution of a double, and the reference's cube |n_i| <= nsum keeps them
// only because it is a cube (at alpha L = 5.6, nsum = 10 the kept ones are
// the 52% inside |n|^2 <= 111).
constexpr double RECIP_KEEP = 1e-17;
// The FP64 forces (recip_force with fp32_outer) take the columns whose
// every vector has a force weight below RECIP_SPLIT of the largest through
// the FP32 kernels (at alpha L = 5.6 the columns with nx^2 + ny^2 >= 49: 45%
// of the vectors); their FP32 rounding of a few 1e-7 then leaves below
// 1e-13 of the reciprocal force.
constexpr double RECIP_SPLIT = 1e-7;
struct Recip {
  int nsum;
  int nk;              // half-space wave vectors of the cube
  int ncol;            // kept columns (set by recip_setup)
  int tsz;             // entries of the kept columns' force tables (compact, set by recip_setup)
  int ncol_in, ncol_out;  // of those, the FP64 and the FP32 columns of the split (set by recip_setup)
  int tsz_in;          // entries of the FP64 columns' compact force tables (set by recip_setup)
  double *S32;         // [P][nk] FP32 complex structure factors of the split's FP32 columns, or NULL
  double *coef;        // [nk] s * exp(-pi^2 G^2/alpha^2) / (pi V G^2), 0 for a dropped vector;
                       // then the same nk values in FP32 (recip_coef_bytes(nk) bytes in all)
  int *kvec;           // kept columns, longest first: int4 (nx | nzmax << 8, ny, first nz,
                       // offset of its first k), then compact table offsets;
                       // recip_cols_ints(nsum) ints
  double *phase;       // [P][3][nsum+1][Ns] complex
  double *S;           // [P][nk] complex
  double *T;           // [P][columns][2 nsum + 1] complex force tables
  double csum;         // sum of coef (host value, set by recip_setup)
};
size_t recip_phase_doubles(const Geo &g, int nsum);
inline size_t recip_coef_bytes(int nk) { return (sizeof(double) + sizeof(float)) * (size_t)nk; }
int recip_count(int nsum);
size_t recip_cols_ints(int nsum);
size_t recip_table_doubles(const Geo &g, int nsum);
cudaError_t recip_setup(const Geo &g, int nsum, double alpha, double qs, Recip &r,
                        cudaStream_t st);
// fp32_outer (with r.S32 set): the split columns through the FP32 kernels
cudaError_t recip_force(const Geo &g, const Recip &r, const double *x, double inv_mP,
                        double *f, cudaStream_t st, bool fp32_outer = false);
cudaError_t recip_energy(const Geo &g, const Recip &r, const double *x, double *acc,
                         double *scratch, cudaStream_t st);

// two species (same P, box and Ewald parameters): a's forces from b's
// structure factors and b's from a's (both Recip's phase, S and T are
// rewritten); the cross energy sum_j sum_{n in H} 2 c(n) Re(S_a S_b*) / P
cudaError_t recip_force_2(const Geo &ga, const Recip &ra, const double *xa, double inv_mPa, double *fa,
                          const Geo &gb, const Recip &rb, const double *xb, double inv_mPb, double *fb,
                          cudaStream_t st);
cudaError_t recip_energy_2(const Geo &ga, const Recip &ra, const double *xa, const Geo &gb, const Recip &rb,
                           const double *xb, double *acc, double *scratch, cudaStream_t st);

// reciprocal-space forces plus per-particle energies
//   e[j*Ns + l] = sum_k c(k) (Re(e^{i k x_l} conj S_j(k)) - 1)  (half space)
// so that sum_l e = the slice's reciprocal energy; forces scaled as recip_force
cudaError_t recip_force_energy(const Geo &g, const Recip &r, const double *x, double scale, double *f,
                               double *e, cudaStream_t st);

// ---- mixed-precision form: FP32 arithmetic, compensated accumulation ----
cudaError_t pair_force32(const Geo &g, const PairPrm &p, const double *x, const double *m,
                         double *f, double *scratch, cudaStream_t st);
// tile shape (warps of 32 x 32 pair tiles per block: 1, 2, 4 or 8) of the
// FP32 pair kernel for a system shape; 8 unless set
void set_pair32_warps(int kind, int D, int N, int P, int warps);
int pair32_warps(int kind, int D, int N, int P);
// needs r.phase sized recip_phase_doubles(g, nsum) * 3 / 2 (FP32 copy behind)
cudaError_t recip_force32(const Geo &g, const Recip &r, const double *x, double inv_mP, double *f,
                          cudaStream_t st);

// static structure factor of slices ja, jb for nq wave vectors qis[3q..]:
// out[q] = (sum_l cos q.x_a)(sum_l cos q.x_b)/N + (sin)(sin)/N
cudaError_t sk_structure(const Geo &g, const double *x, int ja, int jb, const double *qis, int nq, double *out,
                         cudaStream_t st);

// ---- estimators ----
// primitive (ENk2 == nullptr) or virial exchange estimator; res[N] + add is
// added to *acc.  scratch: vbn_scratch_doubles(N) doubles.  G: the cycle
// probabilities G[l][j] (fill_g) of the same ENk, VBN, beta and xi, or null
// (then the reference's recursion is solved).
size_t vbn_scratch_doubles(int N);
cudaError_t vbn_energy(int N, double beta, double vi, double add, const double *ENk,
                       const double *VBN, const double *ENk2, double *acc, double *scratch, cudaStream_t st,
                       const double *G = nullptr);
cudaError_t force_virial(const Geo &g, const double *x, const double *f, const double *m,
                         int image, double *acc, double *scratch, cudaStream_t st);
cudaError_t add_scalar(double *acc, double v, cudaStream_t st);
// 0.5 sum over beads of -(x - c) . f m, c = L/2 (mode 0) or the particle's
// centroid (mode 1), plus `add`, added to *acc.  scratch: 304 doubles
cudaError_t virial_about(const Geo &g, const double *x, const double *f, const double *m, int mode, double add,
                         double *acc, double *scratch, cudaStream_t st);
// whole ring polymers shifted into the box by their first bead's image count
cudaError_t polymer_wrap(const Geo &g, double *x, cudaStream_t st);
// hist[k] = number of (l, q != l) whose bead-0 to bead-jb distance r has
// (int)(r / (rmax / points)) = k < points (minimum image when `image`)
cudaError_t pair_hist(const Geo &g, const double *x, int jb, int points, double rmax, int image, unsigned int *hist,
                      cudaStream_t st);
// f[i] += a[i], i < n
cudaError_t add_into(double *f, const double *a, size_t n, cudaStream_t st);

// ---- persistent ensemble step (xmd_ensemble.cu) ----
// One system's step as the persistent kernel runs it: the reference driver's
// sequence md_update_nhc_VV3_1_x, md_reset_force_x, md_pimd_fast_fill_ENk_x,
// md_pimd_fill_VB_x, md_pimd_fast_fill_force_VB_x, [trap force], [pair
// force, FP32 form], md_update_nhc_VV3_2_x, [md_periodic_boundary_x], with
// the arithmetic of those calls.  Pointers are the system's device buffers.
struct EnsSysDesc {
  Geo g;
  int image;      // minimum image in the springs (the ENk / force calls' flag)
  int wrap;       // periodic boundary at the end of the step
  int trap_kind;  // 0: no trap force
  TrapPrm tp;
  int pair_kind;  // 0: no pair force
  PairPrm pp;     // cut-off, image shifts and inverse mass set as for the force call
  double kT, h, beta, vi, w2;
  double *x, *v, *f, *m, *th, *vt;
  const double *Q, *iQ;
  double *fex;    // exchange spring forces (slots)
  double *xscr;   // partial sums of the end-bead forces (exch_scratch_doubles)
  double *Eint, *ENk, *gl;
  const double *lnn;
  double *VBN, *tmpV, *G;
  double *rs_f, *rs_b;  // recursion scratch, rec_scratch_doubles(N) each
  Recip rc;             // Ewald tables (pair_kind == PAIR_EWALD_REAL, D = 3)
  double inv_mP;        // 1 / (m P) of the reciprocal forces
};
struct EnsLaunch {
  void *plan = nullptr;  // device descriptors, group offsets, barriers, FP32 pair scratch
  void *goff = nullptr, *bar = nullptr;
  int D = 0, L = 0, blocks = 0, bps = 0, groups = 0, nsys = 0;
  size_t smem = 0;
  std::vector<double> cost;    // the estimated cost of each system (caller's order) the plan balanced
  std::vector<int> group_of;   // each system's group
  std::vector<double> load;    // each group's estimated total
};
constexpr int ENS_MAX_GROUPS = 32;
// thread blocks of the persistent kernel that fit on one SM (0: none)
int ensemble_max_blocks_per_sm(int D, int L);
// descriptors uploaded for a grid of blocks_per_sm x SMs blocks (capped at
// what fits) in `groups` groups with their own barriers, the systems spread
// over the groups by estimated cost (the built-in model, or `costs`)
cudaError_t ensemble_prepare(const EnsSysDesc *sys, int n, int D, int L, int blocks_per_sm, int groups,
                             EnsLaunch &e, const double *costs = nullptr);
cudaError_t ensemble_launch(const EnsLaunch &e, cudaStream_t st);
// *failed = 1 when a grid-barrier wait of an earlier launch gave up (its
// step and every later one did not run to completion); phase_us (optional,
// ENS_PHASES + 4 + ENS_MAX_GROUPS values): the last launch's phase
// durations as block 0 saw them (the phases end at the group's barriers;
// the last one at block 0's own end), block 0's own time in phase B for its
// springs, E_l^(1), pair tiles and structure factors, then each group's
// step time (its first block's start to end).  Synchronous.
constexpr int ENS_PHASES = 9;
cudaError_t ensemble_status(const EnsLaunch &e, int *failed, double *phase_us = nullptr);
void ensemble_free(EnsLaunch &e);
// the supported shapes: N <= ENS_MAX_N, L in {4, 8}, D in 1..3, n_sum <= 11
constexpr int ENS_MAX_N = 2048;

}  // namespace xk
