// xmd_learned.cuh -- kernels of the learned Ewald residual (no counterpart in
// MD-Lab): per-particle descriptors, a 64 -> 128 -> 128 -> 4 MLP on the
// tcgen05 tensor cores (BF16 operands, FP32 accumulation in tensor memory),
// its training step, and the kernels that apply and judge the correction.
//
// Rows are (bead slice j, particle l) pairs, row = j*N + l, padded to a
// multiple of 128 (one MMA tile).  Activation tiles live in global memory as
// "images": the exact byte order the tensor cores read from shared memory
// (K-major, no swizzle, 8 x 16-byte core matrices), so a tile moves with one
// bulk copy.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "xmd_kernels.cuh"

namespace xk {

constexpr int MLP_IN = 64, MLP_H = 128, MLP_OUT = 4, MLP_TILE = 128;
constexpr int DESC_BINS = 64;    // radial histogram bins on [0, rc)
constexpr int DESC_SHELLS = 32;  // reciprocal-lattice shells of the |S(k)| features
constexpr int DESC_VSTRIDE = 12; // floats per row of V: 3 vectors, weight, 2 pad
constexpr size_t MLP_TILE_BYTES = (size_t)MLP_TILE * MLP_IN * 2;  // one X tile image

// parameter vector layout (fp32 master copy), offsets in floats
constexpr int MLP_W1 = 0, MLP_B1 = MLP_W1 + MLP_H * MLP_IN, MLP_W2 = MLP_B1 + MLP_H,
              MLP_B2 = MLP_W2 + MLP_H * MLP_H, MLP_W3 = MLP_B2 + MLP_H,
              MLP_B3 = MLP_W3 + MLP_OUT * MLP_H, MLP_NPARAM = MLP_B3 + MLP_OUT;

// byte offset of element (r, k) in a K-major no-swizzle image of a (rows x K)
// BF16 operand: 8-row x 8-element core matrices of 128 contiguous bytes, core
// matrices adjacent along K 128 bytes apart, along the rows 16*K bytes apart
XK_HD inline uint32_t kmaj_off(int r, int k, int K) {
  return (uint32_t)((r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// device view of a network: packed images for the tensor cores, FP32 rest
struct MlpDev {
  const uint8_t *w1img;  // [128 x 64] image (n = output, k = input), 16 KB
  const uint8_t *w2img;  // [128 x 128] image, 32 KB
  const uint8_t *w3img;  // [16 x 128] image, rows 4..15 zero, 4 KB
  const float *b1, *b2, *b3;
  const float *w3f;      // [4][128] the BF16 values of W3 as FP32
};

// descriptor constants (host-computed from the box)
struct DescPrm {
  float rc, inv_h;             // cut-off radius (half the smallest box length), bins per unit
  float box[3], inv_box[3];
  float vmu[3], vinv2s2[3];    // vector radial bases: centres, 1/(2 sigma^2)
  // the same bases, equally spaced with one width (centres mu_m = mu_0 + m D,
  // a = 1/(2 sigma^2)), for the kernel: with t = r - mu_0, q_0 = 2^(-qa t^2),
  // rho = 2^(qc1 t + qc0), q_1 = q_0 rho, q_2 = q_1 rho qk (log2 e folded in)
  float qa, qc1, qc0, qk;
  float vscale[3];             // scale of each vector feature in V
  const float *basis;          // [DESC_BINS][32] histogram -> radial features (Gaussians in r)
  const int4 *kvec;            // half-space wave vectors of the lowest shells: (nx >= 0, ny, nz, shell)
  int nkvec, nmax;             // their count and largest |n_i|
  const float *shell_norm;     // [DESC_SHELLS] 1 / (N x half-space vectors of the shell)
  float *shell;                // [P][DESC_SHELLS] scratch: each slice's shell features (squared)
  const float *fmean, *fistd;  // feature normalisation
};

// features of every (slice, particle): normalised BF16 X tile images and
// scaled vector features V[row][12] (x,y,z of 3 vectors, row weight 1).
// raw != nullptr: also the unnormalised FP32 features raw[row][64] and
// unscaled V (for the statistics of the first data set).
cudaError_t desc_build(const Geo &g, const DescPrm &p, const double *x, uint8_t *ximg, float *V,
                       float *raw, cudaStream_t st);

// inference: Y[row] = MLP(X[row]) for ntiles tiles
cudaError_t mlp_forward(const MlpDev &w, const uint8_t *ximg, int ntiles, float4 *Y, int *err,
                        cudaStream_t st);

struct MlpLoss {
  float we, wf;      // weights of the energy and force terms
  float inv_rows;    // 1 / rows in the batch
};
// one training step's gradients: grad (MLP_NPARAM floats, accumulated with
// atomics, zeroed by the caller) and loss[2] (energy, force terms).  tiles:
// batch tiles drawn from [0, ntiles_data) by a hash of (seed, index); seed 0
// takes tiles 0 .. batch_tiles-1 in order (batch_tiles <= ntiles_data).
// mn_variant: descriptor reading of MN-major operands; only 0 (the one
// tc_selftest confirms) is accepted.
cudaError_t mlp_train_grad(const MlpDev &w, const uint8_t *ximg, const float *V, const float4 *T,
                           int ntiles_data, int batch_tiles, uint32_t seed, MlpLoss loss, float *grad,
                           float *lossacc, int mn_variant, int *err, cudaStream_t st);

// Adam on the FP32 master parameters, then repack the images; zeroes grad
struct AdamPrm {
  float lr, b1, b2, eps, c1, c2;  // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
};
cudaError_t mlp_adam(float *param, float *grad, float *m1, float *m2, AdamPrm a, uint8_t *w1img,
                     uint8_t *w2img, uint8_t *w3img, float *w3f, cudaStream_t st);
// images from the master parameters without an update
cudaError_t mlp_pack(const float *param, uint8_t *w1img, uint8_t *w2img, uint8_t *w3img, float *w3f,
                     cudaStream_t st);

// output scaling of the network (host-computed from the first data set)
struct ResidPrm {
  float e_mean, e_scale;  // e = e_mean + e_scale y0
  float f_scale;          // F = f_scale sum_m y_m V_m
};
// f[j][d][l] += scale * F_row (scale = 1/(m P)), or, with fout != nullptr,
// fout[(j*3 + d)*Ns + l] = F_row; ep != nullptr: ep[j*Ns + l] = e_row
cudaError_t resid_apply(const Geo &g, ResidPrm r, const float4 *Y, const float *V, double scale, double *f,
                        double *fout, double *ep, cudaStream_t st);

// training targets of one configuration: T[row] = ((e_conv - e_trunc - e_mean)/e_scale,
// (F_conv - F_trunc)/f_scale); forces fa/fb and energies ea/eb in SoA slices
cudaError_t resid_targets(const Geo &g, ResidPrm r, const double *fa, const double *fb, const double *ea,
                          const double *eb, float4 *T, cudaStream_t st);

// judge sums (acc holds 3 + 2P doubles, acc[0..2] zeroed by the caller):
// acc[0] += sum |Fp - (Fa - Fb)|^2, acc[1] += sum |Fa|^2, acc[2] += sum
// |Fa - Fb|^2; acc[3 + j] = sum_l ep - (ea - eb), acc[3 + P + j] = sum_l ea - eb
cudaError_t resid_judge(const Geo &g, const double *fp, const double *fa, const double *fb, const double *ep,
                        const double *ea, const double *eb, double *acc, cudaStream_t st);

// w * (sum over slices and particles of e[j*Ns + l]) added to *acc
cudaError_t sum_particles(const Geo &g, const double *e, double w, double *acc, cudaStream_t st);
// status word of tensor-core kernels launched with err == nullptr
cudaError_t tc_status(int *out, bool clear);
// cycles a tensor-core kernel waits on one mbarrier phase before it gives up
// and records an error (default 2^32, about two seconds at 2 GHz)
long long wait_limit();
void set_wait_limit(long long cycles);
// the wait-limit self-test kernel: a barrier whose 16 bytes never arrive,
// waited for with `limit`; *status = the recorded status (4 on a time-out),
// *cycles = the cycles the wait took
cudaError_t wait_probe(long long limit, int *status, long long *cycles, cudaStream_t st);

// tensor-core layout self-test: D = A B^T on one CTA for K-major operands
// and for MN-major A / B under both readings of the descriptor offsets.
// err[0..4]: K-major, A MN (variant 0), A MN (variant 1), B MN (variant 0),
// B MN (variant 1): max |D - reference| over the tile
cudaError_t tc_selftest(double err[5], cudaStream_t st);

}  // namespace xk
