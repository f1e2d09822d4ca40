// pm_learned.h — learned per-cell smoother (no counterpart in the reference):
// a 397 -> 256 -> 256 -> 85 MLP with GELU, BF16 weights and activations and
// FP32 accumulation on the tensor cores (forward layers: tcgen05.mma with
// TMEM accumulators; training gradients: mma.sync m16n8k16), trained on the
// GPU from (residual, error) pairs of the plain solver.
#ifndef PM_LEARNED_H
#define PM_LEARNED_H

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "pm_kernels.h"

namespace pm {

constexpr int kMlpIn = 397;      // 85 local residual + 26 neighbours x 12 summaries
constexpr int kMlpInPad = 400;   // multiple of 16
constexpr int kMlpHidden = 256;
constexpr int kMlpOut = 85;
constexpr int kMlpOutPad = 96;
constexpr int kSummary = 12;
constexpr int kNeighbours = 26;
constexpr float kFeatureClamp = 1.0e3f;  // |feature| bound (features are O(1) residual ratios)

// offsets of the parameter blocks in the flat FP32 parameter vector
constexpr long long kOffW1 = 0;
constexpr long long kOffB1 = kOffW1 + (long long)kMlpHidden * kMlpInPad;
constexpr long long kOffW2 = kOffB1 + kMlpHidden;
constexpr long long kOffB2 = kOffW2 + (long long)kMlpHidden * kMlpHidden;
constexpr long long kOffW3 = kOffB2 + kMlpHidden;
constexpr long long kOffB3 = kOffW3 + (long long)kMlpOutPad * kMlpHidden;
constexpr long long kNumParams = kOffB3 + kMlpOutPad;

struct Mlp {
  int device = 0;
  int max_batch = 0;
  long long step = 0;
  float *P = nullptr, *G = nullptr, *Mo = nullptr, *Vo = nullptr;  // params, grads, Adam moments
  __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W3 = nullptr;      // BF16 copies
  __nv_bfloat16 *W2t = nullptr, *W3t = nullptr;  // BF16 transposes (gradient GEMMs)
  // transposed training operands [rows x ldt] (K = batch rows contiguous)
  __nv_bfloat16 *Tx = nullptr, *Th = nullptr, *Ta = nullptr, *Ty = nullptr;
  int ldt = 0;
  // training workspace (max_batch rows)
  __nv_bfloat16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dYb = nullptr, *dA2b = nullptr,
                *dA1b = nullptr;
  float *pre1 = nullptr, *pre2 = nullptr, *Y = nullptr, *dY = nullptr, *dH = nullptr;
  double *loss = nullptr;
  int *err = nullptr;   // device flags of bounded waits in the tcgen05 layers
  bool tc = true;       // forward layers on tcgen05 (else mma.sync)
  cudaStream_t stream = nullptr;
};

// tcgen05 forward layer (pm_mlp_tc.cu): layer 1 (X [M x 400] -> [M x 256]),
// 2 ([M x 256] -> [M x 256]) or 3 ([M x 256] -> [M x 96]) with bias and, if
// act, GELU; outputs pre-activation (FP32), FP32 and/or BF16 rows.
int mlp_layer_tc(int layer, const __nv_bfloat16 *A, int M, const __nv_bfloat16 *W,
                 const float *bias, int act, float *pre, float *Cf, __nv_bfloat16 *Cb,
                 const int *on, int *err, cudaStream_t s);
// sets the layers' shared-memory limits (once, outside stream capture)
int mlp_tc_init();
// C[rows x n] = A B^T on the tcgen05 path (FP32 out, row pitch ldc) for A
// [rows x k] (pitch lda) and B [n x k] (pitch ldb), both BF16 with k
// contiguous; n in {96, 256, 400}; pitches in elements, multiples of 8
int mlp_gemm_tc(const __nv_bfloat16 *A, int lda, int rows, const __nv_bfloat16 *B, int ldb,
                int n, int k, float *C, int ldc, int *err, cudaStream_t s);

// allocate / free (returns cudaError_t)
cudaError_t mlp_create(Mlp &m, int device, unsigned long long seed, int max_batch);
void mlp_destroy(Mlp &m);
// refresh the BF16 weight copies from the FP32 parameters
int mlp_sync_bf16(const Mlp &m, cudaStream_t s);
// Inference: X [M x 400] BF16 (padded) -> Y [M x 96] FP32; H1/H2 workspaces [M x 256].
int mlp_forward(const Mlp &m, const __nv_bfloat16 *X, int M, __nv_bfloat16 *H1,
                __nv_bfloat16 *H2, float *Y, cudaStream_t s, const int *on = nullptr,
                int *err = nullptr);
// Inference on unpadded FP32 rows: X [M x 397] -> Yout [M x 85] (M <= max_batch)
int mlp_forward_f32(Mlp &m, const float *X, int M, float *Yout, cudaStream_t s);
// Training: X [M x 397] FP32, T [M x 85] FP32 -> loss (device double), grads in m.G
int mlp_loss_grad(Mlp &m, const float *X, const float *T, int M, cudaStream_t s);
int mlp_adamw(Mlp &m, float lr, float b1, float b2, float eps, float wd, cudaStream_t s);

// Features of the cells of one level from the level defect d (precision T):
// summary[c*12 + q] per cell, then X[c*400 + :] (BF16, divided by the cell
// scale) and scale[c] = rms of the cell's 85 local residual entries.
template <typename T>
int launch_cell_summary(const DevCells &cells, int nu, const T *d, float *summary,
                        const int *on, cudaStream_t s);
template <typename T>
int launch_cell_features(const DevCells &cells, int nu, const T *d, const float *summary,
                         const int *nbr, __nv_bfloat16 *Xb, float *Xf, float *scale,
                         const int *on, cudaStream_t s);
// u[dofs] += omega * inv_mult[dof] * scale[c] * Y[c, i] over the cells of one
// colour (velocity Dirichlet DOFs untouched).
template <typename T>
int launch_learned_apply(const DevCells &cells, int nu, int nact, const int *cell_list, int ncol,
                         const float *Y, const float *scale, const float *inv_mult_u, T omega,
                         T *u, const int *on, cudaStream_t s);
// Minimal-residual step length of a correction c with d = f - K u and
// q = P(-K c) (projected like the defect): omega = clamp(-<d,q>/<q,q>,
// 0, omega_max) written to *omega; deterministic two-stage sums in FP64.
// partials needs 2 * 608 + 2 doubles; counter must be 0 and is reset.
template <typename T>
int launch_mr_step(const T *d, const T *q, int n, double *partials, unsigned int *counter,
                   double omega_max, double *omega, const int *on, cudaStream_t s);
// u += (*omega) * c
template <typename T>
int launch_axpy_dev(T *u, const double *omega, const T *c, int n, const int *on, cudaStream_t s);
// harvest targets: T[c*85 + i] = e[dof_i(c)] / scale[c]
template <typename T>
int launch_cell_targets(const DevCells &cells, int nu, const T *e, const float *scale, float *Tg,
                        cudaStream_t s);

}  // namespace pm
#endif
