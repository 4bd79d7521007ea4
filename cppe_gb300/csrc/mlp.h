// Small MLP (64 -> 128 -> 128 -> 4, GELU, FP32) trained and evaluated on the
// GPU by hand-written kernels: tiled GEMMs, fused bias/activation epilogues,
// the loss of the learned initial guess and preconditioner correction, and
// Adam.  No counterpart in the reference.
#pragma once

#include "common.cuh"

namespace cg {

struct Mlp {
  static constexpr int IN = 64, H = 128, OUT = 4;
  static constexpr int NW1 = H * IN, NB1 = H, NW2 = H * H, NB2 = H, NW3 = OUT * H, NB3 = OUT;
  static constexpr int NPARAM = NW1 + NB1 + NW2 + NB2 + NW3 + NB3;
  // target row of the loss: v1 v2 v3 mu* a w e (21) s t pad
  static constexpr int TROW = 24;

  int device          = 0;
  cudaStream_t stream = nullptr;
  DBuf<float> params, grads, adam_m, adam_v;
  DBuf<float> feat_mean, feat_inv_std;  // input normalisation
  int step = 0;
  // workspace for a batch of up to `cap` rows
  int cap = 0;
  DBuf<float> X, Z1, H1, Z2, H2, Y, dY, dA, dB, part;
  DBuf<double> loss_part, loss;
  DBuf<unsigned> ticket;
  DBuf<int> tc_err;  // error code of the tensor-core inference (0: none)

  ~Mlp();
  void init(int device, unsigned seed);
  void reserve(int rows);
  float* W1() { return params.p; }
  float* b1() { return params.p + NW1; }
  float* W2() { return params.p + NW1 + NB1; }
  float* b2() { return params.p + NW1 + NB1 + NW2; }
  float* W3() { return params.p + NW1 + NB1 + NW2 + NB2; }
  float* b3() { return params.p + NW1 + NB1 + NW2 + NB2 + NW3; }
  // Y (rows x 4) for raw descriptors (rows x 64, device); normalises first.
  // forward keeps the intermediate layers (training); infer is one fused pass.
  void forward(int rows, const float* raw, float* Y_out, cudaStream_t s);
  void infer(int rows, const float* raw, float* Y_out, cudaStream_t s);
  // loss and parameter gradients (into grads) for one batch; returns loss.
  double loss_grad(int rows, const float* raw, const float* targets, float lam);
  void adam(float lr, float b1 = 0.9f, float b2 = 0.999f, float eps = 1e-8f);
};

// Y (rows x 4) = MLP(normalised raw) on the tensor cores (tcgen05, TF32
// operands, FP32 accumulation); *err receives 1 if a wait timed out.
void mlp_infer_tc(int device, int rows, const float* raw, const float* params,
                  const float* mean, const float* inv_std, float* Y, int* err, cudaStream_t s);

// C = op(A) op(B) (+ bias over columns), row-major, FP32; split over K into
// `splits` partial products added in fixed order.
void gemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
          float* C, int ldc, const float* bias, int splits, float* part, cudaStream_t s);

}  // namespace cg
