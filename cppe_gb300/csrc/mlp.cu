// MLP kernels: tiled SIMT GEMMs with split-K, bias/GELU epilogues, the loss
// of the learned guess + preconditioner correction with its gradient, Adam.
#include <cmath>
#include <random>

#include "mlp.h"

namespace cg {

constexpr int GT = 64, GK = 16;

// C = op(A) op(B): A(m,k) = TA ? A[k lda + m] : A[m lda + k],
//                  B(k,n) = TB ? B[n ldb + k] : B[k ldb + n].
// Block: 64 x 64 outputs, 256 threads with 4 x 4 each; blockIdx.z = K split.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256)
      k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
             const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc, int kchunk,
             const float* __restrict__ bias) {
  __shared__ float As[GK][GT + 4];
  __shared__ float Bs[GK][GT + 4];
  const int m0 = blockIdx.y * GT, n0 = blockIdx.x * GT;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = kbeg; k0 < kend; k0 += GK) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int e = threadIdx.x + 256 * q;
      int mm, kk;
      if (TA)
        kk = e / GT, mm = e % GT;
      else
        mm = e / GK, kk = e % GK;
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < kend) ? (TA ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k])
                                       : 0.f;
      int nn, kb;
      if (TB)
        nn = e / GK, kb = e % GK;
      else
        kb = e / GT, nn = e % GT;
      const int n = n0 + nn, kx = k0 + kb;
      Bs[kb][nn] = (n < N && kx < kend) ? (TB ? B[(size_t)n * ldb + kx] : B[(size_t)kx * ldb + n])
                                        : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
  float* Cz = C + (size_t)blockIdx.z * M * ldc;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty * 4 + i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx * 4 + j;
      if (n < N) Cz[(size_t)m * ldc + n] = acc[i][j] + (bias ? bias[n] : 0.f);
    }
  }
}

__global__ void k_sum_splits(int M, int N, int ldc, int splits, const float* __restrict__ part,
                             float* __restrict__ C, const float* __restrict__ bias) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)M * N) return;
  const int m = (int)(t / N), n = (int)(t % N);
  float s = bias ? bias[n] : 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * M * ldc + (size_t)m * ldc + n];
  C[(size_t)m * ldc + n] = s;
}

void gemm(bool ta, bool tb, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
          float* C, int ldc, const float* bias, int splits, float* part, cudaStream_t s) {
  splits           = std::max(1, splits);
  const int kchunk = ((K + splits - 1) / splits + GK - 1) / GK * GK;
  splits           = (K + kchunk - 1) / kchunk;
  dim3 grid((N + GT - 1) / GT, (M + GT - 1) / GT, splits);
  float* out        = splits > 1 ? part : C;
  const float* bout = splits > 1 ? nullptr : bias;
#define CG_GEMM(TA_, TB_) \
  k_gemm<TA_, TB_><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, out, splits > 1 ? N : ldc, kchunk, bout)
  if (!ta && !tb) CG_GEMM(false, false);
  if (!ta && tb) CG_GEMM(false, true);
  if (ta && !tb) CG_GEMM(true, false);
  if (ta && tb) CG_GEMM(true, true);
#undef CG_GEMM
  CG_LAUNCH();
  if (splits > 1) {
    const long tot = (long)M * N;
    k_sum_splits<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(M, N, N, splits, part, C, bias);
    CG_LAUNCH();
    (void)ldc;
  }
}

__device__ __forceinline__ float gelu(float z) { return 0.5f * z * (1.f + erff(z * 0.70710678f)); }
__device__ __forceinline__ float gelu_grad(float z) {
  return 0.5f * (1.f + erff(z * 0.70710678f)) + z * __expf(-0.5f * z * z) * 0.39894228f;
}

__global__ void k_gelu(long n, const float* __restrict__ Z, float* __restrict__ Hh) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) Hh[t] = gelu(Z[t]);
}

__global__ void k_gelu_back(long n, const float* __restrict__ dH, const float* __restrict__ Z,
                            float* __restrict__ dZ) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dZ[t] = dH[t] * gelu_grad(Z[t]);
}

__global__ void k_normalize(long rows, const float* __restrict__ raw, const float* __restrict__ mean,
                            const float* __restrict__ inv_std, float* __restrict__ X) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * Mlp::IN) return;
  const int c = (int)(t % Mlp::IN);
  X[t]        = (raw[t] - mean[c]) * inv_std[c];
}

// column sums of a rows x N matrix (bias gradients), rows split over blockIdx.y
__global__ void k_colsum(int rows, int N, const float* __restrict__ D, int rows_per,
                         float* __restrict__ part) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  const int r0 = blockIdx.y * rows_per, r1 = min(rows, r0 + rows_per);
  float s = 0.f;
  for (int r = r0; r < r1; ++r) s += D[(size_t)r * N + n];
  part[(size_t)blockIdx.y * N + n] = s;
}

__global__ void k_colsum_final(int N, int splits, const float* __restrict__ part,
                               float* __restrict__ out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int z = 0; z < splits; ++z) s += part[(size_t)z * N + n];
  out[n] = s;
}

// Loss rows and dL/dY (see oracle/mlp_oracle.py for the definition).
__global__ void k_loss_dy(int B, const float* __restrict__ Y, const float* __restrict__ T,
                          float lam, float* __restrict__ dY, double* partials, unsigned* ticket,
                          double* out) {
  __shared__ double sh[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double l[1] = {0.0};
  if (i < B) {
    const float* t = T + (size_t)i * Mlp::TROW;
    const float* y = Y + (size_t)i * Mlp::OUT;
    const float s = t[21], u = t[22];
    float dg[3], dp[3];
    for (int c = 0; c < 3; ++c) {
      dg[c] = y[0] * t[c] + y[1] * t[3 + c] + y[2] * t[6 + c] - t[9 + c];
      dp[c] = t[12 + c] + y[3] * t[15 + c] - t[18 + c];
    }
    const float invB = 1.f / (float)B;
    float g[4] = {0, 0, 0, 0};
    double lg = 0.0, lp = 0.0;
    for (int c = 0; c < 3; ++c) {
      g[0] += dg[c] * t[c];
      g[1] += dg[c] * t[3 + c];
      g[2] += dg[c] * t[6 + c];
      g[3] += dp[c] * t[15 + c];
      lg += (double)dg[c] * dg[c];
      lp += (double)dp[c] * dp[c];
    }
    float* d = dY + (size_t)i * Mlp::OUT;
    d[0] = 2.f * g[0] / s * invB;
    d[1] = 2.f * g[1] / s * invB;
    d[2] = 2.f * g[2] / s * invB;
    d[3] = 2.f * lam * g[3] / u * invB;
    l[0] = (lg / s + lam * lp / u) / B;
  }
  grid_sum_last<1>(l, sh, partials, ticket, out);
}

__global__ void k_adam(int n, float* __restrict__ w, const float* __restrict__ g,
                       float* __restrict__ m, float* __restrict__ v, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt, v[t] = vt;
  w[t] -= lr * (mt / c1) / (sqrtf(vt / c2) + eps);
}

Mlp::~Mlp() {
  if (stream) {
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    cudaStreamDestroy(stream);
  }
}

void Mlp::init(int dev, unsigned seed) {
  device = dev;
  CG_CUDA(cudaSetDevice(device));
  CG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  std::mt19937 rng(seed);
  std::vector<float> p(NPARAM, 0.f);
  auto fill = [&](int off, int cnt, float scale) {
    std::uniform_real_distribution<float> u(-scale, scale);
    for (int k = 0; k < cnt; ++k) p[off + k] = u(rng);
  };
  fill(0, NW1, 1.f / std::sqrt((float)IN));
  fill(NW1 + NB1, NW2, 1.f / std::sqrt((float)H));
  fill(NW1 + NB1 + NW2 + NB2, NW3, 0.01f / std::sqrt((float)H));
  // output bias: start at the three-term series mu = v1 + v2 + v3 and no correction
  float* b3h = &p[NW1 + NB1 + NW2 + NB2 + NW3];
  b3h[0] = 1.f, b3h[1] = 1.f, b3h[2] = 1.f, b3h[3] = 0.f;
  params.upload(p, stream);
  grads.alloc(NPARAM);
  adam_m.alloc(NPARAM);
  adam_v.alloc(NPARAM);
  adam_m.zero(stream);
  adam_v.zero(stream);
  std::vector<float> mean(IN, 0.f), istd(IN, 1.f);
  feat_mean.upload(mean, stream);
  feat_inv_std.upload(istd, stream);
  loss.alloc(1);
  ticket.alloc(1);
  ticket.zero(stream);
  tc_err.alloc(1);
  tc_err.zero(stream);
  step = 0;
  CG_CUDA(cudaStreamSynchronize(stream));
}

void Mlp::reserve(int rows) {
  if (rows <= cap) return;
  cap = rows;
  X.alloc((size_t)rows * IN);
  Z1.alloc((size_t)rows * H), H1.alloc((size_t)rows * H);
  Z2.alloc((size_t)rows * H), H2.alloc((size_t)rows * H);
  Y.alloc((size_t)rows * OUT), dY.alloc((size_t)rows * OUT);
  dA.alloc((size_t)rows * H), dB.alloc((size_t)rows * H);
  part.alloc((size_t)64 * H * H + (size_t)64 * H);
  loss_part.alloc((rows + 255) / 256 + 1);
}

// Inference on the tensor cores (mlp_tc.cu); tc_err reports a timed-out wait.
void Mlp::infer(int rows, const float* raw, float* Y_out, cudaStream_t s) {
  if (rows <= 0) return;
  tc_err.zero(s);
  mlp_infer_tc(device, rows, raw, params.p, feat_mean.p, feat_inv_std.p, Y_out, tc_err.p, s);
}

void Mlp::forward(int rows, const float* raw, float* Y_out, cudaStream_t s) {
  reserve(rows);
  const long nx = (long)rows * IN, nh = (long)rows * H;
  k_normalize<<<(unsigned)((nx + 255) / 256), 256, 0, s>>>(rows, raw, feat_mean.p, feat_inv_std.p, X.p);
  CG_LAUNCH();
  gemm(false, true, rows, H, IN, X.p, IN, W1(), IN, Z1.p, H, b1(), 1, nullptr, s);
  k_gelu<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(nh, Z1.p, H1.p);
  CG_LAUNCH();
  gemm(false, true, rows, H, H, H1.p, H, W2(), H, Z2.p, H, b2(), 1, nullptr, s);
  k_gelu<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(nh, Z2.p, H2.p);
  CG_LAUNCH();
  gemm(false, true, rows, OUT, H, H2.p, H, W3(), H, Y_out ? Y_out : Y.p, OUT, b3(), 1, nullptr, s);
}

double Mlp::loss_grad(int rows, const float* raw, const float* targets, float lam) {
  CG_CUDA(cudaSetDevice(device));
  cudaStream_t s = stream;
  forward(rows, raw, Y.p, s);
  const long nh = (long)rows * H;
  k_loss_dy<<<(rows + 255) / 256, 256, 0, s>>>(rows, Y.p, targets, lam, dY.p, loss_part.p,
                                                ticket.p, loss.p);
  CG_LAUNCH();
  const int splits = std::max(1, std::min(64, rows / 1024));
  float* gW1 = grads.p;
  float* gb1 = gW1 + NW1;
  float* gW2 = gb1 + NB1;
  float* gb2 = gW2 + NW2;
  float* gW3 = gb2 + NB2;
  float* gb3 = gW3 + NW3;
  const int rows_per = (rows + splits - 1) / splits;
  auto colsum = [&](const float* D, int N, float* out) {
    k_colsum<<<dim3((N + 127) / 128, splits), 128, 0, s>>>(rows, N, D, rows_per, part.p);
    CG_LAUNCH();
    k_colsum_final<<<(N + 127) / 128, 128, 0, s>>>(N, splits, part.p, out);
    CG_LAUNCH();
  };
  // layer 3: dW3 = dY^T H2, db3 = sum dY, dH2 = dY W3
  gemm(true, false, OUT, H, rows, dY.p, OUT, H2.p, H, gW3, H, nullptr, splits, part.p, s);
  colsum(dY.p, OUT, gb3);
  gemm(false, false, rows, H, OUT, dY.p, OUT, W3(), H, dA.p, H, nullptr, 1, nullptr, s);
  k_gelu_back<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(nh, dA.p, Z2.p, dB.p);
  CG_LAUNCH();
  // layer 2: dW2 = dZ2^T H1, db2, dH1 = dZ2 W2
  gemm(true, false, H, H, rows, dB.p, H, H1.p, H, gW2, H, nullptr, splits, part.p, s);
  colsum(dB.p, H, gb2);
  gemm(false, false, rows, H, H, dB.p, H, W2(), H, dA.p, H, nullptr, 1, nullptr, s);
  k_gelu_back<<<(unsigned)((nh + 255) / 256), 256, 0, s>>>(nh, dA.p, Z1.p, dB.p);
  CG_LAUNCH();
  // layer 1: dW1 = dZ1^T X, db1
  gemm(true, false, H, IN, rows, dB.p, H, X.p, IN, gW1, IN, nullptr, splits, part.p, s);
  colsum(dB.p, H, gb1);
  double l = 0.0;
  CG_CUDA(cudaMemcpyAsync(&l, loss.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  return l;
}

void Mlp::adam(float lr, float b1, float b2, float eps) {
  ++step;
  const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
  k_adam<<<(NPARAM + 255) / 256, 256, 0, stream>>>(NPARAM, params.p, grads.p, adam_m.p, adam_v.p,
                                                   lr, b1, b2, eps, c1, c2);
  CG_LAUNCH();
}

}  // namespace cg
