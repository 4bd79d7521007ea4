// Shared host/device helpers of libcppe_gpu: error plumbing, device buffers,
// the pair kernels of the three source orders, and block reductions.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "cppe_gpu.h"

namespace cg {

// ---------------------------------------------------------------------------
// Errors: every C-ABI entry point catches cg::Failure and returns its status.
// ---------------------------------------------------------------------------
struct Failure : std::runtime_error {
  int status;
  Failure(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string& msg);

[[noreturn]] inline void fail(int status, const std::string& msg) { throw Failure(status, msg); }

inline void cuda_check(cudaError_t e, const char* what, const char* file, int line) {
  if (e != cudaSuccess) {
    int st = (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                   ? CPPE_GPU_NO_DEVICE
                   : CPPE_GPU_CUDA_ERROR;
    fail(st, std::string(what) + " failed: " + cudaGetErrorString(e) + " (" + file + ":" +
                   std::to_string(line) + ")");
  }
}
// Kernels launched by this library (every launch site is followed by
// CG_LAUNCH, which checks the launch and counts it).
long long& launch_counter();

#define CG_CUDA(x) ::cg::cuda_check((x), #x, __FILE__, __LINE__)
#define CG_LAUNCH()                                                             \
  do {                                                                          \
    ::cg::cuda_check(cudaGetLastError(), "kernel launch", __FILE__, __LINE__); \
    ++::cg::launch_counter();                                                   \
  } while (0)

// Set while this thread captures a CUDA graph.  Work buffers must have their
// size by then: a cudaFree or cudaMalloc inside the capture would end it.
inline thread_local bool g_capturing = false;
struct CaptureScope {
  CaptureScope() { g_capturing = true; }
  ~CaptureScope() { g_capturing = false; }
};

// Device buffer owning cudaMalloc'd memory.
template <class T>
struct DBuf {
  T* p     = nullptr;
  size_t n = 0;
  DBuf()   = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr, o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    release();
    p = o.p, n = o.n;
    o.p = nullptr, o.n = 0;
    return *this;
  }
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr, n = 0;
  }
  void alloc(size_t count) {
    if (count == n && p) return;
    if (g_capturing) fail(CPPE_GPU_CUDA_ERROR, "device buffer resized during graph capture");
    release();
    if (count == 0) return;
    CG_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T* h, size_t count, cudaStream_t s) {
    alloc(count);
    if (count) CG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s) { upload(h.data(), h.size(), s); }
  void zero(cudaStream_t s) {
    if (n) CG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
  }
};

// ---------------------------------------------------------------------------
// Device math
// ---------------------------------------------------------------------------
__device__ __forceinline__ float rsqrt_t(float x) { return rsqrtf(x); }
__device__ __forceinline__ double rsqrt_t(double x) { return rsqrt(x); }
__device__ __forceinline__ float exp_neg(float v) { return __expf(-v); }
__device__ __forceinline__ double exp_neg(double v) { return exp(-v); }

// Radial factors of the (Thole-damped) interaction at separation r with
// r2 = |r|^2 and damping parameter a = f / (alpha_i alpha_j)^(1/6) (a <= 0:
// undamped), for g(R) = f_v(aR)/R:
//   G1 = (1/R) g'        = -f_E / R^3
//   G2 = (1/R d/dR) G1   =  3 f_T / R^5
//   G3 = (1/R d/dR) G2   = -15 f_D / R^7
// with the exponential Thole screening factors
//   f_v = 1 - (1 + v/2) e^-v,  f_E = f_v - (v^2/2 + v/2) e^-v,
//   f_T = f_E - v^3/6 e^-v,    f_D = f_T - v^4/30 e^-v,   v = a R
// (the factors of src/core/tensors/tensors_recursive.cc:93-114, which the
// generated P2P kernels of src/core/fmm/field_m{0,1,2}.cc differentiate).
// r2 == 0 (a site paired with itself) yields all-zero factors.
// FAST (FP64 only): for v >= 20 the exponential is taken in FP32 (expf of the
// FP32-rounded argument, relative error below 4e-6 in e^-v); the damping
// factors then differ from the all-FP64 ones by less than 1e-11 relative.
template <typename T, int NG, bool FAST = false>
__device__ __forceinline__ void radial(T r2, T a, T* G) {
  const T ir  = r2 > T(0) ? rsqrt_t(r2) : T(0);
  const T ir2 = ir * ir;
  const T ir3 = ir2 * ir;
  G[0]        = -ir3;
  if (NG > 1) G[1] = T(3) * ir3 * ir2;
  if (NG > 2) G[2] = T(-15) * ir3 * ir2 * ir2;
  if (a > T(0)) {
    const T v = a * r2 * ir;
    // e^-v below 2e-22 leaves every factor exactly 1 in FP64.
    if (v < T(50)) {
      const T e = (FAST && sizeof(T) == 8 && v >= T(20)) ? (T)expf(-(float)v) : exp_neg(v);
      const T fE = T(1) - (T(1) + v + T(0.5) * v * v) * e;
      G[0] *= fE;
      if (NG > 1) {
        const T fT = fE - v * v * v * (T(1) / T(6)) * e;
        G[1] *= fT;
        if (NG > 2) G[2] *= fT - v * v * v * v * (T(1) / T(30)) * e;
      }
    }
  }
}

// Field at r = target - source of a charge, a dipole, or a quadrupole with the
// multi-index moments S = (xx, xy, xz, yy, yz, zz), in the sign convention of
// the reference's Tree<m,3> (fmm P2P<m,3>): F_c = -sum_{|k|=m} S_k d_{k+e_c} g.
template <typename T>
__device__ __forceinline__ void field_m0(T x, T y, T z, const T* G, T q, T& fx, T& fy, T& fz) {
  const T c = -q * G[0];
  fx += c * x, fy += c * y, fz += c * z;
}
template <typename T>
__device__ __forceinline__ void field_m1(T x, T y, T z, const T* G, T sx, T sy, T sz, T& fx,
                                         T& fy, T& fz) {
  const T sr = (sx * x + sy * y + sz * z) * G[1];
  fx -= sx * G[0] + sr * x;
  fy -= sy * G[0] + sr * y;
  fz -= sz * G[0] + sr * z;
}
template <typename T>
__device__ __forceinline__ void field_m2(T x, T y, T z, const T* G, const T* S, T& fx, T& fy,
                                         T& fz) {
  const T qxx = S[0], qxy = T(0.5) * S[1], qxz = T(0.5) * S[2], qyy = S[3],
          qyz = T(0.5) * S[4], qzz = S[5];
  const T tr  = qxx + qyy + qzz;
  const T qrx = qxx * x + qxy * y + qxz * z;
  const T qry = qxy * x + qyy * y + qyz * z;
  const T qrz = qxz * x + qyz * y + qzz * z;
  const T rqr = (x * qrx + y * qry + z * qrz) * G[2];
  fx -= G[1] * (tr * x + T(2) * qrx) + rqr * x;
  fy -= G[1] * (tr * y + T(2) * qry) + rqr * y;
  fz -= G[1] * (tr * z + T(2) * qrz) + rqr * z;
}

// Error-free transformation a + b = s + e (Knuth two-sum); used to carry a
// compensation term next to FP32 accumulators.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s        = a + b;
  float bb = s - a;
  e        = (a - (s - bb)) + (b - bb);
}

// ---------------------------------------------------------------------------
// Deterministic grid reductions: each block writes partial sums; the last
// block to finish (ticket counter) adds them in block order and calls fin().
// ---------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double* sh /* >= 32*K */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double x = v[k];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) sh[wid * K + k] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += sh[w * K + k];
      v[k] = s;
    }
  }
  __syncthreads();
}

// The same block sum from FP32 per-thread values (GB300's FP64 pipe runs at
// about 1/75 of its FP32 rate, so the per-thread products and the warp
// reduction stay in FP32): a compensated warp reduction (two-sum, the error
// terms carried along), then the warps' sums in FP64 in thread 0.
template <int K>
__device__ __forceinline__ void block_sum(const float (&vf)[K], double (&v)[K],
                                          double* sh /* >= 32*K */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    float x = vf[k], e = 0.f;
    for (int o = 16; o > 0; o >>= 1) {
      const float xo = __shfl_down_sync(0xffffffffu, x, o);
      const float eo = __shfl_down_sync(0xffffffffu, e, o);
      float t, te;
      two_sum(x, xo, t, te);
      x = t;
      e += eo + te;
    }
    if (lane == 0) sh[wid * K + k] = (double)x + (double)e;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
      double s = 0.0;
      for (int w = 0; w < nw; ++w) s += sh[w * K + k];
      v[k] = s;
    }
  }
  __syncthreads();
}

// Last-block part of grid_sum_last, after the block sum is in thread 0.
template <int K>
__device__ __forceinline__ bool grid_finish_last(double (&v)[K], double* sh, double* partials,
                                                 unsigned* ticket, double* out);

// Returns true in thread 0 of the last block; partials[b*K + k] hold the
// per-block sums, and `out` receives the totals.  The last block adds the
// partials with all its threads (thread t takes blocks t, t + blockDim, ...,
// then a block reduction): a fixed order, so the result does not depend on
// which block finishes last.
template <int K>
__device__ __forceinline__ bool grid_sum_last(double (&v)[K], double* sh, double* partials,
                                              unsigned* ticket, double* out) {
  block_sum<K>(v, sh);
  return grid_finish_last<K>(v, sh, partials, ticket, out);
}
// FP32 per-thread values (see block_sum above).
template <int K>
__device__ __forceinline__ bool grid_sum_last(const float (&vf)[K], double* sh, double* partials,
                                              unsigned* ticket, double* out) {
  double v[K];
  block_sum<K>(vf, v, sh);
  return grid_finish_last<K>(v, sh, partials, ticket, out);
}

template <int K>
__device__ __forceinline__ bool grid_finish_last(double (&v)[K], double* sh, double* partials,
                                                 unsigned* ticket, double* out) {
  __shared__ bool last;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) partials[blockIdx.x * K + k] = v[k];
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    last       = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double s[K];
#pragma unroll
  for (int k = 0; k < K; ++k) s[k] = 0.0;
  for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
#pragma unroll
    for (int k = 0; k < K; ++k) s[k] += __ldcg(partials + b * K + k);
  block_sum<K>(s, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; ++k) out[k] = s[k];
    *ticket = 0;
  }
  return threadIdx.x == 0;
}

}  // namespace cg
