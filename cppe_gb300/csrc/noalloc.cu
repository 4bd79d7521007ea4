// Allocation-free direct-summation apply of the induced-dipole operator.
//
// Some callers cannot allocate GPU memory at the point where they need the
// operator: a quantum-chemistry host that hands us a fixed memory pool and
// forbids further cudaMalloc, or a callback invoked from a real-time loop that
// must not enter the allocator (whose calls can synchronize the device or take
// locks).  For them this file offers cppe_gpu_bmatrix_apply_direct_noalloc:
// the same B = alpha^-1 - T(damped) operator as cppe_gpu_bmatrix_apply with
// direct summation, on caller-owned device buffers, whose only scratch is the
// fixed array below.
//
// The scratch is a file-scope __device__ array, so every GPU that loads this
// library holds it (1.75 MiB) until the process exits.  Host code must not
// pass the array's name to a kernel (on the host it is only a stand-in for the
// device symbol); its device address is looked up once per device with
// cudaGetSymbolAddress, on the first call made with that device current, and
// kept for the life of the process (a cudaDeviceReset invalidates it).
//
// Excluded pairs are skipped inside the pair pass, as the reference skips
// them (bmatrix.cc:28 compares each partner with the target's exclusion
// list), so no large intramolecular term is added and subtracted again.
#include <mutex>

#include "common.cuh"

namespace cg {

constexpr int NOALLOC_MAX_SITES = 8192;
constexpr int NOALLOC_SPLITS    = 8;
constexpr int NOALLOC_BLOCK     = 128;
// per call: packed sites (x, y, z, s) 4n doubles + source-split partial fields
// NOALLOC_SPLITS * 3n doubles
constexpr size_t NOALLOC_SCRATCH_DOUBLES =
      (size_t)NOALLOC_MAX_SITES * 4 + (size_t)NOALLOC_SPLITS * 3 * NOALLOC_MAX_SITES;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

namespace {
std::mutex g_noalloc_mu;
double* g_noalloc_ptr[128] = {};

double* noalloc_scratch(int device) {
  if (device < 0 || device >= 128) fail(CPPE_GPU_INVALID_ARG, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[device]) {
    void* p       = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      cudaGetLastError();
      fail(CPPE_GPU_CUDA_ERROR,
           std::string("cudaGetSymbolAddress(noalloc scratch) failed: ") + cudaGetErrorString(e));
    }
    g_noalloc_ptr[device] = static_cast<double*>(p);
  }
  return g_noalloc_ptr[device];
}
}  // namespace

// (x, y, z, s) per site; s = alpha_iso^(-1/6) when damping applies.
__global__ void k_noalloc_pack(int n, const double* __restrict__ xyz,
                               const double* __restrict__ a6, int damp,
                               double* __restrict__ pos4) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double iso = (a6[6 * i] + a6[6 * i + 3] + a6[6 * i + 5]) / 3.0;
  pos4[4 * i]     = xyz[3 * i];
  pos4[4 * i + 1] = xyz[3 * i + 1];
  pos4[4 * i + 2] = xyz[3 * i + 2];
  pos4[4 * i + 3] = (damp && iso > 0.0) ? pow(iso, -1.0 / 6.0) : 0.0;
}

// Field of all dipoles of one source split at each target.  The self pair
// gives 0; a source in the target's exclusion list is skipped.  Two distinct,
// non-excluded sites at the same position make the operator undefined (the
// reference divides by zero there): the target's output becomes NaN.
__global__ void __launch_bounds__(NOALLOC_BLOCK)
      k_noalloc_pairs(int n, const double* __restrict__ pos4, const double* __restrict__ mu,
                      const int* __restrict__ ep, const int* __restrict__ ei, int damp,
                      double damping, double* __restrict__ part) {
  __shared__ double s_p[NOALLOC_BLOCK * 4];
  __shared__ double s_m[NOALLOC_BLOCK * 3];
  const int i     = blockIdx.x * NOALLOC_BLOCK + threadIdx.x;
  const int split = blockIdx.y;
  const int per   = (n + gridDim.y - 1) / gridDim.y;
  const int j0 = min(n, split * per), j1 = min(n, j0 + per);
  double xi = 0, yi = 0, zi = 0, ai = 0;
  // the first four exclusions in registers, the rest read from the list
  int eb = 0, ee = 0, x0 = -1, x1 = -1, x2 = -1, x3 = -1;
  if (i < n) {
    xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2], ai = damping * pos4[4 * i + 3];
    if (ep) {
      eb = ep[i], ee = ep[i + 1];
      if (eb < ee) x0 = ei[eb];
      if (eb + 1 < ee) x1 = ei[eb + 1];
      if (eb + 2 < ee) x2 = ei[eb + 2];
      if (eb + 3 < ee) x3 = ei[eb + 3];
    }
  }
  double fx = 0, fy = 0, fz = 0;
  bool coincident = false;
  for (int t0 = j0; t0 < j1; t0 += NOALLOC_BLOCK) {
    const int cnt = min(NOALLOC_BLOCK, j1 - t0);
    __syncthreads();
    if (threadIdx.x < cnt) {
      const int j = t0 + threadIdx.x;
      for (int c = 0; c < 4; ++c) s_p[4 * threadIdx.x + c] = pos4[4 * j + c];
      for (int c = 0; c < 3; ++c) s_m[3 * threadIdx.x + c] = mu[3 * j + c];
    }
    __syncthreads();
    if (i < n)
      for (int jj = 0; jj < cnt; ++jj) {
        const int j = t0 + jj;
        bool skip = (j == x0) | (j == x1) | (j == x2) | (j == x3);
        for (int e = eb + 4; e < ee; ++e) skip |= (ei[e] == j);
        if (skip) continue;
        const double x = xi - s_p[4 * jj], y = yi - s_p[4 * jj + 1], z = zi - s_p[4 * jj + 2];
        const double r2 = x * x + y * y + z * z;
        coincident |= (r2 == 0.0) & (j != i);
        double G[2];
        radial<double, 2>(r2, damp ? ai * s_p[4 * jj + 3] : 0.0, G);
        field_m1(x, y, z, G, s_m[3 * jj], s_m[3 * jj + 1], s_m[3 * jj + 2], fx, fy, fz);
      }
  }
  if (i < n) {
    if (coincident) fx = fy = fz = __longlong_as_double(0x7ff8000000000000ULL);
    double* o = part + (size_t)split * 3 * n + 3 * (size_t)i;
    o[0] = fx, o[1] = fy, o[2] = fz;
  }
}

// out_i = sum of split fields + alpha_i^-1 mu_i (thread i reads only site i's
// moments and writes only site i's output).
__global__ void k_noalloc_finish(int n, int nsplit, const double* __restrict__ part,
                                 const double* __restrict__ mu, const double* __restrict__ a6,
                                 double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f[3] = {0, 0, 0};
  for (int s = 0; s < nsplit; ++s)
    for (int c = 0; c < 3; ++c) f[c] += part[(size_t)s * 3 * n + 3 * (size_t)i + c];
  const double* s = a6 + 6 * (size_t)i;
  const double A = s[3] * s[5] - s[4] * s[4], B = s[2] * s[4] - s[1] * s[5],
               C = s[1] * s[4] - s[2] * s[3];
  const double id = 1.0 / (s[0] * A + s[1] * B + s[2] * C);
  const double inv[6] = {A * id, B * id, C * id, (s[0] * s[5] - s[2] * s[2]) * id,
                         (s[1] * s[2] - s[0] * s[4]) * id, (s[0] * s[3] - s[1] * s[1]) * id};
  const double* v = mu + 3 * (size_t)i;
  out[3 * (size_t)i]     = f[0] + inv[0] * v[0] + inv[1] * v[1] + inv[2] * v[2];
  out[3 * (size_t)i + 1] = f[1] + inv[1] * v[0] + inv[3] * v[1] + inv[4] * v[2];
  out[3 * (size_t)i + 2] = f[2] + inv[2] * v[0] + inv[4] * v[1] + inv[5] * v[2];
}

// Whether the byte ranges [a, a + na) and [b, b + nb) share a byte.
static bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
  if (!a || !b) return false;
  const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
  return pa < pb + nb && pb < pa + na;
}

void set_last_error(const std::string& msg);

}  // namespace cg

using namespace cg;

extern "C" int cppe_gpu_bmatrix_apply_direct_noalloc(int n, const double* d_xyz,
                                                     const double* d_alpha6,
                                                     const int* d_excl_ptr,
                                                     const int* d_excl_idx, int damp,
                                                     double damping_factor, const double* d_in,
                                                     double* d_out, void* stream) {
  try {
    if (n < 1 || n > NOALLOC_MAX_SITES)
      fail(CPPE_GPU_INVALID_ARG, "cppe_gpu_bmatrix_apply_direct_noalloc: n must be in [1, " +
                                       std::to_string(NOALLOC_MAX_SITES) + "], got " +
                                       std::to_string(n));
    if (!d_xyz || !d_alpha6 || !d_in || !d_out)
      fail(CPPE_GPU_INVALID_ARG, "cppe_gpu_bmatrix_apply_direct_noalloc: null buffer");
    if ((d_excl_ptr == nullptr) != (d_excl_idx == nullptr))
      fail(CPPE_GPU_INVALID_ARG, "exclusion pointer and index arrays go together");
    {
      // d_out is written while the other buffers are read by other threads
      const size_t v = 3 * (size_t)n * sizeof(double);
      if (overlaps(d_out, v, d_in, v) || overlaps(d_out, v, d_xyz, v) ||
          overlaps(d_out, v, d_alpha6, 2 * v) ||
          overlaps(d_out, v, d_excl_ptr, ((size_t)n + 1) * sizeof(int)))
        fail(CPPE_GPU_INVALID_ARG,
             "cppe_gpu_bmatrix_apply_direct_noalloc: d_out overlaps an input buffer");
    }
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    double* scratch = noalloc_scratch(dev);
    double* pos4    = scratch;
    double* part    = scratch + (size_t)NOALLOC_MAX_SITES * 4;
    cudaStream_t s  = static_cast<cudaStream_t>(stream);
    const int nsplit = std::max(1, std::min(NOALLOC_SPLITS, (n + 1023) / 1024));
    k_noalloc_pack<<<(n + 127) / 128, 128, 0, s>>>(n, d_xyz, d_alpha6, damp, pos4);
    CG_LAUNCH();
    dim3 grid((n + NOALLOC_BLOCK - 1) / NOALLOC_BLOCK, nsplit);
    k_noalloc_pairs<<<grid, NOALLOC_BLOCK, 0, s>>>(n, pos4, d_in, d_excl_ptr, d_excl_idx, damp,
                                                   damping_factor, part);
    CG_LAUNCH();
    k_noalloc_finish<<<(n + 127) / 128, 128, 0, s>>>(n, nsplit, part, d_in, d_alpha6, d_out);
    CG_LAUNCH();
    return CPPE_GPU_OK;
  } catch (const Failure& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return CPPE_GPU_INVALID_ARG;
  }
}
