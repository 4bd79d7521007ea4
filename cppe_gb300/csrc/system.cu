// Solvers of one system: the reference's Jacobi-preconditioned CG in FP64
// (InducedMoments::compute, src/core/electric_fields.cc:191-239) and the
// mixed-precision form (FP32 inner PCG, FP64 residual and refinement).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <numeric>
#include <tuple>

#include "system.h"

namespace cg {

constexpr int VB = 256;  // threads per block of the vector kernels

// ---------------------------------------------------------------------------
// Vector kernels: thread per site; 3x3 symmetric blocks as 6 upper values.
// Scalars live in device memory so a whole iteration can run without the host.
// ---------------------------------------------------------------------------
template <typename A, typename B>
__device__ __forceinline__ void sym3(const A* a, const B* v, B* o) {
  o[0] = (B)(a[0] * v[0] + a[1] * v[1] + a[2] * v[2]);
  o[1] = (B)(a[1] * v[0] + a[3] * v[1] + a[4] * v[2]);
  o[2] = (B)(a[2] * v[0] + a[4] * v[1] + a[5] * v[2]);
}

// r = F - Ax (Ax may be null: zero start), z = alpha r, p = z; rz, rr.
// z4 (may be null): z again as one float4 per site, for the gathers of the
// learned preconditioner.
template <typename T>
__global__ void k_cg_start(int n, const double* __restrict__ F, const T* __restrict__ Ax,
                           const T* __restrict__ a6, T* __restrict__ r, T* __restrict__ z,
                           T* __restrict__ p, ReduceSlots rs, double* scal, int* flags,
                           float4* __restrict__ z4 = nullptr, const int* skip = nullptr) {
  __shared__ double sh[64];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  T v[2] = {T(0), T(0)};  // (FP32 products for the FP32 solve: see block_sum)
  if (i < n) {
    T rv[3], zv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) rv[c] = (T)(F[3 * i + c] - (Ax ? (double)Ax[3 * i + c] : 0.0));
    sym3(a6 + 6 * (size_t)i, rv, zv);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      r[3 * i + c] = rv[c], z[3 * i + c] = zv[c], p[3 * i + c] = zv[c];
      v[0] += rv[c] * zv[c];
      v[1] += rv[c] * rv[c];
    }
    if (z4) z4[i] = make_float4((float)zv[0], (float)zv[1], (float)zv[2], 0.f);
  }
  if (grid_sum_last<2>(v, sh, rs.partials, rs.ticket, rs.out)) {
    scal[S_RZ]    = rs.out[0];
    scal[S_RR]    = rs.out[1];
    scal[S_RNORM] = sqrt(rs.out[1]);
    flags[0]      = skip ? *skip : 0;
    flags[1]      = 0;
  }
}

// One CG update after Ap and p.Ap are known:
//   a = rz / pAp; x += a p; r -= a Ap; z = alpha r; beta = r'z' / rz.
// Sets flags[0] = 1 when ||r|| < thresh, 2 when the iteration limit is hit.
template <typename T>
__global__ void k_cg_update(int n, const T* __restrict__ p, const T* __restrict__ Ap,
                            const T* __restrict__ a6, T* __restrict__ x, T* __restrict__ r,
                            T* __restrict__ z, ReduceSlots rs, double* scal, int* flags,
                            double* hist, double thresh, int maxiter, T* __restrict__ r_old,
                            float4* __restrict__ z4 = nullptr) {
  __shared__ double sh[64];
  if (flags[0]) return;
  const double a = scal[S_RZ] / scal[S_PAP];
  const T aT     = (T)a;
  const int i    = blockIdx.x * blockDim.x + threadIdx.x;
  T v[2]         = {T(0), T(0)};
  if (i < n) {
    T rv[3], zv[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const size_t k = 3 * (size_t)i + c;
      x[k] += aT * p[k];
      if (r_old) r_old[k] = r[k];
      rv[c] = r[k] - aT * Ap[k];
      r[k]  = rv[c];
    }
    sym3(a6 + 6 * (size_t)i, rv, zv);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      z[3 * (size_t)i + c] = zv[c];
      v[0] += rv[c] * rv[c];
      v[1] += rv[c] * zv[c];
    }
    if (z4) z4[i] = make_float4((float)zv[0], (float)zv[1], (float)zv[2], 0.f);
  }
  if (grid_sum_last<2>(v, sh, rs.partials, rs.ticket, rs.out)) {
    const double rn = sqrt(rs.out[0]);
    const int it    = flags[1];
    if (hist) hist[it] = rn;
    flags[1]      = it + 1;
    scal[S_RNORM] = rn;
    scal[S_RZOLD] = scal[S_RZ];
    scal[S_BETA]  = rs.out[1] / scal[S_RZ];
    scal[S_RZ]    = rs.out[1];
    if (rn < (thresh < 0.0 ? scal[S_TOL] : thresh))
      flags[0] = 1;
    else if (it + 1 >= maxiter)
      flags[0] = 2;
  }
}

template <typename T>
__global__ void k_cg_dir(int n3, const T* __restrict__ z, T* __restrict__ p,
                         const double* scal, const int* flags) {
  if (flags[0]) return;
  const T b   = (T)scal[S_BETA];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) p[k] = z[k] + b * p[k];
}

// r = F - Ax in FP64; ||r||.
__global__ void k_residual(int n3, const double* __restrict__ F, const double* __restrict__ Ax,
                           double* __restrict__ r, ReduceSlots rs, double* scal) {
  __shared__ double sh[32];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (k < n3) {
    const double d = F[k] - (Ax ? Ax[k] : 0.0);
    r[k]           = d;
    v[0]           = d * d;
  }
  if (grid_sum_last<1>(v, sh, rs.partials, rs.ticket, rs.out)) scal[S_RNORM] = sqrt(rs.out[0]);
}

// r -= Bd (FP64 -= FP32); ||r||.
__global__ void k_residual_update(int n3, const float* __restrict__ Bd, double* __restrict__ r,
                                  ReduceSlots rs, double* scal) {
  __shared__ double sh[32];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (k < n3) {
    const double d = r[k] - (double)Bd[k];
    r[k]           = d;
    v[0]           = d * d;
  }
  if (grid_sum_last<1>(v, sh, rs.partials, rs.ticket, rs.out)) scal[S_RNORM] = sqrt(rs.out[0]);
}

// r = (r - fl(r)) + r32: the FP64 residual after an inner solve whose
// right-hand side was fl(r) (r rounded to FP32), from the inner solve's own
// final residual r32; ||r||.
__global__ void k_residual_inner(int n3, const float* __restrict__ r32, double* __restrict__ r,
                                 ReduceSlots rs, double* scal) {
  __shared__ double sh[32];
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  double v[1] = {0.0};
  if (k < n3) {
    const double d = (r[k] - (double)(float)r[k]) + (double)r32[k];
    r[k]           = d;
    v[0]           = d * d;
  }
  if (grid_sum_last<1>(v, sh, rs.partials, rs.ticket, rs.out)) scal[S_RNORM] = sqrt(rs.out[0]);
}

// x += d (FP64 += FP32); d is then cleared.
__global__ void k_accumulate(int n3, double* __restrict__ x, float* __restrict__ d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) {
    x[k] += (double)d[k];
    d[k] = 0.f;
  }
}

__global__ void k_to_f32(int n3, const double* __restrict__ a, float* __restrict__ b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) b[k] = (float)a[k];
}

__global__ void k_to_f64(int n3, const float* __restrict__ a, double* __restrict__ b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) b[k] = (double)a[k];
}

__global__ void k_sym_apply(int n, const double* __restrict__ a6, const double* __restrict__ in,
                            double* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) sym3(a6 + 6 * (size_t)i, in + 3 * (size_t)i, out + 3 * (size_t)i);
}

// ---------------------------------------------------------------------------
// System
// ---------------------------------------------------------------------------
System::~System() {
  if (stream) {
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    for (auto& row : inner_exec)
      for (auto& e : row)
        if (e) cudaGraphExecDestroy(e);
    if (side.s) cudaStreamSynchronize(side.s);
    side.destroy();
    cudaStreamDestroy(stream);
  }
  if (h_flags) cudaFreeHost(h_flags);
  if (h_scal) cudaFreeHost(h_scal);
}

static void inv_sym3(const double* s, double* o6) {
  const double a = s[0], b = s[1], c = s[2], d = s[3], e = s[4], f = s[5];
  const double A = d * f - e * e, B = c * e - b * f, C = b * e - c * d;
  const double det = a * A + b * B + c * C;
  const double id  = 1.0 / det;
  o6[0] = A * id;
  o6[1] = B * id;
  o6[2] = C * id;
  o6[3] = (a * f - c * c) * id;
  o6[4] = (b * c - a * e) * id;
  o6[5] = (a * d - b * b) * id;
}

void System::init(int n_, const double* xyz, const double* alpha6, const int* excl_ptr,
                  const int* excl_idx, const cppe_gpu_options& o) {
  n   = n_;
  opt = o;
  if (n <= 0) fail(CPPE_GPU_INVALID_ARG, "system has no polarizable sites");
  if (!xyz || !alpha6) fail(CPPE_GPU_INVALID_ARG, "xyz and alpha6 are required");
  const bool fmm = o.summation == CPPE_GPU_FMM;
  if (fmm && (o.tree_expansion_order < 2 || o.tree_expansion_order > 7))
    fail(CPPE_GPU_INVALID_ARG,
         "tree_expansion_order must be in [2, 7] for induced dipoles (the reference "
         "silently skips unsupported orders)");
  if (fmm && o.tree_ncrit < 1) fail(CPPE_GPU_INVALID_ARG, "tree_ncrit must be >= 1");
  if (o.maxiter < 0) fail(CPPE_GPU_INVALID_ARG, "maxiter must be >= 0");
  int ndev = 0;
  CG_CUDA(cudaGetDeviceCount(&ndev));
  if (o.device < 0 || o.device >= ndev) fail(CPPE_GPU_INVALID_ARG, "bad CUDA device ordinal");
  device = o.device;
  CG_CUDA(cudaSetDevice(device));
  CG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  side.create();

  // Coincident sites make the pair kernels singular (and the reference's tree
  // build recurse without end): reject them up front.
  {
    std::vector<int> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    auto key = [&](int i) { return std::make_tuple(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]); };
    std::sort(idx.begin(), idx.end(), [&](int a, int b) { return key(a) < key(b); });
    for (int k = 1; k < n; ++k)
      if (key(idx[k]) == key(idx[k - 1]))
        fail(CPPE_GPU_INVALID_ARG, "sites " + std::to_string(idx[k - 1]) + " and " +
                                         std::to_string(idx[k]) + " coincide");
  }
  if (excl_ptr) {
    excl_ptr_h.assign(excl_ptr, excl_ptr + n + 1);
    excl_idx_h.assign(excl_idx, excl_idx + excl_ptr[n]);
  }
  std::vector<double> sd(n, 0.0), ainv(6 * (size_t)n), al(6 * (size_t)n);
  for (int i = 0; i < n; ++i) {
    const double* a = alpha6 + 6 * (size_t)i;
    const double iso = (a[0] + a[3] + a[5]) / 3.0;
    if (o.damp && iso > 0.0) sd[i] = std::pow(iso, -1.0 / 6.0);
  }
  geo.damping = o.damp ? o.damping_factor : 0.0;
  geo.build(n, xyz, sd.data(), excl_ptr, excl_idx, fmm, o.tree_ncrit, o.theta, stream);
  if (fmm) {
    ops = std::make_unique<DeviceOps>();
    ops->build(1, o.tree_expansion_order, stream);
  }
  for (int k = 0; k < n; ++k) {
    const double* a = alpha6 + 6 * (size_t)geo.layout.perm[k];
    inv_sym3(a, &ainv[6 * (size_t)k]);
    std::copy(a, a + 6, &al[6 * (size_t)k]);
  }
  std::vector<float> ainvf(ainv.begin(), ainv.end()), alf(al.begin(), al.end());
  ainv64.upload(ainv, stream);
  alpha64.upload(al, stream);
  ainv32.upload(ainvf, stream);
  alpha32.upload(alf, stream);
  const size_t n3 = 3 * (size_t)n;
  for (auto* b : {&F, &x, &r, &z, &p, &Ap, &tmp_in, &tmp_out}) b->alloc(n3);
  for (auto* b : {&r32, &z32, &p32, &Ap32, &d32}) b->alloc(n3);
  scal.alloc(S_NSCAL);
  scal.zero(stream);
  // partial sums of the grid reductions: the widest grid is the learned
  // preconditioner's (eight lanes per site, 128-thread blocks, two sums)
  const size_t maxblocks = std::max<size_t>(1024, (8 * (size_t)n + 127) / 128 + 1);
  partials.alloc(4 * maxblocks);
  hist.alloc(std::max(1, o.maxiter) + 64);
  ticket.alloc(1);
  ticket.zero(stream);
  flags.alloc(4);
  flags.zero(stream);
  CG_CUDA(cudaMallocHost(&h_flags, 8 * sizeof(int)));  // [4]: the model's error code
  CG_CUDA(cudaMallocHost(&h_scal, S_NSCAL * sizeof(double)));
  CG_CUDA(cudaStreamSynchronize(stream));
  setup_inexact(xyz, sd.data());
}

// Opening angles of the inexact inner operators.  At 30,000 water sites
// (FP32 apply 0.212 ms with the operator's 0.5): 0.6 moves 42 % of the
// near-field pairs into M2L (0.146 ms) and differs from the operator by
// 2e-4 - 3e-4 relative; 0.8 moves 75 % (0.089 ms) at 1.2e-3 - 1.9e-3.
constexpr double INEXACT_THETA[System::NINEXACT] = {0.6, 0.8};

void System::setup_inexact(const double* xyz, const double* sd) {
  n_inexact = 0;
  if (!geo.fmm || opt.precision != CPPE_GPU_MIXED) return;
  const size_t n3 = 3 * (size_t)n;
  // a random vector and a smooth one (the response of every site to one
  // uniform field), and the operator on them in FP64 accuracy
  std::vector<double> vin[2] = {std::vector<double>(n3), std::vector<double>(n3)};
  std::vector<double> a64[2] = {std::vector<double>(n3), std::vector<double>(n3)};
  unsigned long long st = 0x9e3779b97f4a7c15ull;
  for (size_t k = 0; k < n3; ++k) {
    st ^= st << 13, st ^= st >> 7, st ^= st << 17;
    vin[0][k] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    vin[1][k] = (k % 3 == 0) ? 1.0 : (k % 3 == 1 ? 0.5 : 0.25);
  }
  for (int trial = 0; trial < 2; ++trial) {
    CG_CUDA(cudaMemcpyAsync(tmp_in.p, vin[trial].data(), n3 * sizeof(double),
                            cudaMemcpyHostToDevice, stream));
    apply64(tmp_in.p, tmp_out.p, false, NEAR_DD);
    CG_CUDA(cudaMemcpyAsync(a64[trial].data(), tmp_out.p, n3 * sizeof(double),
                            cudaMemcpyDeviceToHost, stream));
    CG_CUDA(cudaStreamSynchronize(stream));
  }
  for (int lev = 0; lev < NINEXACT; ++lev) {
    if (opt.theta >= INEXACT_THETA[lev]) break;
    Geometry& gx = geo_x[lev];
    gx.damping   = geo.damping;
    gx.build(n, xyz, sd, excl_ptr_h.empty() ? nullptr : excl_ptr_h.data(),
             excl_idx_h.empty() ? nullptr : excl_idx_h.data(), true, opt.tree_ncrit,
             INEXACT_THETA[lev], stream);
    // the opening angle changes the lists, not the tree: same site order
    if (gx.layout.perm != geo.layout.perm) break;
    double worst = 0.0;
    std::vector<double> out(n3);
    for (int trial = 0; trial < 2; ++trial) {
      CG_CUDA(cudaMemcpyAsync(tmp_in.p, vin[trial].data(), n3 * sizeof(double),
                              cudaMemcpyHostToDevice, stream));
      apply_level = lev;
      n_inexact   = lev + 1;
      apply32_widen(tmp_in.p, tmp_out.p);
      apply_level = -1;
      n_inexact   = lev;
      CG_CUDA(cudaMemcpyAsync(out.data(), tmp_out.p, n3 * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
      CG_CUDA(cudaStreamSynchronize(stream));
      double num = 0.0, den = 0.0;
      for (size_t k = 0; k < n3; ++k) {
        const double d = out[k] - a64[trial][k];
        num += d * d, den += a64[trial][k] * a64[trial][k];
      }
      if (den > 0.0) worst = std::max(worst, std::sqrt(num / den));
    }
    inexact_delta[lev] = 3.0 * worst;
    if (!(worst > 0.0 && inexact_delta[lev] < 1e-2)) break;
    n_inexact = lev + 1;
  }
}

void System::apply32_widen(const double* in, double* out) {
  const int n3 = 3 * n;
  k_to_f32<<<(n3 + VB - 1) / VB, VB, 0, stream>>>(n3, in, p32.p);
  CG_LAUNCH();
  apply32(p32.p, Ap32.p, false);
  k_to_f64<<<(n3 + VB - 1) / VB, VB, 0, stream>>>(n3, Ap32.p, out);
  CG_LAUNCH();
}

void System::phase_timings(int precision, int reps, double* ms) {
  CG_CUDA(cudaSetDevice(device));
  PhaseEvents pe;
  for (auto& e : pe.ev) CG_CUDA(cudaEventCreate(&e));
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const int n3 = 3 * n;
  k_to_f32<<<(n3 + VB - 1) / VB, VB, 0, stream>>>(n3, tmp_in.p, p32.p);
  CG_LAUNCH();
  for (int r = 0; r < reps; ++r) {
    if (precision == CPPE_GPU_MIXED) {
      ReduceSlots rs = slots(S_PAP);
      eval_field<float>(geo, ops.get(), w32, 1, p32.p, opt.damp != 0, opt.damping_factor,
                        FINISH_APPLY, ainv32.p, Ap32.p, nullptr, 1.0, &rs, stream, &pe);
    } else {
      ReduceSlots rs = slots(S_PAP);
      eval_field<double>(geo, ops.get(), w64, 1, tmp_in.p, opt.damp != 0, opt.damping_factor,
                         FINISH_APPLY, ainv64.p, tmp_out.p, nullptr, 1.0, &rs, stream, &pe,
                         precision == 2 ? NEAR_DD : NEAR_FP64);
    }
    CG_CUDA(cudaEventSynchronize(pe.ev[5]));
    float t;
    const int from[6] = {3, 0, 1, 2, 4, 0}, to[6] = {4, 1, 2, 3, 5, 5};
    for (int k = 0; k < 6; ++k) {
      CG_CUDA(cudaEventElapsedTime(&t, pe.ev[from[k]], pe.ev[to[k]]));
      acc[k] += t;
    }
  }
  for (auto& e : pe.ev) cudaEventDestroy(e);
  for (int k = 0; k < 6; ++k) ms[k] = acc[k] / std::max(1, reps);
}

double autotune_schedule(Geometry& geo, SideStream& side, cudaStream_t stream, int reps,
                         const std::function<void()>& apply) {
  reps = std::max(1, reps);
  // the built-in work-item size, for the candidates around it
  long total = 0;
  const TreeLayout& L = geo.layout;
  for (int a = 0; a < L.nleaves; ++a)
    for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q)
      total += (long)(L.leaf_start[a + 1] - L.leaf_start[a]) *
               (L.leaf_start[L.p2p_src[q] + 1] - L.leaf_start[L.p2p_src[q]]);
  const long w0 = std::max<long>(8192, total / (32L * 152));
  const long ws[3]  = {std::max<long>(4096, w0 / 2), w0, 2 * w0};
  const int chs[3]  = {32, 64, 128};
  const int nch     = geo.fmm ? 3 : 1;
  cudaEvent_t e0, e1;
  CG_CUDA(cudaEventCreate(&e0));
  CG_CUDA(cudaEventCreate(&e1));
  auto time_applies = [&]() {
    apply();  // warm-up (sizes the work buffers)
    CG_CUDA(cudaEventRecord(e0, stream));
    for (int r = 0; r < reps; ++r) apply();
    CG_CUDA(cudaEventRecord(e1, stream));
    CG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    return (double)ms / reps;
  };
  double best = 1e300;
  long best_w = w0;
  int best_c  = 64;
  bool best_s = geo.sym_enabled;
  int best_k  = geo.sym_pack;
  int best_t  = geo.multi_tile, best_r = geo.multi_copies;
  // symmetric near field (single systems; two or four sources a lane) or
  // per-target items; for a batch whose snapshots repeat per right-hand
  // side, the multi-RHS tile size and the right-hand sides per pass
  const int nsym = (geo.h_leaf_seg.empty() && geo.ncopies == 1) ? 3 : 1;
  const int tiles[3] = {96, 120, 144};
  const int ntile    = geo.ncopies > 1 ? 3 : 1;
  const int nrc      = geo.ncopies > 4 ? 2 : 1;
  for (int ri = 0; ri < nrc; ++ri)
    for (int ti = 0; ti < ntile; ++ti)
      for (int si = 0; si < nsym; ++si)
        for (long w : ws)
          for (int ci = 0; ci < nch; ++ci) {
            geo.sym_enabled  = nsym == 3 ? si < 2 : geo.sym_enabled;
            geo.sym_pack     = nsym == 3 ? (si == 1 ? 2 : 1) : geo.sym_pack;
            geo.multi_tile   = ntile == 3 ? tiles[ti] : geo.multi_tile;
            geo.multi_copies = nrc == 2 ? (ri == 0 ? 8 : 4) : geo.multi_copies;
            geo.item_pairs   = w;
            geo.m2l_chunk    = chs[ci];
            geo.make_schedules();
            geo.upload_schedules(stream);
            const double ms = time_applies();
            if (ms < best)
              best = ms, best_w = w, best_c = chs[ci], best_s = geo.sym_enabled,
              best_k = geo.sym_pack, best_t = geo.multi_tile, best_r = geo.multi_copies;
          }
  geo.sym_enabled  = best_s;
  geo.sym_pack     = best_k;
  geo.multi_tile   = best_t;
  geo.multi_copies = best_r;
  geo.item_pairs  = best_w;
  geo.m2l_chunk   = best_c;
  geo.make_schedules();
  geo.upload_schedules(stream);
  // priority of the far-field stream under the chosen schedule
  if (geo.fmm) {
    double t_side[2] = {0.0, 0.0};  // high, default priority
    for (int k = 0; k < 2; ++k) {
      side.use_high_priority(k == 0);
      t_side[k] = time_applies();
    }
    side.use_high_priority(t_side[0] <= t_side[1]);
    best = std::min(t_side[0], t_side[1]);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CG_CUDA(cudaStreamSynchronize(stream));
  return best;
}

double System::autotune(int reps) {
  CG_CUDA(cudaSetDevice(device));
  CG_CUDA(cudaMemsetAsync(p32.p, 0, sizeof(float) * 3 * (size_t)n, stream));
  const double best =
        autotune_schedule(geo, side, stream, reps, [&] { apply32(p32.p, Ap32.p, false); });
  // the inexact operators' lists share the leaves: the same near-field form
  for (int k = 0; k < n_inexact; ++k)
    if (geo_x[k].sym_enabled != geo.sym_enabled || geo_x[k].sym_pack != geo.sym_pack) {
      geo_x[k].sym_enabled = geo.sym_enabled;
      geo_x[k].sym_pack    = geo.sym_pack;
      geo_x[k].make_schedules();
      geo_x[k].upload_schedules(stream);
    }
  // captured inner loops hold the old schedule's buffers: rebuild on next use
  for (auto& row : inner_exec)
    for (auto& e : row)
      if (e) cudaGraphExecDestroy(e), e = nullptr;
  size_work_buffers();
  return best;
}

// One FP32 apply with each operator (outside any capture), which gives the
// work buffers the sizes of the current schedules before the inner loops are
// captured again.
void System::size_work_buffers() {
  for (int lev = -1; lev < n_inexact; ++lev) {
    apply_level = lev;
    try {
      apply32(p32.p, Ap32.p, false);
    } catch (...) {
      apply_level = -1;
      throw;
    }
  }
  apply_level = -1;
  CG_CUDA(cudaStreamSynchronize(stream));
}

void System::set_schedule(int near_form, long item_pairs, int m2l_chunk) {
  CG_CUDA(cudaSetDevice(device));
  auto set = [&](Geometry& g) {
    if (near_form >= 0) g.sym_enabled = near_form > 0, g.sym_pack = near_form > 0 ? near_form : 1;
    if (item_pairs > 0) g.item_pairs = item_pairs;
    if (m2l_chunk > 0) g.m2l_chunk = m2l_chunk;
    g.make_schedules();
    g.upload_schedules(stream);
  };
  set(geo);
  for (int k = 0; k < n_inexact; ++k) set(geo_x[k]);
  for (auto& row : inner_exec)
    for (auto& e : row)
      if (e) cudaGraphExecDestroy(e), e = nullptr;
  size_work_buffers();
}

ReduceSlots System::slots(int k) const { return ReduceSlots{partials.p, ticket.p, scal.p + k}; }

void System::apply64(const double* in, double* out, bool with_dot, int near_mode) {
  ReduceSlots rs = slots(S_PAP);
  eval_field<double>(geo, ops.get(), w64, 1, in, opt.damp != 0, opt.damping_factor,
                     FINISH_APPLY, ainv64.p, out, nullptr, 1.0, with_dot ? &rs : nullptr,
                     stream, nullptr, near_mode, &side);
}

void System::apply32(const float* in, float* out, bool with_dot) {
  ReduceSlots rs = slots(S_PAP);
  const bool inexact = apply_level >= 0 && apply_level < n_inexact;
  eval_field<float>(inexact ? geo_x[apply_level] : geo, ops.get(),
                    inexact ? w32x[apply_level] : w32, 1, in,
                    opt.damp != 0, opt.damping_factor, FINISH_APPLY, ainv32.p, out, nullptr, 1.0,
                    with_dot ? &rs : nullptr, stream, nullptr, NEAR_FP64, &side);
}

namespace {
// Host side of a device-resident loop: after each iteration the done flag is
// copied to pinned memory and the previous iteration's copy is inspected, so
// the GPU always has the next iteration queued.
struct Poller {
  cudaStream_t s;
  int* d_flags;
  int* h_flags;
  cudaEvent_t ev[2];
  int k = 0;
  Poller(cudaStream_t s_, int* d, int* h) : s(s_), d_flags(d), h_flags(h) {
    CG_CUDA(cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming));
    CG_CUDA(cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming));
  }
  ~Poller() {
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
  }
  // Returns true once a finished state has been observed.
  bool after_iteration() {
    CG_CUDA(cudaMemcpyAsync(h_flags, d_flags, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaEventRecord(ev[k & 1], s));
    bool done = false;
    if (k > 0) {
      CG_CUDA(cudaEventSynchronize(ev[(k - 1) & 1]));
      done = ((volatile int*)h_flags)[0] != 0;
    }
    ++k;
    return done;
  }
};
}  // namespace

int System::solve_fp64(bool zero_guess, double* hist_out, int hist_cap, int* iters) {
  const int nb   = (n + VB - 1) / VB;
  const int n3   = 3 * n;
  const double t = opt.induced_thresh;
  last           = SolveStats();
  if (!zero_guess) {
    apply64(x.p, Ap.p, false);
    last.fp64_applies++;
  }
  k_cg_start<double><<<nb, VB, 0, stream>>>(n, F.p, zero_guess ? nullptr : Ap.p, alpha64.p,
                                            r.p, z.p, p.p, slots(S_RED), scal.p, flags.p);
  CG_LAUNCH();
  if (use_model) learned_precond<double>(z.p, r.p, p.p, true);
  if (zero_guess) CG_CUDA(cudaMemsetAsync(x.p, 0, sizeof(double) * n3, stream));
  Poller poll(stream, flags.p, h_flags);
  for (int k = 0; k < opt.maxiter; ++k) {
    apply64(p.p, Ap.p, true);
    last.fp64_applies++;
    k_cg_update<double><<<nb, VB, 0, stream>>>(n, p.p, Ap.p, alpha64.p, x.p, r.p, z.p,
                                               slots(S_RED), scal.p, flags.p, hist.p, t,
                                               opt.maxiter, use_model ? lf_rold64.p : nullptr);
    CG_LAUNCH();
    const double* zd = use_model ? learned_precond<double>(z.p, r.p, p.p, false) : z.p;
    k_cg_dir<double><<<(n3 + VB - 1) / VB, VB, 0, stream>>>(n3, zd, p.p, scal.p, flags.p);
    CG_LAUNCH();
    if (poll.after_iteration()) break;
  }
  CG_CUDA(cudaMemcpyAsync(h_flags, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
  CG_CUDA(cudaMemcpyAsync(h_scal, scal.p, S_NSCAL * sizeof(double), cudaMemcpyDeviceToHost,
                          stream));
  CG_CUDA(cudaStreamSynchronize(stream));
  const int it = h_flags[1];
  // applies queued after convergence did no work on x
  last.fp64_applies = std::min(last.fp64_applies, it + (zero_guess ? 0 : 1));
  last.iterations   = it;
  last.final_rnorm  = h_scal[S_RNORM];
  if (iters) *iters = it;
  if (hist_out && hist_cap > 0 && it > 0)
    CG_CUDA(cudaMemcpy(hist_out, hist.p, sizeof(double) * std::min(it, hist_cap),
                       cudaMemcpyDeviceToHost));
  return h_flags[0] == 1 ? CPPE_GPU_OK : CPPE_GPU_NOT_CONVERGED;
}

// Set-up of an inner FP32 solve on the device (no host round trip): its
// threshold max(eta ||r||, 0.5 t) from the residual norm in scal[S_RNORM],
// which is also kept (S_RSTAGE); the iterations of the previous inner solve
// are added to flags[3] (stage 0 clears it); flags[2] = 1 when the residual
// already meets t, which makes the following k_cg_start start a finished solve.
// With inexact operators (delta1, delta2 > 0; 0: absent) the solve runs with
// the operator down to S_TOL = max(final threshold, S_SW1), then with
// inexact operator 1 down to max(final, S_SW2), then with operator 2 down to
// the final threshold S_TOLF.  Hand-over points: where each inexact
// operator's effect on the residual, ~delta ||r||, stays below 0.6 of the
// first stage's target eta ||r0|| (the double-float residual that follows
// is exact; the inner solve's true residual then stays below 1.6 eta ||r0||),
// or, for the last stage, where 1.5 delta ||r|| stays below 0.2 t (the
// residual is then formed from the recursion, which carries those
// differences).
__global__ void k_inner_stage(double* scal, int* flags, double t, double eta, int stage,
                              double delta1, double delta2) {
  const double rn  = scal[S_RNORM];
  const double tol = fmax(eta * rn, 0.5 * t);
  auto sw = [&](double d) {
    if (d <= 0.0) return tol;
    return fmax(tol, stage == 0 ? 0.6 * eta * rn / d : 0.2 * t / (1.5 * d));
  };
  const double sw1 = delta1 > 0.0 ? sw(delta1) : tol;
  const double sw2 = delta2 > 0.0 ? fmin(sw1, sw(delta2)) : tol;
  scal[S_TOLF]   = tol;
  scal[S_SW1]    = sw1;
  scal[S_SW2]    = sw2;
  scal[S_TOL]    = sw1;
  scal[S_RSTAGE] = rn;
  scal[S_RSW1] = scal[S_RSW2] = 0.0;
  flags[3]       = stage == 0 ? 0 : flags[3] + flags[1];
  flags[2]       = 0;
  // flags[2] = 1 makes the following k_cg_start start a finished solve
  if (stage > 0 && rn < t) {
    flags[2]     = 1;  // nothing left to do: no part runs
    scal[S_TOLF] = scal[S_SW1] = scal[S_SW2] = 1e300;
  } else if (stage > 0 && rn < scal[S_TOL]) {
    flags[2] = 1;  // the operator's part has nothing to do
  }
}

// Hand-over to inexact operator `level` (0, 1) inside an inner solve: the
// solve continues (same direction and scalars) unless it has reached the
// next part's threshold or the iteration limit.  flags[0] = 0 lets the
// stopping iteration's skipped direction update run first; 3 (no iteration
// ran yet) skips it, and k_inner_resume then clears it.
__global__ void k_inner_switch(double* scal, int* flags, int level, int last) {
  const double rn  = scal[S_RNORM];
  const double nxt = last ? scal[S_TOLF] : scal[S_SW2];
  scal[level == 0 ? S_RSW1 : S_RSW2] = rn;
  scal[S_TOL]                        = nxt;
  if (flags[0] == 1 && rn >= nxt) flags[0] = flags[1] > 0 ? 0 : 3;
}
__global__ void k_inner_resume(int* flags) {
  if (flags[0] == 3) flags[0] = 0;
}

// Continues the inner graph's while loop until the solve has stopped.
__global__ void k_while_running(cudaGraphConditionalHandle h, const int* flags) {
  cudaGraphSetConditional(h, flags[0] == 0 ? 1u : 0u);
}

// One inner FP32 PCG iteration (apply with p.Ap, update, optional learned
// correction, new direction); every kernel is a no-op once flags[0] is set.
void System::inner_iteration_fp32(int nb, int nb3) {
  apply32(p32.p, Ap32.p, true);
  k_cg_update<float><<<nb, VB, 0, stream>>>(n, p32.p, Ap32.p, alpha32.p, d32.p, r32.p, z32.p,
                                            slots(S_RED), scal.p, flags.p, nullptr, -1.0,
                                            std::max(1, opt.maxiter),
                                            use_model ? lf_rold32.p : nullptr,
                                            use_model ? lf_z4.p : nullptr);
  CG_LAUNCH();
  const float* zd = use_model ? learned_precond<float>(z32.p, r32.p, p32.p, false) : z32.p;
  k_cg_dir<float><<<nb3, VB, 0, stream>>>(3 * n, zd, p32.p, scal.p, flags.p);
  CG_LAUNCH();
}

// The inner loop as a CUDA graph with a conditional while node: the body is
// one iteration captured from the stream (including the far-field side
// stream's fork and join), repeated on the device until k_cg_update sets
// flags[0] (converged, or the iteration limit); a kernel ahead of the loop
// sets its condition, so a solve that is already finished runs no
// iteration.  Built once per system and learned/plain variant and operator,
// after the buffers it uses exist.  Where graph construction is refused, the
// iterations are launched from the host.
bool System::inner_graph_ready(int nb, int nb3, int level) {
  const int v = use_model ? 1 : 0;
  const int l = level >= 0 && level < n_inexact ? level + 1 : 0;
  // CPPE_GPU_GRAPHS=0 launches the iterations from the host instead (same
  // kernels; for profilers that do not descend into conditional graph nodes)
  static const bool graphs = [] {
    const char* e = std::getenv("CPPE_GPU_GRAPHS");
    return !(e && e[0] == '0');
  }();
  if (!graphs) inner_graph_failed = true;
  if (!inner_exec[v][l] && !inner_graph_failed) {
    cudaGraph_t g = nullptr;
    bool ok       = cudaGraphCreate(&g, 0) == cudaSuccess;
    cudaGraphConditionalHandle h{};
    cudaGraphNode_t node{};
    cudaGraphNodeParams np{};
    ok = ok && cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) ==
                     cudaSuccess;
    // the kernel that sets the loop's first condition, captured into g
    cudaGraphNode_t pre{};
    if (ok) {
      ok = cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        k_while_running<<<1, 1, 0, stream>>>(h, flags.p);
        ok = cudaGetLastError() == cudaSuccess;
        cudaGraph_t captured = nullptr;
        ok = (cudaStreamEndCapture(stream, &captured) == cudaSuccess) && ok;
      }
      size_t nn = 1;
      ok = ok && cudaGraphGetNodes(g, &pre, &nn) == cudaSuccess && nn == 1;
    }
    if (ok) {
      np.type                 = cudaGraphNodeTypeConditional;
      np.conditional.handle   = h;
      np.conditional.type     = cudaGraphCondTypeWhile;
      np.conditional.size     = 1;
      ok = cudaGraphAddNode(&node, g, &pre, nullptr, 1, &np) == cudaSuccess;
    }
    if (ok) {
      cudaGraph_t body = np.conditional.phGraph_out[0];
      ok = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        const long long c0 = launch_counter();
        apply_level        = l - 1;
        try {
          CaptureScope cs;
          inner_iteration_fp32(nb, nb3);
          k_while_running<<<1, 1, 0, stream>>>(h, flags.p);
          CG_LAUNCH();
        } catch (const Failure&) {
          ok = false;
        }
        apply_level = -1;
        inner_body_launches[v][l] = launch_counter() - c0;
        launch_counter()       = c0;
        cudaGraph_t captured   = nullptr;
        ok = (cudaStreamEndCapture(stream, &captured) == cudaSuccess) && ok;
      }
    }
    if (ok) ok = cudaGraphInstantiate(&inner_exec[v][l], g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      cudaGetLastError();  // clear the refusal; fall back to host-launched iterations
      if (inner_exec[v][l]) cudaGraphExecDestroy(inner_exec[v][l]);
      inner_exec[v][l]   = nullptr;
      inner_graph_failed = true;
    }
  }
  return inner_exec[v][l] != nullptr;
}

void System::run_inner_fp32(int nb, int nb3) {
  const int v = use_model ? 1 : 0;
  if (inner_graph_ready(nb, nb3)) {
    CG_CUDA(cudaGraphLaunch(inner_exec[v][0], stream));
    CG_CUDA(cudaMemcpyAsync(h_flags, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CG_CUDA(cudaStreamSynchronize(stream));
    launch_counter() += inner_body_launches[v][0] * h_flags[1] + 1;
    return;
  }
  Poller poll(stream, flags.p, h_flags);
  for (int k = 0; k < std::max(1, opt.maxiter); ++k) {
    inner_iteration_fp32(nb, nb3);
    if (poll.after_iteration()) break;
  }
}

int System::solve_mixed(bool zero_guess, double* hist_out, int hist_cap, int* iters) {
  const int nb   = (n + VB - 1) / VB;
  const int n3   = 3 * n;
  const int nb3  = (n3 + VB - 1) / VB;
  const double t = opt.induced_thresh;
  const double eta = 3e-6;   // relative residual reduction asked of each FP32 inner solve
  const int max_outer = 12;
  last = SolveStats();
  std::vector<double> outer_hist;
  int total_inner = 0;
  CG_CUDA(cudaMemsetAsync(d32.p, 0, sizeof(float) * n3, stream));
  // First residual: FP32 operator on the start vector (the refinement below
  // removes its error), or the rhs itself for a zero start.
  if (zero_guess) {
    CG_CUDA(cudaMemsetAsync(x.p, 0, sizeof(double) * n3, stream));
    k_residual<<<nb3, VB, 0, stream>>>(n3, F.p, nullptr, r.p, slots(S_RED), scal.p);
    CG_LAUNCH();
  } else {
    k_to_f32<<<nb3, VB, 0, stream>>>(n3, x.p, p32.p);
    CG_LAUNCH();
    apply32(p32.p, Ap32.p, false);
    last.fp32_applies++;
    k_cg_start<float><<<nb, VB, 0, stream>>>(n, F.p, Ap32.p, alpha32.p, r32.p, z32.p, p32.p,
                                             slots(S_RED), scal.p, flags.p,
                                             use_model ? lf_z4.p : nullptr);
    CG_LAUNCH();
    if (use_model) learned_precond<float>(z32.p, r32.p, p32.p, true);
  }
  bool have_inner_start   = !zero_guess;
  bool have_fp64_residual = zero_guess;  // r = F is exact for a zero start
  int status              = CPPE_GPU_NOT_CONVERGED;
  // Bound of |computed - true| of the FP64 residual's norm where it was not
  // recomputed with the FP64 operator: after an inner solve started from a
  // residual of norm rs, forming the new residual from the FP32 recursion
  // errs by < REC_ERR rs (the recursion's rounding, ~1e-7 per update and
  // FP32 operator error ~1e-7 of ||B d|| ~ rs, times a condition-number
  // margin), an FP32 apply of the correction by < CORR_ERR rs.  A residual is
  // accepted when its norm plus the bound is below t; the cheaper forms are
  // used where their bound stays below t / 10.
  constexpr double REC_ERR = 3e-6, CORR_ERR = 3e-7;
  double rerr = 0.0;
  // The usual course -- FP32 solve, FP64 residual, FP32 solve, residual from
  // the recursion -- queued at once with the decisions on the device and one
  // host synchronisation; the loop below takes over where it does not end
  // the solve (or where the inner iterations cannot run as a graph).
  bool graphs_ok = !zero_guess && inner_graph_ready(nb, nb3);
  for (int lev = 0; lev < n_inexact && graphs_ok; ++lev) graphs_ok = inner_graph_ready(nb, nb3, lev);
  if (graphs_ok) {
    const int v      = use_model ? 1 : 0;
    const int nx     = n_inexact;
    const double d1  = nx > 0 ? inexact_delta[0] : 0.0;
    const double d2  = nx > 1 ? inexact_delta[1] : 0.0;
    // one inner solve: the operator's graph, then for each inexact operator
    // the hand-over and its graph
    auto inner = [&]() {
      CG_CUDA(cudaGraphLaunch(inner_exec[v][0], stream));
      for (int lev = 0; lev < nx; ++lev) {
        k_inner_switch<<<1, 1, 0, stream>>>(scal.p, flags.p, lev, lev + 1 == nx);
        CG_LAUNCH();
        // the direction update the stopping iteration skipped (no-ops if the
        // solve stays finished)
        const float* zd = use_model ? learned_precond<float>(z32.p, r32.p, p32.p, false) : z32.p;
        k_cg_dir<float><<<nb3, VB, 0, stream>>>(3 * n, zd, p32.p, scal.p, flags.p);
        CG_LAUNCH();
        k_inner_resume<<<1, 1, 0, stream>>>(flags.p);
        CG_LAUNCH();
        CG_CUDA(cudaGraphLaunch(inner_exec[v][lev + 1], stream));
      }
    };
    k_inner_stage<<<1, 1, 0, stream>>>(scal.p, flags.p, t, eta, 0, d1, d2);
    CG_LAUNCH();
    inner();
    k_accumulate<<<nb3, VB, 0, stream>>>(n3, x.p, d32.p);
    CG_LAUNCH();
    apply64(x.p, Ap.p, false, NEAR_DD);
    k_residual<<<nb3, VB, 0, stream>>>(n3, F.p, Ap.p, r.p, slots(S_RED), scal.p);
    CG_LAUNCH();
    k_inner_stage<<<1, 1, 0, stream>>>(scal.p, flags.p, t, eta, 1, d1, d2);
    CG_LAUNCH();
    k_cg_start<float><<<nb, VB, 0, stream>>>(n, r.p, nullptr, alpha32.p, r32.p, z32.p, p32.p,
                                             slots(S_RED), scal.p, flags.p,
                                             use_model ? lf_z4.p : nullptr, flags.p + 2);
    CG_LAUNCH();
    if (use_model) learned_precond<float>(z32.p, r32.p, p32.p, true);
    inner();
    k_residual_inner<<<nb3, VB, 0, stream>>>(n3, r32.p, r.p, slots(S_RED), scal.p);
    CG_LAUNCH();
    k_accumulate<<<nb3, VB, 0, stream>>>(n3, x.p, d32.p);
    CG_LAUNCH();
    CG_CUDA(cudaMemcpyAsync(h_flags, flags.p, 4 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CG_CUDA(cudaMemcpyAsync(h_scal, scal.p, S_NSCAL * sizeof(double), cudaMemcpyDeviceToHost,
                            stream));
    CG_CUDA(cudaStreamSynchronize(stream));
    const int it1 = h_flags[3], it2 = h_flags[1];
    total_inner += it1 + it2;
    last.fp32_applies += it1 + it2;
    last.fp64_applies++;
    launch_counter() += inner_body_launches[v][0] * (it1 + it2) + 2 + 8 * nx;
    const double r1 = h_scal[S_RSTAGE];  // FP64 residual after the first inner solve
    outer_hist.push_back(r1);
    have_fp64_residual = true;
    have_inner_start   = false;
    // the residual from the recursion stands where its error bound is below
    // t / 10 (the inexact operator adds ~1.5 delta ||r|| from the hand-over on)
    const double rsw1 = nx > 0 ? std::min(r1, h_scal[S_RSW1]) : 0.0;
    const double rsw2 = nx > 1 ? std::min(r1, h_scal[S_RSW2]) : 0.0;
    const double bound = REC_ERR * r1 + 1.5 * (d1 * rsw1 + d2 * rsw2);
    const bool recursion_ok = r1 < t || bound < 0.4 * t;
    if (recursion_ok && r1 >= t) rerr = bound;
    if (recursion_ok && h_scal[S_RNORM] + rerr < t) {
      if (r1 >= t) outer_hist.push_back(h_scal[S_RNORM]);
      status = CPPE_GPU_OK;
    } else if (!recursion_ok) {
      // recompute the residual of the accumulated x with the FP64 operator
      apply64(x.p, Ap.p, false, NEAR_DD);
      last.fp64_applies++;
      k_residual<<<nb3, VB, 0, stream>>>(n3, F.p, Ap.p, r.p, slots(S_RED), scal.p);
      CG_LAUNCH();
    }
  }
  for (int outer = (int)outer_hist.size(); outer < max_outer && status != CPPE_GPU_OK; ++outer) {
    double rnorm;
    if (!have_inner_start) {
      // r holds the FP64 residual; read its norm and set up the inner solve.
      CG_CUDA(cudaMemcpyAsync(h_scal, scal.p, S_NSCAL * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
      CG_CUDA(cudaStreamSynchronize(stream));
      rnorm = h_scal[S_RNORM];
      outer_hist.push_back(rnorm);
      if (rnorm + rerr < t) {
        status = CPPE_GPU_OK;
        break;
      }
      // inner right-hand side: the FP64 residual
      k_cg_start<float><<<nb, VB, 0, stream>>>(n, r.p, nullptr, alpha32.p, r32.p, z32.p,
                                               p32.p, slots(S_RED), scal.p, flags.p,
                                               use_model ? lf_z4.p : nullptr);
      CG_LAUNCH();
      if (use_model) learned_precond<float>(z32.p, r32.p, p32.p, true);
    } else {
      CG_CUDA(cudaMemcpyAsync(h_scal, scal.p, S_NSCAL * sizeof(double), cudaMemcpyDeviceToHost,
                              stream));
      CG_CUDA(cudaStreamSynchronize(stream));
      rnorm = h_scal[S_RNORM];
    }
    have_inner_start = false;
    // the last inner solve stops at half the threshold: the FP64 residual it
    // leaves differs from the FP32 recursion's by ~1e-7 of the correction
    // (far below the other half)
    const double tol = std::max(eta * rnorm, 0.5 * t);
    // the threshold of this inner solve goes to the device; the loop itself
    // runs as one graph launch (device-side while loop)
    h_scal[S_TOL] = tol;
    CG_CUDA(cudaMemcpyAsync(scal.p + S_TOL, h_scal + S_TOL, sizeof(double),
                            cudaMemcpyHostToDevice, stream));
    run_inner_fp32(nb, nb3);
    CG_CUDA(cudaMemcpyAsync(h_flags, flags.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CG_CUDA(cudaStreamSynchronize(stream));
    total_inner += h_flags[1];
    last.fp32_applies += h_flags[1];
    // After a residual r (exact or within rerr), the inner solve's
    // B d = fl(r) - r32 is known from its own recursion (bound REC_ERR ||r||);
    // where the bounds stay below t / 10 the residual is formed from r32
    // without another apply, else from an FP32 apply of d (CORR_ERR), else
    // with the FP64 operator.
    if (have_fp64_residual && rerr + REC_ERR * rnorm < 0.1 * t) {
      k_residual_inner<<<nb3, VB, 0, stream>>>(n3, r32.p, r.p, slots(S_RED), scal.p);
      CG_LAUNCH();
      k_accumulate<<<nb3, VB, 0, stream>>>(n3, x.p, d32.p);
      CG_LAUNCH();
      rerr += REC_ERR * rnorm;
    } else if (!(have_fp64_residual && rerr + CORR_ERR * rnorm < 0.1 * t)) {
      // x += d; r = F - B64 x: the residual recomputed with the FP64 operator
      k_accumulate<<<nb3, VB, 0, stream>>>(n3, x.p, d32.p);
      CG_LAUNCH();
      apply64(x.p, Ap.p, false, NEAR_DD);
      last.fp64_applies++;
      k_residual<<<nb3, VB, 0, stream>>>(n3, F.p, Ap.p, r.p, slots(S_RED), scal.p);
      CG_LAUNCH();
      have_fp64_residual = true;
      rerr               = 0.0;
    } else {
      // Later corrections are small: r -= B d with B d in FP32 (its error is
      // ~1e-7 of ||B d|| ~ ||r||, far below the threshold), accumulated into
      // the FP64 residual; then x += d.
      apply32(d32.p, Ap32.p, false);
      last.fp32_applies++;
      k_residual_update<<<nb3, VB, 0, stream>>>(n3, Ap32.p, r.p, slots(S_RED), scal.p);
      CG_LAUNCH();
      k_accumulate<<<nb3, VB, 0, stream>>>(n3, x.p, d32.p);
      CG_LAUNCH();
      rerr += CORR_ERR * rnorm;
    }
  }
  if (status != CPPE_GPU_OK) {
    CG_CUDA(cudaMemcpyAsync(h_scal, scal.p, S_NSCAL * sizeof(double), cudaMemcpyDeviceToHost,
                            stream));
    CG_CUDA(cudaStreamSynchronize(stream));
    if (h_scal[S_RNORM] + rerr < t) status = CPPE_GPU_OK;
    outer_hist.push_back(h_scal[S_RNORM]);
  }
  last.iterations  = total_inner;
  last.final_rnorm = outer_hist.empty() ? 0.0 : outer_hist.back();
  // one recorded norm per FP64 refinement residual
  if (iters) *iters = (int)outer_hist.size();
  if (hist_out)
    for (int k = 0; k < std::min<int>(hist_cap, (int)outer_hist.size()); ++k)
      hist_out[k] = outer_hist[k];
  return status;
}

int System::solve_device(const double* d_rhs, const double* d_guess, int make_guess,
                         double* d_mu, int* iters, double* hist_out, int hist_cap) {
  CG_CUDA(cudaSetDevice(device));
  const int n3 = 3 * n;
  permute_in(geo, d_rhs, F.p, 3, stream);
  bool zero = false;
  use_model = make_guess && model != nullptr;
  const bool ran_model = use_model;
  if (use_model) {
    learned_start();
  } else if (make_guess) {
    k_sym_apply<<<(n + VB - 1) / VB, VB, 0, stream>>>(n, alpha64.p, F.p, x.p);
    CG_LAUNCH();
  } else if (d_guess) {
    permute_in(geo, d_guess, x.p, 3, stream);
  } else {
    zero = true;
  }
  (void)n3;
  int st = opt.precision == CPPE_GPU_MIXED ? solve_mixed(zero, hist_out, hist_cap, iters)
                                           : solve_fp64(zero, hist_out, hist_cap, iters);
  if (use_model && st != CPPE_GPU_OK) {
    // plain PCG is the fallback of the learned start and preconditioner
    use_model = false;
    k_sym_apply<<<(n + VB - 1) / VB, VB, 0, stream>>>(n, alpha64.p, F.p, x.p);
    CG_LAUNCH();
    st = opt.precision == CPPE_GPU_MIXED ? solve_mixed(false, hist_out, hist_cap, iters)
                                         : solve_fp64(false, hist_out, hist_cap, iters);
  }
  use_model = false;
  permute_out(geo, x.p, d_mu, 3, stream);
  if (ran_model)
    CG_CUDA(cudaMemcpyAsync(h_flags + 4, model->tc_err.p, sizeof(int), cudaMemcpyDeviceToHost,
                            stream));
  CG_CUDA(cudaStreamSynchronize(stream));
  if (ran_model && h_flags[4])
    fail(CPPE_GPU_TIMEOUT,
         "tensor-core MLP inference: a wait on the MMA barrier timed out (the answer still "
         "met the FP64 stopping rule)");
  return st;
}

// ---------------------------------------------------------------------------
// Learned initial guess and preconditioner correction
// ---------------------------------------------------------------------------
__global__ void k_rows(int n, const float* __restrict__ v1, const float* __restrict__ v2,
                       const float* __restrict__ v3, const double* __restrict__ mu,
                       const float* __restrict__ a, const float* __restrict__ w,
                       const double* __restrict__ x0, float* __restrict__ rows) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float* o = rows + (size_t)i * Mlp::TROW;
  float s = 0.f, t = 0.f;
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)i + c;
    o[c] = v1[k], o[3 + c] = v2[k], o[6 + c] = v3[k], o[9 + c] = (float)mu[k];
    o[12 + c] = a[k], o[15 + c] = w[k], o[18 + c] = (float)(mu[k] - x0[k]);
    s += v1[k] * v1[k];
    t += a[k] * a[k];
  }
  o[21] = s, o[22] = t, o[23] = 0.f;
}

void System::learned_setup() {
  if (near) return;
  near = std::make_unique<NearList>();
  near->build(geo, excl_ptr_h.empty() ? nullptr : excl_ptr_h.data(),
              excl_idx_h.empty() ? nullptr : excl_idx_h.data(), opt.damp, opt.damping_factor,
              stream);
  const size_t n3 = 3 * (size_t)n;
  lf_feats.alloc((size_t)n * Mlp::IN);
  for (auto* b : {&lf_v1, &lf_v2, &lf_v3, &lf_w32, &lf_rold32}) b->alloc(n3);
  lf_Y.alloc((size_t)n * Mlp::OUT);
  lf_c.alloc(n);
  lf_w64.alloc(n3);
  lf_rold64.alloc(n3);
  lf_z4.alloc(n);
}

void System::learned_features_for_F() {
  learned_setup();
  const NearListView nl = view(*near);
  learned_features(nl, alpha32.p, F.p, lf_feats.p, lf_v1.p, stream);
  near_T<float>(nl, alpha32.p, lf_v1.p, lf_v2.p, stream);
  near_T<float>(nl, alpha32.p, lf_v2.p, lf_v3.p, stream);
  learned_basis_features(n, lf_v1.p, lf_v2.p, lf_v3.p, lf_feats.p, stream);
}

void System::learned_start() {
  learned_features_for_F();
  model->infer(n, lf_feats.p, lf_Y.p, stream);
  learned_guess(n, lf_Y.p, lf_v1.p, lf_v2.p, lf_v3.p, x.p, lf_c.p, stream);
}

template <typename T>
T* System::learned_precond(T* zv, const T* rv, T* pv, bool start) {
  const NearListView nl = view(*near);
  if ((8 * (size_t)n + 127) / 128 * 2 > partials.n)
    fail(CPPE_GPU_INVALID_ARG, "reduction buffer too small for the learned preconditioner");
  if constexpr (std::is_same<T, double>::value) {
    precond_near<double>(nl, alpha64.p, lf_c.p, zv, rv, lf_rold64.p, lf_w64.p, pv, start,
                         partials.p, ticket.p, scal.p, flags.p, stream);
    return lf_w64.p;
  } else {
    precond_near<float>(nl, alpha32.p, lf_c.p, zv, rv, lf_rold32.p, lf_w32.p, pv, start,
                        partials.p, ticket.p, scal.p, flags.p, stream, lf_z4.p);
    return lf_w32.p;
  }
}
template double* System::learned_precond<double>(double*, const double*, double*, bool);
template float* System::learned_precond<float>(float*, const float*, float*, bool);

void System::learned_rows(const double* mu_dev, std::vector<float>& feats, std::vector<float>& rows) {
  // F holds the rhs (device order); x0 = alpha F; r0 = F - B x0 (FP64)
  learned_features_for_F();
  const int nb = (n + VB - 1) / VB;
  k_sym_apply<<<nb, VB, 0, stream>>>(n, alpha64.p, F.p, x.p);
  CG_LAUNCH();
  apply64(x.p, Ap.p, false);
  k_residual<<<(3 * n + VB - 1) / VB, VB, 0, stream>>>(3 * n, F.p, Ap.p, r.p, slots(S_RED),
                                                        scal.p);
  CG_LAUNCH();
  // a = alpha r0 (FP64 -> FP32), w = alpha T_near a
  k_sym_apply<<<nb, VB, 0, stream>>>(n, alpha64.p, r.p, tmp_out.p);
  CG_LAUNCH();
  k_to_f32<<<(3 * n + VB - 1) / VB, VB, 0, stream>>>(3 * n, tmp_out.p, lf_w32.p);
  CG_LAUNCH();
  near_T<float>(view(*near), alpha32.p, lf_w32.p, lf_rold32.p, stream);
  DBuf<float> rows_d;
  rows_d.alloc((size_t)n * Mlp::TROW);
  k_rows<<<nb, VB, 0, stream>>>(n, lf_v1.p, lf_v2.p, lf_v3.p, mu_dev, lf_w32.p, lf_rold32.p, x.p,
                                rows_d.p);
  CG_LAUNCH();
  feats.resize((size_t)n * Mlp::IN);
  rows.resize((size_t)n * Mlp::TROW);
  CG_CUDA(cudaMemcpyAsync(feats.data(), lf_feats.p, feats.size() * sizeof(float),
                          cudaMemcpyDeviceToHost, stream));
  CG_CUDA(cudaMemcpyAsync(rows.data(), rows_d.p, rows.size() * sizeof(float),
                          cudaMemcpyDeviceToHost, stream));
  CG_CUDA(cudaStreamSynchronize(stream));
}

}  // namespace cg
