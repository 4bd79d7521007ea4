// The C ABI (include/cppe_gpu.h): argument checking, host<->device copies,
// and dispatch to the System solvers and the field engine.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <random>
#include <string>

#include "batch.h"
#include "system.h"

namespace cg {

static thread_local std::string g_last_error;
long long& launch_counter() {
  static long long c = 0;
  return c;
}

// FMA throughput probe: 8 independent FMA chains per thread.
template <typename T>
__global__ void k_fma_peak(T* out, int iters) {
  T a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = T(threadIdx.x + k) * T(1e-7);
  const T b = T(0.9999999), c = T(1e-9);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == T(-12345)) out[0] = s;
}
void set_last_error(const std::string& msg) { g_last_error = msg; }

template <class F>
static int guard(F&& f) {
  try {
    int st = f();
    if (st == CPPE_GPU_NOT_CONVERGED)
      set_last_error("Failed to converge induced dipole moments.");
    return st;
  } catch (const Failure& e) {
    set_last_error(e.what());
    return e.status;
  } catch (const std::bad_alloc&) {
    set_last_error("host allocation failed");
    return CPPE_GPU_INVALID_ARG;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return CPPE_GPU_INVALID_ARG;
  }
}

static void need(bool ok, const char* what) {
  if (!ok) fail(CPPE_GPU_INVALID_ARG, what);
}

// ---------------------------------------------------------------------------
// Small kernels used by the C ABI only
// ---------------------------------------------------------------------------
// Dense B (row-major 3n x 3n): -T_ij (damped where both partners polarizable)
// off the diagonal, alpha_i^-1 on it (BMatrix::to_dense_matrix, bmatrix.cc:64-92).
__global__ void k_dense(int n, const double4_32a* __restrict__ pos, const double* __restrict__ ainv6,
                        const int* __restrict__ ep, const int* __restrict__ ei, int damp,
                        double damping, double* __restrict__ B) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * n) return;
  const int i = (int)(t / n), j = (int)(t % n);
  double blk[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (i == j) {
    const double* a = ainv6 + 6 * (size_t)i;
    double s[9]     = {a[0], a[1], a[2], a[1], a[3], a[4], a[2], a[4], a[5]};
    for (int k = 0; k < 9; ++k) blk[k] = s[k];
  } else {
    bool excluded = false;
    if (ep)
      for (int e = ep[i]; e < ep[i + 1]; ++e) excluded |= (ei[e] == j);
    if (!excluded) {
      const double4_32a pi = pos[i], pj = pos[j];
      const double x = pj.x - pi.x, y = pj.y - pi.y, z = pj.z - pi.z;
      const double r2 = x * x + y * y + z * z;
      double G[2];
      radial<double, 2>(r2, damp ? damping * pi.w * pj.w : 0.0, G);
      // T2_ab = d_a d_b (1/R) (damped) = delta_ab G1 + r_a r_b G2; B = -T2.
      const double r[3] = {x, y, z};
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) blk[3 * a + b] = -((a == b ? G[0] : 0.0) + r[a] * r[b] * G[1]);
    }
  }
  const size_t N3 = 3 * (size_t)n;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) B[(3 * (size_t)i + a) * N3 + 3 * (size_t)j + b] = blk[3 * a + b];
}

// Gauss-Jordan elimination on [A | I] stored as A (in place) and Inv; one
// pivot column per launch pair.  B is symmetric positive definite for
// physical polarizabilities, so no pivoting is needed.
__global__ void k_gj_pivot(int N, int k, const double* A, double* piv) {
  *piv = A[(size_t)k * N + k];
}
__global__ void k_gj_row(int N, int k, double* A, double* Inv, const double* piv) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < N) {
    const double d = *piv;
    A[(size_t)k * N + c] /= d;
    Inv[(size_t)k * N + c] /= d;
  }
}
__global__ void k_gj_elim(int N, int k, double* A, double* Inv, const double* colk) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)N * N) return;
  const int r = (int)(t / N), c = (int)(t % N);
  if (r == k) return;
  const double f = colk[r];
  A[(size_t)r * N + c] -= f * A[(size_t)k * N + c];
  Inv[(size_t)r * N + c] -= f * Inv[(size_t)k * N + c];
}
__global__ void k_copy_col(int N, int k, const double* A, double* col) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r < N) col[r] = A[(size_t)r * N + k];
}
__global__ void k_eye(int N, double* I) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < (long)N * N) I[t] = (t / N == t % N) ? 1.0 : 0.0;
}

__global__ void k_charge_fields(int nt, const double* __restrict__ xt, int ns,
                                const double* __restrict__ xs, const double* __restrict__ q,
                                double* __restrict__ F) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  double f[3] = {0, 0, 0};
  const double x = xt[3 * i], y = xt[3 * i + 1], z = xt[3 * i + 2];
  for (int k = 0; k < ns; ++k) {
    const double dx = x - xs[3 * k], dy = y - xs[3 * k + 1], dz = z - xs[3 * k + 2];
    const double ir = rsqrt(dx * dx + dy * dy + dz * dz);
    const double c  = q[k] * ir * ir * ir;
    f[0] += c * dx, f[1] += c * dy, f[2] += c * dz;
  }
  F[3 * i] = f[0], F[3 * i + 1] = f[1], F[3 * i + 2] = f[2];
}

// Potential energy of point charges Z_a in the field of the site multipoles:
// sum_a Z_a [q/R + mu.d/R^3 + 1/2 Theta:(3 d d/R^5 - I/R^3)], d = R_a - r_s
// (prefactors_nuclei (-1)^k/k! times symmetry factors, math.cc:77-91).
__global__ void k_mp_energy(int n, const double* __restrict__ xyz, const double* __restrict__ q,
                            const double* __restrict__ mu, const double* __restrict__ quad,
                            int max_order, int na, const double* __restrict__ ax,
                            const double* __restrict__ az, ReduceSlots rs) {
  __shared__ double sh[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e[1] = {0.0};
  if (i < n) {
    for (int a = 0; a < na; ++a) {
      const double dx = ax[3 * a] - xyz[3 * i], dy = ax[3 * a + 1] - xyz[3 * i + 1],
                   dz = ax[3 * a + 2] - xyz[3 * i + 2];
      const double r2 = dx * dx + dy * dy + dz * dz;
      const double ir = rsqrt(r2), ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
      double v        = q ? q[i] * ir : 0.0;
      if (max_order > 0 && mu)
        v += (mu[3 * i] * dx + mu[3 * i + 1] * dy + mu[3 * i + 2] * dz) * ir3;
      if (max_order > 1 && quad) {
        const double* Q = quad + 6 * (size_t)i;
        const double d[3] = {dx, dy, dz};
        const double Qm[9] = {Q[0], Q[1], Q[2], Q[1], Q[3], Q[4], Q[2], Q[4], Q[5]};
        double s = 0.0;
        for (int u = 0; u < 3; ++u)
          for (int w = 0; w < 3; ++w)
            s += Qm[3 * u + w] * (3.0 * d[u] * d[w] * ir5 - (u == w ? ir3 : 0.0));
        v += 0.5 * s;
      }
      e[0] += az[a] * v;
    }
  }
  grid_sum_last<1>(e, sh, rs.partials, rs.ticket, rs.out);
}

// Derivatives of the charge fields with respect to the charges' positions
// (NuclearFields::nuclear_gradient, electric_fields.cc:77-104):
// G[3a + c][3i + d] = q_a T2(r_i - R_a)_{cd}, T2 = grad grad 1/R; a thread per
// (charge, target) pair writes its 3 x 3 block.
__global__ void k_charge_field_grad(int nt, const double* __restrict__ xt, int ns,
                                    const double* __restrict__ xs, const double* __restrict__ q,
                                    double* __restrict__ G) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)nt * ns) return;
  const int a = (int)(t / nt), i = (int)(t % nt);
  const double d[3] = {xt[3 * i] - xs[3 * a], xt[3 * i + 1] - xs[3 * a + 1],
                       xt[3 * i + 2] - xs[3 * a + 2]};
  const double ir = rsqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  const double ir3 = ir * ir * ir, ir5 = ir3 * ir * ir;
  const size_t row = 3 * (size_t)nt;
  for (int c = 0; c < 3; ++c)
    for (int e = 0; e < 3; ++e)
      G[(3 * (size_t)a + c) * row + 3 * (size_t)i + e] =
            q[a] * (3.0 * d[c] * d[e] * ir5 - (c == e ? ir3 : 0.0));
}

// Gradient of sum_a Z_a phi_multipoles(R_a) with respect to the charges'
// positions R_a (MultipoleExpansion::nuclear_gradient,
// multipole_expansion.cc:35-62, through multipole_derivative with l = 1):
//   dE/dR_a = Z_a sum_i [ q_i T1(d) - T2(d) mu_i + 1/2 sum_jk Theta_jk T3(d)_jkm ],
//   d = R_a - r_i, T_n = n-th Cartesian derivative tensor of 1/R, with the
// signs of the reference's Taylor prefactors (-1)^(k+1)/k!.  Block (b, a)
// sums its sites for charge a into partials[(a * gridDim.x + b) * 3 + m].
__global__ void k_mp_energy_grad(int n, const double* __restrict__ xyz,
                                 const double* __restrict__ q, const double* __restrict__ mu,
                                 const double* __restrict__ quad, int max_order,
                                 const double* __restrict__ ax, const double* __restrict__ az,
                                 double* __restrict__ partials) {
  __shared__ double sh[32 * 3];
  const int a = blockIdx.y;
  double g[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d[3] = {ax[3 * a] - xyz[3 * i], ax[3 * a + 1] - xyz[3 * i + 1],
                         ax[3 * a + 2] - xyz[3 * i + 2]};
    const double ir = rsqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    const double ir3 = ir * ir * ir, ir5 = ir3 * ir * ir, ir7 = ir5 * ir * ir;
    // charge: -q d / R^3 (= q T1)
    const double qi = q ? q[i] : 0.0;
    for (int m = 0; m < 3; ++m) g[m] -= qi * d[m] * ir3;
    if (max_order > 0 && mu) {
      // -T2 mu, T2_cm = 3 d_c d_m / R^5 - delta_cm / R^3
      const double* u = mu + 3 * (size_t)i;
      const double du = d[0] * u[0] + d[1] * u[1] + d[2] * u[2];
      for (int m = 0; m < 3; ++m) g[m] -= 3.0 * du * d[m] * ir5 - u[m] * ir3;
    }
    if (max_order > 1 && quad) {
      // 1/2 Theta_jk T3_jkm, T3_jkm = -15 d_j d_k d_m / R^7
      //                              + 3 (delta_jk d_m + delta_jm d_k + delta_km d_j) / R^5
      const double* Q = quad + 6 * (size_t)i;
      const double Qm[3][3] = {{Q[0], Q[1], Q[2]}, {Q[1], Q[3], Q[4]}, {Q[2], Q[4], Q[5]}};
      double Qd[3], dQd = 0.0;
      const double tr = Q[0] + Q[3] + Q[5];
      for (int j = 0; j < 3; ++j) {
        Qd[j] = Qm[j][0] * d[0] + Qm[j][1] * d[1] + Qm[j][2] * d[2];
        dQd += d[j] * Qd[j];
      }
      for (int m = 0; m < 3; ++m)
        g[m] += 0.5 * (-15.0 * dQd * d[m] * ir7 + 3.0 * (tr * d[m] + 2.0 * Qd[m]) * ir5);
    }
  }
  const double z = az[a];
  for (int m = 0; m < 3; ++m) g[m] *= z;
  block_sum<3>(g, sh);
  if (threadIdx.x == 0)
    for (int m = 0; m < 3; ++m) partials[((size_t)a * gridDim.x + blockIdx.x) * 3 + m] = g[m];
}

// grad[a][m] = sum of the blocks' partials in block order (fixed order).
__global__ void k_mp_energy_grad_sum(int na, int nb, const double* __restrict__ partials,
                                     double* __restrict__ grad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 3 * na) return;
  const int a = t / 3, m = t % 3;
  double s = 0.0;
  for (int b = 0; b < nb; ++b) s += partials[((size_t)a * nb + b) * 3 + m];
  grad[t] = s;
}

}  // namespace cg

using namespace cg;

struct cppe_gpu_system {
  System s;
};
struct cppe_gpu_batch {
  BatchSystem b;
};
struct cppe_gpu_mlp {
  Mlp m;
};

extern "C" {

void cppe_gpu_default_options(cppe_gpu_options* o) {
  if (!o) return;
  o->summation            = CPPE_GPU_DIRECT;
  o->tree_ncrit           = 64;
  o->tree_expansion_order = 5;
  o->theta                = 0.5;
  o->damp                 = 0;
  o->damping_factor       = 2.1304;
  o->induced_thresh       = 1e-8;
  o->maxiter              = 50;
  o->precision            = CPPE_GPU_FP64;
  o->device               = 0;
}

int cppe_gpu_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return CPPE_GPU_INVALID_ARG;
  std::strncpy(buf, g_last_error.c_str(), len - 1);
  buf[len - 1] = 0;
  return CPPE_GPU_OK;
}

int cppe_gpu_device_count(int* count) {
  return guard([&]() -> int {
    need(count, "count is null");
    int c        = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
      cudaGetLastError();
      c = 0;
    }
    *count = c;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_create(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
                    const int* excl_idx, const cppe_gpu_options* opts, cppe_gpu_system** out) {
  return guard([&]() -> int {
    need(out && opts, "null argument");
    *out   = nullptr;
    auto h = std::make_unique<cppe_gpu_system>();
    h->s.init(n, xyz, alpha6, excl_ptr, excl_idx, *opts);
    *out = h.release();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_destroy(cppe_gpu_system* sys) {
  return guard([&]() -> int {
    delete sys;
    return CPPE_GPU_OK;
  });
}

// arith: 0 FP64, 1 FP32, 2 FP64 with the double-float near field
static int apply_host(cppe_gpu_system* sys, const double* in, double* out, int arith) {
  return guard([&]() -> int {
    need(sys && in && out, "null argument");
    System& S = sys->s;
    CG_CUDA(cudaSetDevice(S.device));
    const size_t n3 = 3 * (size_t)S.n;
    CG_CUDA(cudaMemcpyAsync(S.tmp_out.p, in, n3 * sizeof(double), cudaMemcpyHostToDevice,
                            S.stream));
    permute_in(S.geo, S.tmp_out.p, S.tmp_in.p, 3, S.stream);
    if (arith == 1)
      S.apply32_widen(S.tmp_in.p, S.tmp_out.p);
    else
      S.apply64(S.tmp_in.p, S.tmp_out.p, false, arith == 2 ? NEAR_DD : NEAR_FP64);
    permute_out(S.geo, S.tmp_out.p, S.tmp_in.p, 3, S.stream);
    CG_CUDA(cudaMemcpyAsync(out, S.tmp_in.p, n3 * sizeof(double), cudaMemcpyDeviceToHost,
                            S.stream));
    CG_CUDA(cudaStreamSynchronize(S.stream));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_bmatrix_apply(cppe_gpu_system* sys, const double* in, double* out) {
  return apply_host(sys, in, out, 0);
}
int cppe_gpu_bmatrix_apply_fp32(cppe_gpu_system* sys, const double* in, double* out) {
  return apply_host(sys, in, out, 1);
}
int cppe_gpu_bmatrix_apply_dd(cppe_gpu_system* sys, const double* in, double* out) {
  return apply_host(sys, in, out, 2);
}

int cppe_gpu_bmatrix_apply_device(cppe_gpu_system* sys, const double* d_in, double* d_out) {
  return guard([&]() -> int {
    need(sys && d_in && d_out, "null argument");
    System& S = sys->s;
    CG_CUDA(cudaSetDevice(S.device));
    permute_in(S.geo, d_in, S.tmp_in.p, 3, S.stream);
    S.apply64(S.tmp_in.p, S.tmp_out.p, false);
    permute_out(S.geo, S.tmp_out.p, d_out, 3, S.stream);
    CG_CUDA(cudaStreamSynchronize(S.stream));
    return CPPE_GPU_OK;
  });
}

static int diag_host(cppe_gpu_system* sys, const double* in, double* out, bool inverse) {
  return guard([&]() -> int {
    need(sys && in && out, "null argument");
    System& S = sys->s;
    // 3x3 blocks per site in caller order (BMatrix::apply_diagonal{,_inverse})
    std::vector<double> a6(6 * (size_t)S.n);
    const DBuf<double>& src = inverse ? S.alpha64 : S.ainv64;
    CG_CUDA(cudaSetDevice(S.device));
    CG_CUDA(cudaMemcpy(a6.data(), src.p, a6.size() * sizeof(double), cudaMemcpyDeviceToHost));
    for (int k = 0; k < S.n; ++k) {
      const int i     = S.geo.layout.perm[k];
      const double* a = &a6[6 * (size_t)k];
      const double* v = in + 3 * (size_t)i;
      double* o       = out + 3 * (size_t)i;
      o[0]            = a[0] * v[0] + a[1] * v[1] + a[2] * v[2];
      o[1]            = a[1] * v[0] + a[3] * v[1] + a[4] * v[2];
      o[2]            = a[2] * v[0] + a[4] * v[1] + a[5] * v[2];
    }
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_apply_diagonal(cppe_gpu_system* sys, const double* in, double* out) {
  return diag_host(sys, in, out, false);
}
int cppe_gpu_apply_diagonal_inverse(cppe_gpu_system* sys, const double* in, double* out) {
  return diag_host(sys, in, out, true);
}

int cppe_gpu_to_dense(cppe_gpu_system* sys, double* out) {
  return guard([&]() -> int {
    need(sys && out, "null argument");
    System& S = sys->s;
    CG_CUDA(cudaSetDevice(S.device));
    const int n     = S.n;
    const size_t N3 = 3 * (size_t)n;
    DBuf<double> B, ainv;
    DBuf<double4_32a> pos;
    B.alloc(N3 * N3);
    // caller-order positions and alpha^-1
    std::vector<double4_32a> p64(n);
    std::vector<double> ai(6 * (size_t)n), aperm(6 * (size_t)n);
    std::vector<double4_32a> pperm(n);
    CG_CUDA(cudaMemcpy(pperm.data(), S.geo.pos64.p, n * sizeof(double4_32a), cudaMemcpyDeviceToHost));
    CG_CUDA(cudaMemcpy(aperm.data(), S.ainv64.p, aperm.size() * sizeof(double),
                       cudaMemcpyDeviceToHost));
    for (int k = 0; k < n; ++k) {
      const int i = S.geo.layout.perm[k];
      p64[i]      = pperm[k];
      std::copy(&aperm[6 * (size_t)k], &aperm[6 * (size_t)k] + 6, &ai[6 * (size_t)i]);
    }
    pos.upload(p64, S.stream);
    ainv.upload(ai, S.stream);
    DBuf<int> ep, ei;
    ep.upload(S.excl_ptr_h, S.stream);
    ei.upload(S.excl_idx_h.empty() ? std::vector<int>{0} : S.excl_idx_h, S.stream);
    const long tot = (long)n * n;
    k_dense<<<(unsigned)((tot + 255) / 256), 256, 0, S.stream>>>(
          n, pos.p, ainv.p, S.excl_ptr_h.empty() ? nullptr : ep.p, ei.p, S.opt.damp,
          S.opt.damping_factor, B.p);
    CG_LAUNCH();
    CG_CUDA(cudaMemcpyAsync(out, B.p, N3 * N3 * sizeof(double), cudaMemcpyDeviceToHost,
                            S.stream));
    CG_CUDA(cudaStreamSynchronize(S.stream));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_direct_inverse(cppe_gpu_system* sys, double* out) {
  return guard([&]() -> int {
    need(sys && out, "null argument");
    System& S       = sys->s;
    const int N     = 3 * S.n;
    const size_t NN = (size_t)N * N;
    std::vector<double> h(NN);
    int st = cppe_gpu_to_dense(sys, h.data());
    if (st) return st;
    CG_CUDA(cudaSetDevice(S.device));
    DBuf<double> A, I, col, piv;
    A.upload(h, S.stream);
    I.alloc(NN);
    col.alloc(N);
    piv.alloc(1);
    const unsigned gNN = (unsigned)((NN + 255) / 256), gN = (unsigned)((N + 255) / 256);
    k_eye<<<gNN, 256, 0, S.stream>>>(N, I.p);
    for (int k = 0; k < N; ++k) {
      k_gj_pivot<<<1, 1, 0, S.stream>>>(N, k, A.p, piv.p);
      k_gj_row<<<gN, 256, 0, S.stream>>>(N, k, A.p, I.p, piv.p);
      k_copy_col<<<gN, 256, 0, S.stream>>>(N, k, A.p, col.p);
      k_gj_elim<<<gNN, 256, 0, S.stream>>>(N, k, A.p, I.p, col.p);
    }
    CG_LAUNCH();
    CG_CUDA(cudaMemcpyAsync(out, I.p, NN * sizeof(double), cudaMemcpyDeviceToHost, S.stream));
    CG_CUDA(cudaStreamSynchronize(S.stream));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_solve_device(cppe_gpu_system* sys, const double* d_rhs, const double* d_guess,
                          int make_guess, double* d_mu, int* iters, double* rnorm_hist,
                          int hist_cap) {
  return guard([&]() -> int {
    need(sys && d_rhs && d_mu, "null argument");
    return sys->s.solve_device(d_rhs, d_guess, make_guess, d_mu, iters, rnorm_hist, hist_cap);
  });
}

int cppe_gpu_solve(cppe_gpu_system* sys, const double* rhs, const double* guess,
                   int make_guess, double* mu, int* iters, double* rnorm_hist, int hist_cap) {
  return guard([&]() -> int {
    need(sys && rhs && mu, "null argument");
    System& S = sys->s;
    CG_CUDA(cudaSetDevice(S.device));
    const size_t n3 = 3 * (size_t)S.n;
    S.io_rhs.upload(rhs, n3, S.stream);
    if (guess && !make_guess) S.io_guess.upload(guess, n3, S.stream);
    S.io_mu.alloc(n3);
    int st = S.solve_device(S.io_rhs.p, (guess && !make_guess) ? S.io_guess.p : nullptr,
                            make_guess, S.io_mu.p, iters, rnorm_hist, hist_cap);
    CG_CUDA(cudaMemcpyAsync(mu, S.io_mu.p, n3 * sizeof(double), cudaMemcpyDeviceToHost,
                            S.stream));
    CG_CUDA(cudaStreamSynchronize(S.stream));
    return st;
  });
}

int cppe_gpu_last_solve_stats(cppe_gpu_system* sys, double* final_rnorm, int* fp64_applies,
                              int* fp32_applies) {
  return guard([&]() -> int {
    need(sys, "null argument");
    if (final_rnorm) *final_rnorm = sys->s.last.final_rnorm;
    if (fp64_applies) *fp64_applies = sys->s.last.fp64_applies;
    if (fp32_applies) *fp32_applies = sys->s.last.fp32_applies;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_multipole_fields(int n, const double* xyz, const double* q, const double* mu,
                              const double* quad, int max_order, const int* polarizable,
                              const double* alpha_iso, const int* excl_ptr,
                              const int* excl_idx, int summation, int ncrit, int order,
                              double theta, int damp, double damping_factor, int device,
                              double* F) {
  return guard([&]() -> int {
    need(n > 0 && xyz && F, "null argument");
    need(max_order >= 0 && max_order <= 2,
         "MultipoleFields::compute_tree only supported up to 2nd order.");
    const bool fmm = summation == CPPE_GPU_FMM;
    if (fmm) {
      // orders the reference's generated operators provide (field_m*.cc dispatch)
      need(order >= 1 && order <= 7, "tree_expansion_order must be in [1, 7]");
      if (max_order >= 1) need(order >= 2, "dipole sources need tree_expansion_order >= 2");
      if (max_order >= 2) need(order >= 3, "quadrupole sources need tree_expansion_order >= 3");
    }
    int ndev = 0;
    CG_CUDA(cudaGetDeviceCount(&ndev));
    need(device >= 0 && device < ndev, "bad CUDA device ordinal");
    CG_CUDA(cudaSetDevice(device));
    cudaStream_t s;
    CG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    struct StreamGuard {
      cudaStream_t s;
      ~StreamGuard() { cudaStreamDestroy(s); }
    } sg{s};
    std::vector<double> sd(n, 0.0);
    if (damp)
      for (int i = 0; i < n; ++i)
        if (polarizable && polarizable[i] && alpha_iso && alpha_iso[i] > 0.0)
          sd[i] = std::pow(alpha_iso[i], -1.0 / 6.0);
    Geometry g;
    g.build(n, xyz, sd.data(), excl_ptr, excl_idx, fmm, ncrit, theta, s);
    const size_t n3 = 3 * (size_t)n;
    DBuf<double> out, tmp, srcp;
    out.alloc(n3);
    out.zero(s);
    FieldWork<double> w;
    auto run = [&](int m, const double* host_src, double sign) {
      const int nc = ncomp(m);
      std::vector<double> h(host_src, host_src + nc * (size_t)n);
      if (m == 2)
        for (int i = 0; i < n; ++i) h[6 * i] *= 0.5, h[6 * i + 3] *= 0.5, h[6 * i + 5] *= 0.5;
      tmp.upload(h, s);
      srcp.alloc(nc * (size_t)n);
      permute_in(g, tmp.p, srcp.p, nc, s);
      std::unique_ptr<DeviceOps> ops;
      if (fmm) {
        ops = std::make_unique<DeviceOps>();
        ops->build(m, order, s);
      }
      eval_field<double>(g, ops.get(), w, m, srcp.p, damp != 0, damping_factor, FINISH_FIELD,
                         nullptr, nullptr, out.p, sign, nullptr, s);
      CG_CUDA(cudaStreamSynchronize(s));
    };
    std::vector<double> zeros;
    if (!q) zeros.assign(n, 0.0);
    run(0, q ? q : zeros.data(), 1.0);
    if (max_order > 0) {
      need(mu, "dipoles missing");
      run(1, mu, -1.0);
    }
    if (max_order > 1) {
      need(quad, "quadrupoles missing");
      run(2, quad, 1.0);
    }
    tmp.alloc(n3);
    permute_out(g, out.p, tmp.p, 3, s);
    CG_CUDA(cudaMemcpyAsync(F, tmp.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_charge_fields(int ntgt, const double* xyz_tgt, int nsrc, const double* xyz_src,
                           const double* q, int device, double* F) {
  return guard([&]() -> int {
    need(ntgt >= 0 && nsrc >= 0 && F, "null argument");
    if (ntgt == 0) return CPPE_GPU_OK;
    if (nsrc == 0) {
      std::fill(F, F + 3 * (size_t)ntgt, 0.0);
      return CPPE_GPU_OK;
    }
    need(xyz_tgt && xyz_src && q, "null argument");
    CG_CUDA(cudaSetDevice(device));
    DBuf<double> xt, xs, dq, dF;
    xt.upload(xyz_tgt, 3 * (size_t)ntgt, 0);
    xs.upload(xyz_src, 3 * (size_t)nsrc, 0);
    dq.upload(q, nsrc, 0);
    dF.alloc(3 * (size_t)ntgt);
    k_charge_fields<<<(ntgt + 127) / 128, 128>>>(ntgt, xt.p, nsrc, xs.p, dq.p, dF.p);
    CG_LAUNCH();
    CG_CUDA(cudaMemcpy(F, dF.p, 3 * (size_t)ntgt * sizeof(double), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_multipole_potential_energy(int n, const double* xyz, const double* q,
                                        const double* mu, const double* quad, int max_order,
                                        int natoms, const double* atom_xyz,
                                        const double* atom_charge, int device,
                                        double* energy) {
  return guard([&]() -> int {
    need(energy, "null argument");
    *energy = 0.0;
    if (n == 0 || natoms == 0) return CPPE_GPU_OK;
    need(xyz && atom_xyz && atom_charge, "null argument");
    CG_CUDA(cudaSetDevice(device));
    DBuf<double> dx, dq, dm, dQ, ax, az, part, outv;
    DBuf<unsigned> tk;
    dx.upload(xyz, 3 * (size_t)n, 0);
    if (q) dq.upload(q, n, 0);
    if (mu && max_order > 0) dm.upload(mu, 3 * (size_t)n, 0);
    if (quad && max_order > 1) dQ.upload(quad, 6 * (size_t)n, 0);
    ax.upload(atom_xyz, 3 * (size_t)natoms, 0);
    az.upload(atom_charge, natoms, 0);
    const int nb = (n + 255) / 256;
    part.alloc(nb + 1);
    outv.alloc(1);
    tk.alloc(1);
    tk.zero(0);
    k_mp_energy<<<nb, 256>>>(n, dx.p, dq.p, dm.p, dQ.p, max_order, natoms, ax.p, az.p,
                             ReduceSlots{part.p, tk.p, outv.p});
    CG_LAUNCH();
    CG_CUDA(cudaMemcpy(energy, outv.p, sizeof(double), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_charge_field_gradient(int ntgt, const double* xyz_tgt, int nsrc,
                                   const double* xyz_src, const double* q, int device,
                                   double* G) {
  return guard([&]() -> int {
    need(ntgt >= 0 && nsrc >= 0 && G, "null argument");
    if (ntgt == 0 || nsrc == 0) return CPPE_GPU_OK;
    need(xyz_tgt && xyz_src && q, "null argument");
    CG_CUDA(cudaSetDevice(device));
    DBuf<double> xt, xs, dq, dG;
    xt.upload(xyz_tgt, 3 * (size_t)ntgt, 0);
    xs.upload(xyz_src, 3 * (size_t)nsrc, 0);
    dq.upload(q, nsrc, 0);
    const size_t cnt = 9 * (size_t)ntgt * nsrc;
    dG.alloc(cnt);
    const long pairs = (long)ntgt * nsrc;
    k_charge_field_grad<<<(unsigned)((pairs + 127) / 128), 128>>>(ntgt, xt.p, nsrc, xs.p, dq.p,
                                                                  dG.p);
    CG_LAUNCH();
    CG_CUDA(cudaMemcpy(G, dG.p, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_multipole_energy_gradient(int n, const double* xyz, const double* q,
                                       const double* mu, const double* quad, int max_order,
                                       int natoms, const double* atom_xyz,
                                       const double* atom_charge, int device, double* grad) {
  return guard([&]() -> int {
    need(natoms >= 0 && n >= 0 && (grad || natoms == 0), "null argument");
    if (natoms == 0) return CPPE_GPU_OK;
    std::fill(grad, grad + 3 * (size_t)natoms, 0.0);
    if (n == 0) return CPPE_GPU_OK;
    need(xyz && atom_xyz && atom_charge, "null argument");
    need(max_order >= 0 && max_order <= 2, "multipoles above order 2 are not supported");
    CG_CUDA(cudaSetDevice(device));
    DBuf<double> dx, dq, dm, dQ, ax, az, part, dg;
    dx.upload(xyz, 3 * (size_t)n, 0);
    if (q) dq.upload(q, n, 0);
    if (mu && max_order > 0) dm.upload(mu, 3 * (size_t)n, 0);
    if (quad && max_order > 1) dQ.upload(quad, 6 * (size_t)n, 0);
    ax.upload(atom_xyz, 3 * (size_t)natoms, 0);
    az.upload(atom_charge, natoms, 0);
    const int nb = std::max(1, std::min((n + 255) / 256, 304));
    part.alloc(3 * (size_t)natoms * nb);
    dg.alloc(3 * (size_t)natoms);
    k_mp_energy_grad<<<dim3(nb, natoms), 256>>>(n, dx.p, dq.p, dm.p, dQ.p, max_order, ax.p,
                                                az.p, part.p);
    CG_LAUNCH();
    k_mp_energy_grad_sum<<<(3 * natoms + 127) / 128, 128>>>(natoms, nb, part.p, dg.p);
    CG_LAUNCH();
    CG_CUDA(cudaMemcpy(grad, dg.p, 3 * (size_t)natoms * sizeof(double), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_stream(cppe_gpu_system* sys, void** stream) {
  return guard([&]() -> int {
    need(sys && stream, "null argument");
    *stream = (void*)sys->s.stream;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_launch_count(long long* count) {
  if (!count) return CPPE_GPU_INVALID_ARG;
  *count = launch_counter();
  return CPPE_GPU_OK;
}

int cppe_gpu_kernel_timings(cppe_gpu_system* sys, int precision, int reps, double* out_ms,
                            long long* near_pairs, long long* m2l_pairs) {
  return guard([&]() -> int {
    need(sys && out_ms && reps > 0, "null argument");
    need(precision >= 0 && precision <= 2, "precision must be 0, 1 or 2");
    System& S = sys->s;
    S.phase_timings(precision, reps, out_ms);
    if (near_pairs) *near_pairs = S.geo.alg_pairs;
    if (m2l_pairs) *m2l_pairs = (long long)S.geo.layout.m2l_src.size();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_autotune(cppe_gpu_system* sys, int reps, double* best_ms) {
  return guard([&]() -> int {
    need(sys && reps > 0, "null argument");
    const double ms = sys->s.autotune(reps);
    if (best_ms) *best_ms = ms;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_set_schedule(cppe_gpu_system* sys, int near_form, long item_pairs,
                          int m2l_chunk) {
  return guard([&]() -> int {
    need(sys, "null argument");
    need(near_form >= -1 && near_form <= 2, "near_form must be -1, 0, 1 or 2");
    need(m2l_chunk <= 0 || m2l_chunk == 32 || m2l_chunk == 64 || m2l_chunk == 128,
         "m2l_chunk must be 32, 64 or 128");
    need(item_pairs <= 0 || item_pairs >= 1024, "item_pairs must be at least 1024");
    sys->s.set_schedule(near_form, item_pairs, m2l_chunk);
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_schedule_info(cppe_gpu_system* sys, int* symmetric_near, long* near_items,
                           int* m2l_chunk) {
  return guard([&]() -> int {
    need(sys, "null argument");
    const Geometry& g = sys->s.geo;
    if (symmetric_near) *symmetric_near = g.has_sym() ? g.sym_pack : 0;
    if (near_items)
      *near_items = (long)(g.has_sym() ? g.h_sym_items.size() : g.h_items.size());
    if (m2l_chunk) *m2l_chunk = g.m2l_chunk > 0 ? g.m2l_chunk : M2L_CHUNK;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_fma_peak(int device, int fp64, double* tflops) {
  return guard([&]() -> int {
    need(tflops, "null argument");
    CG_CUDA(cudaSetDevice(device));
    cudaDeviceProp prop;
    CG_CUDA(cudaGetDeviceProperties(&prop, device));
    const int blocks = prop.multiProcessorCount * 16, threads = 256;
    const int iters  = fp64 ? 64 : 2048;
    DBuf<double> sink;
    sink.alloc(1);
    cudaEvent_t e0, e1;
    CG_CUDA(cudaEventCreate(&e0));
    CG_CUDA(cudaEventCreate(&e1));
    double best = 0.0;
    for (int rep = 0; rep < 4; ++rep) {
      CG_CUDA(cudaEventRecord(e0, 0));
      if (fp64)
        k_fma_peak<double><<<blocks, threads>>>(sink.p, iters);
      else
        k_fma_peak<float><<<blocks, threads>>>((float*)sink.p, iters);
      CG_LAUNCH();
      CG_CUDA(cudaEventRecord(e1, 0));
      CG_CUDA(cudaEventSynchronize(e1));
      float ms;
      CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      const double flop = 2.0 * 8 * 4 * (double)iters * blocks * threads;
      if (rep > 0) best = std::max(best, flop / (ms * 1e-3) / 1e12);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_tree_info(int n, const double* xyz, int ncrit, double theta, int* ncells,
                       int* nleaves, long* nm2l, long* np2p, long* p2p_pairs) {
  return guard([&]() -> int {
    need(xyz, "null argument");
    RefTree t;
    std::string err;
    if (!build_ref_tree(n, xyz, ncrit, theta, t, err)) fail(CPPE_GPU_INVALID_ARG, err);
    TreeLayout L;
    make_layout(t, n, L);
    if (ncells) *ncells = L.ncells;
    if (nleaves) *nleaves = L.nleaves;
    if (nm2l) *nm2l = (long)t.m2l.size();
    if (np2p) *np2p = (long)t.p2p.size();
    if (p2p_pairs) *p2p_pairs = L.p2p_pairs;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_tree_vectors(int n, const double* xyz, int ncrit, double theta, int* nvec,
                          long* nentries) {
  return guard([&]() -> int {
    need(xyz && nvec, "null argument");
    RefTree t;
    std::string err;
    if (!build_ref_tree(n, xyz, ncrit, theta, t, err)) fail(CPPE_GPU_INVALID_ARG, err);
    TreeLayout L;
    make_layout(t, n, L);
    std::vector<int> vid;
    std::vector<double4_32a> vec;
    *nvec = m2l_vectors(L, vid, vec) ? (int)vec.size() : -1;
    if (nentries) *nentries = (long)L.m2l_src.size();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_tree_lists(int n, const double* xyz, int ncrit, double theta, int* m2l, int* p2p) {
  return guard([&]() -> int {
    need(xyz && m2l && p2p, "null argument");
    RefTree t;
    std::string err;
    if (!build_ref_tree(n, xyz, ncrit, theta, t, err)) fail(CPPE_GPU_INVALID_ARG, err);
    for (size_t i = 0; i < t.m2l.size(); ++i) m2l[2 * i] = t.m2l[i].first, m2l[2 * i + 1] = t.m2l[i].second;
    for (size_t i = 0; i < t.p2p.size(); ++i) p2p[2 * i] = t.p2p[i].first, p2p[2 * i + 1] = t.p2p[i].second;
    return CPPE_GPU_OK;
  });
}

// Batched solves: all (snapshot, right-hand side) segments in one
// concatenated geometry, one kernel launch per pass for all of them.
int cppe_gpu_batch_create(int nsys, const int* site_offset, const double* xyz,
                          const double* alpha6, const int* excl_ptr, const int* excl_idx,
                          int nrhs, int direct_below, const cppe_gpu_options* opts,
                          cppe_gpu_batch** out) {
  return guard([&]() -> int {
    need(out && opts && site_offset && xyz && alpha6 && nsys > 0 && nrhs > 0, "null argument");
    *out   = nullptr;
    auto h = std::make_unique<cppe_gpu_batch>();
    h->b.init(nsys, site_offset, xyz, alpha6, excl_ptr, excl_idx, nrhs, direct_below, *opts);
    *out = h.release();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_batch_destroy(cppe_gpu_batch* b) {
  return guard([&]() -> int {
    delete b;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_batch_solve_device(cppe_gpu_batch* bh, const double* d_rhs, double* d_mu,
                                int* iters) {
  return guard([&]() -> int {
    need(bh && d_rhs && d_mu, "null argument");
    return bh->b.solve_device(d_rhs, d_mu, iters);
  });
}

int cppe_gpu_batch_solve(cppe_gpu_batch* bh, const double* rhs, double* mu, int* iters) {
  return guard([&]() -> int {
    need(bh && rhs && mu, "null argument");
    BatchSystem& B  = bh->b;
    const size_t n3 = 3 * (size_t)B.n;
    CG_CUDA(cudaSetDevice(B.device));
    DBuf<double> dr, dm;
    dr.upload(rhs, n3, B.stream);
    dm.alloc(n3);
    int st = B.solve_device(dr.p, dm.p, iters);
    CG_CUDA(cudaMemcpyAsync(mu, dm.p, n3 * sizeof(double), cudaMemcpyDeviceToHost, B.stream));
    CG_CUDA(cudaStreamSynchronize(B.stream));
    return st;
  });
}

int cppe_gpu_batch_stats(cppe_gpu_batch* bh, int* fp64_applies, int* fp32_applies,
                         double* max_rnorm) {
  return guard([&]() -> int {
    need(bh, "null argument");
    BatchSystem& B = bh->b;
    if (fp64_applies) *fp64_applies = B.stats.fp64_applies;
    if (fp32_applies) *fp32_applies = B.stats.fp32_applies;
    if (max_rnorm)
      *max_rnorm = B.last_rnorm.empty()
                         ? 0.0
                         : *std::max_element(B.last_rnorm.begin(), B.last_rnorm.end());
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_batch_host_waits(cppe_gpu_batch* bh, int* waits) {
  return guard([&]() -> int {
    need(bh && waits, "null argument");
    *waits = bh->b.host_waits;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_batch_autotune(cppe_gpu_batch* bh, int reps, double* best_ms) {
  return guard([&]() -> int {
    need(bh && reps > 0, "null argument");
    const double ms = bh->b.autotune(reps);
    if (best_ms) *best_ms = ms;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_batch_stream(cppe_gpu_batch* bh, void** stream) {
  return guard([&]() -> int {
    need(bh && stream, "null argument");
    *stream = (void*)bh->b.stream;
    return CPPE_GPU_OK;
  });
}

// ---------------------------------------------------------------------------
// Learned initial guess / preconditioner: the MLP and its training data
// ---------------------------------------------------------------------------
int cppe_gpu_mlp_nparams(int* n) {
  if (!n) return CPPE_GPU_INVALID_ARG;
  *n = Mlp::NPARAM;
  return CPPE_GPU_OK;
}

int cppe_gpu_mlp_create(int device, unsigned seed, cppe_gpu_mlp** out) {
  return guard([&]() -> int {
    need(out, "null argument");
    *out   = nullptr;
    auto h = std::make_unique<cppe_gpu_mlp>();
    h->m.init(device, seed);
    *out = h.release();
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_destroy(cppe_gpu_mlp* m) {
  return guard([&]() -> int {
    delete m;
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_get_params(cppe_gpu_mlp* h, float* out) {
  return guard([&]() -> int {
    need(h && out, "null argument");
    CG_CUDA(cudaSetDevice(h->m.device));
    CG_CUDA(cudaMemcpy(out, h->m.params.p, Mlp::NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_set_params(cppe_gpu_mlp* h, const float* in) {
  return guard([&]() -> int {
    need(h && in, "null argument");
    CG_CUDA(cudaSetDevice(h->m.device));
    CG_CUDA(cudaMemcpy(h->m.params.p, in, Mlp::NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_normalization(cppe_gpu_mlp* h, const float* mean, const float* inv_std,
                               float* mean_out, float* inv_std_out) {
  return guard([&]() -> int {
    need(h, "null argument");
    CG_CUDA(cudaSetDevice(h->m.device));
    if (mean) CG_CUDA(cudaMemcpy(h->m.feat_mean.p, mean, Mlp::IN * 4, cudaMemcpyHostToDevice));
    if (inv_std)
      CG_CUDA(cudaMemcpy(h->m.feat_inv_std.p, inv_std, Mlp::IN * 4, cudaMemcpyHostToDevice));
    if (mean_out)
      CG_CUDA(cudaMemcpy(mean_out, h->m.feat_mean.p, Mlp::IN * 4, cudaMemcpyDeviceToHost));
    if (inv_std_out)
      CG_CUDA(cudaMemcpy(inv_std_out, h->m.feat_inv_std.p, Mlp::IN * 4, cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_forward(cppe_gpu_mlp* h, int rows, const float* feats, float* y) {
  return guard([&]() -> int {
    need(h && feats && y && rows > 0, "null argument");
    Mlp& M = h->m;
    CG_CUDA(cudaSetDevice(M.device));
    DBuf<float> f, yo;
    f.upload(feats, (size_t)rows * Mlp::IN, M.stream);
    yo.alloc((size_t)rows * Mlp::OUT);
    M.forward(rows, f.p, yo.p, M.stream);
    CG_CUDA(cudaMemcpyAsync(y, yo.p, (size_t)rows * Mlp::OUT * 4, cudaMemcpyDeviceToHost, M.stream));
    CG_CUDA(cudaStreamSynchronize(M.stream));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_infer(cppe_gpu_mlp* h, int rows, const float* feats, float* y) {
  return guard([&]() -> int {
    need(h && feats && y && rows > 0, "null argument");
    Mlp& M = h->m;
    CG_CUDA(cudaSetDevice(M.device));
    DBuf<float> f, yo;
    f.upload(feats, (size_t)rows * Mlp::IN, M.stream);
    yo.alloc((size_t)rows * Mlp::OUT);
    M.infer(rows, f.p, yo.p, M.stream);
    int e = 0;
    CG_CUDA(cudaMemcpyAsync(y, yo.p, (size_t)rows * Mlp::OUT * 4, cudaMemcpyDeviceToHost, M.stream));
    CG_CUDA(cudaMemcpyAsync(&e, M.tc_err.p, sizeof(int), cudaMemcpyDeviceToHost, M.stream));
    CG_CUDA(cudaStreamSynchronize(M.stream));
    if (e) fail(CPPE_GPU_TIMEOUT, "tensor-core MLP inference: a wait on the MMA barrier timed out");
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_mlp_loss_grad(cppe_gpu_mlp* h, int rows, const float* feats, const float* targets,
                           float lam, double* loss, float* grads) {
  return guard([&]() -> int {
    need(h && feats && targets && rows > 0, "null argument");
    Mlp& M = h->m;
    CG_CUDA(cudaSetDevice(M.device));
    DBuf<float> f, t;
    f.upload(feats, (size_t)rows * Mlp::IN, M.stream);
    t.upload(targets, (size_t)rows * Mlp::TROW, M.stream);
    const double l = M.loss_grad(rows, f.p, t.p, lam);
    if (loss) *loss = l;
    if (grads)
      CG_CUDA(cudaMemcpy(grads, M.grads.p, Mlp::NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return CPPE_GPU_OK;
  });
}

__global__ void k_gather_rows(int rows, int width, const int* __restrict__ idx,
                              const float* __restrict__ src, float* __restrict__ dst) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)rows * width) return;
  const int r = (int)(t / width), c = (int)(t % width);
  dst[t] = src[(size_t)idx[r] * width + c];
}

int cppe_gpu_mlp_train(cppe_gpu_mlp* h, int rows, const float* feats, const float* targets,
                       int steps, int batch, float lr, float lam, unsigned seed,
                       double* loss_hist) {
  return guard([&]() -> int {
    need(h && feats && targets && rows > 0 && steps >= 0 && batch > 0, "null argument");
    Mlp& M = h->m;
    CG_CUDA(cudaSetDevice(M.device));
    DBuf<float> f, t, fb, tb;
    DBuf<int> idx;
    f.upload(feats, (size_t)rows * Mlp::IN, M.stream);
    t.upload(targets, (size_t)rows * Mlp::TROW, M.stream);
    batch = std::min(batch, rows);
    fb.alloc((size_t)batch * Mlp::IN);
    tb.alloc((size_t)batch * Mlp::TROW);
    idx.alloc(batch);
    std::mt19937 rng(seed);
    std::uniform_int_distribution<int> pick(0, rows - 1);
    std::vector<int> ih(batch);
    for (int st = 0; st < steps; ++st) {
      for (int b = 0; b < batch; ++b) ih[b] = pick(rng);
      CG_CUDA(cudaMemcpyAsync(idx.p, ih.data(), batch * sizeof(int), cudaMemcpyHostToDevice,
                              M.stream));
      k_gather_rows<<<(unsigned)(((long)batch * Mlp::IN + 255) / 256), 256, 0, M.stream>>>(
            batch, Mlp::IN, idx.p, f.p, fb.p);
      CG_LAUNCH();
      k_gather_rows<<<(unsigned)(((long)batch * Mlp::TROW + 255) / 256), 256, 0, M.stream>>>(
            batch, Mlp::TROW, idx.p, t.p, tb.p);
      CG_LAUNCH();
      const double l = M.loss_grad(batch, fb.p, tb.p, lam);
      M.adam(lr);
      if (loss_hist) loss_hist[st] = l;
    }
    CG_CUDA(cudaStreamSynchronize(M.stream));
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_learned_data(cppe_gpu_system* sys, const double* rhs, const double* mu_star,
                          float* feats, float* rows) {
  return guard([&]() -> int {
    need(sys && rhs && mu_star && feats && rows, "null argument");
    System& S = sys->s;
    CG_CUDA(cudaSetDevice(S.device));
    const size_t n3 = 3 * (size_t)S.n;
    DBuf<double> dr, dm, dmp;
    dr.upload(rhs, n3, S.stream);
    dm.upload(mu_star, n3, S.stream);
    dmp.alloc(n3);
    permute_in(S.geo, dr.p, S.F.p, 3, S.stream);
    permute_in(S.geo, dm.p, dmp.p, 3, S.stream);
    std::vector<float> f, r;
    S.learned_rows(dmp.p, f, r);
    // weights of the loss terms, regularised by 1% of their system mean
    double ms = 0, mt = 0;
    for (int i = 0; i < S.n; ++i) ms += r[(size_t)i * Mlp::TROW + 21], mt += r[(size_t)i * Mlp::TROW + 22];
    ms /= S.n, mt /= S.n;
    for (int i = 0; i < S.n; ++i) {
      r[(size_t)i * Mlp::TROW + 21] += (float)(0.01 * ms + 1e-30);
      r[(size_t)i * Mlp::TROW + 22] += (float)(0.01 * mt + 1e-30);
    }
    std::copy(f.begin(), f.end(), feats);
    std::copy(r.begin(), r.end(), rows);
    return CPPE_GPU_OK;
  });
}

int cppe_gpu_set_model(cppe_gpu_system* sys, cppe_gpu_mlp* mlp) {
  return guard([&]() -> int {
    need(sys, "null argument");
    sys->s.model = mlp ? &mlp->m : nullptr;
    if (mlp) {
      CG_CUDA(cudaSetDevice(sys->s.device));
      sys->s.learned_setup();
      CG_CUDA(cudaStreamSynchronize(sys->s.stream));
    }
    return CPPE_GPU_OK;
  });
}

}  // extern "C"
