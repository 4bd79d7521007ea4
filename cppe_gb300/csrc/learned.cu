// Kernels of the learned initial guess / preconditioner correction.
#include <algorithm>
#include <cmath>

#include "learned.h"
#include "system.h"

namespace cg {

void NearGrid::build(const Geometry& g, const int* cep, const int* cei, cudaStream_t s) {
  n = g.n;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < n; ++k) {
    const double p[3] = {g.h_pos64[k].x, g.h_pos64[k].y, g.h_pos64[k].z};
    for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], p[c]), hi[c] = std::max(hi[c], p[c]);
  }
  for (int c = 0; c < 3; ++c) {
    origin[c] = lo[c];
    dims[c]   = std::max(1, (int)std::floor((hi[c] - lo[c]) / rc) + 1);
  }
  const long ncell = (long)dims[0] * dims[1] * dims[2];
  if (ncell > (1L << 28)) fail(CPPE_GPU_INVALID_ARG, "neighbour grid too large");
  std::vector<int> cnt(ncell + 1, 0), cell_of(n), sites(n);
  for (int k = 0; k < n; ++k) {
    const double p[3] = {g.h_pos64[k].x, g.h_pos64[k].y, g.h_pos64[k].z};
    int ci[3];
    for (int c = 0; c < 3; ++c)
      ci[c] = std::min(dims[c] - 1, std::max(0, (int)std::floor((p[c] - origin[c]) / rc)));
    cell_of[k] = (ci[2] * dims[1] + ci[1]) * dims[0] + ci[0];
    cnt[cell_of[k] + 1]++;
  }
  for (long c = 0; c < ncell; ++c) cnt[c + 1] += cnt[c];
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int k = 0; k < n; ++k) sites[fill[cell_of[k]]++] = k;
  std::vector<int> ep(n + 1, 0), ei;
  if (cep) {
    for (int k = 0; k < n; ++k) {
      const int i = g.layout.perm[k];
      for (int e = cep[i]; e < cep[i + 1]; ++e) {
        const int j = cei[e];
        if (j >= 0 && j < n && j != i) ei.push_back(g.layout.inv_perm[j]);
      }
      ep[k + 1] = (int)ei.size();
    }
  }
  if (ei.empty()) ei.push_back(-1);
  cell_start.upload(cnt, s);
  cell_site.upload(sites, s);
  excl_ptr.upload(ep, s);
  excl_idx.upload(ei, s);
}

NearGridView view(const NearGrid& g) {
  return NearGridView{g.n,       g.rc,         g.origin[0],     g.origin[1],     g.origin[2],
                      g.dims[0], g.dims[1],    g.dims[2],       g.cell_start.p,  g.cell_site.p,
                      g.excl_ptr.p, g.excl_idx.p};
}

// Visits the neighbours j != i within rc of site i (27 grid cells).
template <class F>
__device__ __forceinline__ void for_neighbours(const NearGridView& ng, const double4_32a* pos,
                                               int i, F&& f) {
  const double4_32a pi = pos[i];
  const int cx = min(ng.dx - 1, max(0, (int)floor((pi.x - ng.ox) / ng.rc)));
  const int cy = min(ng.dy - 1, max(0, (int)floor((pi.y - ng.oy) / ng.rc)));
  const int cz = min(ng.dz - 1, max(0, (int)floor((pi.z - ng.oz) / ng.rc)));
  const double rc2 = ng.rc * ng.rc;
  for (int zz = max(0, cz - 1); zz <= min(ng.dz - 1, cz + 1); ++zz)
    for (int yy = max(0, cy - 1); yy <= min(ng.dy - 1, cy + 1); ++yy)
      for (int xx = max(0, cx - 1); xx <= min(ng.dx - 1, cx + 1); ++xx) {
        const int c = (zz * ng.dy + yy) * ng.dx + xx;
        for (int q = ng.cell_start[c]; q < ng.cell_start[c + 1]; ++q) {
          const int j = ng.cell_site[q];
          if (j == i) continue;
          const double4_32a pj = pos[j];
          const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
          const double r2 = dx * dx + dy * dy + dz * dz;
          if (r2 >= rc2) continue;
          f(j, (float)dx, (float)dy, (float)dz, pj.w);
        }
      }
}

__device__ __forceinline__ float aiso6(const float* a) { return (a[0] + a[3] + a[5]) / 3.f; }

__global__ void k_features(NearGridView ng, const double4_32a* __restrict__ pos,
                           const float* __restrict__ a6, const double* __restrict__ F,
                           float* __restrict__ feats, float* __restrict__ v1) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ng.n) return;
  const float* ai = a6 + 6 * (size_t)i;
  const float f0 = (float)F[3 * i], f1 = (float)F[3 * i + 1], f2 = (float)F[3 * i + 2];
  v1[3 * i]     = ai[0] * f0 + ai[1] * f1 + ai[2] * f2;
  v1[3 * i + 1] = ai[1] * f0 + ai[3] * f1 + ai[4] * f2;
  v1[3 * i + 2] = ai[2] * f0 + ai[4] * f1 + ai[5] * f2;
  const float fn  = sqrtf(f0 * f0 + f1 * f1 + f2 * f2);
  const float ifn = fn > 0.f ? 1.f / fn : 0.f;
  const float ux = f0 * ifn, uy = f1 * ifn, uz = f2 * ifn;
  float f[Mlp::IN];
#pragma unroll
  for (int k = 0; k < Mlp::IN; ++k) f[k] = 0.f;
  const float rc = (float)ng.rc;
  const float w16 = (rc - 1.f) / 15.f, w8 = (rc - 1.f) / 7.f;
  int count = 0;
  for_neighbours(ng, pos, i, [&](int j, float dx, float dy, float dz, double) {
    const float r  = sqrtf(dx * dx + dy * dy + dz * dz);
    const float fc = 0.5f * (__cosf(3.14159265f * r / rc) + 1.f);
    const float aj = aiso6(a6 + 6 * (size_t)j) * 0.25f;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const float t = (r - (1.f + k * w16)) / w16;
      const float g = __expf(-t * t) * fc;
      f[1 + k] += g;
      f[17 + k] += aj * g;
    }
    const float ct = (ux * dx + uy * dy + uz * dz) / r;
    const float p2 = 1.5f * ct * ct - 0.5f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const float t = (r - (1.f + k * w8)) / w8;
      const float g = __expf(-t * t) * fc;
      f[33 + k] += g * ct;
      f[41 + k] += g * p2;
      f[55 + k] += g * ct * aj;
    }
    ++count;
  });
  f[0]  = aiso6(ai) * 0.25f - 1.f;
  f[63] = count * 0.01f;
  float* o = feats + (size_t)i * Mlp::IN;
#pragma unroll
  for (int k = 0; k < Mlp::IN; ++k)
    if (k < 49 || k > 54) o[k] = f[k];
}

template <typename T>
__global__ void k_near_T(NearGridView ng, const double4_32a* __restrict__ pos,
                         const T* __restrict__ a6, int damp, T damping, const T* __restrict__ in,
                         T* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ng.n) return;
  const T ai = damping * (T)pos[i].w;
  const int e0 = ng.excl_ptr[i], e1 = ng.excl_ptr[i + 1];
  T fx = 0, fy = 0, fz = 0;
  for_neighbours(ng, pos, i, [&](int j, float, float, float, double sj) {
    for (int e = e0; e < e1; ++e)
      if (ng.excl_idx[e] == j) return;
    const double4_32a pi = pos[i], pj = pos[j];
    const T x = (T)(pi.x - pj.x), y = (T)(pi.y - pj.y), z = (T)(pi.z - pj.z);
    T G[2];
    radial<T, 2>(x * x + y * y + z * z, damp ? ai * (T)sj : T(0), G);
    // field_m1 returns -T v; accumulate T v
    T gx = 0, gy = 0, gz = 0;
    field_m1(x, y, z, G, in[3 * j], in[3 * j + 1], in[3 * j + 2], gx, gy, gz);
    fx -= gx, fy -= gy, fz -= gz;
  });
  const T* a = a6 + 6 * (size_t)i;
  out[3 * i]     = a[0] * fx + a[1] * fy + a[2] * fz;
  out[3 * i + 1] = a[1] * fx + a[3] * fy + a[4] * fz;
  out[3 * i + 2] = a[2] * fx + a[4] * fy + a[5] * fz;
}

__global__ void k_basis_features(int n, const float* __restrict__ v1, const float* __restrict__ v2,
                                 const float* __restrict__ v3, float* __restrict__ feats) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* a = v1 + 3 * i;
  const float* b = v2 + 3 * i;
  const float* c = v3 + 3 * i;
  const float na = sqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  const float nb = sqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  const float nc = sqrtf(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
  const float ia = na > 0.f ? 1.f / na : 0.f, ib = nb > 0.f ? 1.f / nb : 0.f,
              ic = nc > 0.f ? 1.f / nc : 0.f;
  const float ab = (a[0] * b[0] + a[1] * b[1] + a[2] * b[2]) * ia * ib;
  const float ac = (a[0] * c[0] + a[1] * c[1] + a[2] * c[2]) * ia * ic;
  const float bc = (b[0] * c[0] + b[1] * c[1] + b[2] * c[2]) * ib * ic;
  float* o = feats + (size_t)i * Mlp::IN;
  o[49] = nb * ia;
  o[50] = nc * ia;
  o[51] = ab;
  o[52] = ac;
  o[53] = bc;
  o[54] = nb * ia * sqrtf(fmaxf(0.f, 1.f - ab * ab));
}

__global__ void k_guess(int n, const float* __restrict__ Y, const float* __restrict__ v1,
                        const float* __restrict__ v2, const float* __restrict__ v3,
                        double* __restrict__ x, float* __restrict__ c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float* y = Y + (size_t)Mlp::OUT * i;
  for (int q = 0; q < 3; ++q)
    x[3 * i + q] = (double)y[0] * v1[3 * i + q] + (double)y[1] * v2[3 * i + q] +
                   (double)y[2] * v3[3 * i + q];
  c[i] = y[3];
}

template <typename T>
__global__ void k_precond_fix(int n, T* __restrict__ z, const T* __restrict__ w,
                              const float* __restrict__ cw, const T* __restrict__ r,
                              const T* __restrict__ r_old, T* __restrict__ p, int start,
                              ReduceSlots rs, double* scal, const int* flags) {
  __shared__ double sh[64];
  if (!start && flags[0]) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double v[2] = {0.0, 0.0};
  if (i < n) {
    const T c = (T)cw[i];
    for (int q = 0; q < 3; ++q) {
      const size_t k = 3 * (size_t)i + q;
      const T zk     = z[k] + c * w[k];
      z[k]           = zk;
      if (start) p[k] = zk;
      v[0] += (double)zk * r[k];
      if (!start) v[1] += (double)zk * r_old[k];
    }
  }
  if (grid_sum_last<2>(v, sh, rs.partials, rs.ticket, rs.out)) {
    if (!start) scal[S_BETA] = (rs.out[0] - rs.out[1]) / scal[S_RZOLD];
    scal[S_RZ] = rs.out[0];
  }
}

void learned_features(const NearGridView& ng, const double4_32a* pos, const float* a6f,
                      const double* F, float* feats, float* v1, cudaStream_t s) {
  k_features<<<(ng.n + 127) / 128, 128, 0, s>>>(ng, pos, a6f, F, feats, v1);
  CG_LAUNCH();
}

template <typename T>
void near_T(const NearGridView& ng, const double4_32a* pos, const T* a6, int damp, double damping,
            const T* in, T* out, cudaStream_t s) {
  k_near_T<T><<<(ng.n + 127) / 128, 128, 0, s>>>(ng, pos, a6, damp, (T)damping, in, out);
  CG_LAUNCH();
}
template void near_T<float>(const NearGridView&, const double4_32a*, const float*, int, double,
                            const float*, float*, cudaStream_t);
template void near_T<double>(const NearGridView&, const double4_32a*, const double*, int, double,
                             const double*, double*, cudaStream_t);

void learned_basis_features(int n, const float* v1, const float* v2, const float* v3,
                            float* feats, cudaStream_t s) {
  k_basis_features<<<(n + 255) / 256, 256, 0, s>>>(n, v1, v2, v3, feats);
  CG_LAUNCH();
}

void learned_guess(int n, const float* Y, const float* v1, const float* v2, const float* v3,
                   double* x, float* c, cudaStream_t s) {
  k_guess<<<(n + 255) / 256, 256, 0, s>>>(n, Y, v1, v2, v3, x, c);
  CG_LAUNCH();
}

template <typename T>
void precond_fix(int n, T* z, const T* w, const float* c, const T* r, const T* r_old, T* p,
                 bool start, double* partials, unsigned* ticket, double* scal, const int* flags,
                 cudaStream_t s) {
  ReduceSlots rs{partials, ticket, scal + S_RED};
  k_precond_fix<T><<<(n + 255) / 256, 256, 0, s>>>(n, z, w, c, r, r_old, p, start ? 1 : 0, rs,
                                                   scal, flags);
  CG_LAUNCH();
}
template void precond_fix<float>(int, float*, const float*, const float*, const float*,
                                 const float*, float*, bool, double*, unsigned*, double*,
                                 const int*, cudaStream_t);
template void precond_fix<double>(int, double*, const double*, const float*, const double*,
                                  const double*, double*, bool, double*, unsigned*, double*,
                                  const int*, cudaStream_t);

}  // namespace cg
