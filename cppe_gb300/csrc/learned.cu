// Kernels of the learned initial guess / preconditioner correction.
#include <algorithm>
#include <cmath>

#include <cub/device/device_segmented_sort.cuh>

#include "learned.h"
#include "system.h"

namespace cg {

// ---------------------------------------------------------------------------
// Neighbour lists: sites are binned on the host into cubic cells of edge rc;
// a thread per site scans the 27 cells around its own twice on the GPU (count,
// then fill), with FP32 separations from the grid-snapped hi/lo coordinates.
// ---------------------------------------------------------------------------
struct CellGridView {
  int dx, dy, dz;
  const int* cell_start;
  const int* cell_site;
  const int* site_cell;
  const int* excl_ptr;  // device-order exclusions
  const int* excl_idx;
};

template <bool FILL>
__global__ void k_near_build(int n, CellGridView cgv, const float4* __restrict__ hi,
                             const float4* __restrict__ lo, float rc2, int damp, float damping,
                             int* __restrict__ count, const int* __restrict__ ptr,
                             int* __restrict__ idx, __half* __restrict__ t6,
                             float4* __restrict__ d) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 hi_i = hi[i], lo_i = lo[i];
  const int c  = cgv.site_cell[i];
  const int cx = c % cgv.dx, cy = (c / cgv.dx) % cgv.dy, cz = c / (cgv.dx * cgv.dy);
  const int e0 = cgv.excl_ptr[i], e1 = cgv.excl_ptr[i + 1];
  const float ai = damping * hi_i.w;
  int k = FILL ? ptr[i] : 0;
  for (int zz = max(0, cz - 1); zz <= min(cgv.dz - 1, cz + 1); ++zz)
    for (int yy = max(0, cy - 1); yy <= min(cgv.dy - 1, cy + 1); ++yy)
      for (int xx = max(0, cx - 1); xx <= min(cgv.dx - 1, cx + 1); ++xx) {
        const int cc = (zz * cgv.dy + yy) * cgv.dx + xx;
        for (int q = cgv.cell_start[cc]; q < cgv.cell_start[cc + 1]; ++q) {
          const int j = cgv.cell_site[q];
          if (j == i) continue;
          const float4 hj = hi[j], lj = lo[j];
          const float x = (hj.x - hi_i.x) + (lj.x - lo_i.x);
          const float y = (hj.y - hi_i.y) + (lj.y - lo_i.y);
          const float z = (hj.z - hi_i.z) + (lj.z - lo_i.z);
          const float r2 = x * x + y * y + z * z;
          if (r2 >= rc2) continue;
          // excluded partners stay in the list (the descriptors see them) with
          // a zero tensor (the operator skips them)
          bool excluded = false;
          for (int e = e0; e < e1; ++e) excluded |= cgv.excl_idx[e] == j;
          if (FILL) {
            float G[2];
            radial<float, 2>(r2, damp ? ai * hj.w : 0.f, G);
            if (excluded) G[0] = G[1] = 0.f;
            idx[k] = j;
            __half* t = t6 + 6 * (size_t)k;
            t[0] = __float2half(G[0] + G[1] * x * x), t[1] = __float2half(G[1] * x * y);
            t[2] = __float2half(G[1] * x * z), t[3] = __float2half(G[0] + G[1] * y * y);
            t[4] = __float2half(G[1] * y * z), t[5] = __float2half(G[0] + G[1] * z * z);
            d[k] = make_float4(x, y, z, sqrtf(r2));
          }
          ++k;
        }
      }
  if (!FILL) count[i] = k;
}

__global__ void k_iota(long n, int* __restrict__ v) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) v[k] = (int)k;
}

// Entry k of the sorted lists from entry perm[k] of the scan order; the
// packed operator entries alongside.
__global__ void k_near_permute(long nnz, const int* __restrict__ perm, const int* __restrict__ idx,
                               const __half* __restrict__ t6_in, const float4* __restrict__ d_in,
                               __half* __restrict__ t6, float4* __restrict__ d,
                               int4* __restrict__ ent) {
  const long k = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nnz) return;
  const long q = perm[k];
  const __half2* h = reinterpret_cast<const __half2*>(t6_in + 6 * q);
  __half2* o       = reinterpret_cast<__half2*>(t6 + 6 * k);
  const __half2 a = h[0], b = h[1], c = h[2];
  o[0] = a, o[1] = b, o[2] = c;
  d[k] = d_in[q];
  int4 e;
  e.x    = idx[k];
  e.y    = *reinterpret_cast<const int*>(&a);
  e.z    = *reinterpret_cast<const int*>(&b);
  e.w    = *reinterpret_cast<const int*>(&c);
  ent[k] = e;
}

void NearList::build(const Geometry& g, const int* cep, const int* cei, int damp,
                     double damping, cudaStream_t s) {
  n = g.n;
  const double rc = LEARN_RC;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int k = 0; k < n; ++k) {
    const double p[3] = {g.h_pos64[k].x, g.h_pos64[k].y, g.h_pos64[k].z};
    for (int c = 0; c < 3; ++c) lo[c] = std::min(lo[c], p[c]), hi[c] = std::max(hi[c], p[c]);
  }
  int dims[3];
  for (int c = 0; c < 3; ++c) dims[c] = std::max(1, (int)std::floor((hi[c] - lo[c]) / rc) + 1);
  const long ncell = (long)dims[0] * dims[1] * dims[2];
  if (ncell > (1L << 28)) fail(CPPE_GPU_INVALID_ARG, "neighbour grid too large");
  std::vector<int> cnt(ncell + 1, 0), cell_of(n), sites(n);
  for (int k = 0; k < n; ++k) {
    const double p[3] = {g.h_pos64[k].x, g.h_pos64[k].y, g.h_pos64[k].z};
    int ci[3];
    for (int c = 0; c < 3; ++c)
      ci[c] = std::min(dims[c] - 1, std::max(0, (int)std::floor((p[c] - lo[c]) / rc)));
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
  DBuf<int> d_cell_start, d_cell_site, d_site_cell, d_ep, d_ei, d_count;
  d_cell_start.upload(cnt, s);
  d_cell_site.upload(sites, s);
  d_site_cell.upload(cell_of, s);
  d_ep.upload(ep, s);
  d_ei.upload(ei, s);
  d_count.alloc(std::max(1, n));
  const CellGridView cv{dims[0], dims[1], dims[2], d_cell_start.p, d_cell_site.p,
                        d_site_cell.p, d_ep.p, d_ei.p};
  const float rc2 = (float)(rc * rc);
  const int nb    = (n + 127) / 128;
  if (n > 0) {
    k_near_build<false><<<nb, 128, 0, s>>>(n, cv, g.hi32.p, g.lo32.p, rc2, damp, (float)damping,
                                           d_count.p, nullptr, nullptr, nullptr, nullptr);
    CG_LAUNCH();
  }
  std::vector<int> c_h(n), p_h(n + 1, 0);
  if (n > 0)
    CG_CUDA(cudaMemcpyAsync(c_h.data(), d_count.p, n * sizeof(int), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i) p_h[i + 1] = p_h[i] + c_h[i];
  nnz = p_h[n];
  ptr.upload(p_h, s);
  idx.alloc(std::max(1L, nnz));
  t6.alloc(6 * std::max(1L, nnz));
  d.alloc(std::max(1L, nnz));
  DBuf<int> idx0, perm0, perm;
  DBuf<__half> t60;
  DBuf<float4> d0;
  idx0.alloc(std::max(1L, nnz));
  t60.alloc(6 * std::max(1L, nnz));
  d0.alloc(std::max(1L, nnz));
  ent.alloc(std::max(1L, nnz));
  if (n > 0) {
    k_near_build<true><<<nb, 128, 0, s>>>(n, cv, g.hi32.p, g.lo32.p, rc2, damp, (float)damping,
                                          nullptr, ptr.p, idx0.p, t60.p, d0.p);
    CG_LAUNCH();
  }
  if (nnz > 0) {
    // every site's entries in ascending partner order, so that the eight
    // lanes serving a site gather neighbouring partners (shared cache lines)
    perm0.alloc(nnz);
    perm.alloc(nnz);
    k_iota<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, perm0.p);
    CG_LAUNCH();
    size_t tmp_bytes = 0;
    CG_CUDA(cub::DeviceSegmentedSort::SortPairs(nullptr, tmp_bytes, idx0.p, idx.p, perm0.p, perm.p,
                                                nnz, n, ptr.p, ptr.p + 1, s));
    DBuf<unsigned char> tmp;
    tmp.alloc(std::max<size_t>(1, tmp_bytes));
    CG_CUDA(cub::DeviceSegmentedSort::SortPairs(tmp.p, tmp_bytes, idx0.p, idx.p, perm0.p, perm.p,
                                                nnz, n, ptr.p, ptr.p + 1, s));
    k_near_permute<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, perm.p, idx.p, t60.p, d0.p,
                                                                 t6.p, d.p, ent.p);
    CG_LAUNCH();
    CG_CUDA(cudaStreamSynchronize(s));  // the temporaries above are freed on return
  }
  CG_CUDA(cudaStreamSynchronize(s));
}

NearListView view(const NearList& g) {
  return NearListView{g.n, g.ptr.p, g.idx.p, g.t6.p, g.d.p, g.ent.p};
}

__device__ __forceinline__ float aiso6(const float* a) { return (a[0] + a[3] + a[5]) / 3.f; }

// Descriptors: eight lanes per site stride over its neighbour list and the
// partial sums are reduced by shuffles.
__global__ void k_features(NearListView nl, const float* __restrict__ a6,
                           const double* __restrict__ F, float* __restrict__ feats,
                           float* __restrict__ v1) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gid >> 3, sub = gid & 7;
  const bool ok = i < nl.n;
  const int ii  = ok ? i : 0;
  const float* ai = a6 + 6 * (size_t)ii;
  const float f0 = (float)F[3 * ii], f1 = (float)F[3 * ii + 1], f2 = (float)F[3 * ii + 2];
  const float fn  = sqrtf(f0 * f0 + f1 * f1 + f2 * f2);
  const float ifn = fn > 0.f ? 1.f / fn : 0.f;
  const float ux = f0 * ifn, uy = f1 * ifn, uz = f2 * ifn;
  float f[Mlp::IN];
#pragma unroll
  for (int k = 0; k < Mlp::IN; ++k) f[k] = 0.f;
  const float rc = (float)LEARN_RC;
  // Gaussian q of a family of width w centred at 1 + q w: its argument
  // (r - 1 - q w) / w is t0 - q with t0 = (r - 1) / w
  const float iw16 = 15.f / (rc - 1.f), iw8 = 7.f / (rc - 1.f);
  const int k0 = ok ? nl.ptr[ii] : 0, k1 = ok ? nl.ptr[ii + 1] : 0;
  // the next entry's loads (and its dependent polarizability gather) are
  // issued before this entry's arithmetic, which hides their latency
  float4 dv_n = make_float4(0.f, 0.f, 0.f, 1.f);
  float aj_n  = 0.f;
  if (k0 + sub < k1) {
    dv_n = nl.d[k0 + sub];
    aj_n = aiso6(a6 + 6 * (size_t)nl.idx[k0 + sub]);
  }
  for (int k = k0 + sub; k < k1; k += 8) {
    const float4 dv = dv_n;
    const float aj  = aj_n * 0.25f;
    if (k + 8 < k1) {
      dv_n = nl.d[k + 8];
      aj_n = aiso6(a6 + 6 * (size_t)nl.idx[k + 8]);
    }
    const float r   = dv.w;
    const float fc  = 0.5f * (__cosf(3.14159265f * r / rc) + 1.f);
    const float t16 = (r - 1.f) * iw16, t8 = (r - 1.f) * iw8;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const float t = t16 - (float)q;
      const float g = __expf(-t * t) * fc;
      f[1 + q] += g;
      f[17 + q] += aj * g;
    }
    const float ct = (ux * dv.x + uy * dv.y + uz * dv.z) / r;
    const float p2 = 1.5f * ct * ct - 0.5f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const float t = t8 - (float)q;
      const float g = __expf(-t * t) * fc;
      f[33 + q] += g * ct;
      f[41 + q] += g * p2;
      f[55 + q] += g * ct * aj;
    }
  }
#pragma unroll
  for (int k = 1; k < 63; ++k) {
    if (k >= 49 && k <= 54) continue;
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) f[k] += __shfl_down_sync(0xffffffffu, f[k], o, 8);
  }
  if (!ok || sub != 0) return;
  v1[3 * i]     = ai[0] * f0 + ai[1] * f1 + ai[2] * f2;
  v1[3 * i + 1] = ai[1] * f0 + ai[3] * f1 + ai[4] * f2;
  v1[3 * i + 2] = ai[2] * f0 + ai[4] * f1 + ai[5] * f2;
  f[0]  = aiso6(ai) * 0.25f - 1.f;
  f[63] = (k1 - k0) * 0.01f;
  float* o = feats + (size_t)i * Mlp::IN;
#pragma unroll
  for (int k = 0; k < Mlp::IN; ++k)
    if (k < 49 || k > 54) o[k] = f[k];
}

// Lane `sub` of eight: its share of sum_j T_ij in_j over site i's entries,
// NB entries per step with their loads issued together (the loop is bound
// by the latency of the entry load and the dependent gather; about 90
// entries per site make two steps of eight).
template <typename T>
__device__ __forceinline__ void near_T_lane(const NearListView& nl, int i, int sub,
                                            const T* __restrict__ in, T& wx, T& wy, T& wz,
                                            const float4* __restrict__ in4 = nullptr) {
  constexpr int NB = 8;
  const int k0 = nl.ptr[i] + sub, k1 = nl.ptr[i + 1];
  for (int k = k0; k < k1; k += 8 * NB) {
    int4 e[NB];
#pragma unroll
    for (int u = 0; u < NB; ++u) e[u] = k + 8 * u < k1 ? nl.ent[k + 8 * u] : make_int4(-1, 0, 0, 0);
    T v[NB][3];
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int j = e[u].x;
      if (in4) {
        const float4 q = j >= 0 ? in4[j] : make_float4(0.f, 0.f, 0.f, 0.f);
        v[u][0] = (T)q.x, v[u][1] = (T)q.y, v[u][2] = (T)q.z;
      } else {
        v[u][0] = j >= 0 ? in[3 * (size_t)j] : T(0);
        v[u][1] = j >= 0 ? in[3 * (size_t)j + 1] : T(0);
        v[u][2] = j >= 0 ? in[3 * (size_t)j + 2] : T(0);
      }
    }
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&e[u].y));
      const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&e[u].z));
      const float2 c = __half22float2(*reinterpret_cast<const __half2*>(&e[u].w));
      wx += (T)a.x * v[u][0] + (T)a.y * v[u][1] + (T)b.x * v[u][2];
      wy += (T)a.y * v[u][0] + (T)b.y * v[u][1] + (T)c.x * v[u][2];
      wz += (T)b.x * v[u][0] + (T)c.x * v[u][1] + (T)c.y * v[u][2];
    }
  }
}

// out_i = alpha_i sum_j T_ij in_j: eight lanes per site stride over its list
// (coalesced reads of the stored tensors), then a shuffle reduction.
template <typename T>
__global__ void k_near_T(NearListView nl, const T* __restrict__ a6, const T* __restrict__ in,
                         T* __restrict__ out) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gid >> 3, sub = gid & 7;
  T fx = 0, fy = 0, fz = 0;
  if (i < nl.n) {
    near_T_lane<T>(nl, i, sub, in, fx, fy, fz);
  }
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) {
    fx += __shfl_down_sync(0xffffffffu, fx, o, 8);
    fy += __shfl_down_sync(0xffffffffu, fy, o, 8);
    fz += __shfl_down_sync(0xffffffffu, fz, o, 8);
  }
  if (i < nl.n && sub == 0) {
    const T* a     = a6 + 6 * (size_t)i;
    out[3 * i]     = a[0] * fx + a[1] * fy + a[2] * fz;
    out[3 * i + 1] = a[1] * fx + a[3] * fy + a[4] * fz;
    out[3 * i + 2] = a[2] * fx + a[4] * fy + a[5] * fz;
  }
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
__global__ void k_precond_near(NearListView nl, const T* __restrict__ a6,
                               const float* __restrict__ cw, const T* __restrict__ a,
                               const T* __restrict__ r, const T* __restrict__ r_old,
                               T* __restrict__ zc, T* __restrict__ p, int start, ReduceSlots rs,
                               double* scal, const int* flags, const float4* __restrict__ a4) {
  __shared__ double sh[64];
  if (!start && flags[0]) return;
  T v[2] = {T(0), T(0)};  // (FP32 products for the FP32 solve: see block_sum)
  // a grid of a few blocks per SM striding over the sites: fewer partial
  // sums (and tickets) for the grid reduction than a block per 16 sites
  const int per_block = blockDim.x >> 3;
  for (int base = blockIdx.x * per_block; base < nl.n; base += gridDim.x * per_block) {
  const int i = base + (threadIdx.x >> 3), sub = threadIdx.x & 7;
  T wx = 0, wy = 0, wz = 0;
  if (i < nl.n) {
    near_T_lane<T>(nl, i, sub, a, wx, wy, wz, a4);
  }
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) {
    wx += __shfl_down_sync(0xffffffffu, wx, o, 8);
    wy += __shfl_down_sync(0xffffffffu, wy, o, 8);
    wz += __shfl_down_sync(0xffffffffu, wz, o, 8);
  }
  if (i < nl.n && sub == 0) {
    const T* al = a6 + 6 * (size_t)i;
    const T c   = (T)cw[i];
    const T w[3] = {al[0] * wx + al[1] * wy + al[2] * wz, al[1] * wx + al[3] * wy + al[4] * wz,
                    al[2] * wx + al[4] * wy + al[5] * wz};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const size_t k = 3 * (size_t)i + q;
      const T zk     = a[k] + c * w[q];
      zc[k]          = zk;
      if (start) p[k] = zk;
      v[0] += zk * r[k];
      if (!start) v[1] += zk * r_old[k];
    }
  }
  }
  if (grid_sum_last<2>(v, sh, rs.partials, rs.ticket, rs.out)) {
    if (!start) scal[S_BETA] = (rs.out[0] - rs.out[1]) / scal[S_RZOLD];
    scal[S_RZ] = rs.out[0];
  }
}

void learned_features(const NearListView& nl, const float* a6f, const double* F, float* feats,
                      float* v1, cudaStream_t s) {
  const long threads = 8L * nl.n;
  k_features<<<(unsigned)((threads + 127) / 128), 128, 0, s>>>(nl, a6f, F, feats, v1);
  CG_LAUNCH();
}

template <typename T>
void near_T(const NearListView& nl, const T* a6, const T* in, T* out, cudaStream_t s) {
  const long threads = 8L * nl.n;
  k_near_T<T><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(nl, a6, in, out);
  CG_LAUNCH();
}
template void near_T<float>(const NearListView&, const float*, const float*, float*,
                            cudaStream_t);
template void near_T<double>(const NearListView&, const double*, const double*, double*,
                             cudaStream_t);

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

constexpr long PRECOND_BLOCKS = 4 * 152;  // 4 per SM of a GB300 (grid stride beyond)
template <typename T>
void precond_near(const NearListView& nl, const T* a6, const float* c, const T* a, const T* r,
                  const T* r_old, T* zc, T* p, bool start, double* partials, unsigned* ticket,
                  double* scal, const int* flags, cudaStream_t s, const float4* a4) {
  ReduceSlots rs{partials, ticket, scal + S_RED};
  const long blocks = std::min<long>((8L * nl.n + 127) / 128, PRECOND_BLOCKS);
  k_precond_near<T><<<(unsigned)std::max(1L, blocks), 128, 0, s>>>(
        nl, a6, c, a, r, r_old, zc, p, start ? 1 : 0, rs, scal, flags, a4);
  CG_LAUNCH();
}
template void precond_near<float>(const NearListView&, const float*, const float*, const float*,
                                  const float*, const float*, float*, float*, bool, double*,
                                  unsigned*, double*, const int*, cudaStream_t, const float4*);
template void precond_near<double>(const NearListView&, const double*, const float*,
                                   const double*, const double*, const double*, double*, double*,
                                   bool, double*, unsigned*, double*, const int*, cudaStream_t,
                                   const float4*);

}  // namespace cg
