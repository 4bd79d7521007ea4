// Field engine kernels: near-field pair sums (direct summation and FMM P2P),
// the FMM passes (P2M, M2M, M2L, L2L, L2P) and the finishing pass.
//
// Reference counterparts (maxscheurer/cppe, src/core/fmm/):
//   k_p2p      evaluate_direct{,_damping} calculate.cc:262-300,
//              evaluate_P2P_lazy + P2P_Cells{,_damping} calculate.cc:29-72,205-225
//   k_p2m      evaluate_P2M  calculate.cc:129-157
//   k_m2m      evaluate_M2M  calculate.cc:159-184
//   k_m2l      evaluate_M2L_lazy calculate.cc:186-203
//   k_l2l      evaluate_L2L  calculate.cc:227-243
//   k_finish   evaluate_L2P  calculate.cc:245-260, the exclusion rule of
//              P2P_Cells (calculate.cc:37), and BMatrix::apply's "+ alpha^-1 mu"
//              (bmatrix.cc:39)
// Every output element is owned by exactly one thread (no atomics), so
// results are bitwise reproducible run to run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "engine.h"
#include "dd.cuh"
#include "m2l_fixed.cuh"

namespace cg {

constexpr int P2P_BLOCK  = 128;
constexpr int P2P_TILE   = 512;  // source sites staged in shared memory per tile
constexpr int M2L_WARPS  = 4;

// ---------------------------------------------------------------------------
// Table uploads
// ---------------------------------------------------------------------------
void DeviceOps::build(int m, int p, cudaStream_t s) {
  host = make_op_tables(m, p);
  exps.upload(host.exps, s);
  p2m_ptr.upload(host.p2m_ptr, s), p2m_k.upload(host.p2m_k, s), p2m_j.upload(host.p2m_j, s);
  m2m_ptr.upload(host.m2m_ptr, s), m2m_k.upload(host.m2m_k, s), m2m_j.upload(host.m2m_j, s);
  l2l_ptr.upload(host.l2l_ptr, s), l2l_k.upload(host.l2l_k, s), l2l_j.upload(host.l2l_j, s);
  l2p_c.upload(host.l2p_c, s), l2p_n.upload(host.l2p_n, s), l2p_j.upload(host.l2p_j, s);
  std::vector<int> kw(host.m2l_k.size());
  for (size_t t = 0; t < kw.size(); ++t) kw[t] = host.m2l_k[t] | (host.m2l_w[t] << 16);
  m2l_kw.upload(kw, s);
  slots.upload(host.slots, s);
  row_slot_ptr.upload(host.row_slot_ptr, s), row_slot_id.upload(host.row_slot_id, s);
  drec.upload(host.drec, s);
}

OpsView DeviceOps::view() const {
  OpsView v;
  v.m = host.m, v.p = host.p, v.msize = host.msize, v.lsize = host.lsize, v.nt = host.nt;
  v.nm2l_terms = (int)host.m2l_k.size();
  v.nl2p       = (int)host.l2p_c.size();
  v.exps       = exps.p;
  v.p2m_ptr = p2m_ptr.p, v.p2m_k = p2m_k.p, v.p2m_j = p2m_j.p;
  v.m2m_ptr = m2m_ptr.p, v.m2m_k = m2m_k.p, v.m2m_j = m2m_j.p;
  v.l2l_ptr = l2l_ptr.p, v.l2l_k = l2l_k.p, v.l2l_j = l2l_j.p;
  v.l2p_c = l2p_c.p, v.l2p_n = l2p_n.p, v.l2p_j = l2p_j.p;
  v.m2l_kw = m2l_kw.p, v.slots = slots.p, v.row_slot_ptr = row_slot_ptr.p;
  v.row_slot_id = row_slot_id.p, v.drec = drec.p;
  return v;
}

TreeView Geometry::view() const {
  TreeView v;
  v.n = n, v.ncells = layout.ncells, v.nleaves = layout.nleaves;
  v.center    = reinterpret_cast<const double4_32a*>(center.p);
  v.parent    = parent.p, v.child_ptr = child_ptr.p, v.child_idx = child_idx.p;
  v.is_leaf   = is_leaf.p, v.leaf_cell = leaf_cell.p, v.leaf_start = leaf_start.p;
  v.site_leaf = site_leaf.p, v.m2l_ptr = m2l_ptr.p, v.m2l_src = m2l_src.p;
  v.p2p_ptr = p2p_ptr.p, v.p2p_src = p2p_src.p;
  return v;
}

// ---------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------
void Geometry::build(int n_, const double* xyz, const double* s_damp, const int* excl_ptr,
                     const int* excl_idx, bool fmm_, int ncrit_, double theta_,
                     cudaStream_t s) {
  prepare(n_, xyz, s_damp, excl_ptr, excl_idx, fmm_, ncrit_, theta_);
  upload(s);
}

void Geometry::prepare(int n_, const double* xyz, const double* s_damp, const int* excl_ptr,
                       const int* excl_idx, bool fmm_, int ncrit_, double theta_) {
  n     = n_;
  fmm   = fmm_;
  ncrit = ncrit_;
  theta = theta_;
  TreeLayout& L = layout;
  if (fmm) {
    RefTree t;
    std::string err;
    if (!build_ref_tree(n, xyz, ncrit, theta, t, err)) fail(CPPE_GPU_INVALID_ARG, err);
    make_layout(t, n, L);
    level_start = L.level_start;
  } else {
    // Direct summation: chunks of 64 sites in caller order act as "leaves",
    // every chunk interacting with every chunk.
    const int chunk = 64;
    L           = TreeLayout();
    L.n         = n;
    L.nleaves   = (n + chunk - 1) / chunk;
    L.ncells    = L.nleaves;
    L.nlevels   = 1;
    L.level_start = {0, L.ncells};
    L.center.assign(4 * (size_t)L.ncells, 0.0);
    L.parent.assign(L.ncells, -1);
    L.child_ptr.assign(L.ncells + 1, 0);
    L.is_leaf.assign(L.ncells, 1);
    L.leaf_of_cell.resize(L.ncells);
    for (int k = 0; k < L.nleaves; ++k) {
      L.leaf_cell.push_back(k);
      L.leaf_of_cell[k] = k;
      L.leaf_start.push_back(k * chunk);
    }
    L.leaf_start.push_back(n);
    L.perm.resize(n);
    std::iota(L.perm.begin(), L.perm.end(), 0);
    L.inv_perm = L.perm;
    L.m2l_ptr.assign(L.ncells + 1, 0);
    L.p2p_ptr.resize(L.nleaves + 1);
    for (int a = 0; a <= L.nleaves; ++a) L.p2p_ptr[a] = a * L.nleaves;
    L.p2p_src.resize((size_t)L.nleaves * L.nleaves);
    for (int a = 0; a < L.nleaves; ++a)
      for (int b = 0; b < L.nleaves; ++b) L.p2p_src[(size_t)a * L.nleaves + b] = b;
    L.p2p_pairs = (long)n * n;
    level_start = L.level_start;
  }
  near_pairs = L.p2p_pairs;

  h_site_leaf.assign(n, 0);
  std::vector<int>& site_leaf_h = h_site_leaf;
  for (int a = 0; a < L.nleaves; ++a)
    for (int k = L.leaf_start[a]; k < L.leaf_start[a + 1]; ++k) site_leaf_h[k] = a;

  // Coordinates in device order.
  h_pos64.assign(n, double4_32a{});
  h_hi.assign(n, float4{});
  h_lo.assign(n, float4{});
  // FP32 coordinates: relative to the bounding-box centre, snapped to a grid
  // of spacing 2^e with |x| < 2^(e+22), so that every difference of two high
  // parts is exact in FP32; the remainders go to `lo` (the FP32 and DD pair
  // passes use only differences).  s = alpha^(-1/6) is split the same way.
  double lo_c[3] = {1e300, 1e300, 1e300}, hi_c[3] = {-1e300, -1e300, -1e300};
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c)
      lo_c[c] = std::min(lo_c[c], xyz[3 * i + c]), hi_c[c] = std::max(hi_c[c], xyz[3 * i + c]);
  double ctr[3], ext = 1.0;
  for (int c = 0; c < 3; ++c) {
    ctr[c] = n ? 0.5 * (lo_c[c] + hi_c[c]) : 0.0;
    if (n) ext = std::max(ext, 0.5 * (hi_c[c] - lo_c[c]) * 1.0001);
  }
  const double quantum = std::ldexp(1.0, (int)std::ceil(std::log2(ext)) - 22);
  auto& p64 = h_pos64;
  auto& hi  = h_hi;
  auto& lo  = h_lo;
  for (int k = 0; k < n; ++k) {
    const int i  = L.perm[k];
    const double x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
    const double sd = s_damp ? s_damp[i] : 0.0;
    p64[k]         = make_double4_32a(x, y, z, sd);
    double r[3]    = {x - ctr[0], y - ctr[1], z - ctr[2]};
    float h[3], l[3];
    for (int c = 0; c < 3; ++c) {
      h[c] = (float)(std::nearbyint(r[c] / quantum) * quantum);
      l[c] = (float)(r[c] - (double)h[c]);
    }
    const float sh = (float)sd;
    hi[k]          = make_float4(h[0], h[1], h[2], sh);
    lo[k]          = make_float4(l[0], l[1], l[2], (float)(sd - (double)sh));
  }

  // Exclusion corrections: pairs the reference skips but the near-field pass
  // includes.  Direct: every listed exclusion; FMM: those whose source sits in
  // a leaf of the target leaf's P2P list (exclusions are honoured only in P2P,
  // calculate.cc:37).
  h_cptr.assign(n + 1, 0);
  h_cidx.clear();
  auto& cptr = h_cptr;
  auto& cidx = h_cidx;
  if (excl_ptr) {
    std::vector<std::vector<int>> sorted_src;
    if (fmm) {
      sorted_src.resize(L.nleaves);
      for (int a = 0; a < L.nleaves; ++a) {
        sorted_src[a].assign(L.p2p_src.begin() + L.p2p_ptr[a], L.p2p_src.begin() + L.p2p_ptr[a + 1]);
        std::sort(sorted_src[a].begin(), sorted_src[a].end());
      }
    }
    for (int k = 0; k < n; ++k) {
      const int i = L.perm[k];
      std::vector<int> mine;
      for (int e = excl_ptr[i]; e < excl_ptr[i + 1]; ++e) {
        const int j = excl_idx[e];
        if (j < 0 || j >= n || j == i) continue;
        const int kj = L.inv_perm[j];
        if (fmm) {
          const auto& v = sorted_src[site_leaf_h[k]];
          if (!std::binary_search(v.begin(), v.end(), site_leaf_h[kj])) continue;
        }
        mine.push_back(kj);
      }
      std::sort(mine.begin(), mine.end());
      mine.erase(std::unique(mine.begin(), mine.end()), mine.end());
      cidx.insert(cidx.end(), mine.begin(), mine.end());
      cptr[k + 1] = (int)cidx.size();
    }
  }
  // algorithmic pairs: the ordered pairs the reference evaluates in its
  // near-field / direct loops (self pairs and excluded pairs are skipped there)
  alg_pairs = near_pairs - n - (long)cidx.size();
  make_items();
}

// Cuts every target leaf's source list into pieces of about `W` pairs so that
// blocks get similar work, and orders the pieces largest first.
void Geometry::make_items() {
  const TreeLayout& L = layout;
  long total          = 0;
  for (int a = 0; a < L.nleaves; ++a) {
    const long na = L.leaf_start[a + 1] - L.leaf_start[a];
    for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q) {
      const int b = L.p2p_src[q];
      total += na * (L.leaf_start[b + 1] - L.leaf_start[b]);
    }
  }
  const long W = std::max<long>(8192, total / (32L * 152));
  struct It {
    long w;
    int4 v;
  };
  std::vector<It> its;
  h_leaf_nslot.assign(L.nleaves, 0);
  for (int a = 0; a < L.nleaves; ++a) {
    const long na = L.leaf_start[a + 1] - L.leaf_start[a];
    int q0 = L.p2p_ptr[a], slot = 0;
    long acc = 0;
    for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q) {
      const int b = L.p2p_src[q];
      acc += na * (L.leaf_start[b + 1] - L.leaf_start[b]);
      if (acc >= W || q + 1 == L.p2p_ptr[a + 1]) {
        its.push_back({acc, make_int4(a, q0, q + 1, slot++)});
        q0  = q + 1;
        acc = 0;
      }
    }
    if (slot == 0) its.push_back({0, make_int4(a, q0, q0, slot++)});  // empty list: zeros
    h_leaf_nslot[a] = slot;
  }
  std::stable_sort(its.begin(), its.end(), [](const It& x, const It& y) { return x.w > y.w; });
  h_items.resize(its.size());
  nslot = 1;
  for (size_t k = 0; k < its.size(); ++k) {
    h_items[k] = its[k].v;
    nslot      = std::max(nslot, its[k].v.w + 1);
  }
}

void Geometry::upload(cudaStream_t s) {
  items.upload(h_items, s);
  leaf_nslot.upload(h_leaf_nslot, s);
  const TreeLayout& L = layout;
  center.upload(L.center, s);
  parent.upload(L.parent, s);
  child_ptr.upload(L.child_ptr, s);
  child_idx.upload(L.child_idx.empty() ? std::vector<int>{0} : L.child_idx, s);
  is_leaf.upload(L.is_leaf, s);
  leaf_cell.upload(L.leaf_cell, s);
  leaf_start.upload(L.leaf_start, s);
  site_leaf.upload(h_site_leaf, s);
  m2l_ptr.upload(L.m2l_ptr, s);
  m2l_src.upload(L.m2l_src.empty() ? std::vector<int>{0} : L.m2l_src, s);
  p2p_ptr.upload(L.p2p_ptr, s);
  p2p_src.upload(L.p2p_src, s);
  perm.upload(L.perm, s);
  inv_perm.upload(L.inv_perm, s);
  pos64.upload(h_pos64, s);
  hi32.upload(h_hi, s);
  lo32.upload(h_lo, s);
  corr_ptr.upload(h_cptr, s);
  corr_idx.upload(h_cidx.empty() ? std::vector<int>{0} : h_cidx, s);
  CG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Site access helpers, per precision
// ---------------------------------------------------------------------------
template <typename T>
struct SiteRec;
template <>
struct SiteRec<double> {
  double x, y, z, s;
};
// FP32 record: grid-snapped coordinates (x, y, z), their remainders
// (lx, ly, lz), and s = alpha^(-1/6) as s + ls.
template <>
struct SiteRec<float> {
  float x, y, z, s, lx, ly, lz, ls;
};

template <typename T>
struct PosArgs;
template <>
struct PosArgs<double> {
  const double4_32a* pos;
  __device__ SiteRec<double> load(int k) const {
    double4_32a p = pos[k];
    return {p.x, p.y, p.z, p.w};
  }
};
template <>
struct PosArgs<float> {
  const float4* hi;
  const float4* lo;
  __device__ SiteRec<float> load(int k) const {
    float4 h = hi[k], l = lo[k];
    return {h.x, h.y, h.z, h.w, l.x, l.y, l.z, l.w};
  }
};

__device__ __forceinline__ void sep(const SiteRec<double>& a, const SiteRec<double>& b, double& x,
                                    double& y, double& z) {
  x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
}
__device__ __forceinline__ void sep(const SiteRec<float>& a, const SiteRec<float>& b, float& x,
                                    float& y, float& z) {
  x = (a.x - b.x) + (a.lx - b.lx);
  y = (a.y - b.y) + (a.ly - b.ly);
  z = (a.z - b.z) + (a.lz - b.lz);
}

template <typename T, int M, bool DAMP, bool FAST = false>
__device__ __forceinline__ void pair_field(const SiteRec<T>& ti, T ai, const SiteRec<T>& sj,
                                           const T* S, T& fx, T& fy, T& fz) {
  T x, y, z;
  sep(ti, sj, x, y, z);
  const T r2 = x * x + y * y + z * z;
  T G[3];
  radial<T, M + 1, FAST>(r2, DAMP ? ai * sj.s : T(0), G);
  if (M == 0) field_m0(x, y, z, G, S[0], fx, fy, fz);
  if (M == 1) field_m1(x, y, z, G, S[0], S[1], S[2], fx, fy, fz);
  if (M == 2) field_m2(x, y, z, G, S, fx, fy, fz);
}

template <typename T>
struct Acc3 {
  T x = 0, y = 0, z = 0;
};
// FP32 accumulators carry a two-sum compensation term.
template <typename T>
struct Comp3 {
  T x = 0, y = 0, z = 0;
  __device__ void add(T a, T b, T c) { x += a, y += b, z += c; }
  __device__ T gx() const { return x; }
  __device__ T gy() const { return y; }
  __device__ T gz() const { return z; }
};
template <>
struct Comp3<float> {
  float x = 0, y = 0, z = 0, ex = 0, ey = 0, ez = 0;
  __device__ void add(float a, float b, float c) {
    float e;
    two_sum(x, a, x, e), ex += e;
    two_sum(y, b, y, e), ey += e;
    two_sum(z, c, z, e), ez += e;
  }
  __device__ float gx() const { return x + ex; }
  __device__ float gy() const { return y + ey; }
  __device__ float gz() const { return z + ez; }
};

// ---------------------------------------------------------------------------
// Tile planning of the near-field pass.  An item covers positions [cur, b1)
// of its target leaf's P2P list; each round warp 0 takes the next (up to) 32
// source leaves, prefix-sums their sizes across the warp and keeps those that
// start inside a tile of P2P_TILE sites, the last one possibly in part
// (`coff` sites of the first leaf were taken by the previous round).
// ---------------------------------------------------------------------------
struct TilePlan {
  int pstart[33];  // first site of each piece
  int poff[34];    // tile offset of each piece (poff[np] = tile size)
  int np, cur, coff;
};

__device__ __forceinline__ void plan_tile(TilePlan& tp, int b1, const int* __restrict__ p2p_src,
                                          const int* __restrict__ leaf_start) {
  const int lane = threadIdx.x & 31;
  const int cur = tp.cur, coff = tp.coff;
  const int e   = cur + lane;
  int start = 0, cnt = 0;
  if (e < b1) {
    const int Lb = p2p_src[e];
    start        = leaf_start[Lb];
    cnt          = leaf_start[Lb + 1] - start;
    if (lane == 0) start += coff, cnt -= coff;
  }
  int incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int excl     = incl - cnt;
  const bool take    = e < b1 && excl < P2P_TILE;
  const int takecnt  = take ? min(cnt, P2P_TILE - excl) : 0;
  const unsigned msk = __ballot_sync(0xffffffffu, take);
  const int np       = __popc(msk);
  const int last     = max(np - 1, 0);
  const int tot      = __shfl_sync(0xffffffffu, excl + takecnt, last);
  const int lastcnt  = __shfl_sync(0xffffffffu, cnt, last);
  const int lasttake = __shfl_sync(0xffffffffu, takecnt, last);
  if (take) tp.pstart[lane] = start, tp.poff[lane] = excl;
  if (lane == 0) {
    tp.np       = np;
    tp.poff[np] = np ? tot : 0;
    if (np > 0) {
      if (lasttake == lastcnt)
        tp.cur = cur + np, tp.coff = 0;
      else
        tp.cur = cur + last, tp.coff = (last == 0 ? coff : 0) + lasttake;
    }
  }
}

// Site index of tile slot q (the piece k with poff[k] <= q < poff[k + 1]).
__device__ __forceinline__ int tile_site(const TilePlan& tp, int q) {
  int lo = 0, hi = tp.np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tp.poff[mid] <= q)
      lo = mid;
    else
      hi = mid - 1;
  }
  return tp.pstart[lo] + (q - tp.poff[lo]);
}

// ---------------------------------------------------------------------------
// Near field: block per work item (target leaf, piece of its source list).
// Every thread serves two target sites of the leaf against a stride of the
// staged sources (S = 128 / ceil(n_A / 2) groups), so each source read from
// shared memory feeds two pair evaluations; group partials are added in group
// order at the end and written to the item's output slot.
// ---------------------------------------------------------------------------
template <typename T, int M, bool DAMP, bool FAST>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
            const int* __restrict__ p2p_src, PosArgs<T> pa, const T* __restrict__ src,
            T damping, T* __restrict__ Fnear) {
  constexpr int NS = ncomp(M);
  __shared__ SiteRec<T> s_rec[P2P_TILE];
  __shared__ T s_S[P2P_TILE * NS];
  __shared__ TilePlan s_plan;
  __shared__ T s_red[P2P_BLOCK * 6];

  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;

  for (int tb = 0; tb < nA; tb += 2 * P2P_BLOCK) {
    const int nT = min(2 * P2P_BLOCK, nA - tb);
    const int T2 = (nT + 1) >> 1;
    const int S  = P2P_BLOCK / T2;
    const int t = threadIdx.x % T2, g = threadIdx.x / T2;
    const bool active = g < S;
    const bool has1   = t + T2 < nT;
    const SiteRec<T> me0 = pa.load(a0 + tb + t);
    const SiteRec<T> me1 = pa.load(a0 + tb + (has1 ? t + T2 : t));
    const T ai0 = damping * me0.s, ai1 = damping * me1.s;
    Comp3<T> acc0, acc1;
    if (threadIdx.x == 0) s_plan.cur = b0, s_plan.coff = 0;
    __syncthreads();
    while (true) {
      if (threadIdx.x < 32) plan_tile(s_plan, b1, p2p_src, leaf_start);
      __syncthreads();
      const int np = s_plan.np;
      if (np == 0) break;
      const int total = s_plan.poff[np];
      for (int q = threadIdx.x; q < total; q += P2P_BLOCK) {
        const int j = tile_site(s_plan, q);
        s_rec[q]    = pa.load(j);
#pragma unroll
        for (int c = 0; c < NS; ++c) s_S[q * NS + c] = src[(size_t)j * NS + c];
      }
      __syncthreads();
      if (active) {
        T fx0 = 0, fy0 = 0, fz0 = 0, fx1 = 0, fy1 = 0, fz1 = 0;
        for (int jj = g; jj < total; jj += S) {
          const SiteRec<T> sj = s_rec[jj];
          const T* Sj         = &s_S[jj * NS];
          pair_field<T, M, DAMP, FAST>(me0, ai0, sj, Sj, fx0, fy0, fz0);
          pair_field<T, M, DAMP, FAST>(me1, ai1, sj, Sj, fx1, fy1, fz1);
        }
        acc0.add(fx0, fy0, fz0);
        acc1.add(fx1, fy1, fz1);
      }
      __syncthreads();
    }
    if (active) {
      T* r = &s_red[(g * T2 + t) * 6];
      r[0] = acc0.gx(), r[1] = acc0.gy(), r[2] = acc0.gz();
      r[3] = acc1.gx(), r[4] = acc1.gy(), r[5] = acc1.gz();
    }
    __syncthreads();
    if (threadIdx.x < T2) {
      T f[6] = {0, 0, 0, 0, 0, 0};
      for (int gg = 0; gg < S; ++gg)
#pragma unroll
        for (int c = 0; c < 6; ++c) f[c] += s_red[(gg * T2 + threadIdx.x) * 6 + c];
      T* o = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x);
      o[0] = f[0], o[1] = f[1], o[2] = f[2];
      if (threadIdx.x + T2 < nT) {
        T* o1 = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x + T2);
        o1[0] = f[3], o1[1] = f[4], o1[2] = f[5];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Near field, FP32, dipole sources: the inner pass of the mixed solver.
// Positions are taken relative to the first site of the target leaf once per
// staged source (hi/lo differences, ~FP32 accuracy of the relative vector),
// so a pair costs one subtraction per component; the v < 50 cut of the FP64
// path is not needed (expf underflows to 0 there).  Sources are staged as
// float4 {x, y, z, s} and {mu_x, mu_y, mu_z, -}: two shared loads feed the
// two targets of a thread.
// ---------------------------------------------------------------------------
template <bool DAMP>
__device__ __forceinline__ void f32_pair_m1(const float4& ti, float ai, const float4& sj,
                                            const float4& mu, float& fx, float& fy, float& fz) {
  const float x = ti.x - sj.x, y = ti.y - sj.y, z = ti.z - sj.z;
  const float r2 = fmaf(x, x, fmaf(y, y, z * z));
  const float ir = r2 > 0.f ? rsqrtf(r2) : 0.f;
  const float ir2 = ir * ir;
  const float ir3 = ir2 * ir;
  float A = ir3, B = 3.f * ir3 * ir2;  // G1 = -A, G2 = B
  if (DAMP) {
    const float a = ai * sj.w;
    if (a > 0.f) {
      const float v  = a * (r2 * ir);
      const float e  = __expf(-v);
      const float fE = fmaf(-fmaf(v, fmaf(v, 0.5f, 1.f), 1.f), e, 1.f);
      const float fT = fmaf(-(v * v) * (v * (1.f / 6.f)), e, fE);
      A *= fE, B *= fT;
    }
  }
  const float C = (mu.x * x + mu.y * y + mu.z * z) * B;
  fx = fmaf(mu.x, A, fmaf(-x, C, fx));
  fy = fmaf(mu.y, A, fmaf(-y, C, fy));
  fz = fmaf(mu.z, A, fmaf(-z, C, fz));
}

template <bool DAMP>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p32_m1(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
                 const int* __restrict__ p2p_src, const float4* __restrict__ hi,
                 const float4* __restrict__ lo, const float* __restrict__ src, float damping,
                 float* __restrict__ Fnear) {
  __shared__ float4 s_pos[P2P_TILE];
  __shared__ float4 s_mu[P2P_TILE];
  __shared__ TilePlan s_plan;
  __shared__ float s_red[P2P_BLOCK * 6];

  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const float4 oh = hi[a0], ol = lo[a0];
  auto rel = [&](int k) {
    const float4 h = hi[k], l = lo[k];
    return make_float4((h.x - oh.x) + (l.x - ol.x), (h.y - oh.y) + (l.y - ol.y),
                       (h.z - oh.z) + (l.z - ol.z), h.w);
  };

  for (int tb = 0; tb < nA; tb += 2 * P2P_BLOCK) {
    const int nT = min(2 * P2P_BLOCK, nA - tb);
    const int T2 = (nT + 1) >> 1;
    const int S  = P2P_BLOCK / T2;
    const int t = threadIdx.x % T2, g = threadIdx.x / T2;
    const bool active = g < S;
    const bool has1   = t + T2 < nT;
    const float4 me0 = rel(a0 + tb + t);
    const float4 me1 = rel(a0 + tb + (has1 ? t + T2 : t));
    const float ai0 = damping * me0.w, ai1 = damping * me1.w;
    Comp3<float> acc0, acc1;
    if (threadIdx.x == 0) s_plan.cur = b0, s_plan.coff = 0;
    __syncthreads();
    while (true) {
      if (threadIdx.x < 32) plan_tile(s_plan, b1, p2p_src, leaf_start);
      __syncthreads();
      const int np = s_plan.np;
      if (np == 0) break;
      const int total = s_plan.poff[np];
      for (int q = threadIdx.x; q < total; q += P2P_BLOCK) {
        const int j = tile_site(s_plan, q);
        s_pos[q]    = rel(j);
        s_mu[q]     = make_float4(src[3 * (size_t)j], src[3 * (size_t)j + 1],
                                  src[3 * (size_t)j + 2], 0.f);
      }
      __syncthreads();
      if (active) {
        float fx0 = 0, fy0 = 0, fz0 = 0, fx1 = 0, fy1 = 0, fz1 = 0;
        for (int jj = g; jj < total; jj += S) {
          const float4 sj = s_pos[jj];
          const float4 mu = s_mu[jj];
          f32_pair_m1<DAMP>(me0, ai0, sj, mu, fx0, fy0, fz0);
          f32_pair_m1<DAMP>(me1, ai1, sj, mu, fx1, fy1, fz1);
        }
        acc0.add(fx0, fy0, fz0);
        acc1.add(fx1, fy1, fz1);
      }
      __syncthreads();
    }
    if (active) {
      float* r = &s_red[(g * T2 + t) * 6];
      r[0] = acc0.gx(), r[1] = acc0.gy(), r[2] = acc0.gz();
      r[3] = acc1.gx(), r[4] = acc1.gy(), r[5] = acc1.gz();
    }
    __syncthreads();
    if (threadIdx.x < T2) {
      float f[6] = {0, 0, 0, 0, 0, 0};
      for (int gg = 0; gg < S; ++gg)
#pragma unroll
        for (int c = 0; c < 6; ++c) f[c] += s_red[(gg * T2 + threadIdx.x) * 6 + c];
      float* o = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x);
      o[0] = f[0], o[1] = f[1], o[2] = f[2];
      if (threadIdx.x + T2 < nT) {
        float* o1 = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x + T2);
        o1[0] = f[3], o1[1] = f[4], o1[2] = f[5];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Near field in double-float arithmetic (dipole sources): the FP64-accurate
// pass of the mixed solver's residual B x, on the FP32 pipe.  Same items and
// tiles as k_p2p; each pair is evaluated in DD (about 1e-13 relative per
// term), accumulated in DD and written in FP64.  Separations are exact in
// their high parts because the FP32 coordinates are snapped to a common grid.
// ---------------------------------------------------------------------------
template <bool DAMP>
__device__ __forceinline__ void dd_pair_m1(const SiteRec<float>& ti, dd ai,
                                           const SiteRec<float>& sj, const float* mu,
                                           const float2* etab, dd (&f)[3]) {
  const dd x = {ti.x - sj.x, ti.lx - sj.lx};
  const dd y = {ti.y - sj.y, ti.ly - sj.ly};
  const dd z = {ti.z - sj.z, ti.lz - sj.lz};
  const dd r2 = dd_add(dd_add_lazy(dd_sqr_full(x), dd_sqr_full(y)), dd_sqr_full(z));
  if (r2.h == 0.f) return;  // a site paired with itself (direct summation)
  const dd ir  = dd_rsqrt(r2);
  const dd ir2 = dd_sqr(ir);
  const dd ir3 = dd_mul(ir2, ir);
  dd G1        = dd_neg(ir3);
  dd G2        = dd_mul_f(dd_mul(ir3, ir2), 3.f);
  if (DAMP) {
    const dd a = dd_mul(ai, dd{sj.s, sj.ls});
    if (a.h > 0.f) {
      const dd v = dd_mul(a, dd_mul(r2, ir));
      if (v.h < 50.f) {
        dd fE, fT;
        if (v.h < 20.f) {
          const dd e  = dd_exp_neg(v, etab);
          const dd v2 = dd_sqr(v);
          const dd u  = dd_add(dd_two_sum(1.f, v.h), dd{0.5f * v2.h, v.l + 0.5f * v2.l});
          const dd w  = dd_mul(dd_mul(v2, v), dd{1.f / 6.f, DD_SIXTH_LO});
          fE          = dd_sub(dd{1.f, 0.f}, dd_mul(u, e));
          fT          = dd_sub(fE, dd_mul(w, e));
        } else {
          // (1 + v + v^2/2) e^-v < 5e-7 here: FP32 suffices for the deficit
          const float e = expf(-v.h);
          const float u = fmaf(v.h, fmaf(v.h, 0.5f, 1.f), 1.f) * e;
          const float w = v.h * v.h * v.h * (1.f / 6.f) * e;
          fE            = dd_fast_two_sum(1.f, -u);
          fT            = dd_fast_two_sum(1.f, -(u + w));
        }
        G1 = dd_mul(G1, fE);
        G2 = dd_mul(G2, fT);
      }
    }
  }
  const dd mx = {mu[0], mu[3]}, my = {mu[1], mu[4]}, mz = {mu[2], mu[5]};
  const dd mr = dd_add(dd_add_lazy(dd_mul(mx, x), dd_mul(my, y)), dd_mul(mz, z));
  const dd sg = dd_mul(mr, G2);
  f[0] = dd_add_lazy(f[0], dd_neg(dd_add_lazy(dd_mul(mx, G1), dd_mul(sg, x))));
  f[1] = dd_add_lazy(f[1], dd_neg(dd_add_lazy(dd_mul(my, G1), dd_mul(sg, y))));
  f[2] = dd_add_lazy(f[2], dd_neg(dd_add_lazy(dd_mul(mz, G1), dd_mul(sg, z))));
}

template <bool DAMP>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p_dd(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
               const int* __restrict__ p2p_src, PosArgs<float> pa,
               const double* __restrict__ src, double damping, double* __restrict__ Fnear) {
  __shared__ SiteRec<float> s_rec[P2P_TILE];
  __shared__ float s_mu[P2P_TILE * 6];
  __shared__ float2 s_etab[DD_EXP_TAB];
  __shared__ TilePlan s_plan;
  __shared__ double s_red[P2P_BLOCK * 6];

  for (int k = threadIdx.x; k < DD_EXP_TAB; k += P2P_BLOCK) {
    const double e = exp(-0.0625 * k);
    const float h  = (float)e;
    s_etab[k]      = make_float2(h, (float)(e - (double)h));
  }
  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const dd dmp = dd_from(damping);

  for (int tb = 0; tb < nA; tb += 2 * P2P_BLOCK) {
    const int nT = min(2 * P2P_BLOCK, nA - tb);
    const int T2 = (nT + 1) >> 1;
    const int S  = P2P_BLOCK / T2;
    const int t = threadIdx.x % T2, g = threadIdx.x / T2;
    const bool active = g < S;
    const bool has1   = t + T2 < nT;
    const SiteRec<float> me0 = pa.load(a0 + tb + t);
    const SiteRec<float> me1 = pa.load(a0 + tb + (has1 ? t + T2 : t));
    const dd ai0 = dd_mul(dmp, dd{me0.s, me0.ls}), ai1 = dd_mul(dmp, dd{me1.s, me1.ls});
    dd f0[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    dd f1[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (threadIdx.x == 0) s_plan.cur = b0, s_plan.coff = 0;
    __syncthreads();
    while (true) {
      if (threadIdx.x < 32) plan_tile(s_plan, b1, p2p_src, leaf_start);
      __syncthreads();
      const int np = s_plan.np;
      if (np == 0) break;
      const int total = s_plan.poff[np];
      for (int q = threadIdx.x; q < total; q += P2P_BLOCK) {
        const int j = tile_site(s_plan, q);
        s_rec[q]    = pa.load(j);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const dd m = dd_from(src[3 * (size_t)j + c]);
          s_mu[q * 6 + c] = m.h, s_mu[q * 6 + 3 + c] = m.l;
        }
      }
      __syncthreads();
      if (active) {
        for (int jj = g; jj < total; jj += S) {
          const SiteRec<float> sj = s_rec[jj];
          const float* mu         = &s_mu[jj * 6];
          dd_pair_m1<DAMP>(me0, ai0, sj, mu, s_etab, f0);
          dd_pair_m1<DAMP>(me1, ai1, sj, mu, s_etab, f1);
        }
      }
      __syncthreads();
    }
    if (active) {
      double* r = &s_red[(g * T2 + t) * 6];
      r[0] = dd_to(f0[0]), r[1] = dd_to(f0[1]), r[2] = dd_to(f0[2]);
      r[3] = dd_to(f1[0]), r[4] = dd_to(f1[1]), r[5] = dd_to(f1[2]);
    }
    __syncthreads();
    if (threadIdx.x < T2) {
      double f[6] = {0, 0, 0, 0, 0, 0};
      for (int gg = 0; gg < S; ++gg)
#pragma unroll
        for (int c = 0; c < 6; ++c) f[c] += s_red[(gg * T2 + threadIdx.x) * 6 + c];
      double* o = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x);
      o[0] = f[0], o[1] = f[1], o[2] = f[2];
      if (threadIdx.x + T2 < nT) {
        double* o1 = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x + T2);
        o1[0] = f[3], o1[1] = f[4], o1[2] = f[5];
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// FMM passes
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void powers(T d, int p, T* pw) {
  pw[0] = T(1);
#pragma unroll
  for (int a = 1; a <= PMAX; ++a)
    if (a <= p) pw[a] = pw[a - 1] * d * (T(1) / T(a));
}

template <typename T>
__device__ __forceinline__ T mono(const T* px, const T* py, const T* pz, int e) {
  return px[e & 15] * py[(e >> 4) & 15] * pz[e >> 8];
}

// P2M: thread per (leaf, M row); multipole of the leaf's sites about its centre.
template <typename T>
__global__ void k_p2m(TreeView tv, OpsView ov, const double4_32a* __restrict__ pos,
                      const T* __restrict__ src, T* __restrict__ M) {
  const int gid  = blockIdx.x * blockDim.x + threadIdx.x;
  const int leaf = gid / ov.msize, row = gid - (gid / ov.msize) * ov.msize;
  if (leaf >= tv.nleaves) return;
  const int cell  = tv.leaf_cell[leaf];
  const double4_32a c = tv.center[cell];
  const int ns    = ncomp(ov.m);
  const int t0 = ov.p2m_ptr[row], t1 = ov.p2m_ptr[row + 1];
  T acc = 0;
  for (int q = tv.leaf_start[leaf]; q < tv.leaf_start[leaf + 1]; ++q) {
    const double4_32a x = pos[q];
    T px[PMAX + 1], py[PMAX + 1], pz[PMAX + 1];
    powers<T>((T)(c.x - x.x), ov.p, px);
    powers<T>((T)(c.y - x.y), ov.p, py);
    powers<T>((T)(c.z - x.z), ov.p, pz);
    for (int t = t0; t < t1; ++t)
      acc += mono(px, py, pz, ov.exps[ov.p2m_j[t]]) * src[(size_t)q * ns + ov.p2m_k[t]];
  }
  M[(size_t)cell * ov.msize + row] = acc;
}

// M2M for the non-leaf cells of one level: thread per (cell, M row).
template <typename T>
__global__ void k_m2m(TreeView tv, OpsView ov, int c0, int c1, T* __restrict__ M) {
  const int gid  = blockIdx.x * blockDim.x + threadIdx.x;
  const int cell = c0 + gid / ov.msize, row = gid % ov.msize;
  if (cell >= c1 || tv.is_leaf[cell]) return;
  const double4_32a cp = tv.center[cell];
  const int t0 = ov.m2m_ptr[row], t1 = ov.m2m_ptr[row + 1];
  T acc = 0;
  for (int k = tv.child_ptr[cell]; k < tv.child_ptr[cell + 1]; ++k) {
    const int ch     = tv.child_idx[k];
    const double4_32a cc = tv.center[ch];
    T px[PMAX + 1], py[PMAX + 1], pz[PMAX + 1];
    powers<T>((T)(cp.x - cc.x), ov.p, px);
    powers<T>((T)(cp.y - cc.y), ov.p, py);
    powers<T>((T)(cp.z - cc.z), ov.p, pz);
    const T* Mc = M + (size_t)ch * ov.msize;
    for (int t = t0; t < t1; ++t) acc += mono(px, py, pz, ov.exps[ov.m2m_j[t]]) * Mc[ov.m2m_k[t]];
  }
  M[(size_t)cell * ov.msize + row] = acc;
}

// L2L for the cells of one level (>= 1): thread per (cell, L row).
template <typename T>
__global__ void k_l2l(TreeView tv, OpsView ov, int c0, int c1, T* __restrict__ L) {
  const int gid  = blockIdx.x * blockDim.x + threadIdx.x;
  const int cell = c0 + gid / ov.lsize, row = gid % ov.lsize;
  if (cell >= c1) return;
  const int par    = tv.parent[cell];
  const double4_32a cc = tv.center[cell], cp = tv.center[par];
  T px[PMAX + 1], py[PMAX + 1], pz[PMAX + 1];
  const int q = ov.p - ov.m;
  powers<T>((T)(cc.x - cp.x), q, px);
  powers<T>((T)(cc.y - cp.y), q, py);
  powers<T>((T)(cc.z - cp.z), q, pz);
  const T* Lp = L + (size_t)par * ov.lsize;
  T acc       = 0;
  for (int t = ov.l2l_ptr[row]; t < ov.l2l_ptr[row + 1]; ++t)
    acc += mono(px, py, pz, ov.exps[ov.l2l_j[t]]) * Lp[ov.l2l_k[t]];
  L[(size_t)cell * ov.lsize + row] += acc;
}

// M2L: warp per target cell.  Per source cell the warp builds the derivative
// tensor D_j = d^j (1/R) order by order from the recurrence
//   |n| R^2 D_n = -(2|n|-1) sum_i n_i r_i D_{n-e_i} - (|n|-1) sum_i n_i (n_i-1) D_{n-2e_i}
// (differentiate R^2 d_i(1/R) = -r_i/R), then each lane adds its slots of
// D_{n+k} M_k terms.  Slot sums are combined per row in fixed order.
template <typename T>
__global__ void __launch_bounds__(32 * M2L_WARPS)
      k_m2l(TreeView tv, OpsView ov, const T* __restrict__ M, T* __restrict__ L) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int nt = ov.nt, msz = ov.msize;
  int* s_kw    = reinterpret_cast<int*>(smem);
  int* s_drec  = s_kw + ov.nm2l_terms;
  int* s_exps  = s_drec + 8 * nt;
  size_t ioff  = (size_t)(ov.nm2l_terms + 9 * nt) * sizeof(int);
  ioff         = (ioff + 15) & ~(size_t)15;
  T* s_base    = reinterpret_cast<T*>(smem + ioff);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per_warp = nt + msz + 32 * M2L_SLOTS;
  T* D    = s_base + warp * per_warp;
  T* Mb   = D + nt;
  T* part = Mb + msz;
  for (int i = threadIdx.x; i < ov.nm2l_terms; i += blockDim.x) s_kw[i] = ov.m2l_kw[i];
  for (int i = threadIdx.x; i < 8 * nt; i += blockDim.x) s_drec[i] = ov.drec[i];
  for (int i = threadIdx.x; i < nt; i += blockDim.x) s_exps[i] = ov.exps[i];
  __syncthreads();
  const int A = blockIdx.x * M2L_WARPS + warp;
  if (A >= tv.ncells) return;

  int srow[M2L_SLOTS], st0[M2L_SLOTS], st1[M2L_SLOTS];
  T acc[M2L_SLOTS];
#pragma unroll
  for (int s = 0; s < M2L_SLOTS; ++s) {
    const int* sl = ov.slots + (lane * M2L_SLOTS + s) * 3;
    srow[s] = sl[0], st0[s] = sl[1], st1[s] = sl[2];
    acc[s] = T(0);
  }
  (void)srow;
  const double4_32a cA = tv.center[A];
  for (int idx = tv.m2l_ptr[A]; idx < tv.m2l_ptr[A + 1]; ++idx) {
    const int B      = tv.m2l_src[idx];
    const double4_32a cB = tv.center[B];
    const T x = (T)(cA.x - cB.x), y = (T)(cA.y - cB.y), z = (T)(cA.z - cB.z);
    for (int k = lane; k < msz; k += 32) Mb[k] = M[(size_t)B * msz + k];
    const T r2  = x * x + y * y + z * z;
    const T ir2 = T(1) / r2;
    if (lane == 0) D[0] = rsqrt_t(r2);
    __syncwarp();
    for (int o = 1; o <= ov.p; ++o) {
      const int j1 = nterms(o);
      const T c1 = T(2 * o - 1), c2 = T(o - 1), io = T(1) / T(o);
      for (int j = nterms(o - 1) + lane; j < j1; j += 32) {
        const int* q = s_drec + 8 * j;
        const int e  = s_exps[j];
        const int n0 = e & 15, n1 = (e >> 4) & 15, n2 = e >> 8;
        T s1 = 0, s2 = 0;
        if (q[0] >= 0) s1 += T(n0) * x * D[q[0]];
        if (q[1] >= 0) s1 += T(n1) * y * D[q[1]];
        if (q[2] >= 0) s1 += T(n2) * z * D[q[2]];
        if (q[3] >= 0) s2 += T(n0 * (n0 - 1)) * D[q[3]];
        if (q[4] >= 0) s2 += T(n1 * (n1 - 1)) * D[q[4]];
        if (q[5] >= 0) s2 += T(n2 * (n2 - 1)) * D[q[5]];
        D[j] = -(c1 * s1 + c2 * s2) * ir2 * io;
      }
      __syncwarp();
    }
#pragma unroll
    for (int s = 0; s < M2L_SLOTS; ++s) {
      T a = acc[s];
      for (int t = st0[s]; t < st1[s]; ++t) {
        const int kw = s_kw[t];
        a += D[kw >> 16] * Mb[kw & 0xffff];
      }
      acc[s] = a;
    }
    __syncwarp();
  }
#pragma unroll
  for (int s = 0; s < M2L_SLOTS; ++s) part[lane * M2L_SLOTS + s] = acc[s];
  __syncwarp();
  for (int row = lane; row < ov.lsize; row += 32) {
    T v = 0;
    for (int i = ov.row_slot_ptr[row]; i < ov.row_slot_ptr[row + 1]; ++i)
      v += part[ov.row_slot_id[i]];
    L[(size_t)A * ov.lsize + row] = v;
  }
}

// ---------------------------------------------------------------------------
// Finishing pass: thread per site.  Adds the source splits of the near field,
// the far field (L2P of the site's leaf), removes excluded pairs, then either
// adds alpha^-1 src (apply) or accumulates sign * F into an FP64 field.
// ---------------------------------------------------------------------------
template <typename T, int M, int MODE>
__global__ void k_finish(int n, const int* __restrict__ leaf_nslot, const T* __restrict__ Fnear,
                         int use_fmm,
                         TreeView tv, OpsView ov, const T* __restrict__ L, PosArgs<T> pa,
                         const double4_32a* __restrict__ pos64, const T* __restrict__ src,
                         int damp, T damping, const int* __restrict__ corr_ptr,
                         const int* __restrict__ corr_idx, const T* __restrict__ ainv6,
                         T* __restrict__ out, double* __restrict__ out64, double sign,
                         ReduceSlots dot) {
  constexpr int NS = ncomp(M);
  __shared__ double sh[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double dv[1] = {0.0};
  if (i < n) {
    T f[3] = {0, 0, 0};
    const int nsl = leaf_nslot[tv.site_leaf[i]];
    for (int s = 0; s < nsl; ++s) {
      const T* q = Fnear + (size_t)s * 3 * n + 3 * (size_t)i;
      f[0] += q[0], f[1] += q[1], f[2] += q[2];
    }
    if (use_fmm) {
      const int cell  = tv.leaf_cell[tv.site_leaf[i]];
      const double4_32a c = tv.center[cell];
      const double4_32a x = pos64[i];
      T px[PMAX + 1], py[PMAX + 1], pz[PMAX + 1];
      const int q = ov.p - ov.m;
      powers<T>((T)(x.x - c.x), q, px);
      powers<T>((T)(x.y - c.y), q, py);
      powers<T>((T)(x.z - c.z), q, pz);
      const T* Lc = L + (size_t)cell * ov.lsize;
      for (int u = 0; u < ov.nl2p; ++u)
        f[ov.l2p_c[u]] -= mono(px, py, pz, ov.exps[ov.l2p_j[u]]) * Lc[ov.l2p_n[u]];
    }
    const int e0 = corr_ptr[i], e1 = corr_ptr[i + 1];
    if (e0 < e1) {
      const SiteRec<T> me = pa.load(i);
      const T ai          = damping * me.s;
      T cx = 0, cy = 0, cz = 0;
      for (int e = e0; e < e1; ++e) {
        const int j = corr_idx[e];
        if (damp)
          pair_field<T, M, true>(me, ai, pa.load(j), src + (size_t)j * NS, cx, cy, cz);
        else
          pair_field<T, M, false>(me, ai, pa.load(j), src + (size_t)j * NS, cx, cy, cz);
      }
      f[0] -= cx, f[1] -= cy, f[2] -= cz;
    }
    if (MODE == FINISH_APPLY) {
      const T* a  = ainv6 + 6 * (size_t)i;
      const T* sv = src + 3 * (size_t)i;
      const T o0  = f[0] + (a[0] * sv[0] + a[1] * sv[1] + a[2] * sv[2]);
      const T o1  = f[1] + (a[1] * sv[0] + a[3] * sv[1] + a[4] * sv[2]);
      const T o2  = f[2] + (a[2] * sv[0] + a[4] * sv[1] + a[5] * sv[2]);
      out[3 * (size_t)i]     = o0;
      out[3 * (size_t)i + 1] = o1;
      out[3 * (size_t)i + 2] = o2;
      dv[0] = (double)sv[0] * o0 + (double)sv[1] * o1 + (double)sv[2] * o2;
    } else {
      out64[3 * (size_t)i] += sign * (double)f[0];
      out64[3 * (size_t)i + 1] += sign * (double)f[1];
      out64[3 * (size_t)i + 2] += sign * (double)f[2];
    }
  }
  if (dot.site_values) {
    if (i < n) dot.site_values[i] = dv[0];
  } else if (dot.partials) {
    grid_sum_last<1>(dv, sh, dot.partials, dot.ticket, dot.out);
  }
}

// ---------------------------------------------------------------------------
// Host driver
// ---------------------------------------------------------------------------
template <typename T>
static PosArgs<T> pos_args(const Geometry& g);
template <>
PosArgs<double> pos_args<double>(const Geometry& g) {
  return PosArgs<double>{g.pos64.p};
}
template <>
PosArgs<float> pos_args<float>(const Geometry& g) {
  return PosArgs<float>{g.hi32.p, g.lo32.p};
}

template <typename T, int M>
static void launch_p2p(const Geometry& g, bool damp, bool fast, const T* src, T damping,
                       T* Fnear, cudaStream_t s) {
  const int grid = (int)g.h_items.size();
  if constexpr (std::is_same<T, float>::value && M == 1) {
    if (damp)
      k_p2p32_m1<true><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p,
                                                  g.hi32.p, g.lo32.p, src, damping, Fnear);
    else
      k_p2p32_m1<false><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p,
                                                   g.hi32.p, g.lo32.p, src, damping, Fnear);
    CG_LAUNCH();
    return;
  }
#define CG_P2P(D, F)                                                                            \
  k_p2p<T, M, D, F><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p, \
                                               pos_args<T>(g), src, damping, Fnear)
  if (damp && fast)
    CG_P2P(true, true);
  else if (damp)
    CG_P2P(true, false);
  else
    CG_P2P(false, false);
#undef CG_P2P
  CG_LAUNCH();
}

void SideStream::create() {
  CG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  CG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
}
void SideStream::destroy() {
  if (join) cudaEventDestroy(join);
  if (fork) cudaEventDestroy(fork);
  if (s) cudaStreamDestroy(s);
  s = nullptr, fork = join = nullptr;
}

static void launch_p2p_dd(const Geometry& g, bool damp, const double* src, double damping,
                          double* Fnear, cudaStream_t s) {
  const int grid = (int)g.h_items.size();
  if (damp)
    k_p2p_dd<true><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p,
                                              pos_args<float>(g), src, damping, Fnear);
  else
    k_p2p_dd<false><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p,
                                               pos_args<float>(g), src, damping, Fnear);
  CG_LAUNCH();
}

template <typename T>
void eval_field(const Geometry& g, const DeviceOps* ops, FieldWork<T>& w, int m, const T* src,
                bool damp, double damping, FinishMode mode, const T* ainv6, T* out,
                double* out64, double sign, const ReduceSlots* dot, cudaStream_t s,
                const PhaseEvents* pe, int near_mode, const SideStream* side) {
  const TreeView tv = g.view();
  OpsView ov{};
  const int n = g.n;
  auto mark = [&](int k) {
    if (pe) CG_CUDA(cudaEventRecord(pe->ev[k], s));
  };
  mark(0);
  // far-field passes on the side stream when one is given (not while phases
  // are being timed)
  cudaStream_t fs = s;
  if (g.fmm && side && side->s && !pe) {
    CG_CUDA(cudaEventRecord(side->fork, s));
    CG_CUDA(cudaStreamWaitEvent(side->s, side->fork, 0));
    fs = side->s;
  }
  if (g.fmm) {
    if (!ops || ops->host.m != m) fail(CPPE_GPU_INVALID_ARG, "FMM tables missing for order");
    ov = ops->view();
    w.M.alloc((size_t)tv.ncells * ov.msize);
    w.L.alloc((size_t)tv.ncells * ov.lsize);
    const int TB = 128;
    {
      long work = (long)tv.nleaves * ov.msize;
      k_p2m<T><<<(unsigned)((work + TB - 1) / TB), TB, 0, fs>>>(tv, ov, g.pos64.p, src, w.M.p);
      CG_LAUNCH();
    }
    for (int l = (int)g.level_start.size() - 3; l >= 0; --l) {
      const int c0 = g.level_start[l], c1 = g.level_start[l + 1];
      long work    = (long)(c1 - c0) * ov.msize;
      if (work == 0) continue;
      k_m2m<T><<<(unsigned)((work + TB - 1) / TB), TB, 0, fs>>>(tv, ov, c0, c1, w.M.p);
      CG_LAUNCH();
    }
    mark(1);
    if (launch_m2l_fixed<T>(tv, ov.m, ov.p, w.M.p, w.L.p, fs)) {
      CG_LAUNCH();
    } else {
      size_t smem = (size_t)(ov.nm2l_terms + 9 * ov.nt) * sizeof(int);
      smem        = (smem + 15) & ~(size_t)15;
      smem += (size_t)M2L_WARPS * (ov.nt + ov.msize + 32 * M2L_SLOTS) * sizeof(T);
      static bool attr_set[2] = {false, false};
      if (smem > 48 * 1024 && !attr_set[sizeof(T) == 8]) {
        CG_CUDA(cudaFuncSetAttribute(k_m2l<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024));
        attr_set[sizeof(T) == 8] = true;
      }
      const int blocks = (tv.ncells + M2L_WARPS - 1) / M2L_WARPS;
      k_m2l<T><<<blocks, 32 * M2L_WARPS, smem, fs>>>(tv, ov, w.M.p, w.L.p);
      CG_LAUNCH();
    }
    mark(2);
    for (int l = 1; l < (int)g.level_start.size() - 1; ++l) {
      const int c0 = g.level_start[l], c1 = g.level_start[l + 1];
      long work    = (long)(c1 - c0) * ov.lsize;
      if (work == 0) continue;
      k_l2l<T><<<(unsigned)((work + TB - 1) / TB), TB, 0, fs>>>(tv, ov, c0, c1, w.L.p);
      CG_LAUNCH();
    }
    mark(3);
    if (fs != s) CG_CUDA(cudaEventRecord(side->join, fs));
  } else {
    mark(1), mark(2), mark(3);
  }
  w.Fnear.alloc((size_t)g.nslot * 3 * n);
  const T dampT = (T)damping;
  const bool fast = near_mode != NEAR_FP64;
  bool done       = false;
  if constexpr (std::is_same<T, double>::value) {
    if (near_mode == NEAR_DD && m == 1) {
      launch_p2p_dd(g, damp, src, damping, w.Fnear.p, s);
      done = true;
    }
  }
  if (!done && m == 0) launch_p2p<T, 0>(g, damp, fast, src, dampT, w.Fnear.p, s);
  if (!done && m == 1) launch_p2p<T, 1>(g, damp, fast, src, dampT, w.Fnear.p, s);
  if (!done && m == 2) launch_p2p<T, 2>(g, damp, fast, src, dampT, w.Fnear.p, s);
  mark(4);
  if (fs != s) CG_CUDA(cudaStreamWaitEvent(s, side->join, 0));

  const int FB = 256;
  const int nb = (n + FB - 1) / FB;
  ReduceSlots rs{nullptr, nullptr, nullptr};
  if (dot) rs = *dot;
  const T* Lp = g.fmm ? w.L.p : nullptr;
#define CG_FINISH(TT, MM, MODE)                                                               \
  k_finish<TT, MM, MODE><<<nb, FB, 0, s>>>(n, g.leaf_nslot.p, w.Fnear.p, g.fmm ? 1 : 0, tv, ov, Lp, \
                                           pos_args<TT>(g), g.pos64.p, src, damp ? 1 : 0,    \
                                           dampT, g.corr_ptr.p, g.corr_idx.p, ainv6, out,    \
                                           out64, sign, rs)
  if (mode == FINISH_APPLY) {
    if (m != 1) fail(CPPE_GPU_INVALID_ARG, "apply mode needs dipole sources");
    CG_FINISH(T, 1, FINISH_APPLY);
  } else {
    if (m == 0) CG_FINISH(T, 0, FINISH_FIELD);
    if (m == 1) CG_FINISH(T, 1, FINISH_FIELD);
    if (m == 2) CG_FINISH(T, 2, FINISH_FIELD);
  }
#undef CG_FINISH
  CG_LAUNCH();
  mark(5);
}

template void eval_field<double>(const Geometry&, const DeviceOps*, FieldWork<double>&, int,
                                 const double*, bool, double, FinishMode, const double*,
                                 double*, double*, double, const ReduceSlots*, cudaStream_t,
                                 const PhaseEvents*, int, const SideStream*);
template void eval_field<float>(const Geometry&, const DeviceOps*, FieldWork<float>&, int,
                                const float*, bool, double, FinishMode, const float*, float*,
                                double*, double, const ReduceSlots*, cudaStream_t,
                                const PhaseEvents*, int, const SideStream*);

// ---------------------------------------------------------------------------
// Permutations
// ---------------------------------------------------------------------------
__global__ void k_gather(int n, int nc, const int* __restrict__ perm,
                         const double* __restrict__ in, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nc) return;
  const int k = t / nc, c = t - (t / nc) * nc;
  out[t]      = in[(size_t)perm[k] * nc + c];
}
__global__ void k_scatter(int n, int nc, const int* __restrict__ perm,
                          const double* __restrict__ in, double* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * nc) return;
  const int k = t / nc, c = t - (t / nc) * nc;
  out[(size_t)perm[k] * nc + c] = in[t];
}

void permute_in(const Geometry& g, const double* in, double* out, int nc, cudaStream_t s) {
  const int tot = g.n * nc;
  k_gather<<<(tot + 255) / 256, 256, 0, s>>>(g.n, nc, g.perm.p, in, out);
  CG_LAUNCH();
}
void permute_out(const Geometry& g, const double* in, double* out, int nc, cudaStream_t s) {
  const int tot = g.n * nc;
  k_scatter<<<(tot + 255) / 256, 256, 0, s>>>(g.n, nc, g.perm.p, in, out);
  CG_LAUNCH();
}

}  // namespace cg
