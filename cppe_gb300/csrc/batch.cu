// Batched solves: many independent systems (snapshots), each with several
// right-hand sides, solved together.  Every (snapshot, right-hand side) pair
// is a "segment": the segments' geometries are concatenated into one
// Geometry (Geometry::combine) so that each pass of the operator is one
// kernel launch over all segments, and the PCG keeps one set of scalars per
// segment (InducedMoments::compute, src/core/electric_fields.cc:191-239, run
// for every segment at once; a converged segment stops updating).
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <numeric>

#include "batch.h"

namespace cg {

constexpr int BB = 256;
// opening angles of the inexact inner operators (as the single-system solver's)
constexpr double BATCH_INEXACT_THETA[BatchSystem::NINEXACT] = {0.6, 0.8};
// the mixed solve's inner tolerance relative to the residual at its start
constexpr double BATCH_ETA = 3e-6;

// ---------------------------------------------------------------------------
// Geometry concatenation
// ---------------------------------------------------------------------------
void Geometry::combine(const std::vector<const Geometry*>& parts, int copies, Geometry& out) {
  out = Geometry();
  const int np = (int)parts.size();
  std::vector<int> site_off(np + 1, 0);
  for (int g = 0; g < np; ++g) site_off[g + 1] = site_off[g] + parts[g]->n;
  const int nseg = np * copies;
  auto part_of   = [&](int s) { return s / copies; };
  auto copy_of   = [&](int s) { return s % copies; };
  int maxl       = 1;
  bool any_fmm   = false;
  for (auto* p : parts) {
    maxl = std::max(maxl, (int)p->level_start.size() - 1);
    any_fmm |= p->fmm;
  }
  TreeLayout& L = out.layout;
  out.fmm       = any_fmm;
  out.ncrit     = parts[0]->ncrit;
  out.damping   = parts[0]->damping;
  out.theta     = parts[0]->theta;
  out.ncopies   = copies;
  // cells: by (level, segment, cell)
  std::vector<std::vector<int>> cmap(nseg);
  for (int s = 0; s < nseg; ++s) cmap[s].assign(parts[part_of(s)]->layout.ncells, -1);
  L.level_start.assign(maxl + 1, 0);
  int nc = 0;
  for (int l = 0; l < maxl; ++l) {
    L.level_start[l] = nc;
    for (int s = 0; s < nseg; ++s) {
      const Geometry* p = parts[part_of(s)];
      if (l + 1 >= (int)p->level_start.size()) continue;
      for (int c = p->level_start[l]; c < p->level_start[l + 1]; ++c) cmap[s][c] = nc++;
    }
  }
  L.level_start[maxl] = nc;
  L.ncells            = nc;
  L.nlevels           = maxl;
  L.center.assign(4 * (size_t)nc, 0.0);
  L.parent.assign(nc, -1);
  L.is_leaf.assign(nc, 0);
  std::vector<int> seg_of_cell(nc), local_of_cell(nc);
  for (int s = 0; s < nseg; ++s)
    for (int c = 0; c < (int)cmap[s].size(); ++c) {
      const int k      = cmap[s][c];
      seg_of_cell[k]   = s;
      local_of_cell[k] = c;
    }
  out.h_cell_seg = seg_of_cell;
  // the parts' tables of distinct M2L vectors, concatenated (each snapshot
  // keeps its own grid of translation vectors): the FP64 and double-float
  // M2L then read tabulated tensors as they do for one system
  bool tables = true;
  std::vector<int> vec_off(np + 1, 0);
  for (int g = 0; g < np; ++g) {
    const Geometry* p = parts[g];
    if (p->layout.m2l_src.size() != p->h_m2l_vid.size()) tables = false;
    vec_off[g + 1] = vec_off[g] + (int)p->h_vec.size();
  }
  L.child_ptr.assign(nc + 1, 0);
  L.m2l_ptr.assign(nc + 1, 0);
  for (int k = 0; k < nc; ++k) {
    const int s = seg_of_cell[k], c = local_of_cell[k];
    const TreeLayout& P = parts[part_of(s)]->layout;
    for (int q = 0; q < 4; ++q) L.center[4 * (size_t)k + q] = P.center[4 * (size_t)c + q];
    L.parent[k]  = P.parent[c] < 0 ? -1 : cmap[s][P.parent[c]];
    L.is_leaf[k] = P.is_leaf[c];
    for (int q = P.child_ptr[c]; q < P.child_ptr[c + 1]; ++q)
      L.child_idx.push_back(cmap[s][P.child_idx[q]]);
    L.child_ptr[k + 1] = (int)L.child_idx.size();
    for (int q = P.m2l_ptr[c]; q < P.m2l_ptr[c + 1]; ++q) {
      L.m2l_src.push_back(cmap[s][P.m2l_src[q]]);
      if (tables) out.h_m2l_vid.push_back(vec_off[part_of(s)] + parts[part_of(s)]->h_m2l_vid[q]);
    }
    L.m2l_ptr[k + 1] = (int)L.m2l_src.size();
  }
  if (tables && !L.m2l_src.empty())
    for (auto* p : parts) out.h_vec.insert(out.h_vec.end(), p->h_vec.begin(), p->h_vec.end());
  else
    out.h_m2l_vid.clear(), out.h_vec.clear();
  // leaves and particles: segment after segment
  L.leaf_of_cell.assign(nc, -1);
  L.leaf_start.assign(1, 0);
  L.p2p_ptr.assign(1, 0);
  L.n = 0;
  for (int s = 0; s < nseg; ++s) {
    const Geometry* p   = parts[part_of(s)];
    const TreeLayout& P = p->layout;
    const int r = copy_of(s), pi = part_of(s);
    const int leaf0 = (int)L.leaf_cell.size(), site0 = L.n;
    for (int a = 0; a < P.nleaves; ++a) {
      const int k = cmap[s][P.leaf_cell[a]];
      L.leaf_cell.push_back(k);
      out.h_leaf_seg.push_back(s);
      out.h_leaf_copy.push_back(r);
      out.h_leaf_cstride.push_back(make_int2(p->n, P.nleaves));
      L.leaf_of_cell[k] = leaf0 + a;
      L.leaf_start.push_back(site0 + P.leaf_start[a + 1]);
      for (int q = P.p2p_ptr[a]; q < P.p2p_ptr[a + 1]; ++q) L.p2p_src.push_back(leaf0 + P.p2p_src[q]);
      L.p2p_ptr.push_back((int)L.p2p_src.size());
    }
    const int caller0 = copies * site_off[pi] + r * p->n;
    for (int k = 0; k < p->n; ++k) {
      L.perm.push_back(caller0 + P.perm[k]);
      out.h_site_leaf.push_back(leaf0 + p->h_site_leaf[k]);
      out.h_pos64.push_back(p->h_pos64[k]);
      out.h_hi.push_back(p->h_hi[k]);
      out.h_lo.push_back(p->h_lo[k]);
    }
    if (out.h_cptr.empty()) out.h_cptr.push_back(0);
    for (int k = 0; k < p->n; ++k) {
      for (int q = p->h_cptr[k]; q < p->h_cptr[k + 1]; ++q) out.h_cidx.push_back(site0 + p->h_cidx[q]);
      out.h_cptr.push_back((int)out.h_cidx.size());
    }
    L.n += p->n;
    L.p2p_pairs += P.p2p_pairs;
    out.near_pairs += p->near_pairs;
    out.alg_pairs += p->alg_pairs;
  }
  L.nleaves = (int)L.leaf_cell.size();
  out.n     = L.n;
  L.inv_perm.assign(L.n, -1);
  for (int k = 0; k < L.n; ++k) L.inv_perm[L.perm[k]] = k;
  out.level_start = L.level_start;
  out.make_schedules();
}

// ---------------------------------------------------------------------------
// Segmented PCG kernels
// ---------------------------------------------------------------------------
template <typename A, typename B>
__device__ __forceinline__ void bsym3(const A* a, const B* v, B* o) {
  o[0] = (B)(a[0] * v[0] + a[1] * v[1] + a[2] * v[2]);
  o[1] = (B)(a[1] * v[0] + a[3] * v[1] + a[4] * v[2]);
  o[2] = (B)(a[2] * v[0] + a[4] * v[1] + a[5] * v[2]);
}

// Per-segment sums of one or two per-site arrays: block per segment.
__global__ void k_seg_sum(const int* __restrict__ seg_start, const double* __restrict__ a,
                          const double* __restrict__ b, double* __restrict__ oa,
                          double* __restrict__ ob) {
  __shared__ double sh[64];
  const int g = blockIdx.x;
  double v[2] = {0.0, 0.0};
  for (int i = seg_start[g] + threadIdx.x; i < seg_start[g + 1]; i += blockDim.x) {
    v[0] += a[i];
    if (b) v[1] += b[i];
  }
  block_sum<2>(v, sh);
  if (threadIdx.x == 0) {
    oa[g] = v[0];
    if (b) ob[g] = v[1];
  }
}

// r = F - Ax, z = alpha r, p = z per site; site values r.z and r.r.
template <typename T>
__global__ void k_bcg_start(int n, const double* __restrict__ F, const T* __restrict__ Ax,
                            const T* __restrict__ a6, T* __restrict__ r, T* __restrict__ z,
                            T* __restrict__ p, double* __restrict__ s_rz,
                            double* __restrict__ s_rr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  T rv[3], zv[3];
  for (int c = 0; c < 3; ++c) rv[c] = (T)(F[3 * i + c] - (Ax ? (double)Ax[3 * i + c] : 0.0));
  bsym3(a6 + 6 * (size_t)i, rv, zv);
  double rz = 0, rr = 0;
  for (int c = 0; c < 3; ++c) {
    r[3 * i + c] = rv[c], z[3 * i + c] = zv[c], p[3 * i + c] = zv[c];
    rz += (double)rv[c] * zv[c];
    rr += (double)rv[c] * rv[c];
  }
  s_rz[i] = rz, s_rr[i] = rr;
}

__global__ void k_bcg_init_seg(int nseg, const double* __restrict__ rz, const double* __restrict__ rr,
                               double* __restrict__ seg_rz, double* __restrict__ seg_rnorm,
                               int* __restrict__ done, int* __restrict__ iters,
                               const double* __restrict__ tol) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nseg) return;
  seg_rz[g]    = rz[g];
  seg_rnorm[g] = sqrt(rr[g]);
  iters[g]     = 0;
  // a segment whose residual already meets its tolerance takes no step
  done[g] = (tol && seg_rnorm[g] < tol[g]) ? 1 : 0;
}

template <typename T>
__global__ void k_bcg_update(int n, const int* __restrict__ site_seg, const T* __restrict__ p,
                             const T* __restrict__ Ap, const T* __restrict__ a6,
                             T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                             const double* __restrict__ seg_rz, const double* __restrict__ seg_pap,
                             const int* __restrict__ done, double* __restrict__ s_rr,
                             double* __restrict__ s_rz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = site_seg[i];
  if (done[g]) {
    s_rr[i] = 0.0, s_rz[i] = 0.0;
    return;
  }
  const T a = (T)(seg_rz[g] / seg_pap[g]);
  T rv[3], zv[3];
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)i + c;
    x[k] += a * p[k];
    rv[c] = r[k] - a * Ap[k];
    r[k]  = rv[c];
  }
  bsym3(a6 + 6 * (size_t)i, rv, zv);
  double rr = 0, rz = 0;
  for (int c = 0; c < 3; ++c) {
    z[3 * (size_t)i + c] = zv[c];
    rr += (double)rv[c] * rv[c];
    rz += (double)rv[c] * zv[c];
  }
  s_rr[i] = rr, s_rz[i] = rz;
}

// Per segment: ||r||, beta, convergence; counts the segments still running.
__global__ void k_bcg_finalize(int nseg, const double* __restrict__ rr,
                               const double* __restrict__ rznew, double* __restrict__ seg_rz,
                               double* __restrict__ seg_beta, double* __restrict__ seg_rnorm,
                               int* __restrict__ done, int* __restrict__ iters,
                               const double* __restrict__ tol, int maxiter,
                               int* __restrict__ active) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nseg) return;
  if (done[g]) return;
  const double rn = sqrt(rr[g]);
  seg_rnorm[g]    = rn;
  seg_beta[g]     = rznew[g] / seg_rz[g];
  seg_rz[g]       = rznew[g];
  const int it    = iters[g] + 1;
  iters[g]        = it;
  if (rn < tol[g])
    done[g] = 1;
  else if (it >= maxiter)
    done[g] = 2;
  else
    atomicAdd(active, 1);
}

template <typename T>
__global__ void k_bcg_dir(int n, const int* __restrict__ site_seg, const T* __restrict__ z,
                          T* __restrict__ p, const double* __restrict__ seg_beta,
                          const int* __restrict__ done) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int g = site_seg[i];
  if (done[g]) return;
  const T b = (T)seg_beta[g];
  for (int c = 0; c < 3; ++c) p[3 * i + c] = z[3 * i + c] + b * p[3 * i + c];
}

__global__ void k_bres(int n, const double* __restrict__ F, const double* __restrict__ Ax,
                       const float* __restrict__ Bd, double* __restrict__ r,
                       double* __restrict__ s_rr, const float* __restrict__ r32 = nullptr) {
  // r = F - Ax (Ax given), r -= Bd (Bd given) or r = (r - fl(r)) + r32 (the
  // inner solve's final residual r32 for the right-hand side fl(r)); site
  // values of r.r
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double rr = 0;
  for (int c = 0; c < 3; ++c) {
    const size_t k = 3 * (size_t)i + c;
    const double v = Ax   ? F[k] - Ax[k]
                     : Bd ? r[k] - (double)Bd[k]
                          : (r[k] - (double)(float)r[k]) + (double)r32[k];
    r[k]           = v;
    rr += v * v;
  }
  s_rr[i] = rr;
}

__global__ void k_bsqrt(int nseg, const double* __restrict__ rr, double* __restrict__ rn) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < nseg) rn[g] = sqrt(rr[g]);
}

__global__ void k_bacc(int n3, double* __restrict__ x, float* __restrict__ d) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) x[k] += (double)d[k], d[k] = 0.f;
}

__global__ void k_bf32(int n3, const double* __restrict__ a, float* __restrict__ b) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n3) b[k] = (float)a[k];
}

__global__ void k_bguess(int n, const double* __restrict__ a6, const double* __restrict__ F,
                         double* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) bsym3(a6 + 6 * (size_t)i, F + 3 * (size_t)i, x + 3 * (size_t)i);
}

// ---------------------------------------------------------------------------
// BatchSystem
// ---------------------------------------------------------------------------
// Per operator level L (0: the operator, 1 + k: inexact operator k), the
// segments its pass leaves out: finished ones and those at another level.
__global__ void k_blevel_masks(int nseg, int nlev, const int* __restrict__ done,
                               const int* __restrict__ level, int* __restrict__ m0,
                               int* __restrict__ m1, int* __restrict__ m2) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= nseg) return;
  const int d = done[g] != 0, l = level[g];
  m0[g] = d || l != 0;
  if (nlev > 1) m1[g] = d || l != 1;
  if (nlev > 2) m2[g] = d || l != 2;
}

// Whether some running segment is at each operator level: the conditions of
// the graph's per-level passes.
__global__ void k_blevel_any(int nseg, int nlev, const int* __restrict__ done,
                             const int* __restrict__ level, cudaGraphConditionalHandle h0,
                             cudaGraphConditionalHandle h1, cudaGraphConditionalHandle h2) {
  int a0 = 0, a1 = 0, a2 = 0;
  for (int g = threadIdx.x; g < nseg; g += blockDim.x)
    if (!done[g]) {
      const int l = level[g];
      a0 |= l == 0, a1 |= l == 1, a2 |= l == 2;
    }
  a0 = __syncthreads_or(a0);
  a1 = __syncthreads_or(a1);
  a2 = __syncthreads_or(a2);
  if (threadIdx.x == 0) {
    cudaGraphSetConditional(h0, a0 ? 1u : 0u);
    if (nlev > 1) cudaGraphSetConditional(h1, a1 ? 1u : 0u);
    if (nlev > 2) cudaGraphSetConditional(h2, a2 ? 1u : 0u);
  }
}

// Hand-over of a snapshot's running segments (its right-hand sides) to the
// next inexact operator once every one of them is below that operator's
// hand-over point (sw <= 0: never).  The right-hand sides of a snapshot move
// together, so that the near-field pass keeps serving them all from one
// pair tensor.  The residual at the hand-over is kept for the error bound of
// the residual formed from the recursion.
__global__ void k_blevel_update(int nsys, int nrhs, int nx, const double* __restrict__ rnorm,
                                const int* __restrict__ done, int* __restrict__ level,
                                const double* __restrict__ sw0, const double* __restrict__ sw1,
                                double* __restrict__ rsw0, double* __restrict__ rsw1) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  const int g0 = s * nrhs;
  bool any = false, all0 = nx > 0, all1 = nx > 1;
  int l = 0;
  for (int r = 0; r < nrhs; ++r) {
    const int g = g0 + r;
    if (done[g]) continue;
    any = true;
    l   = level[g];  // the same for every running right-hand side
    const double rn = rnorm[g];
    all0 = all0 && rn < sw0[g];
    all1 = all1 && rn < sw1[g];
  }
  if (!any) return;
  const int nl = l == 0 && all0 ? (all1 ? 2 : 1) : (l == 1 && all1 ? 2 : l);
  if (nl == l) return;
  for (int r = 0; r < nrhs; ++r) {
    const int g = g0 + r;
    if (done[g]) continue;
    if (l == 0) rsw0[g] = rnorm[g];
    if (nl == 2) rsw1[g] = rnorm[g];
    level[g] = nl;
  }
}

// The tolerances and hand-over points of a mixed solve's inner solve, per
// snapshot (its right-hand sides share the operator level), from the
// residual norms at its start: stage 0 for the first inner solve, stage 1
// for later ones, where segments whose residual plus its error bound rerr is
// already below the threshold are done at once.
// With inexact operators (nx > 0) also the hand-over points and the starting
// levels: stage 0 hands over where the operator's effect delta ||r|| stays
// below 0.6 of the target eta ||r0||, stage 1 where 1.5 delta ||r|| stays
// below 0.18 t; a snapshot already below a point starts at its level.
__global__ void k_bstage(int nsys, int nrhs, int nx, int stage, double t, double eta,
                         double rerr, const double* __restrict__ rnorm,
                         const double* __restrict__ d0,
                         const double* __restrict__ d1, double* __restrict__ tol,
                         double* __restrict__ sw0, double* __restrict__ sw1,
                         double* __restrict__ rsw0, double* __restrict__ rsw1,
                         int* __restrict__ level) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  bool any = false, all0 = true, all1 = nx > 1;
  for (int r = 0; r < nrhs; ++r) {
    const int g     = s * nrhs + r;
    const double rn = rnorm[g];
    double tl       = fmax(eta * rn, 0.5 * t);
    if (stage > 0 && rn + rerr < t) tl = 1e300;
    tol[g] = tl;
    if (nx == 0) continue;
    auto sw = [&](double d) {
      return d > 0.0 ? fmax(tl, stage == 0 ? 0.6 * eta * rn / d : 0.18 * t / (1.5 * d)) : -1.0;
    };
    const double s0 = sw(d0[g]);
    const double s1 = nx > 1 && s0 > 0.0 ? fmin(s0, sw(d1[g])) : -1.0;
    sw0[g] = s0, sw1[g] = s1;
    if (rn < tl) continue;  // done at once
    any  = true;
    all0 = all0 && rn < s0;
    all1 = all1 && rn < s1;
  }
  if (nx == 0) return;
  const int l = !any ? 0 : (all0 ? (all1 ? 2 : 1) : 0);
  for (int r = 0; r < nrhs; ++r) {
    const int g = s * nrhs + r;
    level[g]    = l;
    rsw0[g]     = l > 0 ? rnorm[g] : 0.0;
    rsw1[g]     = l == 2 ? rnorm[g] : 0.0;
  }
}

BatchSystem::~BatchSystem() {
  if (stream) {
    cudaSetDevice(device);
    cudaStreamSynchronize(stream);
    if (side.s) cudaStreamSynchronize(side.s);
    side.destroy();
    cudaStreamDestroy(stream);
    if (cap_stream) cudaStreamDestroy(cap_stream);
    if (cap_stream2) cudaStreamDestroy(cap_stream2);
  }
  for (auto& e : pcg_exec)
    if (e) cudaGraphExecDestroy(e);
  if (course_exec) cudaGraphExecDestroy(course_exec);
  if (h_active) cudaFreeHost(h_active);
}

void BatchSystem::init(int nsys, const int* site_offset, const double* xyz, const double* alpha6,
                       const int* excl_ptr, const int* excl_idx, int nrhs_, int direct_below,
                       const cppe_gpu_options& o) {
  opt  = o;
  nrhs = nrhs_;
  if (nsys < 1 || nrhs < 1) fail(CPPE_GPU_INVALID_ARG, "empty batch");
  int ndev = 0;
  CG_CUDA(cudaGetDeviceCount(&ndev));
  if (o.device < 0 || o.device >= ndev) fail(CPPE_GPU_INVALID_ARG, "bad CUDA device ordinal");
  device = o.device;
  CG_CUDA(cudaSetDevice(device));
  CG_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  CG_CUDA(cudaStreamCreateWithFlags(&cap_stream, cudaStreamNonBlocking));
  CG_CUDA(cudaStreamCreateWithFlags(&cap_stream2, cudaStreamNonBlocking));
  if_stream = cap_stream;
  side.create();
  if (o.tree_expansion_order < 2 || o.tree_expansion_order > 7)
    fail(CPPE_GPU_INVALID_ARG, "tree_expansion_order must be in [2, 7]");
  std::vector<Geometry> parts(nsys);
  std::vector<const Geometry*> pp;
  // the inexact inner operators' parts (FMM snapshots; a direct snapshot
  // serves every level as it is)
  const bool want_x = o.precision == CPPE_GPU_MIXED;
  std::vector<Geometry> parts_x[NINEXACT];
  bool x_ok[NINEXACT];
  for (int k = 0; k < NINEXACT; ++k) {
    x_ok[k] = want_x && o.theta < BATCH_INEXACT_THETA[k];
    if (x_ok[k]) parts_x[k].resize(nsys);
  }
  std::vector<char> sys_fmm(nsys, 0);
  std::vector<double> a_inv, a_dir;
  sys_sites.assign(site_offset, site_offset + nsys + 1);
  for (int s = 0; s < nsys; ++s) {
    const int o0 = site_offset[s], ns = site_offset[s + 1] - o0;
    if (ns < 1) fail(CPPE_GPU_INVALID_ARG, "snapshot without sites");
    std::vector<double> sd(ns, 0.0);
    for (int i = 0; i < ns; ++i) {
      const double* a = alpha6 + 6 * (size_t)(o0 + i);
      const double iso = (a[0] + a[3] + a[5]) / 3.0;
      if (o.damp && iso > 0.0) sd[i] = std::pow(iso, -1.0 / 6.0);
    }
    std::vector<int> ep, ei;
    if (excl_ptr) {
      ep.resize(ns + 1);
      for (int i = 0; i <= ns; ++i) ep[i] = excl_ptr[o0 + i] - excl_ptr[o0];
      ei.assign(excl_idx + excl_ptr[o0], excl_idx + excl_ptr[o0 + ns]);
    }
    const bool fmm = ns >= direct_below;
    sys_fmm[s]       = fmm;
    parts[s].damping = o.damp ? o.damping_factor : 0.0;
    parts[s].prepare(ns, xyz + 3 * (size_t)o0, sd.data(), excl_ptr ? ep.data() : nullptr,
                     ei.empty() ? nullptr : ei.data(), fmm, o.tree_ncrit, o.theta);
    pp.push_back(&parts[s]);
    for (int k = 0; k < NINEXACT; ++k) {
      if (!x_ok[k] || !fmm) continue;
      Geometry& gx = parts_x[k][s];
      gx.damping   = parts[s].damping;
      gx.prepare(ns, xyz + 3 * (size_t)o0, sd.data(), excl_ptr ? ep.data() : nullptr,
                 ei.empty() ? nullptr : ei.data(), true, o.tree_ncrit, BATCH_INEXACT_THETA[k]);
      // the opening angle changes the lists, not the tree: same site order
      if (gx.layout.perm != parts[s].layout.perm) x_ok[k] = false;
    }
  }
  Geometry::combine(pp, nrhs, geo);
  geo.upload(stream);
  const bool any_fmm = std::any_of(sys_fmm.begin(), sys_fmm.end(), [](char f) { return f; });
  n_inexact = 0;
  for (int k = 0; k < NINEXACT && any_fmm && x_ok[k]; ++k) {
    std::vector<const Geometry*> ppx(nsys);
    for (int s = 0; s < nsys; ++s) ppx[s] = sys_fmm[s] ? &parts_x[k][s] : &parts[s];
    Geometry::combine(ppx, nrhs, geo_x[k]);
    if (geo_x[k].layout.perm != geo.layout.perm) break;
    geo_x[k].upload(stream);
    n_inexact = k + 1;
  }
  for (auto& v : parts_x) v.clear();
  if (geo.fmm) {
    ops = std::make_unique<DeviceOps>();
    ops->build(1, o.tree_expansion_order, stream);
  }
  n    = geo.n;
  nseg = nsys * nrhs;
  // segments in device order and per-site operator data
  std::vector<int> seg_start_h(nseg + 1, 0), site_seg_h(n);
  {
    int k = 0;
    for (int s = 0; s < nsys; ++s)
      for (int r = 0; r < nrhs; ++r) {
        const int ns = site_offset[s + 1] - site_offset[s];
        for (int i = 0; i < ns; ++i) site_seg_h[k + i] = s * nrhs + r;
        k += ns;
        seg_start_h[s * nrhs + r + 1] = k;
      }
  }
  std::vector<double> ainv(6 * (size_t)n), al(6 * (size_t)n);
  for (int k = 0; k < n; ++k) {
    // caller index -> (system, site)
    const int c  = geo.layout.perm[k];
    const int g  = site_seg_h[k];
    const int sy = g / nrhs;
    const int ns = site_offset[sy + 1] - site_offset[sy];
    const int local = (c - nrhs * site_offset[sy]) % ns;
    const double* a = alpha6 + 6 * (size_t)(site_offset[sy] + local);
    const double A = a[3] * a[5] - a[4] * a[4], B = a[2] * a[4] - a[1] * a[5],
                 C = a[1] * a[4] - a[2] * a[3];
    const double id = 1.0 / (a[0] * A + a[1] * B + a[2] * C);
    double* iv = &ainv[6 * (size_t)k];
    iv[0] = A * id, iv[1] = B * id, iv[2] = C * id, iv[3] = (a[0] * a[5] - a[2] * a[2]) * id;
    iv[4] = (a[1] * a[2] - a[0] * a[4]) * id, iv[5] = (a[0] * a[3] - a[1] * a[1]) * id;
    std::copy(a, a + 6, &al[6 * (size_t)k]);
  }
  std::vector<float> ainvf(ainv.begin(), ainv.end()), alf(al.begin(), al.end());
  ainv64.upload(ainv, stream);
  alpha64.upload(al, stream);
  ainv32.upload(ainvf, stream);
  alpha32.upload(alf, stream);
  seg_start.upload(seg_start_h, stream);
  site_seg.upload(site_seg_h, stream);
  const size_t n3 = 3 * (size_t)n;
  for (auto* b : {&F, &x, &r, &z, &p, &Ap}) b->alloc(n3);
  for (auto* b : {&r32, &z32, &p32, &Ap32, &d32}) b->alloc(n3);
  for (auto* b : {&site_a, &site_b}) b->alloc(n);
  for (auto* b : {&seg_rz, &seg_pap, &seg_rr, &seg_rznew, &seg_beta, &seg_rnorm, &seg_tol})
    b->alloc(nseg);
  done.alloc(nseg);
  iters.alloc(nseg);
  active.alloc(1);
  CG_CUDA(cudaMallocHost(&h_active, sizeof(int)));
  if (n_inexact > 0) {
    std::vector<char> seg_fmm(nseg);
    for (int g = 0; g < nseg; ++g) seg_fmm[g] = sys_fmm[g / nrhs];
    measure_inexact(seg_start_h, seg_fmm);
  }
  CG_CUDA(cudaStreamSynchronize(stream));
}

template <typename T>
void BatchSystem::apply_seg(const T* in, T* out, int near_mode, bool skip_done) {
  ReduceSlots rs{nullptr, nullptr, nullptr};
  rs.site_values = site_a.p;
  FieldWork<T>& w = work<T>();
  const T* ainv   = std::is_same<T, double>::value ? (const T*)ainv64.p : (const T*)ainv32.p;
  eval_field<T>(geo, ops.get(), w, 1, in, opt.damp != 0, opt.damping_factor, FINISH_APPLY, ainv,
                out, nullptr, 1.0, &rs, stream, nullptr, near_mode, nested_body ? nullptr : &side,
                skip_done ? done.p : nullptr);
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, nullptr, seg_pap.p, nullptr);
  CG_LAUNCH();
}

void BatchSystem::apply_level32(int k, const float* in, float* out, const int* mask) {
  ReduceSlots rs{nullptr, nullptr, nullptr};
  rs.site_values = site_a.p;
  eval_field<float>(geo_x[k], ops.get(), w32x[k], 1, in, opt.damp != 0, opt.damping_factor,
                    FINISH_APPLY, ainv32.p, out, nullptr, 1.0, &rs, stream, nullptr, NEAR_FP64,
                    &side, mask);
}

// The iteration's FP32 operator: each running segment with the operator of
// its level (the passes of the other operators skip it), then the segments'
// p.Ap sums.
void BatchSystem::apply_levels32(const float* in, float* out) {
  const int gb = (nseg + 127) / 128;
  k_blevel_masks<<<gb, 128, 0, stream>>>(nseg, 1 + n_inexact, done.p, seg_level.p,
                                         lvl_mask[0].p, lvl_mask[1].p, lvl_mask[2].p);
  CG_LAUNCH();
  ReduceSlots rs{nullptr, nullptr, nullptr};
  rs.site_values = site_a.p;
  eval_field<float>(geo, ops.get(), w32, 1, in, opt.damp != 0, opt.damping_factor, FINISH_APPLY,
                    ainv32.p, out, nullptr, 1.0, &rs, stream, nullptr, NEAR_FP64, &side,
                    lvl_mask[0].p);
  for (int k = 0; k < n_inexact; ++k) apply_level32(k, in, out, lvl_mask[1 + k].p);
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, nullptr, seg_pap.p, nullptr);
  CG_LAUNCH();
}

void BatchSystem::apply_levels32_graph(const float* in, float* out) {
  const int gb = (nseg + 127) / 128, nlev = 1 + n_inexact;
  k_blevel_masks<<<gb, 128, 0, stream>>>(nseg, nlev, done.p, seg_level.p, lvl_mask[0].p,
                                         lvl_mask[1].p, lvl_mask[2].p);
  CG_LAUNCH();
  cudaStreamCaptureStatus st{};
  cudaGraph_t cg = nullptr;
  CG_CUDA(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive || !cg)
    fail(CPPE_GPU_CUDA_ERROR, "per-level passes outside a graph capture");
  cudaGraphConditionalHandle hl[1 + NINEXACT] = {};
  for (int l = 0; l < nlev; ++l)
    CG_CUDA(cudaGraphConditionalHandleCreate(&hl[l], cg, 0, cudaGraphCondAssignDefault));
  k_blevel_any<<<1, 256, 0, stream>>>(nseg, nlev, done.p, seg_level.p, hl[0], hl[1],
                                      hl[NINEXACT]);
  CG_LAUNCH();
  ReduceSlots rs{nullptr, nullptr, nullptr};
  rs.site_values = site_a.p;
  for (int l = 0; l < nlev; ++l) {
    // a conditional node after the capture's current tip; the stream's
    // later work follows it
    const cudaGraphNode_t* deps = nullptr;
    size_t nd                   = 0;
    CG_CUDA(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, &deps, nullptr, &nd));
    cudaGraphNodeParams ip{};
    ip.type               = cudaGraphNodeTypeConditional;
    ip.conditional.handle = hl[l];
    ip.conditional.type   = cudaGraphCondTypeIf;
    ip.conditional.size   = 1;
    cudaGraphNode_t node{};
    CG_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, nd, &ip));
    CG_CUDA(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1,
                                                cudaStreamSetCaptureDependencies));
    // the pass itself, captured into the node's body
    CG_CUDA(cudaStreamBeginCaptureToGraph(if_stream, ip.conditional.phGraph_out[0], nullptr,
                                          nullptr, 0, cudaStreamCaptureModeThreadLocal));
    try {
      if (l == 0)
        eval_field<float>(geo, ops.get(), w32, 1, in, opt.damp != 0, opt.damping_factor,
                          FINISH_APPLY, ainv32.p, out, nullptr, 1.0, &rs, if_stream, nullptr,
                          NEAR_FP64, nullptr, lvl_mask[0].p);
      else
        eval_field<float>(geo_x[l - 1], ops.get(), w32x[l - 1], 1, in, opt.damp != 0,
                          opt.damping_factor, FINISH_APPLY, ainv32.p, out, nullptr, 1.0, &rs,
                          if_stream, nullptr, NEAR_FP64, nullptr, lvl_mask[l].p);
    } catch (...) {
      cudaGraph_t dropped = nullptr;
      cudaStreamEndCapture(if_stream, &dropped);
      throw;
    }
    cudaGraph_t captured = nullptr;
    CG_CUDA(cudaStreamEndCapture(if_stream, &captured));
  }
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, nullptr, seg_pap.p, nullptr);
  CG_LAUNCH();
}

// Each segment's relative difference between the operator (double-float)
// and each inexact FP32 operator on a random vector and on a smooth one (the
// response to a uniform field), times 3 as the bound delta used for the
// hand-over points; a segment whose difference reaches 1e-2, or a direct
// snapshot's segment, keeps the operator throughout.
void BatchSystem::measure_inexact(const std::vector<int>& seg_start_h,
                                  const std::vector<char>& seg_fmm) {
  const size_t n3 = 3 * (size_t)n;
  seg_level.alloc(nseg);
  for (int k = 0; k <= NINEXACT; ++k) lvl_mask[k].alloc(nseg);
  for (int k = 0; k < NINEXACT; ++k) seg_sw[k].alloc(nseg), seg_rsw[k].alloc(nseg);
  std::vector<double> vin[2] = {std::vector<double>(n3), std::vector<double>(n3)};
  unsigned long long st = 0x9e3779b97f4a7c15ull;
  for (size_t k = 0; k < n3; ++k) {
    st ^= st << 13, st ^= st >> 7, st ^= st << 17;
    vin[0][k] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    vin[1][k] = (k % 3 == 0) ? 1.0 : (k % 3 == 1 ? 0.5 : 0.25);
  }
  std::vector<double> a64(n3), ax(n3);
  std::vector<float> in32(n3), out32(n3);
  std::vector<double> worst[NINEXACT];
  for (int k = 0; k < n_inexact; ++k) worst[k].assign(nseg, 0.0);
  auto seg_rel = [&](const std::vector<double>& ref, const std::vector<double>& got, int g) {
    double num = 0.0, den = 0.0;
    for (size_t q = 3 * (size_t)seg_start_h[g]; q < 3 * (size_t)seg_start_h[g + 1]; ++q) {
      const double d = got[q] - ref[q];
      num += d * d, den += ref[q] * ref[q];
    }
    return den > 0.0 ? std::sqrt(num / den) : 0.0;
  };
  for (int trial = 0; trial < 2; ++trial) {
    CG_CUDA(cudaMemcpyAsync(x.p, vin[trial].data(), n3 * sizeof(double), cudaMemcpyHostToDevice,
                            stream));
    apply_seg<double>(x.p, Ap.p, NEAR_DD);
    CG_CUDA(cudaMemcpyAsync(a64.data(), Ap.p, n3 * sizeof(double), cudaMemcpyDeviceToHost,
                            stream));
    for (size_t q = 0; q < n3; ++q) in32[q] = (float)vin[trial][q];
    CG_CUDA(cudaMemcpyAsync(p32.p, in32.data(), n3 * sizeof(float), cudaMemcpyHostToDevice,
                            stream));
    for (int k = 0; k < n_inexact; ++k) {
      apply_level32(k, p32.p, Ap32.p, nullptr);
      CG_CUDA(cudaMemcpyAsync(out32.data(), Ap32.p, n3 * sizeof(float), cudaMemcpyDeviceToHost,
                              stream));
      CG_CUDA(cudaStreamSynchronize(stream));
      for (size_t q = 0; q < n3; ++q) ax[q] = out32[q];
      for (int g = 0; g < nseg; ++g) worst[k][g] = std::max(worst[k][g], seg_rel(a64, ax, g));
    }
  }
  for (int k = 0; k < NINEXACT; ++k) h_delta[k].assign(nseg, 0.0);
  for (int g = 0; g < nseg; ++g) {
    if (!seg_fmm[g]) continue;
    for (int k = 0; k < n_inexact; ++k) {
      const double d = 3.0 * worst[k][g];
      if (!(worst[k][g] > 0.0 && d < 1e-2)) break;  // this level and the ones after it off
      h_delta[k][g] = d;
    }
  }
  for (int k = 0; k < NINEXACT; ++k) seg_delta_d[k].upload(h_delta[k], stream);
  CG_CUDA(cudaStreamSynchronize(stream));
}

// Sets the first condition of the batched loop: some segment still running.
__global__ void k_bcg_any(cudaGraphConditionalHandle h, int nseg, const int* __restrict__ done,
                          int* __restrict__ active) {
  int any = 0;
  for (int g = threadIdx.x; g < nseg; g += blockDim.x) any |= done[g] == 0;
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    *active = 0;
    cudaGraphSetConditional(h, any ? 1u : 0u);
  }
}

// Continues the batched loop while k_bcg_finalize counted a running segment.
__global__ void k_bcg_continue(cudaGraphConditionalHandle h, int* __restrict__ active) {
  const int a = *active;
  *active     = 0;
  cudaGraphSetConditional(h, a > 0 ? 1u : 0u);
}

// One PCG iteration over every segment; kernels of converged segments are
// no-ops.  Host-launched, the running-segment counter is cleared here; in the
// graph k_bcg_any / k_bcg_continue clear it.
template <typename T>
void BatchSystem::pcg_iteration(T* xv, T* rv, T* zv, T* pv, T* Apv, const T* a6, int maxiter,
                                bool graph) {
  const int nb = (n + BB - 1) / BB, gb = (nseg + 127) / 128;
  // the near field of finished segments is skipped: their p, Ap and scalars
  // are no longer read; in FP32 with inexact operators each segment takes
  // the operator of its level
  bool levels = false;
  if constexpr (std::is_same<T, float>::value) levels = n_inexact > 0;
  if constexpr (std::is_same<T, float>::value) {
    if (levels && graph)
      apply_levels32_graph(pv, Apv);
    else if (levels)
      apply_levels32(pv, Apv);
  }
  if (!levels) apply_seg<T>(pv, Apv, NEAR_FP64, true);
  k_bcg_update<T><<<nb, BB, 0, stream>>>(n, site_seg.p, pv, Apv, a6, xv, rv, zv, seg_rz.p,
                                         seg_pap.p, done.p, site_a.p, site_b.p);
  CG_LAUNCH();
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rr.p, seg_rznew.p);
  CG_LAUNCH();
  if (!graph) CG_CUDA(cudaMemsetAsync(active.p, 0, sizeof(int), stream));
  k_bcg_finalize<<<gb, 128, 0, stream>>>(nseg, seg_rr.p, seg_rznew.p, seg_rz.p, seg_beta.p,
                                         seg_rnorm.p, done.p, iters.p, seg_tol.p, maxiter,
                                         active.p);
  CG_LAUNCH();
  if (levels) {
    const int nsys = nseg / nrhs;
    k_blevel_update<<<(nsys + 127) / 128, 128, 0, stream>>>(
          nsys, nrhs, n_inexact, seg_rnorm.p, done.p, seg_level.p, seg_sw[0].p, seg_sw[1].p,
          seg_rsw[0].p, seg_rsw[1].p);
    CG_LAUNCH();
  }
  k_bcg_dir<T><<<nb, BB, 0, stream>>>(n, site_seg.p, zv, pv, seg_beta.p, done.p);
  CG_LAUNCH();
}

template <typename T>
bool BatchSystem::pcg_graph_ready(T* xv, T* rv, T* zv, T* pv, T* Apv, const T* a6, int maxiter) {
  const int v = std::is_same<T, double>::value ? 0 : 1;
  static const bool graphs = [] {
    const char* e = std::getenv("CPPE_GPU_GRAPHS");
    return !(e && e[0] == '0');
  }();
  if (!graphs) pcg_graph_failed = true;
  if (!pcg_exec[v] && !pcg_graph_failed) {
    cudaGraph_t g = nullptr;
    bool ok       = cudaGraphCreate(&g, 0) == cudaSuccess;
    cudaGraphConditionalHandle h{};
    ok = ok && cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) ==
                     cudaSuccess;
    cudaGraphNode_t pre{}, node{};
    cudaGraphNodeParams np{};
    if (ok) {
      ok = cudaStreamBeginCaptureToGraph(stream, g, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        k_bcg_any<<<1, 256, 0, stream>>>(h, nseg, done.p, active.p);
        ok = cudaGetLastError() == cudaSuccess;
        cudaGraph_t captured = nullptr;
        ok = (cudaStreamEndCapture(stream, &captured) == cudaSuccess) && ok;
      }
      size_t nn = 1;
      ok = ok && cudaGraphGetNodes(g, &pre, &nn) == cudaSuccess && nn == 1;
    }
    if (ok) {
      np.type               = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type   = cudaGraphCondTypeWhile;
      np.conditional.size   = 1;
      ok = cudaGraphAddNode(&node, g, &pre, nullptr, 1, &np) == cudaSuccess;
    }
    if (ok) {
      cudaGraph_t body = np.conditional.phGraph_out[0];
      ok = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal) == cudaSuccess;
      if (ok) {
        const long long c0 = launch_counter();
        try {
          CaptureScope cs;
          pcg_iteration<T>(xv, rv, zv, pv, Apv, a6, maxiter, true);
          k_bcg_continue<<<1, 1, 0, stream>>>(h, active.p);
          CG_LAUNCH();
        } catch (const Failure&) {
          ok = false;
        }
        pcg_body_launches[v] = launch_counter() - c0;
        launch_counter()     = c0;
        cudaGraph_t captured = nullptr;
        ok = (cudaStreamEndCapture(stream, &captured) == cudaSuccess) && ok;
      }
    }
    if (ok) ok = cudaGraphInstantiate(&pcg_exec[v], g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      cudaGetLastError();  // clear the refusal; fall back to host-launched iterations
      if (pcg_exec[v]) cudaGraphExecDestroy(pcg_exec[v]);
      pcg_exec[v]      = nullptr;
      pcg_graph_failed = true;
    }
  }
  return pcg_exec[v] != nullptr;
}

template <typename T>
int BatchSystem::run_pcg(T* xv, T* rv, T* zv, T* pv, T* Apv, const T* a6, int maxiter) {
  // (r, z, p, per-segment rz / rnorm / done / iters set by the caller's start step)
  const int v = std::is_same<T, double>::value ? 0 : 1;
  int k       = 0;
  if (pcg_graph_ready<T>(xv, rv, zv, pv, Apv, a6, maxiter)) {
    // the whole loop on the device; iterations = the largest segment count
    CG_CUDA(cudaGraphLaunch(pcg_exec[v], stream));
    h_iters.resize(nseg);
    CG_CUDA(cudaMemcpyAsync(h_iters.data(), iters.p, nseg * sizeof(int), cudaMemcpyDeviceToHost,
                            stream));
    host_wait();
    k = *std::max_element(h_iters.begin(), h_iters.end());
    launch_counter() += pcg_body_launches[v] * k + 1;
  } else {
    for (; k < maxiter; ++k) {
      pcg_iteration<T>(xv, rv, zv, pv, Apv, a6, maxiter, false);
      CG_CUDA(cudaMemcpyAsync(h_active, active.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
      host_wait();
      if (*h_active == 0) {
        ++k;
        break;
      }
    }
  }
  if (std::is_same<T, double>::value)
    stats.fp64_applies += k;
  else
    stats.fp32_applies += k;
  return k;
}

double BatchSystem::autotune(int reps) {
  CG_CUDA(cudaSetDevice(device));
  CG_CUDA(cudaMemsetAsync(p32.p, 0, sizeof(float) * 3 * (size_t)n, stream));
  const double best = autotune_schedule(geo, side, stream, reps,
                                        [&] { apply_seg<float>(p32.p, Ap32.p); });
  // captured loops hold the old schedule's buffers: rebuild on next use
  for (auto& e : pcg_exec)
    if (e) cudaGraphExecDestroy(e), e = nullptr;
  if (course_exec) cudaGraphExecDestroy(course_exec), course_exec = nullptr;
  return best;
}

void BatchSystem::capture_pcg_loop(int maxiter) {
  cudaStreamCaptureStatus st{};
  cudaGraph_t cg = nullptr;
  CG_CUDA(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, nullptr, nullptr, nullptr));
  if (st != cudaStreamCaptureStatusActive || !cg)
    fail(CPPE_GPU_CUDA_ERROR, "inner solve outside a graph capture");
  cudaGraphConditionalHandle h{};
  CG_CUDA(cudaGraphConditionalHandleCreate(&h, cg, 0, cudaGraphCondAssignDefault));
  k_bcg_any<<<1, 256, 0, stream>>>(h, nseg, done.p, active.p);
  CG_LAUNCH();
  const cudaGraphNode_t* deps = nullptr;
  size_t nd                   = 0;
  CG_CUDA(cudaStreamGetCaptureInfo(stream, &st, nullptr, &cg, &deps, nullptr, &nd));
  cudaGraphNodeParams wp{};
  wp.type               = cudaGraphNodeTypeConditional;
  wp.conditional.handle = h;
  wp.conditional.type   = cudaGraphCondTypeWhile;
  wp.conditional.size   = 1;
  cudaGraphNode_t node{};
  CG_CUDA(cudaGraphAddNode(&node, cg, deps, nullptr, nd, &wp));
  CG_CUDA(cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1,
                                              cudaStreamSetCaptureDependencies));
  // the body on the second capture stream; its per-level passes on the third
  CG_CUDA(cudaStreamBeginCaptureToGraph(cap_stream, wp.conditional.phGraph_out[0], nullptr,
                                        nullptr, 0, cudaStreamCaptureModeThreadLocal));
  const cudaStream_t outer = stream, outer_if = if_stream;
  stream = cap_stream, if_stream = cap_stream2, nested_body = true;
  const long long c0 = launch_counter();
  try {
    pcg_iteration<float>(d32.p, r32.p, z32.p, p32.p, Ap32.p, alpha32.p, maxiter, true);
    k_bcg_continue<<<1, 1, 0, stream>>>(h, active.p);
    CG_LAUNCH();
  } catch (...) {
    stream = outer, if_stream = outer_if, nested_body = false;
    launch_counter()    = c0;
    cudaGraph_t dropped = nullptr;
    cudaStreamEndCapture(cap_stream, &dropped);
    throw;
  }
  course_body_launches = launch_counter() - c0;
  launch_counter()     = c0;
  stream = outer, if_stream = outer_if, nested_body = false;
  cudaGraph_t captured = nullptr;
  CG_CUDA(cudaStreamEndCapture(cap_stream, &captured));
}

// The usual course of a mixed solve from the guess x = alpha F, as
// solve_device's host loop runs it when every choice goes the usual way.
void BatchSystem::course_body(int maxiter) {
  const int nb = (n + BB - 1) / BB, n3 = 3 * n, nb3 = (n3 + BB - 1) / BB;
  const int gb = (nseg + 127) / 128, nsys = nseg / nrhs, sb = (nsys + 127) / 128;
  const double t = opt.induced_thresh;
  // the start residual F - B x with the FP32 operator
  k_bf32<<<nb3, BB, 0, stream>>>(n3, x.p, p32.p);
  CG_LAUNCH();
  apply_seg<float>(p32.p, Ap32.p);
  CG_CUDA(cudaMemsetAsync(d32.p, 0, sizeof(float) * n3, stream));
  k_bcg_start<float><<<nb, BB, 0, stream>>>(n, F.p, Ap32.p, alpha32.p, r32.p, z32.p, p32.p,
                                            site_a.p, site_b.p);
  CG_LAUNCH();
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rz.p, seg_rr.p);
  CG_LAUNCH();
  k_bsqrt<<<gb, 128, 0, stream>>>(nseg, seg_rr.p, seg_rnorm.p);
  CG_LAUNCH();
  // the first inner solve
  const int nx = n_inexact;
  auto stage = [&](int sg) {
    k_bstage<<<sb, 128, 0, stream>>>(nsys, nrhs, nx, sg, t, BATCH_ETA, 0.0, seg_rnorm.p,
                                     seg_delta_d[0].p, seg_delta_d[1].p, seg_tol.p, seg_sw[0].p,
                                     seg_sw[1].p, seg_rsw[0].p, seg_rsw[1].p, seg_level.p);
    CG_LAUNCH();
  };
  stage(0);
  k_bcg_init_seg<<<gb, 128, 0, stream>>>(nseg, seg_rz.p, seg_rr.p, seg_rz.p, seg_rnorm.p, done.p,
                                          iters.p, seg_tol.p);
  CG_LAUNCH();
  capture_pcg_loop(maxiter);
  CG_CUDA(cudaMemcpyAsync(iters_first.p, iters.p, nseg * sizeof(int), cudaMemcpyDeviceToDevice,
                          stream));
  // the double-float residual of x + d
  k_bacc<<<nb3, BB, 0, stream>>>(n3, x.p, d32.p);
  CG_LAUNCH();
  apply_seg<double>(x.p, Ap.p, NEAR_DD);
  k_bres<<<nb, BB, 0, stream>>>(n, F.p, Ap.p, nullptr, r.p, site_b.p);
  CG_LAUNCH();
  seg_norms_from_site_b();
  CG_CUDA(cudaMemcpyAsync(rn_second.p, seg_rnorm.p, nseg * sizeof(double),
                          cudaMemcpyDeviceToDevice, stream));
  // the second inner solve, for the right-hand side fl(r)
  stage(1);
  k_bcg_start<float><<<nb, BB, 0, stream>>>(n, r.p, nullptr, alpha32.p, r32.p, z32.p, p32.p,
                                            site_a.p, site_b.p);
  CG_LAUNCH();
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rz.p, seg_rr.p);
  CG_LAUNCH();
  k_bcg_init_seg<<<gb, 128, 0, stream>>>(nseg, seg_rz.p, seg_rr.p, seg_rz.p, seg_rnorm.p, done.p,
                                          iters.p, seg_tol.p);
  CG_LAUNCH();
  capture_pcg_loop(maxiter);
  // the residual from the recursion; x += d
  k_bres<<<nb, BB, 0, stream>>>(n, nullptr, nullptr, nullptr, r.p, site_b.p, r32.p);
  CG_LAUNCH();
  k_bacc<<<nb3, BB, 0, stream>>>(n3, x.p, d32.p);
  CG_LAUNCH();
  seg_norms_from_site_b();
}

bool BatchSystem::course_graph_ready(int maxiter) {
  static const bool graphs = [] {
    const char* e = std::getenv("CPPE_GPU_GRAPHS");
    return !(e && e[0] == '0');
  }();
  if (!graphs) course_failed = true;
  if (course_exec || course_failed) return course_exec != nullptr;
  iters_first.alloc(nseg);
  rn_second.alloc(nseg);
  // the operators' work buffers at their sizes (a capture cannot resize
  // them); what these applies write the course writes again first
  apply_seg<float>(p32.p, Ap32.p);
  apply_seg<double>(x.p, Ap.p, NEAR_DD);
  CG_CUDA(cudaStreamSynchronize(stream));
  cudaGraph_t g = nullptr;
  bool ok = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
  const long long c0 = launch_counter();
  if (ok) {
    try {
      CaptureScope cs;
      course_body(maxiter);
    } catch (...) {
      ok = false;  // the capture still ends below, so the stream stays usable
    }
    ok = (cudaStreamEndCapture(stream, &g) == cudaSuccess) && ok;
  }
  course_launches  = launch_counter() - c0;
  launch_counter() = c0;
  if (ok) ok = cudaGraphInstantiate(&course_exec, g, 0) == cudaSuccess;
  if (g) cudaGraphDestroy(g);
  if (!ok) {
    cudaGetLastError();  // clear the refusal; the host loop runs the whole solve
    if (course_exec) cudaGraphExecDestroy(course_exec);
    course_exec   = nullptr;
    course_failed = true;
  }
  return course_exec != nullptr;
}

void BatchSystem::seg_norms_from_site_b() {
  k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_b.p, nullptr, seg_rr.p, nullptr);
  CG_LAUNCH();
  k_bsqrt<<<(nseg + 127) / 128, 128, 0, stream>>>(nseg, seg_rr.p, seg_rnorm.p);
  CG_LAUNCH();
}

void BatchSystem::host_wait() {
  ++host_waits;
  CG_CUDA(cudaStreamSynchronize(stream));
}

int BatchSystem::solve_device(const double* d_rhs, double* d_mu, int* iters_out) {
  CG_CUDA(cudaSetDevice(device));
  stats      = SolveStats();
  host_waits = 0;
  const int nb = (n + BB - 1) / BB, n3 = 3 * n, nb3 = (n3 + BB - 1) / BB;
  const double t = opt.induced_thresh;
  permute_in(geo, d_rhs, F.p, 3, stream);
  // first-call guess alpha F (electric_fields.cc:198-202)
  k_bguess<<<nb, BB, 0, stream>>>(n, alpha64.p, F.p, x.p);
  CG_LAUNCH();
  std::vector<double> tolv(nseg, t);
  CG_CUDA(cudaMemcpyAsync(seg_tol.p, tolv.data(), nseg * sizeof(double), cudaMemcpyHostToDevice,
                          stream));
  int status = CPPE_GPU_NOT_CONVERGED;
  std::vector<int> it_h(nseg, 0), total(nseg, 0);
  if (opt.precision != CPPE_GPU_MIXED) {
    apply_seg<double>(x.p, Ap.p);
    stats.fp64_applies++;
    k_bcg_start<double><<<nb, BB, 0, stream>>>(n, F.p, Ap.p, alpha64.p, r.p, z.p, p.p, site_a.p,
                                               site_b.p);
    CG_LAUNCH();
    k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rz.p, seg_rr.p);
    CG_LAUNCH();
    k_bcg_init_seg<<<(nseg + 127) / 128, 128, 0, stream>>>(nseg, seg_rz.p, seg_rr.p, seg_rz.p,
                                                            seg_rnorm.p, done.p, iters.p, nullptr);
    CG_LAUNCH();
    run_pcg<double>(x.p, r.p, z.p, p.p, Ap.p, alpha64.p, std::max(1, opt.maxiter));
    std::vector<int> dn(nseg);
    CG_CUDA(cudaMemcpyAsync(dn.data(), done.p, nseg * sizeof(int), cudaMemcpyDeviceToHost, stream));
    CG_CUDA(cudaMemcpyAsync(it_h.data(), iters.p, nseg * sizeof(int), cudaMemcpyDeviceToHost,
                            stream));
    host_wait();
    status = std::all_of(dn.begin(), dn.end(), [](int d) { return d == 1; }) ? CPPE_GPU_OK
                                                                             : CPPE_GPU_NOT_CONVERGED;
    total = it_h;
  } else {
    // mixed precision, as System::solve_mixed but with per-segment scalars
    const double eta = BATCH_ETA;
    const int maxit  = std::max(1, opt.maxiter);
    std::vector<double> rn(nseg);
    bool exact = false;
    // bound of the residual norms' error where they were not recomputed with
    // the FP64 operator (as in System::solve_mixed, over the largest norm)
    constexpr double REC_ERR = 3e-6, CORR_ERR = 3e-7;
    double rerr = 0.0;
    std::vector<double> rswv[NINEXACT];
    for (int k = 0; k < NINEXACT; ++k) rswv[k].assign(nseg, 0.0);
    int outer0 = 0;
    if (course_graph_ready(maxit)) {
      // outer iterations 0 and 1 in one launch; the host then takes the
      // choices the course assumed: the solve ends after the double-float
      // residual where every segment is below the threshold (the second
      // inner solve then took no step and changed neither x nor r), the
      // residual from the recursion stands where its bound stays below
      // 0.4 t, and is replaced by the double-float one where it does not
      CG_CUDA(cudaGraphLaunch(course_exec, stream));
      std::vector<int> it1(nseg);
      std::vector<double> rn2(nseg);
      CG_CUDA(cudaMemcpyAsync(it1.data(), iters_first.p, nseg * sizeof(int),
                              cudaMemcpyDeviceToHost, stream));
      CG_CUDA(cudaMemcpyAsync(it_h.data(), iters.p, nseg * sizeof(int), cudaMemcpyDeviceToHost,
                              stream));
      CG_CUDA(cudaMemcpyAsync(rn2.data(), rn_second.p, nseg * sizeof(double),
                              cudaMemcpyDeviceToHost, stream));
      CG_CUDA(cudaMemcpyAsync(rn.data(), seg_rnorm.p, nseg * sizeof(double),
                              cudaMemcpyDeviceToHost, stream));
      for (int k = 0; k < n_inexact; ++k)
        CG_CUDA(cudaMemcpyAsync(rswv[k].data(), seg_rsw[k].p, nseg * sizeof(double),
                                cudaMemcpyDeviceToHost, stream));
      host_wait();
      const int k1 = *std::max_element(it1.begin(), it1.end());
      const int k2 = *std::max_element(it_h.begin(), it_h.end());
      stats.fp32_applies += 1 + k1 + k2;
      stats.fp64_applies += 1;
      launch_counter() += course_launches + course_body_launches * (k1 + k2);
      for (int g = 0; g < nseg; ++g) total[g] = it1[g] + it_h[g];
      exact  = true;
      outer0 = 2;
      if (std::all_of(rn2.begin(), rn2.end(), [&](double v) { return v < t; })) {
        status = CPPE_GPU_OK;
        rn     = rn2;
      } else {
        double extra = 0.0;
        for (int g = 0; g < nseg; ++g)
          extra = std::max(extra, 1.5 * ((n_inexact > 0 ? h_delta[0][g] * rswv[0][g] : 0.0) +
                                         (n_inexact > 1 ? h_delta[1][g] * rswv[1][g] : 0.0)));
        const double bound = REC_ERR * *std::max_element(rn2.begin(), rn2.end()) + extra;
        if (bound < 0.4 * t) {
          rerr = bound;
        } else {
          apply_seg<double>(x.p, Ap.p, NEAR_DD);
          stats.fp64_applies++;
          k_bres<<<nb, BB, 0, stream>>>(n, F.p, Ap.p, nullptr, r.p, site_b.p);
          CG_LAUNCH();
          seg_norms_from_site_b();
          CG_CUDA(cudaMemcpyAsync(rn.data(), seg_rnorm.p, nseg * sizeof(double),
                                  cudaMemcpyDeviceToHost, stream));
          host_wait();
        }
      }
    } else {
      k_bf32<<<nb3, BB, 0, stream>>>(n3, x.p, p32.p);
      CG_LAUNCH();
      apply_seg<float>(p32.p, Ap32.p);
      stats.fp32_applies++;
      CG_CUDA(cudaMemsetAsync(d32.p, 0, sizeof(float) * n3, stream));
      k_bcg_start<float><<<nb, BB, 0, stream>>>(n, F.p, Ap32.p, alpha32.p, r32.p, z32.p, p32.p,
                                                site_a.p, site_b.p);
      CG_LAUNCH();
      k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rz.p, seg_rr.p);
      CG_LAUNCH();
      k_bsqrt<<<(nseg + 127) / 128, 128, 0, stream>>>(nseg, seg_rr.p, seg_rnorm.p);
      CG_LAUNCH();
      CG_CUDA(cudaMemcpyAsync(rn.data(), seg_rnorm.p, nseg * sizeof(double),
                              cudaMemcpyDeviceToHost, stream));
      host_wait();
    }
    for (int outer = outer0; outer < 12 && status != CPPE_GPU_OK; ++outer) {
      if (outer > 0) {
        if (std::all_of(rn.begin(), rn.end(), [&](double v) { return v + rerr < t; })) {
          status = CPPE_GPU_OK;
          break;
        }
      }
      // inner tolerances, hand-over points and starting levels from the
      // norms in seg_rnorm (those in rn): the course's k_bstage
      const int nsys = nseg / nrhs;
      k_bstage<<<(nsys + 127) / 128, 128, 0, stream>>>(
            nsys, nrhs, n_inexact, outer == 0 ? 0 : 1, t, eta, rerr, seg_rnorm.p,
            seg_delta_d[0].p, seg_delta_d[1].p, seg_tol.p, seg_sw[0].p, seg_sw[1].p,
            seg_rsw[0].p, seg_rsw[1].p, seg_level.p);
      CG_LAUNCH();
      if (outer > 0) {
        k_bcg_start<float><<<nb, BB, 0, stream>>>(n, r.p, nullptr, alpha32.p, r32.p, z32.p,
                                                  p32.p, site_a.p, site_b.p);
        CG_LAUNCH();
        k_seg_sum<<<nseg, BB, 0, stream>>>(seg_start.p, site_a.p, site_b.p, seg_rz.p, seg_rr.p);
        CG_LAUNCH();
      }
      k_bcg_init_seg<<<(nseg + 127) / 128, 128, 0, stream>>>(
            nseg, seg_rz.p, seg_rr.p, seg_rz.p, seg_rnorm.p, done.p, iters.p, seg_tol.p);
      CG_LAUNCH();
      run_pcg<float>(d32.p, r32.p, z32.p, p32.p, Ap32.p, alpha32.p, maxit);
      CG_CUDA(cudaMemcpyAsync(it_h.data(), iters.p, nseg * sizeof(int), cudaMemcpyDeviceToHost,
                              stream));
      // the inexact operators' share of the recursion's error: 1.5 delta
      // times the residual at each hand-over
      double extra = 0.0;
      if (n_inexact > 0) {
        for (int k = 0; k < NINEXACT; ++k)
          CG_CUDA(cudaMemcpyAsync(rswv[k].data(), seg_rsw[k].p, nseg * sizeof(double),
                                  cudaMemcpyDeviceToHost, stream));
        host_wait();
        for (int g = 0; g < nseg; ++g)
          extra = std::max(extra, 1.5 * (h_delta[0][g] * rswv[0][g] +
                                         (n_inexact > 1 ? h_delta[1][g] * rswv[1][g] : 0.0)));
      }
      const double rmax = *std::max_element(rn.begin(), rn.end());
      // the residual from the recursion stands where its error bound stays
      // below 0.4 t: the inner solves stop at 0.5 t, so a segment's residual
      // plus the bound stays below t (as System::solve_mixed)
      if (exact && rerr + REC_ERR * rmax + extra < 0.4 * t) {
        // residual from the inner recursion (as System::solve_mixed)
        k_bres<<<nb, BB, 0, stream>>>(n, nullptr, nullptr, nullptr, r.p, site_b.p, r32.p);
        CG_LAUNCH();
        k_bacc<<<nb3, BB, 0, stream>>>(n3, x.p, d32.p);
        CG_LAUNCH();
        rerr += REC_ERR * rmax + extra;
      } else if (!(exact && rerr + CORR_ERR * rmax < 0.1 * t)) {
        k_bacc<<<nb3, BB, 0, stream>>>(n3, x.p, d32.p);
        CG_LAUNCH();
        apply_seg<double>(x.p, Ap.p, NEAR_DD);
        stats.fp64_applies++;
        k_bres<<<nb, BB, 0, stream>>>(n, F.p, Ap.p, nullptr, r.p, site_b.p);
        CG_LAUNCH();
        exact = true;
        rerr  = 0.0;
      } else {
        apply_seg<float>(d32.p, Ap32.p);
        stats.fp32_applies++;
        k_bres<<<nb, BB, 0, stream>>>(n, nullptr, nullptr, Ap32.p, r.p, site_b.p);
        CG_LAUNCH();
        k_bacc<<<nb3, BB, 0, stream>>>(n3, x.p, d32.p);
        CG_LAUNCH();
        rerr += CORR_ERR * rmax;
      }
      seg_norms_from_site_b();
      CG_CUDA(cudaMemcpyAsync(rn.data(), seg_rnorm.p, nseg * sizeof(double),
                              cudaMemcpyDeviceToHost, stream));
      host_wait();
      for (int g = 0; g < nseg; ++g) total[g] += it_h[g];
    }
    if (status != CPPE_GPU_OK &&
        std::all_of(rn.begin(), rn.end(), [&](double v) { return v + rerr < t; }))
      status = CPPE_GPU_OK;
    last_rnorm = rn;
  }
  if (iters_out) {
    // caller order: [system][rhs]
    for (int g = 0; g < nseg; ++g) iters_out[g] = total[g];
  }
  permute_out(geo, x.p, d_mu, 3, stream);
  host_wait();
  return status;
}

}  // namespace cg
