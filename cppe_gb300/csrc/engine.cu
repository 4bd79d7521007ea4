// Field engine kernels: near-field pair sums (direct summation and FMM P2P),
// the FMM passes and the finishing pass.
//
// Reference counterparts (maxscheurer/cppe, src/core/fmm/):
//   k_p2p, k_p2p32_m1, k_p2p_dd2
//              evaluate_direct{,_damping} calculate.cc:262-300,
//              evaluate_P2P_lazy + P2P_Cells{,_damping} calculate.cc:29-72,205-225
//   k_p2m_tasks + k_msum
//              evaluate_P2M + evaluate_M2M calculate.cc:129-184 (each cell's
//              multipole formed directly from its subtree: the same moments
//              the M2M shifts produce, without the level-by-level passes)
//   k_m2l, k_m2l_m1_p5/p6 (m2l_fixed.cuh)
//              evaluate_M2L_lazy calculate.cc:186-203
//   k_finish   evaluate_L2L + evaluate_L2P calculate.cc:227-260 (L2P of every
//              ancestor's M2L-only expansion in place of the L2L shifts), the
//              exclusion rule of P2P_Cells (calculate.cc:37), and
//              BMatrix::apply's "+ alpha^-1 mu" (bmatrix.cc:39)
// Every output element is owned by exactly one thread (no atomics), so
// results are bitwise reproducible run to run.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>
#include <unordered_map>

#include "engine.h"
#include "dd.cuh"
#include "m2l_fixed.cuh"


namespace cg {

constexpr int P2P_BLOCK  = 128;
constexpr int P2P_TILE   = 512;  // source sites staged in shared memory per tile
// lower bound of the Thole argument v from which a near-field pair is
// evaluated without damping in FP32 (1 - f_T < 2e-9 there) and without the
// double-float exponential in the residual pass
constexpr double P2P_UNDAMPED_V = 27.0;
constexpr int M2L_WARPS  = 4;
constexpr int P2M_LEAF_SITES  = 128;  // sites staged per round of the leaf P2M
constexpr int M2M_TASK_LEAVES = 8;    // leaf multipoles shifted per upward-pass task
// M2L_CHUNK (engine.h): sources of one target cell per M2L warp
constexpr bool M2L_TABLE_FP64 = true;  // FP64 M2L from tabulated derivative tensors
constexpr int PW = PMAX + 1;          // powers 0..PMAX of one coordinate
constexpr int FINISH_BLOCK = 128;

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
  v.cell_off = cell_off.p, v.cell_ref = cell_ref.p;
  v.lanc_ptr = lanc_ptr.p, v.lanc_cell = lanc_cell.p;
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
  make_schedules();
  make_vectors();
}

bool m2l_vectors(const TreeLayout& L, std::vector<int>& vid, std::vector<double4_32a>& vec) {
  vid.clear();
  vec.clear();
  if (L.m2l_src.empty()) return true;
  // centres are the root centre plus multiples of the deepest half-width
  double rmin = 1e300;
  for (int c = 0; c < L.ncells; ++c) rmin = std::min(rmin, L.center[4 * (size_t)c + 3]);
  if (!(rmin > 0.0)) return false;
  const double u = 0.5 * rmin;
  constexpr long long OFF = 1LL << 20;
  std::unordered_map<long long, int> ids;
  vid.resize(L.m2l_src.size());
  for (int A = 0; A < L.ncells; ++A)
    for (int q = L.m2l_ptr[A]; q < L.m2l_ptr[A + 1]; ++q) {
      const int B = L.m2l_src[q];
      long long k[3];
      for (int c = 0; c < 3; ++c) {
        const double d = (L.center[4 * (size_t)A + c] - L.center[4 * (size_t)B + c]) / u;
        k[c]           = std::llround(d);
        if (std::fabs(d - (double)k[c]) > 1e-3 || std::llabs(k[c]) >= OFF) {
          vid.clear();  // off the grid
          vec.clear();
          return false;
        }
      }
      const long long key = (k[0] + OFF) | ((k[1] + OFF) << 21) | ((k[2] + OFF) << 42);
      const auto it       = ids.find(key);
      if (it == ids.end()) {
        ids.emplace(key, (int)vec.size());
        vid[q] = (int)vec.size();
        double4_32a v;
        v.x = (double)k[0] * u, v.y = (double)k[1] * u, v.z = (double)k[2] * u, v.w = 0.0;
        vec.push_back(v);
      } else {
        vid[q] = it->second;
      }
    }
  return true;
}

void Geometry::make_vectors() {
  // off the grid: the M2L builds each tensor itself
  if (!fmm || !m2l_vectors(layout, h_m2l_vid, h_vec)) h_m2l_vid.clear(), h_vec.clear();
}

// Cuts every target leaf's source list into pieces of about `W` pairs so that
// blocks get similar work, and orders the pieces largest first.
void Geometry::make_schedules() {
  const TreeLayout& L = layout;
  // ---- FMM upward / downward schedules
  h_p2m_tasks.clear(), h_task_leaf.clear(), h_lanc_cell.clear();
  h_cell_task_ptr.assign(L.ncells + 1, 0);
  h_lanc_ptr.assign(L.nleaves + 1, 0);
  h_cell_ref.assign(L.ncells, 0);
  h_cell_off.assign(L.ncells, make_float4(0.f, 0.f, 0.f, 0.f));
  if (fmm && L.ncells > 0) {
    std::vector<char> need_m(L.ncells, 0), has_l(L.ncells, 0);
    for (int c = 0; c < L.ncells; ++c) {
      has_l[c] = L.m2l_ptr[c + 1] > L.m2l_ptr[c];
      for (int q = L.m2l_ptr[c]; q < L.m2l_ptr[c + 1]; ++q) need_m[L.m2l_src[q]] = 1;
    }
    std::vector<std::vector<int>> sub(L.ncells);  // subtree leaves of the cells needing M
    std::vector<int> ref(L.ncells, -1);
    for (int a = 0; a < L.nleaves; ++a) {
      for (int c = L.leaf_cell[a]; c >= 0; c = L.parent[c]) {
        if (need_m[c]) sub[c].push_back(a);
        if (ref[c] < 0 && L.leaf_start[a + 1] > L.leaf_start[a]) ref[c] = L.leaf_start[a];
        if (has_l[c]) h_lanc_cell.push_back(c);
      }
      h_lanc_ptr[a + 1] = (int)h_lanc_cell.size();
    }
    for (int c = 0; c < L.ncells; ++c) {
      const int r    = std::max(0, ref[c]);
      h_cell_ref[c]  = r;
      const double* cc = &L.center[4 * (size_t)c];
      h_cell_off[c] = make_float4((float)(cc[0] - h_pos64[r].x), (float)(cc[1] - h_pos64[r].y),
                                  (float)(cc[2] - h_pos64[r].z), 0.f);
      // non-leaf cells: tasks of <= M2M_TASK_LEAVES subtree leaves (leaf
      // multipoles are formed by k_p2m_leaf)
      if (!L.is_leaf[c]) {
        for (size_t k0 = 0; k0 < sub[c].size(); k0 += M2M_TASK_LEAVES) {
          const size_t k1 = std::min(sub[c].size(), k0 + M2M_TASK_LEAVES);
          const int first = (int)h_task_leaf.size();
          for (size_t k = k0; k < k1; ++k) h_task_leaf.push_back(sub[c][k]);
          h_p2m_tasks.push_back(make_int4(c, first, (int)h_task_leaf.size(), 0));
        }
      }
      h_cell_task_ptr[c + 1] = (int)h_p2m_tasks.size();
    }
  }
  if (h_task_leaf.empty()) h_task_leaf.push_back(0);
  // M2L chunks: at most M2L_CHUNK sources of one target cell each
  h_m2l_chunks.clear();
  h_cell_chunk_ptr.assign(L.ncells + 1, 0);
  const int chunk = m2l_chunk > 0 ? m2l_chunk : M2L_CHUNK;
  if (fmm)
    for (int c = 0; c < L.ncells; ++c) {
      for (int q = L.m2l_ptr[c]; q < L.m2l_ptr[c + 1]; q += chunk)
        h_m2l_chunks.push_back(make_int4(c, q, std::min(q + chunk, L.m2l_ptr[c + 1]), 0));
      h_cell_chunk_ptr[c + 1] = (int)h_m2l_chunks.size();
    }
  if (h_lanc_cell.empty()) h_lanc_cell.push_back(0);
  // ---- damping split of every target's source list, from a lower bound of
  // the Thole argument v = damping s_i s_j R over the two leaves (box
  // distance, smallest s; a site without damping partner counts as
  // s = infinity): leaves with v >= 27 for every pair (Thole factors 1 to
  // FP32 rounding, and the double-float exponential not needed) are moved to
  // the end of the list (stable, so a second call changes nothing), from
  // position h_leaf_split[a] on.
  if ((int)h_leaf_split.size() != L.nleaves) {
    h_leaf_split.assign(L.nleaves, 0);
    for (int a = 0; a < L.nleaves; ++a) h_leaf_split[a] = L.p2p_ptr[a + 1];
    if (damping > 0.0 && L.nleaves > 0) {
      std::vector<double> box(6 * (size_t)L.nleaves), smin(L.nleaves);
      for (int a = 0; a < L.nleaves; ++a) {
        double* bx = &box[6 * (size_t)a];
        bx[0] = bx[1] = bx[2] = 1e300;
        bx[3] = bx[4] = bx[5] = -1e300;
        smin[a] = 1e300;
        for (int k = L.leaf_start[a]; k < L.leaf_start[a + 1]; ++k) {
          const double4_32a& q = h_pos64[k];
          bx[0] = std::min(bx[0], q.x), bx[1] = std::min(bx[1], q.y), bx[2] = std::min(bx[2], q.z);
          bx[3] = std::max(bx[3], q.x), bx[4] = std::max(bx[4], q.y), bx[5] = std::max(bx[5], q.z);
          smin[a] = std::min(smin[a], q.w > 0.0 ? q.w : 1e300);
        }
      }
      std::vector<int> nearer, farther;
      for (int a = 0; a < L.nleaves; ++a) {
        const double* ba = &box[6 * (size_t)a];
        nearer.clear(), farther.clear();
        for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q) {
          const int b      = L.p2p_src[q];
          const double* bb = &box[6 * (size_t)b];
          double r2 = 0.0;
          for (int c = 0; c < 3; ++c) {
            const double d = std::max(0.0, std::max(ba[c] - bb[c + 3], bb[c] - ba[c + 3]));
            r2 += d * d;
          }
          const double v = 0.999 * damping * smin[a] * smin[b] * std::sqrt(r2);
          (v >= P2P_UNDAMPED_V ? farther : nearer).push_back(b);
        }
        int q = L.p2p_ptr[a];
        for (int b : nearer) layout.p2p_src[q++] = b;
        h_leaf_split[a] = q;
        for (int b : farther) layout.p2p_src[q++] = b;
      }
    }
  }
  // ---- near-field work items
  long total          = 0;
  for (int a = 0; a < L.nleaves; ++a) {
    const long na = L.leaf_start[a + 1] - L.leaf_start[a];
    for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q) {
      const int b = L.p2p_src[q];
      total += na * (L.leaf_start[b + 1] - L.leaf_start[b]);
    }
  }
  const long W = item_pairs > 0 ? item_pairs : std::max<long>(8192, total / (32L * 152));
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
  h_item_split.resize(its.size());
  nslot = 1;
  for (size_t k = 0; k < its.size(); ++k) {
    const int4 v    = its[k].v;
    h_items[k]      = v;
    h_item_split[k] = std::max(v.y, std::min(v.z, h_leaf_split[v.x]));
    nslot           = std::max(nslot, v.w + 1);
  }
  // the symmetric schedule of single systems (a batch keeps per-leaf items:
  // its passes skip finished segments and serve several right-hand sides)
  if (sym_enabled && h_leaf_seg.empty() && ncopies == 1)
    make_sym_schedule(W);
  else
    h_usrc.clear(), h_sym_items.clear();
  // a batch's copy-0 items, for the near-field pass over all its copies
  h_mitems.clear(), h_mitem_split.clear(), h_mitem_stride.clear();
  if (ncopies > 1 && (int)h_leaf_copy.size() == L.nleaves)
    for (size_t k = 0; k < h_items.size(); ++k)
      if (h_leaf_copy[h_items[k].x] == 0) {
        h_mitems.push_back(h_items[k]);
        h_mitem_split.push_back(h_item_split[k]);
        h_mitem_stride.push_back(h_leaf_cstride[h_items[k].x]);
      }
}

// Upper lists (partners B >= A of each leaf A, in the order of A's P2P list:
// damping class first), items over them of about W target-source pairs
// (each cross pair counts twice: both directions are evaluated), and the
// output rows: per item one row of its target leaf, and per (item, partner
// B != A) one row of B, numbered leaf by leaf in item order.
void Geometry::make_sym_schedule(long W) {
  const TreeLayout& L = layout;
  const int nl        = L.nleaves;
  h_usrc.clear(), h_usrc_off.clear(), h_sym_split.clear(), h_sym_aoff.clear();
  h_sym_items.clear();
  h_sym_leaf_rows.assign(nl, 0);
  h_sym_leaf_off.assign(nl + 1, 0);
  if (nl == 0) return;
  auto nsite = [&](int a) { return (long)(L.leaf_start[a + 1] - L.leaf_start[a]); };
  std::vector<int> uptr(nl + 1, 0), usplit(nl, 0);
  for (int a = 0; a < nl; ++a) {
    for (int q = L.p2p_ptr[a]; q < L.p2p_ptr[a + 1]; ++q) {
      if (q == h_leaf_split[a]) usplit[a] = (int)h_usrc.size();
      if (L.p2p_src[q] >= a) h_usrc.push_back(L.p2p_src[q]);
    }
    if (h_leaf_split[a] >= L.p2p_ptr[a + 1]) usplit[a] = (int)h_usrc.size();
    uptr[a + 1] = (int)h_usrc.size();
  }
  // items: pieces of the upper lists, and their row owners
  struct Item {
    long w;
    int4 v;
    int split;
  };
  std::vector<Item> its;
  std::vector<int> item_of_entry(h_usrc.size(), -1);
  for (int a = 0; a < nl; ++a) {
    const long na = nsite(a);
    int q0        = uptr[a];
    long acc      = 0;
    for (int q = uptr[a]; q < uptr[a + 1]; ++q) {
      const int b = h_usrc[q];
      acc += (b == a ? 1 : 2) * na * nsite(b);
      if (acc >= W || q + 1 == uptr[a + 1]) {
        its.push_back({acc, make_int4(a, q0, q + 1, 0), std::max(q0, std::min(q + 1, usplit[a]))});
        q0 = q + 1, acc = 0;
      }
    }
    if (uptr[a] == uptr[a + 1])  // no partner at all (not even itself): zeros
      its.push_back({0, make_int4(a, uptr[a], uptr[a], 0), uptr[a]});
  }
  // rows, leaf by leaf: first each leaf's own items, then its rows as a partner
  std::vector<std::vector<std::pair<int, int>>> partner_rows(nl);  // (item, entry)
  for (size_t k = 0; k < its.size(); ++k)
    for (int q = its[k].v.y; q < its[k].v.z; ++q)
      if (h_usrc[q] != its[k].v.x) partner_rows[h_usrc[q]].push_back({(int)k, q});
  std::vector<std::vector<int>> own(nl);
  for (size_t k = 0; k < its.size(); ++k) own[its[k].v.x].push_back((int)k);
  h_sym_aoff.assign(its.size(), 0);
  h_usrc_off.assign(h_usrc.size(), -1);
  long long off = 0;
  for (int a = 0; a < nl; ++a) {
    h_sym_leaf_off[a] = off;
    const long row    = 3 * nsite(a);
    for (int k : own[a]) h_sym_aoff[k] = off, off += row;
    for (const auto& pr : partner_rows[a]) h_usrc_off[pr.second] = off, off += row;
    h_sym_leaf_rows[a] = (int)(own[a].size() + partner_rows[a].size());
  }
  h_sym_leaf_off[nl] = off;
  sym_floats         = off;
  // largest first; the row offsets travel with the items
  std::vector<int> order(its.size());
  for (size_t k = 0; k < its.size(); ++k) order[k] = (int)k;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return its[x].w > its[y].w; });
  h_sym_items.resize(its.size());
  h_sym_split.resize(its.size());
  std::vector<long long> aoff(its.size());
  for (size_t k = 0; k < its.size(); ++k) {
    h_sym_items[k] = its[order[k]].v;
    h_sym_split[k] = its[order[k]].split;
    aoff[k]        = h_sym_aoff[order[k]];
  }
  h_sym_aoff.swap(aoff);
}

void Geometry::upload_schedules(cudaStream_t s) {
  if (has_sym()) {
    usrc.upload(h_usrc, s);
    usrc_off.upload(h_usrc_off, s);
    sym_split.upload(h_sym_split, s);
    sym_aoff.upload(h_sym_aoff, s);
    sym_items.upload(h_sym_items, s);
    sym_leaf_rows.upload(h_sym_leaf_rows, s);
    sym_leaf_off.upload(h_sym_leaf_off, s);
  }
  if (!h_mitems.empty()) {
    mitems.upload(h_mitems, s);
    mitem_split.upload(h_mitem_split, s);
    mitem_stride.upload(h_mitem_stride, s);
  }
  items.upload(h_items, s);
  item_split.upload(h_item_split, s);
  leaf_nslot.upload(h_leaf_nslot, s);
  if (!h_m2l_chunks.empty()) m2l_chunks.upload(h_m2l_chunks, s);
  cell_chunk_ptr.upload(h_cell_chunk_ptr, s);
}

void Geometry::upload(cudaStream_t s) {
  {
    std::vector<float2> tab(DD_EXP_TAB);
    for (int k = 0; k < DD_EXP_TAB; ++k) {
      const double e = std::exp(-0.0625 * k);
      tab[k]         = make_float2((float)e, (float)(e - (double)(float)e));
    }
    dd_exp.upload(tab, s);
  }
  items.upload(h_items, s);
  item_split.upload(h_item_split, s);
  leaf_nslot.upload(h_leaf_nslot, s);
  if (has_sym()) {
    usrc.upload(h_usrc, s);
    usrc_off.upload(h_usrc_off, s);
    sym_split.upload(h_sym_split, s);
    sym_aoff.upload(h_sym_aoff, s);
    sym_items.upload(h_sym_items, s);
    sym_leaf_rows.upload(h_sym_leaf_rows, s);
    sym_leaf_off.upload(h_sym_leaf_off, s);
  }
  if (!h_vec.empty()) {
    m2l_vid.upload(h_m2l_vid, s);
    vec.upload(h_vec, s);
  }
  if (!h_mitems.empty()) {
    mitems.upload(h_mitems, s);
    mitem_split.upload(h_mitem_split, s);
    mitem_stride.upload(h_mitem_stride, s);
  }
  if (!h_leaf_seg.empty()) leaf_seg.upload(h_leaf_seg, s);
  if (!h_cell_seg.empty()) cell_seg.upload(h_cell_seg, s);
  if (!h_p2m_tasks.empty()) p2m_tasks.upload(h_p2m_tasks, s);
  task_leaf.upload(h_task_leaf, s);
  if (!h_m2l_chunks.empty()) m2l_chunks.upload(h_m2l_chunks, s);
  cell_chunk_ptr.upload(h_cell_chunk_ptr, s);
  cell_task_ptr.upload(h_cell_task_ptr, s);
  lanc_ptr.upload(h_lanc_ptr, s);
  lanc_cell.upload(h_lanc_cell, s);
  cell_ref.upload(h_cell_ref.empty() ? std::vector<int>{0} : h_cell_ref, s);
  cell_off.upload(h_cell_off.empty() ? std::vector<float4>{float4{}} : h_cell_off, s);
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
// start inside a tile of TILE sites, the last one possibly in part
// (`coff` sites of the first leaf were taken by the previous round).
// ---------------------------------------------------------------------------
struct TilePlan {
  int pstart[33];  // first site of each piece
  int poff[34];    // tile offset of each piece (poff[np] = tile size)
  int np, cur, coff;
  int cur0;        // list position of the tile's first piece
};

template <int TILE = P2P_TILE>
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
  const bool take    = e < b1 && excl < TILE;
  const int takecnt  = take ? min(cnt, TILE - excl) : 0;
  const unsigned msk = __ballot_sync(0xffffffffu, take);
  const int np       = __popc(msk);
  const int last     = max(np - 1, 0);
  const int tot      = __shfl_sync(0xffffffffu, excl + takecnt, last);
  const int lastcnt  = __shfl_sync(0xffffffffu, cnt, last);
  const int lasttake = __shfl_sync(0xffffffffu, takecnt, last);
  if (take) tp.pstart[lane] = start, tp.poff[lane] = excl;
  if (lane == 0) {
    tp.cur0     = cur;
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
            T damping, T* __restrict__ Fnear, const int* __restrict__ leaf_seg,
            const int* __restrict__ seg_done) {
  constexpr int NS = ncomp(M);
  __shared__ SiteRec<T> s_rec[P2P_TILE];
  __shared__ T s_S[P2P_TILE * NS];
  __shared__ TilePlan s_plan;
  __shared__ T s_red[P2P_BLOCK * 6];

  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  if (seg_done && seg_done[leaf_seg[A]]) return;  // finished segment of a batch
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
// Packed FP32x2 arithmetic (__ffma2_rn / __fmul2_rn / __fadd2_rn, sm_100 and
// later) evaluates one target against two sources per instruction: sources
// are staged in pairs ({x_j, x_j+1, y_j, y_j+1}, ... in four SoA arrays), the
// target's coordinates are broadcast into both halves once, and each thread
// serves two targets, so every pair of staged sources read from shared
// memory feeds four pair evaluations.
//  - Positions are relative to the first site of the target leaf, formed once
//    per staged source from the hi/lo coordinates; separations are taken as
//    source - target (the dipole field is even in r).
//  - Damped: 1/R is capped at 1e4 (real pairs have R > 1e-4 bohr), which
//    turns the self pair (R = 0, v = 0, f_E = f_T = 0) into an exact zero
//    without a branch; sites without a damping partner (s = 0) are staged
//    with s = 1e15, i.e. e^-v = 0 and f = 1 (the exponent is clamped at
//    2^-126 so that the damping polynomials stay finite).
//  - Undamped: the self pair is removed by a select on R^2 > 0.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// 1/sqrt(x) as one MUFU operation (inputs are squared distances: never
// subnormal; 0 gives +inf)
__device__ __forceinline__ float rsqrt_approx(float x) {
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
// ln 2 and the products of its powers that the damping polynomials take in
// t = -v log2(e)
constexpr float LN2       = 0.6931471805599453f;
constexpr float LN2SQ_2   = 0.2402265069591007f;   // (ln 2)^2 / 2
constexpr float LN2SQ_3_2 = 0.7206795208773021f;   // 3 (ln 2)^2 / 2
constexpr float LN2CU_2   = 0.16651232599446472f;  // (ln 2)^3 / 2

// two sources in the halves of packed operands
struct Src2 {
  float4 xy;   // x_j, x_j+1, y_j, y_j+1
  float4 zs;   // z_j, z_j+1, s_j, s_j+1
  float4 mxy;  // mx_j, mx_j+1, my_j, my_j+1
  float2 mz;   // mz_j, mz_j+1
};

// The pair tensor of a target against two sources (one per half): the
// separation (source - target), A = R^-3 f_E and Bn = -3 R^-5 f_T, so that
// the field of a dipole mu is mu A + r (mu.r) Bn (even in r: the same tensor
// serves both directions).
template <bool DAMP>
__device__ __forceinline__ void f32x2_tensor_m1(const float2& nX, const float2& nY,
                                                const float2& nZ, const float2& AI,
                                                const float2& sx, const float2& sy,
                                                const float2& sz, const float2& ss, float2& x,
                                                float2& y, float2& z, float2& A, float2& Bn) {
  x               = __fadd2_rn(sx, nX);
  y               = __fadd2_rn(sy, nY);
  z               = __fadd2_rn(sz, nZ);
  const float2 r2 = __ffma2_rn(x, x, __ffma2_rn(y, y, __fmul2_rn(z, z)));
  float2 ir;
  if (DAMP) {
    ir.x = fminf(rsqrt_approx(r2.x), 1e4f);
    ir.y = fminf(rsqrt_approx(r2.y), 1e4f);
  } else {
    ir.x = r2.x > 0.f ? rsqrt_approx(r2.x) : 0.f;
    ir.y = r2.y > 0.f ? rsqrt_approx(r2.y) : 0.f;
  }
  const float2 ir2 = __fmul2_rn(ir, ir);
  const float2 ir3 = __fmul2_rn(ir2, ir);
  const float2 ir5 = __fmul2_rn(ir3, ir2);
  if (DAMP) {
    // t = -v log2(e) with v = damping s_i s_j R (AI = -log2(e) damping s_i);
    // with v = -t ln 2 the damping functions are
    //   f_E = 1 - e^-v (1 + v + v^2/2)          = 1 + e np,
    //   f_T = 1 - e^-v (1 + v + v^2/2 + v^3/6)  = 1 - e q3 / 3,
    // np = -1 + t ln2 - t^2 ln2^2/2, q3 = 3 - 3 t ln2 + 3 t^2 ln2^2/2 - t^3 ln2^3/2
    float2 t = __fmul2_rn(__fmul2_rn(AI, ss), __fmul2_rn(r2, ir));
    t.x = fmaxf(t.x, -126.f);
    t.y = fmaxf(t.y, -126.f);
    const float2 e  = make_float2(ex2_approx(t.x), ex2_approx(t.y));
    const float2 np = __ffma2_rn(t, __ffma2_rn(t, f2(-LN2SQ_2), f2(LN2)), f2(-1.f));
    const float2 q3 = __ffma2_rn(
          t, __ffma2_rn(t, __ffma2_rn(t, f2(-LN2CU_2), f2(LN2SQ_3_2)), f2(-3.f * LN2)), f2(3.f));
    A  = __fmul2_rn(ir3, __ffma2_rn(np, e, f2(1.f)));   // R^-3 f_E
    Bn = __fmul2_rn(ir5, __ffma2_rn(q3, e, f2(-3.f)));  // -3 R^-5 f_T
  } else {
    A  = ir3;
    Bn = __fmul2_rn(ir5, f2(-3.f));
  }
}

// F += mu A + r (mu.r) Bn for packed moments (mx, my, mz)
__device__ __forceinline__ void f32x2_apply_m1(const float2& x, const float2& y, const float2& z,
                                               const float2& A, const float2& Bn,
                                               const float2& mx, const float2& my,
                                               const float2& mz, float2& FX, float2& FY,
                                               float2& FZ) {
  const float2 md = __ffma2_rn(mx, x, __ffma2_rn(my, y, __fmul2_rn(mz, z)));
  const float2 nC = __fmul2_rn(md, Bn);
  FX = __ffma2_rn(x, nC, __ffma2_rn(mx, A, FX));
  FY = __ffma2_rn(y, nC, __ffma2_rn(my, A, FY));
  FZ = __ffma2_rn(z, nC, __ffma2_rn(mz, A, FZ));
}

template <bool DAMP>
__device__ __forceinline__ void f32x2_pair_m1(const float2& nX, const float2& nY,
                                              const float2& nZ, const float2& AI,
                                              const Src2& q, float2& FX, float2& FY,
                                              float2& FZ) {
  float2 x, y, z, A, Bn;
  f32x2_tensor_m1<DAMP>(nX, nY, nZ, AI, make_float2(q.xy.x, q.xy.y), make_float2(q.xy.z, q.xy.w),
                        make_float2(q.zs.x, q.zs.y), make_float2(q.zs.z, q.zs.w), x, y, z, A, Bn);
  f32x2_apply_m1(x, y, z, A, Bn, make_float2(q.mxy.x, q.mxy.y), make_float2(q.mxy.z, q.mxy.w),
                 q.mz, FX, FY, FZ);
}

constexpr int P2P32_PAIRS = 512;  // staged source pairs per tile (1,024 sources)
template <bool DAMP>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p32_m1(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
                 const int* __restrict__ item_split, const int* __restrict__ p2p_src, const float4* __restrict__ hi,
                 const float4* __restrict__ lo, const float* __restrict__ src, float damping,
                 float* __restrict__ Fnear, const int* __restrict__ leaf_seg,
                 const int* __restrict__ seg_done) {
  constexpr int TILE = 2 * P2P32_PAIRS;
  __shared__ float4 s_xy[P2P32_PAIRS];   // x_j, x_j+1, y_j, y_j+1
  __shared__ float4 s_zs[P2P32_PAIRS];   // z_j, z_j+1, s_j, s_j+1
  __shared__ float4 s_mxy[P2P32_PAIRS];  // mx_j, mx_j+1, my_j, my_j+1
  __shared__ float2 s_mz[P2P32_PAIRS];   // mz_j, mz_j+1
  __shared__ TilePlan s_plan;
  __shared__ float s_red[P2P_BLOCK * 6];

  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  if (seg_done && seg_done[leaf_seg[A]]) return;  // finished segment of a batch
  const int sp = item_split[blockIdx.x];
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const float4 oh = hi[a0], ol = lo[a0];
  auto rel = [&](int k) {
    const float4 h = hi[k], l = lo[k];
    return make_float4((h.x - oh.x) + (l.x - ol.x), (h.y - oh.y) + (l.y - ol.y),
                       (h.z - oh.z) + (l.z - ol.z), h.w > 0.f ? h.w : 1e15f);
  };

  for (int tb = 0; tb < nA; tb += 2 * P2P_BLOCK) {
    const int nT = min(2 * P2P_BLOCK, nA - tb);
    const int T  = (nT + 1) >> 1;  // threads per group
    const int S  = P2P_BLOCK / T;  // groups
    const int t = threadIdx.x % T, g = threadIdx.x / T;
    const bool active = g < S;
    float2 nX[2], nY[2], nZ[2], AI[2];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
      const int k    = t + p * T;
      const float4 m = rel(a0 + tb + (k < nT ? k : t));
      nX[p] = f2(-m.x), nY[p] = f2(-m.y), nZ[p] = f2(-m.z);
      AI[p] = f2(-1.4426950408889634f * damping * m.w);
    }
    Comp3<float> acc[2];
    // phase 0: sources [b0, sp) with the Thole factors; phase 1: [sp, b1),
    // every pair with v >= 27 (the factors equal 1 to FP32 rounding)
    for (int ph = 0; ph < 2; ++ph) {
    const int pend = ph == 0 ? sp : b1;
    if (threadIdx.x == 0) s_plan.cur = ph == 0 ? b0 : sp, s_plan.coff = 0;
    __syncthreads();
    while (true) {
      if (threadIdx.x < 32) plan_tile<TILE>(s_plan, pend, p2p_src, leaf_start);
      __syncthreads();
      const int np = s_plan.np;
      if (np == 0) break;
      const int total  = s_plan.poff[np];
      const int npairs = (total + 1) >> 1;
      for (int q = threadIdx.x; q < npairs; q += P2P_BLOCK) {
        const int j0 = tile_site(s_plan, 2 * q);
        const float4 r0 = rel(j0);
        const float mx0 = src[3 * (size_t)j0], my0 = src[3 * (size_t)j0 + 1],
                    mz0 = src[3 * (size_t)j0 + 2];
        // an odd tile ends with a source of zero moment far from the leaf
        float4 r1 = make_float4(1e4f, 0.f, 0.f, 1.f);
        float mx1 = 0.f, my1 = 0.f, mz1 = 0.f;
        if (2 * q + 1 < total) {
          const int j1 = tile_site(s_plan, 2 * q + 1);
          r1 = rel(j1);
          mx1 = src[3 * (size_t)j1], my1 = src[3 * (size_t)j1 + 1], mz1 = src[3 * (size_t)j1 + 2];
        }
        s_xy[q]  = make_float4(r0.x, r1.x, r0.y, r1.y);
        s_zs[q]  = make_float4(r0.z, r1.z, r0.w, r1.w);
        s_mxy[q] = make_float4(mx0, mx1, my0, my1);
        s_mz[q]  = make_float2(mz0, mz1);
      }
      __syncthreads();
      if (active) {
        float2 FX[2], FY[2], FZ[2];
#pragma unroll
        for (int p = 0; p < 2; ++p) FX[p] = FY[p] = FZ[p] = f2(0.f);
        auto sweep = [&](auto damped) {
          constexpr bool D = decltype(damped)::value;
#pragma unroll 1
          for (int jj = g; jj < npairs; jj += S) {
            Src2 q;
            q.xy = s_xy[jj], q.zs = s_zs[jj], q.mxy = s_mxy[jj], q.mz = s_mz[jj];
#pragma unroll
            for (int p = 0; p < 2; ++p)
              f32x2_pair_m1<D>(nX[p], nY[p], nZ[p], AI[p], q, FX[p], FY[p], FZ[p]);
          }
        };
        if (DAMP && ph == 0)
          sweep(std::true_type{});
        else
          sweep(std::false_type{});
#pragma unroll
        for (int p = 0; p < 2; ++p) acc[p].add(FX[p].x + FX[p].y, FY[p].x + FY[p].y, FZ[p].x + FZ[p].y);
      }
      __syncthreads();
    }
    }
    if (active) {
      float* r = &s_red[(g * T + t) * 6];
#pragma unroll
      for (int k = 0; k < 2; ++k)
        r[3 * k] = acc[k].gx(), r[3 * k + 1] = acc[k].gy(), r[3 * k + 2] = acc[k].gz();
    }
    __syncthreads();
    if (threadIdx.x < T) {
      for (int k = 0; k < 2; ++k) {
        const int idx = threadIdx.x + k * T;
        if (idx >= nT) continue;
        float f0 = 0.f, f1 = 0.f, f2v = 0.f;
        for (int gg = 0; gg < S; ++gg) {
          const float* r = &s_red[(gg * T + threadIdx.x) * 6 + 3 * k];
          f0 += r[0], f1 += r[1], f2v += r[2];
        }
        float* o = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + idx);
        o[0] = f0, o[1] = f1, o[2] = f2v;
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Near field, FP32, dipole sources, every unordered leaf pair once.
// The P2P lists are symmetric (B is in A's list exactly when A is in B's), so
// an item of leaf A takes its upper list (partners B >= A, damping class
// first; see Geometry::make_sym_schedule) and evaluates each pair tensor once
// for both directions (T(r) = T(-r)): 21 of a damped pair's 31 operations are
// the tensor, so a cross pair costs 41 operations instead of 62.
//  - Lanes own sources: each warp takes consecutive sources of a 256-source
//    tile, two or four per lane (one or two packed FP32x2 pairs; 4 or 2
//    warps), with positions relative to the first site of A (hi/lo
//    differences) in registers.
//  - The targets of A (64 per pass) are staged in shared memory and broadcast
//    one at a time.  Per target the lane's pair tensors give the sources'
//    fields (F_j += T mu_i, accumulated in registers over all targets) and
//    the target's field (T mu_j, summed over the lane's sources).  The
//    targets' fields of eight targets are reduce-scattered over the warp (9
//    shuffles and adds per component) and added, compensated, to the warp's
//    accumulators in shared memory.
//  - A source's field goes to its leaf's output row for this item; the self
//    leaf (B = A) is evaluated one way only.  The warps' target fields
//    are added in warp order into the item's row of A.  Rows are fixed at
//    set-up and added by the finishing pass in a fixed order (no atomics).
//  - Damping as in k_p2p32_m1: the damping class first with the Thole
//    factors, then the partners with v >= 27 for every pair without them;
//    1/R capped at 1e4 (self pairs give an exact zero); lanes without a
//    source hold a zero moment 1e4 bohr away.
// ---------------------------------------------------------------------------
constexpr int SYM_TILE = 256;  // sources per tile: (4 / NPK) warps x 32 lanes x 2 NPK
constexpr int SYM_TGT  = 64;   // targets per pass over the sources

// NPK packed source pairs per lane: 1 (128 threads, two sources a lane) or 2
// (64 threads, four sources a lane: the target broadcasts and reduce-scatters
// are shared by twice the pairs, at fewer resident warps).  The schedule
// autotuner picks one (Geometry::sym_pack).
template <int NPK>
constexpr int sym_threads() { return 128 / NPK; }
template <int NPK>
constexpr int sym_min_blocks() { return NPK == 1 ? 6 : 10; }

template <bool DAMP, int NPK>
__global__ void __launch_bounds__(sym_threads<NPK>(), sym_min_blocks<NPK>())
      k_p2p32_m1_sym(const int* __restrict__ leaf_start, const int4* __restrict__ items,
                     const int* __restrict__ item_split, const long long* __restrict__ item_aoff,
                     const int* __restrict__ usrc, const long long* __restrict__ usrc_off,
                     const float4* __restrict__ hi, const float4* __restrict__ lo,
                     const float* __restrict__ src, float damping, float* __restrict__ rows) {
  constexpr int NW  = 4 / NPK;  // warps
  constexpr int SPL = 2 * NPK;  // sources per lane
  __shared__ float4 s_t[SYM_TGT];   // target x, y, z, AI (padded to a multiple of 8)
  __shared__ float4 s_tm[SYM_TGT];  // target mx, my, mz
  __shared__ float s_acc[NW][SYM_TGT][6];  // per warp: target field sums and their errors
  __shared__ TilePlan s_plan;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z;
  const int sp = item_split[blockIdx.x];
  const long long aoff = item_aoff[blockIdx.x];
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const float4 oh = hi[a0], ol = lo[a0];
  auto rel = [&](int k) {
    const float4 h = hi[k], l = lo[k];
    return make_float4((h.x - oh.x) + (l.x - ol.x), (h.y - oh.y) + (l.y - ol.y),
                       (h.z - oh.z) + (l.z - ol.z), h.w > 0.f ? h.w : 1e15f);
  };
  for (int tb = 0; tb < nA; tb += SYM_TGT) {
    const int nT = min(SYM_TGT, nA - tb);
    __syncthreads();
    for (int k = threadIdx.x; k < SYM_TGT; k += blockDim.x) {
      if (k < nT) {
        const float4 m = rel(a0 + tb + k);
        s_t[k]  = make_float4(-m.x, -m.y, -m.z, -1.4426950408889634f * damping * m.w);
        const size_t j = a0 + tb + k;
        s_tm[k] = make_float4(src[3 * j], src[3 * j + 1], src[3 * j + 2], 0.f);
      } else {  // padding: a zero moment far away (its fields are dropped)
        s_t[k]  = make_float4(-1e4f, 0.f, 0.f, -1.4426950408889634f * damping);
        s_tm[k] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int w = 0; w < NW; ++w)
#pragma unroll
        for (int c = 0; c < 6; ++c) s_acc[w][k][c] = 0.f;
    }
    for (int ph = 0; ph < 2; ++ph) {
      const int pend = ph == 0 ? sp : b1;
      if (threadIdx.x == 0) s_plan.cur = ph == 0 ? b0 : sp, s_plan.coff = 0;
      __syncthreads();
      while (true) {
        if (threadIdx.x < 32) plan_tile<SYM_TILE>(s_plan, pend, usrc, leaf_start);
        __syncthreads();
        const int np = s_plan.np;
        if (np == 0) break;
        const int total = s_plan.poff[np];
        // this lane's sources, packed in pairs
        float2 sx[NPK], sy[NPK], sz[NPK], ss[NPK], mx[NPK], my[NPK], mz[NPK];
        long long o[SPL];  // output positions (-1: none)
        {
          float4 r[SPL];
          float m[SPL][3];
#pragma unroll
          for (int h = 0; h < SPL; ++h) {
            const int q = 32 * SPL * warp + SPL * lane + h;
            o[h] = -1;
            if (q < total) {
              // piece of tile slot q (as tile_site) and its list entry
              int lo_ = 0, hi_ = np - 1;
              while (lo_ < hi_) {
                const int mid = (lo_ + hi_ + 1) >> 1;
                if (s_plan.poff[mid] <= q) lo_ = mid; else hi_ = mid - 1;
              }
              const int j = s_plan.pstart[lo_] + (q - s_plan.poff[lo_]);
              const int e = s_plan.cur0 + lo_;
              const int B = usrc[e];
              r[h] = rel(j);
              m[h][0] = src[3 * (size_t)j], m[h][1] = src[3 * (size_t)j + 1],
              m[h][2] = src[3 * (size_t)j + 2];
              if (B != A) o[h] = usrc_off[e] + 3 * (long long)(j - leaf_start[B]);
            } else {
              r[h] = make_float4(1e4f, 0.f, 0.f, 1.f);
              m[h][0] = m[h][1] = m[h][2] = 0.f;
            }
          }
#pragma unroll
          for (int k = 0; k < NPK; ++k) {
            const int h0 = 2 * k, h1 = 2 * k + 1;
            sx[k] = make_float2(r[h0].x, r[h1].x), sy[k] = make_float2(r[h0].y, r[h1].y);
            sz[k] = make_float2(r[h0].z, r[h1].z), ss[k] = make_float2(r[h0].w, r[h1].w);
            mx[k] = make_float2(m[h0][0], m[h1][0]), my[k] = make_float2(m[h0][1], m[h1][1]);
            mz[k] = make_float2(m[h0][2], m[h1][2]);
          }
        }
        float2 FX[NPK], FY[NPK], FZ[NPK];
#pragma unroll
        for (int k = 0; k < NPK; ++k) FX[k] = FY[k] = FZ[k] = f2(0.f);
        auto sweep = [&](auto damped) {
          constexpr bool D = decltype(damped)::value;
#pragma unroll 1
          for (int g = 0; g < nT; g += 8) {
            // eight targets (padded with zero moments); their fields from the
            // lane's sources stay per lane until the reduce-scatter below
            float p[8][3];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
              const float4 t = s_t[g + u], tm = s_tm[g + u];
              float2 cx = f2(0.f), cy = f2(0.f), cz = f2(0.f);
#pragma unroll
              for (int k = 0; k < NPK; ++k) {
                float2 x, y, z, Av, Bn;
                f32x2_tensor_m1<D>(f2(t.x), f2(t.y), f2(t.z), f2(t.w), sx[k], sy[k], sz[k],
                                   ss[k], x, y, z, Av, Bn);
                f32x2_apply_m1(x, y, z, Av, Bn, f2(tm.x), f2(tm.y), f2(tm.z), FX[k], FY[k],
                               FZ[k]);
                f32x2_apply_m1(x, y, z, Av, Bn, mx[k], my[k], mz[k], cx, cy, cz);
              }
              p[u][0] = cx.x + cx.y, p[u][1] = cy.x + cy.y, p[u][2] = cz.x + cz.y;
            }
            // reduce-scatter over the warp: after the xor-16, -8 and -4 steps
            // lane l holds target (l >> 2) & 7 for its quarter of lanes, the
            // xor-2 and -1 steps add the four quarters
            const bool h16 = lane & 16, h8 = lane & 8, h4 = lane & 4;
            float q4[4][3], q2[2][3], q1[3];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const float keep = h16 ? p[u + 4][c] : p[u][c];
                const float send = h16 ? p[u][c] : p[u + 4][c];
                q4[u][c]         = keep + __shfl_xor_sync(0xffffffffu, send, 16);
              }
#pragma unroll
            for (int u = 0; u < 2; ++u)
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const float keep = h8 ? q4[u + 2][c] : q4[u][c];
                const float send = h8 ? q4[u][c] : q4[u + 2][c];
                q2[u][c]         = keep + __shfl_xor_sync(0xffffffffu, send, 8);
              }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              const float keep = h4 ? q2[1][c] : q2[0][c];
              const float send = h4 ? q2[0][c] : q2[1][c];
              float v          = keep + __shfl_xor_sync(0xffffffffu, send, 4);
              v += __shfl_xor_sync(0xffffffffu, v, 2);
              v += __shfl_xor_sync(0xffffffffu, v, 1);
              q1[c] = v;
            }
            const int u = (lane >> 2) & 7;
            if ((lane & 3) == 0 && g + u < nT) {
              // compensated accumulation of this warp's share of target g + u
              float* acc = s_acc[warp][g + u];
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                float sum, err;
                two_sum(acc[c], q1[c], sum, err);
                acc[c] = sum, acc[3 + c] += err;
              }
            }
          }
        };
        if (DAMP && ph == 0)
          sweep(std::true_type{});
        else
          sweep(std::false_type{});
#pragma unroll
        for (int k = 0; k < NPK; ++k) {
          const long long oa = o[2 * k], ob = o[2 * k + 1];
          if (oa >= 0) rows[oa] = FX[k].x, rows[oa + 1] = FY[k].x, rows[oa + 2] = FZ[k].x;
          if (ob >= 0) rows[ob] = FX[k].y, rows[ob + 1] = FY[k].y, rows[ob + 2] = FZ[k].y;
        }
        __syncthreads();
      }
    }
    // the targets' fields: the warps' sums in warp order
    __syncthreads();
    for (int k = threadIdx.x; k < nT; k += blockDim.x) {
      float* o = rows + aoff + 3 * (long long)(tb + k);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float v = 0.f;
#pragma unroll
        for (int w = 0; w < NW; ++w) v += s_acc[w][k][c] + s_acc[w][k][3 + c];
        o[c] = v;
      }
    }
  }
}


// ---------------------------------------------------------------------------
// Near field, FP32, dipole sources, for the right-hand sides of a batch
// together.  A batch repeats each snapshot's geometry once per right-hand
// side (segments s*R + r, r < R, laid out one after another: copy r of a
// site sits `stride.x` sites, and of a leaf `stride.y` leaves, after copy 0).
// The pair tensor (separation, 1/R powers, Thole factors) does not depend on
// the right-hand side, so this kernel runs the items of copy 0 only and
// applies each tensor to the R copies' source moments: about 21 of the 31
// FP32 operations of a damped pair are shared, leaving 10 per right-hand
// side.  Same tiles, damping split and self-pair handling as k_p2p32_m1,
// one target per thread (the accumulators of R right-hand sides take the
// registers of the second target).  Copies whose segments have finished
// take no work (their output is not read); items whose copies have all
// finished return at once.
// ---------------------------------------------------------------------------
// staged source pairs per tile: 96, 120 or 144 (built in; static shared
// memory stays below 48 KB), chosen by the batch's schedule autotuner
// (Geometry::multi_tile)
constexpr int P2PM_PAIRS = 144;
constexpr int P2PM_MAXR  = 8;    // right-hand sides per launch
template <bool DAMP, int PAIRS = P2PM_PAIRS, int RC = P2PM_MAXR>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p32_m1_multi(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
                       const int* __restrict__ item_split, const int2* __restrict__ item_stride,
                       int c0, int nr, const int* __restrict__ p2p_src,
                       const float4* __restrict__ hi, const float4* __restrict__ lo,
                       const float* __restrict__ src, float damping, float* __restrict__ Fnear,
                       const int* __restrict__ leaf_seg, const int* __restrict__ seg_done) {
  constexpr int TILE = 2 * PAIRS;
  constexpr int R    = RC;  // right-hand sides per pass
  __shared__ float4 s_xy[PAIRS];       // x_j, x_j+1, y_j, y_j+1
  __shared__ float4 s_zs[PAIRS];       // z_j, z_j+1, s_j, s_j+1
  __shared__ float4 s_mxy[PAIRS * R];  // per copy: mx_j, mx_j+1, my_j, my_j+1
  __shared__ float2 s_mz[PAIRS * R];   // per copy: mz_j, mz_j+1
  __shared__ int s_site[TILE];              // copy-0 site of each tile slot
  __shared__ TilePlan s_plan;
  __shared__ float s_red[P2P_BLOCK * 3 * R];

  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int2 st = item_stride[blockIdx.x];  // sites, leaves between copies
  // copies c0 .. c0 + nr - 1 of this launch; those still iterating (bit r)
  unsigned live = 0;
  for (int r = 0; r < nr; ++r)
    if (!seg_done || seg_done[leaf_seg[A + (c0 + r) * st.y]] == 0) live |= 1u << r;
  if (!live) return;
  const int sp = item_split[blockIdx.x];
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const float4 oh = hi[a0], ol = lo[a0];
  auto rel = [&](int k) {
    const float4 h = hi[k], l = lo[k];
    return make_float4((h.x - oh.x) + (l.x - ol.x), (h.y - oh.y) + (l.y - ol.y),
                       (h.z - oh.z) + (l.z - ol.z), h.w > 0.f ? h.w : 1e15f);
  };

  for (int tb = 0; tb < nA; tb += P2P_BLOCK) {
    const int nT = min(P2P_BLOCK, nA - tb);
    const int S  = P2P_BLOCK / nT;  // groups of nT threads
    const int t = threadIdx.x % nT, g = threadIdx.x / nT;
    const bool active = g < S;
    float2 nX, nY, nZ, AI;
    {
      const float4 m = rel(a0 + tb + t);
      nX = f2(-m.x), nY = f2(-m.y), nZ = f2(-m.z);
      AI = f2(-1.4426950408889634f * damping * m.w);
    }
    Comp3<float> acc[R];
    for (int ph = 0; ph < 2; ++ph) {
      const int pend = ph == 0 ? sp : b1;
      if (threadIdx.x == 0) s_plan.cur = ph == 0 ? b0 : sp, s_plan.coff = 0;
      __syncthreads();
      while (true) {
        if (threadIdx.x < 32) plan_tile<TILE>(s_plan, pend, p2p_src, leaf_start);
        __syncthreads();
        const int np = s_plan.np;
        if (np == 0) break;
        const int total  = s_plan.poff[np];
        const int npairs = (total + 1) >> 1;
        for (int q = threadIdx.x; q < npairs; q += P2P_BLOCK) {
          const int j0    = tile_site(s_plan, 2 * q);
          const float4 r0 = rel(j0);
          // an odd tile ends with a source of zero moment far from the leaf
          const bool two  = 2 * q + 1 < total;
          const int j1    = two ? tile_site(s_plan, 2 * q + 1) : j0;
          const float4 r1 = two ? rel(j1) : make_float4(1e4f, 0.f, 0.f, 1.f);
          s_xy[q] = make_float4(r0.x, r1.x, r0.y, r1.y);
          s_zs[q] = make_float4(r0.z, r1.z, r0.w, r1.w);
          s_site[2 * q]     = j0;
          s_site[2 * q + 1] = two ? j1 : -1;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < npairs * nr; e += P2P_BLOCK) {
          const int q = e / nr, r = e - q * nr;
          if (!((live >> r) & 1u)) continue;
          const float* m0 = src + 3 * ((size_t)s_site[2 * q] + (size_t)(c0 + r) * st.x);
          float mx1 = 0.f, my1 = 0.f, mz1 = 0.f;
          if (s_site[2 * q + 1] >= 0) {
            const float* m1 = src + 3 * ((size_t)s_site[2 * q + 1] + (size_t)(c0 + r) * st.x);
            mx1 = m1[0], my1 = m1[1], mz1 = m1[2];
          }
          s_mxy[q * R + r] = make_float4(m0[0], mx1, m0[1], my1);
          s_mz[q * R + r]  = make_float2(m0[2], mz1);
        }
        __syncthreads();
        if (active) {
          float2 FX[R], FY[R], FZ[R];
#pragma unroll
          for (int r = 0; r < R; ++r) FX[r] = FY[r] = FZ[r] = f2(0.f);
          // every copy live: the copies' updates run unguarded, so that
          // their eight independent chains interleave
          const bool all_live = nr == R && live == (R == 32 ? ~0u : (1u << R) - 1u);
          auto sweep = [&](auto damped, auto all) {
            constexpr bool D  = decltype(damped)::value;
            constexpr bool AL = decltype(all)::value;
#pragma unroll 1
            for (int jj = g; jj < npairs; jj += S) {
              const float4 xy = s_xy[jj], zs = s_zs[jj];
              const float2 x  = __fadd2_rn(make_float2(xy.x, xy.y), nX);
              const float2 y  = __fadd2_rn(make_float2(xy.z, xy.w), nY);
              const float2 z  = __fadd2_rn(make_float2(zs.x, zs.y), nZ);
              const float2 r2 = __ffma2_rn(x, x, __ffma2_rn(y, y, __fmul2_rn(z, z)));
              float2 ir;
              if (D) {
                ir.x = fminf(rsqrt_approx(r2.x), 1e4f);
                ir.y = fminf(rsqrt_approx(r2.y), 1e4f);
              } else {
                ir.x = r2.x > 0.f ? rsqrt_approx(r2.x) : 0.f;
                ir.y = r2.y > 0.f ? rsqrt_approx(r2.y) : 0.f;
              }
              const float2 ir2 = __fmul2_rn(ir, ir);
              const float2 ir3 = __fmul2_rn(ir2, ir);
              const float2 ir5 = __fmul2_rn(ir3, ir2);
              float2 Af, Bn;
              if (D) {
                float2 tt = __fmul2_rn(__fmul2_rn(AI, make_float2(zs.z, zs.w)), __fmul2_rn(r2, ir));
                tt.x = fmaxf(tt.x, -126.f);
                tt.y = fmaxf(tt.y, -126.f);
                const float2 e  = make_float2(ex2_approx(tt.x), ex2_approx(tt.y));
                const float2 np2 = __ffma2_rn(tt, __ffma2_rn(tt, f2(-LN2SQ_2), f2(LN2)), f2(-1.f));
                const float2 q3 = __ffma2_rn(
                      tt, __ffma2_rn(tt, __ffma2_rn(tt, f2(-LN2CU_2), f2(LN2SQ_3_2)), f2(-3.f * LN2)),
                      f2(3.f));
                Af = __fmul2_rn(ir3, __ffma2_rn(np2, e, f2(1.f)));
                Bn = __fmul2_rn(ir5, __ffma2_rn(q3, e, f2(-3.f)));
              } else {
                Af = ir3;
                Bn = __fmul2_rn(ir5, f2(-3.f));
              }
#pragma unroll
              for (int r = 0; r < R; ++r) {
                if (AL || ((live >> r) & 1u)) {
                  const float4 mxy = s_mxy[jj * R + r];
                  const float2 mz  = s_mz[jj * R + r];
                  const float2 mx = make_float2(mxy.x, mxy.y), my = make_float2(mxy.z, mxy.w);
                  const float2 md = __ffma2_rn(mx, x, __ffma2_rn(my, y, __fmul2_rn(mz, z)));
                  const float2 nC = __fmul2_rn(md, Bn);
                  FX[r] = __ffma2_rn(x, nC, __ffma2_rn(mx, Af, FX[r]));
                  FY[r] = __ffma2_rn(y, nC, __ffma2_rn(my, Af, FY[r]));
                  FZ[r] = __ffma2_rn(z, nC, __ffma2_rn(mz, Af, FZ[r]));
                }
              }
            }
          };
          if (all_live) {
            if (DAMP && ph == 0)
              sweep(std::true_type{}, std::true_type{});
            else
              sweep(std::false_type{}, std::true_type{});
          } else {
            if (DAMP && ph == 0)
              sweep(std::true_type{}, std::false_type{});
            else
              sweep(std::false_type{}, std::false_type{});
          }
#pragma unroll
          for (int r = 0; r < R; ++r)
            acc[r].add(FX[r].x + FX[r].y, FY[r].x + FY[r].y, FZ[r].x + FZ[r].y);
        }
        __syncthreads();
      }
    }
    if (active) {
      float* rr = &s_red[(g * nT + t) * 3 * R];
#pragma unroll
      for (int r = 0; r < R; ++r)
        rr[3 * r] = acc[r].gx(), rr[3 * r + 1] = acc[r].gy(), rr[3 * r + 2] = acc[r].gz();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < nT * nr; e += P2P_BLOCK) {
      const int i = e / nr, r = e - i * nr;
      if (!((live >> r) & 1u)) continue;
      float f0 = 0.f, f1 = 0.f, f2v = 0.f;
      for (int gg = 0; gg < S; ++gg) {
        const float* rr = &s_red[(gg * nT + i) * 3 * R + 3 * r];
        f0 += rr[0], f1 += rr[1], f2v += rr[2];
      }
      float* o = Fnear + (size_t)slot * 3 * n + 3 * ((size_t)a0 + tb + i + (size_t)(c0 + r) * st.x);
      o[0] = f0, o[1] = f1, o[2] = f2v;
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Near field in double-float arithmetic (dipole sources): the FP64-accurate
// pass of the mixed solver's residual B x, on the FP32 pipe.  Same items,
// tiles and damping split as the FP32 pass; each pair is evaluated in
// double-float (about 1e-13 relative per term), accumulated in double-float
// and written in FP64.  Separations are exact in their high parts because
// the FP32 coordinates are snapped to a common grid.  Packed FP32x2
// arithmetic evaluates one target against two staged sources per operation
// (the dd2 helpers of dd.cuh); the per-pair branches become per-half
// selects: the self pair (R = 0), sites without a damping partner
// (a = 0) and v >= 50 keep the undamped tensor; with MODE 0 the damping
// factors come from the double-float exponential where v < 20 and from the
// FP32 deficit (< 5e-7 there) elsewhere; with MODE 1 (every v >= 20) from
// the FP32 deficit only.
// ---------------------------------------------------------------------------
// Thole factors of pairs whose v = a R is at least 20 (every pair of the
// partners with v >= 27 for the whole leaf pair): 1 - f_E = (1 + v + v^2/2)
// e^-v <= 4.6e-7 and 1 - f_T = 1 - f_E + v^3/6 e^-v, so G1 f_E = G1 - G1 (1 -
// f_E) with the correction formed in FP32 from FP32 v (its rounding, ~1e-7 of
// a term below 4.6e-7 of G1, stays below 1e-13 of G1) and added to the low
// part; pairs with v >= 50 or without a damping partner (a = 0) keep G1, G2.
__device__ __forceinline__ void dd2_damp_far(const float2& a, const float2& v, dd2& G1,
                                             dd2& G2) {
  const bool dx = a.x > 0.f && v.x < 50.f, dy = a.y > 0.f && v.y < 50.f;
  const float2 e = make_float2(expf(-v.x), expf(-v.y));
  const float2 u = pmul(pfma(v, pfma(v, p2(0.5f), p2(1.f)), p2(1.f)), e);
  const float2 w = pmul(pmul(pmul(pmul(v, v), v), p2(1.f / 6.f)), e);
  G1.l = psel(dx, dy, pfma(pneg(G1.h), u, G1.l), G1.l);
  G2.l = psel(dx, dy, pfma(pneg(G2.h), padd(u, w), G2.l), G2.l);
}

// The Thole factors of a packed pair, in place on G1 = -R^-3 and
// G2 = 3 R^-5: v in FP32 chooses the form, the double-float exponential
// where v < 20 (MODE 0 only) and the FP32 correction of dd2_damp_far
// elsewhere.
template <int MODE>
__device__ __forceinline__ void dd2_thole(const dd2& ai, const dd2& s, const dd2& r2,
                                          const dd2& ir, const float* eh, const float* el,
                                          dd2& G1, dd2& G2) {
  const dd2 zero = {p2(0.f), p2(0.f)};
  const float2 a32 = pmul(ai.h, s.h);
  const float2 v32 = pmul(a32, pmul(r2.h, ir.h));
  const bool sx = MODE == 0 && v32.x < 20.f, sy = MODE == 0 && v32.y < 20.f;
  dd2 G1n = G1, G2n = G2;
  if (sx || sy) {
    const dd2 a   = dd2_mul(ai, s);
    const dd2 v   = dd2_mul(a, dd2_mul(r2, ir));
    const dd2 vc  = dd2_sel(sx, sy, v, zero);  // in range of the exponential's table
    const dd2 e   = dd2_exp_neg(vc, eh, el);
    const dd2 v2  = dd2_sqr(vc);
    const dd2 u   = dd2_add(dd2_two_sum(p2(1.f), vc.h),
                            {pmul(p2(0.5f), v2.h), pfma(p2(0.5f), v2.l, vc.l)});
    const dd2 w   = dd2_mul(dd2_mul(v2, vc), {p2(1.f / 6.f), p2(DD_SIXTH_LO)});
    const dd2 fEd = dd2_add(dd2{p2(1.f), p2(0.f)}, dd2_neg(dd2_mul(u, e)));
    const dd2 fTd = dd2_add(fEd, dd2_neg(dd2_mul(w, e)));
    const bool nx = sx && a.h.x > 0.f, ny = sy && a.h.y > 0.f;
    G1n = dd2_sel(nx, ny, dd2_mul(G1, fEd), G1);
    G2n = dd2_sel(nx, ny, dd2_mul(G2, fTd), G2);
  }
  dd2_damp_far(a32, v32, G1, G2);
  G1 = dd2_sel(sx, sy, G1n, G1);
  G2 = dd2_sel(sx, sy, G2n, G2);
}

struct DDSrc2 {
  dd2 x, y, z, s, mx, my, mz;
};
template <bool DAMP, int MODE>
__device__ __forceinline__ void dd2_pair_m1(const dd2& tx, const dd2& ty, const dd2& tz,
                                            const dd2& ai, const DDSrc2& q, const float* eh,
                                            const float* el, dd2 (&f)[3]) {
  const dd2 x  = {psub(tx.h, q.x.h), psub(tx.l, q.x.l)};
  const dd2 y  = {psub(ty.h, q.y.h), psub(ty.l, q.y.l)};
  const dd2 z  = {psub(tz.h, q.z.h), psub(tz.l, q.z.l)};
  const dd2 r2 = dd2_add(dd2_add_lazy(dd2_sqr_full(x), dd2_sqr_full(y)), dd2_sqr_full(z));
  const bool okx = r2.h.x > 0.f, oky = r2.h.y > 0.f;  // false: a site paired with itself
  const dd2 zero = {p2(0.f), p2(0.f)};
  const dd2 ir   = dd2_sel(okx, oky, dd2_rsqrt(dd2_sel(okx, oky, r2, {p2(1.f), p2(0.f)})), zero);
  const dd2 ir2  = dd2_sqr(ir);
  const dd2 ir3  = dd2_mul(ir2, ir);
  dd2 G1         = dd2_neg(ir3);
  dd2 G2         = dd2_mul_f(dd2_mul(ir3, ir2), p2(3.f));
  if (DAMP && MODE < 2) dd2_thole<MODE>(ai, q.s, r2, ir, eh, el, G1, G2);
  const dd2 mr = dd2_add(dd2_add_lazy(dd2_mul(q.mx, x), dd2_mul(q.my, y)), dd2_mul(q.mz, z));
  const dd2 sg = dd2_mul(mr, G2);
  f[0] = dd2_add_lazy(f[0], dd2_neg(dd2_add_lazy(dd2_mul(q.mx, G1), dd2_mul(sg, x))));
  f[1] = dd2_add_lazy(f[1], dd2_neg(dd2_add_lazy(dd2_mul(q.my, G1), dd2_mul(sg, y))));
  f[2] = dd2_add_lazy(f[2], dd2_neg(dd2_add_lazy(dd2_mul(q.mz, G1), dd2_mul(sg, z))));
}

// One target per thread (its packed accumulators are already 4 x 3 floats),
// sources staged in pairs: positions (high and low parts), s and the
// double-float moments in seven float4 columns per source pair.
constexpr int P2P_DD_PAIRS = 256;  // staged source pairs per tile (512 sources)
template <bool DAMP>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p_dd2(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
                const int* __restrict__ item_split, const int* __restrict__ p2p_src,
                PosArgs<float> pa, const float2* __restrict__ src,
                const float2* __restrict__ etab, double damping, double* __restrict__ Fnear) {
  constexpr int TILE = 2 * P2P_DD_PAIRS;
  __shared__ float4 s_q[7][P2P_DD_PAIRS];
  __shared__ float s_eh[DD_EXP_TAB], s_el[DD_EXP_TAB];
  __shared__ TilePlan s_plan;
  __shared__ double s_red[P2P_BLOCK * 3];

  for (int k = threadIdx.x; k < DD_EXP_TAB; k += P2P_BLOCK) {
    const float2 e = etab[k];
    s_eh[k] = e.x, s_el[k] = e.y;
  }
  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int sp = item_split[blockIdx.x];
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const dd dmp = dd_from(damping);

  for (int tb = 0; tb < nA; tb += P2P_BLOCK) {
    const int nT = min(P2P_BLOCK, nA - tb);
    const int S  = P2P_BLOCK / nT;
    const int t = threadIdx.x % nT, g = threadIdx.x / nT;
    const bool active = g < S;
    const SiteRec<float> me = pa.load(a0 + tb + t);
    const dd2 tx = {p2(me.x), p2(me.lx)}, ty = {p2(me.y), p2(me.ly)}, tz = {p2(me.z), p2(me.lz)};
    const dd ai1 = dd_mul(dmp, dd{me.s, me.ls});
    const dd2 ai = {p2(ai1.h), p2(ai1.l)};
    const dd2 zero = {p2(0.f), p2(0.f)};
    dd2 f[3] = {zero, zero, zero};
    // phase 0: sources [b0, sp); phase 1: [sp, b1), every pair with v >= 27
    for (int ph = 0; ph < 2; ++ph) {
      const int pend = ph == 0 ? sp : b1;
      if (threadIdx.x == 0) s_plan.cur = ph == 0 ? b0 : sp, s_plan.coff = 0;
      __syncthreads();
      while (true) {
        if (threadIdx.x < 32) plan_tile<TILE>(s_plan, pend, p2p_src, leaf_start);
        __syncthreads();
        const int np = s_plan.np;
        if (np == 0) break;
        const int total  = s_plan.poff[np];
        const int npairs = (total + 1) >> 1;
        for (int q = threadIdx.x; q < npairs; q += P2P_BLOCK) {
          const int j0 = tile_site(s_plan, 2 * q);
          const SiteRec<float> r0 = pa.load(j0);
          const float2 m0x = src[3 * (size_t)j0], m0y = src[3 * (size_t)j0 + 1],
                       m0z = src[3 * (size_t)j0 + 2];
          // an odd tile ends with a source of zero moment far from the leaf
          SiteRec<float> r1 = r0;
          r1.x += 1e4f, r1.s = 1.f, r1.ls = 0.f;
          float2 m1x = make_float2(0.f, 0.f), m1y = m1x, m1z = m1x;
          if (2 * q + 1 < total) {
            const int j1 = tile_site(s_plan, 2 * q + 1);
            r1  = pa.load(j1);
            m1x = src[3 * (size_t)j1], m1y = src[3 * (size_t)j1 + 1], m1z = src[3 * (size_t)j1 + 2];
          }
          s_q[0][q] = make_float4(r0.x, r1.x, r0.y, r1.y);
          s_q[1][q] = make_float4(r0.z, r1.z, r0.s, r1.s);
          s_q[2][q] = make_float4(r0.lx, r1.lx, r0.ly, r1.ly);
          s_q[3][q] = make_float4(r0.lz, r1.lz, r0.ls, r1.ls);
          s_q[4][q] = make_float4(m0x.x, m1x.x, m0y.x, m1y.x);
          s_q[5][q] = make_float4(m0z.x, m1z.x, m0x.y, m1x.y);
          s_q[6][q] = make_float4(m0y.y, m1y.y, m0z.y, m1z.y);
        }
        __syncthreads();
        if (active) {
          auto sweep = [&](auto mode) {
            constexpr int MD = decltype(mode)::value;
#pragma unroll 1
            for (int jj = g; jj < npairs; jj += S) {
              const float4 A0 = s_q[0][jj], B0 = s_q[1][jj], C0 = s_q[2][jj], D0 = s_q[3][jj];
              const float4 E0 = s_q[4][jj], F0 = s_q[5][jj], G0 = s_q[6][jj];
              DDSrc2 q;
              q.x  = {make_float2(A0.x, A0.y), make_float2(C0.x, C0.y)};
              q.y  = {make_float2(A0.z, A0.w), make_float2(C0.z, C0.w)};
              q.z  = {make_float2(B0.x, B0.y), make_float2(D0.x, D0.y)};
              q.s  = {make_float2(B0.z, B0.w), make_float2(D0.z, D0.w)};
              q.mx = {make_float2(E0.x, E0.y), make_float2(F0.z, F0.w)};
              q.my = {make_float2(E0.z, E0.w), make_float2(G0.x, G0.y)};
              q.mz = {make_float2(F0.x, F0.y), make_float2(G0.z, G0.w)};
              dd2_pair_m1<DAMP, MD>(tx, ty, tz, ai, q, s_eh, s_el, f);
            }
          };
          if (!DAMP || ph == 0)
            sweep(std::integral_constant<int, 0>{});
          else
            sweep(std::integral_constant<int, 1>{});
        }
        __syncthreads();
      }
    }
    if (active) {
      double* r = &s_red[(g * nT + t) * 3];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        // the two halves' sums, added in double-float, then widened
        const dd h0 = {f[c].h.x, f[c].l.x}, h1 = {f[c].h.y, f[c].l.y};
        r[c] = dd_to(dd_add(h0, h1));
      }
    }
    __syncthreads();
    if (threadIdx.x < nT) {
      double o3[3] = {0, 0, 0};
      for (int gg = 0; gg < S; ++gg)
#pragma unroll
        for (int c = 0; c < 3; ++c) o3[c] += s_red[(gg * nT + threadIdx.x) * 3 + c];
      double* o = Fnear + (size_t)slot * 3 * n + 3 * (size_t)(a0 + tb + threadIdx.x);
      o[0] = o3[0], o[1] = o3[1], o[2] = o3[2];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Double-float near field over a batch's right-hand sides together (the
// residual counterpart of k_p2p32_m1_multi): the pair tensor G1 I + G2 r r^T
// in double-float (separation, 1/R powers, Thole factors) once per pair,
// applied to the source moments of every copy.  Same arithmetic per term as
// dd2_pair_m1; one target per thread with R packed accumulators; the
// per-copy sums are reduced and written one copy at a time.
// ---------------------------------------------------------------------------
template <bool DAMP, int MODE>
__device__ __forceinline__ void dd2_pair_tensor(const dd2& tx, const dd2& ty, const dd2& tz,
                                                const dd2& ai, const dd2& qx, const dd2& qy,
                                                const dd2& qz, const dd2& qs, const float* eh,
                                                const float* el, dd2& x, dd2& y, dd2& z,
                                                dd2& G1, dd2& G2) {
  x = {psub(tx.h, qx.h), psub(tx.l, qx.l)};
  y = {psub(ty.h, qy.h), psub(ty.l, qy.l)};
  z = {psub(tz.h, qz.h), psub(tz.l, qz.l)};
  const dd2 r2 = dd2_add(dd2_add_lazy(dd2_sqr_full(x), dd2_sqr_full(y)), dd2_sqr_full(z));
  const bool okx = r2.h.x > 0.f, oky = r2.h.y > 0.f;  // false: a site paired with itself
  const dd2 zero = {p2(0.f), p2(0.f)};
  const dd2 ir   = dd2_sel(okx, oky, dd2_rsqrt(dd2_sel(okx, oky, r2, {p2(1.f), p2(0.f)})), zero);
  const dd2 ir2  = dd2_sqr(ir);
  const dd2 ir3  = dd2_mul(ir2, ir);
  G1 = dd2_neg(ir3);
  G2 = dd2_mul_f(dd2_mul(ir3, ir2), p2(3.f));
  if (DAMP && MODE < 2) dd2_thole<MODE>(ai, qs, r2, ir, eh, el, G1, G2);
}

constexpr int P2PM_DD_PAIRS = 80;  // staged source pairs per tile (160 sources)
template <bool DAMP>
__global__ void __launch_bounds__(P2P_BLOCK)
      k_p2p_dd2_multi(int n, const int* __restrict__ leaf_start, const int4* __restrict__ items,
                      const int* __restrict__ item_split, const int2* __restrict__ item_stride,
                      int c0, int nr, const int* __restrict__ p2p_src, PosArgs<float> pa,
                      const float2* __restrict__ src, const float2* __restrict__ etab,
                      double damping, double* __restrict__ Fnear) {
  constexpr int TILE = 2 * P2PM_DD_PAIRS;
  constexpr int R    = P2PM_MAXR;
  __shared__ float4 s_g[4][P2PM_DD_PAIRS];       // positions (high, low) and s
  __shared__ float4 s_m[3][P2PM_DD_PAIRS * R];   // per copy: the moments' pairs
  __shared__ int s_site[TILE];
  __shared__ float s_eh[DD_EXP_TAB], s_el[DD_EXP_TAB];
  __shared__ TilePlan s_plan;
  __shared__ double s_red[P2P_BLOCK * 3];

  for (int k = threadIdx.x; k < DD_EXP_TAB; k += P2P_BLOCK) {
    const float2 e = etab[k];
    s_eh[k] = e.x, s_el[k] = e.y;
  }
  const int4 it = items[blockIdx.x];
  const int A = it.x, b0 = it.y, b1 = it.z, slot = it.w;
  const int2 st = item_stride[blockIdx.x];
  const int sp  = item_split[blockIdx.x];
  const int a0 = leaf_start[A], nA = leaf_start[A + 1] - a0;
  const dd dmp = dd_from(damping);

  for (int tb = 0; tb < nA; tb += P2P_BLOCK) {
    const int nT = min(P2P_BLOCK, nA - tb);
    const int S  = P2P_BLOCK / nT;
    const int t = threadIdx.x % nT, g = threadIdx.x / nT;
    const bool active = g < S;
    const SiteRec<float> me = pa.load(a0 + tb + t);
    const dd2 tx = {p2(me.x), p2(me.lx)}, ty = {p2(me.y), p2(me.ly)}, tz = {p2(me.z), p2(me.lz)};
    const dd ai1 = dd_mul(dmp, dd{me.s, me.ls});
    const dd2 ai = {p2(ai1.h), p2(ai1.l)};
    const dd2 zero = {p2(0.f), p2(0.f)};
    dd2 f[R][3];
#pragma unroll
    for (int r = 0; r < R; ++r) f[r][0] = f[r][1] = f[r][2] = zero;
    for (int ph = 0; ph < 2; ++ph) {
      const int pend = ph == 0 ? sp : b1;
      if (threadIdx.x == 0) s_plan.cur = ph == 0 ? b0 : sp, s_plan.coff = 0;
      __syncthreads();
      while (true) {
        if (threadIdx.x < 32) plan_tile<TILE>(s_plan, pend, p2p_src, leaf_start);
        __syncthreads();
        const int np = s_plan.np;
        if (np == 0) break;
        const int total  = s_plan.poff[np];
        const int npairs = (total + 1) >> 1;
        for (int q = threadIdx.x; q < npairs; q += P2P_BLOCK) {
          const int j0 = tile_site(s_plan, 2 * q);
          const SiteRec<float> r0 = pa.load(j0);
          // an odd tile ends with a source of zero moment far from the leaf
          SiteRec<float> r1 = r0;
          r1.x += 1e4f, r1.s = 1.f, r1.ls = 0.f;
          int j1 = -1;
          if (2 * q + 1 < total) j1 = tile_site(s_plan, 2 * q + 1), r1 = pa.load(j1);
          s_g[0][q] = make_float4(r0.x, r1.x, r0.y, r1.y);
          s_g[1][q] = make_float4(r0.z, r1.z, r0.s, r1.s);
          s_g[2][q] = make_float4(r0.lx, r1.lx, r0.ly, r1.ly);
          s_g[3][q] = make_float4(r0.lz, r1.lz, r0.ls, r1.ls);
          s_site[2 * q] = j0, s_site[2 * q + 1] = j1;
        }
        __syncthreads();
        for (int e = threadIdx.x; e < npairs * nr; e += P2P_BLOCK) {
          const int q = e / nr, r = e - q * nr;
          const float2* m0 = src + 3 * ((size_t)s_site[2 * q] + (size_t)(c0 + r) * st.x);
          float2 m1x = make_float2(0.f, 0.f), m1y = m1x, m1z = m1x;
          if (s_site[2 * q + 1] >= 0) {
            const float2* m1 = src + 3 * ((size_t)s_site[2 * q + 1] + (size_t)(c0 + r) * st.x);
            m1x = m1[0], m1y = m1[1], m1z = m1[2];
          }
          const float2 m0x = m0[0], m0y = m0[1], m0z = m0[2];
          // {mx.h pair, my.h pair}, {mz.h pair, mx.l pair}, {my.l pair, mz.l pair}
          s_m[0][q * R + r] = make_float4(m0x.x, m1x.x, m0y.x, m1y.x);
          s_m[1][q * R + r] = make_float4(m0z.x, m1z.x, m0x.y, m1x.y);
          s_m[2][q * R + r] = make_float4(m0y.y, m1y.y, m0z.y, m1z.y);
        }
        __syncthreads();
        if (active) {
          // all R copies in this pass: their updates run unguarded
          auto sweep = [&](auto mode, auto all) {
            constexpr int MD  = decltype(mode)::value;
            constexpr bool AL = decltype(all)::value;
#pragma unroll 1
            for (int jj = g; jj < npairs; jj += S) {
              const float4 A0 = s_g[0][jj], B0 = s_g[1][jj], C0 = s_g[2][jj], D0 = s_g[3][jj];
              const dd2 qx = {make_float2(A0.x, A0.y), make_float2(C0.x, C0.y)};
              const dd2 qy = {make_float2(A0.z, A0.w), make_float2(C0.z, C0.w)};
              const dd2 qz = {make_float2(B0.x, B0.y), make_float2(D0.x, D0.y)};
              const dd2 qs = {make_float2(B0.z, B0.w), make_float2(D0.z, D0.w)};
              dd2 x, y, z, G1, G2;
              dd2_pair_tensor<DAMP, MD>(tx, ty, tz, ai, qx, qy, qz, qs, s_eh, s_el, x, y, z, G1,
                                        G2);
#pragma unroll
              for (int r = 0; r < R; ++r) {
                if (AL || r < nr) {
                  const float4 E0 = s_m[0][jj * R + r], F0 = s_m[1][jj * R + r],
                               G0 = s_m[2][jj * R + r];
                  const dd2 mx = {make_float2(E0.x, E0.y), make_float2(F0.z, F0.w)};
                  const dd2 my = {make_float2(E0.z, E0.w), make_float2(G0.x, G0.y)};
                  const dd2 mz = {make_float2(F0.x, F0.y), make_float2(G0.z, G0.w)};
                  const dd2 mr =
                        dd2_add(dd2_add_lazy(dd2_mul(mx, x), dd2_mul(my, y)), dd2_mul(mz, z));
                  const dd2 sg = dd2_mul(mr, G2);
                  f[r][0] = dd2_add_lazy(f[r][0], dd2_neg(dd2_add_lazy(dd2_mul(mx, G1), dd2_mul(sg, x))));
                  f[r][1] = dd2_add_lazy(f[r][1], dd2_neg(dd2_add_lazy(dd2_mul(my, G1), dd2_mul(sg, y))));
                  f[r][2] = dd2_add_lazy(f[r][2], dd2_neg(dd2_add_lazy(dd2_mul(mz, G1), dd2_mul(sg, z))));
                }
              }
            }
          };
          if (nr == R) {
            if (!DAMP || ph == 0)
              sweep(std::integral_constant<int, 0>{}, std::true_type{});
            else
              sweep(std::integral_constant<int, 1>{}, std::true_type{});
          } else {
            if (!DAMP || ph == 0)
              sweep(std::integral_constant<int, 0>{}, std::false_type{});
            else
              sweep(std::integral_constant<int, 1>{}, std::false_type{});
          }
        }
        __syncthreads();
      }
    }
    // one copy at a time through the reduction buffer
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (r >= nr) break;
      if (active) {
        double* rr = &s_red[(g * nT + t) * 3];
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          const dd h0 = {f[r][c].h.x, f[r][c].l.x}, h1 = {f[r][c].h.y, f[r][c].l.y};
          rr[c] = dd_to(dd_add(h0, h1));
        }
      }
      __syncthreads();
      if (threadIdx.x < nT) {
        double o3[3] = {0, 0, 0};
        for (int gg = 0; gg < S; ++gg)
#pragma unroll
          for (int c = 0; c < 3; ++c) o3[c] += s_red[(gg * nT + threadIdx.x) * 3 + c];
        double* o = Fnear + (size_t)slot * 3 * n +
                    3 * ((size_t)a0 + tb + threadIdx.x + (size_t)(c0 + r) * st.x);
        o[0] = o3[0], o[1] = o3[1], o[2] = o3[2];
      }
      __syncthreads();
    }
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
// Powers of an offset, kept in shared memory (x, y, z blocks of PW values)
// so that the table-driven monomials index them without local memory.
template <typename T>
__device__ __forceinline__ void powers3(T x, T y, T z, int p, T* pw) {
  powers<T>(x, p, pw);
  powers<T>(y, p, pw + PW);
  powers<T>(z, p, pw + 2 * PW);
}
template <typename T>
__device__ __forceinline__ T mono3(const T* pw, int e) {
  return pw[e & 15] * pw[PW + ((e >> 4) & 15)] * pw[2 * PW + (e >> 8)];
}

// Offset c - x_q of site q from the expansion centre of cell c.
template <typename T>
struct CellPos;
template <>
struct CellPos<double> {
  const double4_32a* center;
  const double4_32a* pos;
  __device__ void d(int c, int q, double& x, double& y, double& z) const {
    const double4_32a cc = center[c], p = pos[q];
    x = cc.x - p.x, y = cc.y - p.y, z = cc.z - p.z;
  }
};
template <>
struct CellPos<float> {
  const float4* off;
  const int* ref;
  const float4* hi;
  const float4* lo;
  __device__ void d(int c, int q, float& x, float& y, float& z) const {
    const float4 o = off[c];
    const int r    = ref[c];
    const float4 hr = hi[r], lr = lo[r], hq = hi[q], lq = lo[q];
    x = o.x + ((hr.x - hq.x) + (lr.x - lq.x));
    y = o.y + ((hr.y - hq.y) + (lr.y - lq.y));
    z = o.z + ((hr.z - hq.z) + (lr.z - lq.z));
  }
};

// Centre difference c_a - c_b (FP32 path: through the cells' reference sites).
template <typename T>
__device__ __forceinline__ void centre_diff(const TreeView& tv, const CellPos<T>& cp, int a, int b,
                                            T& x, T& y, T& z);
template <>
__device__ __forceinline__ void centre_diff<double>(const TreeView& tv, const CellPos<double>& cp,
                                                    int a, int b, double& x, double& y,
                                                    double& z) {
  const double4_32a ca = tv.center[a], cb = tv.center[b];
  x = ca.x - cb.x, y = ca.y - cb.y, z = ca.z - cb.z;
}
template <>
__device__ __forceinline__ void centre_diff<float>(const TreeView& tv, const CellPos<float>& cp,
                                                   int a, int b, float& x, float& y, float& z) {
  // c_a - c_b = (c_a - x_ref(a)) - (c_b - x_ref(b)) + (x_ref(a) - x_ref(b))
  const float4 oa = cp.off[a], ob = cp.off[b];
  const int ra = cp.ref[a], rb = cp.ref[b];
  const float4 ha = cp.hi[ra], la = cp.lo[ra], hb = cp.hi[rb], lb = cp.lo[rb];
  x = (oa.x - ob.x) + ((ha.x - hb.x) + (la.x - lb.x));
  y = (oa.y - ob.y) + ((ha.y - hb.y) + (la.y - lb.y));
  z = (oa.z - ob.z) + ((ha.z - hb.z) + (la.z - lb.z));
}

// Leaf multipoles (P2M): block per leaf, thread per multipole row; the powers
// of each site's offset from the leaf centre and its moments are staged in
// shared memory.
template <typename T>
__global__ void __launch_bounds__(128)
      k_p2m_leaf(TreeView tv, OpsView ov, CellPos<T> cp, const T* __restrict__ src,
                 T* __restrict__ M) {
  __shared__ T s_pw[P2M_LEAF_SITES * 3 * PW];
  __shared__ T s_src[P2M_LEAF_SITES * 6];
  const int leaf = blockIdx.x, cell = tv.leaf_cell[leaf];
  const int ns = ncomp(ov.m), row = threadIdx.x;
  const int a0 = tv.leaf_start[leaf], a1 = tv.leaf_start[leaf + 1];
  int t0 = 0, t1 = 0;
  if (row < ov.msize) t0 = ov.p2m_ptr[row], t1 = ov.p2m_ptr[row + 1];
  T acc = 0;
  for (int b0 = a0; b0 < a1; b0 += P2M_LEAF_SITES) {
    const int nb = min(P2M_LEAF_SITES, a1 - b0);
    __syncthreads();
    for (int t = threadIdx.x; t < nb; t += blockDim.x) {
      T x, y, z;
      cp.d(cell, b0 + t, x, y, z);
      powers3<T>(x, y, z, ov.p, s_pw + 3 * PW * t);
      for (int c = 0; c < ns; ++c) s_src[ns * t + c] = src[(size_t)(b0 + t) * ns + c];
    }
    __syncthreads();
    if (row < ov.msize)
      for (int q = 0; q < nb; ++q)
        for (int t = t0; t < t1; ++t)
          acc += mono3(s_pw + 3 * PW * q, ov.exps[ov.p2m_j[t]]) * s_src[ns * q + ov.p2m_k[t]];
  }
  if (row < ov.msize) M[(size_t)cell * ov.msize + row] = acc;
}

// Upward pass above the leaves, one block per task {cell, leaves}: thread
// `row` adds the M2M shifts of the task's leaf multipoles straight to the
// cell centre (the shift is exact, so going through the intermediate levels
// changes nothing).  Partial expansions per task; k_msum adds a cell's tasks.
template <typename T>
__global__ void __launch_bounds__(128)
      k_m2m_tasks(TreeView tv, OpsView ov, const int4* __restrict__ tasks,
                  const int* __restrict__ task_leaf, CellPos<T> cp, const T* __restrict__ M,
                  T* __restrict__ Mpart) {
  __shared__ T s_pw[M2M_TASK_LEAVES * 3 * PW];
  __shared__ int s_lc[M2M_TASK_LEAVES];
  const int4 tk  = tasks[blockIdx.x];
  const int cell = tk.x, row = threadIdx.x, nl = tk.z - tk.y;
  if (threadIdx.x < nl) {
    const int lc = tv.leaf_cell[task_leaf[tk.y + threadIdx.x]];
    T x, y, z;
    centre_diff<T>(tv, cp, cell, lc, x, y, z);
    powers3<T>(x, y, z, ov.p, s_pw + 3 * PW * threadIdx.x);
    s_lc[threadIdx.x] = lc;
  }
  __syncthreads();
  if (row >= ov.msize) return;
  const int t0 = ov.m2m_ptr[row], t1 = ov.m2m_ptr[row + 1];
  T acc = 0;
  for (int k = 0; k < nl; ++k) {
    const T* Mc = M + (size_t)s_lc[k] * ov.msize;
    const T* pw = s_pw + 3 * PW * k;
    for (int t = t0; t < t1; ++t) acc += mono3(pw, ov.exps[ov.m2m_j[t]]) * Mc[ov.m2m_k[t]];
  }
  Mpart[(size_t)blockIdx.x * ov.msize + row] = acc;
}

// Downward pass: block per leaf, thread per local-expansion row; the M2L-only
// expansions of the cells on the leaf's path to the root are shifted to the
// leaf centre and summed (the leaf's own, at zero shift, included).
constexpr int L2L_STAGE = 32;
template <typename T>
__global__ void __launch_bounds__(128)
      k_l2l_leaf(TreeView tv, OpsView ov, CellPos<T> cp, const T* __restrict__ L,
                 T* __restrict__ Lleaf) {
  __shared__ T s_pw[L2L_STAGE * 3 * PW];
  __shared__ int s_c[L2L_STAGE];
  const int leaf = blockIdx.x, lc = tv.leaf_cell[leaf], row = threadIdx.x;
  const int u0 = tv.lanc_ptr[leaf], u1 = tv.lanc_ptr[leaf + 1];
  const int q = ov.p - ov.m;
  int t0 = 0, t1 = 0;
  if (row < ov.lsize) t0 = ov.l2l_ptr[row], t1 = ov.l2l_ptr[row + 1];
  T acc = 0;
  for (int b0 = u0; b0 < u1; b0 += L2L_STAGE) {
    const int nb = min(L2L_STAGE, u1 - b0);
    __syncthreads();
    if (threadIdx.x < nb) {
      const int c = tv.lanc_cell[b0 + threadIdx.x];
      T x, y, z;
      centre_diff<T>(tv, cp, lc, c, x, y, z);
      powers3<T>(x, y, z, q, s_pw + 3 * PW * threadIdx.x);
      s_c[threadIdx.x] = c;
    }
    __syncthreads();
    if (row < ov.lsize)
      for (int k = 0; k < nb; ++k) {
        const T* Lc = L + (size_t)s_c[k] * ov.lsize;
        const T* pw = s_pw + 3 * PW * k;
        for (int t = t0; t < t1; ++t) acc += mono3(pw, ov.exps[ov.l2l_j[t]]) * Lc[ov.l2l_k[t]];
      }
  }
  if (row < ov.lsize) Lleaf[(size_t)leaf * ov.lsize + row] = acc;
}

// ---------------------------------------------------------------------------
// The same passes for dipole sources at the orders with straight-line
// operators (m2l_gen.cuh): every thread applies a whole operator (all rows)
// with the powers, monomials and accumulators in registers, instead of one
// table-driven row per thread.
//  - P2M: block per leaf; thread t takes sites t, t + 64, ...; the threads'
//    expansions are added in thread order through shared memory.
//  - M2M: eight tasks per block, a thread per task leaf; the leaves' shifts
//    of a task are added in leaf order.
//  - L2L: thread per leaf, its M2L-only ancestors in order.
// ---------------------------------------------------------------------------
constexpr int SHIFT_THREADS = 64;
template <int P>
struct Shifts;
#define CPPE_DEF_SHIFTS(MM, PP, LS, MS)                                                          \
  template <>                                                                                   \
  struct Shifts<PP> {                                                                           \
    static constexpr int ls = LS, ms = MS, mst = m_stride(MS);                                  \
    template <typename T>                                                                       \
    __device__ static void p2m(T x, T y, T z, T s0, T s1, T s2, T* acc) {                      \
      p2m_m1_p##PP<T>(x, y, z, s0, s1, s2, acc);                                                \
    }                                                                                           \
    template <typename T>                                                                       \
    __device__ static void m2m(T x, T y, T z, const T* Mc, T* acc) {                           \
      m2m_m1_p##PP<T>(x, y, z, Mc, acc);                                                        \
    }                                                                                           \
    template <typename T>                                                                       \
    __device__ static void l2l(T x, T y, T z, const T* Lc, T* acc) {                           \
      l2l_m1_p##PP<T>(x, y, z, Lc, acc);                                                        \
    }                                                                                           \
    template <typename T>                                                                       \
    __device__ static void l2p(T x, T y, T z, const T* Lc, T& f0, T& f1, T& f2) {              \
      l2p_m1_p##PP<T>(x, y, z, Lc, f0, f1, f2);                                                 \
    }                                                                                           \
  };
CPPE_SHIFTS_GENERATED(CPPE_DEF_SHIFTS)
#undef CPPE_DEF_SHIFTS

template <typename T, int P>
__global__ void __launch_bounds__(SHIFT_THREADS)
      k_p2m_leaf_fixed(TreeView tv, CellPos<T> cp, const T* __restrict__ src, T* __restrict__ M,
                       const int* __restrict__ leaf_seg, const int* __restrict__ seg_done) {
  constexpr int MS = Shifts<P>::ms, MST = Shifts<P>::mst;
  __shared__ T s_part[SHIFT_THREADS * (MS + 1)];
  const int leaf = blockIdx.x, cell = tv.leaf_cell[leaf];
  if (seg_done && seg_done[leaf_seg[leaf]]) return;  // finished segment of a batch
  const int a0 = tv.leaf_start[leaf], a1 = tv.leaf_start[leaf + 1];
  T acc[MS];
#pragma unroll
  for (int r = 0; r < MS; ++r) acc[r] = T(0);
  for (int q = a0 + (int)threadIdx.x; q < a1; q += SHIFT_THREADS) {
    T x, y, z;
    cp.d(cell, q, x, y, z);
    const T* sq = src + 3 * (size_t)q;
    Shifts<P>::p2m(x, y, z, sq[0], sq[1], sq[2], acc);
  }
#pragma unroll
  for (int r = 0; r < MS; ++r) s_part[threadIdx.x * (MS + 1) + r] = acc[r];
  __syncthreads();
  for (int r = threadIdx.x; r < MST; r += SHIFT_THREADS) {
    T v = T(0);
    if (r < MS)
      for (int t = 0; t < SHIFT_THREADS; ++t) v += s_part[t * (MS + 1) + r];
    M[(size_t)cell * MST + r] = v;
  }
}

template <typename T, int P>
__global__ void __launch_bounds__(SHIFT_THREADS)
      k_m2m_tasks_fixed(TreeView tv, const int4* __restrict__ tasks, int ntask,
                        const int* __restrict__ task_leaf, CellPos<T> cp, const T* __restrict__ M,
                        T* __restrict__ Mpart, const int* __restrict__ cell_seg,
                        const int* __restrict__ seg_done) {
  constexpr int MS  = Shifts<P>::ms, MST = Shifts<P>::mst;
  constexpr int TPB = SHIFT_THREADS / M2M_TASK_LEAVES;  // tasks per block
  __shared__ T s_part[SHIFT_THREADS * (MS + 1)];
  const int g = threadIdx.x / M2M_TASK_LEAVES, sl = threadIdx.x % M2M_TASK_LEAVES;
  const int task = blockIdx.x * TPB + g;
  T acc[MS];
#pragma unroll
  for (int r = 0; r < MS; ++r) acc[r] = T(0);
  // a batch's masked segment: its partials are not read
  const bool live = task < ntask && !(seg_done && seg_done[cell_seg[tasks[task].x]]);
  if (live) {
    const int4 tk = tasks[task];
    if (tk.y + sl < tk.z) {
      const int lc = tv.leaf_cell[task_leaf[tk.y + sl]];
      T x, y, z;
      centre_diff<T>(tv, cp, tk.x, lc, x, y, z);
      Shifts<P>::m2m(x, y, z, M + (size_t)lc * MST, acc);
    }
  }
#pragma unroll
  for (int r = 0; r < MS; ++r) s_part[threadIdx.x * (MS + 1) + r] = acc[r];
  __syncthreads();
  for (int idx = threadIdx.x; idx < TPB * MST; idx += SHIFT_THREADS) {
    const int gg = idx / MST, r = idx - gg * MST, tsk = blockIdx.x * TPB + gg;
    if (tsk >= ntask) continue;
    T v = T(0);
    if (r < MS)
      for (int k = 0; k < M2M_TASK_LEAVES; ++k)
        v += s_part[(gg * M2M_TASK_LEAVES + k) * (MS + 1) + r];
    Mpart[(size_t)tsk * MST + r] = v;
  }
}

template <typename T, int P>
__global__ void __launch_bounds__(SHIFT_THREADS)
      k_l2l_leaf_fixed(TreeView tv, CellPos<T> cp, const T* __restrict__ L,
                       T* __restrict__ Lleaf, const int* __restrict__ leaf_seg,
                       const int* __restrict__ seg_done) {
  constexpr int LS = Shifts<P>::ls;
  const int leaf = blockIdx.x * SHIFT_THREADS + threadIdx.x;
  if (leaf >= tv.nleaves) return;
  if (seg_done && seg_done[leaf_seg[leaf]]) return;  // a batch's masked segment
  const int lc = tv.leaf_cell[leaf];
  T acc[LS];
#pragma unroll
  for (int r = 0; r < LS; ++r) acc[r] = T(0);
  for (int u = tv.lanc_ptr[leaf]; u < tv.lanc_ptr[leaf + 1]; ++u) {
    const int c = tv.lanc_cell[u];
    T x, y, z;
    centre_diff<T>(tv, cp, lc, c, x, y, z);
    Shifts<P>::l2l(x, y, z, L + (size_t)c * LS, acc);
  }
#pragma unroll
  for (int r = 0; r < LS; ++r) Lleaf[(size_t)leaf * LS + r] = acc[r];
}

// M of every cell with upward tasks: the sum of its task partials in order.
template <typename T>
__global__ void k_msum(int ncells, int msize, const int* __restrict__ cell_task_ptr,
                       const T* __restrict__ Mpart, T* __restrict__ M,
                       const int* __restrict__ cell_seg, const int* __restrict__ seg_done) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int cell = (int)(gid / msize), row = (int)(gid % msize);
  if (cell >= ncells) return;
  if (seg_done && seg_done[cell_seg[cell]]) return;  // a batch's masked segment
  const int t0 = cell_task_ptr[cell], t1 = cell_task_ptr[cell + 1];
  if (t0 == t1) return;
  T acc = 0;
  for (int t = t0; t < t1; ++t) acc += Mpart[(size_t)t * msize + row];
  M[(size_t)cell * msize + row] = acc;
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
// Rows of the symmetric near field (Geometry::sym_*), read by the finishing
// pass in place of the near-field slots when `buf` is set.
template <typename T>
struct SymRows {
  const int* rows = nullptr;        // rows per leaf
  const long long* off = nullptr;   // first float of each leaf's rows
  const T* buf = nullptr;
};

// Segments whose sites the finishing pass leaves alone (a batch's segments
// that are finished or evaluated by another operator): skip[leaf_seg[leaf]].
struct SegSkip {
  const int* leaf_seg = nullptr;
  const int* skip     = nullptr;
};

template <typename T, int M, int MODE, int P = 0>
__global__ void __launch_bounds__(FINISH_BLOCK) k_finish(int n, const int* __restrict__ leaf_nslot, const T* __restrict__ Fnear,
                         SymRows<T> sr, SegSkip sk,
                         int use_fmm,
                         TreeView tv, OpsView ov, const T* __restrict__ L, PosArgs<T> pa,
                         CellPos<T> cp, const T* __restrict__ src,
                         int damp, T damping, const int* __restrict__ corr_ptr,
                         const int* __restrict__ corr_idx, const T* __restrict__ ainv6,
                         T* __restrict__ out, double* __restrict__ out64, double sign,
                         ReduceSlots dot) {
  constexpr int NS = ncomp(M);
  __shared__ double sh[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  T dv[1]     = {T(0)};  // (FP32 products for the FP32 apply: see block_sum)
  if (sk.skip && i < n && sk.skip[sk.leaf_seg[tv.site_leaf[i]]]) return;  // (no grid sum then)
  if (i < n) {
    T f[3] = {0, 0, 0};
    if (sr.buf) {
      // the site's rows of the symmetric near field, in row order
      const int Lf = tv.site_leaf[i];
      const int a  = tv.leaf_start[Lf];
      const long long stride = 3 * (long long)(tv.leaf_start[Lf + 1] - a);
      const T* q = sr.buf + sr.off[Lf] + 3 * (long long)(i - a);
      for (int k = 0; k < sr.rows[Lf]; ++k, q += stride) f[0] += q[0], f[1] += q[1], f[2] += q[2];
    } else {
      const int nsl = leaf_nslot[tv.site_leaf[i]];
      for (int s = 0; s < nsl; ++s) {
        const T* q = Fnear + (size_t)s * 3 * n + 3 * (size_t)i;
        f[0] += q[0], f[1] += q[1], f[2] += q[2];
      }
    }
    if (use_fmm) {
      // L2P of the leaf's accumulated local expansion
      const int leaf = tv.site_leaf[i];
      T dx, dy, dz;
      cp.d(tv.leaf_cell[leaf], i, dx, dy, dz);
      const T* Lc = L + (size_t)leaf * ov.lsize;
      if constexpr (P > 0) {
        Shifts<P>::l2p(-dx, -dy, -dz, Lc, f[0], f[1], f[2]);
      } else {
        __shared__ T s_pw[FINISH_BLOCK * 3 * PW];
        T* pw = s_pw + 3 * PW * threadIdx.x;
        powers3<T>(-dx, -dy, -dz, ov.p - ov.m, pw);
        for (int w = 0; w < ov.nl2p; ++w) {
          const T v   = mono3(pw, ov.exps[ov.l2p_j[w]]) * Lc[ov.l2p_n[w]];
          const int c = ov.l2p_c[w];  // (no dynamic index into f: keeps it in registers)
          f[0] -= c == 0 ? v : T(0);
          f[1] -= c == 1 ? v : T(0);
          f[2] -= c == 2 ? v : T(0);
        }
      }
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
      dv[0] = sv[0] * o0 + sv[1] * o1 + sv[2] * o2;
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
template <typename T>
static CellPos<T> cell_pos(const Geometry& g);
template <>
CellPos<double> cell_pos<double>(const Geometry& g) {
  return CellPos<double>{reinterpret_cast<const double4_32a*>(g.center.p), g.pos64.p};
}
template <>
CellPos<float> cell_pos<float>(const Geometry& g) {
  return CellPos<float>{g.cell_off.p, g.cell_ref.p, g.hi32.p, g.lo32.p};
}

template <typename T, int M>
static void launch_p2p(const Geometry& g, bool damp, bool fast, const T* src, T damping,
                       T* Fnear, cudaStream_t s, const int* seg_done) {
  const int grid = (int)g.h_items.size();
  const int* lseg = seg_done ? g.leaf_seg.p : nullptr;
  if (seg_done && !lseg) fail(CPPE_GPU_INVALID_ARG, "segment mask without segments");
  if constexpr (std::is_same<T, float>::value && M == 1) {
    if (!g.h_mitems.empty() && g.ncopies > 1) {
      // a batch's right-hand sides together, up to P2PM_MAXR per launch
      const int mg = (int)g.h_mitems.size();
      // right-hand sides per pass (8, or 4 with fewer registers) and tile size,
      // as the batch's schedule autotuner chose them
      const int rc = g.multi_copies == 4 ? 4 : P2PM_MAXR;
      for (int c0 = 0; c0 < g.ncopies; c0 += rc) {
        const int nr = std::min(rc, g.ncopies - c0);
#define CG_MULTI(D, P, R)                                                                   \
  k_p2p32_m1_multi<D, P, R><<<mg, P2P_BLOCK, 0, s>>>(                                       \
        g.n, g.leaf_start.p, g.mitems.p, g.mitem_split.p, g.mitem_stride.p, c0, nr,         \
        g.p2p_src.p, g.hi32.p, g.lo32.p, src, damping, Fnear, lseg, seg_done)
#define CG_MULTI_R(D, P) \
  if (rc == 4) CG_MULTI(D, P, 4); else CG_MULTI(D, P, P2PM_MAXR)
        const int tile = g.multi_tile > 0 ? g.multi_tile : P2PM_PAIRS;
        if (tile == 96) {
          if (damp) { CG_MULTI_R(true, 96); } else { CG_MULTI_R(false, 96); }
        } else if (tile == 120) {
          if (damp) { CG_MULTI_R(true, 120); } else { CG_MULTI_R(false, 120); }
        } else {
          if (damp) { CG_MULTI_R(true, P2PM_PAIRS); } else { CG_MULTI_R(false, P2PM_PAIRS); }
        }
#undef CG_MULTI_R
#undef CG_MULTI
        CG_LAUNCH();
      }
      return;
    }
    if (damp)
      k_p2p32_m1<true><<<grid, P2P_BLOCK, 0, s>>>(
            g.n, g.leaf_start.p, g.items.p, g.item_split.p, g.p2p_src.p, g.hi32.p, g.lo32.p, src,
            damping, Fnear, lseg, seg_done);
    else
      k_p2p32_m1<false><<<grid, P2P_BLOCK, 0, s>>>(
            g.n, g.leaf_start.p, g.items.p, g.item_split.p, g.p2p_src.p, g.hi32.p, g.lo32.p, src,
            damping, Fnear, lseg, seg_done);
    CG_LAUNCH();
    return;
  }
#define CG_P2P(D, F)                                                                            \
  k_p2p<T, M, D, F><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.p2p_src.p, \
                                               pos_args<T>(g), src, damping, Fnear, lseg,   \
                                               seg_done)
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
  // By default the far-field chain runs at the highest priority: where it is
  // shorter than the near-field pass (a chain of small, latency-bound
  // kernels) its blocks are scheduled ahead of the near field's instead of
  // after them.  Where the chain is the longer part (high orders, large
  // systems) the default priority lets the two share the GPU better; the
  // schedule tuner picks between them by measurement.
  int least = 0, greatest = 0;
  CG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  CG_CUDA(cudaStreamCreateWithPriority(&hi, cudaStreamNonBlocking, greatest));
  CG_CUDA(cudaStreamCreateWithPriority(&lo, cudaStreamNonBlocking, least));
  s = hi;
  CG_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
  CG_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
}
void SideStream::destroy() {
  if (hi) cudaStreamSynchronize(hi);
  if (lo) cudaStreamSynchronize(lo);
  if (join) cudaEventDestroy(join);
  if (fork) cudaEventDestroy(fork);
  if (hi) cudaStreamDestroy(hi);
  if (lo) cudaStreamDestroy(lo);
  s = hi = lo = nullptr, fork = join = nullptr;
}

__global__ void k_split_dd_vec(long n, const double* __restrict__ in, float2* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = in[i];
  const float h  = (float)v;
  out[i]         = make_float2(h, (float)(v - (double)h));
}

__global__ void k_split_dd(long n, const double* __restrict__ in, float2* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = in[i];
  const float h  = (float)v;
  out[i]         = make_float2(h, (float)(v - (double)h));
}

static void launch_p2p_dd(const Geometry& g, bool damp, const double* src, double damping,
                          FieldWork<double>& w, cudaStream_t s) {
  const long n3 = 3L * g.n;
  w.dd_src.alloc(std::max(1L, n3));
  k_split_dd<<<(unsigned)((n3 + 255) / 256), 256, 0, s>>>(n3, src, w.dd_src.p);
  CG_LAUNCH();
  if (!g.h_mitems.empty() && g.ncopies > 1) {
    // a batch's right-hand sides together, up to P2PM_MAXR per launch
    const int mg = (int)g.h_mitems.size();
    for (int c0 = 0; c0 < g.ncopies; c0 += P2PM_MAXR) {
      const int nr = std::min(P2PM_MAXR, g.ncopies - c0);
      if (damp)
        k_p2p_dd2_multi<true><<<mg, P2P_BLOCK, 0, s>>>(
              g.n, g.leaf_start.p, g.mitems.p, g.mitem_split.p, g.mitem_stride.p, c0, nr,
              g.p2p_src.p, pos_args<float>(g), w.dd_src.p, g.dd_exp.p, damping, w.Fnear.p);
      else
        k_p2p_dd2_multi<false><<<mg, P2P_BLOCK, 0, s>>>(
              g.n, g.leaf_start.p, g.mitems.p, g.mitem_split.p, g.mitem_stride.p, c0, nr,
              g.p2p_src.p, pos_args<float>(g), w.dd_src.p, g.dd_exp.p, damping, w.Fnear.p);
      CG_LAUNCH();
    }
    return;
  }
  const int grid = (int)g.h_items.size();
  if (damp)
    k_p2p_dd2<true><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.item_split.p,
                                               g.p2p_src.p, pos_args<float>(g), w.dd_src.p,
                                               g.dd_exp.p, damping, w.Fnear.p);
  else
    k_p2p_dd2<false><<<grid, P2P_BLOCK, 0, s>>>(g.n, g.leaf_start.p, g.items.p, g.item_split.p,
                                                g.p2p_src.p, pos_args<float>(g), w.dd_src.p,
                                                g.dd_exp.p, damping, w.Fnear.p);
  CG_LAUNCH();
}

template <typename T>
void eval_field(const Geometry& g, const DeviceOps* ops, FieldWork<T>& w, int m, const T* src,
                bool damp, double damping, FinishMode mode, const T* ainv6, T* out,
                double* out64, double sign, const ReduceSlots* dot, cudaStream_t s,
                const PhaseEvents* pe, int near_mode, const SideStream* side,
                const int* seg_done) {
  const TreeView tv = g.view();
  OpsView ov{};
  int fixedP  = 0;  // order of the straight-line expansion operators in use (0: tables)
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
  // finished segments of a batch (near field, leaf multipoles and M2L skip them)
  const int* lseg = seg_done ? g.leaf_seg.p : nullptr;
  const int* cseg = seg_done ? g.cell_seg.p : nullptr;
  if (seg_done && (!lseg || (g.fmm && !cseg)))
    fail(CPPE_GPU_INVALID_ARG, "segment mask without segments");
  if (g.fmm) {
    if (!ops || ops->host.m != m) fail(CPPE_GPU_INVALID_ARG, "FMM tables missing for order");
    ov = ops->view();
    fixedP = (m == 1 && (ov.p == 5 || ov.p == 6)) ? ov.p : 0;
    // the fixed-order kernels store multipoles with a stride of a multiple
    // of four coefficients (16-byte aligned rows, vector loads in M2L)
    const int mst = fixedP ? m_stride(ov.msize) : ov.msize;
    w.M.alloc((size_t)tv.ncells * mst);
    w.L.alloc((size_t)tv.ncells * ov.lsize);
    const int TB = 128;
    const int ntask = (int)g.h_p2m_tasks.size();
    if (tv.nleaves > 0) {
      if (fixedP == 5)
        k_p2m_leaf_fixed<T, 5><<<tv.nleaves, SHIFT_THREADS, 0, fs>>>(tv, cell_pos<T>(g), src, w.M.p,
                                                                       lseg, seg_done);
      else if (fixedP == 6)
        k_p2m_leaf_fixed<T, 6><<<tv.nleaves, SHIFT_THREADS, 0, fs>>>(tv, cell_pos<T>(g), src, w.M.p,
                                                                       lseg, seg_done);
      else
        k_p2m_leaf<T><<<tv.nleaves, TB, 0, fs>>>(tv, ov, cell_pos<T>(g), src, w.M.p);
      CG_LAUNCH();
    }
    if (ntask > 0) {
      w.Mpart.alloc((size_t)ntask * mst);
      const int tb = (ntask + SHIFT_THREADS / M2M_TASK_LEAVES - 1) / (SHIFT_THREADS / M2M_TASK_LEAVES);
      if (fixedP == 5)
        k_m2m_tasks_fixed<T, 5><<<tb, SHIFT_THREADS, 0, fs>>>(
              tv, g.p2m_tasks.p, ntask, g.task_leaf.p, cell_pos<T>(g), w.M.p, w.Mpart.p, cseg,
              seg_done);
      else if (fixedP == 6)
        k_m2m_tasks_fixed<T, 6><<<tb, SHIFT_THREADS, 0, fs>>>(
              tv, g.p2m_tasks.p, ntask, g.task_leaf.p, cell_pos<T>(g), w.M.p, w.Mpart.p, cseg,
              seg_done);
      else
        k_m2m_tasks<T><<<ntask, TB, 0, fs>>>(tv, ov, g.p2m_tasks.p, g.task_leaf.p,
                                            cell_pos<T>(g), w.M.p, w.Mpart.p);
      CG_LAUNCH();
      const long work = (long)tv.ncells * mst;
      k_msum<T><<<(unsigned)((work + 255) / 256), 256, 0, fs>>>(
            tv.ncells, mst, g.cell_task_ptr.p, w.Mpart.p, w.M.p, cseg, seg_done);
      CG_LAUNCH();
    }
    mark(1);
    w.Lpart.alloc((size_t)std::max<size_t>(1, g.h_m2l_chunks.size()) * ov.lsize);
    bool m2l_done = false;
    // tabulated tensors of the distinct M2L vectors (fixed orders): in FP64
    // and double-float, where the recurrence is the expensive part; the FP32
    // translation builds its tensor in registers faster than it loads one
    const T* dtab_t = nullptr;
    if constexpr (std::is_same<T, double>::value)
      if (fixedP && M2L_TABLE_FP64)
        dtab_t = static_cast<const T*>(m2l_dtab<T>(g, ov.m, ov.p, w, false, fs));
    if constexpr (std::is_same<T, double>::value) {
      if (near_mode == NEAR_DD) {
        w.Mdd.alloc((size_t)std::max(1, tv.ncells) * mst);
        const float2* dtdd =
              static_cast<const float2*>(m2l_dtab<T>(g, ov.m, ov.p, w, true, fs));
        m2l_done = launch_m2l_dd(tv, ov.m, ov.p, g.m2l_chunks.p, (int)g.h_m2l_chunks.size(),
                                 g.cell_chunk_ptr.p, w.M.p, mst, w.Mdd.p, w.Lpart.p, w.L.p,
                                 ov.lsize, fs, dtdd, dtdd ? g.m2l_vid.p : nullptr);
      }
    }
    if (m2l_done ||
        launch_m2l_fixed<T>(tv, ov.m, ov.p, g.m2l_chunks.p, (int)g.h_m2l_chunks.size(),
                            g.cell_chunk_ptr.p, w.M.p, w.Lpart.p, w.L.p, ov.lsize, fs, cseg,
                            seg_done, dtab_t, dtab_t ? g.m2l_vid.p : nullptr)) {
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
    w.Lleaf.alloc((size_t)std::max(1, tv.nleaves) * ov.lsize);
    if (tv.nleaves > 0) {
      const int lb = (tv.nleaves + SHIFT_THREADS - 1) / SHIFT_THREADS;
      if (fixedP == 5)
        k_l2l_leaf_fixed<T, 5><<<lb, SHIFT_THREADS, 0, fs>>>(tv, cell_pos<T>(g), w.L.p, w.Lleaf.p,
                                                             lseg, seg_done);
      else if (fixedP == 6)
        k_l2l_leaf_fixed<T, 6><<<lb, SHIFT_THREADS, 0, fs>>>(tv, cell_pos<T>(g), w.L.p, w.Lleaf.p,
                                                             lseg, seg_done);
      else
        k_l2l_leaf<T><<<tv.nleaves, 128, 0, fs>>>(tv, ov, cell_pos<T>(g), w.L.p, w.Lleaf.p);
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
  SymRows<T> sym_rows;  // set when the symmetric near field ran
  if constexpr (std::is_same<T, double>::value) {
    if (near_mode == NEAR_DD && m == 1) {
      launch_p2p_dd(g, damp, src, damping, w, s);
      done = true;
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    if (!done && m == 1 && g.has_sym() && !seg_done) {
      // every unordered pair once (k_p2p32_m1_sym), then each site's rows
      w.Fsym.alloc((size_t)g.sym_floats);
      const int ni = (int)g.h_sym_items.size();
#define CG_SYM(D, K)                                                                    \
  k_p2p32_m1_sym<D, K><<<ni, sym_threads<K>(), 0, s>>>(                                 \
        g.leaf_start.p, g.sym_items.p, g.sym_split.p, g.sym_aoff.p, g.usrc.p, g.usrc_off.p, \
        g.hi32.p, g.lo32.p, src, dampT, w.Fsym.p)
      if (g.sym_pack == 2) {
        if (damp) CG_SYM(true, 2); else CG_SYM(false, 2);
      } else {
        if (damp) CG_SYM(true, 1); else CG_SYM(false, 1);
      }
#undef CG_SYM
      CG_LAUNCH();
      sym_rows.rows = g.sym_leaf_rows.p, sym_rows.off = g.sym_leaf_off.p, sym_rows.buf = w.Fsym.p;
      done          = true;
    }
  }
  if (!done && m == 0) launch_p2p<T, 0>(g, damp, fast, src, dampT, w.Fnear.p, s, seg_done);
  if (!done && m == 1) launch_p2p<T, 1>(g, damp, fast, src, dampT, w.Fnear.p, s, seg_done);
  if (!done && m == 2) launch_p2p<T, 2>(g, damp, fast, src, dampT, w.Fnear.p, s, seg_done);
  mark(4);
  if (fs != s) CG_CUDA(cudaStreamWaitEvent(s, side->join, 0));

  const int FB = FINISH_BLOCK;
  const int nb = (n + FB - 1) / FB;
  ReduceSlots rs{nullptr, nullptr, nullptr};
  if (dot) rs = *dot;
  const T* Lp = g.fmm ? w.Lleaf.p : nullptr;
  SegSkip sk;  // a batch's masked segments (site-value dots only: no grid sum)
  if (seg_done && (!dot || !dot->partials)) sk.leaf_seg = g.leaf_seg.p, sk.skip = seg_done;
#define CG_FINISH(TT, MM, MODE, PP)                                                           \
  k_finish<TT, MM, MODE, PP><<<nb, FB, 0, s>>>(n, g.leaf_nslot.p, w.Fnear.p, sym_rows, sk, g.fmm ? 1 : 0, tv, ov, Lp, \
                                           pos_args<TT>(g), cell_pos<TT>(g), src, damp ? 1 : 0, \
                                           dampT, g.corr_ptr.p, g.corr_idx.p, ainv6, out,    \
                                           out64, sign, rs)
  if (mode == FINISH_APPLY) {
    if (m != 1) fail(CPPE_GPU_INVALID_ARG, "apply mode needs dipole sources");
    if (fixedP == 5)
      CG_FINISH(T, 1, FINISH_APPLY, 5);
    else if (fixedP == 6)
      CG_FINISH(T, 1, FINISH_APPLY, 6);
    else
      CG_FINISH(T, 1, FINISH_APPLY, 0);
  } else {
    if (m == 0) CG_FINISH(T, 0, FINISH_FIELD, 0);
    if (m == 1 && fixedP == 5) CG_FINISH(T, 1, FINISH_FIELD, 5);
    if (m == 1 && fixedP == 6) CG_FINISH(T, 1, FINISH_FIELD, 6);
    if (m == 1 && fixedP == 0) CG_FINISH(T, 1, FINISH_FIELD, 0);
    if (m == 2) CG_FINISH(T, 2, FINISH_FIELD, 0);
  }
#undef CG_FINISH
  CG_LAUNCH();
  mark(5);
}

template void eval_field<double>(const Geometry&, const DeviceOps*, FieldWork<double>&, int,
                                 const double*, bool, double, FinishMode, const double*,
                                 double*, double*, double, const ReduceSlots*, cudaStream_t,
                                 const PhaseEvents*, int, const SideStream*, const int*);
template void eval_field<float>(const Geometry&, const DeviceOps*, FieldWork<float>&, int,
                                const float*, bool, double, FinishMode, const float*, float*,
                                double*, double, const ReduceSlots*, cudaStream_t,
                                const PhaseEvents*, int, const SideStream*, const int*);

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
