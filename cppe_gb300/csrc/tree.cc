// Host-side octree + interaction lists (reference semantics) and the
// level-/leaf-contiguous layout uploaded to the GPU.
//
// Semantics kept from the reference (src/core/fmm/tree.cc, calculate.cc):
//  * root centre = mean site position, half-width 1.001 * max |x - mean|
//    over the three axes, rmax = sqrt(3 r^2)                   (tree.cc:158-188)
//  * sites are inserted in input order; a cell whose count reaches ncrit is
//    split at once, its ncrit sites re-inserted in their stored order, and a
//    split cell keeps counting arrivals                         (tree.cc:189-209, :111-132)
//  * octant = (x > cx) + 2 (y > cy) + 4 (z > cz); child centre = parent
//    centre +- r/2 per axis                                     (tree.cc:94-109)
//  * dual-tree walk from (root, root): R theta > rmax_A + rmax_B -> M2L(B->A);
//    both leaves -> P2P(A<-B); else split A if B is a leaf or (rmax_A >=
//    rmax_B and A is not a leaf), otherwise split B            (calculate.cc:74-127)
//  * the M2L list is ordered by source cell                    (tree.cc:224-227)
// This file must be compiled without floating-point contraction
// (-ffp-contract=off): the acceptance distance sits exactly on the theta
// boundary for cells offset by (4,4,4) half-widths, and the reference's golden
// FMM errors are reproduced by the uncontracted evaluation only.
#include "tree.h"

#include <algorithm>
#include <cmath>
#include <numeric>

namespace cg {

namespace {

struct Builder {
  const double* xyz;
  int ncrit;
  RefTree& t;

  int add_cell(double x, double y, double z, double r, int parent, int level) {
    int c = (int)t.x.size();
    t.x.push_back(x), t.y.push_back(y), t.z.push_back(z), t.r.push_back(r);
    t.rmax.push_back(std::sqrt(3 * r * r));
    t.parent.push_back(parent), t.level.push_back(level);
    t.nleaf.push_back(0), t.nchild.push_back(0u);
    for (int o = 0; o < 8; ++o) t.child.push_back(0);
    t.leaf.emplace_back();
    t.leaf.back().reserve(ncrit);
    return c;
  }

  int octant(int i, int c) const {
    return (xyz[3 * i] > t.x[c]) + ((xyz[3 * i + 1] > t.y[c]) << 1) +
           ((xyz[3 * i + 2] > t.z[c]) << 2);
  }

  int child_of(int p, int o) {
    if (!(t.nchild[p] & (1u << o))) {
      const double h = t.r[p] / 2.0;
      int c          = add_cell(t.x[p] + h * ((o & 1) * 2 - 1), t.y[p] + h * ((o & 2) - 1),
                                t.z[p] + h * ((o & 4) / 2 - 1), h, p, t.level[p] + 1);
      t.child[8 * p + o] = c;
      t.nchild[p] |= (1u << o);
    }
    return t.child[8 * p + o];
  }

  // Appends site i to cell c and splits c when it becomes full.
  bool place(int c, int i, int depth) {
    t.leaf[c].push_back(i);
    t.nleaf[c] += 1;
    if (t.nleaf[c] < ncrit) return true;
    if (depth > 96) return false;
    for (int k = 0; k < ncrit; ++k) {
      int s  = t.leaf[c][k];
      int ch = child_of(c, octant(s, c));
      if (!place(ch, s, depth + 1)) return false;
    }
    return true;
  }

  bool insert(int i) {
    int c = 0, depth = 0;
    while (t.nleaf[c] >= ncrit) {
      t.nleaf[c] += 1;
      c = child_of(c, octant(i, c));
      if (++depth > 96) return false;
    }
    return place(c, i, depth);
  }
};

void walk(const RefTree& t, int A, int B, double theta, int ncrit,
          std::vector<std::pair<int, int>>& m2l, std::vector<std::pair<int, int>>& p2p) {
  const double dx = t.x[A] - t.x[B];
  const double dy = t.y[A] - t.y[B];
  const double dz = t.z[A] - t.z[B];
  const double R  = std::sqrt(dx * dx + dy * dy + dz * dz);
  const bool leafA = t.nchild[A] == 0, leafB = t.nchild[B] == 0;
  if (R * theta > t.rmax[A] + t.rmax[B]) {
    m2l.emplace_back(B, A);
  } else if (leafA && leafB) {
    if (t.nleaf[B] >= ncrit)
      m2l.emplace_back(B, A);  // unreachable for well-formed trees
    else
      p2p.emplace_back(A, B);
  } else if (leafB || (t.rmax[A] >= t.rmax[B] && !leafA)) {
    for (int o = 0; o < 8; ++o)
      if (t.nchild[A] & (1u << o)) walk(t, t.child[8 * A + o], B, theta, ncrit, m2l, p2p);
  } else {
    for (int o = 0; o < 8; ++o)
      if (t.nchild[B] & (1u << o)) walk(t, A, t.child[8 * B + o], theta, ncrit, m2l, p2p);
  }
}

}  // namespace

bool build_ref_tree(int n, const double* xyz, int ncrit, double theta, RefTree& t,
                    std::string& err) {
  t       = RefTree();
  t.ncrit = ncrit;
  t.theta = theta;
  if (n <= 0) {
    err = "empty system";
    return false;
  }
  if (ncrit < 1) {
    err = "tree_ncrit must be >= 1";
    return false;
  }
  double xa = 0, ya = 0, za = 0;
  for (int i = 0; i < n; ++i) {
    if (!std::isfinite(xyz[3 * i]) || !std::isfinite(xyz[3 * i + 1]) ||
        !std::isfinite(xyz[3 * i + 2])) {
      err = "non-finite site position " + std::to_string(i);
      return false;
    }
    xa += xyz[3 * i], ya += xyz[3 * i + 1], za += xyz[3 * i + 2];
  }
  xa /= n, ya /= n, za /= n;
  double xm = 0, ym = 0, zm = 0;
  for (int i = 0; i < n; ++i) {
    xm = std::max(xm, std::abs(xyz[3 * i] - xa));
    ym = std::max(ym, std::abs(xyz[3 * i + 1] - ya));
    zm = std::max(zm, std::abs(xyz[3 * i + 2] - za));
  }
  double r = (xm > ym ? (xm > zm ? xm : zm) : (ym > zm ? ym : zm)) * 1.001;
  Builder b{xyz, ncrit, t};
  b.add_cell(xa, ya, za, r, 0, 0);
  for (int i = 0; i < n; ++i)
    if (!b.insert(i)) {
      err = "octree depth limit reached: sites coincide (at least " + std::to_string(ncrit) +
            " sites at one position)";
      return false;
    }
  walk(t, 0, 0, theta, ncrit, t.m2l, t.p2p);
  std::stable_sort(t.m2l.begin(), t.m2l.end(),
                   [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
                     return a.first < b.first;
                   });
  return true;
}

void make_layout(const RefTree& t, int n, TreeLayout& L) {
  const int nc = (int)t.x.size();
  L        = TreeLayout();
  L.n      = n;
  L.ncells = nc;
  // Renumber cells by (level, creation index).
  int maxl = 0;
  for (int c = 0; c < nc; ++c) maxl = std::max(maxl, t.level[c]);
  L.nlevels = maxl + 1;
  L.level_start.assign(L.nlevels + 1, 0);
  for (int c = 0; c < nc; ++c) L.level_start[t.level[c] + 1]++;
  for (int l = 0; l < L.nlevels; ++l) L.level_start[l + 1] += L.level_start[l];
  std::vector<int> fill(L.level_start.begin(), L.level_start.end() - 1);
  std::vector<int> new_of_old(nc);
  L.old_of_new.resize(nc);
  for (int c = 0; c < nc; ++c) {
    int k           = fill[t.level[c]]++;
    new_of_old[c]   = k;
    L.old_of_new[k] = c;
  }
  L.center.resize(4 * (size_t)nc);
  L.parent.resize(nc);
  L.is_leaf.assign(nc, 0);
  L.child_ptr.assign(nc + 1, 0);
  for (int k = 0; k < nc; ++k) {
    int c               = L.old_of_new[k];
    L.center[4 * k]     = t.x[c];
    L.center[4 * k + 1] = t.y[c];
    L.center[4 * k + 2] = t.z[c];
    L.center[4 * k + 3] = t.r[c];
    L.parent[k]         = c == 0 ? -1 : new_of_old[t.parent[c]];
    L.is_leaf[k]        = t.nleaf[c] < t.ncrit ? 1 : 0;
    for (int o = 0; o < 8; ++o)
      if (t.nchild[c] & (1u << o)) L.child_idx.push_back(new_of_old[t.child[8 * c + o]]);
    L.child_ptr[k + 1] = (int)L.child_idx.size();
  }
  // Leaves in renumbered order; particles leaf-contiguous.
  L.leaf_of_cell.assign(nc, -1);
  L.leaf_start.push_back(0);
  L.perm.reserve(n);
  for (int k = 0; k < nc; ++k) {
    if (!L.is_leaf[k]) continue;
    int c                = L.old_of_new[k];
    L.leaf_of_cell[k]    = (int)L.leaf_cell.size();
    L.leaf_cell.push_back(k);
    for (int q = 0; q < t.nleaf[c]; ++q) L.perm.push_back(t.leaf[c][q]);
    L.leaf_start.push_back((int)L.perm.size());
  }
  L.nleaves = (int)L.leaf_cell.size();
  L.inv_perm.assign(n, -1);
  for (int k = 0; k < (int)L.perm.size(); ++k) L.inv_perm[L.perm[k]] = k;
  // M2L grouped by target (stable: keeps the reference's source order).
  L.m2l_ptr.assign(nc + 1, 0);
  for (auto& pr : t.m2l) L.m2l_ptr[new_of_old[pr.second] + 1]++;
  for (int k = 0; k < nc; ++k) L.m2l_ptr[k + 1] += L.m2l_ptr[k];
  L.m2l_src.resize(t.m2l.size());
  {
    std::vector<int> pos(L.m2l_ptr.begin(), L.m2l_ptr.end() - 1);
    for (auto& pr : t.m2l) L.m2l_src[pos[new_of_old[pr.second]]++] = new_of_old[pr.first];
  }
  // P2P grouped by target leaf (walk order).
  L.p2p_ptr.assign(L.nleaves + 1, 0);
  for (auto& pr : t.p2p) L.p2p_ptr[L.leaf_of_cell[new_of_old[pr.first]] + 1]++;
  for (int k = 0; k < L.nleaves; ++k) L.p2p_ptr[k + 1] += L.p2p_ptr[k];
  L.p2p_src.resize(t.p2p.size());
  {
    std::vector<int> pos(L.p2p_ptr.begin(), L.p2p_ptr.end() - 1);
    for (auto& pr : t.p2p) {
      int a                  = L.leaf_of_cell[new_of_old[pr.first]];
      int b                  = L.leaf_of_cell[new_of_old[pr.second]];
      L.p2p_src[pos[a]++]    = b;
      L.p2p_pairs += (long)t.nleaf[pr.first] * t.nleaf[pr.second];
    }
  }
}

}  // namespace cg
