// Host-side octree and interaction lists with the reference's semantics, and
// their flat device-ready layout.
//
// The tree is built once per geometry (the reference rebuilds it on every
// BMatrix::apply, src/core/bmatrix.cc:28-29); the lists are then renumbered
// into level-contiguous cell order and leaf-contiguous particle order so that
// every GPU pass reads contiguous ranges.
#pragma once

#include <string>
#include <utility>
#include <vector>

namespace cg {

// Cells in the reference's creation order (tree.cc:134-237).
struct RefTree {
  int ncrit = 64;
  double theta = 0.5;
  std::vector<double> x, y, z, r, rmax;
  std::vector<int> parent, level, nleaf;
  std::vector<unsigned> nchild;          // occupancy bit mask, bit o = octant o
  std::vector<int> child;                // 8 per cell, valid where the bit is set
  std::vector<std::vector<int>> leaf;    // particle indices (valid while nleaf < ncrit)
  std::vector<std::pair<int, int>> m2l;  // (source, target), sorted by source
  std::vector<std::pair<int, int>> p2p;  // (target, source)
};

// Builds the tree and both lists.  Returns false (with a message) on input the
// reference cannot handle either (coincident sites recurse without end there).
bool build_ref_tree(int n, const double* xyz, int ncrit, double theta, RefTree& t,
                    std::string& err);

// Device-ready layout.
struct TreeLayout {
  int ncells = 0, nlevels = 0, nleaves = 0, n = 0;
  std::vector<int> level_start;   // nlevels+1, cells of level l: [level_start[l], level_start[l+1])
  std::vector<int> old_of_new;    // reference cell index of each renumbered cell
  std::vector<double> center;     // 4 per cell: x, y, z, r
  std::vector<int> parent;        // renumbered parent (root: -1)
  std::vector<int> child_ptr;     // ncells+1, children (octant order) in child_idx
  std::vector<int> child_idx;
  std::vector<int> is_leaf;       // 1 for cells holding particles (nleaf < ncrit)
  std::vector<int> leaf_cell;     // nleaves: renumbered cell of each leaf (ascending)
  std::vector<int> leaf_of_cell;  // ncells: leaf index or -1
  std::vector<int> leaf_start;    // nleaves+1: particle range of each leaf (permuted order)
  std::vector<int> perm;          // n: perm[k] = caller's index of permuted particle k
  std::vector<int> inv_perm;      // n: inverse of perm
  std::vector<int> m2l_ptr;       // ncells+1 (target cells), sources in m2l_src
  std::vector<int> m2l_src;
  std::vector<int> p2p_ptr;       // nleaves+1 (target leaves), source leaves in p2p_src
  std::vector<int> p2p_src;
  long p2p_pairs = 0;             // sum over leaf pairs of n_A * n_B
};

void make_layout(const RefTree& t, int n, TreeLayout& L);

}  // namespace cg
