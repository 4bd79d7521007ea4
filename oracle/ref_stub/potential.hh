// Test infrastructure (oracle). Minimal stand-in for the reference's
// src/core/potential.hh so that the reference's Eigen-free FMM sources
// (src/core/fmm/*.cc) compile in place without Eigen. It exposes only the
// members those sources touch (tree.cc:134-165): the site position pointer,
// the exclusion list, the polarizable flag and the isotropic polarizability.
#pragma once
#include <algorithm>
#include <vector>

namespace libcppe {

struct Polarizability {
  double iso = 0.0;
  double get_isotropic_value() { return iso; }
};

class Potential {
 public:
  std::vector<double> m_R{0.0, 0.0, 0.0};
  std::vector<int> m_exclusions;
  Polarizability m_pol;
  bool m_is_polarizable = false;

  double* ptr_position() { return m_R.data(); }
  std::vector<int>& get_exclusions() { return m_exclusions; }
  bool is_polarizable() { return m_is_polarizable; }
  Polarizability& get_polarizability() { return m_pol; }
};

}  // namespace libcppe
