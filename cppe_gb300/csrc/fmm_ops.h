// Index tables of the Cartesian FMM operators for source order m and
// expansion order p, in the reference's convention (Dehnen/fmmgen, as in
// src/core/fmm/field_m{0,1,2}.cc):
//   multi-indices ordered by total order, then x-power descending, then
//   y-power descending; M holds orders m..p (Msize = Nterms(p) - Nterms(m-1)),
//   L holds orders 0..p-m (Lsize = Nterms(p-m))   (src/core/fmm/utils.cc:3-20)
//   P2M/M2M  Ms_n += sum_{k<=n, |k|>=m} d^(n-k)/(n-k)! M_k,  d = centre - source
//   M2L      L_n  += sum_{|k|>=m, |n|+|k|<=p} D_(n+k)(d) M_k, D = derivatives of 1/R
//   L2L      Ls_n += sum_{k>=n} d^(k-n)/(k-n)! L_k,           d = child - parent
//   L2P      F_c  -= sum_{n>=e_c} t^(n-e_c)/(n-e_c)! L_n,      t = particle - centre
#pragma once

#include <vector>

namespace cg {

constexpr int PMAX = 8;  // highest supported expansion order (reference: 7)

constexpr int nterms(int p) { return p < 0 ? 0 : (p + 1) * (p + 2) * (p + 3) / 6; }
constexpr int ncomp(int m) { return (m + 1) * (m + 2) / 2; }

// Lanes of the warp-per-target M2L kernel own "slots": a contiguous run of
// terms of one output row.  Long rows are cut so that lanes get similar work.
constexpr int M2L_SLOTS = 8;

struct OpTables {
  int m = 0, p = 0, msize = 0, lsize = 0, moff = 0, nt = 0;
  std::vector<int> exps;  // per multi-index j <= p: a | b << 4 | c << 8
  // CSR rows of (source index, exponent index) terms
  std::vector<int> p2m_ptr, p2m_k, p2m_j;  // rows: M rows; k: source component
  std::vector<int> m2m_ptr, m2m_k, m2m_j;  // rows: M rows; k: M row of child
  std::vector<int> l2l_ptr, l2l_k, l2l_j;  // rows: L rows; k: L row of parent
  std::vector<int> l2p_c, l2p_n, l2p_j;    // flat: component, L row, exponent
  // M2L terms, row-major: term t adds D[m2l_w[t]] * M[m2l_k[t]] to row m2l_row[t]
  std::vector<int> m2l_row, m2l_k, m2l_w;
  // slot schedule: slot s of lane l is slots[(l * M2L_SLOTS + s) * 3 + {row, t0, t1}]
  std::vector<int> slots;
  // per row, the slot ids (l * M2L_SLOTS + s) contributing to it, in fixed order
  std::vector<int> row_slot_ptr, row_slot_id;
  // derivative recurrence for j >= 1 (see fmm.cu): 8 ints per j
  //   q1x q1y q1z (index of n - e_i or -1), q2x q2y q2z (n - 2 e_i or -1),
  //   order o, unused; coefficients are (2o-1) n_i and (o-1) n_i (n_i - 1)
  std::vector<int> drec;
};

OpTables make_op_tables(int m, int p);

}  // namespace cg
