// Test infrastructure (oracle) -- never linked into the product.
//
// A thin C ABI over the reference's own FMM/direct-sum engine
// (src/core/fmm/{tree,calculate,utils,field_m0,field_m1,field_m2}.cc), which
// the recipe in oracle/Makefile compiles in place from the reference tree into
// oracle/_ref/libcppe_ref.so.  The functions below restate, on top of that
// engine, the few lines of reference glue that need Eigen:
//   ref_multipole_fields  <- MultipoleFields::compute   src/core/electric_fields.cc:106-189
//   ref_bmatrix_apply     <- BMatrix::apply             src/core/bmatrix.cc:9-40
//                            BMatrix::apply_diagonal    src/core/bmatrix.cc:53-62
//   ref_solve             <- InducedMoments::compute    src/core/electric_fields.cc:191-239
// plus accessors that expose the reference tree and its interaction lists
// (tree.cc:134-237, calculate.cc:74-127) so the product's tree builder can be
// checked list-for-list.
#include <cmath>
#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "calculate.hh"
#include "tree.hh"
#include "utils.hh"

namespace libcppe {
int multipole_components(int k) { return (k + 1) * (k + 2) / 2; }
}  // namespace libcppe

namespace {

std::vector<libcppe::Potential> make_potentials(int n, const double* xyz,
                                                const int* polarizable,
                                                const double* alpha_iso,
                                                const int* excl_ptr,
                                                const int* excl_idx) {
  std::vector<libcppe::Potential> pots(n);
  for (int i = 0; i < n; ++i) {
    pots[i].m_R = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
    if (excl_ptr) {
      for (int e = excl_ptr[i]; e < excl_ptr[i + 1]; ++e)
        pots[i].m_exclusions.push_back(excl_idx[e]);
    }
    if (polarizable && polarizable[i]) {
      pots[i].m_is_polarizable = true;
      pots[i].m_pol.iso        = alpha_iso[i];
    }
  }
  return pots;
}

template <int M>
void field_of(std::vector<libcppe::Potential>& pots, std::vector<double>& S, int fmm,
              int ncrit, int order, double theta, double damping, double* F) {
  auto tree = build_shared_tree<M, 3>(pots, S.data(), ncrit, order, theta, damping);
  if (fmm)
    tree->compute_field_fmm(F);
  else
    tree->compute_field_exact(F);
}

// 3x3 inverse by cofactors (row-major, symmetric input from 6 upper values).
void inv3_from6(const double* a6, double* out9) {
  double a[9] = {a6[0], a6[1], a6[2], a6[1], a6[3], a6[4], a6[2], a6[4], a6[5]};
  double c00 = a[4] * a[8] - a[5] * a[7];
  double c01 = a[5] * a[6] - a[3] * a[8];
  double c02 = a[3] * a[7] - a[4] * a[6];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  double id  = 1.0 / det;
  out9[0]    = c00 * id;
  out9[1]    = (a[2] * a[7] - a[1] * a[8]) * id;
  out9[2]    = (a[1] * a[5] - a[2] * a[4]) * id;
  out9[3]    = c01 * id;
  out9[4]    = (a[0] * a[8] - a[2] * a[6]) * id;
  out9[5]    = (a[2] * a[3] - a[0] * a[5]) * id;
  out9[6]    = c02 * id;
  out9[7]    = (a[1] * a[6] - a[0] * a[7]) * id;
  out9[8]    = (a[0] * a[4] - a[1] * a[3]) * id;
}

struct RefBMatrix {
  int n;
  std::vector<libcppe::Potential> pots;
  std::vector<double> ainv;  // 9 per site
  std::vector<double> a6;
  int fmm, ncrit, order;
  double theta, damping;

  void apply(const double* in, double* out) {
    std::vector<double> S(in, in + 3 * n);
    std::vector<double> F(3 * n, 0.0);
    field_of<1>(pots, S, fmm, ncrit, order, theta, damping, F.data());
    for (int i = 0; i < n; ++i) {
      const double* A = &ainv[9 * i];
      for (int r = 0; r < 3; ++r)
        out[3 * i + r] = F[3 * i + r] + (A[3 * r] * in[3 * i] + A[3 * r + 1] * in[3 * i + 1] +
                                         A[3 * r + 2] * in[3 * i + 2]);
    }
  }
  void apply_alpha(const double* in, double* out) {
    for (int i = 0; i < n; ++i) {
      const double* s = &a6[6 * i];
      double x = in[3 * i], y = in[3 * i + 1], z = in[3 * i + 2];
      out[3 * i]     = s[0] * x + s[1] * y + s[2] * z;
      out[3 * i + 1] = s[1] * x + s[3] * y + s[4] * z;
      out[3 * i + 2] = s[2] * x + s[4] * y + s[5] * z;
    }
  }
};

RefBMatrix make_bmatrix(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
                        const int* excl_idx, int fmm, int ncrit, int order, double theta,
                        double damping) {
  RefBMatrix B;
  B.n = n;
  std::vector<int> pol(n, 1);
  std::vector<double> iso(n);
  for (int i = 0; i < n; ++i)
    iso[i] = (alpha6[6 * i] + alpha6[6 * i + 3] + alpha6[6 * i + 5]) / 3.0;
  B.pots = make_potentials(n, xyz, pol.data(), iso.data(), excl_ptr, excl_idx);
  B.ainv.resize(9 * n);
  for (int i = 0; i < n; ++i) inv3_from6(&alpha6[6 * i], &B.ainv[9 * i]);
  B.a6.assign(alpha6, alpha6 + 6 * n);
  B.fmm     = fmm;
  B.ncrit   = ncrit;
  B.order   = order;
  B.theta   = theta;
  B.damping = damping;
  return B;
}

double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0.0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

}  // namespace

extern "C" {

// Field of order-m sources S (m = 0, 1, 2; S holds (m+1)(m+2)/2 values per site)
// at every site, exactly as Tree<m,3>::compute_field_{fmm,exact} returns it.
int ref_field(int m, int n, const double* xyz, const double* S_in, const int* polarizable,
              const double* alpha_iso, const int* excl_ptr, const int* excl_idx, int fmm,
              int ncrit, int order, double theta, double damping, double* F) {
  auto pots = make_potentials(n, xyz, polarizable, alpha_iso, excl_ptr, excl_idx);
  int ns    = (m + 1) * (m + 2) / 2;
  std::vector<double> S(S_in, S_in + ns * n);
  if (m == 0)
    field_of<0>(pots, S, fmm, ncrit, order, theta, damping, F);
  else if (m == 1)
    field_of<1>(pots, S, fmm, ncrit, order, theta, damping, F);
  else if (m == 2)
    field_of<2>(pots, S, fmm, ncrit, order, theta, damping, F);
  else
    return 2;
  return 0;
}

// MultipoleFields::compute (electric_fields.cc:106-189). quad holds the raw
// traceless quadrupoles (xx,xy,xz,yy,yz,zz); the diagonal halving of :146-151
// happens here.  max_order is the largest multipole order of any site.
int ref_multipole_fields(int n, const double* xyz, const double* q, const double* mu,
                         const double* quad, int max_order, const int* polarizable,
                         const double* alpha_iso, const int* excl_ptr, const int* excl_idx,
                         int fmm, int ncrit, int order, double theta, double damping,
                         double* F) {
  if (max_order > 2) return 2;
  auto pots = make_potentials(n, xyz, polarizable, alpha_iso, excl_ptr, excl_idx);
  std::vector<double> charges(q, q + n);
  std::vector<double> f(3 * n);
  for (int i = 0; i < 3 * n; ++i) F[i] = 0.0;
  // compute_field_exact accumulates into its output (calculate.cc:262-300), so
  // each tree gets a fresh zeroed buffer as in electric_fields.cc:158,170,181.
  field_of<0>(pots, charges, fmm, ncrit, order, theta, damping, f.data());
  for (int i = 0; i < 3 * n; ++i) F[i] += f[i];
  if (max_order > 0) {
    std::vector<double> dip(mu, mu + 3 * n);
    std::fill(f.begin(), f.end(), 0.0);
    field_of<1>(pots, dip, fmm, ncrit, order, theta, damping, f.data());
    for (int i = 0; i < 3 * n; ++i) F[i] -= f[i];
  }
  if (max_order > 1) {
    std::vector<double> qd(6 * n);
    for (int i = 0; i < n; ++i) {
      qd[6 * i + 0] = 0.5 * quad[6 * i + 0];
      qd[6 * i + 1] = quad[6 * i + 1];
      qd[6 * i + 2] = quad[6 * i + 2];
      qd[6 * i + 3] = 0.5 * quad[6 * i + 3];
      qd[6 * i + 4] = quad[6 * i + 4];
      qd[6 * i + 5] = 0.5 * quad[6 * i + 5];
    }
    std::fill(f.begin(), f.end(), 0.0);
    field_of<2>(pots, qd, fmm, ncrit, order, theta, damping, f.data());
    for (int i = 0; i < 3 * n; ++i) F[i] += f[i];
  }
  return 0;
}

// BMatrix::apply (bmatrix.cc:9-40): field of the dipoles `in` plus alpha^-1 in.
int ref_bmatrix_apply(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
                      const int* excl_idx, int fmm, int ncrit, int order, double theta,
                      double damping, const double* in, double* out) {
  RefBMatrix B = make_bmatrix(n, xyz, alpha6, excl_ptr, excl_idx, fmm, ncrit, order, theta,
                              damping);
  B.apply(in, out);
  return 0;
}

// InducedMoments::compute (electric_fields.cc:191-239), Jacobi-preconditioned CG
// with the absolute stopping rule ||r||_2 < thresh.  Returns 0 when converged,
// 1 when maxiter was reached (where the reference throws).
int ref_solve(int n, const double* xyz, const double* alpha6, const int* excl_ptr,
              const int* excl_idx, int fmm, int ncrit, int order, double theta,
              double damping, const double* rhs_in, const double* guess, int make_guess,
              double thresh, int maxiter, double* mu, int* iters, double* rnorm_hist) {
  RefBMatrix B = make_bmatrix(n, xyz, alpha6, excl_ptr, excl_idx, fmm, ncrit, order, theta,
                              damping);
  const size_t N = 3 * (size_t)n;
  std::vector<double> rhs(rhs_in, rhs_in + N), x(N), r(N), z(N), p(N), Ap(N), tmp(N);
  if (make_guess)
    B.apply_alpha(rhs.data(), x.data());
  else
    for (size_t i = 0; i < N; ++i) x[i] = guess ? guess[i] : 0.0;
  B.apply(x.data(), tmp.data());
  for (size_t i = 0; i < N; ++i) r[i] = rhs[i] - tmp[i];
  B.apply_alpha(r.data(), z.data());
  p = z;
  bool converged = false;
  int k          = 0;
  for (; k < maxiter; ++k) {
    B.apply(p.data(), Ap.data());
    double rz    = dot(r, z);
    double alpha = rz / dot(p, Ap);
    for (size_t i = 0; i < N; ++i) x[i] += alpha * p[i];
    for (size_t i = 0; i < N; ++i) r[i] -= alpha * Ap[i];
    double rnorm = std::sqrt(dot(r, r));
    if (rnorm_hist) rnorm_hist[k] = rnorm;
    if (rnorm < thresh) {
      converged = true;
      break;
    }
    std::vector<double> z1(N);
    B.apply_alpha(r.data(), z1.data());
    double beta = dot(z1, r) / rz;
    for (size_t i = 0; i < N; ++i) p[i] = z1[i] + beta * p[i];
    z.swap(z1);
  }
  for (size_t i = 0; i < N; ++i) mu[i] = x[i];
  if (iters) *iters = converged ? k + 1 : k;
  return converged ? 0 : 1;
}

// Sizes of the reference tree for the given geometry (Tree<1,3>, no damping).
int ref_tree_info(int n, const double* xyz, int ncrit, int order, double theta, int* ncells,
                  long* nm2l, long* np2p) {
  auto pots = make_potentials(n, xyz, nullptr, nullptr, nullptr, nullptr);
  std::vector<double> S(3 * n, 0.0);
  auto tree = build_shared_tree<1, 3>(pots, S.data(), ncrit, order, theta, 0.0);
  *ncells   = (int)tree->cells.size();
  *nm2l     = (long)tree->M2L_list.size();
  *np2p     = (long)tree->P2P_list.size();
  return 0;
}

// Full dump of the reference tree: per cell (in creation order) the centre and
// half-width, parent, level, child-occupancy mask and nleaf; the particle
// indices of every cell with nleaf < ncrit (ncrit slots per cell, -1 padded);
// and the M2L (source, target) and P2P (target, source) lists in the reference's
// order (M2L after its sort by source).
int ref_tree_lists(int n, const double* xyz, int ncrit, int order, double theta,
                   double* cell_xyzr, int* cell_parent, int* cell_level, int* cell_nchild,
                   int* cell_nleaf, int* cell_leaves, int* m2l, int* p2p) {
  auto pots = make_potentials(n, xyz, nullptr, nullptr, nullptr, nullptr);
  std::vector<double> S(3 * n, 0.0);
  auto tree = build_shared_tree<1, 3>(pots, S.data(), ncrit, order, theta, 0.0);
  for (size_t c = 0; c < tree->cells.size(); ++c) {
    const Cell& C        = tree->cells[c];
    cell_xyzr[4 * c + 0] = C.x;
    cell_xyzr[4 * c + 1] = C.y;
    cell_xyzr[4 * c + 2] = C.z;
    cell_xyzr[4 * c + 3] = C.r;
    cell_parent[c]       = (int)C.parent;
    cell_level[c]        = (int)C.level;
    cell_nchild[c]       = (int)C.nchild;
    cell_nleaf[c]        = (int)C.nleaf;
    for (int s = 0; s < ncrit; ++s)
      cell_leaves[c * ncrit + s] =
            ((size_t)s < C.nleaf && C.nleaf < (size_t)ncrit) ? (int)C.leaf[s] : -1;
  }
  for (size_t i = 0; i < tree->M2L_list.size(); ++i) {
    m2l[2 * i]     = (int)tree->M2L_list[i].first;
    m2l[2 * i + 1] = (int)tree->M2L_list[i].second;
  }
  for (size_t i = 0; i < tree->P2P_list.size(); ++i) {
    p2p[2 * i]     = (int)tree->P2P_list[i].first;
    p2p[2 * i + 1] = (int)tree->P2P_list[i].second;
  }
  return 0;
}

}  // extern "C"
