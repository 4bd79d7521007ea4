// BMatrix, InducedMoments, MultipoleFields, NuclearFields and
// MultipoleExpansion of the host layer: argument packing and calls into the
// C ABI.  All arithmetic of these classes runs in libcppe_gpu.
#include <algorithm>
#include <cmath>
#include <iomanip>
#include <sstream>

#include "cppe_gpu.h"
#include "cppe_host.hh"

namespace libcppe {

cppe_gpu_options to_gpu(const PeOptions& o) {
  cppe_gpu_options g;
  cppe_gpu_default_options(&g);
  // any string other than "fmm" means direct summation (bmatrix.cc:31-36)
  g.summation            = o.summation_induced_fields == "fmm" ? CPPE_GPU_FMM : CPPE_GPU_DIRECT;
  g.tree_ncrit           = o.tree_ncrit;
  g.tree_expansion_order = o.tree_expansion_order;
  g.theta                = o.theta;
  g.damp                 = o.damp_induced ? 1 : 0;
  g.damping_factor       = o.damping_factor_induced;
  g.induced_thresh       = o.induced_thresh;
  g.maxiter              = o.maxiter;
  g.precision            = gpu_config().precision;
  g.device               = gpu_config().device;
  return g;
}

void pack_exclusions(const std::vector<Potential>& pots, std::vector<int>& ptr,
                     std::vector<int>& idx) {
  ptr.assign(1, 0);
  idx.clear();
  for (const auto& p : pots) {
    for (int e : p.get_exclusions()) idx.push_back(e);
    ptr.push_back((int)idx.size());
  }
}

namespace {
void check_size(const Vector& v, size_t n, const char* what) {
  if (v.size() != n)
    throw std::invalid_argument(std::string(what) + ": expected a vector of length " +
                                std::to_string(n) + ", got " + std::to_string(v.size()));
}
}  // namespace

// --- GpuSystem ----------------------------------------------------------------
GpuSystem::GpuSystem(const std::vector<Potential>& polsites, const PeOptions& o)
      : m_n((int)polsites.size()), m_opt(o) {
  m_xyz.reserve(3 * polsites.size());
  m_alpha6.reserve(6 * polsites.size());
  for (const auto& p : polsites) {
    m_xyz.insert(m_xyz.end(), {p.m_x, p.m_y, p.m_z});
    auto a = p.get_polarizability().get_values_vec();
    m_alpha6.insert(m_alpha6.end(), a.begin(), a.end());
  }
  // Exclusions stay global site indices compared against polarizable-site
  // indices, as in the reference tree (tree.cc:145).
  pack_exclusions(polsites, m_eptr, m_eidx);
}

GpuSystem::~GpuSystem() {
  if (m_sys) cppe_gpu_destroy(m_sys);
}

cppe_gpu_system* GpuSystem::get() {
  if (!m_sys) {
    cppe_gpu_options g = to_gpu(m_opt);
    throw_on_status(cppe_gpu_create(m_n, m_xyz.data(), m_alpha6.data(), m_eptr.data(),
                                    m_eidx.empty() ? nullptr : m_eidx.data(), &g, &m_sys));
  }
  return m_sys;
}

// --- BMatrix (bmatrix.cc) -------------------------------------------------------
BMatrix::BMatrix(std::vector<Potential> polsites, const PeOptions& options)
      : m_polsites(std::move(polsites)), m_n_polsites(m_polsites.size()), m_options(options) {
  m_gpu = std::make_shared<GpuSystem>(m_polsites, m_options);
}

Vector BMatrix::apply(const Vector& v) {
  check_size(v, 3 * m_n_polsites, "BMatrix.apply");
  Vector out(v.size());
  throw_on_status(cppe_gpu_bmatrix_apply(m_gpu->get(), v.data(), out.data()));
  return out;
}

Vector BMatrix::apply_diagonal_inverse(const Vector& v) {
  check_size(v, 3 * m_n_polsites, "BMatrix.apply_diagonal_inverse");
  Vector out(v.size());
  throw_on_status(cppe_gpu_apply_diagonal_inverse(m_gpu->get(), v.data(), out.data()));
  return out;
}

Vector BMatrix::apply_diagonal(const Vector& v) {
  check_size(v, 3 * m_n_polsites, "BMatrix.apply_diagonal");
  Vector out(v.size());
  throw_on_status(cppe_gpu_apply_diagonal(m_gpu->get(), v.data(), out.data()));
  return out;
}

Matrix BMatrix::to_dense_matrix() {
  Matrix B(3 * m_n_polsites, 3 * m_n_polsites);
  throw_on_status(cppe_gpu_to_dense(m_gpu->get(), B.data.data()));
  return B;
}

Matrix BMatrix::direct_inverse() {
  Matrix B(3 * m_n_polsites, 3 * m_n_polsites);
  throw_on_status(cppe_gpu_direct_inverse(m_gpu->get(), B.data.data()));
  return B;
}

// --- NuclearFields (electric_fields.cc:58-75) -----------------------------------
NuclearFields::NuclearFields(Molecule mol, std::vector<Potential> potentials)
      : m_potentials(std::move(potentials)), m_mol(std::move(mol)) {
  m_polsites = get_polarizable_sites(m_potentials);
}

Vector NuclearFields::compute() {
  const int n = (int)m_polsites.size();
  Vector F(3 * (size_t)n, 0.0);
  if (n == 0 || m_mol.empty()) return F;
  std::vector<double> xt, xs, q;
  for (const auto& p : m_polsites) xt.insert(xt.end(), {p.m_x, p.m_y, p.m_z});
  for (const auto& a : m_mol) {
    xs.insert(xs.end(), {a.m_x, a.m_y, a.m_z});
    q.push_back((double)a.charge);
  }
  throw_on_status(cppe_gpu_charge_fields(n, xt.data(), (int)m_mol.size(), xs.data(), q.data(),
                                         gpu_config().device, F.data()));
  return F;
}

Matrix NuclearFields::nuclear_gradient() {
  const int n = (int)m_polsites.size(), na = (int)m_mol.size();
  Matrix G(3 * (size_t)na, 3 * (size_t)n);
  if (n == 0 || na == 0) return G;
  std::vector<double> xt, xs, q;
  for (const auto& p : m_polsites) xt.insert(xt.end(), {p.m_x, p.m_y, p.m_z});
  for (const auto& a : m_mol) {
    xs.insert(xs.end(), {a.m_x, a.m_y, a.m_z});
    q.push_back((double)a.charge);
  }
  throw_on_status(cppe_gpu_charge_field_gradient(n, xt.data(), na, xs.data(), q.data(),
                                                 gpu_config().device, G.data.data()));
  return G;
}

// --- MultipoleFields (electric_fields.cc:106-189) -------------------------------
Vector MultipoleFields::compute() {
  const int n = (int)m_potentials.size();
  std::vector<double> xyz, q(n, 0.0), mu(3 * (size_t)n, 0.0), quad(6 * (size_t)n, 0.0),
        aiso(n, 0.0);
  std::vector<int> pol(n, 0);
  int max_order = 0;
  for (int i = 0; i < n; ++i) {
    const Potential& p = m_potentials[i];
    xyz.insert(xyz.end(), {p.m_x, p.m_y, p.m_z});
    const int mo = p.max_multipole_order();
    max_order    = std::max(max_order, mo);
    if (mo > 2)
      throw std::runtime_error("MultipoleFields::compute_tree only supported up to 2nd order.");
    if (p.is_polarizable()) {
      pol[i]  = 1;
      aiso[i] = p.get_polarizability().get_isotropic_value();
    }
    const auto& ms = p.get_multipoles();
    if (ms.empty()) continue;
    // the reference reads orders 0, 1, 2 from the first three multipoles
    q[i] = ms[0].get_values_vec().at(0);
    if (mo > 0) {
      auto v = ms.at(1).get_values_vec();
      for (int c = 0; c < 3; ++c) mu[3 * i + c] = v.at(c);
    }
    if (mo > 1) {
      auto v = ms.at(2).get_values_vec();
      for (int c = 0; c < 6; ++c) quad[6 * i + c] = v.at(c);
    }
  }
  Vector F(3 * (size_t)n, 0.0);
  if (n == 0) return F;
  std::vector<int> eptr, eidx;
  pack_exclusions(m_potentials, eptr, eidx);
  const int summation =
        m_options.summation_induced_fields == "fmm" ? CPPE_GPU_FMM : CPPE_GPU_DIRECT;
  throw_on_status(cppe_gpu_multipole_fields(
        n, xyz.data(), q.data(), mu.data(), quad.data(), max_order, pol.data(), aiso.data(),
        eptr.data(), eidx.empty() ? nullptr : eidx.data(), summation, m_options.tree_ncrit,
        m_options.tree_expansion_order, m_options.theta, m_options.damp_multipole ? 1 : 0,
        m_options.damping_factor_multipole, gpu_config().device, F.data()));
  return F;
}

// --- InducedMoments (electric_fields.cc:191-239) --------------------------------
InducedMoments::InducedMoments(std::vector<Potential> potentials, const PeOptions& options)
      : m_potentials(std::move(potentials)), m_options(options) {
  m_polsites   = get_polarizable_sites(m_potentials);
  m_n_polsites = m_polsites.size();
  m_gpu        = std::make_shared<GpuSystem>(m_polsites, m_options);
}

Vector InducedMoments::compute(const Vector& rhs, Vector guess, bool make_guess) {
  check_size(rhs, 3 * m_n_polsites, "InducedMoments.compute");
  if (!make_guess) check_size(guess, 3 * m_n_polsites, "InducedMoments.compute guess");
  Vector mu(rhs.size(), 0.0);
  const int cap = std::max(1, m_options.maxiter) + 64;
  std::vector<double> hist(cap, 0.0);
  int iters = 0;
  int st    = cppe_gpu_solve(m_gpu->get(), rhs.data(), make_guess ? nullptr : guess.data(),
                             make_guess ? 1 : 0, mu.data(), &iters, hist.data(), cap);
  double rn = 0.0;
  cppe_gpu_last_solve_stats(m_gpu->get(), &rn, &last_fp64_applies, &last_fp32_applies);
  last_iterations = iters;
  last_rnorm      = rn;
  // The reference prints "k --- Norm: ||r||" once per iteration (:222-225);
  // the device loop records the norms and they are printed here in order.  In
  // mixed precision the norms are those of the FP64 refinement residuals.
  for (int k = 0; k < std::min(iters, cap); ++k) {
    std::stringstream ss;
    ss.precision(12);
    ss << std::fixed << hist[k];
    m_printer(std::to_string(k) + " --- Norm: " + ss.str());
  }
  if (st == CPPE_GPU_NOT_CONVERGED)
    throw std::runtime_error("Failed to converge induced dipole moments.");
  throw_on_status(st);
  return mu;
}

// --- MultipoleExpansion (multipole_expansion.cc:10-62) --------------------------
namespace {
struct PackedSites {
  std::vector<double> xyz, q, mu, quad, ax, az;
  int max_order = 0;
};
PackedSites pack_multipoles(const std::vector<Potential>& pots, const Molecule& mol) {
  PackedSites p;
  const size_t n = pots.size();
  p.q.assign(n, 0.0), p.mu.assign(3 * n, 0.0), p.quad.assign(6 * n, 0.0);
  for (size_t i = 0; i < n; ++i) {
    const Potential& s = pots[i];
    p.xyz.insert(p.xyz.end(), {s.m_x, s.m_y, s.m_z});
    for (const auto& m : s.get_multipoles()) {
      auto v = m.get_values_vec();
      if (m.m_k == 0)
        p.q[i] += v.at(0);
      else if (m.m_k == 1)
        for (int c = 0; c < 3; ++c) p.mu[3 * i + c] += v.at(c);
      else if (m.m_k == 2)
        for (int c = 0; c < 6; ++c) p.quad[6 * i + c] += v.at(c);
      else
        throw std::runtime_error("multipoles above order 2 are not supported");
      p.max_order = std::max<int>(p.max_order, m.m_k);
    }
  }
  for (const auto& a : mol) {
    p.ax.insert(p.ax.end(), {a.m_x, a.m_y, a.m_z});
    p.az.push_back((double)a.charge);
  }
  return p;
}
}  // namespace

double MultipoleExpansion::interaction_energy() {
  const int n = (int)m_potentials.size();
  if (n == 0 || m_mol.empty()) return 0.0;
  const PackedSites p = pack_multipoles(m_potentials, m_mol);
  double e = 0.0;
  throw_on_status(cppe_gpu_multipole_potential_energy(
        n, p.xyz.data(), p.q.data(), p.mu.data(), p.quad.data(), p.max_order,
        (int)m_mol.size(), p.ax.data(), p.az.data(), gpu_config().device, &e));
  return e;
}

Matrix MultipoleExpansion::nuclear_gradient() {
  const int n = (int)m_potentials.size(), na = (int)m_mol.size();
  Matrix G(na, 3);
  if (n == 0 || na == 0) return G;
  const PackedSites p = pack_multipoles(m_potentials, m_mol);
  throw_on_status(cppe_gpu_multipole_energy_gradient(
        n, p.xyz.data(), p.q.data(), p.mu.data(), p.quad.data(), p.max_order, na,
        p.ax.data(), p.az.data(), gpu_config().device, G.data.data()));
  return G;
}

// --- DipoleTree (fmm/tree.cc:350-394, Tree<1,3>) -------------------------------
DipoleTree::DipoleTree(std::vector<double> xyz, int ncrit, int order, double theta,
                       double damping, std::vector<double> alpha_iso,
                       std::vector<std::vector<int>> exclusions)
      : m_xyz(std::move(xyz)), m_ncrit(ncrit), m_order(order), m_theta(theta),
        m_damping(damping) {
  if (m_xyz.size() % 3 != 0) throw std::invalid_argument("positions must be n x 3");
  const size_t n = m_xyz.size() / 3;
  m_aiso         = alpha_iso.empty() ? std::vector<double>(n, 0.0) : std::move(alpha_iso);
  if (m_aiso.size() != n) throw std::invalid_argument("one polarizability per site");
  if (m_damping > 0.0)
    for (double a : m_aiso)
      if (!(a > 0.0))
        throw std::invalid_argument("Thole damping needs a positive polarizability per site");
  if (!exclusions.empty() && exclusions.size() != n)
    throw std::invalid_argument("one exclusion list per site");
  m_eptr.assign(1, 0);
  for (size_t i = 0; i < n; ++i) {
    if (!exclusions.empty())
      for (int e : exclusions[i]) m_eidx.push_back(e);
    m_eptr.push_back((int)m_eidx.size());
  }
}

void DipoleTree::compute_field(const double* S, double* F, bool fmm) const {
  const int n = size();
  if (n == 0) return;
  // MultipoleFields' dipole term is -F_tree(mu) (electric_fields.cc:164-176):
  // the static-field entry point with only dipoles gives -F_tree.
  std::vector<double> q(n, 0.0), quad(6 * (size_t)n, 0.0), out(3 * (size_t)n, 0.0);
  std::vector<int> pol(n, 1);
  throw_on_status(cppe_gpu_multipole_fields(
        n, m_xyz.data(), q.data(), S, quad.data(), 1, pol.data(), m_aiso.data(),
        m_eptr.data(), m_eidx.empty() ? nullptr : m_eidx.data(),
        fmm ? CPPE_GPU_FMM : CPPE_GPU_DIRECT, m_ncrit, m_order, m_theta,
        m_damping > 0.0 ? 1 : 0, m_damping, gpu_config().device, out.data()));
  for (size_t i = 0; i < out.size(); ++i) F[i] = -out[i];
}

}  // namespace libcppe
