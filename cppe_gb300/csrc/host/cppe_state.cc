// CppeState (src/core/cppe_state.{hh,cc}): the SCF-facing state object.
// One InducedMoments (and so one GPU system with its tree and buffers) is
// kept across update_induced_moments calls; the reference rebuilt it, and its
// tree, on every call and every apply.
#include <iomanip>
#include <map>
#include <numeric>
#include <sstream>

#include "cppe_gpu.h"
#include "cppe_host.hh"

namespace libcppe {

CppeState::CppeState(const PeOptions& options, Molecule mol, PrintCallback printer)
      : m_mol(std::move(mol)), m_options(options), m_printer(std::move(printer)) {
  m_pe_energy     = PeEnergy{};
  auto potentials = PotfileReader(m_options.potfile).read();
  PotManipulator manip(potentials, m_mol);
  manip.set_print_callback(m_printer);
  potentials = manip.manipulate(m_options);
  set_potentials(std::move(potentials));
  const std::map<std::string, std::vector<std::string>> terms{
        {"Electrostatic", {"Electronic", "Nuclear", "Multipoles"}},
        {"Polarization", {"Electronic", "Nuclear", "Multipoles"}}};
  for (const auto& it : terms)
    for (const auto& nm : it.second) m_pe_energy[it.first][nm] = 0.0;
}

void CppeState::set_potentials(std::vector<Potential> potentials) {
  m_potentials        = std::move(potentials);
  m_polarizable_sites = 0;
  for (const auto& p : m_potentials) m_polarizable_sites += p.is_polarizable() ? 1 : 0;
  m_induced_moments.assign(3 * m_polarizable_sites, 0.0);
  m_positions             = Matrix(m_potentials.size(), 3);
  m_positions_polarizable = Matrix(m_polarizable_sites, 3);
  size_t k                = 0;
  for (size_t i = 0; i < m_potentials.size(); ++i) {
    const auto& p       = m_potentials[i];
    m_positions(i, 0)   = p.m_x;
    m_positions(i, 1)   = p.m_y;
    m_positions(i, 2)   = p.m_z;
    if (p.is_polarizable()) {
      m_positions_polarizable(k, 0) = p.m_x;
      m_positions_polarizable(k, 1) = p.m_y;
      m_positions_polarizable(k, 2) = p.m_z;
      ++k;
    }
  }
  m_solver.reset();
  m_eef.reset();
}

void CppeState::calculate_static_energies_and_fields() {
  MultipoleExpansion mexp(m_mol, m_potentials);
  m_pe_energy["Electrostatic"]["Nuclear"] = mexp.interaction_energy();
  NuclearFields nf(m_mol, m_potentials);
  m_nuc_fields = nf.compute();
  MultipoleFields mf(m_potentials, m_options);
  m_multipole_fields = mf.compute();
}

Vector CppeState::get_static_fields() const {
  if (m_nuc_fields.size() != m_multipole_fields.size())
    throw std::runtime_error(
          "static fields: nuclear fields (polarizable sites) and multipole fields (all "
          "sites) differ in length");
  Vector s(m_nuc_fields.size());
  for (size_t i = 0; i < s.size(); ++i) s[i] = m_nuc_fields[i] + m_multipole_fields[i];
  return s;
}

void CppeState::update_induced_moments(const Vector& elec_fields, bool elec_only) {
  Vector total;
  if (elec_only) {
    total = elec_fields;
  } else {
    total = elec_fields;
    if (m_nuc_fields.size() != total.size() || m_multipole_fields.size() != total.size())
      throw std::invalid_argument(
            "update_induced_moments: call calculate_static_energies_and_fields first "
            "(field lengths differ)");
    for (size_t i = 0; i < total.size(); ++i) total[i] += m_nuc_fields[i] + m_multipole_fields[i];
  }
  if (!m_solver) m_solver = std::make_shared<InducedMoments>(m_potentials, m_options);
  m_solver->set_print_callback(m_printer);
  m_induced_moments = m_solver->compute(total, m_induced_moments, m_make_guess);
  if (m_make_guess) m_make_guess = false;
  auto dot = [&](const Vector& a) {
    double s = 0.0;
    for (size_t i = 0; i < a.size(); ++i) s += m_induced_moments[i] * a[i];
    return s;
  };
  m_pe_energy["Polarization"]["Electronic"] = -0.5 * dot(elec_fields);
  if (!elec_only) {
    m_pe_energy["Polarization"]["Nuclear"]    = -0.5 * dot(m_nuc_fields);
    m_pe_energy["Polarization"]["Multipoles"] = -0.5 * dot(m_multipole_fields);
  }
}

namespace {
// The three unit-field solves of induced_moments_eef as one batch (one system,
// three right-hand sides): one set of launches per iteration for all three,
// with the near-field pair tensors shared between them.
struct EefBatch {
  cppe_gpu_batch* b = nullptr;
  int n             = 0;
  ~EefBatch() {
    if (b) cppe_gpu_batch_destroy(b);
  }
};
}  // namespace

// CppeState::induced_moments_eef (cppe_state.cc:111-128): induced moments for
// unit external fields along x, y and z at every polarizable site, each from
// the first-call guess alpha F to the same threshold.  The reference solves
// them one after another with a new InducedMoments; here they are one batched
// solve on a handle kept across calls.  The printer receives one line per
// field direction with its iteration count (the batch records no per-iteration
// norms).
Matrix CppeState::induced_moments_eef() {
  const size_t n3 = 3 * m_polarizable_sites;
  Matrix ret(n3, 3);
  if (m_polarizable_sites == 0) return ret;
  if (!m_eef) {
    auto polsites = get_polarizable_sites(m_potentials);
    std::vector<double> xyz, a6;
    for (const auto& p : polsites) {
      xyz.insert(xyz.end(), {p.m_x, p.m_y, p.m_z});
      auto a = p.get_polarizability().get_values_vec();
      a6.insert(a6.end(), a.begin(), a.end());
    }
    std::vector<int> eptr, eidx;
    pack_exclusions(polsites, eptr, eidx);
    const int n               = (int)polsites.size();
    const int off[2]          = {0, n};
    cppe_gpu_options g        = to_gpu(m_options);
    const int direct_below    = g.summation == CPPE_GPU_FMM ? 0 : n + 1;
    auto eb                   = std::make_shared<EefBatch>();
    eb->n                     = n;
    throw_on_status(cppe_gpu_batch_create(1, off, xyz.data(), a6.data(), eptr.data(),
                                          eidx.empty() ? nullptr : eidx.data(), 3,
                                          direct_below, &g, &eb->b));
    m_eef = eb;
  }
  auto* eb = static_cast<EefBatch*>(m_eef.get());
  Vector f(3 * n3, 0.0), mu(3 * n3, 0.0);
  for (int a = 0; a < 3; ++a)
    for (size_t s = 0; s < m_polarizable_sites; ++s) f[a * n3 + 3 * s + a] = 1.0;
  int iters[3] = {0, 0, 0};
  const int st = cppe_gpu_batch_solve(eb->b, f.data(), mu.data(), iters);
  for (int a = 0; a < 3; ++a)
    m_printer("eef " + std::string(1, "xyz"[a]) + ": " + std::to_string(iters[a]) +
              " iterations");
  if (st == CPPE_GPU_NOT_CONVERGED)
    throw std::runtime_error("Failed to converge induced dipole moments.");
  throw_on_status(st);
  for (int a = 0; a < 3; ++a)
    for (size_t i = 0; i < n3; ++i) ret(i, a) = mu[a * n3 + i];
  return ret;
}

// CppeState::nuclear_interaction_energy_gradient / nuclear_field_gradient
// (cppe_state.cc:73-81)
Matrix CppeState::nuclear_interaction_energy_gradient() {
  return MultipoleExpansion(m_mol, m_potentials).nuclear_gradient();
}

Matrix CppeState::nuclear_field_gradient() {
  return NuclearFields(m_mol, m_potentials).nuclear_gradient();
}

double CppeState::get_total_energy_for_category(const std::string& c) {
  double s = 0.0;
  for (const auto& kv : m_pe_energy[c]) s += kv.second;
  return s;
}

double CppeState::get_total_energy() {
  return get_total_energy_for_category("Electrostatic") +
         get_total_energy_for_category("Polarization");
}

std::string CppeState::get_energy_summary_string() {
  const size_t w = 30;
  const std::string off(3, ' '), off2(6, ' ');
  std::stringstream ss;
  ss << std::string(2 * w + 10, '-') << std::endl;
  ss << "Polarizable Embedding Summary:";
  ss << std::setprecision(12) << std::endl << std::endl;
  auto block = [&](const char* title, const char* cat) {
    ss << off << title << std::endl;
    ss << off2 << "Electronic:" << std::string(w - 11, ' ') << m_pe_energy[cat]["Electronic"]
       << std::endl;
    ss << off2 << "Nuclear:" << std::string(w - 8, ' ') << m_pe_energy[cat]["Nuclear"]
       << std::endl;
    ss << off2 << "Multipole:" << std::string(w - 10, ' ') << m_pe_energy[cat]["Multipoles"]
       << std::endl;
    ss << off2 << "Total:" << std::string(w - 6, ' ') << get_total_energy_for_category(cat)
       << std::endl;
    ss << std::endl;
  };
  block("Electrostatics:", "Electrostatic");
  block("Polarization:", "Polarization");
  ss << off << "Total Energy:" << std::string(w - 10, ' ')
     << get_total_energy_for_category("Electrostatic") +
              get_total_energy_for_category("Polarization")
     << std::endl;
  ss << std::string(2 * w + 10, '-') << std::endl << std::endl;
  return ss.str();
}

}  // namespace libcppe
