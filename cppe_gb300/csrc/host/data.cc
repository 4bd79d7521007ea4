// Data model, potfile reading, potential manipulation and math helpers of the
// host layer (host-side setup code; no field arithmetic).
#include <algorithm>
#include <string_view>
#include <cctype>
#include <charconv>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <set>
#include <sstream>

#include "cppe_host.hh"
#include "cppe_gpu.h"

namespace libcppe {

const std::vector<std::string> valid_option_keys{
      "potfile",          "iso_pol",
      "induced_thresh",   "maxiter",
      "damp_induced",     "damping_factor_induced",
      "damp_multipole",   "damping_factor_multipole",
      "summation_induced_fields", "tree_expansion_order",
      "tree_ncrit",       "theta",
      "pe_border",        "border_type",
      "border_rmin",      "border_nredist",
      "border_redist_order", "border_redist_pol"};

GpuConfig& gpu_config() {
  static GpuConfig c = [] {
    GpuConfig g;
    if (const char* p = std::getenv("CPPE_GPU_PRECISION")) {
      std::string v(p);
      if (v == "mixed") g.precision = 1;
    }
    if (const char* d = std::getenv("CPPE_GPU_DEVICE")) g.device = std::atoi(d);
    return g;
  }();
  return c;
}

const PrintCallback default_printer = [](std::string s) {
  std::cout << std::setprecision(12) << s << std::endl;
};

void throw_on_status(int status) {
  if (status == CPPE_GPU_OK) return;
  if (status == CPPE_GPU_NOT_CONVERGED)
    throw std::runtime_error("Failed to converge induced dipole moments.");
  char buf[1024];
  cppe_gpu_last_error(buf, sizeof buf);
  if (status == CPPE_GPU_INVALID_ARG) throw std::invalid_argument(buf);
  throw std::runtime_error(std::string("cppe_gb300 GPU error: ") + buf);
}

// --- Multipole / Polarizability / Potential (potential.hh:11-127) -----------
void Multipole::remove_trace() {
  if (m_k == 2) {
    if (m_values.size() < 6) throw std::runtime_error("quadrupole needs 6 values");
    const double tr = (m_values[0] + m_values[3] + m_values[5]) / 3.0;
    m_values[0] -= tr, m_values[3] -= tr, m_values[5] -= tr;
  } else if (m_k > 2) {
    throw std::runtime_error("remove_trace() not implemented for multipoles of order > 2");
  }
}

Polarizability::Polarizability(const std::vector<double>& v) {
  if (v.size() != 6)
    throw std::runtime_error(
          "Invalid number of elements to construct polarizability. Vector must have "
          "exactly 6 elements.");
  m_values = triangle_to_mat(v);
}

void Polarizability::make_isotropic() {
  const double iso = get_isotropic_value();
  m_values.fill(0.0);
  m_values[0] = m_values[4] = m_values[8] = iso;
}

Vector Polarizability::get_values_vec() const { return mat_to_triangle(m_values); }

bool Potential::excludes_site(int other) const {
  return std::find(m_exclusions.begin(), m_exclusions.end(), other) != m_exclusions.end();
}

int Potential::max_multipole_order() const {
  int k = 0;
  for (const auto& m : m_multipoles) k = std::max<int>(k, m.m_k);
  return k;
}

std::vector<Potential> get_polarizable_sites(const std::vector<Potential>& potentials) {
  std::vector<Potential> out;
  for (const auto& p : potentials)
    if (p.is_polarizable()) out.push_back(p);
  return out;
}

// --- PotfileReader (potfile_reader.cc:22-179) -------------------------------
// The file is read into memory once and scanned line by line; tokens are
// string views and numbers are parsed with std::from_chars (locale-free), so
// a million-site file is read without per-token allocations.
namespace {
const double kAngToBohr = 1.8897261246;

struct Scanner {
  std::string buf;
  size_t pos = 0;
  bool next(std::string_view& line) {
    if (pos >= buf.size()) return false;
    size_t e = buf.find('\n', pos);
    if (e == std::string::npos) e = buf.size();
    line = std::string_view(buf).substr(pos, e - pos);
    if (!line.empty() && line.back() == '\r') line.remove_suffix(1);
    pos = e + 1;
    return true;
  }
};

// whitespace-separated tokens of a line (views into it)
void tokens(std::string_view line, std::vector<std::string_view>& t) {
  t.clear();
  size_t i = 0;
  const size_t n = line.size();
  while (i < n) {
    while (i < n && std::isspace((unsigned char)line[i])) ++i;
    size_t j = i;
    while (j < n && !std::isspace((unsigned char)line[j])) ++j;
    if (j > i) t.push_back(line.substr(i, j - i));
    i = j;
  }
}
std::string trimmed(std::string_view s) {
  std::vector<std::string_view> t;
  tokens(s, t);
  std::string out;
  for (size_t i = 0; i < t.size(); ++i) out += (i ? " " : "") + std::string(t[i]);
  return out;
}
double num(std::string_view t) {
  if (!t.empty() && t[0] == '+') t.remove_prefix(1);
  double v      = 0.0;
  const auto rc = std::from_chars(t.data(), t.data() + t.size(), v);
  if (rc.ec != std::errc() || rc.ptr != t.data() + t.size())
    throw std::invalid_argument("invalid number in potential file: " + std::string(t));
  return v;
}
int inum(std::string_view t) {
  if (!t.empty() && t[0] == '+') t.remove_prefix(1);
  int v         = 0;
  const auto rc = std::from_chars(t.data(), t.data() + t.size(), v);
  if (rc.ec != std::errc()) throw std::invalid_argument("invalid integer in potential file");
  return v;
}
}  // namespace

PotfileReader::PotfileReader(std::string name) : m_potfile(std::move(name)) {
  std::ifstream f(m_potfile);
  if (!f.good()) throw std::runtime_error("Potential file does not exist.");
}

std::vector<Potential> PotfileReader::read() {
  Scanner sc;
  {
    std::ifstream in(m_potfile, std::ios::binary);
    std::ostringstream ss;
    ss << in.rdbuf();
    sc.buf = ss.str();
  }
  std::vector<Potential> pots;
  std::string_view line;
  std::vector<std::string_view> t;
  int num_sites = 0;
  auto next     = [&]() {
    if (!sc.next(line)) throw std::runtime_error("unexpected end of potential file");
    return line;
  };
  while (sc.next(line)) {
    if (line.find("@COORDINATES") != std::string_view::npos) {
      tokens(next(), t);
      num_sites        = inum(t.at(0));
      std::string unit = trimmed(next());
      double conv;
      if (unit == "AA")
        conv = kAngToBohr;
      else if (unit == "AU")
        conv = 1.0;
      else
        throw std::runtime_error("Invalid unit for potential file.");
      pots.reserve(num_sites);
      for (int i = 0; i < num_sites; ++i) {
        tokens(next(), t);
        if (t.size() < 4) throw std::runtime_error("malformed coordinate line");
        pots.emplace_back(num(t[1]) * conv, num(t[2]) * conv, num(t[3]) * conv,
                          std::string(t[0]), i);
      }
    }
    if (line.find("ORDER") != std::string_view::npos) {
      std::vector<std::string_view> h;
      tokens(line, h);
      if (h.size() == 2) {
        const int order = inum(h[1]);
        const int ncomp = multipole_components(order);
        tokens(next(), t);
        const int count = inum(t.at(0));
        int before      = -1;
        auto zero_mul   = [&](int site) {
          Multipole m(order);
          for (int v = 0; v < ncomp; ++v) m.add_value(0.0);
          pots.at(site).add_multipole(std::move(m));
        };
        for (int k = 0; k < count; ++k) {
          tokens(next(), t);
          int site = inum(t.at(0)) - 1;
          for (int d = before + 1; d < site; ++d) zero_mul(d);  // sites without values
          Multipole m(order);
          for (int v = 1; v <= ncomp; ++v) m.add_value(num(t.at(v)));
          m.remove_trace();
          pots.at(site).add_multipole(std::move(m));
          before = site;
          if (k == count - 1)
            for (int d = site + 1; d < num_sites; ++d) zero_mul(d);
        }
      } else if (h.size() == 3) {
        if (inum(h[1]) != 1 || inum(h[2]) != 1)
          throw std::runtime_error(
                "Only dipole-dipole polarizabilities are currently supported.");
        tokens(next(), t);
        const int count = inum(t.at(0));
        for (int k = 0; k < count; ++k) {
          tokens(next(), t);
          int site = inum(t.at(0)) - 1;
          std::vector<double> v(6);
          for (int c = 1; c <= 6; ++c) v[c - 1] = num(t.at(c));
          Polarizability p(v);
          if (pots.at(site).is_polarizable())
            throw std::runtime_error("Potential can only have one polarizability.");
          pots.at(site).set_polarizability(p);
        }
      } else {
        throw std::runtime_error("Invalid number in potfile ORDER.");
      }
    }
    if (line.find("EXCLISTS") != std::string_view::npos) {
      tokens(next(), t);
      const int count = inum(t.at(0));
      for (int k = 0; k < count; ++k) {
        tokens(next(), t);
        int site = inum(t.at(0)) - 1;
        for (size_t c = 1; c < t.size(); ++c) {
          int e = inum(t[c]) - 1;
          if (e >= 0) pots.at(site).add_exclusion(e);
        }
      }
    }
  }
  return pots;
}

// --- PotManipulator (pot_manipulation.cc:15-138) ----------------------------
std::vector<Potential> PotManipulator::manipulate(const PeOptions& o) {
  if (o.iso_pol)
    for (auto& p : m_potentials) p.get_polarizability().make_isotropic();
  return manipulate_border(o);
}

std::vector<Potential> PotManipulator::manipulate_border(const PeOptions& o) {
  if (!o.pe_border) return m_potentials;
  std::set<int> changed;
  for (const Atom& a : m_mol)
    for (const Potential& p : m_potentials) {
      const double dx = a.m_x - p.m_x, dy = a.m_y - p.m_y, dz = a.m_z - p.m_z;
      if (std::sqrt(dx * dx + dy * dy + dz * dz) <= o.border_rmin) changed.insert(p.index);
    }
  if (changed.empty()) return m_potentials;
  std::vector<Potential> out;
  if (o.border_type == "remove") {
    for (const Potential& p : m_potentials) {
      if (!changed.count(p.index))
        out.push_back(p);
      else
        m_printer("     Removing all parameters on site: " + std::to_string(p.index));
    }
  } else if (o.border_type == "redist") {
    m_printer("     Redistributing moments in " + std::to_string(o.border_rmin) +
              " a.u. proximity.");
    int nredist = o.border_nredist;
    if (nredist == -1) {
      m_printer("     Border sites will be redistributed to all other sites.");
      nredist = (int)(m_potentials.size() - changed.size());
    }
    if (nredist > (int)m_potentials.size())
      throw std::runtime_error("Cannot redistribute to more sites than available sites.");
    for (int site : changed) {
      std::vector<std::pair<int, double>> nb;
      m_printer("     Redistributing site: " + std::to_string(site));
      for (const Potential& p : m_potentials) {
        if (changed.count(p.index)) continue;
        const Potential& s = m_potentials[site];
        const double dx = s.m_x - p.m_x, dy = s.m_y - p.m_y, dz = s.m_z - p.m_z;
        nb.emplace_back(p.index, std::sqrt(dx * dx + dy * dy + dz * dz));
      }
      std::sort(nb.begin(), nb.end(),
                [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
                  return a.second < b.second;
                });
      for (int k = 0; k < nredist; ++k) {
        Potential& p = m_potentials[nb[k].first];
        if (p.index == site) continue;
        m_printer("       to neighbor " + std::to_string(p.index));
        int mi = 0;
        for (Multipole& m : p.get_multipoles()) {
          const auto& sm = m_potentials[site].get_multipoles();
          if ((int)m.m_k < o.border_redist_order && mi < (int)sm.size() && m.m_k == sm[mi].m_k)
            for (int c = 0; c < multipole_components(m.m_k); ++c)
              m.get_values()[c] += sm[mi].get_values_vec()[c] / (double)nredist;
          ++mi;
        }
        if (o.border_redist_pol && p.is_polarizable() && m_potentials[site].is_polarizable()) {
          auto& pm       = p.get_polarizability().get_matrix();
          const auto& sp = m_potentials[site].get_polarizability().get_matrix();
          for (int c = 0; c < 9; ++c) pm[c] += sp[c] / (double)nredist;
        }
      }
    }
    double total_charge = 0.0;
    for (const Potential& p : m_potentials) {
      if (!changed.count(p.index)) {
        out.push_back(p);
        for (const auto& m : p.get_multipoles()) {
          if (m.m_k == 0)
            total_charge += m.get_values_vec()[0];
          else
            break;
        }
      } else {
        m_printer("     Removing all parameters on site: " + std::to_string(p.index));
      }
    }
    m_printer("    Total charge of the classical region: " + std::to_string(total_charge));
  }
  if (out.size() > m_potentials.size())
    throw std::runtime_error(
          "Manipulated potentials cannot have more sites than original ones.");
  return out;
}

// --- math helpers (math.cc:7-99) --------------------------------------------
double factorial(int n) {
  double x = 1.0;
  for (int i = 2; i <= n; ++i) x *= i;
  return x;
}

void make_df(unsigned k, std::vector<double>& df) {
  double f = -1.0;
  for (unsigned i = 1; i <= k; ++i) f *= double(i) / double(2 * i - 1);
  df.resize((k + 1) * (k + 2) / 2);
  for (unsigned ix = 0, j = 0; ix <= k; ++ix)
    for (unsigned iy = 0; iy <= ix; ++iy, ++j) {
      unsigned kx = k - ix, ky = ix - iy, kz = k - kx - ky;
      df[j]       = f / (factorial(kx) * factorial(ky) * factorial(kz));
    }
}

int trinom(int i, int j, int k) {
  return (int)(factorial(i + j + k) / (factorial(i) * factorial(j) * factorial(k)));
}

std::vector<double> symmetry_factors(unsigned k) {
  std::vector<double> pf;
  for (int x = k; x >= 0; --x)
    for (int y = k - x; y >= 0; --y) pf.push_back((double)trinom(x, y, k - x - y));
  return pf;
}

std::vector<double> prefactors(unsigned k) {
  auto pf = symmetry_factors(k);
  for (double& v : pf) v *= -1.0 / factorial(k);
  return pf;
}

std::vector<double> prefactors_nuclei(unsigned k) {
  auto pf         = symmetry_factors(k);
  const double tf = (k % 2 == 0 ? 1.0 : -1.0) / factorial(k);
  for (double& v : pf) v *= tf;
  return pf;
}

int multipole_components(int k) { return (k + 1) * (k + 2) / 2; }

std::array<double, 9> triangle_to_mat(const std::vector<double>& y) {
  return {y[0], y[1], y[2], y[1], y[3], y[4], y[2], y[4], y[5]};
}

std::vector<double> mat_to_triangle(const std::array<double, 9>& m) {
  return {m[0], m[1], m[2], m[4], m[5], m[8]};
}

}  // namespace libcppe
