// C++ host layer: the reference's libcppe class interface (names, arguments,
// defaults, exceptions) on top of the C ABI of libcppe_gpu.  Every numeric
// call of the induced-dipole path goes to the GPU; nothing here computes
// fields, applies the operator or iterates the solver on the CPU.
//
// Counterparts (maxscheurer/cppe):
//   PeOptions, valid_option_keys   src/core/pe_options.hh:8-69
//   Multipole, Polarizability,
//   Potential                      src/core/potential.hh:11-127
//   Atom, Molecule                 src/core/molecule.hh:9-21
//   PotfileReader                  src/core/potfile_reader.{hh,cc}
//   PotManipulator                 src/core/pot_manipulation.{hh,cc}
//   BMatrix                        src/core/bmatrix.{hh,cc}
//   MultipoleFields, NuclearFields,
//   InducedMoments                 src/core/electric_fields.{hh,cc}
//   MultipoleExpansion             src/core/multipole_expansion.{hh,cc}
//   CppeState                      src/core/cppe_state.{hh,cc}
//   math helpers                   src/core/math.{hh,cc}
//
// The reference's Eigen vectors become std::vector<double> (site-major xyz)
// and its Eigen matrices a row-major Matrix; the Python module converts both
// to numpy arrays exactly where the reference's pybind11 layer did.
#pragma once

#include <array>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "cppe_gpu.h"

struct cppe_gpu_system;

namespace libcppe {

using Vector = std::vector<double>;

struct Matrix {
  size_t rows = 0, cols = 0;
  std::vector<double> data;  // row-major
  Matrix() = default;
  Matrix(size_t r, size_t c) : rows(r), cols(c), data(r * c, 0.0) {}
  double& operator()(size_t r, size_t c) { return data[r * cols + c]; }
  double operator()(size_t r, size_t c) const { return data[r * cols + c]; }
};

struct PeOptions {
  std::string potfile{"potential.pot"};
  bool iso_pol                    = false;
  double induced_thresh           = 1e-8;
  int maxiter                     = 50;
  bool damp_induced               = false;
  double damping_factor_induced   = 2.1304;
  bool damp_multipole             = false;
  double damping_factor_multipole = 2.1304;
  std::string summation_induced_fields{"direct"};
  int tree_ncrit           = 64;
  int tree_expansion_order = 5;
  double theta             = 0.5;
  bool pe_border           = false;
  std::string border_type{"remove"};
  double border_rmin       = 2.2;
  int border_nredist       = -1;
  int border_redist_order  = 1;
  bool border_redist_pol   = false;
};

extern const std::vector<std::string> valid_option_keys;

// GPU settings that have no PeOptions key (the reference's option set is
// kept exactly as it is).
struct GpuConfig {
  int precision = 0;  // 0 = FP64, 1 = mixed (FP32 inner solves + FP64 refinement)
  int device    = 0;
};
GpuConfig& gpu_config();

class Multipole {
 private:
  std::vector<double> m_values;

 public:
  explicit Multipole(unsigned k) : m_k(k) {}
  void add_value(double v) { m_values.push_back(v); }
  void remove_trace();
  std::vector<double>& get_values() { return m_values; }
  Vector get_values_vec() const { return m_values; }
  unsigned m_k;
};

class Polarizability {
 private:
  std::array<double, 9> m_values{};

 public:
  Polarizability() = default;
  explicit Polarizability(const std::vector<double>& values);
  void make_isotropic();
  double get_isotropic_value() const { return (m_values[0] + m_values[4] + m_values[8]) / 3.0; }
  Vector get_values_vec() const;  // xx, xy, xz, yy, yz, zz
  std::array<double, 9>& get_matrix() { return m_values; }
  const std::array<double, 9>& get_matrix() const { return m_values; }
};

class Potential {
 private:
  std::vector<Multipole> m_multipoles;
  Polarizability m_polarizability;
  bool m_is_polarizable = false;
  std::vector<int> m_exclusions;

 public:
  Potential(double x, double y, double z, std::string element, int idx)
        : m_x(x), m_y(y), m_z(z), m_element(std::move(element)), index(idx) {}
  double m_x, m_y, m_z;
  std::string m_element;
  int index;

  void add_multipole(const Multipole& m) { m_multipoles.push_back(m); }
  void add_multipole(Multipole&& m) { m_multipoles.push_back(std::move(m)); }
  void add_exclusion(int e) { m_exclusions.push_back(e); }
  bool excludes_site(int other) const;
  std::vector<int>& get_exclusions() { return m_exclusions; }
  const std::vector<int>& get_exclusions() const { return m_exclusions; }
  std::vector<Multipole>& get_multipoles() { return m_multipoles; }
  const std::vector<Multipole>& get_multipoles() const { return m_multipoles; }
  void set_polarizability(const Polarizability& p) {
    m_polarizability = p;
    m_is_polarizable = true;
  }
  int max_multipole_order() const;
  Polarizability& get_polarizability() { return m_polarizability; }
  const Polarizability& get_polarizability() const { return m_polarizability; }
  bool is_polarizable() const { return m_is_polarizable; }
  std::array<double, 3> get_site_position() const { return {m_x, m_y, m_z}; }
};

struct Atom {
  int atomic_number;
  int charge;
  double m_x = 0, m_y = 0, m_z = 0;
  explicit Atom(int an) : atomic_number(an), charge(an) {}
  Atom(int an, double x, double y, double z)
        : atomic_number(an), charge(an), m_x(x), m_y(y), m_z(z) {}
  std::array<double, 3> get_position() const { return {m_x, m_y, m_z}; }
};
using Molecule = std::vector<Atom>;

using PrintCallback = std::function<void(std::string)>;
extern const PrintCallback default_printer;

class PotfileReader {
  std::string m_potfile;

 public:
  explicit PotfileReader(std::string potfile_name);
  std::vector<Potential> read();
};

class PotManipulator {
  std::vector<Potential> m_potentials;
  Molecule m_mol;
  PrintCallback m_printer = [](std::string) {};

 public:
  PotManipulator(std::vector<Potential> potentials, Molecule mol)
        : m_potentials(std::move(potentials)), m_mol(std::move(mol)) {}
  void set_print_callback(PrintCallback p) { m_printer = std::move(p); }
  std::vector<Potential> manipulate(const PeOptions& o);
  std::vector<Potential> manipulate_border(const PeOptions& o);
};

std::vector<Potential> get_polarizable_sites(const std::vector<Potential>& potentials);

// Owns one cppe_gpu_system for a set of polarizable sites and options; built
// on first use so that objects can be constructed without a GPU present.
class GpuSystem {
 public:
  GpuSystem(const std::vector<Potential>& polsites, const PeOptions& o);
  ~GpuSystem();
  GpuSystem(const GpuSystem&) = delete;
  GpuSystem& operator=(const GpuSystem&) = delete;
  cppe_gpu_system* get();
  int n() const { return m_n; }

 private:
  int m_n;
  std::vector<double> m_xyz, m_alpha6;
  std::vector<int> m_eptr, m_eidx;
  PeOptions m_opt;
  cppe_gpu_system* m_sys = nullptr;
};

class BMatrix {
  std::vector<Potential> m_polsites;
  size_t m_n_polsites;
  PeOptions m_options;
  std::shared_ptr<GpuSystem> m_gpu;

 public:
  BMatrix(std::vector<Potential> polsites, const PeOptions& options);
  Vector apply(const Vector& induced_moments);
  Vector apply_diagonal_inverse(const Vector& in);
  Vector apply_diagonal(const Vector& in);
  Matrix to_dense_matrix();
  Matrix direct_inverse();
};

class NuclearFields {
  std::vector<Potential> m_potentials, m_polsites;
  Molecule m_mol;

 public:
  NuclearFields(Molecule mol, std::vector<Potential> potentials);
  Vector compute();
  // (3 natoms) x (3 npolsites): d(field at site i)/d(position of atom a)
  Matrix nuclear_gradient();
};

class MultipoleFields {
  std::vector<Potential> m_potentials;
  PeOptions m_options;

 public:
  MultipoleFields(std::vector<Potential> potentials, const PeOptions& options)
        : m_potentials(std::move(potentials)), m_options(options) {}
  Vector compute();
};

class InducedMoments {
  std::vector<Potential> m_potentials, m_polsites;
  size_t m_n_polsites;
  PeOptions m_options;
  PrintCallback m_printer = [](std::string s) { std::cout << s << std::endl; };
  std::shared_ptr<GpuSystem> m_gpu;

 public:
  InducedMoments(std::vector<Potential> potentials, const PeOptions& options);
  void set_print_callback(PrintCallback p) { m_printer = std::move(p); }
  Vector compute(const Vector& rhs, Vector guess, bool make_guess);
  Vector compute(const Vector& total_fields, bool make_guess) {
    return compute(total_fields, Vector(total_fields.size(), 0.0), make_guess);
  }
  // Counters of the last solve: iterations, FP64 and FP32 operator applies.
  int last_iterations = 0, last_fp64_applies = 0, last_fp32_applies = 0;
  double last_rnorm = 0.0;
};

class MultipoleExpansion {
  Molecule m_mol;
  std::vector<Potential> m_potentials;

 public:
  MultipoleExpansion(Molecule core, std::vector<Potential> potentials)
        : m_mol(std::move(core)), m_potentials(std::move(potentials)) {}
  double interaction_energy();
  // natoms x 3: gradient of interaction_energy with respect to the atom positions
  Matrix nuclear_gradient();
};

using PeEnergy = std::unordered_map<std::string, std::unordered_map<std::string, double>>;

class CppeState {
  Molecule m_mol;
  std::vector<Potential> m_potentials;
  size_t m_polarizable_sites = 0;
  Vector m_nuc_fields, m_multipole_fields, m_induced_moments;
  Matrix m_positions, m_positions_polarizable;
  PeOptions m_options;
  bool m_make_guess = true;
  PrintCallback m_printer;
  std::shared_ptr<InducedMoments> m_solver;  // reused across SCF steps
  std::shared_ptr<void> m_eef;               // 3-right-hand-side batch of induced_moments_eef

 public:
  CppeState() = default;
  CppeState(const PeOptions& options, Molecule mol, PrintCallback printer = default_printer);
  void set_options(const PeOptions& o) { m_options = o; }
  PeOptions get_options() const { return m_options; }
  void set_molecule(Molecule mol) { m_mol = std::move(mol); }
  void set_potentials(std::vector<Potential> potentials);
  std::vector<Potential> get_potentials() const { return m_potentials; }
  Matrix get_positions() const { return m_positions; }
  Matrix get_positions_polarizable() const { return m_positions_polarizable; }
  void calculate_static_energies_and_fields();
  std::vector<double> get_induced_moments() const { return m_induced_moments; }
  Vector get_induced_moments_vec() const { return m_induced_moments; }
  PeEnergy m_pe_energy;
  double get_total_energy_for_category(const std::string& c);
  double get_total_energy();
  void update_induced_moments(const Vector& elec_fields, bool elec_only = false);
  size_t get_polarizable_site_number() const { return m_polarizable_sites; }
  Vector get_static_fields() const;
  Vector get_nuclear_fields() const { return m_nuc_fields; }
  Vector get_multipole_fields() const { return m_multipole_fields; }
  std::string get_energy_summary_string();
  Matrix induced_moments_eef();
  Matrix nuclear_interaction_energy_gradient();
  Matrix nuclear_field_gradient();
};

// Field of dipole sources at the sites, as the reference's Tree<1,3>
// computes it (src/core/fmm/tree.cc:350-394): F = -T S, by FMM or direct
// summation, on the GPU.  The reference's Python module exposes the class as
// fmm.Tree without a constructor (src/python_iface/export_fmm.cc:25-31); this
// one is built from positions and options.
class DipoleTree {
  std::vector<double> m_xyz, m_aiso;
  std::vector<int> m_eptr, m_eidx;
  int m_ncrit, m_order;
  double m_theta, m_damping;

 public:
  DipoleTree(std::vector<double> xyz, int ncrit, int order, double theta, double damping,
             std::vector<double> alpha_iso, std::vector<std::vector<int>> exclusions);
  int size() const { return (int)m_aiso.size(); }
  // S: 3n dipoles; F: 3n field values (overwritten)
  void compute_field(const double* S, double* F, bool fmm) const;
};

// math.hh helpers
double factorial(int n);
void make_df(unsigned k, std::vector<double>& df);
int trinom(int i, int j, int k);
std::vector<double> symmetry_factors(unsigned k);
std::vector<double> prefactors(unsigned k);
std::vector<double> prefactors_nuclei(unsigned k);
int multipole_components(int k);
std::array<double, 9> triangle_to_mat(const std::vector<double>& y);
std::vector<double> mat_to_triangle(const std::array<double, 9>& m);

// tensors submodule (tensors_autogen.hh, tensors_recursive.hh): Cartesian
// derivative tensors of 1/R and of the Thole-damped potential
Vector T_tensor(int k, const std::array<double, 3>& R);
Vector T_tensor_damp_thole(int k, const std::array<double, 3>& R, double a);
Vector T_recursive(int k, const std::array<double, 3>& R, double damping_factor = 0.0);
int xyz2idx(int x, int y, int z);

// PeOptions as C-ABI options (precision and device from gpu_config()), and a
// site list's exclusions as CSR (global site indices, as the reference keeps them)
cppe_gpu_options to_gpu(const PeOptions& o);
void pack_exclusions(const std::vector<Potential>& pots, std::vector<int>& ptr,
                     std::vector<int>& idx);

// Throws the exception that matches a C-ABI status (std::runtime_error with
// the library message; NOT_CONVERGED carries the reference's message).
void throw_on_status(int status);

}  // namespace libcppe
