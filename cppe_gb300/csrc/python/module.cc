// pybind11 module `pycppe`: the Python surface of the reference's module
// (src/python_iface/export_*.cc) -- same class, method, property and argument
// names, numpy float64 arrays where the reference passed Eigen objects -- on
// top of the GPU-backed host layer.
#include <pybind11/functional.h>
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>
#include <pybind11/stl_bind.h>

#include "cppe_gpu.h"
#include "cppe_host.hh"

namespace py = pybind11;
using namespace libcppe;

using MapSD  = std::unordered_map<std::string, double>;
using MapMSD = std::unordered_map<std::string, MapSD>;
PYBIND11_MAKE_OPAQUE(std::vector<libcppe::Atom>);
PYBIND11_MAKE_OPAQUE(MapSD);
PYBIND11_MAKE_OPAQUE(MapMSD);

namespace {

using Arr = py::array_t<double, py::array::c_style | py::array::forcecast>;

Vector to_vec(const Arr& a) { return Vector(a.data(), a.data() + a.size()); }
py::array_t<double> from_vec(const Vector& v) {
  py::array_t<double> a(v.size());
  std::copy(v.begin(), v.end(), a.mutable_data());
  return a;
}
py::array_t<double> from_mat(const Matrix& m) {
  py::array_t<double> a({m.rows, m.cols});
  std::copy(m.data.begin(), m.data.end(), a.mutable_data());
  return a;
}
py::array_t<double> from3(const std::array<double, 3>& v) {
  return from_vec(Vector(v.begin(), v.end()));
}

// _dict_to_options (export_state.cc:21-69)
PeOptions dict_to_options(const py::dict& d) {
  PeOptions o;
  for (const auto& kv : d) {
    const std::string key = kv.first.cast<std::string>();
    const auto v          = kv.second;
    if (std::find(valid_option_keys.begin(), valid_option_keys.end(), key) ==
        valid_option_keys.end())
      throw std::invalid_argument("Option key '" + key + "' is invalid.");
    if (key == "potfile") o.potfile = v.cast<std::string>();
    else if (key == "iso_pol") o.iso_pol = v.cast<bool>();
    else if (key == "induced_thresh") o.induced_thresh = v.cast<double>();
    else if (key == "maxiter") o.maxiter = v.cast<int>();
    else if (key == "damp_induced") o.damp_induced = v.cast<bool>();
    else if (key == "damp_multipole") o.damp_multipole = v.cast<bool>();
    else if (key == "damping_factor_induced") o.damping_factor_induced = v.cast<double>();
    else if (key == "damping_factor_multipole") o.damping_factor_multipole = v.cast<double>();
    else if (key == "summation_induced_fields") o.summation_induced_fields = v.cast<std::string>();
    else if (key == "tree_ncrit") o.tree_ncrit = v.cast<int>();
    else if (key == "tree_expansion_order") o.tree_expansion_order = v.cast<int>();
    else if (key == "theta") o.theta = v.cast<double>();
    else if (key == "pe_border") o.pe_border = v.cast<bool>();
    else if (key == "border_type") o.border_type = v.cast<std::string>();
    else if (key == "border_rmin") o.border_rmin = v.cast<double>();
    else if (key == "border_nredist") o.border_nredist = v.cast<int>();
    else if (key == "border_redist_order") o.border_redist_order = v.cast<int>();
    else if (key == "border_redist_pol") o.border_redist_pol = v.cast<bool>();
  }
  return o;
}

// _options_to_dict (export_state.cc:78-123)
py::dict options_to_dict(const PeOptions& o) {
  py::dict d;
  d["potfile"]                  = o.potfile;
  d["iso_pol"]                  = o.iso_pol;
  d["induced_thresh"]           = o.induced_thresh;
  d["maxiter"]                  = o.maxiter;
  d["damp_induced"]             = o.damp_induced;
  d["damping_factor_induced"]   = o.damping_factor_induced;
  d["damp_multipole"]           = o.damp_multipole;
  d["damping_factor_multipole"] = o.damping_factor_multipole;
  d["summation_induced_fields"] = o.summation_induced_fields;
  d["tree_expansion_order"]     = o.tree_expansion_order;
  d["tree_ncrit"]               = o.tree_ncrit;
  d["theta"]                    = o.theta;
  d["pe_border"]                = o.pe_border;
  d["border_type"]              = o.border_type;
  d["border_rmin"]              = o.border_rmin;
  d["border_nredist"]           = o.border_nredist;
  d["border_redist_order"]      = o.border_redist_order;
  d["border_redist_pol"]        = o.border_redist_pol;
  return d;
}

std::array<double, 3> vec3(const Arr& a, const char* what) {
  if (a.size() != 3) throw std::invalid_argument(std::string(what) + " must have 3 components");
  return {a.data()[0], a.data()[1], a.data()[2]};
}

// fmm.Tree: a DipoleTree and the caller's source array
struct PyDipoleTree {
  std::shared_ptr<DipoleTree> tree;
  py::object sources = py::none();
  void compute(py::array field, bool fmm) {
    const size_t n3 = 3 * (size_t)tree->size();
    if (sources.is_none()) throw std::runtime_error("Tree: call set_sources first");
    auto S = py::array_t<double, py::array::c_style | py::array::forcecast>::ensure(sources);
    if (!S || (size_t)S.size() != n3)
      throw std::invalid_argument("Tree: sources must hold 3 values per site");
    if (!py::isinstance<py::array_t<double>>(field) || (size_t)field.size() != n3 ||
        !(field.flags() & py::array::c_style) || !field.writeable())
      throw std::invalid_argument(
            "Tree: field must be a writable C-contiguous float64 array of 3 values per site");
    tree->compute_field(S.data(), static_cast<double*>(field.mutable_data()), fmm);
  }
};


}  // namespace

PYBIND11_MODULE(pycppe, m) {
  m.doc()                  = "Python interface for CPPE (GB300 induced-dipole path)";
  m.attr("__build_type__") = "Release";
  m.attr("__parallel__")   = true;

  // export_molecule.cc
  py::class_<Atom>(m, "Atom", "Atom class")
        .def(py::init<int, double, double, double>())
        .def_readwrite("atomic_number", &Atom::atomic_number)
        .def_readwrite("charge", &Atom::charge)
        .def_readwrite("x", &Atom::m_x)
        .def_readwrite("y", &Atom::m_y)
        .def_readwrite("z", &Atom::m_z)
        .def_property_readonly("position", [](const Atom& a) { return from3(a.get_position()); });
  py::bind_vector<std::vector<Atom>>(m, "Molecule");

  // export_potential.cc
  py::class_<Multipole>(m, "Multipole")
        .def(py::init<unsigned>())
        .def_readwrite("k", &Multipole::m_k)
        .def_property_readonly("values", [](const Multipole& x) { return from_vec(x.get_values_vec()); })
        .def("remove_trace", &Multipole::remove_trace)
        .def("add_value", &Multipole::add_value);
  py::class_<Polarizability>(m, "Polarizability")
        .def(py::init<>())
        .def_property_readonly("values", [](const Polarizability& p) { return from_vec(p.get_values_vec()); })
        .def_property_readonly("isotropic_value", &Polarizability::get_isotropic_value);
  py::class_<Potential>(m, "Potential", "Potential (Site)")
        .def(py::init<double, double, double, std::string, int>())
        .def_readwrite("x", &Potential::m_x, "x coordinate")
        .def_readwrite("y", &Potential::m_y, "y coordinate")
        .def_readwrite("z", &Potential::m_z, "z coordinate")
        .def_readwrite("element", &Potential::m_element, "element")
        .def_property_readonly("is_polarizable", &Potential::is_polarizable)
        .def("excludes_site", &Potential::excludes_site)
        .def_property_readonly("exclusions", [](const Potential& p) { return p.get_exclusions(); })
        .def_property_readonly("position", [](const Potential& p) { return from3(p.get_site_position()); })
        .def_property_readonly("multipoles", [](const Potential& p) { return p.get_multipoles(); })
        .def_property_readonly("polarizability", [](const Potential& p) { return p.get_polarizability(); })
        .def_readwrite("index", &Potential::index, "site index");

  // export_utils.cc
  py::class_<PotfileReader>(m, "PotfileReader", "Reader for potential files")
        .def(py::init<std::string>())
        .def("read", &PotfileReader::read, "Read the potential file");
  py::class_<PotManipulator>(m, "PotManipulator", "Manipulator for potentials")
        .def(py::init<std::vector<Potential>, Molecule>());

  // export_state.cc
  py::bind_map<MapSD>(m, "UnorderedMapStringDouble");
  py::bind_map<MapMSD>(m, "UnorderedMapMapStringDouble");
  py::class_<CppeState, std::shared_ptr<CppeState>>(m, "CppeState")
        .def(py::init([](py::dict options, Molecule mol, PrintCallback printer) {
               return std::make_shared<CppeState>(dict_to_options(options), mol, printer);
             }),
             "Create a CppeState using a dictionary with options, molecule, and print callback",
             py::arg("options") = py::dict(), py::arg("molecule") = Molecule(),
             py::arg("printer") = default_printer)
        .def_property_readonly("positions", [](const CppeState& s) { return from_mat(s.get_positions()); })
        .def_property_readonly("positions_polarizable",
                               [](const CppeState& s) { return from_mat(s.get_positions_polarizable()); })
        .def("set_potentials", &CppeState::set_potentials)
        .def("calculate_static_energies_and_fields", &CppeState::calculate_static_energies_and_fields)
        .def("nuclear_interaction_energy_gradient",
             [](CppeState& s) { return from_mat(s.nuclear_interaction_energy_gradient()); })
        .def("nuclear_field_gradient",
             [](CppeState& s) { return from_mat(s.nuclear_field_gradient()); })
        .def("get_induced_moments", &CppeState::get_induced_moments)
        .def("induced_moments_eef", [](CppeState& s) { return from_mat(s.induced_moments_eef()); })
        .def_readwrite("energies", &CppeState::m_pe_energy)
        .def_property_readonly("total_energy", &CppeState::get_total_energy)
        .def("update_induced_moments",
             [](CppeState& s, Arr f, bool elec_only) { s.update_induced_moments(to_vec(f), elec_only); },
             py::arg("elec_fields"), py::arg("elec_only") = false)
        .def_property_readonly("static_fields", [](const CppeState& s) { return from_vec(s.get_static_fields()); })
        .def_property_readonly("nuclear_fields", [](const CppeState& s) { return from_vec(s.get_nuclear_fields()); })
        .def_property_readonly("multipole_fields",
                               [](const CppeState& s) { return from_vec(s.get_multipole_fields()); })
        .def_property_readonly("summary_string", &CppeState::get_energy_summary_string)
        .def_property_readonly("potentials", &CppeState::get_potentials)
        .def("get_polarizable_site_number", &CppeState::get_polarizable_site_number)
        .def_property_readonly("options", [](const CppeState& s) { return options_to_dict(s.get_options()); });
  m.attr("valid_option_keys") = py::cast(valid_option_keys);

  // export_fields.cc
  py::class_<NuclearFields>(m, "NuclearFields", "Electric fields created by nuclei")
        .def(py::init<Molecule, std::vector<Potential>>())
        .def("compute", [](NuclearFields& f) { return from_vec(f.compute()); })
        .def("nuclear_gradient", [](NuclearFields& f) { return from_mat(f.nuclear_gradient()); });
  py::class_<MultipoleFields, std::shared_ptr<MultipoleFields>>(m, "MultipoleFields",
                                                                "Electric fields created by multipoles")
        .def(py::init([](std::vector<Potential> p, py::dict o) {
          return std::make_shared<MultipoleFields>(p, dict_to_options(o));
        }))
        .def("compute", [](MultipoleFields& f) { return from_vec(f.compute()); });
  py::class_<InducedMoments, std::shared_ptr<InducedMoments>>(m, "InducedMoments")
        .def(py::init([](std::vector<Potential> p, py::dict o) {
          return std::make_shared<InducedMoments>(p, dict_to_options(o));
        }))
        .def("compute",
             [](InducedMoments& im, Arr f, bool make_guess) {
               return from_vec(im.compute(to_vec(f), make_guess));
             },
             "Compute the induced moments solving the classical response equation using a CG "
             "solver",
             py::arg("total_fields"), py::arg("make_guess"))
        .def("set_print_callback", &InducedMoments::set_print_callback)
        .def_property_readonly("last_stats", [](const InducedMoments& im) {
          py::dict d;
          d["iterations"]   = im.last_iterations;
          d["fp64_applies"] = im.last_fp64_applies;
          d["fp32_applies"] = im.last_fp32_applies;
          d["rnorm"]        = im.last_rnorm;
          return d;
        });
  m.def("get_polarizable_sites", &get_polarizable_sites);
  py::class_<BMatrix, std::shared_ptr<BMatrix>>(m, "BMatrix")
        .def(py::init([](std::vector<Potential> p, py::dict o) {
          return std::make_shared<BMatrix>(p, dict_to_options(o));
        }))
        .def("direct_inverse", [](BMatrix& b) { return from_mat(b.direct_inverse()); })
        .def("to_dense_matrix", [](BMatrix& b) { return from_mat(b.to_dense_matrix()); })
        .def("apply", [](BMatrix& b, Arr v) { return from_vec(b.apply(to_vec(v))); })
        .def("apply_diagonal", [](BMatrix& b, Arr v) { return from_vec(b.apply_diagonal(to_vec(v))); })
        .def("apply_diagonal_inverse",
             [](BMatrix& b, Arr v) { return from_vec(b.apply_diagonal_inverse(to_vec(v))); });
  py::class_<MultipoleExpansion, std::shared_ptr<MultipoleExpansion>>(m, "MultipoleExpansion")
        .def(py::init<Molecule, std::vector<Potential>>())
        .def("interaction_energy", &MultipoleExpansion::interaction_energy)
        .def("nuclear_gradient",
             [](MultipoleExpansion& e) { return from_mat(e.nuclear_gradient()); });

  // export_math.cc
  m.def("triangle_to_mat", [](std::vector<double> y) {
    auto a = triangle_to_mat(y);
    Matrix M(3, 3);
    std::copy(a.begin(), a.end(), M.data.begin());
    return from_mat(M);
  });
  m.def("mat_to_triangle", [](Arr a) {
    std::array<double, 9> v{};
    if (a.size() != 9) throw std::invalid_argument("mat_to_triangle expects a 3x3 matrix");
    std::copy(a.data(), a.data() + 9, v.begin());
    return from_vec(mat_to_triangle(v));
  });
  m.def("factorial", &factorial);
  m.def("make_df", [](unsigned k, std::vector<double> df) {
    make_df(k, df);
    return df;
  });
  m.def("trinom", &trinom);
  m.def("symmetry_factors", &symmetry_factors);
  m.def("prefactors", &prefactors, "Prefactors for the multipole components (alphabetical order)");
  m.def("prefactors_nuclei", &prefactors_nuclei);
  m.def("multipole_components", &multipole_components);

  // export_tensors.cc: Cartesian derivative tensors of 1/R and of the
  // Thole-damped potential.  The reference binds T1_damp_thole under the name
  // T0_damp_thole (export_tensors.cc:32), so it is unreachable there; here
  // every order has its own name.
  py::module ten = m.def_submodule("tensors", "Tensor submodule");
  ten.def("T_recursive",
          [](int k, Arr R, double damping_factor) {
            return from_vec(T_recursive(k, vec3(R, "Rij"), damping_factor));
          },
          py::arg("k"), py::arg("Rij"), py::arg("damping_factor") = 0.0);
  ten.def("xyz2idx", &xyz2idx);
  py::list T, Td;
  for (int k = 0; k <= 6; ++k) {
    auto f  = [k](Arr R) { return from_vec(T_tensor(k, vec3(R, "rij"))); };
    auto fd = [k](Arr R, double a) { return from_vec(T_tensor_damp_thole(k, vec3(R, "rij"), a)); };
    const std::string nm = "T" + std::to_string(k);
    ten.def(nm.c_str(), f);
    ten.def((nm + "_damp_thole").c_str(), fd);
    T.append(ten.attr(nm.c_str()));
    Td.append(ten.attr((nm + "_damp_thole").c_str()));
  }
  ten.attr("T")            = T;
  ten.attr("T_damp_thole") = Td;

  // export_fmm.cc: Tree<1,3> -- the field of dipole sources at the sites by
  // FMM or by direct summation.  The reference gives the class no Python
  // constructor; this one takes positions (n x 3, bohr) and the tree options.
  // set_sources keeps a reference to the caller's array (the reference keeps a
  // pointer to it), read again by every compute call.
  py::module fmm = m.def_submodule("fmm", "Module for fast multipole methods.");
  py::class_<PyDipoleTree, std::shared_ptr<PyDipoleTree>>(fmm, "Tree", "Tree class for FMM/BH.")
        .def(py::init([](Arr positions, int ncrit, int order, double theta, double damping,
                         py::object polarizabilities, py::object exclusions) {
               auto t = std::make_shared<PyDipoleTree>();
               std::vector<double> aiso;
               if (!polarizabilities.is_none()) aiso = to_vec(polarizabilities.cast<Arr>());
               std::vector<std::vector<int>> ex;
               if (!exclusions.is_none()) ex = exclusions.cast<std::vector<std::vector<int>>>();
               t->tree = std::make_shared<DipoleTree>(to_vec(positions), ncrit, order, theta,
                                                      damping, aiso, ex);
               return t;
             }),
             py::arg("positions"), py::arg("ncrit") = 64, py::arg("order") = 5,
             py::arg("theta") = 0.5, py::arg("damping") = 0.0,
             py::arg("polarizabilities") = py::none(), py::arg("exclusions") = py::none())
        .def("set_sources", [](PyDipoleTree& t, py::array sources) { t.sources = sources; })
        .def("compute_field_fmm", [](PyDipoleTree& t, py::array field) { t.compute(field, true); })
        .def("compute_field_exact",
             [](PyDipoleTree& t, py::array field) { t.compute(field, false); });

  // GPU controls (no counterpart in the reference)
  m.def("set_gpu_options",
        [](const std::string& precision, int device) {
          if (precision != "fp64" && precision != "mixed")
            throw std::invalid_argument("precision must be 'fp64' or 'mixed'");
          gpu_config().precision = precision == "mixed" ? 1 : 0;
          gpu_config().device    = device;
        },
        py::arg("precision") = "fp64", py::arg("device") = 0);
  m.def("get_gpu_options", []() {
    py::dict d;
    d["precision"] = gpu_config().precision == 1 ? "mixed" : "fp64";
    d["device"]    = gpu_config().device;
    return d;
  });
  m.def("device_count", []() {
    int c = 0;
    cppe_gpu_device_count(&c);
    return c;
  });
}
