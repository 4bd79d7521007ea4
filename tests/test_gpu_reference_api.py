"""The reference's own functional tests, restated through
``import cppe_gb300 as cppe`` on the GPU.

* tests/test_solver.py:36-146 (both tests): the B matrix assembled from
  T_recursive against BMatrix.apply, the matrix rebuilt column by column from
  applies, the CppeState solve against the inverse, InducedMoments.compute,
  and BMatrix.direct_inverse -- with the same tolerances;
* tests/test_functionality.py:38-90: the electrostatic nuclear energy against
  pelib's -0.321349401430 (decimal 9), the energy container, and iso_pol;
* tests/test_gradients.py:32-95: MultipoleExpansion.nuclear_gradient and
  NuclearFields.nuclear_gradient against 5-point finite differences
  (step 1e-3 bohr, atol 1e-10);
* fmm.Tree (src/python_iface/export_fmm.cc): the dipole field by FMM and by
  direct summation against the oracle.

The molecule is the reference tests' p-nitroaniline (tests/golden/
pna_molecule.json, from the reference's tests/dump_pyscf.py).
"""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


def triangle_to_mat(y):
    mat = np.empty((3, 3))
    mat[0, 0] = y[0]
    mat[0, 1] = mat[1, 0] = y[1]
    mat[0, 2] = mat[2, 0] = y[2]
    mat[1, 1] = y[3]
    mat[1, 2] = mat[2, 1] = y[4]
    mat[2, 2] = y[5]
    return mat


def block(s1, s2):
    return (slice(3 * s1, 3 * s1 + 3), slice(3 * s2, 3 * s2 + 3))


@pytest.fixture(scope="module")
def pna_mol():
    import cppe_gb300 as cppe
    with open(os.path.join(HERE, "golden", "pna_molecule.json")) as f:
        m = json.load(f)
    mol = cppe.Molecule()
    for z, xyz in zip(m["Z"], m["xyz_bohr"]):
        mol.append(cppe.Atom(z, *xyz))
    return mol


@pytest.mark.parametrize("damped", [False, True])
def test_solver_by_inversion(gpu, unpacked, pna_mol, damped):
    import cppe_gb300 as cppe
    from cppe_gb300 import T_recursive
    options = {"potfile": unpacked["pna_6w.pot"], "induced_thresh": 1e-12}
    if damped:
        options["damp_induced"] = True
    cppe_state = cppe.CppeState(options, pna_mol, lambda s: None)
    cppe_state.calculate_static_energies_and_fields()
    static_fields = cppe_state.static_fields
    zeros = np.zeros_like(static_fields)
    cppe_state.update_induced_moments(zeros, False)

    potentials = cppe_state.potentials
    polsites = cppe.get_polarizable_sites(potentials)
    npolsites = cppe_state.get_polarizable_site_number()
    bmat = np.zeros((3 * npolsites, 3 * npolsites))
    for s1, pot1 in enumerate(polsites):
        pol = pot1.polarizability
        bmat[block(s1, s1)] = np.linalg.inv(triangle_to_mat(pol.values))
        for s2, pot2 in enumerate(polsites):
            if pot1.excludes_site(pot2.index) or s1 == s2:
                continue
            diff = pot2.position - pot1.position
            if damped:
                v = 2.1304 / (pol.isotropic_value * pot2.polarizability.isotropic_value) ** (1 / 6)
                T12 = T_recursive(2, diff, v)
            else:
                T12 = T_recursive(2, diff)
            if s1 > s2:
                bmat[block(s1, s2)] = -triangle_to_mat(T12)
                bmat[block(s2, s1)] = -triangle_to_mat(T12)

    bmatrix_cpp = cppe.BMatrix(polsites, options)
    np.testing.assert_allclose(bmatrix_cpp.apply(static_fields), bmat @ static_fields,
                               atol=1e-12)
    Afull = np.stack([bmatrix_cpp.apply(e) for e in np.eye(static_fields.size)], axis=1)
    np.testing.assert_allclose(Afull, bmat, atol=1e-20)

    induced_moments_direct = np.linalg.inv(bmat) @ static_fields
    np.testing.assert_almost_equal(cppe_state.get_induced_moments(), induced_moments_direct,
                                   decimal=9)
    ind_mom = cppe.InducedMoments(potentials, options)
    res_cg = ind_mom.compute(static_fields, True)
    np.testing.assert_allclose(res_cg, induced_moments_direct, atol=1e-10)
    binv = bmatrix_cpp.direct_inverse()
    np.testing.assert_allclose(binv @ static_fields, induced_moments_direct, atol=1e-15)


def test_compute_nuclear_interaction_energy(gpu, unpacked, pna_mol):
    import cppe_gb300 as cppe
    cppe_state = cppe.CppeState({"potfile": unpacked["pna_6w.pot"]}, pna_mol, lambda s: None)
    assert cppe_state.get_polarizable_site_number() == 18
    cppe_state.calculate_static_energies_and_fields()
    en_el_nuc = cppe_state.energies["Electrostatic"]["Nuclear"]
    np.testing.assert_almost_equal(en_el_nuc, -0.321349401430, decimal=9)  # pelib
    bla = cppe_state.energies["Electrostatic"]
    bla["Nuclear"] = -10.0
    assert bla["Nuclear"] == -10.0
    cppe_state.energies["Electrostatic"]["Nuclear"] = -20.0
    assert cppe_state.energies["Electrostatic"]["Nuclear"] == -20.0
    cppe_state.energies["Electrostatic"]["Electronic"] = 1.0
    cppe_state.energies["Electrostatic"]["Nuclear"] = 2.0
    cppe_state.energies["Electrostatic"]["Multipoles"] = 3.0
    cppe_state.energies["Polarization"]["Electronic"] = 4.0
    cppe_state.energies["Polarization"]["Nuclear"] = 5.0
    cppe_state.energies["Polarization"]["Multipole"] = 6.0
    total_energy = (
        cppe_state.energies["Electrostatic"]["Electronic"]
        + cppe_state.energies["Electrostatic"]["Nuclear"]
        + cppe_state.energies["Electrostatic"]["Multipoles"]
        + cppe_state.energies["Polarization"]["Electronic"]
        + cppe_state.energies["Polarization"]["Nuclear"]
        + cppe_state.energies["Polarization"]["Multipole"]
    )
    assert cppe_state.total_energy == total_energy


def test_iso_pol(gpu, unpacked, pna_mol):
    import cppe_gb300 as cppe

    def solve(options):
        st = cppe.CppeState(options, pna_mol, lambda s: None)
        st.calculate_static_energies_and_fields()
        np.testing.assert_allclose(st.static_fields, st.nuclear_fields + st.multipole_fields)
        st.update_induced_moments(np.zeros_like(st.static_fields), False)
        return st

    test = solve({"potfile": unpacked["pna_6w.pot"], "iso_pol": True})
    ref = solve({"potfile": unpacked["pna_6w_isopol.pot"]})
    for pt, pr in zip(test.potentials, ref.potentials):
        np.testing.assert_almost_equal(pt.polarizability.values, pr.polarizability.values)
    np.testing.assert_almost_equal(test.get_induced_moments(), ref.get_induced_moments(),
                                   decimal=8)


STENCIL = (np.array([-2, -1, 1, 2]), np.array([1.0, -8.0, 8.0, -1.0]) / 12.0)


def _mol(cppe, atoms, coords):
    m = cppe.Molecule()
    for z, c in zip(atoms, coords):
        m.append(cppe.Atom(z, *c))
    return m


def test_nuclear_gradients_match_finite_differences(gpu, unpacked, pna_mol):
    import cppe_gb300 as cppe
    potentials = cppe.PotfileReader(unpacked["pna_6w.pot"]).read()
    atoms = [a.atomic_number for a in pna_mol]
    coords = np.array([a.position for a in pna_mol])
    natoms = len(atoms)
    polsites = cppe.get_polarizable_sites(potentials)
    step = 1e-3
    g_e = np.zeros((natoms, 3))
    g_f = np.zeros((natoms, 3, len(polsites), 3))
    for i in range(natoms):
        for c in range(3):
            for f, p in zip(*STENCIL):
                cp = coords.copy()
                cp[i, c] += f * step
                mol_p = _mol(cppe, atoms, cp)
                g_e[i, c] += p * cppe.MultipoleExpansion(mol_p, potentials).interaction_energy() / step
                g_f[i, c] += p * cppe.NuclearFields(mol_p, potentials).compute().reshape(
                    len(polsites), 3) / step
    grad_nuc = cppe.MultipoleExpansion(pna_mol, potentials).nuclear_gradient()
    np.testing.assert_allclose(g_e, grad_nuc, atol=1e-10)
    grad_field = cppe.NuclearFields(pna_mol, potentials).nuclear_gradient().reshape(
        (natoms, 3, len(polsites), 3))
    np.testing.assert_allclose(g_f, grad_field, atol=1e-10)
    st = cppe.CppeState({"potfile": unpacked["pna_6w.pot"]}, pna_mol, lambda s: None)
    np.testing.assert_allclose(st.nuclear_interaction_energy_gradient(), grad_nuc, rtol=0,
                               atol=0)
    np.testing.assert_allclose(st.nuclear_field_gradient().reshape(grad_field.shape),
                               grad_field, rtol=0, atol=0)


def test_fmm_tree_dipole_field(gpu, port):
    import cppe_gb300 as cppe
    from cppe_gb300 import synthetic
    b = synthetic.water_box(300, seed=21)
    S = np.random.default_rng(4).normal(size=(b.n, 3))
    ex = [list(b.excl_idx[b.excl_ptr[i]:b.excl_ptr[i + 1]]) for i in range(b.n)]
    for damping in (0.0, 2.1304):
        tree = cppe.fmm.Tree(b.xyz, ncrit=32, order=5, theta=0.5, damping=damping,
                             polarizabilities=b.alpha_iso, exclusions=ex)
        tree.set_sources(S)
        f_fmm = np.zeros(3 * b.n)
        f_ex = np.zeros(3 * b.n)
        tree.compute_field_fmm(f_fmm)
        tree.compute_field_exact(f_ex)
        for fmm, got in ((1, f_fmm), (0, f_ex)):
            ref = port.field(1, b.xyz, S, polarizable=np.ones(b.n, np.int32),
                             alpha_iso=b.alpha_iso, excl_ptr=b.excl_ptr, excl_idx=b.excl_idx,
                             fmm=fmm, ncrit=32, order=5, theta=0.5, damping=damping)
            np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    # the sources are read at compute time (the reference keeps a pointer)
    S *= 2.0
    tree.compute_field_exact(f_ex)
    np.testing.assert_allclose(f_ex, 2.0 * ref, rtol=0, atol=2e-12 * np.abs(ref).max())
