"""CPU-side checks of the product: the C ABI library loads and exports every
declared symbol, the host tree build matches the reference's lists, and the
reference-facing Python API (options, potfile reader, data classes) behaves
like the reference's on CPU (no GPU calls)."""
import ctypes
import hashlib

import numpy as np
import pytest

import cabi


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(cabi.LIB_PATH)
    names = cabi.declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_default_options_match_reference():
    o = cabi.options()
    assert (o.tree_ncrit, o.tree_expansion_order, o.theta, o.maxiter) == (64, 5, 0.5, 50)
    assert o.induced_thresh == 1e-8 and o.damping_factor == 2.1304 and o.damp == 0


def _hash(m2l, p2p):
    h = hashlib.sha256()
    h.update(np.sort(m2l.view(np.int64).ravel()).tobytes())
    h.update(np.sort(p2p.view(np.int64).ravel()).tobytes())
    return h.hexdigest()


@pytest.mark.parametrize("tag,nw,seed", [("c0", 333, 0), ("c1", 10000, 1)])
def test_tree_lists_match_reference(golden_vectors, tag, nw, seed):
    from cppe_gb300 import synthetic
    b = synthetic.water_box(nw, seed=seed)
    info, m2l, p2p = cabi.tree_lists(b.xyz, ncrit=64, theta=0.5)
    counts = golden_vectors[f"tree_{tag}_counts"]
    assert (info["ncells"], info["nm2l"], info["np2p"]) == tuple(counts)
    assert _hash(m2l, p2p) == str(golden_vectors[f"tree_{tag}_hash"][0])


def test_tree_lists_match_oracle_deep_tree(loprop, port):
    # ncrit 16 puts many cell pairs exactly on the theta = 0.5 boundary
    info, m2l, p2p = cabi.tree_lists(loprop.xyz, ncrit=16, theta=0.5)
    t = port.tree_lists(loprop.xyz, ncrit=16, theta=0.5)
    np.testing.assert_array_equal(p2p, t["p2p"])
    np.testing.assert_array_equal(np.sort(m2l.view(np.int64).ravel()),
                                  np.sort(t["m2l"].view(np.int64).ravel()))


@pytest.mark.parametrize("nw,ncrit", [(1000, 64), (3000, 16)])
def test_m2l_translation_vectors(port, nw, ncrit):
    """The FMM tabulates its M2L derivative tensors per distinct centre
    difference: the count it finds equals the distinct differences of the
    oracle tree's M2L list, and is well below the list's length (the ratio
    grows with the tree: 4,832 for 14.6 M entries at 300k sites)."""
    from cppe_gb300 import synthetic
    b = synthetic.water_box(nw, seed=7)
    nvec, nent = cabi.tree_vectors(b.xyz, ncrit=ncrit, theta=0.5)
    t = port.tree_lists(b.xyz, ncrit=ncrit, order=5, theta=0.5)
    c, m = t["cells"][:, :3], t["m2l"]
    assert nent == len(m)
    # differences are multiples of the deepest half-width: exact on its grid
    u = 0.5 * t["cells"][:, 3].min()
    keys = np.round((c[m[:, 1]] - c[m[:, 0]]) / u).astype(np.int64)
    assert nvec == len(np.unique(keys, axis=0))
    assert 0 < nvec < nent // 4


def test_tree_rejects_coincident_sites():
    xyz = np.zeros((80, 3))
    with pytest.raises(RuntimeError, match="coincide"):
        cabi.tree_info(xyz, ncrit=64)


# --- reference-facing Python API (host side only) ----------------------------
@pytest.fixture(scope="module")
def cppe():
    import cppe_gb300
    return cppe_gb300


DEFAULT_OPTIONS = {
    "iso_pol": False, "induced_thresh": 1e-8, "maxiter": 50, "damp_induced": False,
    "damp_multipole": False, "damping_factor_induced": 2.1304,
    "damping_factor_multipole": 2.1304, "summation_induced_fields": "direct",
    "tree_expansion_order": 5, "tree_ncrit": 64, "theta": 0.5, "pe_border": False,
    "border_type": "remove", "border_rmin": 2.2, "border_nredist": -1,
    "border_redist_order": 1, "border_redist_pol": False,
}


def test_options_defaults(cppe, unpacked):
    # tests/test_options.py:35-44
    s = cppe.CppeState({"potfile": unpacked["pna_6w.pot"]})
    opts = dict(s.options)
    opts.pop("potfile")
    assert len(opts) == len(DEFAULT_OPTIONS)
    for k, v in DEFAULT_OPTIONS.items():
        assert opts[k] == v


def test_options_set_all(cppe, unpacked):
    # tests/test_options.py:46-71
    custom = {"potfile": unpacked["pna_6w.pot"], "iso_pol": True, "induced_thresh": 1e-4,
              "maxiter": 500, "damp_induced": True, "damp_multipole": True,
              "damping_factor_induced": 213.04, "damping_factor_multipole": 213.04,
              "summation_induced_fields": "fmm", "tree_expansion_order": 4, "tree_ncrit": 12,
              "theta": 0.2, "pe_border": True, "border_type": "redist", "border_rmin": 2.6,
              "border_nredist": 2, "border_redist_order": 2, "border_redist_pol": True}
    s = cppe.CppeState(custom)
    for k, v in custom.items():
        assert s.options[k] == v


def test_options_invalid_key(cppe):
    # tests/test_options.py:73-77
    with pytest.raises(ValueError):
        cppe.CppeState({"invalid_key": 42})
    assert len(cppe.valid_option_keys) == 18


def test_read_potfile(cppe, unpacked):
    # tests/test_functionality.py:33-36
    pots = cppe.PotfileReader(unpacked["pna_6w.pot"]).read()
    assert len(pots) == 18
    p = pots[0]
    np.testing.assert_allclose(p.position, np.array([9.371, 2.953, -6.078]) * 1.8897261246)
    assert p.exclusions == [1, 2] and p.excludes_site(2) and not p.excludes_site(3)
    assert [m.k for m in p.multipoles] == [0, 1, 2]
    q = p.multipoles[2].values
    assert abs(q[0] + q[3] + q[5]) < 1e-12  # traceless after reading
    np.testing.assert_allclose(p.polarizability.values,
                               [2.30791521, 0.59643991, 0.58658837, 2.61100398, -0.10257978,
                                2.60785108])
    with pytest.raises(RuntimeError, match="does not exist"):
        cppe.PotfileReader("/nonexistent.pot")


def test_potfile_reader_matches_oracle_reader(cppe, unpacked, loprop):
    pots = cppe.PotfileReader(unpacked["loprop_solvated_20.pot"]).read()
    assert len(pots) == loprop.n
    xyz = np.array([p.position for p in pots])
    np.testing.assert_array_equal(xyz, loprop.xyz)
    quad = np.array([p.multipoles[2].values for p in pots])
    np.testing.assert_allclose(quad, loprop.quad, atol=1e-15)


def test_iso_pol_makes_isotropic(cppe, unpacked):
    s = cppe.CppeState({"potfile": unpacked["pna_6w.pot"], "iso_pol": True})
    r = cppe.CppeState({"potfile": unpacked["pna_6w_isopol.pot"]})
    for pt, pr in zip(s.potentials, r.potentials):
        np.testing.assert_almost_equal(pt.polarizability.values, pr.polarizability.values)


def test_state_positions_and_counts(cppe, unpacked):
    s = cppe.CppeState({"potfile": unpacked["pna_6w.pot"]})
    assert s.get_polarizable_site_number() == 18
    assert s.positions.shape == (18, 3) and s.positions_polarizable.shape == (18, 3)
    assert len(s.get_induced_moments()) == 54
    en = s.energies["Electrostatic"]
    en["Nuclear"] = -10.0
    assert s.energies["Electrostatic"]["Nuclear"] == -10.0


def test_math_helpers(cppe):
    assert cppe.factorial(5) == 120 and cppe.trinom(1, 1, 0) == 2
    assert cppe.multipole_components(2) == 6
    assert list(cppe.symmetry_factors(2)) == [1, 2, 2, 1, 2, 1]
    np.testing.assert_allclose(cppe.prefactors(1), [-1, -1, -1])
    np.testing.assert_allclose(cppe.prefactors_nuclei(2), [0.5, 1, 1, 0.5, 1, 0.5])
    m = cppe.triangle_to_mat([1, 2, 3, 4, 5, 6])
    np.testing.assert_array_equal(cppe.mat_to_triangle(m), [1, 2, 3, 4, 5, 6])


def test_gpu_calls_fail_loudly_without_device(cppe, unpacked):
    if cabi.device_count() > 0:
        pytest.skip("a GPU is present")
    pots = cppe.PotfileReader(unpacked["pna_6w.pot"]).read()
    b = cppe.BMatrix(cppe.get_polarizable_sites(pots), {})
    with pytest.raises(RuntimeError):
        b.apply(np.zeros(54))


def test_synthetic_potfile_round_trip(cppe, tmp_path):
    from cppe_gb300 import synthetic
    b = synthetic.water_box(40, seed=5)
    path = str(tmp_path / "w.pot")
    synthetic.write_potfile(b, path)
    pots = cppe.PotfileReader(path).read()
    xyz = np.array([p.position for p in pots])
    np.testing.assert_allclose(xyz, b.xyz, atol=1e-10)
    assert all(p.exclusions == list(b.excl_idx[2 * i:2 * i + 2]) for i, p in enumerate(pots))
    np.testing.assert_allclose([p.polarizability.isotropic_value for p in pots], b.alpha_iso)


def _straight_line_m2l(gen, m, p, x, y, z, Mb):
    """Evaluates the generated straight-line translation (C source of
    m2l_gen.cuh) in FP64 by rewriting it as Python."""
    import re
    code, _, ls, _ = gen.emit(m, p)
    body = code.split("\n}\n", 1)[0].split("{", 1)[1]  # the first function
    lines = []
    for ln in body.split("\n"):
        ln = ln.strip().replace("const T ", "").replace("cinv<T>(", "1.0/(").replace("T(", "float(")
        ln = ln.replace("rsqrt_t(r2)", "r2**-0.5")
        ln = re.sub(r"fma\((D\d+), mk, (acc\[\d+\])\)", r"\1*mk + \2", ln)
        ln = ln.replace("{ ", "").replace(";", "").replace("}", "").strip()
        if ln:
            lines.append(ln)
    env = dict(x=x, y=y, z=z, Mb=Mb, acc=[0.0] * ls)
    exec("\n".join(lines), env)
    return np.array(env["acc"])


@pytest.mark.parametrize("m,p", [(1, 5), (1, 6)])
def test_m2l_loop_tables_match_straight_line(m, p):
    """The tables of the loop-form (double-float) M2L encode the same
    translation as the generated straight-line code: the derivative
    recurrence and every D_{n+k} M_k term, evaluated here in FP64."""
    import os
    import re
    import sys
    sys.path.insert(0, os.path.join(cabi.LIB_PATH.rsplit(os.sep, 1)[0], "csrc"))
    import gen_m2l as gen
    rng = np.random.default_rng(p)
    tcode, _, nt = gen.emit_tables(m, p)
    arrs = re.findall(r"\{\n  (.*?)\};", tcode, re.S)
    rec = np.array([int(v) for v in arrs[0].split(",")]).reshape(nt, 8)
    coef = np.array([float(v.strip().rstrip("f")) for v in arrs[1].split(",")]).reshape(nt, 8)
    w = [int(v) for v in arrs[2].split(",")]
    mi = gen.multi_indices(p)
    moff, ls, ms = gen.nterms(m - 1), gen.nterms(p - m), gen.nterms(p) - gen.nterms(m - 1)
    for _ in range(4):
        x, y, z = rng.normal(size=3) * 3.0
        Mb = rng.normal(size=ms)
        ref = _straight_line_m2l(gen, m, p, x, y, z, Mb)
        r2 = x * x + y * y + z * z
        D = np.zeros(nt)
        D[0] = r2 ** -0.5
        for j in range(1, nt):
            q, c = rec[j], coef[j]
            s = sum(c[i] * rv * D[q[i]] for i, rv in enumerate((x, y, z)) if q[i] >= 0)
            s += sum(c[3 + i] * D[q[3 + i]] for i in range(3) if q[3 + i] >= 0)
            D[j] = -s / r2 * (c[6] + c[7])
        out, t = np.zeros(ls), 0
        for k in range(moff, nt):
            for n in range(gen.nterms(p - sum(mi[k]))):
                out[n] += D[w[t]] * Mb[k - moff]
                t += 1
        assert t == len(w)
        np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)))


# --- potfile ingest into arrays and CSR (cppe_gpu_potfile_*) -----------------
@pytest.mark.parametrize("name", ["pna_6w.pot", "pna_6w_isopol.pot", "loprop_solvated_20.pot"])
def test_potfile_arrays_match_oracle_reader(unpacked, name):
    from oracle import oracle as O
    got = cabi.read_potfile(unpacked[name])
    ref = O.read_potfile(unpacked[name])
    np.testing.assert_array_equal(got["xyz"], ref.xyz)
    np.testing.assert_array_equal(got["q"], ref.q)
    np.testing.assert_array_equal(got["mu"], ref.mu)
    np.testing.assert_array_equal(got["quad"], ref.quad)
    np.testing.assert_array_equal(got["alpha6"], ref.alpha6)
    np.testing.assert_array_equal(got["polarizable"], ref.polarizable)
    np.testing.assert_array_equal(got["excl_ptr"], ref.excl_ptr)
    np.testing.assert_array_equal(got["excl_idx"], ref.excl_idx)
    assert got["elements"] == list(ref.elements)


def test_potfile_arrays_million_sites(tmp_path):
    """A 1,000,002-site water box written as a .pot file (AA, 12 decimals) and
    read back into arrays and CSR exclusions; the object reader
    (PotfileReader.read) gives the same sites."""
    import time
    import cppe_gb300 as cppe
    from cppe_gb300 import synthetic
    b = synthetic.water_box(333334, seed=4)
    path = str(tmp_path / "w1m.pot")
    synthetic.write_potfile(b, path)
    t0 = time.perf_counter()
    got = cabi.read_potfile(path)
    t_soa = time.perf_counter() - t0
    assert got["xyz"].shape == (1000002, 3)
    np.testing.assert_allclose(got["xyz"], b.xyz, rtol=0, atol=1e-10)
    np.testing.assert_allclose(got["mu"], b.mu, rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["quad"], b.quad, rtol=0, atol=1e-12)
    np.testing.assert_allclose(got["alpha6"], b.alpha6, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(got["excl_ptr"], b.excl_ptr)
    np.testing.assert_array_equal(got["excl_idx"], b.excl_idx)
    t0 = time.perf_counter()
    pots = cppe.PotfileReader(path).read()
    t_obj = time.perf_counter() - t0
    assert len(pots) == b.n
    for i in (0, 1, 499999, b.n - 1):
        np.testing.assert_array_equal(pots[i].position, got["xyz"][i])
        assert sorted(pots[i].exclusions) == sorted(
            got["excl_idx"][got["excl_ptr"][i]:got["excl_ptr"][i + 1]])
    print(f"1M-site potfile: arrays + CSR {t_soa:.2f} s, objects {t_obj:.2f} s")
