"""GPU parity: the CUDA path (through the C ABI, and through the reference-
facing Python API) against the oracle and the reference's golden vectors.

Tolerances: FP64 kernels against the reference to 1e-12 absolute on applies
(the reference's own test uses 1e-12, tests/test_solver.py:67) and to the
reference test's solver tolerances; FP32 applies to 2e-6 relative; solves
to the 1e-8 residual rule with the polarization energy within 1e-7 Hartree.
"""
import numpy as np
import pytest

import cabi
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def T2(diff, v=0.0):
    """Damped dipole tensor T_ab = d_a d_b f_v(vR)/R (numpy, reference test style)."""
    r = np.linalg.norm(diff)
    fE = fT = 1.0
    if v > 0:
        x = v * r
        e = np.exp(-x)
        fE = 1 - (1 + x + x * x / 2) * e
        fT = fE - x ** 3 / 6 * e
    return 3 * fT * np.outer(diff, diff) / r ** 5 - fE * np.eye(3) / r ** 3


def dense_B(xyz, alpha6, excl_ptr, excl_idx, damping=0.0):
    n = xyz.shape[0]
    B = np.zeros((3 * n, 3 * n))
    iso = (alpha6[:, 0] + alpha6[:, 3] + alpha6[:, 5]) / 3
    for i in range(n):
        a = alpha6[i]
        A = np.array([[a[0], a[1], a[2]], [a[1], a[3], a[4]], [a[2], a[4], a[5]]])
        B[3 * i:3 * i + 3, 3 * i:3 * i + 3] = np.linalg.inv(A)
        ex = set(excl_idx[excl_ptr[i]:excl_ptr[i + 1]])
        for j in range(n):
            if j == i or j in ex:
                continue
            v = damping / (iso[i] * iso[j]) ** (1 / 6) if damping > 0 else 0.0
            B[3 * i:3 * i + 3, 3 * j:3 * j + 3] = -T2(xyz[j] - xyz[i], v)
    return B


@pytest.fixture(scope="module")
def pna(unpacked):
    return O.read_potfile(unpacked["pna_6w.pot"])


@pytest.mark.parametrize("tag,damp", [("plain", False), ("damped", True)])
def test_pna_apply_dense_inverse_solve(gpu, pna, golden_vectors, tag, damp):
    g = golden_vectors
    s = cabi.System(pna.xyz, pna.alpha6, pna.excl_ptr, pna.excl_idx, damp=damp, thresh=1e-12)
    np.testing.assert_allclose(s.apply(g["pna_vec"]), g[f"pna_apply_{tag}"], atol=1e-12)
    B = dense_B(pna.xyz, pna.alpha6, pna.excl_ptr, pna.excl_idx, 2.1304 if damp else 0.0)
    np.testing.assert_allclose(s.dense(), B, atol=1e-12)
    # apply to unit vectors rebuilds B (tests/test_solver.py:69-75)
    cols = np.stack([s.apply(e) for e in np.eye(3 * pna.n)], axis=1)
    np.testing.assert_allclose(cols, B, atol=1e-12)
    F = g["pna_mulfields"]
    mu_inv = np.linalg.solve(B, F)
    np.testing.assert_allclose(s.inverse() @ F, mu_inv, atol=1e-10)
    mu, it, hist, rc = s.solve(F)
    np.testing.assert_allclose(mu, mu_inv, atol=1e-10)
    np.testing.assert_allclose(mu, g[f"pna_mu_{tag}"], atol=1e-10)
    np.testing.assert_allclose(hist, g[f"pna_hist_{tag}"][: len(hist)], rtol=1e-6, atol=1e-13)
    assert len(hist) == len(g[f"pna_hist_{tag}"])
    v = g["pna_vec"]
    a6 = pna.alpha6
    am = np.array([[[a[0], a[1], a[2]], [a[1], a[3], a[4]], [a[2], a[4], a[5]]] for a in a6])
    np.testing.assert_allclose(s.apply_diagonal(v, inverse=True),
                               np.einsum("nij,nj->ni", am, v.reshape(-1, 3)).ravel(), atol=1e-14)
    np.testing.assert_allclose(s.apply_diagonal(v),
                               np.einsum("nij,nj->ni", np.linalg.inv(am), v.reshape(-1, 3)).ravel(),
                               atol=1e-12)


def test_config0_direct_solve(gpu, golden_vectors):
    from cppe_gb300 import synthetic
    g = golden_vectors
    c0 = synthetic.water_box(333, seed=0)
    s = cabi.System(c0.xyz, c0.alpha6, c0.excl_ptr, c0.excl_idx, damp=True)
    rhs = c0.external_field() + g["c0_mulfields"]
    mu, it, hist, rc = s.solve(rhs)
    assert it == int(g["c0_iters"][0])
    np.testing.assert_allclose(mu, g["c0_mu"], atol=1e-9)
    E = c0.external_field()
    assert abs(-0.5 * mu @ E - (-0.5 * g["c0_mu"] @ E)) < 1e-7
    # the reference's stopping rule, evaluated independently
    assert np.linalg.norm(rhs - s.apply(mu)) < 1e-8


def test_multipole_fields_direct_golden(gpu, loprop, fmuls_golden):
    s = loprop
    F = cabi.multipole_fields(s.xyz, s.q, s.mu, s.quad, 2, s.polarizable, s.alpha_iso,
                              s.excl_ptr, s.excl_idx)
    np.testing.assert_allclose(F, fmuls_golden, rtol=0, atol=1e-12)


@pytest.mark.parametrize("theta,order", [(0.5, 3), (0.5, 5), (0.7, 3), (0.7, 5), (0.99, 3),
                                         (0.99, 5), (0.2, 7), (0.3, 5)])
def test_multipole_fields_fmm_errors_golden(gpu, loprop, fmuls_golden, fmm_errors_golden,
                                            theta, order):
    s = loprop
    F = cabi.multipole_fields(s.xyz, s.q, s.mu, s.quad, 2, s.polarizable, s.alpha_iso,
                              s.excl_ptr, s.excl_idx, fmm=True, theta=theta, order=order)
    fs = fmuls_golden.reshape(-1, 3)
    err = np.linalg.norm(fs - F.reshape(-1, 3), axis=1) / np.linalg.norm(fs, axis=1)
    np.testing.assert_allclose(fmm_errors_golden[f"err_F_{theta}_{order}"], err, atol=1e-8)


def test_water120_fields_and_fmm_apply(gpu, golden_vectors):
    from cppe_gb300 import synthetic
    g = golden_vectors
    b = synthetic.water_box(120, seed=7)
    ones = np.ones(b.n, np.int32)
    for fmm, tag in ((0, "direct"), (1, "fmm")):
        for damp, dtag in ((False, "plain"), (True, "damped")):
            F = cabi.multipole_fields(b.xyz, b.q, b.mu, b.quad, 2, ones, b.alpha_iso,
                                      b.excl_ptr, b.excl_idx, fmm=bool(fmm), ncrit=16, order=5,
                                      damp=damp)
            ref = g[f"w120_mulfields_{tag}_{dtag}"]
            np.testing.assert_allclose(F, ref, atol=1e-12 * np.abs(ref).max())
    for order in (5, 6):
        s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, ncrit=16,
                        order=order, damp=True)
        ref = g[f"w120_apply_fmm_p{order}"]
        np.testing.assert_allclose(s.apply(g["w120_vec"]), ref, atol=1e-12 * np.abs(ref).max())
        a32 = s.apply(g["w120_vec"], fp32=True)
        assert np.abs(a32 - ref).max() < 2e-6 * np.abs(ref).max()
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, ncrit=16,
                    order=5, damp=True, thresh=1e-10)
    mu, it, hist, rc = s.solve(g["w120_rhs_fmm"])
    np.testing.assert_allclose(mu, g["w120_mu_fmm"], atol=1e-9)


@pytest.mark.parametrize("fmm", [False, True])
def test_mixed_precision_solve(gpu, port, fmm):
    from cppe_gb300 import synthetic
    b = synthetic.water_box(2000, seed=21)
    rhs = b.external_field() + port.multipole_fields(O.Sites(
        xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
        alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32), excl_ptr=b.excl_ptr,
        excl_idx=b.excl_idx), fmm=fmm)
    kw = dict(summation=cabi.FMM if fmm else cabi.DIRECT, damp=True)
    s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.FP64, **kw)
    smx = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED, **kw)
    mu64, it64, _, _ = s64.solve(rhs)
    mumx, itmx, hist, _ = smx.solve(rhs)
    st = smx.stats()
    # FP64 residual of the mixed solution with the FP64 operator
    assert np.linalg.norm(rhs - s64.apply(mumx)) < 1e-8
    assert st["rnorm"] < 1e-8 and st["fp32_applies"] > 0
    E = b.external_field()
    assert abs(0.5 * (mu64 - mumx) @ E) < 1e-7
    np.testing.assert_allclose(mumx, mu64, atol=1e-7)


@pytest.mark.parametrize("fmm,damp,order", [(False, True, 5), (True, True, 5),
                                            (True, False, 5), (True, True, 6)])
def test_double_float_apply_matches_fp64(gpu, fmm, damp, order):
    """The mixed solver's residual operator (double-float near field and M2L)
    equals the FP64 operator to FP64-level accuracy."""
    from cppe_gb300 import synthetic
    b = synthetic.water_box(1500, seed=31)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx,
                    summation=cabi.FMM if fmm else cabi.DIRECT, damp=damp, order=order)
    v = np.random.default_rng(5).normal(0, 0.1, size=3 * b.n)
    a64 = s.apply(v)
    add = s.apply(v, dd=True)
    a32 = s.apply(v, fp32=True)
    err_dd = np.linalg.norm(add - a64) / np.linalg.norm(a64)
    err_32 = np.linalg.norm(a32 - a64) / np.linalg.norm(a64)
    # DD pairs carry ~1e-13 relative error; sums with cancellation reach ~1e-12
    assert err_dd < 5e-12, err_dd
    assert err_dd < 1e-3 * err_32


@pytest.mark.parametrize("thresh", [1e-8, 1e-11])
def test_mixed_solve_meets_the_threshold(gpu, thresh):
    """The mixed solver's answer meets the threshold with the FP64 operator,
    both where its residuals come from the inner recursion (1e-8) and where
    the first inner solve leaves too large a residual for that, so that the
    solver recomputes them with the FP64 operator (1e-11)."""
    from cppe_gb300 import synthetic
    b = synthetic.water_box(2000, seed=33)
    kw = dict(summation=cabi.FMM, damp=True, thresh=thresh, maxiter=80)
    s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.FP64, **kw)
    smx = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED, **kw)
    rhs = b.external_field() + 0.05 * np.random.default_rng(7).normal(size=3 * b.n)
    mu, _, hist, rc = smx.solve(rhs)
    st = smx.stats()
    res = np.linalg.norm(rhs - s64.apply(mu))
    assert res < thresh, (res, hist)
    assert st["rnorm"] < thresh and abs(st["rnorm"] - res) < 0.1 * thresh
    if thresh < 1e-10:
        assert st["fp64_applies"] >= 2  # the residual was recomputed


def test_autotune_keeps_the_operator(gpu):
    """The schedule autotuner changes the work partition, not the operator."""
    from cppe_gb300 import synthetic
    b = synthetic.water_box(1500, seed=32)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, damp=True,
                    precision=cabi.MIXED)
    v = np.random.default_rng(6).normal(0, 0.1, size=3 * b.n)
    a64, a32 = s.apply(v), s.apply(v, fp32=True)
    ms = s.autotune(2)
    assert ms > 0
    b64, b32 = s.apply(v), s.apply(v, fp32=True)
    np.testing.assert_allclose(b64, a64, rtol=0, atol=1e-12 * np.abs(a64).max())
    np.testing.assert_allclose(b32, a32, rtol=0, atol=2e-6 * np.abs(a32).max())
    rhs = b.external_field()
    mu, it, _, _ = s.solve(rhs)
    assert np.linalg.norm(rhs - s.apply(mu)) < 1e-8


@pytest.mark.parametrize("fmm", [False, True])
def test_near_field_forms_give_the_operator(gpu, fmm):
    """The FP32 near field per target leaf and in both symmetric forms (two
    and four sources a lane), at two work-item sizes: the same operator to
    FP32 accuracy, and the mixed solve meets the threshold with each."""
    from cppe_gb300 import synthetic
    b = synthetic.water_box(1700, seed=35)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED,
                    summation=cabi.FMM if fmm else cabi.DIRECT, damp=True)
    v = np.random.default_rng(8).normal(0, 0.1, size=3 * b.n)
    a64 = s.apply(v)
    scale = np.abs(a64).max()
    rhs = b.external_field()
    for form in (0, 1, 2):
        for pairs in (4096, 65536):
            s.set_schedule(form, pairs)
            sched = s.schedule()
            assert sched["sym_pack"] == form or (form > 0 and not sched["symmetric_near"])
            np.testing.assert_allclose(s.apply(v, fp32=True), a64, rtol=0, atol=2e-6 * scale,
                                       err_msg=f"form {form}, {pairs} pairs")
        mu, _, _, _ = s.solve(rhs)
        assert np.linalg.norm(rhs - s.apply(mu)) < 1e-8, f"form {form}"
    s.close()


def test_fmm_solve_matches_oracle(gpu, port):
    from cppe_gb300 import synthetic
    b = synthetic.water_box(1500, seed=4)
    rhs = b.external_field()
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, damp=True)
    mu, it, hist, rc = s.solve(rhs)
    mu_o, it_o, hist_o, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, fmm=1,
                                        damping=2.1304)
    assert ok and it == it_o
    np.testing.assert_allclose(mu, mu_o, atol=1e-9)
    v = np.random.default_rng(1).normal(size=3 * b.n)
    a = s.apply(v)
    ao = port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, fmm=1, damping=2.1304)
    np.testing.assert_allclose(a, ao, atol=1e-12 * np.abs(ao).max())


def test_not_converged_status(gpu):
    from cppe_gb300 import synthetic
    b = synthetic.water_box(50, seed=2)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, damp=True, thresh=1e-30, maxiter=4)
    mu, it, hist, rc = s.solve(b.external_field(), allow_not_converged=True)
    assert rc == cabi.NOT_CONVERGED and it == 4
    assert "Failed to converge" in cabi.last_error()


# --- the reference-facing Python API on the GPU ------------------------------
def test_python_api_state_and_solver(gpu, unpacked, golden_vectors):
    import cppe_gb300 as cppe
    g = golden_vectors
    lines = []
    pots = cppe.PotfileReader(unpacked["pna_6w.pot"]).read()
    polsites = cppe.get_polarizable_sites(pots)
    opts = {"induced_thresh": 1e-12}
    F = cppe.MultipoleFields(pots, opts).compute()
    np.testing.assert_allclose(F, g["pna_mulfields"], atol=1e-14)
    bm = cppe.BMatrix(polsites, opts)
    np.testing.assert_allclose(bm.apply(g["pna_vec"]), g["pna_apply_plain"], atol=1e-12)
    ind = cppe.InducedMoments(pots, opts)
    ind.set_print_callback(lines.append)
    mu = ind.compute(F, True)
    np.testing.assert_allclose(mu, g["pna_mu_plain"], atol=1e-10)
    assert lines[0].startswith("0 --- Norm: ") and len(lines) == len(g["pna_hist_plain"])
    state = cppe.CppeState({"potfile": unpacked["pna_6w.pot"], "induced_thresh": 1e-12},
                           cppe.Molecule(), lambda s: None)
    state.calculate_static_energies_and_fields()
    np.testing.assert_allclose(state.static_fields, g["pna_mulfields"], atol=1e-14)
    state.update_induced_moments(np.zeros(54), False)
    np.testing.assert_allclose(state.get_induced_moments(), g["pna_mu_plain"], atol=1e-10)
    epol = state.energies["Polarization"]["Multipoles"]
    assert abs(epol - (-0.5 * g["pna_mu_plain"] @ g["pna_mulfields"])) < 1e-12
    eef = state.induced_moments_eef()
    assert eef.shape == (54, 3)
    # CppeState::induced_moments_eef (cppe_state.cc:111-128): three solves
    # for unit fields along x, y, z at every polarizable site
    from oracle import oracle as O
    sites = O.read_potfile(unpacked["pna_6w.pot"])
    pol = np.flatnonzero(sites.polarizable)
    assert len(pol) == 18
    port = O.PortOracle()
    for a in range(3):
        f = np.zeros(54)
        f[a::3] = 1.0
        mu_o, _, _, ok = port.solve(sites.xyz[pol], sites.alpha6[pol], sites.excl_ptr,
                                    sites.excl_idx, f, thresh=1e-12)
        assert ok
        np.testing.assert_allclose(eef[:, a], mu_o, atol=1e-10)
    # warm start: a second call converges immediately from the previous moments
    state.update_induced_moments(np.zeros(54), False)
    np.testing.assert_allclose(state.get_induced_moments(), g["pna_mu_plain"], atol=1e-10)


def test_python_api_nuclear_fields_and_energy(gpu, unpacked):
    import cppe_gb300 as cppe
    pots = cppe.PotfileReader(unpacked["pna_6w.pot"]).read()
    mol = cppe.Molecule()
    rng = np.random.default_rng(3)
    atoms = [(6, *rng.uniform(10, 20, 3)), (1, *rng.uniform(10, 20, 3))]
    for a in atoms:
        mol.append(cppe.Atom(*a))
    nf = cppe.NuclearFields(mol, pots).compute()
    ref = np.zeros((18, 3))
    for i, p in enumerate(pots):
        for a in atoms:
            d = p.position - np.array(a[1:])
            ref[i] += a[0] * d / np.linalg.norm(d) ** 3
    np.testing.assert_allclose(nf, ref.ravel(), atol=1e-14)
    e = cppe.MultipoleExpansion(mol, pots).interaction_energy()
    eref = 0.0
    for p in pots:
        for a in atoms:
            d = np.array(a[1:]) - p.position
            r = np.linalg.norm(d)
            q = p.multipoles[0].values[0]
            mu = p.multipoles[1].values
            Q = p.multipoles[2].values
            Qm = np.array([[Q[0], Q[1], Q[2]], [Q[1], Q[3], Q[4]], [Q[2], Q[4], Q[5]]])
            T2m = 3 * np.outer(d, d) / r ** 5 - np.eye(3) / r ** 3
            eref += a[0] * (q / r + mu @ d / r ** 3 + 0.5 * np.sum(Qm * T2m))
    assert abs(e - eref) < 1e-10
