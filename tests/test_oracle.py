"""The oracle (CPU restatement, oracle/cppe_oracle.cc) pinned against the
reference's golden vectors and against the reference's own engine."""
import os

import numpy as np
import pytest

from oracle import oracle as O

# (theta, order) columns of tests/ref_fmm_errors.csv; the reference's test
# (tests/test_fmm.py:34-59) checks theta in {0.5, 0.7, 0.99} x order {3, 5};
# the restatement reproduces every column of the file.
ALL_COLUMNS = [(t, o) for t in (0.2, 0.3, 0.5, 0.7, 0.99) for o in (3, 5, 7)]


def test_multipole_fields_direct_golden(port, loprop, fmuls_golden):
    # tests/test_fmm.py:14-25: MultipoleFields, default options, 8,805 sites
    F = port.multipole_fields(loprop)
    np.testing.assert_allclose(F, fmuls_golden, rtol=0, atol=1e-12)


@pytest.mark.parametrize("theta,order", ALL_COLUMNS)
def test_fmm_errors_golden(port, loprop, fmuls_golden, fmm_errors_golden, theta, order):
    # tests/test_fmm.py:26-59: per-site relative FMM error vs direct, atol 1e-8
    Ft = port.multipole_fields(loprop, fmm=True, theta=theta, order=order)
    fs = fmuls_golden.reshape(-1, 3)
    err = np.linalg.norm(fs - Ft.reshape(-1, 3), axis=1) / np.linalg.norm(fs, axis=1)
    np.testing.assert_allclose(fmm_errors_golden[f"err_F_{theta}_{order}"], err, atol=1e-8)


def test_pna_apply_and_solve(port, unpacked, golden_vectors):
    g = golden_vectors
    s = O.read_potfile(unpacked["pna_6w.pot"])
    np.testing.assert_allclose(port.multipole_fields(s), g["pna_mulfields"], atol=1e-14)
    for damp, tag in ((0.0, "plain"), (2.1304, "damped")):
        a = port.bmatrix_apply(s.xyz, s.alpha6, s.excl_ptr, s.excl_idx, g["pna_vec"],
                               damping=damp)
        np.testing.assert_allclose(a, g[f"pna_apply_{tag}"], atol=1e-12)
        mu, it, hist, ok = port.solve(s.xyz, s.alpha6, s.excl_ptr, s.excl_idx,
                                      g["pna_mulfields"], thresh=1e-12, damping=damp)
        assert ok
        np.testing.assert_allclose(mu, g[f"pna_mu_{tag}"], atol=1e-10)


def test_water120_fmm(port, golden_vectors):
    from cppe_gb300 import synthetic
    g = golden_vectors
    b = synthetic.water_box(120, seed=7)
    np.testing.assert_array_equal(b.xyz, g["w120_xyz"])
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32),
                    excl_ptr=b.excl_ptr, excl_idx=b.excl_idx)
    for fmm, tag in ((0, "direct"), (1, "fmm")):
        for dm, dtag in ((0.0, "plain"), (2.1304, "damped")):
            F = port.multipole_fields(sites, fmm=fmm, ncrit=16, order=5, theta=0.5, damping=dm)
            ref = g[f"w120_mulfields_{tag}_{dtag}"]
            np.testing.assert_allclose(F, ref, atol=1e-12 * np.abs(ref).max())
    for order in (5, 6):
        a = port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, g["w120_vec"], fmm=1,
                               ncrit=16, order=order, theta=0.5, damping=2.1304)
        ref = g[f"w120_apply_fmm_p{order}"]
        np.testing.assert_allclose(a, ref, atol=1e-12 * np.abs(ref).max())
    mu, it, hist, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, g["w120_rhs_fmm"],
                                  thresh=1e-10, fmm=1, ncrit=16, order=5, theta=0.5,
                                  damping=2.1304)
    assert ok
    np.testing.assert_allclose(mu, g["w120_mu_fmm"], atol=1e-9)


def test_config0_solve(port, golden_vectors):
    from cppe_gb300 import synthetic
    g = golden_vectors
    c0 = synthetic.water_box(333, seed=0)
    rhs = c0.external_field() + g["c0_mulfields"]
    mu, it, hist, ok = port.solve(c0.xyz, c0.alpha6, c0.excl_ptr, c0.excl_idx, rhs,
                                  thresh=1e-8, damping=2.1304)
    assert ok and it == int(g["c0_iters"][0])
    np.testing.assert_allclose(mu, g["c0_mu"], atol=1e-9)


def test_nonconvergence_reported(port, golden_vectors):
    from cppe_gb300 import synthetic
    c0 = synthetic.water_box(60, seed=3)
    rhs = c0.external_field()
    mu, it, hist, ok = port.solve(c0.xyz, c0.alpha6, c0.excl_ptr, c0.excl_idx, rhs,
                                  thresh=1e-30, maxiter=3, damping=2.1304)
    assert not ok and it == 3


@pytest.mark.skipif(not os.path.isdir(os.environ.get("CPPE_REFERENCE_DIR", "/root/reference")),
                    reason="reference sources not mounted")
def test_port_lists_equal_reference_build(loprop):
    assert O.build_ref()
    R = O.RefOracle()
    P = O.PortOracle()
    for ncrit in (16, 64):
        a = P.tree_lists(loprop.xyz, ncrit=ncrit, theta=0.5)
        b = R.tree_lists(loprop.xyz, ncrit=ncrit, theta=0.5)
        for k in ("cells", "parent", "level", "nchild", "nleaf", "leaves", "p2p"):
            np.testing.assert_array_equal(a[k], b[k])
        np.testing.assert_array_equal(np.sort(a["m2l"].view(np.int64).ravel()),
                                      np.sort(b["m2l"].view(np.int64).ravel()))
