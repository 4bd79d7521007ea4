"""GPU parity at the benchmark's system sizes, against the oracle and the
reference engine.

* 30,000 sites, FMM order 5 (theta 0.5, ncrit 64): the static fields, one FP64
  FMM apply and the full FP64 PCG against the oracle port (1e-12 relative on
  applies, same iteration count, mu to 1e-9), the mixed solve by the oracle's
  own residual rule, and both solves against the reference engine's committed
  solution summary.
* 300,000 sites, FMM order 6: FP64, double-float and FP32 applies against the
  oracle's apply, and the mixed solve by the oracle's residual rule and the
  reference summary.
* the batch: two snapshots of the batch generator (direct summation below
  4,000 sites, FMM order 5 above), two right-hand sides each, solved as one
  batch in FP64 and in mixed precision, against full oracle solves.
* 1,000,002 sites, FMM order 6: the mixed solve with the shipped model, by the
  oracle's residual rule and against the reference summary; and, at that
  size, bitwise-repeatable solves and FP32 applies and the double-float
  operator's linearity (5e-12 in norm).

The reference summaries (tests/golden/config_solutions.json) hold the
reference engine's solutions of the same seeded boxes (energy, mu and F at 64
seeded sites and over 64 site blocks), made by
tests/golden/make_config_solutions.py.

Tolerances: applies 1e-12 (FP64) and 2e-6 (FP32) relative to the largest
entry, the double-float apply 5e-12 in norm (2e-11 of the largest entry); solves to the reference's rule
||F - B mu||_2 < 1e-8 with the oracle's FP64 operator, the polarization energy
-1/2 mu.F within 1e-7 Hartree of the reference's, and mu within 1e-9 (FP64
against the oracle's iterates) or 5e-8 (mixed against the reference's answer).
"""
import json
import os

import numpy as np
import pytest

import cabi

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
MODEL = os.path.join(os.path.dirname(HERE), "cppe_gb300", "data", "learned_water.npz")
DAMPING = 2.1304


def summary(name):
    with open(os.path.join(HERE, "golden", "config_solutions.json")) as f:
        return json.load(f)[name]


def box(name):
    from cppe_gb300 import synthetic
    g = summary(name)
    return synthetic.water_box(g["waters"], seed=g["seed"]), g


def gpu_rhs(b, order):
    F = cabi.multipole_fields(b.xyz, b.q, b.mu, b.quad, 2, np.ones(b.n, np.int32), b.alpha_iso,
                              b.excl_ptr, b.excl_idx, fmm=True, ncrit=64, order=order)
    return b.external_field() + F


def check_against_summary(g, rhs, mu, mu_tol):
    idx = np.asarray(g["sample_sites"])
    f3, m3 = rhs.reshape(-1, 3), mu.reshape(-1, 3)
    fs = np.asarray(g["F_samples"])
    assert np.abs(f3[idx] - fs).max() < 1e-11 * max(1.0, np.abs(fs).max()), "static fields"
    assert abs(-0.5 * mu @ rhs - g["epol"]) < 1e-7, "polarization energy"
    assert np.abs(m3[idx] - np.asarray(g["mu_samples"])).max() < mu_tol, "mu at sampled sites"
    edges = np.linspace(0, g["sites"], len(g["mu_block_sums"]) + 1).astype(np.int64)
    blocks = np.array([m3[a:c].sum(axis=0) for a, c in zip(edges[:-1], edges[1:])])
    assert np.abs(blocks - np.asarray(g["mu_block_sums"])).max() < 1e3 * mu_tol, "mu blocks"


def check_applies(s, v, ref):
    """FP64 apply to 1e-12 of the largest entry; the double-float apply to
    5e-12 in norm (its stated accuracy) and 2e-11 of the largest entry; FP32
    to 2e-6 of the largest entry."""
    scale = np.abs(ref).max()
    assert np.abs(s.apply(v) - ref).max() < 1e-12 * scale
    add = s.apply(v, dd=True)
    assert np.linalg.norm(add - ref) < 5e-12 * np.linalg.norm(ref)
    assert np.abs(add - ref).max() < 2e-11 * scale
    assert np.abs(s.apply(v, fp32=True) - ref).max() < 2e-6 * scale


def oracle_residual(port, b, rhs, mu, order, fmm=True):
    Bmu = port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, mu, fmm=int(fmm),
                             ncrit=64, order=order, theta=0.5, damping=DAMPING)
    return np.linalg.norm(rhs - Bmu)


def test_config_30k_fields_apply_and_solves(gpu, port):
    from oracle import oracle as O
    b, g = box("30k")
    rhs = gpu_rhs(b, 5)
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32), excl_ptr=b.excl_ptr,
                    excl_idx=b.excl_idx)
    rhs_o = b.external_field() + port.multipole_fields(sites, fmm=True, order=5)
    np.testing.assert_allclose(rhs, rhs_o, rtol=0, atol=1e-12 * np.abs(rhs_o).max())

    kw = dict(summation=cabi.FMM, order=5, ncrit=64, theta=0.5, damp=True, thresh=1e-8)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, **kw)
    v = np.random.default_rng(11).normal(size=3 * b.n)
    ref = port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, fmm=1, ncrit=64,
                             order=5, theta=0.5, damping=DAMPING)
    check_applies(s, v, ref)

    mu, it, hist, rc = s.solve(rhs)
    mu_o, it_o, hist_o, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs,
                                        fmm=1, ncrit=64, order=5, theta=0.5, damping=DAMPING)
    assert ok and it == it_o == g["iterations"]
    np.testing.assert_allclose(mu, mu_o, rtol=0, atol=1e-9)
    np.testing.assert_allclose(hist, hist_o, rtol=1e-6)
    check_against_summary(g, rhs, mu, 1e-9)
    s.close()

    smx = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED, **kw)
    mu_mx, _, _, _ = smx.solve(rhs)
    assert oracle_residual(port, b, rhs, mu_mx, 5) < 1e-8
    assert abs(0.5 * (mu_mx - mu_o) @ rhs) < 1e-7
    check_against_summary(g, rhs, mu_mx, 5e-8)
    smx.close()


def test_config_300k_applies_and_mixed_solve(gpu, port):
    b, g = box("300k")
    kw = dict(summation=cabi.FMM, order=6, ncrit=64, theta=0.5, damp=True, thresh=1e-8)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED, **kw)
    v = np.random.default_rng(12).normal(size=3 * b.n)
    ref = port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, fmm=1, ncrit=64,
                             order=6, theta=0.5, damping=DAMPING)
    check_applies(s, v, ref)
    rhs = gpu_rhs(b, 6)
    mu, _, _, _ = s.solve(rhs)
    assert oracle_residual(port, b, rhs, mu, 6) < 1e-8
    check_against_summary(g, rhs, mu, 5e-8)
    s.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_config_batch_snapshots_match_oracle(gpu, port, precision):
    from cppe_gb300 import learned, synthetic
    sizes = synthetic.snapshot_sizes(256, seed=1000)
    i_dir = next(i for i, n in enumerate(sizes) if n < 4000)
    i_fmm = next(i for i, n in enumerate(sizes) if n >= 4000)
    boxes = [synthetic.water_box(int(sizes[i]) // 3, seed=1000 + i) for i in (i_dir, i_fmm)]
    nrhs = 2
    rhs = [learned.generator_rhs(b, nrhs, 5000 + i) for i, b in zip((i_dir, i_fmm), boxes)]
    prec = cabi.FP64 if precision == "fp64" else cabi.MIXED
    batch = cabi.Batch(boxes, nrhs, direct_below=4000, precision=prec, damp=True, order=5,
                       ncrit=64, theta=0.5, thresh=1e-8)
    mu_all, _ = batch.solve(np.concatenate([np.concatenate(r) for r in rhs]))
    off = 0
    for b, rr in zip(boxes, rhs):
        fmm = b.n >= 4000
        for r in rr:
            mu = mu_all[off:off + 3 * b.n]
            off += 3 * b.n
            mu_o, it_o, _, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, r,
                                           fmm=int(fmm), ncrit=64, order=5, theta=0.5,
                                           damping=DAMPING)
            assert ok
            assert oracle_residual(port, b, r, mu, 5, fmm) < 1e-8
            assert abs(0.5 * (mu - mu_o) @ r) < 1e-7
            np.testing.assert_allclose(mu, mu_o, rtol=0,
                                       atol=1e-9 if precision == "fp64" else 5e-8)
    batch.close()


def test_config_1m_mixed_learned_solve(gpu, port):
    from cppe_gb300 import learned
    b, g = box("1m")
    kw = dict(summation=cabi.FMM, order=6, ncrit=64, theta=0.5, damp=True, thresh=1e-8)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=cabi.MIXED, **kw)
    s.set_model(learned.load(MODEL))
    rhs = gpu_rhs(b, 6)
    mu, _, _, _ = s.solve(rhs)
    assert np.linalg.norm(rhs - s.apply(mu)) < 1e-8  # the library's FP64 operator
    assert oracle_residual(port, b, rhs, mu, 6) < 1e-8  # the oracle's
    check_against_summary(g, rhs, mu, 5e-8)
    # size-independent properties at full size: a repeated solve gives the
    # same bits (no atomics in any reduction), and the double-float operator
    # is linear to its accuracy
    mu2, _, _, _ = s.solve(rhs)
    assert np.array_equal(mu, mu2)
    v = np.random.default_rng(13).normal(size=3 * b.n)
    a1, a2 = s.apply(mu, dd=True), s.apply(v, dd=True)
    a12 = s.apply(mu + 0.5 * v, dd=True)
    assert np.linalg.norm(a12 - (a1 + 0.5 * a2)) < 5e-12 * np.linalg.norm(a12)
    assert np.array_equal(s.apply(v, fp32=True), s.apply(v, fp32=True))
    s.set_model(None)
    s.close()
