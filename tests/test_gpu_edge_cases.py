"""Edge cases of the operator and the solver on the GPU, against the oracle.

* One leaf: a 45-site system (fewer sites than ncrit) has no far field, so
  the FMM operator is the direct one; FMM and direct applies and solves
  against the oracle's direct ones.
* A dimer: two polarizable sites with anisotropic polarizabilities and one
  damped pair, in every arithmetic (FP64, double-float, FP32, mixed solve).
* Ragged exclusion lists: 48 sites (16 whole molecules) of a 900-site box
  exclude each other, so their lists hold 47 entries against 2 for the
  others (src/core/bmatrix.cc:9-40 skips excluded pairs).
* A masked static field: every second site non-polarizable; fields are
  computed at polarizable sites only (electric_fields.cc:106-189).
* A zero right-hand side: the reference's PCG (electric_fields.cc:191-239)
  forms alpha = (r.z) / (p.Ap) = 0 / 0 on its first iteration and reports
  that it did not converge; the FP64 solver behaves the same way.

Tolerances as in the other parity tests: FP64 1e-12 of the largest entry,
double-float 5e-12 in norm, FP32 2e-6 of the largest entry, solves to the
reference's residual rule with the oracle's operator.
"""
import numpy as np
import pytest

import cabi

pytestmark = pytest.mark.gpu

DAMPING = 2.1304


def _box(nw, seed):
    from cppe_gb300 import synthetic
    return synthetic.water_box(nw, seed=seed)


def _check_applies(s, ref_apply, v, fp32=True):
    ref = ref_apply(v)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(s.apply(v), ref, rtol=0, atol=1e-12 * scale)
    add = s.apply(v, dd=True)
    assert np.linalg.norm(add - ref) < 5e-12 * np.linalg.norm(ref)
    if fp32:
        np.testing.assert_allclose(s.apply(v, fp32=True), ref, rtol=0, atol=2e-6 * scale)


@pytest.mark.parametrize("fmm", [False, True])
def test_one_leaf_system(gpu, port, fmm):
    b = _box(15, 41)
    assert b.n < 64
    kw = dict(summation=cabi.FMM if fmm else cabi.DIRECT, damp=True, ncrit=64, order=5)
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, **kw)
    v = np.random.default_rng(1).normal(size=3 * b.n)
    _check_applies(s, lambda x: port.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, x,
                                                   fmm=False, damping=DAMPING), v)
    rhs = b.external_field()
    mu, it, _, _ = s.solve(rhs)
    mu_o, it_o, _, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, fmm=False,
                                   damping=DAMPING)
    assert ok and it == it_o
    np.testing.assert_allclose(mu, mu_o, rtol=0, atol=1e-10)
    s.close()


@pytest.mark.parametrize("fmm", [False, True])
def test_dimer(gpu, port, fmm):
    xyz = np.array([[0.0, 0.0, 0.0], [1.1, -2.3, 1.7]])
    alpha6 = np.array([[5.1, 0.3, -0.2, 4.4, 0.1, 6.0],
                       [2.2, -0.1, 0.05, 2.6, 0.2, 2.0]])
    ep, ei = np.zeros(3, np.int32), np.zeros(0, np.int32)
    kw = dict(summation=cabi.FMM if fmm else cabi.DIRECT, damp=True)
    s = cabi.System(xyz, alpha6, ep, ei, precision=cabi.MIXED, **kw)
    v = np.random.default_rng(2).normal(size=6)
    _check_applies(s, lambda x: port.bmatrix_apply(xyz, alpha6, ep, ei, x, fmm=False,
                                                   damping=DAMPING), v)
    rhs = np.array([0.01, -0.02, 0.005, 0.03, 0.01, -0.01])
    mu_o, it_o, _, ok = port.solve(xyz, alpha6, ep, ei, rhs, fmm=False, damping=DAMPING)
    assert ok
    mu, _, _, _ = s.solve(rhs)
    Bmu = port.bmatrix_apply(xyz, alpha6, ep, ei, mu, fmm=False, damping=DAMPING)
    assert np.linalg.norm(rhs - Bmu) < 1e-8
    np.testing.assert_allclose(mu, mu_o, rtol=0, atol=5e-8)
    s.close()
    s64 = cabi.System(xyz, alpha6, ep, ei, **kw)
    mu64, it64, _, _ = s64.solve(rhs)
    assert it64 == it_o
    np.testing.assert_allclose(mu64, mu_o, rtol=0, atol=1e-12)
    s64.close()


def _grouped_exclusions(b, group):
    """CSR exclusions where the sites of `group` exclude each other and the
    other sites keep their molecule's."""
    g = set(group)
    ptr, idx = [0], []
    for i in range(b.n):
        if i in g:
            mine = [j for j in group if j != i]
        else:
            mine = list(b.excl_idx[b.excl_ptr[i]:b.excl_ptr[i + 1]])
        idx.extend(sorted(mine))
        ptr.append(len(idx))
    return np.array(ptr, np.int32), np.array(idx, np.int32)


@pytest.mark.parametrize("fmm", [False, True])
def test_ragged_exclusion_lists(gpu, port, fmm):
    b = _box(300, 42)
    ep, ei = _grouped_exclusions(b, list(range(48)))
    lens = np.diff(ep)
    assert lens.max() == 47 and lens.min() == 2
    kw = dict(summation=cabi.FMM if fmm else cabi.DIRECT, damp=True, ncrit=64, order=5)
    s = cabi.System(b.xyz, b.alpha6, ep, ei, precision=cabi.MIXED, **kw)
    v = np.random.default_rng(3).normal(size=3 * b.n)
    _check_applies(s, lambda x: port.bmatrix_apply(b.xyz, b.alpha6, ep, ei, x, fmm=fmm,
                                                   damping=DAMPING), v)
    rhs = b.external_field()
    mu, _, _, _ = s.solve(rhs)
    mu_o, _, _, ok = port.solve(b.xyz, b.alpha6, ep, ei, rhs, fmm=fmm, damping=DAMPING)
    assert ok
    Bmu = port.bmatrix_apply(b.xyz, b.alpha6, ep, ei, mu, fmm=fmm, damping=DAMPING)
    assert np.linalg.norm(rhs - Bmu) < 1e-8
    np.testing.assert_allclose(mu, mu_o, rtol=0, atol=5e-8)
    s.close()


@pytest.mark.parametrize("fmm", [False, True])
def test_masked_multipole_fields(gpu, port, fmm):
    from oracle import oracle as O
    b = _box(200, 43)
    mask = (np.arange(b.n) % 2).astype(np.int32)
    F = cabi.multipole_fields(b.xyz, b.q, b.mu, b.quad, 2, mask, b.alpha_iso, b.excl_ptr,
                              b.excl_idx, fmm=fmm, order=5)
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=mask, excl_ptr=b.excl_ptr,
                    excl_idx=b.excl_idx)
    F_o = port.multipole_fields(sites, fmm=fmm, order=5)
    np.testing.assert_allclose(F, F_o, rtol=0, atol=1e-12 * np.abs(F_o).max())


def test_zero_rhs_does_not_converge_like_the_reference(gpu, port):
    b = _box(30, 44)
    rhs = np.zeros(3 * b.n)
    _, _, _, ok = port.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, fmm=False,
                             damping=DAMPING)
    assert not ok
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.DIRECT, damp=True)
    _, _, _, rc = s.solve(rhs, allow_not_converged=True)
    assert rc == cabi.NOT_CONVERGED
    s.close()
