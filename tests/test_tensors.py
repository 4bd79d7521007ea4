"""The tensors submodule (src/python_iface/export_tensors.cc:17-40): Cartesian
derivative tensors of 1/R and of the Thole-damped potential, host-side
utilities (no GPU).  Checked against closed forms (T1, T2, the Thole
screening factors of tensors_recursive.cc:93-114), central finite differences
between consecutive orders, the component order of xyz2idx, and the
reference's refusal of damped tensors above third order."""
import numpy as np
import pytest

R = np.array([1.3, -0.7, 2.1])


@pytest.fixture(scope="module")
def cppe():
    import cppe_gb300
    return cppe_gb300


def test_closed_forms(cppe):
    r = np.linalg.norm(R)
    iu = np.triu_indices(3)
    np.testing.assert_allclose(cppe.tensors.T0(R), [1 / r], rtol=1e-15)
    np.testing.assert_allclose(cppe.tensors.T1(R), -R / r ** 3, rtol=1e-14)
    T2 = 3 * np.outer(R, R) / r ** 5 - np.eye(3) / r ** 3
    np.testing.assert_allclose(cppe.T_recursive(2, R), T2[iu], rtol=1e-13, atol=1e-16)
    a = 0.9
    v = a * r
    e = np.exp(-v)
    fv = 1 - (1 + v / 2) * e
    fE = 1 - (1 + v + v * v / 2) * e
    fT = fE - v ** 3 / 6 * e
    np.testing.assert_allclose(cppe.T_recursive(0, R, a), [fv / r], rtol=1e-14)
    np.testing.assert_allclose(cppe.T_recursive(1, R, a), -fE * R / r ** 3, rtol=1e-13)
    T2d = 3 * fT * np.outer(R, R) / r ** 5 - fE * np.eye(3) / r ** 3
    np.testing.assert_allclose(cppe.T_recursive(2, R, a), T2d[iu], rtol=1e-13, atol=1e-16)
    np.testing.assert_allclose(cppe.tensors.T2_damp_thole(R, a), T2d[iu], rtol=1e-13,
                               atol=1e-16)


def _components(k):
    return [(x, y, k - x - y) for x in range(k, -1, -1) for y in range(k - x, -1, -1)]


@pytest.mark.parametrize("damped", [False, True])
def test_consecutive_orders_by_finite_differences(cppe, damped):
    a, h = 0.9, 1e-5
    f = (lambda k, x: cppe.T_damp_thole[k](x, a)) if damped else (lambda k, x: cppe.T[k](x))
    for k in range(6):
        low = _components(k)
        got, want = [], f(k + 1, R)
        for (x, y, z) in _components(k + 1):
            ax = 0 if x else (1 if y else 2)
            c = [x, y, z]
            c[ax] -= 1
            d = np.zeros(3)
            d[ax] = h
            i = low.index(tuple(c))
            got.append((f(k, R + d)[i] - f(k, R - d)[i]) / (2 * h))
        np.testing.assert_allclose(got, want, rtol=0, atol=2e-9 * np.abs(want).max())


def test_xyz2idx_and_sizes(cppe):
    for k in range(7):
        for i, c in enumerate(_components(k)):
            assert cppe.xyz2idx(*c) == i
        assert len(cppe.tensors.T[k](R)) == (k + 1) * (k + 2) // 2
        assert len(cppe.T_recursive(k, R)) == (k + 1) * (k + 2) // 2


def test_damped_recursive_limited_to_third_order(cppe):
    cppe.T_recursive(3, R, 0.5)
    with pytest.raises(RuntimeError, match="third order"):
        cppe.T_recursive(4, R, 0.5)
    assert hasattr(cppe.fmm, "Tree")
