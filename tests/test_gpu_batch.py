"""Batched solves (many snapshots x right-hand sides in one set of launches)
against one-at-a-time solves of the same segments."""
import numpy as np
import pytest

import cabi

pytestmark = pytest.mark.gpu


def _snapshots():
    from cppe_gb300 import synthetic
    sizes = [100, 300, 500, 800, 200]  # waters: 300 .. 2,400 sites
    return [synthetic.water_box(nw, seed=100 + k) for k, nw in enumerate(sizes)]


def _rhs(boxes, nrhs, seed=0):
    from cppe_gb300 import synthetic
    rng = np.random.default_rng(seed)
    out = []
    for b in boxes:
        for r in range(nrhs):
            c = b.xyz.mean(axis=0) + rng.uniform(-4, 4, size=(12, 3))
            q = rng.normal(0, 0.5, size=12)
            out.append(synthetic.point_charge_field(b.xyz, c, q))
    return np.concatenate(out)


@pytest.mark.parametrize("precision", [cabi.FP64, cabi.MIXED])
def test_batch_matches_individual_solves(gpu, precision):
    boxes = _snapshots()
    nrhs = 3
    rhs = _rhs(boxes, nrhs)
    batch = cabi.Batch(boxes, nrhs, direct_below=1000, damp=True, precision=precision)
    mu, its = batch.solve(rhs)
    st = batch.stats()
    assert st["fp64_applies"] >= 1
    if precision == cabi.MIXED:
        assert st["fp32_applies"] > st["fp64_applies"]
    off = 0
    for bi, b in enumerate(boxes):
        summ = cabi.FMM if b.n >= 1000 else cabi.DIRECT
        s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=summ, damp=True)
        for r in range(nrhs):
            seg = slice(off, off + 3 * b.n)
            ref, it, _, _ = s64.solve(rhs[seg])
            # the reference's rule, evaluated with the FP64 operator of this segment
            assert np.linalg.norm(rhs[seg] - s64.apply(mu[seg])) < 1e-8
            np.testing.assert_allclose(mu[seg], ref, atol=5e-8 if precision == cabi.MIXED else 1e-9)
            if precision == cabi.FP64:
                assert its[bi * nrhs + r] == it
            off += 3 * b.n
    assert off == rhs.size
