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


def test_batch_autotune_keeps_the_solution(gpu):
    boxes = _snapshots()
    nrhs = 2
    rhs = _rhs(boxes, nrhs, seed=1)
    batch = cabi.Batch(boxes, nrhs, direct_below=1000, damp=True, precision=cabi.FP64)
    mu1, its1 = batch.solve(rhs)
    ms = batch.autotune(2)
    assert ms > 0.0
    mu2, its2 = batch.solve(rhs)
    # only the partition of the work into launches changed
    np.testing.assert_array_equal(its1, its2)
    np.testing.assert_allclose(mu2, mu1, rtol=0, atol=1e-10)


def test_batch_autotune_mixed_keeps_the_solution(gpu):
    """In mixed precision the tuner also picks the multi-RHS near field's tile
    size (96, 120 or 144 source pairs): the FP32 sums are reordered, the
    answer still meets the same FP64 stopping rule."""
    boxes = _snapshots()
    nrhs = 2
    rhs = _rhs(boxes, nrhs, seed=3)
    batch = cabi.Batch(boxes, nrhs, direct_below=1000, damp=True, precision=cabi.MIXED)
    mu1, _ = batch.solve(rhs)
    assert batch.autotune(2) > 0.0
    mu2, _ = batch.solve(rhs)
    assert batch.stats()["max_rnorm"] < 1e-8
    np.testing.assert_allclose(mu2, mu1, rtol=0, atol=5e-8)


_HOST_LOOP = r"""
import os, sys, numpy as np
sys.path[:0] = [sys.argv[1], os.path.dirname(sys.argv[1])]
import cabi
from test_gpu_batch import _snapshots, _rhs
boxes = _snapshots()
b = cabi.Batch(boxes, 2, direct_below=1000, damp=True, precision=int(sys.argv[3]))
mu, its = b.solve(_rhs(boxes, 2, seed=2))
np.savez(sys.argv[2], mu=mu, its=its)
"""


@pytest.mark.parametrize("precision", [cabi.FP64, cabi.MIXED])
def test_batch_graph_loop_matches_host_loop(gpu, precision, tmp_path):
    """The device-side loop (conditional graph node) takes the same steps as
    the host-launched iterations (CPPE_GPU_GRAPHS=0, a separate process)."""
    import os
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    out = str(tmp_path / "host.npz")
    env = dict(os.environ, CPPE_GPU_GRAPHS="0")
    subprocess.run([sys.executable, "-c", _HOST_LOOP, here, out, str(precision)], env=env,
                   check=True, timeout=600)
    host = np.load(out)
    boxes = _snapshots()
    b = cabi.Batch(boxes, 2, direct_below=1000, damp=True, precision=precision)
    mu, its = b.solve(_rhs(boxes, 2, seed=2))
    np.testing.assert_array_equal(its, host["its"])
    np.testing.assert_allclose(mu, host["mu"], rtol=0, atol=1e-12)
    if precision == cabi.MIXED:
        # the mixed solve ran its usual course as one graph launch: one wait
        # for its results and one for the copy-out
        assert b.stats()["host_waits"] == 2


def test_batch_course_hands_over_to_the_host_loop(gpu):
    """Inner solves capped at five iterations: the one-launch course of a
    mixed solve ends short of the threshold and the host loop takes further
    outer iterations; every segment still meets the reference's stopping
    rule with its own FP64 operator."""
    boxes = _snapshots()[:3]
    nrhs = 2
    rhs = _rhs(boxes, nrhs, seed=4)
    batch = cabi.Batch(boxes, nrhs, direct_below=1000, damp=True, precision=cabi.MIXED,
                       maxiter=5)
    mu, _ = batch.solve(rhs)
    assert batch.stats()["host_waits"] > 2
    off = 0
    for b in boxes:
        summ = cabi.FMM if b.n >= 1000 else cabi.DIRECT
        s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=summ, damp=True)
        for r in range(nrhs):
            seg = slice(off, off + 3 * b.n)
            assert np.linalg.norm(rhs[seg] - s64.apply(mu[seg])) < 1e-8
            off += 3 * b.n
        s64.close()
    batch.close()


def test_batch_mixed_direct_snapshots_in_one_launch(gpu):
    """A mixed batch of direct-summation snapshots only (no inexact
    operators): its course runs as one graph launch too, and every segment
    meets the reference's stopping rule with its own FP64 operator."""
    boxes = _snapshots()[:3]
    nrhs = 2
    rhs = _rhs(boxes, nrhs, seed=5)
    batch = cabi.Batch(boxes, nrhs, direct_below=10**6, damp=True, precision=cabi.MIXED)
    mu, _ = batch.solve(rhs)
    assert batch.stats()["host_waits"] == 2
    off = 0
    for b in boxes:
        s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.DIRECT,
                          damp=True)
        for r in range(nrhs):
            seg = slice(off, off + 3 * b.n)
            assert np.linalg.norm(rhs[seg] - s64.apply(mu[seg])) < 1e-8
            off += 3 * b.n
        s64.close()
    batch.close()


def test_batch_more_rhs_than_one_pass(gpu):
    """Ten right-hand sides per snapshot: the near-field passes take a
    snapshot's copies eight at a time; every segment still meets the
    reference's stopping rule with its own FP64 operator."""
    boxes = _snapshots()[:2]  # 300 sites (direct) and 900 sites (FMM)
    nrhs = 10
    rhs = _rhs(boxes, nrhs, seed=3)
    batch = cabi.Batch(boxes, nrhs, direct_below=500, damp=True, precision=cabi.MIXED)
    mu, its = batch.solve(rhs)
    assert its.shape == (len(boxes) * nrhs,)
    off = 0
    for b in boxes:
        summ = cabi.FMM if b.n >= 500 else cabi.DIRECT
        s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=summ, damp=True)
        for r in range(nrhs):
            seg = slice(off, off + 3 * b.n)
            assert np.linalg.norm(rhs[seg] - s64.apply(mu[seg])) < 1e-8
            off += 3 * b.n
    assert off == rhs.size
