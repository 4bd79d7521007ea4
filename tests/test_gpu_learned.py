"""The learned initial guess / preconditioner correction on the GPU.

* its training kernels (forward, loss, backward) against the numpy oracle
  (oracle/mlp_oracle.py) on real descriptor rows;
* training lowers the loss;
* on held-out systems the trained network converges to the same answer (the
  unchanged 1e-8 FP64 stopping rule) in fewer PCG iterations than plain PCG.
"""
import numpy as np
import pytest

import cabi
from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _boxes(sizes, seed0):
    from cppe_gb300 import synthetic
    return [synthetic.water_box(nw, seed=seed0 + k) for k, nw in enumerate(sizes)]


def _rhs_for(b, nrhs, seed):
    from cppe_gb300 import synthetic
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(nrhs):
        c = b.xyz.mean(axis=0) + rng.uniform(-6, 6, size=(12, 3))
        q = rng.normal(0, 0.5, size=12)
        out.append(synthetic.point_charge_field(b.xyz, c, q))
    return out


def _unpack(p):
    H, I, O = 128, 64, 4
    k = 0
    W1 = p[k:k + H * I].reshape(H, I); k += H * I
    b1 = p[k:k + H]; k += H
    W2 = p[k:k + H * H].reshape(H, H); k += H * H
    b2 = p[k:k + H]; k += H
    W3 = p[k:k + O * H].reshape(O, H); k += O * H
    b3 = p[k:k + O]
    return [W1, b1, W2, b2, W3, b3]


def test_mlp_gradients_match_oracle(gpu):
    from cppe_gb300 import learned
    boxes = _boxes([150], 200)
    feats, rows = learned.training_rows(boxes, [_rhs_for(boxes[0], 1, 1)])
    model = cabi.Mlp(seed=3)
    mean, std = feats.mean(0), feats.std(0)
    inv = np.where(std > 1e-6, 1 / np.maximum(std, 1e-6), 0.0)
    model.set_normalization(mean, inv)
    p = model.params
    # perturb the output layer so every gradient block is non-trivial
    rng = np.random.default_rng(0)
    p[-(4 * 128 + 4):] += rng.normal(0, 0.05, size=4 * 128 + 4).astype(np.float32)
    model.params = p
    X = (feats - mean) * inv
    L, g = model.loss_grad(feats, rows, lam=0.7)
    Lr, gr = mlp_oracle.loss_and_grads(_unpack(p.astype(np.float64)), X, rows, lam=0.7)
    assert abs(L - Lr) < 1e-4 * abs(Lr)
    gref = np.concatenate([x.ravel() for x in gr])
    scale = np.abs(gref).max()
    np.testing.assert_allclose(g, gref, rtol=0, atol=2e-4 * scale)
    y = model.forward(feats[:100])
    yr, _ = mlp_oracle.forward(_unpack(p.astype(np.float64)), X[:100])
    np.testing.assert_allclose(y, yr, rtol=0, atol=1e-4 * np.abs(yr).max())


def test_learned_guess_reduces_iterations(gpu):
    from cppe_gb300 import learned
    train = _boxes([120, 200, 260, 330, 160, 300, 240, 180], 300)
    feats, rows = learned.training_rows(train, [_rhs_for(b, 2, 10 + k) for k, b in enumerate(train)])
    model, losses = learned.fit(feats, rows, steps=300, batch=4096, lr=3e-3)
    assert losses[-20:].mean() < 0.5 * losses[:5].mean()
    test = _boxes([280, 350], 900)
    gained = 0
    for k, b in enumerate(test):
        for rhs in _rhs_for(b, 2, 77 + k):
            plain = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, damp=True)
            mu_p, it_p, _, _ = plain.solve(rhs)
            ml = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, damp=True)
            ml.set_model(model)
            mu_l, it_l, _, _ = ml.solve(rhs)
            # same stopping rule, same answer
            assert np.linalg.norm(rhs - plain.apply(mu_l)) < 1e-8
            np.testing.assert_allclose(mu_l, mu_p, atol=1e-8)
            gained += it_p - it_l
            assert it_l <= it_p
    assert gained > 0


def test_shipped_model_on_a_large_system(gpu):
    """The shipped model drives a 75,000-site mixed solve (the learned
    preconditioner's reductions span n/32 blocks) to the FP64 criterion."""
    import os
    from cppe_gb300 import learned, synthetic
    path = os.path.join(os.path.dirname(__file__), "..", "cppe_gb300", "data", "learned_water.npz")
    b = synthetic.water_box(25000, seed=41)
    rhs = _rhs_for(b, 1, 5)[0]
    s = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, damp=True,
                    precision=cabi.MIXED)
    s.set_model(learned.load(path))
    mu, it, _, _ = s.solve(rhs)
    s.set_model(None)
    s64 = cabi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=cabi.FMM, damp=True)
    assert np.linalg.norm(rhs - s64.apply(mu)) < 1e-8


@pytest.mark.parametrize("rows", [1000, 131072 + 77])
def test_tensor_core_inference_matches_fp32(gpu, rows):
    """The tcgen05 inference kernel (TF32 operands rounded to nearest, FP32
    accumulation in tensor memory) against the FP32 GEMM forward pass, with
    the shipped model, on descriptor-like rows (partial last tile, and many
    tiles per CTA).  Bound: 1e-2 of the largest output and 1e-3 in norm; TF32
    keeps 11 significant bits per operand (2^-12 relative rounding)."""
    import os
    from cppe_gb300 import learned
    m = learned.load(learned.DEFAULT_MODEL)
    mean, inv = m.normalization()
    rng = np.random.default_rng(rows)
    std = np.where(inv > 0, 1.0 / np.maximum(inv, 1e-30), 0.0)
    feats = (mean + std * rng.normal(size=(rows, 64))).astype(np.float32)
    y32 = m.forward(feats)
    ytc = m.infer(feats)
    assert np.all(np.isfinite(ytc))
    scale = np.abs(y32).max()
    assert np.abs(ytc - y32).max() < 1e-2 * scale
    assert np.linalg.norm(ytc - y32) < 1e-3 * np.linalg.norm(y32)
    ytc2 = m.infer(feats)
    np.testing.assert_array_equal(ytc, ytc2)  # deterministic
    m.close()
