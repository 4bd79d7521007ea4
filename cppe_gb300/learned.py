"""Training and use of the learned initial guess / preconditioner correction.

The network and its training run on the GPU (``cppe_gpu_mlp_*``); this module
only orchestrates: it solves training systems with the plain PCG (whose
solutions are the training targets), extracts per-site descriptor and target rows
(``cppe_gpu_learned_data``), sets the descriptor normalisation and runs the
Adam steps.  A trained model is attached to a system with ``System.set_model``;
first-call solves then start from the learned guess and use the corrected
preconditioner, and fall back to plain PCG if they do not converge.
"""
from __future__ import annotations

import os

import numpy as np

from . import capi


def training_rows(boxes, rhs_list, summation=None, direct_below=4000, device=0, **opts):
    """Solve every (system, rhs) with plain FP64 PCG and return stacked rows.

    boxes: systems with xyz, alpha6, excl_ptr, excl_idx; rhs_list: one list of
    right-hand sides per system."""
    feats, rows = [], []
    for b, rhss in zip(boxes, rhs_list):
        summ = summation if summation is not None else (
            capi.FMM if b.xyz.shape[0] >= direct_below else capi.DIRECT)
        s = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=summ, damp=True,
                        device=device, **opts)
        for rhs in rhss:
            mu, it, _, _ = s.solve(rhs)
            f, r = s.learned_data(rhs, mu)
            feats.append(f)
            rows.append(r)
        s.close()
    return np.concatenate(feats), np.concatenate(rows)


def fit(feats, rows, steps=400, batch=4096, lr=3e-3, lam=1.0, seed=0, device=0, model=None):
    """Train (or continue training) a model on stacked rows; returns (model, losses)."""
    if model is None:
        model = capi.Mlp(seed=seed, device=device)
        mean = feats.mean(axis=0)
        std = feats.std(axis=0)
        inv = np.where(std > 1e-6, 1.0 / np.maximum(std, 1e-6), 0.0)
        model.set_normalization(mean, inv)
    losses = model.train(feats, rows, steps, batch=batch, lr=lr, lam=lam, seed=seed)
    return model, losses


def generator_rhs(box, nrhs, seed):
    """External fields of `nrhs` random point-charge sets (12 charges N(0, 0.5) e
    within 3 A of the box centre, as the benchmark generator draws them)."""
    from . import synthetic
    rng = np.random.default_rng(seed)
    out = []
    centre = box.xyz.mean(axis=0)
    for _ in range(nrhs):
        v = rng.normal(size=(12, 3))
        v *= (3.0 * synthetic.ANG2BOHR) * rng.random((12, 1)) ** (1 / 3) / np.linalg.norm(
            v, axis=1, keepdims=True)
        out.append(synthetic.point_charge_field(box.xyz, centre + v, rng.normal(0, 0.5, 12)))
    return out


def train_from_generators(n_snapshots=250, nrhs=8, sample_frac=0.1, steps=1500, batch=16384,
                          lr=2e-3, seed=7, device=0, max_waters=6667, log=print):
    """Trains on n_snapshots x nrhs solves of the batched-configuration
    generator (snapshots of 500-20,000 sites, log-uniform; direct summation
    below 4,000 sites, FMM order 5 above), keeping a random `sample_frac` of
    each solve's site rows."""
    from . import synthetic
    rng = np.random.default_rng(seed)
    sizes = synthetic.snapshot_sizes(n_snapshots, seed=seed)
    feats, rows = [], []
    for k, ns in enumerate(sizes):
        nw = min(int(ns) // 3, max_waters)
        box = synthetic.water_box(nw, seed=10000 + seed * 1000 + k)
        f, r = training_rows([box], [generator_rhs(box, nrhs, seed * 7919 + k)], device=device)
        keep = rng.random(f.shape[0]) < sample_frac
        feats.append(f[keep])
        rows.append(r[keep])
        if log and (k + 1) % 25 == 0:
            log(f"  training data: {k + 1}/{n_snapshots} snapshots, "
                f"{sum(x.shape[0] for x in feats)} rows")
    feats, rows = np.concatenate(feats), np.concatenate(rows)
    model, losses = fit(feats, rows, steps=steps, batch=batch, lr=lr, seed=seed, device=device)
    return model, losses, feats.shape[0]


def save(model, path):
    m, s = model.normalization()
    np.savez(path, params=model.params, mean=m, inv_std=s)


def load(path, device=0):
    d = np.load(path)
    model = capi.Mlp(device=device)
    model.params = d["params"]
    model.set_normalization(d["mean"], d["inv_std"])
    return model


DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                             "learned_water.npz")


def main(argv=None):
    """Trains the shipped model on the GPU: `python -m cppe_gb300.learned --out PATH`."""
    import argparse
    import time
    ap = argparse.ArgumentParser(description=main.__doc__)
    ap.add_argument("--out", default=DEFAULT_MODEL)
    ap.add_argument("--snapshots", type=int, default=250)
    ap.add_argument("--nrhs", type=int, default=8)
    ap.add_argument("--steps", type=int, default=1500)
    ap.add_argument("--seed", type=int, default=7)
    ap.add_argument("--device", type=int, default=0)
    a = ap.parse_args(argv)
    t0 = time.time()
    model, losses, rows = train_from_generators(n_snapshots=a.snapshots, nrhs=a.nrhs,
                                                steps=a.steps, seed=a.seed, device=a.device)
    os.makedirs(os.path.dirname(a.out) or ".", exist_ok=True)
    save(model, a.out)
    print(f"trained on {a.snapshots * a.nrhs} solves ({rows} site rows), loss "
          f"{losses[:10].mean():.4g} -> {losses[-50:].mean():.4g}, {time.time() - t0:.1f} s; "
          f"wrote {a.out}", flush=True)


if __name__ == "__main__":
    main()
