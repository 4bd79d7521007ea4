"""Reference solutions of the benchmark's water boxes, as compact summaries.

Runs the reference's own FMM engine (compiled in place by oracle/Makefile into
oracle/_ref; the BMatrix/InducedMoments loops restated in oracle/ref_glue.cc)
on the seeded water boxes of the 30,000-, 300,000- and 1,000,002-site
workloads and writes config_solutions.json:

* the right-hand side F = field of the 12 point charges + MultipoleFields
  (FMM with the workload's order, theta 0.5, ncrit 64, undamped multipoles);
* the FP64 PCG solution mu from the first-call guess alpha F to
  ||F - B mu||_2 < 1e-8 with the FMM operator (Thole damping 2.1304);
* summaries small enough to commit: iteration count and residual history,
  the polarization energy -1/2 mu.F, norms, the sums of mu and F over 64
  contiguous blocks, and mu and F at 64 seeded site indices.

The full vectors are too large to commit at these sizes; the summaries pin a
GPU solution to the reference's (energy to 1e-7 Hartree, entries and block
sums to the solve's tolerance).  Run where the reference is mounted:

    python tests/golden/make_config_solutions.py [30k 300k 1m]

At 1M sites the reference engine needs about 15 minutes on 8 cores.
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from cppe_gb300 import synthetic  # noqa: E402

# name: (waters, seed, order) -- the seeded boxes of bench.py's workloads
WORKLOADS = {"30k": (10000, 1, 5), "300k": (100000, 2, 6), "1m": (333334, 4, 6)}
NBLOCK = 64
NSAMPLE = 64
OUT = os.path.join(HERE, "config_solutions.json")


def block_sums(v, nsites):
    """Sums of a site-major 3-vector field over NBLOCK contiguous site blocks."""
    edges = np.linspace(0, nsites, NBLOCK + 1).astype(np.int64)
    v = v.reshape(-1, 3)
    return [v[a:b].sum(axis=0).tolist() for a, b in zip(edges[:-1], edges[1:])]


def sample_sites(nsites, seed):
    return np.sort(np.random.default_rng(seed).choice(nsites, NSAMPLE, replace=False))


def summarize(name):
    nw, seed, order = WORKLOADS[name]
    R = O.RefOracle()
    b = synthetic.water_box(nw, seed=seed)
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32), excl_ptr=b.excl_ptr,
                    excl_idx=b.excl_idx)
    t0 = time.time()
    F = b.external_field() + R.multipole_fields(sites, fmm=True, order=order)
    t_f = time.time() - t0
    t0 = time.time()
    mu, it, hist, ok = R.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, F, fmm=True, ncrit=64,
                               order=order, theta=0.5, damping=2.1304, thresh=1e-8)
    t_s = time.time() - t0
    assert ok, f"{name}: the reference solve did not converge"
    idx = sample_sites(b.n, 7)
    m3, f3 = mu.reshape(-1, 3), F.reshape(-1, 3)
    return {
        "sites": int(b.n), "waters": nw, "seed": seed, "order": order, "theta": 0.5,
        "ncrit": 64, "damping": 2.1304, "thresh": 1e-8,
        "iterations": int(it), "rnorm_history": [float(x) for x in hist],
        "epol": float(-0.5 * mu @ F), "mu_norm": float(np.linalg.norm(mu)),
        "mu_maxabs": float(np.abs(mu).max()), "F_norm": float(np.linalg.norm(F)),
        "mu_block_sums": block_sums(mu, b.n), "F_block_sums": block_sums(F, b.n),
        "sample_sites": idx.tolist(), "mu_samples": m3[idx].tolist(),
        "F_samples": f3[idx].tolist(),
        "engine": "reference FMM engine (oracle/_ref), OpenMP",
        "seconds": {"fields": round(t_f, 1), "solve": round(t_s, 1)},
    }


def main():
    names = sys.argv[1:] or list(WORKLOADS)
    if not O.build_ref():
        raise SystemExit("reference sources not found")
    out = {}
    if os.path.exists(OUT):
        with open(OUT) as f:
            out = json.load(f)
    for name in names:
        out[name] = summarize(name)
        print(name, out[name]["iterations"], out[name]["epol"], out[name]["seconds"],
              flush=True)
        with open(OUT, "w") as f:
            json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
