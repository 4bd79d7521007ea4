"""Regenerates the golden fixtures of tests/golden/ from the reference.

Run in a checkout where the reference sources are mounted (default
/root/reference, or $CPPE_REFERENCE_DIR):

    python tests/golden/make_golden.py

1. Copies (gzip) the reference's own test data used to pin the path:
   tests/potfiles/{pna_6w,pna_6w_isopol,loprop_solvated_20}.pot,
   tests/potfiles/fmuls_loprop_solvated_20.txt (MultipoleFields, direct
   summation, 8,805 sites) and tests/ref_fmm_errors.csv (per-site FMM errors).
2. Runs the reference's own FMM/direct-sum engine (compiled in place by
   oracle/Makefile into oracle/_ref) on small systems and stores its outputs in
   ref_vectors.npz: BMatrix applies, PCG solutions, MultipoleFields, and the
   sizes plus a hash of the interaction lists of the benchmark geometries.
"""
import gzip
import hashlib
import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from cppe_gb300 import synthetic  # noqa: E402

REF = os.environ.get("CPPE_REFERENCE_DIR", "/root/reference")


def gz(src, name):
    with open(src, "rb") as fi, gzip.open(os.path.join(HERE, name + ".gz"), "wb", 9) as fo:
        shutil.copyfileobj(fi, fo)


def list_hash(m2l, p2p):
    a = np.sort(m2l.view(np.int64).ravel())
    b = np.sort(p2p.view(np.int64).ravel())
    h = hashlib.sha256()
    h.update(a.tobytes())
    h.update(b.tobytes())
    return h.hexdigest()


def main():
    for f in ("pna_6w.pot", "pna_6w_isopol.pot", "loprop_solvated_20.pot",
              "fmuls_loprop_solvated_20.txt"):
        gz(os.path.join(REF, "tests", "potfiles", f), f)
    gz(os.path.join(REF, "tests", "ref_fmm_errors.csv"), "ref_fmm_errors.csv")

    if not O.build_ref():
        raise SystemExit("reference sources not found")
    R = O.RefOracle()
    out = {}

    # pna_6w: 18 sites, anisotropic polarizabilities, exclusions
    s = O.read_potfile(os.path.join(REF, "tests", "potfiles", "pna_6w.pot"))
    rng = np.random.default_rng(11)
    v = rng.normal(size=3 * s.n)
    Fm = R.multipole_fields(s)
    out["pna_mulfields"] = Fm
    out["pna_vec"] = v
    for damp, tag in ((0.0, "plain"), (2.1304, "damped")):
        out[f"pna_apply_{tag}"] = R.bmatrix_apply(s.xyz, s.alpha6, s.excl_ptr, s.excl_idx, v,
                                                  damping=damp)
        mu, it, hist, ok = R.solve(s.xyz, s.alpha6, s.excl_ptr, s.excl_idx, Fm,
                                   thresh=1e-12, damping=damp)
        assert ok
        out[f"pna_mu_{tag}"] = mu
        out[f"pna_hist_{tag}"] = hist

    # 120 waters: FMM with a multi-level tree (ncrit 16)
    b = synthetic.water_box(120, seed=7)
    aiso = b.alpha_iso
    pol = np.ones(b.n, np.int32)
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=pol, excl_ptr=b.excl_ptr, excl_idx=b.excl_idx)
    out["w120_xyz"] = b.xyz
    for fmm, tag in ((0, "direct"), (1, "fmm")):
        for dm, dtag in ((0.0, "plain"), (2.1304, "damped")):
            out[f"w120_mulfields_{tag}_{dtag}"] = R.multipole_fields(
                sites, fmm=fmm, ncrit=16, order=5, theta=0.5, damping=dm)
    v = np.random.default_rng(12).normal(size=3 * b.n)
    out["w120_vec"] = v
    for fmm, tag in ((0, "direct"), (1, "fmm")):
        for order in ((5, 6) if fmm else (5,)):
            out[f"w120_apply_{tag}_p{order}"] = R.bmatrix_apply(
                b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, fmm=fmm, ncrit=16, order=order,
                theta=0.5, damping=2.1304)
        rhs = b.external_field() + out[f"w120_mulfields_{tag}_plain"]
        mu, it, hist, ok = R.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, thresh=1e-10,
                                   fmm=fmm, ncrit=16, order=5, theta=0.5, damping=2.1304)
        assert ok
        out[f"w120_rhs_{tag}"] = rhs
        out[f"w120_mu_{tag}"] = mu

    # configuration 0 (333 waters, seed 0): direct, damped, FP64, tol 1e-8
    c0 = synthetic.water_box(333, seed=0)
    s0 = O.Sites(xyz=c0.xyz, elements=c0.elements, q=c0.q, mu=c0.mu, quad=c0.quad, max_order=2,
                 alpha6=c0.alpha6, polarizable=np.ones(c0.n, np.int32), excl_ptr=c0.excl_ptr,
                 excl_idx=c0.excl_idx)
    Fm0 = R.multipole_fields(s0)
    E0 = c0.external_field()
    mu, it, hist, ok = R.solve(c0.xyz, c0.alpha6, c0.excl_ptr, c0.excl_idx, E0 + Fm0,
                               thresh=1e-8, damping=2.1304)
    assert ok
    out["c0_mulfields"] = Fm0
    out["c0_mu"] = mu
    out["c0_iters"] = np.array([it])
    out["c0_hist"] = hist

    # interaction lists of the benchmark geometries (ncrit 64, theta 0.5)
    for tag, nw, seed in (("c0", 333, 0), ("c1", 10000, 1)):
        bx = synthetic.water_box(nw, seed=seed)
        t = R.tree_lists(bx.xyz, ncrit=64, theta=0.5)
        out[f"tree_{tag}_counts"] = np.array([len(t["cells"]), len(t["m2l"]), len(t["p2p"])])
        out[f"tree_{tag}_hash"] = np.array([list_hash(t["m2l"], t["p2p"])])

    np.savez_compressed(os.path.join(HERE, "ref_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_vectors.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
