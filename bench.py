#!/usr/bin/env python
"""Benchmark of the induced-dipole solve (time to a 1e-8 residual).

Workload (default, the largest single-GPU configuration): 333,334 rigid
waters = 1,000,002 polarizable sites, FMM expansion order 6, theta 0.5,
ncrit 64, Thole damping a = 2.1304, one right-hand side = field of 12 point
charges + static multipole field, solved from the reference's first-call
guess alpha*F to ||F - B mu||_2 < 1e-8 with the FP64 FMM operator.  A step is
one complete solve.

value     the method: mixed-precision solve (FP32 inner PCG + FP64-accurate
          refinement) with the trained guess/preconditioner model, inputs and
          outputs resident on the GPU, CUDA events on the library's stream.
e2e       the same solve through the C ABI with host buffers
          (cppe_gpu_solve: H2D of F, D2H of mu inside the timed region).
plain     the plain FP64 GPU PCG (the reference's algorithm on the GPU) on the
          same system, reported next to the headline.
vs_oracle the headline's answer checked against the reference: the oracle's
          FP64 operator applied to the GPU solution (the reference's own
          stopping criterion), and the reference engine's committed solution
          summary of the same box (tests/golden/config_solutions.json).

Extra sections: the 30,000-site order-5 system (with a full oracle solve to
compare against), the 300,000-site order-6 system, and the 256 x 8 batch.

`--impl reference` times the reference algorithm on the host cores (the
oracle's C++ restatement with OpenMP, all threads) on the same workload: full
solves where one fits a few seconds, else FMM applies (tree rebuilt per
apply, as the reference does) times the reference's applies per solve.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: (waters, seed, summation, order, description)
    "999-direct": (333, 0, "direct", 5, "999 sites, direct summation"),
    "30k-fmm5": (10000, 1, "fmm", 5, "30,000 sites, FMM order 5, theta 0.5, ncrit 64"),
    "300k-fmm6": (100000, 2, "fmm", 6, "300,000 sites, FMM order 6, theta 0.5, ncrit 64"),
    "1m-fmm6": (333334, 4, "fmm", 6, "1,000,002 sites, FMM order 6, theta 0.5, ncrit 64"),
}
METRIC = "induced-dipole solve time to 1e-8 residual"
FLOP_PER_PAIR = 45  # damped dipole pair, see include/cppe_gpu/work_model.h
DD_RESIDUAL = 2     # kernel_timings mode: FP64 operator with the double-float near field


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """SM clock and clock-event reasons sampled during the timed region: NVML
    through ctypes every ~2 ms when libnvidia-ml loads (read-only queries),
    else nvidia-smi every 50 ms."""

    # clock-event reason bits of NVML (nvmlClocksEventReason*)
    BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
            0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []  # (sm_mhz, max_mhz, reasons set)
        self.proc = None
        self.nvml = None
        self.stop = threading.Event()

    def _nvml_open(self):
        import ctypes
        lib = ctypes.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = ctypes.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(self.device, ctypes.byref(h)) != 0:
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, reasons

    def _nvml_loop(self):
        import ctypes
        lib, h, reasons = self.nvml
        clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
        lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        while not self.stop.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk)) == 0 and \
                    reasons(h, ctypes.byref(rs)) == 0:
                self.rows.append((float(clk.value), float(mx.value),
                                  {n for bit, n in self.BITS.items() if rs.value & bit}))
            time.sleep(0.002)

    def _smi_loop(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.proc.stdout:
            r = [c.strip() for c in line.split(",")]
            try:
                self.rows.append((float(r[0]), float(r[1]),
                                  {names[k] for k in range(4) if r[3 + k].lower() == "active"}))
            except (ValueError, IndexError):
                pass

    def __enter__(self):
        try:
            self.nvml = self._nvml_open()
        except (OSError, AttributeError):
            self.nvml = None
        if self.nvml:
            self.t = threading.Thread(target=self._nvml_loop, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._smi_loop, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.stop.set()
        if self.nvml:
            self.t.join(timeout=1)
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = list(self.rows)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(r[0] for r in rows),
                "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(set().union(*(r[2] for r in rows))),
                "samples": len(rows), "source": "nvml" if self.nvml else "nvidia-smi"}


def workload_config(cfg, n):
    """The workload as both arms report it."""
    return {"workload": f"{cfg}: {CONFIGS[cfg][4]}, Thole damping 2.1304, 1 RHS (12 point "
                        "charges + static multipole field), tol 1e-8 on ||F - B mu||_2 with "
                        "the FP64 operator, PCG from alpha*F", "sites": n}


def make_problem(cfg):
    from cppe_gb300 import synthetic
    nw, seed, summation, order, _ = CONFIGS[cfg]
    b = synthetic.water_box(nw, seed=seed)
    return b, summation, order


def static_rhs_gpu(b, summation, order):
    from cppe_gb300 import capi
    Fm = capi.multipole_fields(b.xyz, b.q, b.mu, b.quad, 2, np.ones(b.n, np.int32),
                               b.alpha_iso, b.excl_ptr, b.excl_idx,
                               fmm=(summation == "fmm"), ncrit=64, order=order)
    return (b.external_field() + Fm).ravel()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


GOLDEN_PATH = os.path.join(ROOT, "tests", "golden", "config_solutions.json")
GOLDEN_KEY = {"30k-fmm5": "30k", "300k-fmm6": "300k", "1m-fmm6": "1m"}
# configurations whose reference solve takes too long for a bench step: the
# reference arm times FMM applies and scales them by the applies per solve
APPLY_SAMPLED = {"300k-fmm6", "1m-fmm6"}


def golden(cfg):
    """The reference engine's solution summary of a workload's box, or None."""
    if cfg not in GOLDEN_KEY or not os.path.exists(GOLDEN_PATH):
        return None
    with open(GOLDEN_PATH) as f:
        return json.load(f).get(GOLDEN_KEY[cfg])


def oracle_port():
    from oracle import oracle as O
    if not os.path.exists(O.PORT_LIB):
        O.build_port()
    return O.port()


def oracle_kw(summation, order):
    return dict(fmm=int(summation == "fmm"), ncrit=64, order=order, theta=0.5, damping=2.1304)


def run_reference(args):
    """The reference algorithm on the host cores (oracle restatement)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    P = oracle_port()
    b, summation, order = make_problem(args.config)
    kw = oracle_kw(summation, order)
    cores = os.cpu_count()
    if args.config in APPLY_SAMPLED:
        g = golden(args.config)
        iters = g["iterations"] if g else None
        if iters is None:
            print(json.dumps({"impl": "reference", "unavailable":
                              "no reference iteration count for this workload"}), flush=True)
            return
        applies = iters + 1  # one apply per PCG iteration plus the initial residual
        v = b.external_field().ravel()
        for _ in range(args.warmup):
            P.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, **kw)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            P.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, v, **kw)
            times.append(time.perf_counter() - t0)
        t_apply = float(np.mean(times))
        v_solve = t_apply * applies
        sample = (f"{args.steps} FMM applies B*v of the {b.n:,}-site system (octree rebuilt per "
                  "apply, as the reference does), OpenMP over all host threads; solve time = "
                  f"{t_apply:.3f} s per apply x {applies} applies (the reference engine's PCG "
                  f"takes {iters} iterations on this system, "
                  "tests/golden/config_solutions.json)")
    else:
        rhs = b.external_field().ravel() + P.multipole_fields(
            _oracle_sites(b), fmm=summation == "fmm", order=order)
        for _ in range(args.warmup):
            P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, thresh=1e-8, **kw)
        times, its = [], []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            mu, it, hist, ok = P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs,
                                       thresh=1e-8, **kw)
            times.append(time.perf_counter() - t0)
            its.append(it)
        v_solve = float(np.mean(times))
        sample = (f"{args.steps} full solves ({int(np.mean(its))} CG iterations each), OpenMP "
                  "over all host threads")
    line = {
        "impl": "reference", "metric": METRIC, "value": v_solve, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v_solve * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded water box, 12 point charges)",
        "config": dict(workload_config(args.config, b.n), parallelism="host threads"),
        "cpu_baseline": {"value": v_solve, "unit": "s", "cores": cores, "kind": "port",
                         "sample": sample},
        "e2e": {"value": v_solve, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def _oracle_sites(b):
    from oracle import oracle as O
    return O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                   alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32), excl_ptr=b.excl_ptr,
                   excl_idx=b.excl_idx)


def oracle_residual(P, b, rhs, mu, summation, order):
    """||rhs - B mu||_2 with the oracle's FP64 operator (the reference's
    stopping criterion evaluated by the reference algorithm) and its time."""
    t0 = time.perf_counter()
    Bmu = P.bmatrix_apply(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, mu,
                          **oracle_kw(summation, order))
    return float(np.linalg.norm(rhs - Bmu)), time.perf_counter() - t0


def vs_reference_solution(cfg, rhs, mu):
    """A GPU solution against the reference engine's committed summary of the
    same box: energy -1/2 mu.F, mu at 64 seeded sites, mu over 64 site blocks,
    and the right-hand side (static fields) at the same sites."""
    g = golden(cfg)
    if g is None or g["sites"] * 3 != mu.size:
        return None
    idx = np.asarray(g["sample_sites"])
    m3, f3 = mu.reshape(-1, 3), rhs.reshape(-1, 3)
    edges = np.linspace(0, g["sites"], len(g["mu_block_sums"]) + 1).astype(np.int64)
    blocks = np.array([m3[a:c].sum(axis=0) for a, c in zip(edges[:-1], edges[1:])])
    return {"epol_hartree_diff": float(abs(-0.5 * mu @ rhs - g["epol"])),
            "mu_sample_maxabs": float(np.abs(m3[idx] - np.asarray(g["mu_samples"])).max()),
            "mu_block_sum_maxabs": float(np.abs(blocks - np.asarray(g["mu_block_sums"])).max()),
            "F_sample_maxabs": float(np.abs(f3[idx] - np.asarray(g["F_samples"])).max()),
            "reference_iterations": g["iterations"], "reference_epol": g["epol"]}


def _event_time(stream, fn):
    """Seconds of fn() on `stream`, CUDA events on that stream."""
    import torch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    out = fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) * 1e-3, out


def batched_section(dev, steps, flush, compare=True):
    """256 snapshots of 500-20,000 sites (log-uniform; direct summation below
    4,000 sites, FMM p5 above), 8 point-charge right-hand sides each, solved
    as one batch in mixed precision; against the plain FP64 GPU PCG solving the
    same segments one at a time."""
    import torch
    from cppe_gb300 import capi, learned, synthetic
    sizes = synthetic.snapshot_sizes(256, seed=1000)
    boxes = [synthetic.water_box(int(ns) // 3, seed=1000 + i) for i, ns in enumerate(sizes)]
    nrhs = 8
    rhs = [learned.generator_rhs(b, nrhs, 5000 + i) for i, b in enumerate(boxes)]
    flat = np.concatenate([np.concatenate(r) for r in rhs])
    t0 = time.perf_counter()
    batch = capi.Batch(boxes, nrhs, direct_below=4000, precision=capi.MIXED, damp=True,
                       order=5, ncrit=64, theta=0.5, thresh=1e-8, device=dev)
    setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    tuned_ms = batch.autotune(2)
    tune = time.perf_counter() - t0
    d_rhs = torch.tensor(flat, dtype=torch.float64, device=f"cuda:{dev}")
    d_mu = torch.zeros_like(d_rhs)
    st = torch.cuda.ExternalStream(batch.stream())
    batch.solve_device(d_rhs.data_ptr(), d_mu.data_ptr())  # warm-up
    times = []
    for _ in range(steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t, its = _event_time(st, lambda: batch.solve_device(d_rhs.data_ptr(), d_mu.data_ptr()))
        times.append(t)
    bst = batch.stats()
    t_batch = float(np.mean(times))
    if not compare:
        # the batch alone (profiling): no one-at-a-time FP64 solves
        return {"workload": "256 snapshots x 8 RHS (batch only)", "value": t_batch, "unit": "s",
                "fp32_applies": bst["fp32_applies"], "fp64_applies": bst["fp64_applies"],
                "host_waits": bst["host_waits"], "max_rnorm": bst["max_rnorm"]}
    mu = d_mu.cpu().numpy()
    # plain FP64, one segment at a time: the first right-hand side of every
    # snapshot is solved and timed; the 8 right-hand sides of a snapshot cost
    # the same, so the total is 8x the measured sum
    plain, worst, off = 0.0, 0.0, 0
    for i, b in enumerate(boxes):
        summ = capi.FMM if b.n >= 4000 else capi.DIRECT
        s64 = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, summation=summ, order=5,
                          ncrit=64, theta=0.5, damp=True, thresh=1e-8, precision=capi.FP64,
                          device=dev)
        r0 = torch.tensor(rhs[i][0], dtype=torch.float64, device=f"cuda:{dev}")
        m0 = torch.zeros_like(r0)
        s64.solve_device(r0.data_ptr(), m0.data_ptr())  # warm-up
        torch.cuda.synchronize()
        t, _ = _event_time(torch.cuda.ExternalStream(s64.stream()),
                           lambda: s64.solve_device(r0.data_ptr(), m0.data_ptr()))
        plain += t
        # FP64 residual of the batched mixed solution (first rhs of each snapshot)
        seg = mu[off:off + 3 * b.n]
        worst = max(worst, float(np.linalg.norm(rhs[i][0] - s64.apply(seg))))
        off += nrhs * 3 * b.n
        s64.close()
    plain *= nrhs
    # against the oracle: its FP64 operator's residual of every right-hand side
    # of four snapshots (the smallest and largest direct-summation ones, the
    # smallest and largest FMM ones), and full oracle solves of the first
    # right-hand side of the largest direct and the largest FMM snapshot
    P = oracle_port()
    offs = np.concatenate([[0], np.cumsum([nrhs * 3 * b.n for b in boxes])])
    direct = [i for i, b in enumerate(boxes) if b.n < 4000]
    fmm = [i for i, b in enumerate(boxes) if b.n >= 4000]
    by_n = lambda ids: sorted(ids, key=lambda i: boxes[i].n)  # noqa: E731
    picks = [by_n(direct)[0], by_n(direct)[-1], by_n(fmm)[0], by_n(fmm)[-1]]
    worst_o, mu_diff = 0.0, {}
    for i in picks:
        b = boxes[i]
        summation = "fmm" if b.n >= 4000 else "direct"
        for r in range(nrhs):
            seg = mu[offs[i] + r * 3 * b.n:offs[i] + (r + 1) * 3 * b.n]
            worst_o = max(worst_o, oracle_residual(P, b, rhs[i][r], seg, summation, 5)[0])
    for i in (picks[1], picks[3]):
        b = boxes[i]
        summation = "fmm" if b.n >= 4000 else "direct"
        mu_o, it_o, _, ok = P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs[i][0],
                                    thresh=1e-8, **oracle_kw(summation, 5))
        mu_diff[f"{summation}_{b.n}_sites"] = float(
            np.abs(mu[offs[i]:offs[i] + 3 * b.n] - mu_o).max())
    vs_oracle = {"snapshots": [int(boxes[i].n) for i in picks],
                 "max_oracle_residual": worst_o, "rhs_checked": 4 * nrhs,
                 "mu_maxabs_vs_oracle_solve": mu_diff}
    return {"workload": "256 snapshots x 8 RHS, sites log-uniform 500-20,000 "
                        f"({int(sum(sizes))} sites, {int(sum(sizes)) * nrhs} site-RHS), direct "
                        "< 4,000 sites, FMM p5 above, mixed precision, tol 1e-8",
            "value": t_batch, "unit": "s", "solves": len(boxes) * nrhs,
            "plain_fp64_sequential_s": plain,
            "plain_fp64_note": "first RHS of each snapshot solved and timed one at a time, x8",
            "speedup_vs_plain_fp64": plain / t_batch,
            "fp32_applies": bst["fp32_applies"], "fp64_applies": bst["fp64_applies"],
            "host_waits": bst["host_waits"], "max_fp64_residual": worst, "vs_oracle": vs_oracle, "setup_s": setup,
            "autotune_s": tune, "fp32_apply_ms": tuned_ms}


def system_section(cfg, dev, flush, steps, model_path=None, oracle_check="residual"):
    """One system solved by the plain FP64 PCG and by the mixed solver with and
    without the trained model.  Errors of the mixed solutions against the FP64
    one: induced dipoles, polarization energy (-1/2 mu.E_ext), the induced field
    B mu and the FP64 residual.  Against the reference: a full oracle solve
    (`oracle_check="solve"`) or the oracle operator's residual of the mixed
    solution ("residual"), and the reference engine's committed summary."""
    import torch
    from cppe_gb300 import capi, learned
    t0 = time.perf_counter()
    b, summation, order = make_problem(cfg)
    rhs = static_rhs_gpu(b, summation, order)
    setup = time.perf_counter() - t0
    kw = dict(summation=capi.FMM if summation == "fmm" else capi.DIRECT, ncrit=64, order=order,
              theta=0.5, damp=True, thresh=1e-8, device=dev)
    d_rhs = torch.tensor(rhs, dtype=torch.float64, device=f"cuda:{dev}")
    d_mu = torch.zeros_like(d_rhs)
    E = b.external_field().ravel()
    out = {"workload": f"{cfg}: {CONFIGS[cfg][4]}, Thole damping, tol 1e-8", "sites": b.n,
           "setup_s": setup}

    def timed(sys_):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t, _ = _event_time(torch.cuda.ExternalStream(sys_.stream()),
                           lambda: sys_.solve_device(d_rhs.data_ptr(), d_mu.data_ptr()))
        return t

    s64 = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.FP64, **kw)
    s64.apply(rhs)  # first-use allocations
    t64 = timed(s64)
    mu64 = d_mu.cpu().numpy()
    it64 = s64.stats()["fp64_applies"] - 1
    out["plain_fp64"] = {"s": t64, "iterations": it64}
    Bmu64 = s64.apply(mu64)
    smx = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.MIXED, **kw)
    t0 = time.perf_counter()
    out["autotune"] = {"apply_ms": smx.autotune(2), "s": time.perf_counter() - t0}  # set-up
    variants = [("mixed", None)]
    if model_path and os.path.exists(model_path):
        variants.append(("mixed_learned", learned.load(model_path, device=dev)))
    mus = {"plain_fp64": mu64}
    for name, model in variants:
        smx.set_model(model)
        timed(smx)  # warm-up (first-use allocations)
        ts = [timed(smx) for _ in range(steps)]
        mu = d_mu.cpu().numpy()
        st = smx.stats()
        Bmu = s64.apply(mu)
        mus[name] = mu
        out[name] = {
            "s": float(np.mean(ts)), "fp32_applies": st["fp32_applies"],
            "fp64_applies": st["fp64_applies"], "speedup_vs_plain_fp64": t64 / float(np.mean(ts)),
            "error_vs_fp64": {
                "mu_maxabs": float(np.abs(mu - mu64).max()),
                "epol_hartree": float(abs(0.5 * (mu - mu64) @ E)),
                "induced_field_rel": float(np.linalg.norm(Bmu - Bmu64) / np.linalg.norm(Bmu64)),
                "fp64_residual": float(np.linalg.norm(rhs - Bmu))}}
    smx.set_model(None)
    smx.close()
    s64.close()
    best = variants[-1][0]
    P = oracle_port()
    if oracle_check == "solve":
        t0 = time.perf_counter()
        mu_o, it_o, _, ok = P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, thresh=1e-8,
                                    **oracle_kw(summation, order))
        vo = {"oracle_solve_s": time.perf_counter() - t0, "oracle_iterations": it_o,
              "plain_fp64_iterations": it64}
        for name, mu in mus.items():
            vo[name] = {"mu_maxabs": float(np.abs(mu - mu_o).max()),
                        "epol_hartree": float(abs(0.5 * (mu - mu_o) @ rhs))}
        vo["oracle_residual_" + best], _ = oracle_residual(P, b, rhs, mus[best], summation,
                                                           order)
    else:
        r, t = oracle_residual(P, b, rhs, mus[best], summation, order)
        vo = {"oracle_residual_" + best: r, "oracle_apply_s": t}
    out["vs_oracle"] = vo
    out["vs_reference_solution"] = {k: vs_reference_solution(cfg, rhs, mus[k])
                                    for k in ("plain_fp64", best)}
    return out


def ingest_section(dev):
    """The 1,000,002-site water box as a .pot file (AA, 12 decimals; written
    before timing), read into arrays with CSR exclusions through the C ABI
    (cppe_gpu_potfile_read + _arrays), read into the reference's per-site
    objects (PotfileReader.read), and turned into a GPU system (octree, lists
    and uploads: cppe_gpu_create, FMM order 6)."""
    import ctypes
    import tempfile
    import cppe_gb300 as cppe
    from cppe_gb300 import capi, synthetic
    b = synthetic.water_box(333334, seed=4)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "w1m.pot")
        synthetic.write_potfile(b, path)
        size = os.path.getsize(path)
        L = capi.lib()
        h = ctypes.c_void_p()
        t0 = time.perf_counter()
        capi.check(L.cppe_gpu_potfile_read(os.fsencode(path), ctypes.byref(h)))
        n = b.n
        xyz, a6 = np.zeros((n, 3)), np.zeros((n, 6))
        q, mu, quad = np.zeros(n), np.zeros((n, 3)), np.zeros((n, 6))
        pol, ep, ei = np.zeros(n, np.int32), np.zeros(n + 1, np.int32), np.zeros(2 * n, np.int32)
        capi.check(L.cppe_gpu_potfile_arrays(h, capi.dp(xyz), capi.dp(q), capi.dp(mu),
                                             capi.dp(quad), capi.dp(a6), capi.ip(pol),
                                             capi.ip(ep), capi.ip(ei), None))
        t_arrays = time.perf_counter() - t0
        L.cppe_gpu_potfile_free(h)
        t0 = time.perf_counter()
        pots = cppe.PotfileReader(path).read()
        t_obj = time.perf_counter() - t0
        del pots
    t0 = time.perf_counter()
    s = capi.System(xyz, a6, ep, ei, summation=capi.FMM, order=6, ncrit=64, theta=0.5,
                    damp=True, device=dev)
    t_create = time.perf_counter() - t0
    s.close()
    return {"workload": "1,000,002-site water box, .pot file in AA", "file_bytes": size,
            "arrays_csr_s": t_arrays, "objects_s": t_obj, "gpu_system_create_s": t_create,
            "exclusions_match": bool(np.array_equal(ep, b.excl_ptr) and
                                     np.array_equal(ei, b.excl_idx))}


def profiled_traffic(md_name):
    """DRAM bytes (read + write) per launch from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", md_name)
    if not os.path.exists(path):
        return None
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    tot, found = 0.0, 0
    with open(path) as f:
        for line in f:
            for key in ("dram__bytes_read.sum", "dram__bytes_write.sum"):
                if f"`{key}`" in line:
                    cells = [c.strip() for c in line.strip().strip("|").split("|")]
                    tot += float(cells[1]) * scale.get(cells[2], 1.0)
                    found += 1
    return tot if found == 2 else None


# committed ncu summaries of the FP32 near field, by workload and form
# (workload, near-field form: 0 per target, 1 or 2 symmetric with two or
# four sources a lane) -> the committed capture of that kernel
PROFILE_OF = {("30k-fmm5", 0): "k_p2p32_m1_30k_sites.md",
              ("30k-fmm5", 1): "k_p2p32_m1_sym_30k_sites.md",
              ("1m-fmm6", 1): "k_p2p32_m1_sym_1m_sites.md",
              ("1m-fmm6", 2): "k_p2p32_m1_sym_4src_1m_sites.md"}


def run_ours(args):
    import torch
    from cppe_gb300 import capi

    rank, world, local = dist_env()
    dev = local
    torch.cuda.set_device(dev)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    b, summation, order = make_problem(args.config)
    rhs = static_rhs_gpu(b, summation, order)
    summ = capi.FMM if summation == "fmm" else capi.DIRECT
    kw = dict(summation=summ, ncrit=64, order=order, theta=0.5, damp=True, thresh=1e-8,
              device=dev)
    smx = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.MIXED, **kw)
    s64 = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.FP64, **kw)
    if args.apply_only:
        # operator applies only (FP32 then FP64), e.g. for kernel profiling
        if args.near_form >= 0:
            smx.set_schedule(args.near_form)
        t32 = smx.kernel_timings(capi.MIXED, reps=args.apply_only)
        tdd = smx.kernel_timings(DD_RESIDUAL, reps=args.apply_only)
        t64 = s64.kernel_timings(capi.FP64, reps=args.apply_only) if not args.no_fp64 else \
            ({}, 0, 0)
        print(json.dumps({"apply_only": args.apply_only, "config": args.config,
                          "fp32_ms": t32[0], "dd_ms": tdd[0], "fp64_ms": t64[0],
                          "alg_pairs": t32[1], "m2l_pairs": t32[2]}), flush=True)
        return
    tuned_ms = smx.autotune(3) if not args.no_autotune else None  # setup, not timed
    d_rhs = torch.tensor(rhs, dtype=torch.float64, device=f"cuda:{dev}")
    d_mu = torch.zeros_like(d_rhs)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{dev}")  # 256 MB
    ext = torch.cuda.ExternalStream(smx.stream())
    ext64 = torch.cuda.ExternalStream(s64.stream())
    model = None
    if not args.no_learned and args.model and os.path.exists(args.model):
        from cppe_gb300 import learned
        model = learned.load(args.model, device=dev)
    if args.solve_only:
        # mixed solves only (with the model when given), e.g. for launch lists
        smx.set_model(model)
        ts = []
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t, _ = _event_time(ext, lambda: smx.solve_device(d_rhs.data_ptr(), d_mu.data_ptr(),
                                                             make_guess=True))
            if k >= args.warmup:
                ts.append(t)
        print(json.dumps({"solve_only": args.steps, "config": args.config,
                          "ms": [t * 1e3 for t in ts], "stats": smx.stats(),
                          "learned": model is not None}), flush=True)
        return

    def timed_solve(sys_, stream):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        it, hist = sys_.solve_device(d_rhs.data_ptr(), d_mu.data_ptr(), make_guess=True)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) * 1e-3, it

    # the method: mixed precision, with the trained model when one is shipped
    smx.set_model(model)
    for _ in range(args.warmup):
        timed_solve(smx, ext)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = capi.launch_count()
    times = []
    with ClockSampler(dev) as clk:
        for _ in range(args.steps):
            t, it = timed_solve(smx, ext)
            times.append(t)
        torch.cuda.synchronize()
    launches = capi.launch_count() - l0
    st = smx.stats()
    mu_head = d_mu.cpu().numpy()
    t_head = float(np.mean(times))
    if world > 1:
        tt = torch.tensor([t_head], device=f"cuda:{dev}")
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_head = float(tt.item())

    # end to end through the C ABI with host buffers (same method): F and mu
    # in pinned host memory
    rhs_pin = torch.from_numpy(np.ascontiguousarray(rhs, dtype=np.float64)).pin_memory()
    mu_pin = torch.zeros(rhs.size, dtype=torch.float64).pin_memory()
    rhs_h, mu_h = rhs_pin.numpy(), mu_pin.numpy()
    e2e = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        smx.solve(rhs_h, out=mu_h)
        e2e.append(time.perf_counter() - t0)
    e2e_v = float(np.mean(e2e))

    # the mixed solver without the model, for the learned part's gain
    lrn = None
    if model is not None:
        smx.set_model(None)
        timed_solve(smx, ext)
        tw = [timed_solve(smx, ext)[0] for _ in range(args.steps)]
        lrn = {"with_model_s": t_head, "with_model_stats": st,
               "without_model_s": float(np.mean(tw)), "without_model_stats": smx.stats(),
               "gain": 1.0 - t_head / float(np.mean(tw)),
               "model": os.path.relpath(args.model, ROOT)}
        smx.set_model(model)

    # plain FP64 GPU PCG on the same system (one solve after a warm-up apply)
    s64.apply(rhs)
    plain, _ = timed_solve(s64, ext64)
    mu64 = d_mu.cpu().numpy()
    st64 = s64.stats()

    # roofline of the dominant kernel (FP32 near-field pair pass)
    tim32, alg_pairs, m2l_pairs = smx.kernel_timings(capi.MIXED, reps=5)
    timdd, _, _ = smx.kernel_timings(DD_RESIDUAL, reps=3)
    tim64, _, _ = s64.kernel_timings(capi.FP64, reps=2)
    sched = smx.schedule()
    near_kernel = (f"k_p2p32_m1_sym<true, {sched['sym_pack']}> (FP32 dipole near field, each "
                   f"leaf pair once, {2 * sched['sym_pack']} sources a lane)") \
        if sched["symmetric_near"] else "k_p2p32_m1<true> (FP32 dipole near field)"
    prof = PROFILE_OF.get((args.config, sched["sym_pack"]))
    fp32_peak = capi.fma_peak_tflops(False, dev)
    fp64_peak = capi.fma_peak_tflops(True, dev)
    achieved = alg_pairs * FLOP_PER_PAIR / (tim32["near"] * 1e-3) / 1e12
    achieved64 = alg_pairs * FLOP_PER_PAIR / (tim64["near"] * 1e-3) / 1e12
    pairs_per_s = {"fp32": alg_pairs / (tim32["near"] * 1e-3),
                   "double_float": alg_pairs / (timdd["near"] * 1e-3),
                   "fp64": alg_pairs / (tim64["near"] * 1e-3)}
    pk, pk_kind = peaks()

    E = b.external_field().ravel()
    Bmu_head = s64.apply(mu_head)
    Bmu64 = s64.apply(mu64)
    parity = {
        "fp64_residual": float(np.linalg.norm(rhs - Bmu_head)),
        "vs_plain_fp64_gpu": {
            "mu_maxabs": float(np.abs(mu_head - mu64).max()),
            "epol_hartree": float(abs(0.5 * (mu_head - mu64) @ E)),
            "induced_field_rel": float(np.linalg.norm(Bmu_head - Bmu64) /
                                       np.linalg.norm(Bmu64))}}
    smx.set_model(None)
    smx.close()
    s64.close()
    del d_rhs, d_mu
    sections = {}
    if not args.no_large and world == 1:
        if args.config != "30k-fmm5":
            sections["small_30k"] = system_section("30k-fmm5", dev, flush, args.steps,
                                                   args.model, oracle_check="solve")
        if args.config != "300k-fmm6":
            sections["precision_300k"] = system_section("300k-fmm6", dev, flush, 2,
                                                        args.model)
        sections["ingest_1m"] = ingest_section(dev)
    batched = batched_section(dev, 1, flush) if (not args.no_batched and world == 1) else None
    if rank != 0:
        return
    # against the reference: the oracle's FP64 operator applied to the headline
    # solution (timed: the CPU baseline sample) and the reference engine's summary
    cpu, vs_oracle = None, None
    if not args.no_cpu:
        P = oracle_port()
        r_o, t_o = oracle_residual(P, b, rhs, mu_head, summation, order)
        g = golden(args.config)
        applies = (g["iterations"] + 1) if g else (st64["fp64_applies"])
        cpu = {"value": t_o * applies, "unit": "s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"1 FMM apply B*mu of the {b.n:,}-site system by the oracle "
                         "(octree rebuilt, as the reference does per apply), OpenMP over all "
                         f"host threads, {t_o:.3f} s, x {applies} applies per reference solve"}
        vs_oracle = {"oracle_residual": r_o,
                     "reference_solution": vs_reference_solution(args.config, rhs, mu_head),
                     "plain_fp64_gpu_vs_reference_solution":
                         vs_reference_solution(args.config, rhs, mu64)}
    total = world
    line = {
        "metric": METRIC, "value": t_head, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_head * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded water box, 12 point charges)",
        "config": dict(workload_config(args.config, b.n),
                       l2="256 MB buffer written between timed steps; the system's "
                          "device data exceed L2" if b.n > 100000 else
                          "256 MB buffer written between timed steps",
                       parallelism=f"replicas x{world}" if world > 1 else "1 GPU"),
        "solves_per_s": total / t_head,
        "method": "mixed precision + learned guess/preconditioner" if lrn else
                  "mixed precision (no trained model found)",
        "plain_fp64_s": plain, "speedup_vs_plain_fp64": plain / t_head,
        "learned": lrn,
        "autotuned_fp32_apply_ms": tuned_ms,
        "iterations": {"fp32_applies": st["fp32_applies"],
                       "fp64_applies": st["fp64_applies"],
                       "plain_fp64_iterations": st64["fp64_applies"] - 1},
        "parity": parity,
        "vs_oracle": vs_oracle,
        "sections": sections or None,
        "batched": batched,
        "roofline": {"bound": "fp32", "kernel": near_kernel,
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak,
                     "traffic": profiled_traffic(prof) if prof else None,
                     "traffic_note": ("DRAM bytes per launch from the committed ncu capture "
                                      f"profiles/{prof}" +
                                      ("; mostly the output rows the gather pass adds"
                                       if sched["symmetric_near"] else "")) if prof else
                                     "no committed capture of this form and workload",
                     "schedule": sched,
                     "peak_kind": "measured FFMA probe (cppe_gpu_fma_peak), no FP32 CUDA-core "
                                  "figure in MEASURED_PEAKS.json",
                     "algorithmic": f"{alg_pairs} pairs x {FLOP_PER_PAIR} FLOP per launch"},
        "roofline_fp64": {"bound": "fp64", "achieved": achieved64, "peak": fp64_peak,
                          "unit": "TFLOP/s", "frac": achieved64 / fp64_peak},
        "phases_ms": {"fp32": tim32, "double_float_residual": timdd, "fp64": tim64},
        "m2l_translations_per_apply": m2l_pairs,
        "near_pairs_per_s": pairs_per_s,
        "peaks": {"hbm_gbs": pk.get("hbm_gbs"), "bf16_tflops": pk.get("bf16_tflops"),
                  "kind": pk_kind, "fp32_fma_tflops": fp32_peak, "fp64_fma_tflops": fp64_peak},
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": int(rhs.nbytes),
                "d2h_bytes_per_step": int(rhs.nbytes)},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="1m-fmm6", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched section")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in near-field / M2L schedule")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the extra 30k- and 300k-site sections")
    ap.add_argument("--no-fp64", action="store_true",
                    help="with --apply-only: skip the FP64 operator")
    ap.add_argument("--near-form", type=int, default=-1, choices=(-1, 0, 1, 2),
                    help="with --apply-only: FP32 near-field form (0 per target, 1 or 2 "
                         "symmetric with two or four sources a lane; -1 the built-in one)")
    ap.add_argument("--no-learned", action="store_true", help="skip the trained model")
    ap.add_argument("--model", default=os.path.join(ROOT, "cppe_gb300", "data",
                                                    "learned_water.npz"))
    ap.add_argument("--solve-only", action="store_true",
                    help="time the mixed solves only (no FP64, e2e or CPU legs)")
    ap.add_argument("--apply-only", type=int, default=0, metavar="K",
                    help="run K FP32 and K FP64 operator applies and print phase timings")
    ap.add_argument("--batch-only", action="store_true",
                    help="time the batched solve alone (no one-at-a-time FP64 solves)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.batch_only:
        import torch
        torch.cuda.set_device(0)
        flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda:0")
        print(json.dumps({"batch_only": batched_section(0, args.steps, flush, compare=False)}),
              flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
