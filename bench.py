#!/usr/bin/env python
"""Benchmark of the induced-dipole solve (time to a 1e-8 residual).

Workload (default): 10,000 rigid waters = 30,000 polarizable sites, FMM
expansion order 5, theta 0.5, ncrit 64, Thole damping a = 2.1304, one
right-hand side = field of 12 point charges + static multipole field, solved
from the reference's first-call guess alpha*F to ||F - B mu||_2 < 1e-8 with
the FP64 FMM operator.  A step is one complete solve.

value     mixed-precision solve (FP32 inner PCG + FP64 refinement), inputs and
          outputs resident on the GPU, CUDA events on the library's stream.
e2e       the same solve through the C ABI with host buffers
          (cppe_gpu_solve: H2D of F, D2H of mu inside the timed region).
plain     the plain FP64 GPU PCG (the reference's algorithm on the GPU) on the
          same system, reported next to the headline.

`--impl reference` times the reference algorithm on the host cores (the
oracle's C++ restatement with OpenMP, all threads) on the same workload.
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
    return b.external_field() + Fm


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def run_reference(args):
    """The reference algorithm on the host cores (oracle restatement)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    if not os.path.exists(O.PORT_LIB):
        O.build_port()
    P = O.port()
    b, summation, order = make_problem(args.config)
    fmm = summation == "fmm"
    sites = O.Sites(xyz=b.xyz, elements=b.elements, q=b.q, mu=b.mu, quad=b.quad, max_order=2,
                    alpha6=b.alpha6, polarizable=np.ones(b.n, np.int32), excl_ptr=b.excl_ptr,
                    excl_idx=b.excl_idx)
    rhs = b.external_field() + P.multipole_fields(sites, fmm=fmm, order=order)
    kw = dict(fmm=int(fmm), ncrit=64, order=order, theta=0.5, damping=2.1304, thresh=1e-8)
    for _ in range(args.warmup):
        P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, **kw)
    times, its = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        mu, it, hist, ok = P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, **kw)
        times.append(time.perf_counter() - t0)
        its.append(it)
    v = float(np.mean(times))
    cores = os.cpu_count()
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded water box, 12 point charges)",
        "config": dict(workload_config(args.config, b.n), parallelism="host threads"),
        "cpu_baseline": {"value": v, "unit": "s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full solves ({int(np.mean(its))} CG "
                                   "iterations each), OpenMP over all host threads"},
        "e2e": {"value": v, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_sample(b, rhs, summation, order):
    """One bounded CPU solve of the same workload (oracle restatement)."""
    from oracle import oracle as O
    if not os.path.exists(O.PORT_LIB):
        O.build_port()
    P = O.port()
    kw = dict(fmm=int(summation == "fmm"), ncrit=64, order=order, theta=0.5, damping=2.1304,
              thresh=1e-8)
    t0 = time.perf_counter()
    mu, it, hist, ok = P.solve(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, rhs, **kw)
    dt = time.perf_counter() - t0
    return {"value": dt, "unit": "s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"1 full solve of the same system ({it} CG iterations), OpenMP over all "
                      "host threads"}, mu


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
                "max_rnorm": bst["max_rnorm"]}
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
    return {"workload": "256 snapshots x 8 RHS, sites log-uniform 500-20,000 "
                        f"({int(sum(sizes))} sites, {int(sum(sizes)) * nrhs} site-RHS), direct "
                        "< 4,000 sites, FMM p5 above, mixed precision, tol 1e-8",
            "value": t_batch, "unit": "s", "solves": len(boxes) * nrhs,
            "plain_fp64_sequential_s": plain,
            "plain_fp64_note": "first RHS of each snapshot solved and timed one at a time, x8",
            "speedup_vs_plain_fp64": plain / t_batch,
            "fp32_applies": bst["fp32_applies"], "fp64_applies": bst["fp64_applies"],
            "max_fp64_residual": worst, "setup_s": setup, "autotune_s": tune,
            "fp32_apply_ms": tuned_ms}


def large_section(cfg, dev, flush, model_path=None, zero_guess=True):
    """One larger system solved once per arithmetic: plain FP64 PCG (from
    alpha*F and, optionally, from zero), mixed precision, and mixed precision
    with the trained model.  Errors of the mixed solutions against the FP64
    one: induced dipoles, polarization energy (-1/2 mu.E_ext), the induced
    field B mu and the FP64 residual."""
    import torch
    from cppe_gb300 import capi, learned
    t0 = time.perf_counter()
    b, summation, order = make_problem(cfg)
    rhs = static_rhs_gpu(b, summation, order)
    setup = time.perf_counter() - t0
    kw = dict(summation=capi.FMM, ncrit=64, order=order, theta=0.5, damp=True, thresh=1e-8,
              device=dev)
    d_rhs = torch.tensor(rhs, dtype=torch.float64, device=f"cuda:{dev}")
    d_mu = torch.zeros_like(d_rhs)
    E = b.external_field()
    out = {"workload": f"{cfg}: {CONFIGS[cfg][4]}, Thole damping, tol 1e-8", "sites": b.n,
           "setup_s": setup}

    def timed(sys_, make_guess=True):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t, _ = _event_time(torch.cuda.ExternalStream(sys_.stream()),
                           lambda: sys_.solve_device(d_rhs.data_ptr(), d_mu.data_ptr(),
                                                     make_guess=make_guess))
        return t, d_mu.cpu().numpy(), sys_.stats()

    s64 = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.FP64, **kw)
    t64, mu64, st64 = timed(s64)
    out["plain_fp64"] = {"s": t64, "iterations": st64["fp64_applies"] - 1}
    if zero_guess:
        tz, _, stz = timed(s64, make_guess=False)
        out["plain_fp64_zero_guess"] = {"s": tz, "iterations": stz["fp64_applies"]}
    Bmu64 = s64.apply(mu64)
    smx = capi.System(b.xyz, b.alpha6, b.excl_ptr, b.excl_idx, precision=capi.MIXED, **kw)
    t0 = time.perf_counter()
    out["autotune"] = {"apply_ms": smx.autotune(2), "s": time.perf_counter() - t0}  # set-up
    timed(smx)  # warm-up (first-use allocations)
    variants = [("mixed", None)]
    if model_path and os.path.exists(model_path):
        variants.append(("mixed_learned", learned.load(model_path, device=dev)))
    for name, model in variants:
        smx.set_model(model)
        if model is not None:
            timed(smx)
        t, mu, st = timed(smx)
        Bmu = s64.apply(mu)
        out[name] = {
            "s": t, "fp32_applies": st["fp32_applies"], "fp64_applies": st["fp64_applies"],
            "speedup_vs_plain_fp64": t64 / t,
            "error_vs_fp64": {
                "mu_maxabs": float(np.abs(mu - mu64).max()),
                "epol_hartree": float(abs(0.5 * (mu - mu64) @ E)),
                "induced_field_rel": float(np.linalg.norm(Bmu - Bmu64) / np.linalg.norm(Bmu64)),
                "fp64_residual": float(np.linalg.norm(rhs - Bmu))}}
    smx.set_model(None)
    smx.close()
    s64.close()
    return out


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
        t32 = smx.kernel_timings(capi.MIXED, reps=args.apply_only)
        tdd = smx.kernel_timings(DD_RESIDUAL, reps=args.apply_only)
        t64 = s64.kernel_timings(capi.FP64, reps=args.apply_only)
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
    if args.solve_only:
        # mixed solves only (with the model when given), e.g. for launch lists
        if args.model and os.path.exists(args.model) and not args.no_learned:
            from cppe_gb300 import learned
            smx.set_model(learned.load(args.model, device=dev))
        ts = []
        for k in range(args.warmup + args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t, _ = _event_time(ext, lambda: smx.solve_device(d_rhs.data_ptr(), d_mu.data_ptr(),
                                                             make_guess=True))
            if k >= args.warmup:
                ts.append(t)
        print(json.dumps({"solve_only": args.steps, "config": args.config, "ms": [t * 1e3 for t in ts],
                          "stats": smx.stats(), "learned": smx._model is not None
                          if hasattr(smx, "_model") else False}), flush=True)
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
    model = None
    if not args.no_learned and args.model and os.path.exists(args.model):
        from cppe_gb300 import learned
        model = learned.load(args.model, device=dev)
    smx.set_model(model)
    for _ in range(args.warmup):
        timed_solve(smx, ext)
        timed_solve(s64, ext64)
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

    # end to end through the C ABI with host buffers (same method)
    rhs_h = np.ascontiguousarray(rhs)
    e2e = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        mu_h, _, _, _ = smx.solve(rhs_h)
        e2e.append(time.perf_counter() - t0)
    e2e_v = float(np.mean(e2e))

    # the mixed solver without the model, for the learned part's gain
    without = None
    if model is not None:
        smx.set_model(None)
        timed_solve(smx, ext)
        tw = [timed_solve(smx, ext)[0] for _ in range(args.steps)]
        without = {"s": float(np.mean(tw)), "stats": smx.stats()}
    lrn = None
    if model is not None:
        lrn = {"with_model_s": t_head, "with_model_stats": st, "without_model_s": without["s"],
               "without_model_stats": without["stats"],
               "model": os.path.relpath(args.model, ROOT)}

    # plain FP64 GPU PCG on the same system
    t64 = []
    for _ in range(max(1, min(args.steps, 3))):
        t, it64 = timed_solve(s64, ext64)
        t64.append(t)
    mu64 = d_mu.cpu().numpy()
    st64 = s64.stats()
    plain = float(np.mean(t64))

    # roofline of the dominant kernel (FP32 near-field pair pass)
    tim32, alg_pairs, m2l_pairs = smx.kernel_timings(capi.MIXED, reps=5)
    tim64, _, _ = s64.kernel_timings(capi.FP64, reps=3)
    timdd, _, _ = smx.kernel_timings(DD_RESIDUAL, reps=3)
    fp32_peak = capi.fma_peak_tflops(False, dev)
    fp64_peak = capi.fma_peak_tflops(True, dev)
    achieved = alg_pairs * FLOP_PER_PAIR / (tim32["near"] * 1e-3) / 1e12
    achieved64 = alg_pairs * FLOP_PER_PAIR / (tim64["near"] * 1e-3) / 1e12
    pairs_per_s = {"fp32": alg_pairs / (tim32["near"] * 1e-3),
                   "double_float": alg_pairs / (timdd["near"] * 1e-3),
                   "fp64": alg_pairs / (tim64["near"] * 1e-3)}
    pk, pk_kind = peaks()

    resid = float(np.linalg.norm(rhs - s64.apply(mu_head)))
    E = b.external_field()
    de = float(abs(0.5 * (mu_head - mu64) @ E))
    batched = batched_section(dev, 1, flush) if (not args.no_batched and world == 1) else None
    large = {}
    if not args.no_large and world == 1:
        large["precision_300k"] = large_section("300k-fmm6", dev, flush, zero_guess=False)
        large["learned_1m"] = large_section("1m-fmm6", dev, flush, model_path=args.model)
    if rank != 0:
        return
    cpu, _ = cpu_baseline_sample(b, rhs, summation, order) if not args.no_cpu else (None, None)
    total = world
    line = {
        "metric": METRIC, "value": t_head, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_head * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded water box, 12 point charges)",
        "config": dict(workload_config(args.config, b.n),
                       l2="256 MB buffer written between timed steps",
                       parallelism=f"replicas x{world}" if world > 1 else "1 GPU"),
        "solves_per_s": total / t_head,
        "method": "mixed precision + learned guess/preconditioner" if lrn else
                  "mixed precision (no trained model found)",
        "plain_fp64_s": plain, "speedup_vs_plain_fp64": plain / t_head,
        "learned": lrn,
        "autotuned_fp32_apply_ms": tuned_ms,
        "iterations": {"fp32_applies": st["fp32_applies"],
                       "fp64_applies": st["fp64_applies"],
                       "plain_fp64_iterations": st64["fp64_applies"]},
        "parity": {"fp64_residual": resid, "mu_maxabs_vs_fp64": float(
            np.abs(mu_head - mu64).max()), "epol_diff_hartree": de},
        "batched": batched,
        "large": large or None,
        "roofline": {"bound": "fp32", "kernel": "k_p2p32_m1<true> (FP32 dipole near field)",
                     "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": achieved / fp32_peak,
                     "traffic": profiled_traffic("k_p2p32_m1_30k_sites.md")
                     if args.config == "30k-fmm5" else None,
                     "traffic_note": "DRAM bytes per launch from the committed ncu capture of "
                                     "this workload (profiles/k_p2p32_m1_30k_sites.md); the "
                                     "kernel's working set is L2-resident",
                     "peak_kind": "measured FFMA probe (cppe_gpu_fma_peak), no FP32 CUDA-core "
                                  "figure in MEASURED_PEAKS.json",
                     "algorithmic": f"{alg_pairs} pairs x {FLOP_PER_PAIR} FLOP per launch"},
        "roofline_fp64": {"bound": "fp64", "achieved": achieved64, "peak": fp64_peak,
                          "unit": "TFLOP/s", "frac": achieved64 / fp64_peak},
        "phases_ms": {"fp32": tim32, "double_float_residual": timdd, "fp64": tim64},
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
    ap.add_argument("--config", default="30k-fmm5", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched section")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the built-in near-field / M2L schedule")
    ap.add_argument("--no-large", action="store_true",
                    help="skip the 300k- and 1M-site sections")
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
