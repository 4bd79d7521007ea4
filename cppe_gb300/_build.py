"""In-tree build of the native parts of cppe_gb300.

* ``libcppe_gpu.so`` -- the CUDA kernels and the C ABI of ``include/cppe_gpu.h``
  (nvcc, sm_103a only, CUDA runtime linked statically).
* ``pycppe*.so`` -- the C++ host layer (``csrc/host``: the reference's class
  interface) and its pybind11 module (``csrc/python``), linked against
  ``libcppe_gpu.so`` through an ``$ORIGIN`` rpath.  pybind11 comes from the
  headers bundled with PyTorch, which exist wherever torch is installed.

Translation units compile in parallel and are skipped when their object is
newer than every source and header they may include.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libcppe_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"] + ARCH
# Host-only sources: the tree build must not contract floating-point
# expressions (see csrc/tree.cc).
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cppe_gb300")


def _cuda_home():
    return os.path.dirname(os.path.dirname(_nvcc()))


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _headers(d):
    return glob.glob(os.path.join(d, "*.h")) + glob.glob(os.path.join(d, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def build_gpu_lib(jobs=8, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    # straight-line fixed-order M2L translations (rewritten only when changed)
    _run([sys.executable, os.path.join(CSRC, "gen_m2l.py"), os.path.join(CSRC, "m2l_gen.cuh")])
    nvcc = _nvcc()
    hdrs = _headers(CSRC)
    steps = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([nvcc, *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cc"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append(["g++", *CXX_FLAGS, "-I", INCLUDE, "-I", CSRC,
                          "-I", os.path.join(_cuda_home(), "include"), "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for r in ex.map(_run, steps):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
    if _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-cudart", "static"])
    return LIB


def _py_ext_suffix():
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def build_python_module(jobs=8, verbose=False):
    import torch.utils.cpp_extension as ce  # only for the bundled pybind11 headers

    torch_inc = ce.include_paths()
    py_inc = sysconfig.get_paths()["include"]
    host_dir = os.path.join(CSRC, "host")
    py_dir = os.path.join(CSRC, "python")
    hdrs = glob.glob(os.path.join(host_dir, "*.hh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    inc = ["-I", INCLUDE, "-I", host_dir, "-I", py_inc] + sum((["-isystem", d] for d in torch_inc), [])
    out = os.path.join(PKG, "pycppe" + _py_ext_suffix())
    steps, objs = [], []
    for src in sorted(glob.glob(os.path.join(host_dir, "*.cc")) + glob.glob(os.path.join(py_dir, "*.cc"))):
        obj = os.path.join(BUILD, "py_" + os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append(["g++", "-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden",
                          "-DPYBIND11_DETAILED_ERROR_MESSAGES", *inc, "-c", src, "-o", obj])
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        for r in ex.map(_run, steps):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr, file=sys.stderr)
    if _stale(out, objs + [LIB]):
        _run(["g++", "-shared", "-o", out, *objs, "-L", PKG, "-lcppe_gpu",
              "-Wl,-rpath,$ORIGIN"])
    return out


def build(verbose=False):
    build_gpu_lib(verbose=verbose)
    build_python_module(verbose=verbose)


if __name__ == "__main__":
    build(verbose=True)
