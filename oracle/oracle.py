"""Test infrastructure: the CPU oracle for the induced-dipole hot path.

Nothing in the product imports this module.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py`` (its ``cpu_baseline`` leg and the
``--impl reference`` arm) use it, and only as the checker / the timed CPU
baseline.

Two libraries sit behind it:

* ``_build/libcppe_oracle.so`` -- ``cppe_oracle.cc``, a C++ restatement of the
  reference algorithm (tree, interaction lists, Cartesian FMM operators, direct
  sums, MultipoleFields, BMatrix, the PCG).  Built on every machine.
* ``_ref/libcppe_ref.so`` -- the reference's own ``src/core/fmm`` sources
  compiled in place (see ``Makefile``), wrapped by ``ref_glue.cc``.  Exists only
  where the reference source tree is mounted; used to pin the restatement.

The restatement is pinned against the reference's golden vectors
(``tests/golden/fmuls_loprop_solvated_20.txt.gz``,
``tests/golden/ref_fmm_errors.csv.gz``) and, where ``_ref`` exists, against the
reference build itself.
"""
from __future__ import annotations

import ctypes
import gzip
import os
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "libcppe_oracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libcppe_ref.so")

# potfile_reader.cc:10
ANG2BOHR = 1.8897261246


@dataclass
class Sites:
    """Flat site arrays as read from a potfile (units: bohr, a.u.)."""

    xyz: np.ndarray                     # (n, 3)
    elements: list
    q: np.ndarray                       # (n,)
    mu: np.ndarray                      # (n, 3)
    quad: np.ndarray                    # (n, 6) traceless, xx xy xz yy yz zz
    max_order: int
    alpha6: np.ndarray                  # (n, 6) upper triangle
    polarizable: np.ndarray             # (n,) int32
    excl_ptr: np.ndarray                # (n+1,) int32 CSR
    excl_idx: np.ndarray                # int32, 0-based global site indices
    orders_present: list = field(default_factory=list)

    @property
    def n(self):
        return self.xyz.shape[0]

    @property
    def alpha_iso(self):
        return (self.alpha6[:, 0] + self.alpha6[:, 3] + self.alpha6[:, 5]) / 3.0


def _open(path):
    return gzip.open(path, "rt") if path.endswith(".gz") else open(path)


def read_potfile(path: str) -> Sites:
    """Restatement of PotfileReader::read (src/core/potfile_reader.cc:31-179)."""
    with _open(path) as f:
        lines = f.read().splitlines()
    n = 0
    xyz = elements = None
    q = mu = quad = alpha6 = pol = None
    excl = None
    max_order = 0
    orders = []
    i = 0
    while i < len(lines):
        line = lines[i]
        if "@COORDINATES" in line:
            n = int(lines[i + 1].split()[0])
            unit = lines[i + 2].strip()
            if unit == "AA":
                conv = ANG2BOHR
            elif unit == "AU":
                conv = 1.0
            else:
                raise RuntimeError("Invalid unit for potential file.")
            rows = [lines[i + 3 + k].split() for k in range(n)]
            elements = [r[0] for r in rows]
            xyz = np.array([[float(r[1]), float(r[2]), float(r[3])] for r in rows]) * conv
            q = np.zeros(n)
            mu = np.zeros((n, 3))
            quad = np.zeros((n, 6))
            alpha6 = np.zeros((n, 6))
            pol = np.zeros(n, dtype=np.int32)
            excl = [[] for _ in range(n)]
            i += 3 + n
            continue
        if "ORDER" in line:
            tok = line.split()
            if len(tok) == 2:
                order = int(tok[1])
                cnt = int(lines[i + 1])
                ncomp = (order + 1) * (order + 2) // 2
                for k in range(cnt):
                    r = lines[i + 2 + k].split()
                    s = int(r[0]) - 1
                    vals = np.array([float(v) for v in r[1:1 + ncomp]])
                    if order == 0:
                        q[s] = vals[0]
                    elif order == 1:
                        mu[s] = vals
                    elif order == 2:
                        tr = (vals[0] + vals[3] + vals[5]) / 3.0   # Multipole::remove_trace
                        vals[[0, 3, 5]] -= tr
                        quad[s] = vals
                    else:
                        raise RuntimeError("multipole order > 2 is not supported")
                max_order = max(max_order, order)
                orders.append(order)
                i += 2 + cnt
                continue
            elif len(tok) == 3:
                if int(tok[1]) != 1 or int(tok[2]) != 1:
                    raise RuntimeError("Only dipole-dipole polarizabilities are currently supported.")
                cnt = int(lines[i + 1])
                for k in range(cnt):
                    r = lines[i + 2 + k].split()
                    s = int(r[0]) - 1
                    if pol[s]:
                        raise RuntimeError("Potential can only have one polarizability.")
                    alpha6[s] = [float(v) for v in r[1:7]]
                    pol[s] = 1
                i += 2 + cnt
                continue
            else:
                raise RuntimeError("Invalid number in potfile ORDER.")
        if "EXCLISTS" in line:
            cnt = int(lines[i + 1].split()[0])
            for k in range(cnt):
                r = lines[i + 2 + k].split()
                s = int(r[0]) - 1
                for v in r[1:]:
                    e = int(v) - 1
                    if e >= 0:
                        excl[s].append(e)
            i += 2 + cnt
            continue
        i += 1
    ptr = np.zeros(n + 1, dtype=np.int32)
    ptr[1:] = np.cumsum([len(e) for e in excl])
    idx = np.array([v for e in excl for v in e], dtype=np.int32)
    return Sites(xyz=xyz, elements=elements, q=q, mu=mu, quad=quad, max_order=max_order,
                 alpha6=alpha6, polarizable=pol, excl_ptr=ptr, excl_idx=idx,
                 orders_present=orders)


# ----------------------------------------------------------------------------
# ctypes plumbing
# ----------------------------------------------------------------------------
_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_L = ctypes.POINTER(ctypes.c_long)


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(_D)


def _ip(a):
    if a is None:
        return None
    return a.ctypes.data_as(_I)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.int32)


class _Lib:
    prefix = ""

    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)
        p = self.prefix
        f = getattr(self.lib, p + "field")
        f.argtypes = [ctypes.c_int, ctypes.c_int, _D, _D, _I, _D, _I, _I, ctypes.c_int,
                      ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double, _D]
        f = getattr(self.lib, p + "multipole_fields")
        f.argtypes = [ctypes.c_int, _D, _D, _D, _D, ctypes.c_int, _I, _D, _I, _I,
                      ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                      ctypes.c_double, _D]
        f = getattr(self.lib, p + "bmatrix_apply")
        f.argtypes = [ctypes.c_int, _D, _D, _I, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                      ctypes.c_double, ctypes.c_double, _D, _D]
        f = getattr(self.lib, p + "solve")
        f.argtypes = [ctypes.c_int, _D, _D, _I, _I, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                      ctypes.c_double, ctypes.c_double, _D, _D, ctypes.c_int,
                      ctypes.c_double, ctypes.c_int, _D, _I, _D]
        f = getattr(self.lib, p + "tree_info")
        f.argtypes = [ctypes.c_int, _D, ctypes.c_int, ctypes.c_int, ctypes.c_double, _I,
                      _L, _L]
        f = getattr(self.lib, p + "tree_lists")
        f.argtypes = [ctypes.c_int, _D, ctypes.c_int, ctypes.c_int, ctypes.c_double, _D,
                      _I, _I, _I, _I, _I, _I, _I]

    def _fn(self, name):
        return getattr(self.lib, self.prefix + name)

    # -- Tree<m,3>::compute_field_{exact,fmm} ---------------------------------
    def field(self, m, xyz, S, *, polarizable=None, alpha_iso=None, excl_ptr=None,
              excl_idx=None, fmm=False, ncrit=64, order=5, theta=0.5, damping=0.0):
        xyz = _f64(xyz)
        n = xyz.shape[0]
        S = _f64(S)
        F = np.zeros(3 * n)
        rc = self._fn("field")(m, n, _dp(xyz), _dp(S), _ip(_i32(polarizable)),
                               _dp(_f64(alpha_iso)), _ip(_i32(excl_ptr)),
                               _ip(_i32(excl_idx)), int(fmm), ncrit, order, theta,
                               damping, _dp(F))
        if rc:
            raise RuntimeError(f"oracle field failed: {rc}")
        return F

    # -- MultipoleFields::compute ----------------------------------------------
    def multipole_fields(self, sites: Sites, *, fmm=False, ncrit=64, order=5, theta=0.5,
                         damping=0.0):
        n = sites.n
        F = np.zeros(3 * n)
        rc = self._fn("multipole_fields")(
            n, _dp(_f64(sites.xyz)), _dp(_f64(sites.q)), _dp(_f64(sites.mu)),
            _dp(_f64(sites.quad)), sites.max_order, _ip(_i32(sites.polarizable)),
            _dp(_f64(sites.alpha_iso)), _ip(_i32(sites.excl_ptr)), _ip(_i32(sites.excl_idx)),
            int(fmm), ncrit, order, theta, damping, _dp(F))
        if rc:
            raise RuntimeError(f"oracle multipole_fields failed: {rc}")
        return F

    # -- BMatrix::apply --------------------------------------------------------
    def bmatrix_apply(self, xyz, alpha6, excl_ptr, excl_idx, vec, *, fmm=False, ncrit=64,
                      order=5, theta=0.5, damping=0.0):
        xyz = _f64(xyz)
        n = xyz.shape[0]
        out = np.zeros(3 * n)
        rc = self._fn("bmatrix_apply")(n, _dp(xyz), _dp(_f64(alpha6)), _ip(_i32(excl_ptr)),
                                       _ip(_i32(excl_idx)), int(fmm), ncrit, order, theta,
                                       damping, _dp(_f64(vec)), _dp(out))
        if rc:
            raise RuntimeError(f"oracle bmatrix_apply failed: {rc}")
        return out

    # -- InducedMoments::compute -----------------------------------------------
    def solve(self, xyz, alpha6, excl_ptr, excl_idx, rhs, *, guess=None, make_guess=True,
              thresh=1e-8, maxiter=50, fmm=False, ncrit=64, order=5, theta=0.5,
              damping=0.0):
        xyz = _f64(xyz)
        n = xyz.shape[0]
        mu = np.zeros(3 * n)
        it = ctypes.c_int(0)
        hist = np.zeros(max(maxiter, 1))
        rc = self._fn("solve")(n, _dp(xyz), _dp(_f64(alpha6)), _ip(_i32(excl_ptr)),
                               _ip(_i32(excl_idx)), int(fmm), ncrit, order, theta, damping,
                               _dp(_f64(rhs)), _dp(_f64(guess)), int(make_guess), thresh,
                               maxiter, _dp(mu), ctypes.byref(it), _dp(hist))
        return mu, it.value, hist[: it.value], rc == 0

    # -- tree / interaction lists ------------------------------------------------
    def tree_lists(self, xyz, ncrit=64, order=5, theta=0.5):
        xyz = _f64(xyz)
        n = xyz.shape[0]
        nc = ctypes.c_int(0)
        nm = ctypes.c_long(0)
        npp = ctypes.c_long(0)
        self._fn("tree_info")(n, _dp(xyz), ncrit, order, theta, ctypes.byref(nc),
                              ctypes.byref(nm), ctypes.byref(npp))
        nc, nm, npp = nc.value, nm.value, npp.value
        cxyzr = np.zeros((nc, 4))
        parent = np.zeros(nc, np.int32)
        level = np.zeros(nc, np.int32)
        nchild = np.zeros(nc, np.int32)
        nleaf = np.zeros(nc, np.int32)
        leaves = np.zeros((nc, ncrit), np.int32)
        m2l = np.zeros((nm, 2), np.int32)
        p2p = np.zeros((npp, 2), np.int32)
        self._fn("tree_lists")(n, _dp(xyz), ncrit, order, theta, _dp(cxyzr), _ip(parent),
                               _ip(level), _ip(nchild), _ip(nleaf), _ip(leaves), _ip(m2l),
                               _ip(p2p))
        return dict(cells=cxyzr, parent=parent, level=level, nchild=nchild, nleaf=nleaf,
                    leaves=leaves, m2l=m2l, p2p=p2p)


class PortOracle(_Lib):
    """The C++ restatement (cppe_oracle.cc)."""

    prefix = "orc_"

    def __init__(self, path=PORT_LIB):
        super().__init__(path)


class RefOracle(_Lib):
    """The reference's own sources compiled in place (ref_glue.cc)."""

    prefix = "ref_"

    def __init__(self, path=REF_LIB):
        super().__init__(path)


def build_port(force=False):
    """Compile the restatement (portable flags) into oracle/_build."""
    import subprocess
    subprocess.run(["make", "-s", "-C", HERE, "port"] + (["-B"] if force else []),
                   check=True)


def build_ref():
    """Compile the reference sources in place; only where they are mounted."""
    import subprocess
    ref = os.environ.get("CPPE_REFERENCE_DIR", "/root/reference")
    if not os.path.isdir(os.path.join(ref, "src", "core", "fmm")):
        return False
    subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True,
                   stderr=subprocess.DEVNULL)
    return True


def port():
    return PortOracle()


def ref():
    return RefOracle() if os.path.exists(REF_LIB) else None
