"""ctypes binding of libcppe_gpu.so (the C ABI of include/cppe_gpu.h).

This is the binding a Python caller (or the reference's own code through
ctypes) uses to reach the GPU library without the pybind11 layer; tests and
bench.py use it too."""
import ctypes
import os
import re

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "cppe_gb300", "libcppe_gpu.so")
HEADER = os.path.join(ROOT, "include", "cppe_gpu.h")

OK, NOT_CONVERGED, INVALID_ARG, CUDA_ERROR, TIMEOUT, NO_DEVICE = range(6)
DIRECT, FMM = 0, 1
FP64, MIXED = 0, 1

D = ctypes.POINTER(ctypes.c_double)
I = ctypes.POINTER(ctypes.c_int)
L = ctypes.POINTER(ctypes.c_long)


class Options(ctypes.Structure):
    _fields_ = [("summation", ctypes.c_int), ("tree_ncrit", ctypes.c_int),
                ("tree_expansion_order", ctypes.c_int), ("theta", ctypes.c_double),
                ("damp", ctypes.c_int), ("damping_factor", ctypes.c_double),
                ("induced_thresh", ctypes.c_double), ("maxiter", ctypes.c_int),
                ("precision", ctypes.c_int), ("device", ctypes.c_int)]


def declared_functions():
    """Names of the functions declared in include/cppe_gpu.h."""
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cppe_gpu_\w+)\s*\(", src)))


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIB_PATH)
        l = _lib
        l.cppe_gpu_default_options.argtypes = [ctypes.POINTER(Options)]
        l.cppe_gpu_default_options.restype = None
        l.cppe_gpu_last_error.argtypes = [ctypes.c_char_p, ctypes.c_size_t]
        l.cppe_gpu_create.argtypes = [ctypes.c_int, D, D, I, I, ctypes.POINTER(Options),
                                      ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_destroy.argtypes = [ctypes.c_void_p]
        for f in ("cppe_gpu_bmatrix_apply", "cppe_gpu_bmatrix_apply_fp32",
                  "cppe_gpu_bmatrix_apply_dd",
                  "cppe_gpu_apply_diagonal", "cppe_gpu_apply_diagonal_inverse"):
            getattr(l, f).argtypes = [ctypes.c_void_p, D, D]
        l.cppe_gpu_to_dense.argtypes = [ctypes.c_void_p, D]
        l.cppe_gpu_direct_inverse.argtypes = [ctypes.c_void_p, D]
        l.cppe_gpu_solve.argtypes = [ctypes.c_void_p, D, D, ctypes.c_int, D, I, D, ctypes.c_int]
        l.cppe_gpu_last_solve_stats.argtypes = [ctypes.c_void_p, D, I, I]
        l.cppe_gpu_multipole_fields.argtypes = [
            ctypes.c_int, D, D, D, D, ctypes.c_int, I, D, I, I, ctypes.c_int, ctypes.c_int,
            ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, D]
        l.cppe_gpu_tree_info.argtypes = [ctypes.c_int, D, ctypes.c_int, ctypes.c_double, I, I,
                                         L, L, L]
        l.cppe_gpu_tree_lists.argtypes = [ctypes.c_int, D, ctypes.c_int, ctypes.c_double, I, I]
        l.cppe_gpu_tree_vectors.argtypes = [ctypes.c_int, D, ctypes.c_int, ctypes.c_double, I, L]
        l.cppe_gpu_device_count.argtypes = [I]
        l.cppe_gpu_batch_create.argtypes = [ctypes.c_int, I, D, D, I, I, ctypes.c_int,
                                            ctypes.c_int, ctypes.POINTER(Options),
                                            ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_batch_destroy.argtypes = [ctypes.c_void_p]
        l.cppe_gpu_batch_solve.argtypes = [ctypes.c_void_p, D, D, I]
        l.cppe_gpu_batch_solve_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                                  ctypes.c_void_p, I]
        l.cppe_gpu_solve_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p, I, D, ctypes.c_int]
        l.cppe_gpu_bmatrix_apply_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                                    ctypes.c_void_p]
        l.cppe_gpu_stream.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_launch_count.argtypes = [ctypes.POINTER(ctypes.c_longlong)]
        l.cppe_gpu_kernel_timings.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, D,
                                              ctypes.POINTER(ctypes.c_longlong),
                                              ctypes.POINTER(ctypes.c_longlong)]
        l.cppe_gpu_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int, D]
        l.cppe_gpu_batch_stats.argtypes = [ctypes.c_void_p, I, I, D]
        l.cppe_gpu_batch_host_waits.argtypes = [ctypes.c_void_p, I]
        l.cppe_gpu_batch_stream.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_batch_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int, D]
        F = ctypes.POINTER(ctypes.c_float)
        l.cppe_gpu_mlp_nparams.argtypes = [I]
        l.cppe_gpu_mlp_create.argtypes = [ctypes.c_int, ctypes.c_uint,
                                          ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_mlp_destroy.argtypes = [ctypes.c_void_p]
        l.cppe_gpu_mlp_get_params.argtypes = [ctypes.c_void_p, F]
        l.cppe_gpu_mlp_set_params.argtypes = [ctypes.c_void_p, F]
        l.cppe_gpu_mlp_normalization.argtypes = [ctypes.c_void_p, F, F, F, F]
        l.cppe_gpu_mlp_forward.argtypes = [ctypes.c_void_p, ctypes.c_int, F, F]
        l.cppe_gpu_mlp_infer.argtypes = [ctypes.c_void_p, ctypes.c_int, F, F]
        l.cppe_gpu_mlp_loss_grad.argtypes = [ctypes.c_void_p, ctypes.c_int, F, F,
                                             ctypes.c_float, D, F]
        l.cppe_gpu_mlp_train.argtypes = [ctypes.c_void_p, ctypes.c_int, F, F, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                         ctypes.c_uint, D]
        l.cppe_gpu_learned_data.argtypes = [ctypes.c_void_p, D, D, F, F]
        l.cppe_gpu_set_model.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        l.cppe_gpu_potfile_read.argtypes = [ctypes.c_char_p, ctypes.POINTER(ctypes.c_void_p)]
        l.cppe_gpu_potfile_info.argtypes = [ctypes.c_void_p, I, I, I, L]
        l.cppe_gpu_potfile_arrays.argtypes = [ctypes.c_void_p, D, D, D, D, D, I, I, I,
                                              ctypes.c_char_p]
        l.cppe_gpu_potfile_free.argtypes = [ctypes.c_void_p]
    return _lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def fp(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


N_IN, N_OUT, TROW = 64, 4, 24


class Mlp:
    """The learned-guess network (cppe_gpu_mlp) on the GPU."""

    def __init__(self, seed=0, device=0):
        h = ctypes.c_void_p()
        check(lib().cppe_gpu_mlp_create(device, seed, ctypes.byref(h)))
        self.h = h
        n = ctypes.c_int(0)
        lib().cppe_gpu_mlp_nparams(ctypes.byref(n))
        self.nparams = n.value

    def close(self):
        if self.h:
            lib().cppe_gpu_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def params(self):
        out = np.zeros(self.nparams, np.float32)
        check(lib().cppe_gpu_mlp_get_params(self.h, fp(out)))
        return out

    @params.setter
    def params(self, p):
        p = f32(p)
        assert p.size == self.nparams
        check(lib().cppe_gpu_mlp_set_params(self.h, fp(p)))

    def set_normalization(self, mean, inv_std):
        check(lib().cppe_gpu_mlp_normalization(self.h, fp(f32(mean)), fp(f32(inv_std)), None,
                                               None))

    def normalization(self):
        m = np.zeros(N_IN, np.float32)
        s = np.zeros(N_IN, np.float32)
        check(lib().cppe_gpu_mlp_normalization(self.h, None, None, fp(m), fp(s)))
        return m, s

    def forward(self, feats):
        feats = f32(feats)
        y = np.zeros((feats.shape[0], N_OUT), np.float32)
        check(lib().cppe_gpu_mlp_forward(self.h, feats.shape[0], fp(feats), fp(y)))
        return y

    def infer(self, feats):
        """The tensor-core inference kernel (TF32 operands, FP32 accumulation)."""
        feats = f32(feats)
        y = np.zeros((feats.shape[0], N_OUT), np.float32)
        check(lib().cppe_gpu_mlp_infer(self.h, feats.shape[0], fp(feats), fp(y)))
        return y

    def loss_grad(self, feats, rows, lam=1.0):
        feats, rows = f32(feats), f32(rows)
        g = np.zeros(self.nparams, np.float32)
        l = ctypes.c_double(0)
        check(lib().cppe_gpu_mlp_loss_grad(self.h, feats.shape[0], fp(feats), fp(rows), lam,
                                           ctypes.byref(l), fp(g)))
        return l.value, g

    def train(self, feats, rows, steps, batch=4096, lr=3e-3, lam=1.0, seed=0):
        feats, rows = f32(feats), f32(rows)
        hist = np.zeros(max(steps, 1))
        check(lib().cppe_gpu_mlp_train(self.h, feats.shape[0], fp(feats), fp(rows), steps,
                                       batch, lr, lam, seed, dp(hist)))
        return hist[:steps]


class Batch:
    """One cppe_gpu_batch: snapshots x right-hand sides solved together.

    systems: list of objects with xyz (n,3), alpha6 (n,6), excl_ptr, excl_idx.
    rhs / mu layout: [system][rhs][3 n_s] concatenated."""

    def __init__(self, systems, nrhs, direct_below=4000, **opts):
        off = np.zeros(len(systems) + 1, np.int32)
        off[1:] = np.cumsum([s.xyz.shape[0] for s in systems])
        self.off = off
        self.nrhs = nrhs
        xyz = f64(np.concatenate([s.xyz for s in systems]))
        a6 = f64(np.concatenate([s.alpha6 for s in systems]))
        ep = [0]
        ei = []
        for s in systems:
            ep.extend(int(ep[-1]) + np.asarray(s.excl_ptr[1:]) - s.excl_ptr[0])
            ei.append(np.asarray(s.excl_idx))
        ep = i32(ep)
        ei = i32(np.concatenate(ei)) if ei else i32([0])
        self._keep = [off, xyz, a6, ep, ei]
        self.opts = options(**opts)
        h = ctypes.c_void_p()
        check(lib().cppe_gpu_batch_create(len(systems), ip(off), dp(xyz), dp(a6), ip(ep), ip(ei),
                                          nrhs, direct_below, ctypes.byref(self.opts),
                                          ctypes.byref(h)))
        self.h = h
        self.nseg = len(systems) * nrhs

    def close(self):
        if self.h:
            lib().cppe_gpu_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, rhs, allow_not_converged=False):
        rhs = f64(rhs)
        mu = np.zeros_like(rhs)
        its = np.zeros(self.nseg, np.int32)
        rc = lib().cppe_gpu_batch_solve(self.h, dp(rhs), dp(mu), ip(its))
        check(rc, (OK, NOT_CONVERGED) if allow_not_converged else (OK,))
        return mu, its

    def solve_device(self, d_rhs, d_mu):
        its = np.zeros(self.nseg, np.int32)
        lib().cppe_gpu_batch_solve_device.argtypes = [ctypes.c_void_p, ctypes.c_void_p,
                                                      ctypes.c_void_p, I]
        check(lib().cppe_gpu_batch_solve_device(self.h, d_rhs, d_mu, ip(its)))
        return its

    def stats(self):
        a, b, r = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0)
        check(lib().cppe_gpu_batch_stats(self.h, ctypes.byref(a), ctypes.byref(b),
                                         ctypes.byref(r)))
        w = ctypes.c_int(0)
        check(lib().cppe_gpu_batch_host_waits(self.h, ctypes.byref(w)))
        return dict(fp64_applies=a.value, fp32_applies=b.value, max_rnorm=r.value,
                    host_waits=w.value)

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().cppe_gpu_batch_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def autotune(self, reps=3):
        """Keeps the fastest near-field / M2L schedule and far-field stream
        priority for this batch's FP32 operator; returns its apply time (ms)."""
        ms = ctypes.c_double(0)
        check(lib().cppe_gpu_batch_autotune(self.h, reps, ctypes.byref(ms)))
        return ms.value


def launch_count():
    c = ctypes.c_longlong(0)
    lib().cppe_gpu_launch_count(ctypes.byref(c))
    return c.value


def fma_peak_tflops(fp64=False, device=0):
    t = ctypes.c_double(0)
    check(lib().cppe_gpu_fma_peak(device, int(fp64), ctypes.byref(t)))
    return t.value


def last_error():
    buf = ctypes.create_string_buffer(1024)
    lib().cppe_gpu_last_error(buf, 1024)
    return buf.value.decode()


def check(rc, allow=(OK,)):
    if rc not in allow:
        raise RuntimeError(f"cppe_gpu status {rc}: {last_error()}")
    return rc


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def dp(a):
    return None if a is None else a.ctypes.data_as(D)


def ip(a):
    return None if a is None else a.ctypes.data_as(I)


def options(summation=DIRECT, ncrit=64, order=5, theta=0.5, damp=False, damping=2.1304,
            thresh=1e-8, maxiter=50, precision=FP64, device=0):
    o = Options()
    lib().cppe_gpu_default_options(ctypes.byref(o))
    o.summation, o.tree_ncrit, o.tree_expansion_order, o.theta = summation, ncrit, order, theta
    o.damp, o.damping_factor, o.induced_thresh, o.maxiter = int(damp), damping, thresh, maxiter
    o.precision, o.device = precision, device
    return o


def device_count():
    c = ctypes.c_int(0)
    lib().cppe_gpu_device_count(ctypes.byref(c))
    return c.value


class System:
    """One cppe_gpu_system."""

    def __init__(self, xyz, alpha6, excl_ptr=None, excl_idx=None, **opts):
        self._keep = [f64(xyz), f64(alpha6), i32(excl_ptr) if excl_ptr is not None else None,
                      i32(excl_idx) if excl_idx is not None else None]
        self.n = self._keep[0].shape[0]
        self.opts = options(**opts)
        self.device = self.opts.device
        h = ctypes.c_void_p()
        check(lib().cppe_gpu_create(self.n, dp(self._keep[0]), dp(self._keep[1]),
                                    ip(self._keep[2]), ip(self._keep[3]),
                                    ctypes.byref(self.opts), ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            lib().cppe_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def apply(self, v, fp32=False, dd=False):
        v = f64(v)
        out = np.zeros_like(v)
        fn = (lib().cppe_gpu_bmatrix_apply_fp32 if fp32 else
              lib().cppe_gpu_bmatrix_apply_dd if dd else lib().cppe_gpu_bmatrix_apply)
        check(fn(self.h, dp(v), dp(out)))
        return out

    def apply_diagonal(self, v, inverse=False):
        v = f64(v)
        out = np.zeros_like(v)
        fn = lib().cppe_gpu_apply_diagonal_inverse if inverse else lib().cppe_gpu_apply_diagonal
        check(fn(self.h, dp(v), dp(out)))
        return out

    def dense(self):
        out = np.zeros((3 * self.n, 3 * self.n))
        check(lib().cppe_gpu_to_dense(self.h, dp(out)))
        return out

    def inverse(self):
        out = np.zeros((3 * self.n, 3 * self.n))
        check(lib().cppe_gpu_direct_inverse(self.h, dp(out)))
        return out

    def solve(self, rhs, guess=None, make_guess=True, allow_not_converged=False, out=None):
        """out: optional float64 array of rhs's size that receives mu (for
        example a view of pinned host memory, which the copies then use
        directly)."""
        rhs = f64(rhs)
        if out is None:
            mu = np.zeros_like(rhs)
        else:
            if out.dtype != np.float64 or out.size != rhs.size or not out.flags.c_contiguous:
                raise ValueError("out must be a contiguous float64 array of the rhs's size")
            mu = out
        it = ctypes.c_int(0)
        cap = self.opts.maxiter + 64
        hist = np.zeros(cap)
        g = f64(guess) if guess is not None else None
        rc = lib().cppe_gpu_solve(self.h, dp(rhs), dp(g), int(make_guess), dp(mu),
                                  ctypes.byref(it), dp(hist), cap)
        check(rc, (OK, NOT_CONVERGED) if allow_not_converged else (OK,))
        return mu, it.value, hist[: it.value], rc

    def solve_device(self, d_rhs, d_mu, make_guess=True, d_guess=None):
        """Device-pointer solve (ints from e.g. torch.Tensor.data_ptr())."""
        it = ctypes.c_int(0)
        cap = self.opts.maxiter + 64
        hist = np.zeros(cap)
        rc = lib().cppe_gpu_solve_device(self.h, d_rhs, d_guess, int(make_guess), d_mu,
                                         ctypes.byref(it), dp(hist), cap)
        check(rc)
        return it.value, hist[: it.value]

    def stream(self):
        s = ctypes.c_void_p()
        check(lib().cppe_gpu_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    def learned_data(self, rhs, mu_star):
        """Descriptor rows (n x 64) and target rows (n x 24) of one solve."""
        rhs, mu_star = f64(rhs), f64(mu_star)
        feats = np.zeros((self.n, N_IN), np.float32)
        rows = np.zeros((self.n, TROW), np.float32)
        check(lib().cppe_gpu_learned_data(self.h, dp(rhs), dp(mu_star), fp(feats), fp(rows)))
        return feats, rows

    def set_model(self, mlp):
        self._model = mlp
        check(lib().cppe_gpu_set_model(self.h, mlp.h if mlp is not None else None))

    def autotune(self, reps=3):
        """Picks the fastest near-field item size and M2L chunk; returns ms per apply."""
        ms = ctypes.c_double(0)
        lib().cppe_gpu_autotune.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_double)]
        check(lib().cppe_gpu_autotune(self.h, reps, ctypes.byref(ms)))
        return ms.value

    def schedule(self):
        """The schedule in use: symmetric near field (and its packed source
        pairs per lane, 0 when per target), near-field items, M2L chunk."""
        sym, items, ch = ctypes.c_int(0), ctypes.c_long(0), ctypes.c_int(0)
        lib().cppe_gpu_schedule_info.argtypes = [ctypes.c_void_p, I, L, I]
        check(lib().cppe_gpu_schedule_info(self.h, ctypes.byref(sym), ctypes.byref(items),
                                           ctypes.byref(ch)))
        return dict(symmetric_near=bool(sym.value), sym_pack=sym.value, near_items=items.value,
                    m2l_chunk=ch.value)

    def set_schedule(self, near_form=-1, item_pairs=0, m2l_chunk=0):
        """Sets the schedule: near_form 0 per target, 1 or 2 symmetric with two
        or four sources a lane (-1 keeps it); item_pairs and m2l_chunk <= 0
        keep theirs."""
        lib().cppe_gpu_set_schedule.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_long,
                                                ctypes.c_int]
        check(lib().cppe_gpu_set_schedule(self.h, near_form, item_pairs, m2l_chunk))

    def kernel_timings(self, precision=FP64, reps=5):
        ms = np.zeros(6)
        npair, nm2l = ctypes.c_longlong(0), ctypes.c_longlong(0)
        check(lib().cppe_gpu_kernel_timings(self.h, precision, reps, dp(ms), ctypes.byref(npair),
                                            ctypes.byref(nm2l)))
        names = ["near", "p2m_m2m", "m2l", "l2l", "finish", "apply"]
        return dict(zip(names, ms)), npair.value, nm2l.value

    def stats(self):
        r = ctypes.c_double(0)
        a = ctypes.c_int(0)
        b = ctypes.c_int(0)
        check(lib().cppe_gpu_last_solve_stats(self.h, ctypes.byref(r), ctypes.byref(a),
                                              ctypes.byref(b)))
        return dict(rnorm=r.value, fp64_applies=a.value, fp32_applies=b.value)


def multipole_fields(xyz, q, mu, quad, max_order, polarizable=None, alpha_iso=None,
                     excl_ptr=None, excl_idx=None, fmm=False, ncrit=64, order=5, theta=0.5,
                     damp=False, damping=2.1304, device=0):
    xyz = f64(xyz)
    n = xyz.shape[0]
    F = np.zeros(3 * n)
    args = [f64(q), f64(mu), f64(quad), i32(polarizable) if polarizable is not None else None,
            f64(alpha_iso) if alpha_iso is not None else None,
            i32(excl_ptr) if excl_ptr is not None else None,
            i32(excl_idx) if excl_idx is not None else None]
    check(lib().cppe_gpu_multipole_fields(
        n, dp(xyz), dp(args[0]), dp(args[1]), dp(args[2]), max_order, ip(args[3]),
        dp(args[4]), ip(args[5]), ip(args[6]), FMM if fmm else DIRECT, ncrit, order, theta,
        int(damp), damping, device, dp(F)))
    return F


def read_potfile(path):
    """Sites of a .pot file as arrays (cppe_gpu_potfile_*): xyz (n,3) bohr, q,
    mu (n,3), quad (n,6), alpha6 (n,6), polarizable, excl_ptr, excl_idx
    (CSR), elements, max_order."""
    h = ctypes.c_void_p()
    check(lib().cppe_gpu_potfile_read(os.fsencode(path), ctypes.byref(h)))
    try:
        n, mo, npol, ne = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0), ctypes.c_long(0)
        check(lib().cppe_gpu_potfile_info(h, ctypes.byref(n), ctypes.byref(mo),
                                          ctypes.byref(npol), ctypes.byref(ne)))
        n, ne = n.value, ne.value
        out = dict(xyz=np.zeros((n, 3)), q=np.zeros(n), mu=np.zeros((n, 3)),
                   quad=np.zeros((n, 6)), alpha6=np.zeros((n, 6)),
                   polarizable=np.zeros(n, np.int32), excl_ptr=np.zeros(n + 1, np.int32),
                   excl_idx=np.zeros(max(ne, 1), np.int32))
        el = ctypes.create_string_buffer(4 * max(n, 1))
        check(lib().cppe_gpu_potfile_arrays(
            h, dp(out["xyz"]), dp(out["q"]), dp(out["mu"]), dp(out["quad"]), dp(out["alpha6"]),
            ip(out["polarizable"]), ip(out["excl_ptr"]), ip(out["excl_idx"]), el))
        out["excl_idx"] = out["excl_idx"][:ne]
        raw = el.raw  # one copy of the buffer (each .raw access copies it)
        out["elements"] = [raw[4 * i:4 * i + 4].rstrip(b"\0").decode() for i in range(n)]
        out["max_order"] = mo.value
        return out
    finally:
        lib().cppe_gpu_potfile_free(h)


def tree_info(xyz, ncrit=64, theta=0.5):
    xyz = f64(xyz)
    nc, nl = ctypes.c_int(0), ctypes.c_int(0)
    nm, npp, pairs = ctypes.c_long(0), ctypes.c_long(0), ctypes.c_long(0)
    check(lib().cppe_gpu_tree_info(xyz.shape[0], dp(xyz), ncrit, theta, ctypes.byref(nc),
                                   ctypes.byref(nl), ctypes.byref(nm), ctypes.byref(npp),
                                   ctypes.byref(pairs)))
    return dict(ncells=nc.value, nleaves=nl.value, nm2l=nm.value, np2p=npp.value,
                p2p_pairs=pairs.value)


def tree_vectors(xyz, ncrit=64, theta=0.5):
    """(distinct M2L translation vectors, M2L list entries) of the tree; the
    count is -1 where the table would not be used."""
    xyz = f64(xyz)
    nv, ne = ctypes.c_int(0), ctypes.c_long(0)
    check(lib().cppe_gpu_tree_vectors(xyz.shape[0], dp(xyz), ncrit, theta, ctypes.byref(nv),
                                      ctypes.byref(ne)))
    return nv.value, ne.value


def tree_lists(xyz, ncrit=64, theta=0.5):
    info = tree_info(xyz, ncrit, theta)
    xyz = f64(xyz)
    m2l = np.zeros((info["nm2l"], 2), np.int32)
    p2p = np.zeros((info["np2p"], 2), np.int32)
    check(lib().cppe_gpu_tree_lists(xyz.shape[0], dp(xyz), ncrit, theta, ip(m2l), ip(p2p)))
    return info, m2l, p2p
