"""Generates m2l_gen.cuh: straight-line M2L translations for fixed expansion
orders, so that the derivative tensor and the local expansion live in
registers.

The operator is the reference's Cartesian M2L in the Dehnen/fmmgen
convention (src/core/fmm/field_m*.cc, calculate.cc:186-203):

    L_n += sum_{k : m <= |k|, |n| + |k| <= p} D_{n+k}(r) M_k,   D_j = d^j (1/R)

with multi-indices ordered by total order, then x-power descending, then
y-power descending.  D is built from the recurrence

    |n| R^2 D_n = -(2|n|-1) sum_i n_i r_i D_{n-e_i} - (|n|-1) sum_i n_i (n_i-1) D_{n-2e_i}

(differentiate R^2 d_i (1/R) = -r_i / R).  The functions are templates over
the arithmetic type: float, double, or the double-float pair `ddv` (dd.cuh),
which supplies the operators, `fma`, `rsqrt_t` and `cinv<T>(o)` = 1/o.
This file is run by the build
(cppe_gb300/_build.py) and its output is not edited by hand.
"""
import os
import sys

# (source order m, expansion order p) pairs to emit
ORDERS = [(1, 5), (1, 6)]


def nterms(p):
    return 0 if p < 0 else (p + 1) * (p + 2) * (p + 3) // 6


def multi_indices(p):
    out = []
    for o in range(p + 1):
        for a in range(o, -1, -1):
            for b in range(o - a, -1, -1):
                out.append((a, b, o - a - b))
    return out


def emit(m, p):
    mi = multi_indices(p)
    idx = {t: j for j, t in enumerate(mi)}
    moff = nterms(m - 1)
    ls = nterms(p - m)
    lines = []
    name = f"m2l_m{m}_p{p}"
    lines.append(f"// M2L, source order {m}, expansion order {p}: Msize {nterms(p) - moff}, "
                 f"Lsize {ls}")
    lines.append("template <typename T>")
    lines.append(f"__device__ __forceinline__ void {name}(T x, T y, T z, const T* __restrict__ Mb, "
                 "T* __restrict__ acc) {")
    lines.append("  const T r2 = x * x + y * y + z * z;")
    lines.append("  const T ir2 = T(1) / r2;")
    lines.append("  const T D0 = rsqrt_t(r2);")
    rvar = ("x", "y", "z")
    for j, (a, b, c) in enumerate(mi):
        if j == 0:
            continue
        n = (a, b, c)
        o = a + b + c
        t1, t2 = [], []
        for i in range(3):
            if n[i] >= 1:
                q = list(n)
                q[i] -= 1
                coef = n[i]
                t1.append((f"T({coef}) * " if coef != 1 else "") + f"{rvar[i]} * D{idx[tuple(q)]}")
            if n[i] >= 2:
                q = list(n)
                q[i] -= 2
                t2.append(f"T({n[i] * (n[i] - 1)}) * D{idx[tuple(q)]}")
        e1 = " + ".join(t1)
        expr = f"T({2 * o - 1}) * ({e1})"
        if t2 and o > 1:
            expr += f" + T({o - 1}) * ({' + '.join(t2)})"
        lines.append(f"  const T D{j} = -({expr}) * ir2 * cinv<T>({o});")
    for k in range(moff, nterms(p)):
        ka, kb, kc = mi[k]
        ko = ka + kb + kc
        lines.append(f"  {{ const T mk = Mb[{k - moff}];")
        for nidx in range(nterms(p - ko)):
            na, nb, nc = mi[nidx]
            w = idx[(na + ka, nb + kb, nc + kc)]
            lines.append(f"    acc[{nidx}] = fma(D{w}, mk, acc[{nidx}]);")
        lines.append("  }")
    lines.append("}")
    return "\n".join(lines), name, ls, nterms(p) - moff


def main(out_path):
    parts = ["// Generated by gen_m2l.py -- do not edit.", "#pragma once", ""]
    table = []
    for m, p in ORDERS:
        code, name, ls, ms = emit(m, p)
        parts.append(code)
        parts.append("")
        table.append((m, p, name, ls, ms))
    parts.append("#define CPPE_M2L_GENERATED(X) \\")
    parts.append(" \\\n".join(f"  X({m}, {p}, {name}, {ls}, {ms})" for m, p, name, ls, ms in table))
    parts.append("")
    src = "\n".join(parts)
    if os.path.exists(out_path) and open(out_path).read() == src:
        return
    with open(out_path, "w") as f:
        f.write(src)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.path.join(os.path.dirname(os.path.abspath(__file__)), "m2l_gen.cuh"))
