"""Generates m2l_gen.cuh: straight-line M2L translations for fixed expansion
orders, so that the derivative tensor and the local expansion live in
registers, and straight-line forms of the other expansion operators (P2M of
a dipole, M2M and L2L shifts, L2P field evaluation) for the same orders.

The operator is the reference's Cartesian M2L in the Dehnen/fmmgen
convention (src/core/fmm/field_m*.cc, calculate.cc:186-203):

    L_n += sum_{k : m <= |k|, |n| + |k| <= p} D_{n+k}(r) M_k,   D_j = d^j (1/R)

with multi-indices ordered by total order, then x-power descending, then
y-power descending.  D is built from the recurrence

    |n| R^2 D_n = -(2|n|-1) sum_i n_i r_i D_{n-e_i} - (|n|-1) sum_i n_i (n_i-1) D_{n-2e_i}

(differentiate R^2 d_i (1/R) = -r_i / R).  The functions are templates over
the arithmetic type: float, double, or the double-float pair `ddv` (dd.cuh),
which supplies the operators, `fma`, `rsqrt_t` and `cinv<T>(o)` = 1/o.
The shifts are the index tables of fmm_ops.cc written out term by term
(calculate.cc:129-260 with the field_m*.cc P2M/M2M/L2L/L2P kernels): with
the scaled powers px_a = x^a / a! (and y, z alike) and the monomial
mono(a, b, c) = px_a py_b pz_c,

    P2M  M_n += sum_{|k| = 1, k <= n} mono(n - k) s_k        (s: the dipole)
    M2M  M_n += sum_{k <= n} mono(n - k) M'_k
    L2L  L_n += sum_{k >= n} mono(k - n) L'_k
    L2P  f_c -= sum_{n_c >= 1} mono(n - e_c) L_n

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
    dlines = lines[3:]  # the derivative recurrence (r2, ir2, D0 .. D{nt-1})
    contr = []
    for k in range(moff, nterms(p)):
        ka, kb, kc = mi[k]
        ko = ka + kb + kc
        contr.append(f"  {{ const T mk = Mb[{k - moff}];")
        for nidx in range(nterms(p - ko)):
            na, nb, nc = mi[nidx]
            w = idx[(na + ka, nb + kb, nc + kc)]
            contr.append(f"    acc[{nidx}] = fma(D{w}, mk, acc[{nidx}]);")
        contr.append("  }")
    lines += contr
    lines.append("}")
    # the derivative tensor alone (tabulated once per distinct translation
    # vector) and the contraction with a tabulated tensor
    nt = nterms(p)
    lines.append(f"// derivative tensor D_j = d^j (1/R), j < {nt}, of M2L m{m} p{p}")
    lines.append("template <typename T>")
    lines.append(f"__device__ __forceinline__ void dtensor_m{m}_p{p}(T x, T y, T z, "
                 "T* __restrict__ Dout) {")
    lines += dlines
    for j in range(nt):
        lines.append(f"  Dout[{j}] = D{j};")
    lines.append("}")
    lines.append(f"// M2L m{m} p{p} with the derivative tensor read from Dt")
    lines.append("template <typename T>")
    lines.append(f"__device__ __forceinline__ void {name}_pre(const T* __restrict__ Dt, "
                 "const T* __restrict__ Mb, T* __restrict__ acc) {")
    for j in range(nt):
        lines.append(f"  const T D{j} = Dt[{j}];")
    lines += contr
    lines.append("}")
    return "\n".join(lines), name, ls, nterms(p) - moff


def emit_tables(m, p):
    """Tables of the loop form of the same translation (the double-float M2L,
    whose straight-line form is too long for the instruction cache):
    rec[j] = {D indices of n-e_x, n-e_y, n-e_z, n-2e_x, n-2e_y, n-2e_z (-1:
    none), |n|, 0}, coef[j] = {(2|n|-1) n_i (3), (|n|-1) n_i (n_i-1) (3),
    1/|n| as a double-float pair}, and w: for every multipole coefficient k
    (in order) the D index of n + k for the local coefficients n < nterms(p -
    |k|), so that L_n += D_w M_k."""
    mi = multi_indices(p)
    idx = {t: j for j, t in enumerate(mi)}
    nt, moff = nterms(p), nterms(m - 1)
    rec, coef = [], []
    for j, n in enumerate(mi):
        o = sum(n)
        q, c = [-1] * 6, [0.0] * 6
        if j > 0:
            for i in range(3):
                if n[i] >= 1:
                    t = list(n)
                    t[i] -= 1
                    q[i], c[i] = idx[tuple(t)], float((2 * o - 1) * n[i])
                if n[i] >= 2:
                    t = list(n)
                    t[i] -= 2
                    q[3 + i], c[3 + i] = idx[tuple(t)], float((o - 1) * n[i] * (n[i] - 1))
        inv = 1.0 / o if o > 0 else 0.0
        import struct
        hi = struct.unpack("f", struct.pack("f", inv))[0]
        lo = struct.unpack("f", struct.pack("f", inv - hi))[0]
        rec.append(q + [o, 0])
        coef.append(c + [hi, lo])
    w = []
    for k in range(moff, nt):
        ka, kb, kc = mi[k]
        for nidx in range(nterms(p - (ka + kb + kc))):
            na, nb, nc = mi[nidx]
            w.append(idx[(na + ka, nb + kb, nc + kc)])
    name = f"m{m}_p{p}"
    fl = lambda v: repr(float(v)) + "f"
    lines = [f"// loop-form tables of M2L, source order {m}, expansion order {p}"]
    lines.append(f"static __constant__ short m2l_rec_{name}[{8 * nt}] = {{")
    lines.append("  " + ", ".join(str(v) for r in rec for v in r) + "};")
    lines.append(f"static __constant__ float m2l_coef_{name}[{8 * nt}] = {{")
    lines.append("  " + ", ".join(fl(v) for r in coef for v in r) + "};")
    lines.append(f"static __constant__ unsigned char m2l_w_{name}[{len(w)}] = {{")
    lines.append("  " + ", ".join(str(v) for v in w) + "};")
    return "\n".join(lines), name, nt


def powers_lines(q):
    """Scaled powers px_a = x^a / a!, a = 1..q (px_0 = 1 is left out)."""
    out = []
    for v in "xyz":
        for a in range(1, q + 1):
            if a == 1:
                out.append(f"  const T p{v}1 = {v};")
            else:
                out.append(f"  const T p{v}{a} = p{v}{a - 1} * {v} * cinv<T>({a});")
    return out


def mono(e):
    """mono(a, b, c) as the product (px_a py_b) pz_c with unit factors left out
    (the table-driven form multiplies by them: exact)."""
    f = [f"p{v}{a}" for v, a in zip("xyz", e) if a > 0]
    return " * ".join(f) if f else "T(1)"


def emit_shifts(m, p):
    mi = multi_indices(p + 1)
    idx = {t: j for j, t in enumerate(mi)}
    moff, nt, ls = nterms(m - 1), nterms(p), nterms(p - m)
    ms = nt - moff
    sub = lambda n, k: tuple(a - b for a, b in zip(mi[n], mi[k]))
    ge = lambda d: all(v >= 0 for v in d)
    out = []

    def body(q, terms, used):
        # terms: list of (input expression, [(output index, exponent)])
        lines = powers_lines(q)
        for e in sorted(used, key=lambda e: idx[e]):
            if sum(e) > 1 and sum(1 for v in e if v) > 1:
                lines.append(f"  const T m_{e[0]}_{e[1]}_{e[2]} = {mono(e)};")
        for inp, outs in terms:
            lines.append(f"  {{ const T v = {inp};")
            for o, e in outs:
                me = f"m_{e[0]}_{e[1]}_{e[2]}" if sum(e) > 1 and sum(1 for v in e if v) > 1 \
                    else mono(e)
                lines.append(f"    {o} = fma({me}, v, {o});")
            lines.append("  }")
        return lines

    # P2M of a dipole (source order 1 only)
    if m == 1:
        terms, used = [], set()
        for k in range(moff, nterms(m)):
            outs = []
            for n in range(moff, nt):
                d = sub(n, k)
                if ge(d):
                    outs.append((f"acc[{n - moff}]", d))
                    used.add(d)
            terms.append((f"s{k - moff}", outs))
        out.append(f"// P2M of a dipole (s0, s1, s2) at offset (x, y, z) = centre - site, order {p}")
        out.append("template <typename T>")
        out.append(f"__device__ __forceinline__ void p2m_m{m}_p{p}(T x, T y, T z, T s0, T s1, T s2, "
                   "T* __restrict__ acc) {")
        out += body(p - 1, terms, used)
        out.append("}")
    # M2M
    terms, used = [], set()
    for k in range(moff, nt):
        outs = []
        for n in range(k, nt):
            d = sub(n, k)
            if ge(d):
                outs.append((f"acc[{n - moff}]", d))
                used.add(d)
        terms.append((f"Mc[{k - moff}]", outs))
    out.append(f"// M2M: multipole Mc about a centre at (x, y, z) from this one, order {p}")
    out.append("template <typename T>")
    out.append(f"__device__ __forceinline__ void m2m_m{m}_p{p}(T x, T y, T z, const T* __restrict__ Mc, "
               "T* __restrict__ acc) {")
    out += body(p - 1, terms, used)
    out.append("}")
    # L2L
    terms, used = [], set()
    for k in range(ls):
        outs = []
        for n in range(0, k + 1):
            d = sub(k, n)
            if ge(d):
                outs.append((f"acc[{n}]", d))
                used.add(d)
        terms.append((f"Lc[{k}]", outs))
    out.append(f"// L2L: local expansion Lc about a centre at -(x, y, z) from this one, order {p}")
    out.append("template <typename T>")
    out.append(f"__device__ __forceinline__ void l2l_m{m}_p{p}(T x, T y, T z, const T* __restrict__ Lc, "
               "T* __restrict__ acc) {")
    out += body(p - m, terms, used)
    out.append("}")
    # L2P
    terms, used = [], set()
    for n in range(1, ls):
        outs = []
        for c in range(3):
            e = list(mi[n])
            if e[c] == 0:
                continue
            e[c] -= 1
            e = tuple(e)
            outs.append((f"f{c}", e))
            used.add(e)
        terms.append((f"-Lc[{n}]", outs))
    out.append(f"// L2P: field -grad of the local expansion Lc at offset (x, y, z) = site - centre, "
               f"order {p}")
    out.append("template <typename T>")
    out.append(f"__device__ __forceinline__ void l2p_m{m}_p{p}(T x, T y, T z, const T* __restrict__ Lc, "
               "T& f0, T& f1, T& f2) {")
    out += body(max(p - m - 1, 1), terms, used)
    out.append("}")
    return "\n".join(out), ls, ms


def main(out_path):
    parts = ["// Generated by gen_m2l.py -- do not edit.", "#pragma once", ""]
    table = []
    for m, p in ORDERS:
        code, name, ls, ms = emit(m, p)
        parts.append(code)
        parts.append("")
        table.append((m, p, name, ls, ms))
    for m, p in ORDERS:
        code, ls, ms = emit_shifts(m, p)
        parts.append(code)
        parts.append("")
    tabs = []
    for m, p in ORDERS:
        code, name, nt = emit_tables(m, p)
        parts.append(code)
        parts.append("")
        tabs.append((m, p, name, nt))
    parts.append("#define CPPE_M2L_GENERATED(X) \\")
    parts.append(" \\\n".join(f"  X({m}, {p}, {name}, {ls}, {ms})" for m, p, name, ls, ms in table))
    parts.append("")
    # (m, p, Lsize, Msize) of the straight-line shifts
    parts.append("#define CPPE_SHIFTS_GENERATED(X) \\")
    parts.append(" \\\n".join(f"  X({m}, {p}, {ls}, {ms})" for m, p, name, ls, ms in table))
    parts.append("")
    # (m, p, name suffix of the tables, nterms(p), Lsize, Msize) of the loop form
    parts.append("#define CPPE_M2L_TABLES(X) \\")
    parts.append(" \\\n".join(f"  X({m}, {p}, {name}, {nt}, {ls}, {ms})"
                              for (m, p, name, nt), (_, _, _, ls, ms) in zip(tabs, table)))
    parts.append("")
    src = "\n".join(parts)
    if os.path.exists(out_path) and open(out_path).read() == src:
        return
    with open(out_path, "w") as f:
        f.write(src)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.path.join(os.path.dirname(os.path.abspath(__file__)), "m2l_gen.cuh"))
