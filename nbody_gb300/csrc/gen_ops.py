"""Generates fmm_ops.inc: straight-line Cartesian FMM operators per order.

Multi-indices n = (nx, ny, nz), |n| <= p, are stored in total-degree order
(within a degree: nx descending, then ny descending); index(n) =
d(d+1)(d+2)/6 + s(s+1)/2 + nz with d = |n|, s = ny + nz.

Kernel: psi(r) = (|r|^2 + eps^2)^(-1/2).  D_n = d^n psi.  Derivatives come
from differentiating s * d_i psi + x_i psi = 0 (s = |r|^2 + eps^2) with the
Leibniz rule, which gives, for any axis i with n_i >= 1,

  s D_n = -[ (2 n_i - 1) x_i D_{n-e_i} + 2 sum_{d != i} n_d x_d D_{n-e_d}
             + (n_i - 1)^2 D_{n-2e_i} + sum_{d != i} n_d (n_d - 1) D_{n-2e_d} ]

so every D_n needs only lower-order entries of the same array.

Expansions:  M_n = sum_j q_j y_j^n / n!           (y_j = x_j - c_source)
             L_k = sum_n (-1)^|n| M_n D_{n+k}(c_target - c_source)
             psi(c + y) = sum_k L_k y^k / k!,  E = grad psi.
Run: python gen_ops.py > fmm_ops.inc
"""
import sys

PMAX = 8


def terms(p):
    out = []
    for d in range(p + 1):
        for nx in range(d, -1, -1):
            for ny in range(d - nx, -1, -1):
                out.append((nx, ny, d - nx - ny))
    return out


def idx(n):
    nx, ny, nz = n
    d = nx + ny + nz
    s = ny + nz
    return d * (d + 1) * (d + 2) // 6 + s * (s + 1) // 2 + nz


def T(p):
    return (p + 1) * (p + 2) * (p + 3) // 6


def sub(n, d, k=1):
    m = list(n)
    m[d] -= k
    return tuple(m)


def add(a, b):
    return (a[0] + b[0], a[1] + b[1], a[2] + b[2])


def lit(v):
    return f"S({v})"


def gen_derivs(p, o):
    o.append("  template <int ST = 1>")
    o.append(f"  static __device__ __forceinline__ void derivs(S x, S y, S z, S eps2, S* D) {{")
    o.append("    const S s = x * x + y * y + z * z + eps2;")
    o.append("    D[0] = nb_rsqrt_n(s);")
    o.append("    const S is = D[0] * D[0];")
    X = ["x", "y", "z"]
    for n in terms(p)[1:]:
        i = 0 if n[0] > 0 else (1 if n[1] > 0 else 2)
        parts = []
        c = 2 * n[i] - 1
        parts.append(f"{lit(c)} * {X[i]} * D[{idx(sub(n, i))} * ST]" if c != 1 else f"{X[i]} * D[{idx(sub(n, i))} * ST]")
        for d in range(3):
            if d != i and n[d] >= 1:
                parts.append(f"{lit(2 * n[d])} * {X[d]} * D[{idx(sub(n, d))} * ST]")
        if n[i] >= 2:
            c = (n[i] - 1) ** 2
            parts.append(f"{lit(c)} * D[{idx(sub(n, i, 2))} * ST]" if c != 1 else f"D[{idx(sub(n, i, 2))} * ST]")
        for d in range(3):
            if d != i and n[d] >= 2:
                parts.append(f"{lit(n[d] * (n[d] - 1))} * D[{idx(sub(n, d, 2))} * ST]")
        o.append(f"    D[{idx(n)} * ST] = -is * ({' + '.join(parts)});")
    o.append("  }")


def m2l_flops(p):
    """Flops of one far-field cell pair at order p: displacement (3), s (5),
    reciprocal and rsqrt (2), each derivative entry (its products, sums and
    the scaling), and the contraction (one FMA = 2 per (n, k) pair)."""
    f = 3 + 5 + 2
    for n in terms(p)[1:]:
        i = 0 if n[0] > 0 else (1 if n[1] > 0 else 2)
        k = 0
        f2 = 0
        c = 2 * n[i] - 1
        f2 += 2 if c != 1 else 1
        k += 1
        for d in range(3):
            if d != i and n[d] >= 1:
                f2 += 2
                k += 1
        if n[i] >= 2:
            f2 += 1 if (n[i] - 1) ** 2 != 1 else 0
            k += 1
        for d in range(3):
            if d != i and n[d] >= 2:
                f2 += 1
                k += 1
        f += f2 + (k - 1) + 1
    pairs = sum(T(p - sum(n)) for n in terms(p))
    return f + 2 * pairs


def gen_m2l(p, o):
    # L[k] += sum_n (-1)^|n| M[n] D[n+k]; M streamed from memory
    o.append("  template <int ST = 1>")
    o.append("  static __device__ __forceinline__ void m2l(const S* __restrict__ M, const S* D, S* L) {")
    for n in terms(p):
        dn = sum(n)
        o.append(f"    {{ const S m = {'-' if dn % 2 else ''}M[{idx(n)}];")
        for k in terms(p - dn):
            o.append(f"      L[{idx(k)} * ST] = nb_fma(m, D[{idx(add(n, k))} * ST], L[{idx(k)} * ST]);")
        o.append("    }")
    o.append("  }")


def gen_m2l_v(p, o):
    """M2L contraction reading the source row M in aligned groups of 4
    (nb_ld4: one 16-byte load for float, two for double); M must be
    16-byte aligned and padded to a multiple of 4 entries."""
    o.append("  template <int ST = 1>")
    o.append("  static __device__ __forceinline__ void m2l_v(const S* __restrict__ M, const S* D, S* L) {")
    o.append("    S mq[4];")
    for n in terms(p):
        i = idx(n)
        if i % 4 == 0:
            o.append(f"    nb_ld4(M + {i}, mq);")
        dn = sum(n)
        o.append(f"    {{ const S m = {'-' if dn % 2 else ''}mq[{i % 4}];")
        for k in terms(p - dn):
            o.append(f"      L[{idx(k)} * ST] = nb_fma(m, D[{idx(add(n, k))} * ST], L[{idx(k)} * ST]);")
        o.append("    }")
    o.append("  }")


def gen_mono(p, o, name="mono"):
    o.append(f"  static __device__ __forceinline__ void {name}(S x, S y, S z, S* Y) {{")
    o.append("    Y[0] = S(1);")
    X = ["x", "y", "z"]
    for n in terms(p)[1:]:
        i = 0 if n[0] > 0 else (1 if n[1] > 0 else 2)
        c = n[i]
        if c == 1:
            o.append(f"    Y[{idx(n)}] = Y[{idx(sub(n, i))}] * {X[i]};")
        else:
            o.append(f"    Y[{idx(n)}] = Y[{idx(sub(n, i))}] * {X[i]} * S({1.0 / c!r});")
    o.append("  }")


def gen_p2m(p, o):
    o.append("  static __device__ __forceinline__ void p2m(S q, S x, S y, S z, S* M) {")
    o.append(f"    S Y[{T(p)}];")
    o.append("    mono(x, y, z, Y);")
    for n in terms(p):
        o.append(f"    M[{idx(n)}] = nb_fma(q, Y[{idx(n)}], M[{idx(n)}]);")
    o.append("  }")


def gen_l2p(p, o):
    # E_d = sum_{|k|<=p-1} L[k+e_d] y^k/k!, psi = sum_k L[k] y^k/k!
    o.append("  static __device__ __forceinline__ void l2p(const S* __restrict__ L, S x, S y, S z, "
             "S& ex, S& ey, S& ez, S& psi) {")
    o.append(f"    S Y[{T(p)}];")
    o.append("    mono(x, y, z, Y);")
    o.append("    S a0 = L[0], a1 = L[1], a2 = L[2], a3 = L[3];")
    for k in terms(p)[1:]:
        o.append(f"    a0 = nb_fma(L[{idx(k)}], Y[{idx(k)}], a0);")
    for k in terms(p - 1)[1:]:
        o.append(f"    a1 = nb_fma(L[{idx(add(k, (1, 0, 0)))}], Y[{idx(k)}], a1);")
        o.append(f"    a2 = nb_fma(L[{idx(add(k, (0, 1, 0)))}], Y[{idx(k)}], a2);")
        o.append(f"    a3 = nb_fma(L[{idx(add(k, (0, 0, 1)))}], Y[{idx(k)}], a3);")
    o.append("    psi = a0; ex = a1; ey = a2; ez = a3;")
    o.append("  }")


def gen_l2p_hess(p, o):
    """h = H nu with H_de = sum_{|k| <= p-2} L[k + e_d + e_e] y^k/k! (Hessian of the
    local expansion at y), used by the adjoint of L2P."""
    o.append("  static __device__ __forceinline__ void l2p_hess(const S* __restrict__ L, S x, S y, S z, S nx, S ny, "
             "S nz, S& hx, S& hy, S& hz) {")
    if p < 2:
        o.append("    hx = S(0); hy = S(0); hz = S(0);")
        o.append("  }")
        return
    o.append(f"    S Y[{T(p - 2)}];")
    o.append("    mono_lo(x, y, z, Y);")
    names = {(0, 0): "xx", (0, 1): "xy", (0, 2): "xz", (1, 1): "yy", (1, 2): "yz", (2, 2): "zz"}
    E = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]
    for (d, e), nm in names.items():
        o.append(f"    S h{nm} = L[{idx(add(E[d], E[e]))}];")
    for k in terms(p - 2)[1:]:
        for (d, e), nm in names.items():
            o.append(f"    h{nm} = nb_fma(L[{idx(add(k, add(E[d], E[e])))}], Y[{idx(k)}], h{nm});")
    o.append("    hx = hxx * nx + hxy * ny + hxz * nz;")
    o.append("    hy = hxy * nx + hyy * ny + hyz * nz;")
    o.append("    hz = hxz * nx + hyz * ny + hzz * nz;")
    o.append("  }")


def shift_tables(p):
    ts = terms(p)
    m2m, l2l = [], []
    # M2M: Mp[a] += Mc[b] * Y[a-b], b <= a componentwise
    for a in ts:
        for b in ts:
            c = (a[0] - b[0], a[1] - b[1], a[2] - b[2])
            if min(c) >= 0:
                m2m.append((idx(a), idx(b), idx(c)))
    # L2L: Lc[a] += Lp[a+c] * Y[c], |a+c| <= p
    for a in ts:
        for c in terms(p - sum(a)):
            l2l.append((idx(a), idx(add(a, c)), idx(c)))
    return m2m, l2l


def main():
    o = ["// Generated by gen_ops.py -- do not edit.", "#pragma once", ""]
    o.append("template <int P> struct nb_terms { static constexpr int value = (P + 1) * (P + 2) * (P + 3) / 6; };")
    o.append("// multipole row stride: terms rounded up to a multiple of 4 (16-byte rows for float, 32 for double)")
    o.append("template <int P> struct nb_tm { static constexpr int value = (nb_terms<P>::value + 3) & ~3; };")
    o.append("template <typename S, int P> struct Ops;")
    for p in range(1, PMAX + 1):
        o.append("")
        o.append(f"template <typename S> struct Ops<S, {p}> {{")
        o.append(f"  static constexpr int T = {T(p)};")
        gen_derivs(p, o)
        gen_m2l(p, o)
        gen_m2l_v(p, o)
        gen_mono(p, o)
        if p >= 2:
            lo = []
            gen_mono(p - 2, lo, name="mono_lo")
            o.extend(lo)
        gen_p2m(p, o)
        gen_l2p(p, o)
        gen_l2p_hess(p, o)
        o.append("};")
    # shift tables: (out, in, mono) triples, grouped by output index
    for p in range(1, PMAX + 1):
        m2m, l2l = shift_tables(p)
        for name, tab in (("m2m", m2m), ("l2l", l2l)):
            # row starts per output index for lane-parallel evaluation
            starts = [0] * (T(p) + 1)
            for a, _, _ in tab:
                starts[a + 1] += 1
            for a in range(T(p)):
                starts[a + 1] += starts[a]
            flat = ",".join(f"{b},{c}" for _, b, c in tab)
            o.append(f"__device__ const unsigned short nb_{name}_p{p}_start[{T(p) + 1}] = {{{','.join(map(str, starts))}}};")
            o.append(f"__device__ const unsigned short nb_{name}_p{p}_pairs[{2 * len(tab)}] = {{{flat}}};")
    # multi-index exponents and 1/(nx! ny! nz!) in the global term order
    ts = terms(PMAX)
    fact = [1]
    for i in range(1, 20):
        fact.append(fact[-1] * i)
    o.append(f"__device__ const unsigned char nb_mi[{T(PMAX)}][3] = {{" +
             ",".join(f"{{{a},{b},{c}}}" for a, b, c in ts) + "};")
    o.append(f"__device__ const double nb_invfact[{T(PMAX)}] = {{" +
             ",".join(repr(1.0 / (fact[a] * fact[b] * fact[c])) for a, b, c in ts) + "};")
    o.append("constexpr long long nb_m2l_flops_tab[" + str(PMAX + 1) + "] = {0," +
             ",".join(str(m2l_flops(p)) for p in range(1, PMAX + 1)) + "};")
    o.append("template <int P> struct Tabs;")
    for p in range(1, PMAX + 1):
        o.append(f"template <> struct Tabs<{p}> {{")
        for name in ("m2m", "l2l"):
            o.append(f"  static __device__ __forceinline__ const unsigned short* {name}_start() {{ return nb_{name}_p{p}_start; }}")
            o.append(f"  static __device__ __forceinline__ const unsigned short* {name}_pairs() {{ return nb_{name}_p{p}_pairs; }}")
        o.append("};")
    o.append("")
    sys.stdout.write("\n".join(o) + "\n")


if __name__ == "__main__":
    main()
