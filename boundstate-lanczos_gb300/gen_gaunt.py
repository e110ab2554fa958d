"""Generate csrc/bsl_gaunt.h: the product expansion of the basis's real
spherical harmonics.

For the tesseral functions of the reference's basis (normalised associated
Legendre functions times 1/sqrt(2 pi), cos(m phi)/sqrt(pi) or sin(|m| phi)/sqrt(pi),
HvCalc/linRotCartSphHvRoutines.cpp:293-434), every product of two basis
functions is a finite sum of real spherical harmonics of degree L <= 2 l_max:

    Y_s(u) Y_s'(u) = sum_LM G[s s'][LM] Y_LM(u)      for every direction u,

G[s s'][LM] being the Gaunt integral of the three functions.  The potential
blocks are the angular quadrature of V (ContinuousAngularGrid/
linRotCartSphHvContGridRoutines.cpp:7-152),

    <s|V|s'>(p) = sum_nodes w Y_s Y_s' V(p, node) = sum_LM G[s s'][LM] c_LM(p),
    c_LM(p) = sum_nodes w Y_LM V(p, node),

exactly, whatever V and the quadrature are, because the identity holds node by
node.  So nn (nn + 1) / 2 block elements per grid point are nc coefficients
c_LM: 66 instead of 231 for odd l <= 5.

The header holds, per supported basis, the sparse G in FP64 (for the prep that
recovers c from the FP64 blocks) and a device function that rebuilds the
block elements from c in FP32 and multiplies them into a vector.  The Gaunt
integrals are computed here with a quadrature that is exact for the products
(Gauss-Legendre in cos(theta), uniform in phi).

    python boundstate-lanczos_gb300/gen_gaunt.py      (rewrites csrc/bsl_gaunt.h)
"""
import math
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "bsl_gaunt.h")

# (l_max, symmetry) of the bases with a generated expansion: the odd-l (ortho)
# and even-l (para) blocks of the benchmark and batched workloads, and odd l <= 3
BASES = [(5, "Odd"), (4, "Even"), (3, "Odd")]


def basis(lmax, sym):
    """Packed (l, m) functions in the reference's order (m outer, l inner)."""
    out = []
    for m in range(-lmax, lmax + 1):
        for l in range(abs(m), lmax + 1):
            if sym == "All" or (sym == "Even" and l % 2 == 0) or (sym == "Odd" and l % 2 == 1):
                out.append((l, m))
    return out


def norm_legendre(L, x):
    """Normalised associated Legendre functions as the reference builds them
    (P_ll by the recurrence without the Condon-Shortley phase, then the factor
    (-1)^m sqrt((l - m)! (2l + 1) / (2 (l + m)!)))."""
    P = np.zeros((L + 1, L + 1) + x.shape)
    rf = np.sqrt(1.0 - x * x)
    P[0, 0] = 1.0
    for l in range(1, L + 1):
        P[l, l] = (2 * l - 1) * P[l - 1, l - 1] * rf
    for m in range(0, L):
        for l in range(m, L):
            prev = P[l - 1, m] if l - 1 >= m else 0.0
            P[l + 1, m] = ((2 * l + 1) * x * P[l, m] - (l + m) * prev) / (l - m + 1)
    for l in range(L + 1):
        for m in range(l + 1):
            P[l, m] *= (-1) ** m * math.sqrt(math.factorial(l - m) * (2 * l + 1) / (2 * math.factorial(l + m)))
    return P


def trig(m, phi):
    if m == 0:
        return np.full_like(phi, 1.0 / math.sqrt(2.0 * math.pi))
    if m > 0:
        return np.cos(m * phi) / math.sqrt(math.pi)
    return np.sin(-m * phi) / math.sqrt(math.pi)


def expansion(lmax, sym):
    """(pairs (s, s') with s <= s', (L, M) list, dense G[pairs][LM])."""
    fun = basis(lmax, sym)
    Lmax = 2 * lmax
    step = 1 if sym == "All" else 2
    lm = [(L, M) for L in range(0, Lmax + 1, step) for M in range(-L, L + 1)]
    x, wx = np.polynomial.legendre.leggauss(3 * lmax + 4)
    nphi = 6 * lmax + 8
    phi = (np.arange(nphi) + 0.5) * 2.0 * math.pi / nphi
    w = wx[:, None] * (2.0 * math.pi / nphi)
    P = norm_legendre(Lmax, x)

    def Y(l, m):
        return P[l, abs(m)][:, None] * trig(m, phi)[None, :]

    pairs = [(a, b) for a in range(len(fun)) for b in range(a, len(fun))]
    G = np.zeros((len(pairs), len(lm)))
    for i, (a, b) in enumerate(pairs):
        yy = Y(*fun[a]) * Y(*fun[b])
        for k, (L, M) in enumerate(lm):
            G[i, k] = np.sum(w * yy * Y(L, M))
    G[np.abs(G) < 1e-13] = 0.0
    # the identity holds node by node: check it on random directions
    rng = np.random.default_rng(1)
    xs, ps = rng.uniform(-1, 1, 64), rng.uniform(0, 2 * math.pi, 64)
    Pr = norm_legendre(Lmax, xs)
    yr = lambda l, m: Pr[l, abs(m)] * trig(m, ps)
    for i, (a, b) in enumerate(pairs):
        lhs = yr(*fun[a]) * yr(*fun[b])
        rhs = sum(G[i, k] * yr(L, M) for k, (L, M) in enumerate(lm) if G[i, k] != 0.0)
        assert np.max(np.abs(lhs - rhs)) < 1e-12, (lmax, sym, fun[a], fun[b])
    return fun, pairs, lm, G


def hexf(x):
    return float(np.float32(x)).hex() + "f"


def emit():
    lines = ["// Generated by boundstate-lanczos_gb300/gen_gaunt.py -- do not edit.",
             "//",
             "// Products of two basis functions as sums of real spherical harmonics:",
             "//   Y_s Y_s' = sum_k G[t][k] Y_k,  t = (s, s') with s <= s' row by row, k = (L, M),",
             "// so the potential block element t of a grid point is sum_k G[t][k] c_k(p).",
             "#pragma once", "", "namespace bsl {", "namespace gaunt {", "",
             "struct Term {", "  short t, k;  // block element (s <= s' row by row), coefficient (L, M)",
             "  double g;", "};", ""]
    table = []
    for lmax, sym in BASES:
        fun, pairs, lm, G = expansion(lmax, sym)
        nn, nc, nz = len(fun), len(lm), int(np.count_nonzero(G))
        tag = "%s%d" % (sym.lower(), lmax)
        lines.append("// %s l <= %d: %d functions, %d block elements, %d coefficients (L <= %d), %d terms"
                     % (sym.lower(), lmax, nn, len(pairs), nc, 2 * lmax, nz))
        lines.append("constexpr Term k_%s[%d] = {" % (tag, nz))
        row = []
        for t in range(len(pairs)):
            for k in range(nc):
                if G[t, k] != 0.0:
                    row.append("{%d, %d, %r}" % (t, k, float(G[t, k])))
        for i in range(0, len(row), 4):
            lines.append("    " + ", ".join(row[i:i + 4]) + ",")
        lines.append("};")
        table.append((lmax, sym, nn, nc, nz, tag, pairs, G))
    lines += ["", "struct Basis {", "  int l_max, symmetry, nn, nc, nterms;  // symmetry: BSL_SYM_*",
              "  const Term* terms;", "};", ""]
    symcode = {"All": 0, "Even": 1, "Odd": 2}
    lines.append("constexpr Basis kBases[%d] = {" % len(table))
    for lmax, sym, nn, nc, nz, tag, pairs, G in table:
        lines.append("    {%d, %d, %d, %d, %d, k_%s}," % (lmax, symcode[sym], nn, nc, nz, tag))
    lines.append("};")
    lines += ["", "#ifdef __CUDACC__",
              "// u[s] += sum_s' V[s][s'] v[s'] with V rebuilt from the coefficients c in FP32",
              "template <int NN>", "struct Apply;"]
    for lmax, sym, nn, nc, nz, tag, pairs, G in table:
        lines.append("template <>")
        lines.append("struct Apply<%d> {" % nn)
        lines.append("  static constexpr int kNC = %d;" % nc)
        lines.append("  static __device__ __forceinline__ void run(const float (&c)[%d], const float (&v)[%d], "
                     "float (&u)[%d]) {" % (nc, nn, nn))
        lines.append("    float x;")
        for t, (s, q) in enumerate(pairs):
            ks = [k for k in range(nc) if G[t, k] != 0.0]
            if not ks:
                continue
            expr = "__fmul_rn(%s, c[%d])" % (hexf(G[t, ks[0]]), ks[0])
            for k in ks[1:]:
                expr = "__fmaf_rn(%s, c[%d], %s)" % (hexf(G[t, k]), k, expr)
            lines.append("    x = %s;" % expr)
            if s == q:
                lines.append("    u[%d] = __fmaf_rn(x, v[%d], u[%d]);" % (s, s, s))
            else:
                lines.append("    u[%d] = __fmaf_rn(x, v[%d], u[%d]);" % (s, q, s))
                lines.append("    u[%d] = __fmaf_rn(x, v[%d], u[%d]);" % (q, s, q))
        lines.append("  }")
        lines.append("};")
    lines += ["#endif", "", "}  // namespace gaunt", "}  // namespace bsl", ""]
    return "\n".join(lines)


if __name__ == "__main__":
    text = emit()
    if len(sys.argv) > 1 and sys.argv[1] == "--check":
        sys.exit(0 if open(OUT).read() == text else 1)
    with open(OUT, "w") as f:
        f.write(text)
    print(OUT)
