"""Generate the coefficient tables of the device Hankel evaluator.

Writes hankel_coeffs.h next to this file.  The evaluator (hankel.cuh) covers
x = k r > 0 in three pieces:

  x <= 4   power-series form of the regular parts, as polynomials in
           v = x^2 / 16 (A&S 9.1.10-9.1.13):
             J0 = A0(v)                    J1 = x A1(v)
             Y0 = (2/pi) ln(x) J0 + B0(v)  Y1 = (2/pi) ln(x) J1 - 2/(pi x) + x B1(v)
  4 < x <= 8 and x > 8
           modulus-phase form (A&S 9.2.5-9.2.6):
             H_nu(x) = sqrt(2/(pi x)) (P_nu + i Q_nu) exp(i(x - (2nu+1) pi/4))
           with P_nu and (x/X) Q_nu as polynomials in t = 2 s' - 1, where
           s = (X/x)^2 and s' rescales the interval's s-range onto [0,1].

The polynomials are Chebyshev interpolants computed with mpmath at 50 digits
and converted to monomial form in the local variable; the term count is the
smallest that reaches |c_k| < 2e-18 (FP64 tables) or 3e-9 (FP32 tables).

Run:  python bem2d_gb300/csrc/gen_hankel.py
"""
from __future__ import annotations

import os

import mpmath as mp

mp.mp.dps = 50
HERE = os.path.dirname(os.path.abspath(__file__))


def cheb_nodes_coeffs(f, n):
    xs = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n) for k in range(n)]
    fx = [f(x) for x in xs]
    c = []
    for j in range(n):
        s = mp.fsum(fx[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / n) for k in range(n))
        c.append(2 * s / n)
    c[0] /= 2
    return c


def cheb_to_monomial(c):
    """Chebyshev series sum c_k T_k(t) -> monomial coefficients in t."""
    n = len(c)
    # T_k monomial coefficient rows by recurrence
    T = [[mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]]
    for k in range(2, n):
        a = [mp.mpf(0)] + [2 * v for v in T[k - 1]]
        b = T[k - 2] + [mp.mpf(0)] * (len(a) - len(T[k - 2]))
        T.append([a[i] - b[i] for i in range(len(a))])
    out = [mp.mpf(0)] * n
    for k in range(n):
        for i, v in enumerate(T[k]):
            out[i] += c[k] * v
    return out


def fit(f, tol, nmax=40):
    c = cheb_nodes_coeffs(f, nmax)
    scale = max(abs(v) for v in c)
    nt = max(i for i, v in enumerate(c) if abs(v) > tol * max(scale, 1e-3)) + 1
    return cheb_to_monomial(c[:nt])


def small_funcs():
    def x_of(t):  # t in [-1,1] -> v in [0,1] -> x in [0,4]
        v = (t + 1) / 2
        return 4 * mp.sqrt(v) + mp.mpf(10) ** -40

    def A0(t):
        return mp.besselj(0, x_of(t))

    def A1(t):
        x = x_of(t)
        return mp.besselj(1, x) / x

    def B0(t):
        x = x_of(t)
        return mp.bessely(0, x) - 2 / mp.pi * mp.log(x) * mp.besselj(0, x)

    def B1(t):
        x = x_of(t)
        return (mp.bessely(1, x) - 2 / mp.pi * mp.log(x) * mp.besselj(1, x)
                + 2 / (mp.pi * x)) / x

    return [A0, A1, B0, B1]


def pq_funcs(X, xhi):
    """P0, Q0*x/X, P1, Q1*x/X on x in [X, xhi] as functions of t in [-1,1]."""
    slo = (mp.mpf(X) / xhi) ** 2 if xhi is not None else mp.mpf(0)

    def x_of(t):
        s = slo + (1 - slo) * (t + 1) / 2
        return X / mp.sqrt(s)

    def make(nu, part):
        def f(t):
            x = x_of(t)
            h = mp.hankel1(nu, x)
            ph = x - (2 * nu + 1) * mp.pi / 4
            v = h * mp.exp(-1j * ph) * mp.sqrt(mp.pi * x / 2)
            return mp.re(v) if part == 0 else mp.im(v) * x / X
        return f

    return [make(0, 0), make(0, 1), make(1, 0), make(1, 1)], slo


def emit_polys(prefix, polys, ctype):
    """One inline Horner function per polynomial: PREFIX_<i>(t)."""
    lines = []
    suf = "f" if ctype == "float" else ""
    for i, p in enumerate(polys):
        coeffs = [mp.nstr(v, 21 if ctype == "double" else 10, strip_zeros=False) + suf
                  for v in p]
        expr = coeffs[-1]
        for c in reversed(coeffs[:-1]):
            expr = "fma(%s, t, %s)" % (expr, c)
        lines.append("__host__ __device__ __forceinline__ %s %s_%d(%s t) {\n"
                     "  return %s;\n}" % (ctype, prefix, i, ctype, expr))
    return "\n".join(lines) + "\n"


def split_ff(v):
    """Nearest float pair (hi, lo) with hi + lo ~ v to 2^-48."""
    import numpy as np
    hi = np.float32(float(v))
    lo = np.float32(float(v - mp.mpf(float(hi))))
    return float(hi), float(lo)


def f32(v):
    import numpy as np
    return float(np.float32(float(v)))


# index 3 (4 <= x < 8) was added after the first three; the order keeps the
# generated names of the others
FF_INTERVALS = ((8, 16), (16, 64), (64, None), (4, 8))
FF_TAIL_BOUND = 1.5e-8


def emit_ff_polys(idx, polys):
    """Compensated evaluation of monomial polynomials in t (|t| <= 1): the
    tail sum_{k>=m} c_k t^(k-m), bounded by FF_TAIL_BOUND, in FP32 Horner on
    t.hi; the head c_0 .. c_{m-1} in float-float Horner, with the cheaper
    ff_horner_fast step wherever |c_k| bounds the rest of the polynomial."""
    out = []
    for i, p in enumerate(polys):
        tails = [sum(abs(v) for v in p[k:]) for k in range(len(p))] + [0]
        m = next(k for k in range(len(p) + 1) if tails[k] < FF_TAIL_BOUND)
        m = max(m, 1)
        lines = ["__host__ __device__ __forceinline__ ff hkff_%d_%d(ff t) {" % (idx, i)]
        if m < len(p):
            expr = "%.9ef" % f32(p[-1])
            for c in reversed(p[m:-1]):
                expr = "fmaf(%s, t.hi, %.9ef)" % (expr, f32(c))
            lines.append("  const float tail = %s;" % expr)
            hi, lo = split_ff(p[m - 1])
            lines.append("  ff y = ff_add_f(ff_make(%.9ef, %.9ef), t.hi * tail);" % (hi, lo))
        else:
            hi, lo = split_ff(p[m - 1])
            lines.append("  ff y = ff_make(%.9ef, %.9ef);" % (hi, lo))
        for kk in reversed(range(m - 1)):
            hi, lo = split_ff(p[kk])
            # |y| <= sum_{j>kk} |c_j| on |t| <= 1; the fast step needs
            # |c_kk| >= |t y| (margin for the float rounding of c_kk)
            if abs(p[kk]) >= tails[kk + 1] * (1 + 1e-6):
                lines.append("  y = ff_horner_fast(ff_make(%.9ef, %.9ef), t, y);" % (hi, lo))
            else:
                lines.append("  y = ff_add_fast(ff_make(%.9ef, %.9ef), ff_mul(t, y));"
                             % (hi, lo))
        lines.append("  return y;")
        lines.append("}")
        out.append("\n".join(lines))
    return "\n".join(out) + "\n"


def main():
    out = ["// Generated by gen_hankel.py: polynomial pieces of the device Hankel",
           "// evaluator (see hankel.cuh).  Do not edit by hand.",
           "#pragma once", "#include <cmath>", ""]
    for ctype, tol, suffix in (("double", 2e-18, "d"), ("float", 3e-9, "f")):
        small = [fit(f, tol) for f in small_funcs()]
        out.append("// x <= 4: J0 = A0, J1 = x A1, Y0 = (2/pi) ln x J0 + B0,")
        out.append("//         Y1 = (2/pi) ln x J1 - 2/(pi x) + x B1;  t = x^2/8 - 1")
        out.append(emit_polys("hk_small_" + suffix, small, ctype))
        mid, _ = pq_funcs(4, mp.mpf(8))
        mid = [fit(f, tol) for f in mid]
        out.append("// 4 < x <= 8: P0, (x/4) Q0, P1, (x/4) Q1;  t = 2 ((4/x)^2 - 1/4)/(3/4) - 1")
        out.append(emit_polys("hk_mid_" + suffix, mid, ctype))
        far, _ = pq_funcs(8, None)
        far = [fit(f, tol) for f in far]
        out.append("// x > 8: P0, (x/8) Q0, P1, (x/8) Q1;  t = 2 (8/x)^2 - 1")
        out.append(emit_polys("hk_far_" + suffix, far, ctype))
        out.append("constexpr int hk_terms_%s[3] = {%d, %d, %d};\n"
                   % (suffix, max(map(len, small)), max(map(len, mid)), max(map(len, far))))
    with open(os.path.join(HERE, "hankel_coeffs.h"), "w") as f:
        f.write("\n".join(out) + "\n")
    # float-float tables: x >= 4 (four intervals) and x <= 4
    out = ["// Generated by gen_hankel.py: float-float pieces of the Hankel evaluator",
           "// for x >= 4 (see hankel_ff.cuh).  Do not edit by hand.",
           "#pragma once", '#include "ff.cuh"', "", "namespace bem2d_gpu {", ""]
    for idx, (X, xhi) in enumerate(FF_INTERVALS):
        funcs, slo = pq_funcs(X, mp.mpf(xhi) if xhi else None)
        polys = [fit(f, 2e-18) for f in funcs]
        out.append("// x in [%d, %s): P0, (x/%d) Q0, P1, (x/%d) Q1 in t = 2 (s - %s)/(1 - %s) - 1,"
                   % (X, xhi if xhi else "inf", X, X, mp.nstr(slo, 6), mp.nstr(slo, 6)))
        out.append("// s = (%d/x)^2" % X)
        out.append(emit_ff_polys(idx, polys))
    # index 4: the small-argument pieces A0, A1, B0, B1 (x <= 4) in t = x^2/8 - 1
    small = [fit(f, 2e-18) for f in small_funcs()]
    out.append("// x <= 4: J0 = A0, J1 = x A1, Y0 = (2/pi) ln x J0 + B0,")
    out.append("//         Y1 = (2/pi) ln x J1 - 2/(pi x) + x B1;  t = x^2/8 - 1")
    out.append(emit_ff_polys(len(FF_INTERVALS), small))
    out.append("}  // namespace bem2d_gpu")
    with open(os.path.join(HERE, "hankel_ff_coeffs.h"), "w") as f:
        f.write("\n".join(out) + "\n")


if __name__ == "__main__":
    main()
