#!/usr/bin/env python3
"""Writes fb_ewald_fit.h: piecewise polynomial fits of the two screened
lattice-sum functions of the Ewald terms, for their double-float kernels.

  E(x) = erfc(x)                                   (assemble_ewald)
  H(x) = erfc(x) + 2 x exp(-x^2) / sqrt(pi)        (Dassemble_ewald)

on [0, 5.5] (the kernels skip x = kappa z > 5.5, where erfc(x) < 1e-14).
The range is cut into 22 intervals of width 1/4; on each, the function is
interpolated at the 13 Chebyshev points in 40-digit arithmetic (mpmath) and
the degree-12 polynomial is written in the local variable t = 8 (x - a) - 1
in [-1, 1], monomial coefficients lowest first, each as a pair of floats
(hi, lo).  The interpolation error is below 1e-18 on every interval, far
under the ~1e-14 relative error of the double-float evaluation.

Run: python gen_ewald_fit.py > fb_ewald_fit.h
"""
import mpmath as mp

mp.mp.dps = 40
XMAX = mp.mpf("5.5")
WIDTH = mp.mpf(1) / 4
DEG = 12


def E(x):
    return mp.erfc(x)


def H(x):
    return mp.erfc(x) + 2 * x * mp.exp(-x * x) / mp.sqrt(mp.pi)


def fit(f, a, b):
    n = DEG + 1
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / n) for k in range(n)]
    fv = [f((a + b) / 2 + (b - a) / 2 * t) for t in nodes]
    c = [2 * mp.fsum(fv[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / n) for k in range(n)) / n for j in range(n)]
    c[0] /= 2
    T = [[mp.mpf(1)], [mp.mpf(0), mp.mpf(1)]]
    for j in range(2, n):
        p = [mp.mpf(0)] + [2 * v for v in T[j - 1]]
        for k in range(len(T[j - 2])):
            p[k] -= T[j - 2][k]
        T.append(p)
    mono = [mp.mpf(0)] * n
    for j in range(n):
        for k, v in enumerate(T[j]):
            mono[k] += c[j] * v
    err = mp.mpf(0)
    for q in range(101):
        t = -1 + mp.mpf(2) * q / 100
        p = mp.mpf(0)
        for k in reversed(range(n)):
            p = p * t + mono[k]
        err = max(err, abs(p - f((a + b) / 2 + (b - a) / 2 * t)))
    return mono, err


def split(v):
    import numpy as np
    hi = np.float32(float(v))
    lo = np.float32(float(v - mp.mpf(float(hi))))
    return hi, lo


def main():
    nint = int(XMAX / WIDTH)
    out = ["// fb_ewald_fit.h -- generated by gen_ewald_fit.py; do not edit.",
           "// Piecewise degree-%d fits of erfc(x) and erfc(x) + 2x exp(-x^2)/sqrt(pi) on"
           " [0, %s]," % (DEG, mp.nstr(XMAX, 3)),
           "// %d intervals of width 1/4, t = 8 (x - a) - 1, coefficients lowest first as" % nint,
           "// (hi, lo) float pairs: EW_FIT[f][interval][k][2], f = 0 erfc, 1 the force function.",
           "#pragma once", "", "namespace fb {", "",
           "constexpr int EW_FIT_NINT = %d, EW_FIT_NC = %d;" % (nint, DEG + 1),
           "constexpr float EW_FIT_XMAX = %sf;" % mp.nstr(XMAX, 3), "",
           "__device__ const float EW_FIT[2][%d][%d][2] = {" % (nint, DEG + 1)]
    worst = mp.mpf(0)
    for f in (E, H):
        out.append("  {")
        for i in range(nint):
            a = i * WIDTH
            mono, err = fit(f, a, a + WIDTH)
            worst = max(worst, err)
            pairs = []
            for v in mono:
                hi, lo = split(v)
                pairs.append("{%.9ef, %.9ef}" % (hi, lo))
            out.append("    {" + ", ".join(pairs) + "},")
        out.append("  },")
    out.append("};")
    out.append("")
    out.append("// largest interpolation error of the fits: %s" % mp.nstr(worst, 3))
    out.append("")
    out.append("}  // namespace fb")
    print("\n".join(out))


if __name__ == "__main__":
    main()
