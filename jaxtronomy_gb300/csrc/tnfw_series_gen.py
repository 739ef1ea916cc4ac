"""Derives the large-x series of the TNFW deflection bracket used by the FP32
many-deflector path and prints it as C statements for prepare.cu.

TNFW (tnfw.py:331-349):  g(x) = tau^2/(tau^2+1)^2 * b(x) with
  b(x) = (tau^2 + 1 + 2 (x^2 - 1)) F(x) + tau pi + (tau^2 - 1) ln tau
         + r (-pi + L (tau^2 - 1)/tau),   r = sqrt(tau^2 + x^2), L = ln(x/(tau + r)).
With eps = 1/x:  F = eps (pi/2 - asin eps)/sqrt(1 - eps^2),  r = sqrt(1 + tau^2 eps^2)/eps,
L = -asinh(tau eps), and b(eps) = sum_k b_k(tau) eps^k (the 1/eps terms cancel).  Truncated
after eps^15 the series is within 1e-8 (relative) of b for x >= max(3 tau, 3).

Usage:  python jaxtronomy_gb300/csrc/tnfw_series_gen.py
"""

import sympy as sp

N = 16


def coefficients():
    e, t = sp.symbols("epsilon tau", positive=True)
    F = e * (sp.pi / 2 - sp.asin(e)) / sp.sqrt(1 - e ** 2)
    b = ((2 / e ** 2 + t ** 2 - 1) * F + t * sp.pi + (t ** 2 - 1) * sp.log(t)
         + sp.sqrt(1 + t ** 2 * e ** 2) / e * (-sp.pi - sp.asinh(t * e) * (t ** 2 - 1) / t))
    ser = sp.expand(sp.series(b, e, 0, N).removeO())
    return t, [sp.expand(ser.coeff(e, k)) for k in range(N)]


def main():
    t, cs = coefficients()
    tau = sp.Symbol("tau")
    for k, c in enumerate(cs):
        c = sp.expand_log(c.subs(t, tau), force=True)
        print("        d[%d] = %s;" % (12 + k, sp.ccode(sp.nsimplify(c))))


if __name__ == "__main__":
    main()
