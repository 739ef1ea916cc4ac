"""The TNFW bracket polynomial of the many-deflector kernels, restated on the
host.  The prepare kernel fits the bracket b(x) of TNFW's g(x) = tau^2/(tau^2+1)^2
b(x) (tnfw.py:331-349) outside x = s = max(tau, 1) by its Chebyshev interpolant
in t = 2 s/x - 1 at 12 nodes and stores the interpolant's monomial coefficients
in t; the bulk and multi-plane kernels evaluate them by Horner's rule (FP64 for
strong halos, FP32 for subhalos).  Checked here against the oracle's closed form:
the fit itself within 1.3e-9 relative for tau in [0.05, 300], and the same
coefficients rounded to FP32 and evaluated in FP32 within a few FP32 ulps."""

import numpy as np
import pytest

from oracle import lens as olens

NC = 12  # terms of the polynomial (TNFW_NC)


def bracket(x, tau):
    return olens.tnfw_g(x, tau) * (tau ** 2 + 1) ** 2 / tau ** 2


def fit(tau):
    """Monomial coefficients in t of the NC-node Chebyshev interpolant of b(s/z),
    z = (1 + t)/2 in [0, 1]."""
    s = max(tau, 1.0)
    k = np.arange(NC)
    t = np.cos(np.pi * (k + 0.5) / NC)
    f = bracket(2.0 * s / (1.0 + t), tau)
    ch = (2.0 / NC) * np.cos(np.outer(k, np.arccos(t))) @ f
    ch[0] /= 2.0
    return np.polynomial.chebyshev.cheb2poly(ch), s


def horner(c, t, dtype):
    c = c.astype(dtype)
    t = t.astype(dtype)
    b = np.full_like(t, c[-1])
    for ck in c[-2::-1]:
        b = (b * t + ck).astype(dtype)
    return b


@pytest.mark.parametrize("tau", [0.05, 0.3, 1.0, 1.05, 2.0, 10.0, 40.0, 300.0])
def test_bracket_polynomial_matches_the_closed_form(tau):
    mono, s = fit(tau)
    z = np.concatenate([np.geomspace(1e-4, 1.0, 400), np.linspace(0.5, 1.0, 101)])
    x = s / z
    ref = bracket(x, tau)
    t = 2.0 * z - 1.0
    rel64 = np.abs(horner(mono, t, np.float64) - ref) / np.abs(ref)
    assert rel64.max() <= 1.5e-9, (tau, rel64.max())
    # the coefficients' absolute values sum to below 2 b: Horner's rule stays
    # well conditioned in FP32
    assert np.abs(mono).sum() <= 2.0 * np.abs(ref).min()
    rel32 = np.abs(horner(mono, t, np.float32).astype(np.float64) - ref) / np.abs(ref)
    assert rel32.max() <= 3e-7, (tau, rel32.max())
