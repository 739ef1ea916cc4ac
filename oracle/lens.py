"""Lens-profile deflections and single-plane ray shooting (oracle, FP64).

Every profile function takes 1d FP64 ray coordinates and the profile's kwargs
exactly as named by the reference's ``param_names`` and returns (alpha_x,
alpha_y).  Citations are relative to the JAXtronomy source tree.
"""

import numpy as np

# ---------------------------------------------------------------------------
# geometry helpers
# ---------------------------------------------------------------------------


def ellipticity2phi_q(e1, e2):
    """``jaxtronomy/Util/param_util.py:88-99``."""
    phi = np.arctan2(e2, e1) / 2
    c = np.sqrt(e1 ** 2 + e2 ** 2)
    c = np.minimum(c, 0.9999)
    q = (1 - c) / (1 + c)
    return phi, q


def rotate(x, y, angle):
    """``jaxtronomy/Util/util.py:103-113`` (counter-clockwise by ``angle``)."""
    return x * np.cos(angle) + y * np.sin(angle), -x * np.sin(angle) + y * np.cos(angle)


def _f(x):
    return np.asarray(x, dtype=float)


# ---------------------------------------------------------------------------
# SHEAR  (jaxtronomy/LensModel/Profiles/shear.py:39-53)
# ---------------------------------------------------------------------------


def shear(x, y, gamma1, gamma2, ra_0=0.0, dec_0=0.0):
    x_ = _f(x) - ra_0
    y_ = _f(y) - dec_0
    return gamma1 * x_ + gamma2 * y_, gamma2 * x_ - gamma1 * y_


# ---------------------------------------------------------------------------
# NIE / SIE  (jaxtronomy/LensModel/Profiles/nie.py, sie.py)
# ---------------------------------------------------------------------------


def nie_param_conv(theta_E, e1, e2, s_scale):
    """``nie.py:182-200`` with ``_theta_E_prod_average2major_axis`` (:255-272)."""
    phi_G, q = ellipticity2phi_q(e1, e2)
    theta_E_conv = theta_E / np.sqrt((1.0 + q ** 2) / (2.0 * q))
    b = theta_E_conv * np.sqrt((1 + q ** 2) / 2)
    s = s_scale / np.sqrt(q)
    return b, s, q, phi_G


def nie_major_axis(x, y, b, s, q):
    """``NIEMajorAxis.derivatives`` ``nie.py:280-294``."""
    q = np.where(q >= 1, 0.99999999, q)
    psi = np.sqrt(q ** 2 * (s ** 2 + x ** 2) + y ** 2)
    sq = np.sqrt(1.0 - q ** 2)
    f_x = b / sq * np.arctan(sq * x / (psi + s))
    f_y = b / sq * np.arctanh(sq * y / (psi + q ** 2 * s))
    return f_x, f_y


def nie(x, y, theta_E, e1, e2, s_scale, center_x=0.0, center_y=0.0):
    """``NIE.derivatives`` ``nie.py:86-107``."""
    b, s, q, phi_G = nie_param_conv(theta_E, e1, e2, s_scale)
    x_, y_ = rotate(_f(x) - center_x, _f(y) - center_y, phi_G)
    fx, fy = nie_major_axis(x_, y_, b, s, q)
    return rotate(fx, fy, -phi_G)


SIE_S_SCALE = 0.0000000001  # sie.py:56 (SIE routes to NIE with this s_scale)


def sie(x, y, theta_E, e1, e2, center_x=0.0, center_y=0.0):
    """``SIE.derivatives`` ``sie.py:105-124`` (NIE branch, the default)."""
    return nie(x, y, theta_E, e1, e2, SIE_S_SCALE, center_x, center_y)


# ---------------------------------------------------------------------------
# EPL  (jaxtronomy/LensModel/Profiles/epl.py, jaxtronomy/Util/hyp2f1_util.py)
# ---------------------------------------------------------------------------


def hyp2f1_lopez_temme_8(a, b, c, z, nmax=75):
    """``hyp2f1_util.py:135-176``: Lopez & Temme (2013) eq. 8 with the contiguous
    recurrence F_n = ((n-1) F_{n-2} - (2b-c) F_{n-1}) / (c+n-1)."""
    z = np.asarray(z, dtype=complex)
    w = z / (z - 2.0)
    pref = a * w
    prev_prev_F = 1.0
    prev_F = 1.0 - 2.0 * b / c
    total = 1 + pref * prev_F
    for n in range(2, nmax):
        pref = pref * ((a + n - 1.0) / n) * w
        new_F = ((n - 1.0) * prev_prev_F - (2.0 * b - c) * prev_F) / (c + n - 1.0)
        total = total + pref * new_F
        prev_prev_F = prev_F
        prev_F = new_F
    return (1.0 - z / 2.0) ** (-a) * total


def epl_nmax(f):
    """Series length chosen from f = (1-q)/(1+q), ``epl.py:311-319``.
    Returns 0 for the f == 0 case, where the reference returns 1 exactly."""
    if f == 0:
        return 0
    if f < 0.12:
        return 10
    if f < 0.4:
        return 20
    if f < 0.6:
        return 35
    if f < 0.73:
        return 50
    if f < 0.86:
        return 100
    if f < 0.92:
        return 200
    return 500


def epl_param_conv(theta_E, gamma, e1, e2):
    """``EPL._param_conv`` ``epl.py:111-124``."""
    t = gamma - 1
    phi_G, q = ellipticity2phi_q(e1, e2)
    b = theta_E * np.sqrt(q)
    return b, t, q, phi_G


def epl_major_axis(x, y, b, t, q):
    """``EPLMajorAxis.derivatives`` ``epl.py:366-394``."""
    Z = q * x + y * 1j
    R = np.abs(Z)
    R = np.maximum(R, 0.000000001)
    f = (1.0 - q) / (1.0 + q)
    nmax = epl_nmax(float(f))
    if nmax == 0:
        hyp = np.ones_like(Z)
    else:
        B = t / 2.0
        C = 2.0 - B
        with np.errstate(invalid="ignore", divide="ignore"):
            hyp = hyp2f1_lopez_temme_8(1, B, C, -f * Z / np.conj(Z), nmax=nmax)
    R_omega = Z * hyp
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        alpha = 2 / (1 + q) * (b / R) ** t * R_omega
    ar = np.nan_to_num(alpha.real, posinf=10 ** 10, neginf=-(10 ** 10))
    ai = np.nan_to_num(alpha.imag, posinf=10 ** 10, neginf=-(10 ** 10))
    return ar, ai


def epl(x, y, theta_E, gamma, e1, e2, center_x=0.0, center_y=0.0):
    """``EPL.derivatives`` ``epl.py:179-200``."""
    b, t, q, phi_G = epl_param_conv(theta_E, gamma, e1, e2)
    x_, y_ = rotate(_f(x) - center_x, _f(y) - center_y, phi_G)
    fx, fy = epl_major_axis(x_, y_, b, t, q)
    return rotate(fx, fy, -phi_G)


# ---------------------------------------------------------------------------
# NFW  (jaxtronomy/LensModel/Profiles/nfw.py)
# ---------------------------------------------------------------------------


def nfw_alpha2rho0(alpha_Rs, Rs):
    """``nfw.py:386-395``."""
    return alpha_Rs / (4.0 * Rs ** 2 * (1.0 + np.log(1.0 / 2.0)))


def nfw_g(X):
    """``nfw.py:347-365``."""
    X = np.where(X < 0.000001, 0.000001, X)
    with np.errstate(invalid="ignore", divide="ignore"):
        lo = np.log(X / 2.0) + 1 / np.sqrt(1 - X ** 2) * np.arccosh(1.0 / X)
        hi = np.log(X / 2) + 1 / np.sqrt(X ** 2 - 1) * np.arccos(1.0 / X)
    return np.where(X < 1, lo, np.where(X == 1, 1 + np.log(1.0 / 2.0), hi))


def nfw(x, y, Rs, alpha_Rs, center_x=0.0, center_y=0.0):
    """``NFW.derivatives`` ``nfw.py:88-105`` -> ``nfw_alpha`` :259-279."""
    rho0 = nfw_alpha2rho0(alpha_Rs, Rs)
    Rs = np.where(Rs < 0.0000001, 0.0000001, Rs)
    x_ = _f(x) - center_x
    y_ = _f(y) - center_y
    R = np.sqrt(x_ ** 2 + y_ ** 2)
    R = np.maximum(R, 0.00000001)
    X = R / Rs
    a = 4 * rho0 * Rs * nfw_g(X) / X ** 2
    return a * x_, a * y_


# ---------------------------------------------------------------------------
# TNFW  (jaxtronomy/LensModel/Profiles/tnfw.py)
# ---------------------------------------------------------------------------

TNFW_S = 0.001  # tnfw.py:43


def tnfw_F(x):
    """``TNFW.F`` ``tnfw.py:290-304``."""
    x = np.maximum(x, TNFW_S)
    with np.errstate(invalid="ignore", divide="ignore"):
        lo = (1 - x ** 2) ** -0.5 * np.arctanh((1 - x ** 2) ** 0.5)
        hi = (x ** 2 - 1) ** -0.5 * np.arctan((x ** 2 - 1) ** 0.5)
    r = np.where(x < 1, lo, x)
    return np.where(x > 1, hi, r)


def tnfw_L(x, tau):
    """``TNFW._L`` ``tnfw.py:278-286``."""
    x = np.maximum(x, TNFW_S)
    return np.log(x * (tau + np.sqrt(tau ** 2 + x ** 2)) ** -1)


def tnfw_g(x, tau):
    """``TNFW._g`` ``tnfw.py:331-349``."""
    x = np.maximum(x, TNFW_S)
    return tau ** 2 / (tau ** 2 + 1) ** 2 * (
        (tau ** 2 + 1 + 2 * (x ** 2 - 1)) * tnfw_F(x)
        + tau * np.pi
        + (tau ** 2 - 1) * np.log(tau)
        + np.sqrt(tau ** 2 + x ** 2) * (-np.pi + tnfw_L(x, tau) * (tau ** 2 - 1) / tau)
    )


def tnfw(x, y, Rs, alpha_Rs, r_trunc, center_x=0.0, center_y=0.0):
    """``TNFW.derivatives`` ``tnfw.py:69-87`` -> ``tnfw_alpha`` :228-248."""
    rho0 = nfw_alpha2rho0(alpha_Rs, Rs)
    x_ = _f(x) - center_x
    y_ = _f(y) - center_y
    R = np.sqrt(x_ ** 2 + y_ ** 2)
    R = np.maximum(R, TNFW_S * Rs)
    X = np.maximum(R / Rs, TNFW_S)
    tau = r_trunc / Rs
    a = 4 * rho0 * Rs * tnfw_g(X, tau) / X ** 2
    return a * x_, a * y_


# ---------------------------------------------------------------------------
# registry and single-plane ray shooting
# ---------------------------------------------------------------------------

PROFILES = {
    "SIE": (sie, ["theta_E", "e1", "e2", "center_x", "center_y"]),
    "NIE": (nie, ["theta_E", "e1", "e2", "s_scale", "center_x", "center_y"]),
    "EPL": (epl, ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"]),
    "SHEAR": (shear, ["gamma1", "gamma2", "ra_0", "dec_0"]),
    "NFW": (nfw, ["Rs", "alpha_Rs", "center_x", "center_y"]),
    "TNFW": (tnfw, ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"]),
}

# defaults of optional keyword arguments in the profile signatures
DEFAULTS = {"center_x": 0.0, "center_y": 0.0, "ra_0": 0.0, "dec_0": 0.0}


def deflection(name, x, y, kwargs):
    func, names = PROFILES[name]
    args = {k: kwargs[k] if k in kwargs else DEFAULTS[k] for k in names}
    return func(x, y, **args)


def alpha(lens_model_list, x, y, kwargs_list, alpha_scaling=1.0):
    """``SinglePlane.alpha`` ``single_plane.py:113-139``."""
    x = _f(x)
    y = _f(y)
    fx = np.zeros_like(x)
    fy = np.zeros_like(y)
    for name, kw in zip(lens_model_list, kwargs_list):
        ax, ay = deflection(name, x, y, kw)
        fx = fx + ax
        fy = fy + ay
    return fx * alpha_scaling, fy * alpha_scaling


def ray_shooting(lens_model_list, x, y, kwargs_list, alpha_scaling=1.0):
    """``SinglePlane.ray_shooting`` ``single_plane.py:39-56``."""
    ax, ay = alpha(lens_model_list, x, y, kwargs_list, alpha_scaling)
    return _f(x) - ax, _f(y) - ay
