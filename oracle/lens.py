"""Lens-profile deflections, single-plane and multi-plane bulk ray shooting
(oracle, FP64; test infrastructure).

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
# CONVERGENCE  (jaxtronomy/LensModel/Profiles/convergence.py:33-46)
# ---------------------------------------------------------------------------


def convergence(x, y, kappa, ra_0=0.0, dec_0=0.0):
    return kappa * (_f(x) - ra_0), kappa * (_f(y) - dec_0)


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
# NFW_ELLIPSE_CSE  (jaxtronomy/LensModel/Profiles/nfw_ellipse_cse.py,
#                   cored_steep_ellipsoid.py)
# ---------------------------------------------------------------------------

# Oguri (2021, arXiv:2106.11464) Table 1: the 44-term cored-steep-ellipsoid
# decomposition of the NFW profile, (a_k, s_k) in units of the scale radius,
# as used by the reference's high_accuracy=True default (nfw_ellipse_cse.py:15-156).
CSE_NFW_A = np.array([
    1.648988e-18, 6.274458e-16, 3.646620e-17, 3.459206e-15, 2.457389e-14, 1.059319e-13,
    4.211597e-13, 1.142832e-12, 4.391215e-12, 1.556500e-11, 6.951271e-11, 3.147466e-10,
    1.379109e-09, 3.829778e-09, 1.384858e-08, 5.370951e-08, 1.804384e-07, 5.788608e-07,
    3.205256e-06, 1.102422e-05, 4.093971e-05, 1.282206e-04, 4.575541e-04, 7.995270e-04,
    5.013701e-03, 1.403508e-02, 5.230727e-02, 1.898907e-01, 3.643448e-01, 7.203734e-01,
    1.717667e+00, 2.217566e+00, 3.187447e+00, 8.194898e+00, 1.765210e+01, 1.974319e+01,
    2.783688e+01, 4.482311e+01, 5.598897e+01, 1.426485e+02, 2.279833e+02, 5.401335e+02,
    9.743682e+02, 1.775124e+03])
CSE_NFW_S = np.array([
    1.082411e-06, 8.786566e-06, 3.292868e-06, 1.860019e-05, 3.274231e-05, 6.232485e-05,
    9.256333e-05, 1.546762e-04, 2.097321e-04, 3.391140e-04, 5.178790e-04, 8.636736e-04,
    1.405152e-03, 2.193855e-03, 3.179572e-03, 4.970987e-03, 7.631970e-03, 1.119413e-02,
    1.827267e-02, 2.945251e-02, 4.562723e-02, 6.782509e-02, 1.596987e-01, 1.127751e-01,
    2.169469e-01, 3.423835e-01, 5.194527e-01, 8.623185e-01, 1.382737e+00, 2.034929e+00,
    3.402979e+00, 5.594276e+00, 8.052345e+00, 1.349045e+01, 2.603825e+01, 4.736823e+01,
    6.559320e+01, 1.087932e+02, 1.477673e+02, 2.495341e+02, 4.305999e+02, 7.760206e+02,
    2.143057e+03, 1.935749e+03])


def cse_major_axis(x, y, a, s, q):
    """``CSEMajorAxis.derivatives`` ``cored_steep_ellipsoid.py:227-245``."""
    psi = np.sqrt(q ** 2 * (s ** 2 + x ** 2) + y ** 2)
    Phi = (psi + s) ** 2 + (1 - q ** 2) * x ** 2
    f_x = q * x * (psi + q ** 2 * s) / (s * psi * Phi)
    f_y = q * y * (psi + s) / (s * psi * Phi)
    return a * f_x, a * f_y


def cse_product_avg_set(x, y, a_list, s_list, q):
    """``CSEProductAvgSet.derivatives`` :536-564 over ``CSEProductAvg.derivatives``
    :463-477 (product-average conversion :434-443)."""
    fx = np.zeros_like(x)
    fy = np.zeros_like(y)
    for a, s in zip(a_list, s_list):
        xa, ya = x * np.sqrt(q), y * np.sqrt(q)
        ax, ay = cse_major_axis(xa, ya, a / q, s, q)
        fx = fx + np.sqrt(q) * ax
        fy = fy + np.sqrt(q) * ay
    return fx, fy


def nfw_ellipse_cse(x, y, Rs, alpha_Rs, e1, e2, center_x=0.0, center_y=0.0):
    """``NFW_ELLIPSE_CSE.derivatives`` ``nfw_ellipse_cse.py:250-280`` with
    ``_normalization`` :338-349."""
    phi_q, q = ellipticity2phi_q(e1, e2)
    x_, y_ = rotate(_f(x) - center_x, _f(y) - center_y, phi_q)
    fx, fy = cse_product_avg_set(x_ / Rs, y_ / Rs, CSE_NFW_A, CSE_NFW_S, q)
    fx, fy = rotate(fx, fy, -phi_q)
    const = 4 * nfw_alpha2rho0(alpha_Rs, Rs) * Rs ** 3 / Rs
    return const * fx, const * fy


# ---------------------------------------------------------------------------
# circular multipoles and EPL_MULTIPOLE_M1M3M4
# (jaxtronomy/LensModel/Profiles/multipole.py, epl_multipole_m1m3m4.py)
# ---------------------------------------------------------------------------


def multipole(x, y, m, a_m, phi_m, center_x=0.0, center_y=0.0, r_E=1.0):
    """``Multipole.derivatives`` ``multipole.py:72-119`` (Xu et al. 2013, B12)."""
    dx = _f(x) - center_x
    dy = _f(y) - center_y
    r = np.sqrt(dx ** 2 + dy ** 2)
    phi = np.arctan2(dy, dx)
    if m == 1:
        r = np.maximum(r, 0.000001)
        f_x = a_m / 2 * (np.cos(phi_m) * np.log(r / r_E) + np.cos(phi - phi_m) * np.cos(phi))
        f_y = a_m / 2 * (np.sin(phi_m) * np.log(r / r_E) + np.cos(phi - phi_m) * np.sin(phi))
        return f_x, f_y
    f_x = np.cos(phi) * a_m / (1 - m ** 2) * np.cos(m * (phi - phi_m)) \
        + np.sin(phi) * m * a_m / (1 - m ** 2) * np.sin(m * (phi - phi_m))
    f_y = np.sin(phi) * a_m / (1 - m ** 2) * np.cos(m * (phi - phi_m)) \
        - np.cos(phi) * m * a_m / (1 - m ** 2) * np.sin(m * (phi - phi_m))
    return f_x, f_y


def epl_multipole_m1m3m4(x, y, theta_E, gamma, e1, e2, a1_a, delta_phi_m1, a3_a, delta_phi_m3,
                         a4_a, delta_phi_m4, center_x=0.0, center_y=0.0):
    """``EPL_MULTIPOLE_M1M3M4.derivatives`` ``epl_multipole_m1m3m4.py:608-678``
    with ``_param_split`` :463-535."""
    phi, q = ellipticity2phi_q(e1, e2)
    rescale_am = theta_E / np.sqrt(q)
    fx, fy = epl(x, y, theta_E, gamma, e1, e2, center_x, center_y)
    f3 = multipole(x, y, 3, a3_a * rescale_am, phi + delta_phi_m3, center_x, center_y)
    f4 = multipole(x, y, 4, a4_a * rescale_am, phi + delta_phi_m4, center_x, center_y)
    f1 = multipole(x, y, 1, a1_a * rescale_am, phi + delta_phi_m1, center_x, center_y,
                   r_E=theta_E)
    return fx + f3[0] + f4[0] + f1[0], fy + f3[1] + f4[1] + f1[1]


# ---------------------------------------------------------------------------
# registry and single-plane ray shooting
# ---------------------------------------------------------------------------

PROFILES = {
    "SIE": (sie, ["theta_E", "e1", "e2", "center_x", "center_y"]),
    "NIE": (nie, ["theta_E", "e1", "e2", "s_scale", "center_x", "center_y"]),
    "EPL": (epl, ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"]),
    "SHEAR": (shear, ["gamma1", "gamma2", "ra_0", "dec_0"]),
    "CONVERGENCE": (convergence, ["kappa", "ra_0", "dec_0"]),
    "NFW": (nfw, ["Rs", "alpha_Rs", "center_x", "center_y"]),
    "TNFW": (tnfw, ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"]),
    "NFW_ELLIPSE_CSE": (nfw_ellipse_cse, ["Rs", "alpha_Rs", "e1", "e2", "center_x", "center_y"]),
    "EPL_MULTIPOLE_M1M3M4": (epl_multipole_m1m3m4,
                             ["theta_E", "gamma", "e1", "e2", "center_x", "center_y", "a1_a",
                              "delta_phi_m1", "a3_a", "delta_phi_m3", "a4_a", "delta_phi_m4"]),
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


# ---------------------------------------------------------------------------
# many-deflector single-plane ray shooting
# ---------------------------------------------------------------------------

def bulk_prepare(unique_lens_model_list, lens_model_list, kwargs_lens, num_deflectors=None):
    """``SinglePlaneBulk.prepare_ray_shooting_kwargs`` ``single_plane_bulk.py:47-106``."""
    if len(lens_model_list) != len(kwargs_lens):
        raise ValueError("length of lens model list and kwargs_lens do not match")
    if num_deflectors is None:
        num_deflectors = len(lens_model_list)
    elif num_deflectors < len(lens_model_list):
        raise ValueError("num_deflectors is smaller than the length of lens_model_list")
    num_filler = num_deflectors - len(kwargs_lens)
    index_list = [unique_lens_model_list.index(m) for m in lens_model_list]
    index_list += [len(unique_lens_model_list)] * num_filler
    names = set(p for m in unique_lens_model_list if m != "NULL" for p in PROFILES[m][1])
    all_kwargs = {}
    for k in names:
        all_kwargs[k] = np.array([kw.get(k, 0) for kw in kwargs_lens] + [0] * num_filler,
                                 dtype=float)
    return {"all_kwargs": all_kwargs, "index_list": np.array(index_list)}


def bulk_ray_shooting(unique_lens_model_list, x, y, all_kwargs, index_list):
    """``SinglePlaneBulk.ray_shooting`` ``single_plane_bulk.py:109-131``: one
    deflection per index (``lax.switch`` clamps the index into the unique list
    plus the trailing NULL profile), summed over deflectors.

    The reference binds each profile's arrays POSITIONALLY in ``param_names``
    order (``_select_kwargs``, ``profile_list_base.py:768-778``).  For
    EPL_MULTIPOLE_M1M3M4 that order (centre before the multipoles,
    ``epl_multipole_m1m3m4.py:415-428``) differs from the ``derivatives``
    signature (multipoles before the centre, :608-622), so in the bulk path its
    centre values land in a1_a / delta_phi_m1 and so on; the positional call
    below reproduces that."""
    x = _f(x)
    y = _f(y)
    n_u = len(unique_lens_model_list)
    fx = np.zeros_like(x)
    fy = np.zeros_like(y)
    for i, k in enumerate(np.asarray(index_list)):
        k = min(max(int(k), 0), n_u)
        name = unique_lens_model_list[k] if k < n_u else "NULL"
        if name == "NULL":
            continue
        func, names = PROFILES[name]
        ax, ay = func(x, y, *[float(all_kwargs[p][i]) for p in names])
        fx = fx + ax
        fy = fy + ay
    return x - fx, y - fy


# ---------------------------------------------------------------------------
# many-deflector multi-plane ray shooting
# ---------------------------------------------------------------------------

def multi_plane_distances(lens_redshift_list, z_source, d_xy, T_xy):
    """``MultiPlaneBulk._set_T_zs_and_T_ijs`` (``multi_plane_bulk.py:226-272``) for a
    SORTED redshift array, given the background's angular diameter distance
    ``d_xy(z1, z2)`` and transverse comoving distance ``T_xy(z1, z2)``:
    (T_ij list, T_z list, reduced2physical factors), the source appended."""
    z = np.asarray(lens_redshift_list, dtype=float)
    r2p = [d_xy(0, z_source) / d_xy(zi, z_source) for zi in z]
    T_ij, T_z = [], []
    z_before, tz = 0, 0
    for zi in list(z) + [z_source]:
        if z_before == zi:
            dt = 0
        else:
            tz = T_xy(0, zi)
            dt = T_xy(z_before, zi)
        T_ij.append(dt)
        T_z.append(tz)
        z_before = zi
    return T_ij, T_z, r2p


def multi_plane_prepare(unique_lens_model_list, lens_model_list, kwargs_lens, z_source,
                        lens_redshift_list, d_xy, T_xy, num_deflectors=None):
    """``MultiPlaneBulk.prepare_ray_shooting_kwargs`` (``multi_plane_bulk.py:57-150``):
    redshift sort (``np.argsort``, :203-224), index list with NULL entries for the
    source step and the fillers, zero-filled parameter arrays and the padded
    distance lists."""
    n = len(lens_model_list)
    if n != len(kwargs_lens) or n != len(lens_redshift_list):
        raise ValueError("lens model list, kwargs_lens and redshift list lengths differ")
    if num_deflectors is None:
        num_deflectors = n
    elif num_deflectors < n:
        raise ValueError("num_deflectors is smaller than the length of lens_model_list")
    z = np.array(lens_redshift_list)
    order = np.argsort(z)
    models = [lens_model_list[i] for i in order]
    kws = [kwargs_lens[i] for i in order]
    z = z[order]
    num_filler = num_deflectors - n
    index_list = [unique_lens_model_list.index(m) for m in models]
    index_list += [len(unique_lens_model_list)] * (num_filler + 1)
    names = set(p for m in unique_lens_model_list if m != "NULL" for p in PROFILES[m][1])
    all_kwargs = {k: np.array([kw.get(k, 0) for kw in kws] + [0] * (num_filler + 1), dtype=float)
                  for k in names}
    T_ij, T_z, r2p = multi_plane_distances(z, z_source, d_xy, T_xy)
    T_ij = np.array(T_ij + [0] * num_filler, dtype=float)
    T_z = np.array(T_z + [T_z[-1]] * num_filler, dtype=float)
    r2p = np.array(list(r2p) + [0] * (num_filler + 1), dtype=float)
    return {"all_kwargs": all_kwargs, "index_list": np.array(index_list), "T_ij_list": T_ij,
            "T_z_list": T_z, "reduced2physical_factor": r2p}


def multi_plane_ray_shooting(unique_lens_model_list, alpha_x, alpha_y, all_kwargs, index_list,
                             T_ij_list, T_z_list, reduced2physical_factor):
    """``MultiPlaneBulk.ray_shooting`` (``multi_plane_bulk.py:152-200``): the
    ``lax.scan`` over steps, x += alpha T_ij; alpha -= r2p * alpha_i(x / T_z);
    beta = x / T_z[-1].  Parameters are bound positionally as in
    :func:`bulk_ray_shooting`."""
    ax = _f(alpha_x).copy()
    ay = _f(alpha_y).copy()
    x = np.zeros_like(ax)
    y = np.zeros_like(ay)
    n_u = len(unique_lens_model_list)
    T_ij = _f(T_ij_list)
    T_z = _f(T_z_list)
    r2p = _f(reduced2physical_factor)
    for i, k in enumerate(np.asarray(index_list)):
        x = x + ax * T_ij[i]
        y = y + ay * T_ij[i]
        k = min(max(int(k), 0), n_u)
        name = unique_lens_model_list[k] if k < n_u else "NULL"
        if name == "NULL":
            continue
        func, names = PROFILES[name]
        fx, fy = func(x / T_z[i], y / T_z[i], *[float(all_kwargs[p][i]) for p in names])
        ax = ax - fx * r2p[i]
        ay = ay - fy * r2p[i]
    return x / T_z[-1], y / T_z[-1]
