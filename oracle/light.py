"""Light-profile surface brightness (oracle, FP64).

Citations are relative to the JAXtronomy source tree.
"""

import numpy as np

SMOOTHING = 0.0001  # SersicUtil default smoothing, sersic_utils.py:13


def b_n(n):
    """``SersicUtil.b_n`` ``sersic_utils.py:69-80``."""
    return np.maximum(1.9992 * n - 0.3271, 0.00001)


def transform_e1e2_product_average(x, y, e1, e2, center_x, center_y):
    """``jaxtronomy/Util/param_util.py:103-123``."""
    x_shift = x - center_x
    y_shift = y - center_y
    norm = np.maximum(np.sqrt(np.abs(1 - e1 ** 2 - e2 ** 2)), 0.000001)
    x_ = ((1 - e1) * x_shift - e2 * y_shift) / norm
    y_ = (-e2 * x_shift + (1 + e1) * y_shift) / norm
    return x_, y_


def r_sersic(R, R_sersic, n_sersic, max_R_frac=1000.0):
    """``SersicUtil._r_sersic`` ``sersic_utils.py:248-267`` with ``_R_stable``
    :239-245."""
    R_ = np.maximum(SMOOTHING, R)
    R_sersic_ = np.maximum(SMOOTHING, R_sersic)
    bn = b_n(n_sersic)
    R_frac = R_ / R_sersic_
    exponent = -bn * (R_frac ** (1.0 / n_sersic) - 1.0)
    with np.errstate(over="ignore"):
        result = np.where(R_frac <= max_R_frac, np.exp(exponent), 0)
    return np.nan_to_num(result)


def sersic_ellipse(x, y, amp, R_sersic, n_sersic, e1, e2, center_x=0.0, center_y=0.0,
                   max_R_frac=1000.0):
    """``SersicElliptic.function`` ``LightModel/Profiles/sersic_ellipse.py:62-93``
    (product-average radius, ``sersic_major_axis=False`` default,
    ``sersic_utils.py:83-110``)."""
    R_sersic = np.maximum(0, R_sersic)
    x_, y_ = transform_e1e2_product_average(np.asarray(x, float), np.asarray(y, float),
                                            e1, e2, center_x, center_y)
    R = np.sqrt(x_ ** 2 + y_ ** 2)
    return amp * r_sersic(R, R_sersic, n_sersic, max_R_frac)


def sersic(x, y, amp, R_sersic, n_sersic, center_x=0.0, center_y=0.0, max_R_frac=1000.0):
    """``Sersic.function`` ``LightModel/Profiles/sersic.py:54-73`` (e1 = e2 = 0)."""
    x_ = np.asarray(x, float) - center_x
    y_ = np.asarray(y, float) - center_y
    R = np.sqrt(x_ ** 2 + y_ ** 2)
    return amp * r_sersic(R, R_sersic, n_sersic, max_R_frac)


PROFILES = {
    "SERSIC": (sersic, ["amp", "R_sersic", "n_sersic", "center_x", "center_y"]),
    "SERSIC_ELLIPSE": (sersic_ellipse,
                       ["amp", "R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y"]),
}

DEFAULTS = {"center_x": 0.0, "center_y": 0.0}


def profile(name, x, y, kwargs):
    func, names = PROFILES[name]
    args = {k: kwargs[k] if k in kwargs else DEFAULTS[k] for k in names}
    return func(x, y, **args)


def surface_brightness(light_model_list, x, y, kwargs_list, k=None):
    """``LightModelBase.surface_brightness`` ``light_model_base.py:230-252``."""
    x = np.asarray(x, float)
    flux = np.zeros_like(x)
    for i, (name, kw) in enumerate(zip(light_model_list, kwargs_list)):
        if k is None or i == k or (isinstance(k, (list, tuple)) and i in k):
            flux = flux + profile(name, x, y, kw)
    return flux
