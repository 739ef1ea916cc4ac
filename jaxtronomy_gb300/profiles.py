"""Profile registry: names, parameter order and kwargs packing.

Parameter names and their order are the reference profiles' ``param_names``
(JAXtronomy: ``LensModel/Profiles/sie.py:40``, ``nie.py:19``, ``epl.py:50``,
``shear.py:16``, ``convergence.py:15``, ``nfw.py:49``, ``tnfw.py:27``, ``nfw_ellipse_cse.py:172``,
``epl_multipole_m1m3m4.py:415-428``,
``LightModel/Profiles/sersic.py:27``, ``sersic_ellipse.py:25``).  The packed
row layout is the one documented in ``include/lensgb.h``.
"""

import numpy as np

from . import _lib

LENS_PARAMS = {
    "SIE": ["theta_E", "e1", "e2", "center_x", "center_y"],
    "NIE": ["theta_E", "e1", "e2", "s_scale", "center_x", "center_y"],
    "EPL": ["theta_E", "gamma", "e1", "e2", "center_x", "center_y"],
    "SHEAR": ["gamma1", "gamma2", "ra_0", "dec_0"],
    "CONVERGENCE": ["kappa", "ra_0", "dec_0"],
    "NFW": ["Rs", "alpha_Rs", "center_x", "center_y"],
    "TNFW": ["Rs", "alpha_Rs", "r_trunc", "center_x", "center_y"],
    "NFW_ELLIPSE_CSE": ["Rs", "alpha_Rs", "e1", "e2", "center_x", "center_y"],
    "EPL_MULTIPOLE_M1M3M4": ["theta_E", "gamma", "e1", "e2", "center_x", "center_y", "a1_a",
                             "delta_phi_m1", "a3_a", "delta_phi_m3", "a4_a", "delta_phi_m4"],
}

# Positional order of each lens profile's ``derivatives`` signature where it
# differs from ``param_names`` (epl_multipole_m1m3m4.py:608-622 vs :415-428).
# The reference's bulk path binds parameter arrays positionally in param_names
# order (profile_list_base.py:768-778), so for these profiles the bulk
# evaluation sees the values shifted into the signature's slots.
DERIVATIVES_SIGNATURE = {
    "EPL_MULTIPOLE_M1M3M4": ["theta_E", "gamma", "e1", "e2", "a1_a", "delta_phi_m1", "a3_a",
                             "delta_phi_m3", "a4_a", "delta_phi_m4", "center_x", "center_y"],
}

LIGHT_PARAMS = {
    "SERSIC": ["amp", "R_sersic", "n_sersic", "center_x", "center_y"],
    "SERSIC_ELLIPSE": ["amp", "R_sersic", "n_sersic", "e1", "e2", "center_x", "center_y"],
}

# optional arguments of the profile functions and their defaults
DEFAULTS = {"center_x": 0.0, "center_y": 0.0, "ra_0": 0.0, "dec_0": 0.0}

assert set(LENS_PARAMS) == set(_lib.LENS_CODES)
assert set(LIGHT_PARAMS) == set(_lib.LIGHT_CODES)


def check_names(model_list, table, what):
    for name in model_list:
        if name not in table:
            raise ValueError("%s model of type %s not supported! Supported models are %s"
                             % (what, name, sorted(table)))


def check_parameters(model_list, table, kwargs_list, what):
    """Mirror of ``ProfileListBase.check_parameters`` (profile_list_base.py:278-306)
    and ``LightModelBase.check_parameters`` (light_model_base.py:373-401)."""
    if len(kwargs_list) != len(model_list):
        raise ValueError("length of input parameter list %s does not match number of %s models %s"
                         % (len(kwargs_list), what, len(model_list)))
    for i, name in enumerate(model_list):
        names = table[name]
        for key in kwargs_list[i]:
            if key not in names:
                raise ValueError("parameter %s in %s model is not part of model %s (%s). "
                                 "Parameters allowed are %s" % (key, what, i, name, names))
        for key in names:
            if key not in kwargs_list[i]:
                raise ValueError("%s model %s (%s) requires parameter %s which is not provided "
                                 "in input." % (what, i, name, key))


def batch_size(*kwargs_lists):
    """Common leading length of array-valued kwargs (1 for scalars)."""
    b = None
    for kl in kwargs_lists:
        for kw in kl or []:
            for v in kw.values():
                if isinstance(v, (float, int)):  # Python and NumPy float scalars
                    continue
                a = np.asarray(v)
                if a.ndim == 0:
                    continue
                n = a.reshape(-1).shape[0] if a.ndim == 1 else a.shape[0]
                if b is None:
                    b = n
                elif n != b:
                    raise ValueError("inconsistent batch sizes in kwargs: %d vs %d" % (b, n))
    return 1 if b is None else b


def pack(model_list, table, kwargs_list, rows, col0, what):
    """Write the kwargs of ``model_list`` into ``rows[:, col0:]``; returns the next
    free column."""
    if kwargs_list is None:
        kwargs_list = [{} for _ in model_list]
    if len(kwargs_list) != len(model_list):
        raise ValueError("length of %s kwargs list %d does not match the %d %s models"
                         % (what, len(kwargs_list), len(model_list), what))
    col = col0
    for name, kw in zip(model_list, kwargs_list):
        for key in table[name]:
            if key in kw:
                v = kw[key]
                if isinstance(v, (float, int)):  # a scalar: broadcast without an array
                    rows[:, col] = v
                else:
                    rows[:, col] = np.asarray(v, dtype=np.float64).reshape(-1)
            elif key in DEFAULTS:
                rows[:, col] = DEFAULTS[key]
            else:
                raise ValueError("%s model %s requires parameter %s which is not provided"
                                 % (what, name, key))
            col += 1
    return col


def n_params(model_list, table):
    return sum(len(table[n]) for n in model_list)
