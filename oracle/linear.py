"""Linear amplitude solve of ``ImageLinearFit`` (oracle, FP64; test infrastructure).

Restates ``jaxtronomy/ImSim/image_linear_solve.py:98-341`` for an empty
point-source list -- the unit-amplitude response of every light profile
(``linear_response_matrix``, ``:362-456``; lenstronomy's
``Image2SourceMapping.image_flux_split`` at ``:392``), the data-based error
response (``ImageModel.error_response``), the weighted least-squares solve
``de_lens.get_param_WLS`` (``de_lens.py:8-38``), the flat-prior marginalisation
constant (``de_lens.py:41-49``) and the positive-flux penalty
(``image_linear_solve.py:320-340``) -- on the scenes of :mod:`oracle.image`.
"""

import sys

import numpy as np

from . import image as oimage

EPSILON = sys.float_info.epsilon


def response(scene, kwargs_lens, kwargs_source, kwargs_lens_light, kwargs_ps=None,
             kwargs_special=None):
    """(n_linear, ny, nx): each source lensed alone and each lens-light profile
    alone, amp = 1 (flux scaling included, as ``linear_response_matrix`` applies it),
    then each point image alone at amp = 1 (``image_linear_solve.py:440-456``, no flux
    scaling; positions shifted as ``point_source_linear_response_set`` does,
    ``:559-600``), rendered with ``scene["ps_kernel"]`` at ``scene["ps_subgrid"]``."""
    src = scene.get("source_light_model_list", [])
    ll = scene.get("lens_light_model_list", [])
    dsl = scene.get("deflection_scaling_list")
    out = []
    for j, name in enumerate(src):
        sc = dict(scene, source_light_model_list=[name], lens_light_model_list=[],
                  deflection_scaling_list=None if dsl is None else [dsl[j]])
        out.append(oimage.image(sc, kwargs_lens, [dict(kwargs_source[j], amp=1.0)], []))
    for j, name in enumerate(ll):
        sc = dict(scene, source_light_model_list=[], lens_light_model_list=[name],
                  deflection_scaling_list=None)
        out.append(oimage.image(sc, kwargs_lens, [], [dict(kwargs_lens_light[j], amp=1.0)]))
    if kwargs_ps:
        from . import point_source as ops
        ra = np.concatenate([np.atleast_1d(np.asarray(p["ra_image"], float)) for p in kwargs_ps])
        dec = np.concatenate([np.atleast_1d(np.asarray(p["dec_image"], float))
                              for p in kwargs_ps])
        ra, dec = ops.displace_astrometry(ra, dec, kwargs_special)
        for j in range(len(ra)):
            out.append(ops.render(scene["nx"], scene["ny"], scene["transform_pix2angle"],
                                  scene["ra_at_xy_0"], scene["dec_at_xy_0"], ra[j:j + 1],
                                  dec[j:j + 1], [1.0], scene["ps_kernel"],
                                  scene.get("ps_subgrid", 1)))
    return np.nan_to_num(np.array(out))


def get_param_wls(A, C_D_inv, d, inv_bool=True):
    """``de_lens.get_param_WLS`` (``de_lens.py:8-38``); A is Nd x Ns."""
    M = A.T.dot(np.multiply(C_D_inv, A.T).T)
    stable = np.linalg.cond(M) < 5 / EPSILON
    R = A.T.dot(np.multiply(C_D_inv, d))
    if inv_bool:
        M_inv = np.nan_to_num(np.linalg.inv(M), nan=0, posinf=0, neginf=0) if stable else \
            np.zeros_like(M)
        B = M_inv.dot(R)
    else:
        B = np.zeros(len(A.T))
        if stable:
            b = np.linalg.solve(M, R).T
            B = b if np.all(np.isfinite(b)) else np.zeros(len(A.T))
        M_inv = None
    return B, M_inv, A.dot(B)


def marginalisation_const(M_inv):
    """``de_lens.py:41-49``."""
    sign, log_det = np.linalg.slogdet(M_inv)
    return -(10 ** 15) if sign == 0 else sign * log_det / 2


def likelihood(scene, kwargs_lens, kwargs_source, kwargs_lens_light, data, mask,
               background_rms, exposure_time=None, noise_map=None, source_marg=False,
               check_positive_flux=False, kwargs_ps=None):
    """(logL, amplitudes, model image, M^-1 or None) of ``likelihood_data_given_model``
    with the linear solve (``image_linear_solve.py:229-341``)."""
    mask = np.asarray(mask, dtype=bool)
    A = response(scene, kwargs_lens, kwargs_source, kwargs_lens_light, kwargs_ps)[:, mask]
    if noise_map is not None:
        c_d = np.asarray(noise_map, float) ** 2
    else:
        c_d = oimage.covariance_matrix(np.asarray(data, float), background_rms,
                                       oimage.exposure_floor(exposure_time))
    d = np.asarray(data, float)[mask]
    param, cov, wls = get_param_wls(A.T, 1 / c_d[mask], d, inv_bool=source_marg)
    model = np.zeros(np.shape(data))
    model[mask] = wls
    logl = oimage.log_likelihood(model, data, mask.astype(float), background_rms,
                                 exposure_time=exposure_time, noise_map=noise_map)
    if source_marg:
        logl = logl + marginalisation_const(cov)
    if check_positive_flux and np.any(param < 0):
        logl = logl - 10 ** 8
    return logl, param, model, cov
