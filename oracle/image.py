"""``ImageModel.image`` and the image log-likelihood (oracle, FP64).

Restates ``jaxtronomy/ImSim/image_model.py:163-492`` for an empty point-source
list together with ``Numerics.re_size_convolve`` (``numerics.py:158-177``),
``RegularGrid.flux_array2image_low_high`` (``grid.py:102-117``) and lenstronomy's
``Image2SourceMapping.image_flux_joint`` (called at ``image_model.py:347-354``):
for a single lens plane, source ``i`` is evaluated at
``theta - deflection_scaling[i] * alpha(theta)``.

A *scene* is a plain dict describing one ImageModel:

``nx, ny, transform_pix2angle (2x2), ra_at_xy_0, dec_at_xy_0,
supersampling_factor, psf_type ('NONE'|'PIXEL'|'GAUSSIAN'), kernel (PIXEL,
already normalised), fwhm and truncation (GAUSSIAN), convolution_type,
lens_model_list, source_light_model_list, lens_light_model_list,
flux_scaling, alpha_scaling, deflection_scaling_list``.
"""

import numpy as np

from . import grid, lens, light, numerics


def _source_scalings(scene):
    n = len(scene.get("source_light_model_list", []))
    dsl = scene.get("deflection_scaling_list")
    if dsl is None:
        return [1.0] * n
    return [float(v) for v in dsl]


def _subframe(scene):
    """``NumericsSubFrame._init_sub_frame`` / ``_sub_pixel_grid`` / ``_cut_frame``
    (numerics_subframe.py:151-200): the bounding box of ``flux_evaluate_indexes``
    (rows x0..x1 = axis 0, columns y0..y1 = axis 1) and the sub-frame scene,
    whose origin is ``map_pix2coord(x0, y0)`` -- the axis-0 index in the pixel-x
    slot, as the reference passes it -- and whose pixel mask is the cut of
    ``flux_evaluate_indexes``."""
    fei = np.asarray(scene["flux_evaluate_indexes"], dtype=bool)
    rows, cols = np.where(fei)
    x0, x1, y0, y1 = rows.min(), rows.max(), cols.min(), cols.max()
    M = np.asarray(scene["transform_pix2angle"], float)
    sub = dict(scene)
    sub["flux_evaluate_indexes"] = None
    sub["nx"] = x1 - x0 + 1
    sub["ny"] = y1 - y0 + 1
    sub["ra_at_xy_0"] = scene["ra_at_xy_0"] + x0 * M[0, 0] + y0 * M[0, 1]
    sub["dec_at_xy_0"] = scene["dec_at_xy_0"] + x0 * M[1, 0] + y0 * M[1, 1]
    sub["pixel_mask"] = fei[x0:x1 + 1, y0:y1 + 1]
    return sub, (x0, x1, y0, y1)


def _mask_rays(scene, flux):
    """Zero the rays of pixels outside the evaluation mask (RegularGrid with
    flux_evaluate_indexes evaluates only those, grid.py:48-64,134-148)."""
    m = scene.get("pixel_mask")
    if m is None:
        return flux
    s = scene["supersampling_factor"]
    mm = np.repeat(np.repeat(np.asarray(m, float), s, axis=0), s, axis=1)
    return flux * mm.reshape(-1)


def ray_fluxes(scene, kwargs_lens, kwargs_source, kwargs_lens_light,
               source_add=True, lens_light_add=True):
    """Per-ray flux (before re-binning) of the source (lensed, x flux_scaling)
    and the lens light, on the supersampled grid in row-major order."""
    s = scene["supersampling_factor"]
    ra, dec = grid.supersampled_coordinates(scene["nx"], scene["ny"], scene["transform_pix2angle"],
                                            scene["ra_at_xy_0"], scene["dec_at_xy_0"], s)
    src = np.zeros_like(ra)
    ll = np.zeros_like(ra)
    src_list = scene.get("source_light_model_list", [])
    if source_add and len(src_list) > 0:
        ax, ay = lens.alpha(scene.get("lens_model_list", []), ra, dec, kwargs_lens or [],
                            scene.get("alpha_scaling", 1.0))
        for i, (name, kw) in enumerate(zip(src_list, kwargs_source)):
            sc = _source_scalings(scene)[i]
            src = src + light.profile(name, ra - sc * ax, dec - sc * ay, kw)
        src = src * scene.get("flux_scaling", 1.0)
    ll_list = scene.get("lens_light_model_list", [])
    if lens_light_add and len(ll_list) > 0:
        ll = light.surface_brightness(ll_list, ra, dec, kwargs_lens_light)
    return _mask_rays(scene, src), _mask_rays(scene, ll)


def re_size_convolve(scene, flux, unconvolved=False):
    """``Numerics.re_size_convolve`` ``numerics.py:158-177`` (regular compute
    mode, no sub-frame)."""
    nx, ny, s = scene["nx"], scene["ny"], scene["supersampling_factor"]
    img = grid.array2image(flux, nx * s, ny * s)
    low = grid.re_size(img, s)
    psf_type = scene.get("psf_type", "NONE")
    ctype = scene.get("convolution_type", "fft")
    pw = grid.pixel_width(scene["transform_pix2angle"])
    if (scene.get("supersampling_convolution", False) and s > 1 and not unconvolved
            and psf_type != "NONE"):
        if psf_type == "PIXEL":
            # SubgridKernelConvolution.re_size_convolve (convolution.py:154-166);
            # `kernel` is the supersampled kernel (cut, numerics.py:196-213)
            ssk = scene.get("supersampling_kernel_size", 5)
            if ssk is None:
                high, lowk = scene["kernel"], None
            else:
                lowk, high = numerics.split_kernel(scene["kernel"], ssk, s)
            conv = grid.re_size(numerics.pixel_convolve(img, high, ctype), s)
            if lowk is not None:
                conv = conv + numerics.pixel_convolve(low, lowk, ctype)
        else:
            # GaussianConvolution with supersampling_convolution (convolution.py:194-250)
            sigma = numerics.fwhm2sigma(scene["fwhm"]) / pw * s
            kernel, radius = numerics.gaussian_kernel(sigma, scene.get("truncation", 5.0))
            conv = grid.re_size(numerics.gaussian_convolve(img, kernel, radius), s)
        return conv * pw ** 2
    if unconvolved or psf_type == "NONE":
        conv = low
    elif psf_type == "PIXEL":
        conv = numerics.pixel_convolve(low, scene["kernel"], scene.get("convolution_type", "fft"))
    elif psf_type == "GAUSSIAN":
        pw = grid.pixel_width(scene["transform_pix2angle"])
        sigma = numerics.fwhm2sigma(scene["fwhm"]) / pw
        kernel, radius = numerics.gaussian_kernel(sigma, scene.get("truncation", 5.0))
        conv = numerics.gaussian_convolve(low, kernel, radius)
    else:
        raise ValueError("psf_type %s not valid!" % psf_type)
    return conv * grid.pixel_width(scene["transform_pix2angle"]) ** 2


def image(scene, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
          unconvolved=False, source_add=True, lens_light_add=True):
    """``ImageModel.image`` ``image_model.py:432-492`` (point sources empty)."""
    if scene.get("flux_evaluate_indexes") is not None:
        # NumericsSubFrame: compute on the sub-frame, zeros elsewhere (:87-100,134-149)
        sub, (x0, x1, y0, y1) = _subframe(scene)
        img = image(sub, kwargs_lens, kwargs_source, kwargs_lens_light, unconvolved,
                    source_add, lens_light_add)
        out = np.zeros((scene["ny"], scene["nx"]))
        out[x0:x1 + 1, y0:y1 + 1] = img
        return out
    nx, ny = scene["nx"], scene["ny"]
    model = np.zeros((ny, nx))
    src, ll = ray_fluxes(scene, kwargs_lens, kwargs_source, kwargs_lens_light,
                         source_add, lens_light_add)
    if source_add and len(scene.get("source_light_model_list", [])) > 0:
        model = model + re_size_convolve(scene, src, unconvolved)
    if lens_light_add and len(scene.get("lens_light_model_list", [])) > 0:
        model = model + re_size_convolve(scene, ll, unconvolved) * scene.get("flux_scaling", 1.0)
    return model


def covariance_matrix(data, background_rms, exposure_map):
    """``jaxtronomy/Data/image_noise.py:115-137``."""
    d_pos = np.where(data >= 0, data, 0)
    return d_pos / exposure_map + background_rms ** 2


def exposure_floor(exposure_time):
    """``image_noise.py:52-54``."""
    return np.where(np.asarray(exposure_time) <= 10 ** (-10), 10 ** (-10), exposure_time)


def log_likelihood(model, data, mask, background_rms, exposure_time=None, noise_map=None,
                   additional_error_map=0.0):
    """``ImageData._log_likelihood`` ``imaging_data.py:159-182`` with
    ``ImageNoise.C_D_model`` ``image_noise.py:100-110``."""
    if noise_map is not None:
        c_d = np.asarray(noise_map, float) ** 2
    else:
        c_d = covariance_matrix(model, background_rms, exposure_floor(exposure_time))
    chi2 = (model - data) ** 2
    chi2 = chi2 / (c_d + np.abs(additional_error_map))
    chi2 = chi2 * mask
    return -np.sum(chi2) / 2
