"""Generate the golden vectors in this folder by running the reference itself.

The reference (JAXtronomy) is pure Python on top of ``jax`` and ``lenstronomy``,
neither of which is installed where this script runs.  ``refshim`` supplies a
NumPy-backed ``jax`` and restates the handful of lenstronomy names on the image
path, so that the reference's own source (``jaxtronomy/...``) computes every
value stored here, in FP64.

Usage (needs the reference source tree; the output files are committed):

    python tests/golden/make_golden.py /path/to/jaxtronomy-source [file ...]

or with the source tree in the environment variable ``JAXTRONOMY_SOURCE``.
Naming files (e.g. ``serving_scenes.npz``) regenerates only those.

Outputs (all .npz, metadata as a JSON string under key ``meta``):
  profiles.npz  per-profile deflections / surface brightness at seeded points
  hyp2f1.npz    hyp2f1_lopez_temme_8 at the reference's own test points
  images.npz    ImageModel.image and likelihood_data_given_model on small scenes
  bulk.npz      LensModelBulk.ray_shooting through many deflectors
  multiplane.npz LensModelBulk (multi-plane): prepared kwargs and ray shooting
  point_sources.npz ImageModel with LENSED_POSITION / UNLENSED point sources
  linear.npz    ImageLinearFit: linear amplitude solve, model image, logL
  serving_scenes.npz ImageModel.image of the four serving lens stacks with two
                sources at 100x100, supersampling 4, a 41x41 Moffat kernel
  grad_fd.npz   central differences of likelihood_data_given_model (the
                reference's own likelihood) on gradient-workload scenes
  hessians.npz  LensModel.hessian of EPL_MULTIPOLE_M1M3M4, NFW_ELLIPSE_CSE and
                CONVERGENCE
"""

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refshim  # noqa: E402


def _points(rng, n, lo=-2.5, hi=2.5):
    x = rng.uniform(lo, hi, n)
    y = rng.uniform(lo, hi, n)
    # include exact-centre and near-centre rays, which exercise the floors
    x[:4] = [0.0, 1e-7, -3e-4, 0.02]
    y[:4] = [0.0, 0.0, 2e-4, -0.01]
    return x, y


def gen_profiles(rng):
    from jaxtronomy.LensModel.lens_model import LensModel
    from jaxtronomy.LightModel.light_model import LightModel

    cases = []
    lens_cases = [
        ("SIE", {"theta_E": 1.1, "e1": 0.12, "e2": -0.07, "center_x": 0.03, "center_y": -0.02}),
        ("SIE", {"theta_E": 0.9, "e1": 0.0, "e2": 0.0, "center_x": 0.0, "center_y": 0.0}),
        ("NIE", {"theta_E": 1.3, "e1": -0.2, "e2": 0.1, "s_scale": 0.05,
                 "center_x": -0.1, "center_y": 0.05}),
        ("SHEAR", {"gamma1": 0.03, "gamma2": -0.04, "ra_0": 0.1, "dec_0": -0.2}),
        ("SHEAR", {"gamma1": -0.05, "gamma2": 0.02}),
        ("NFW", {"Rs": 0.8, "alpha_Rs": 0.6, "center_x": 0.1, "center_y": -0.1}),
        ("TNFW", {"Rs": 0.05, "alpha_Rs": 0.004, "r_trunc": 0.5, "center_x": 0.2,
                  "center_y": 0.3}),
        ("TNFW", {"Rs": 0.9, "alpha_Rs": 0.7, "r_trunc": 3.0, "center_x": 0.0,
                  "center_y": 0.0}),
    ]
    # EPL across every series-length branch (f = |e|): 0, <0.12, <0.4, <0.6,
    # <0.73, <0.86, <0.92, >=0.92
    for e in [0.0, 0.05, 0.25, 0.5, 0.65, 0.8, 0.9, 0.95]:
        lens_cases.append(("EPL", {"theta_E": 1.2, "gamma": 2.13, "e1": e * np.cos(0.7),
                                   "e2": e * np.sin(0.7), "center_x": 0.04,
                                   "center_y": -0.03}))
    lens_cases.append(("EPL", {"theta_E": 0.85, "gamma": 1.82, "e1": -0.08, "e2": 0.03,
                               "center_x": 0.0, "center_y": 0.0}))
    lens_cases += [
        ("NFW_ELLIPSE_CSE", {"Rs": 8.0, "alpha_Rs": 1.3, "e1": 0.1, "e2": -0.2, "center_x": 0.1,
                             "center_y": 0.0}),
        ("NFW_ELLIPSE_CSE", {"Rs": 0.5, "alpha_Rs": 0.2, "e1": -0.05, "e2": 0.02,
                             "center_x": -0.3, "center_y": 0.4}),
        ("EPL_MULTIPOLE_M1M3M4", {"theta_E": 1.2, "gamma": 2.05, "e1": 0.1, "e2": 0.05,
                                  "center_x": 0.02, "center_y": -0.01, "a1_a": 0.01,
                                  "delta_phi_m1": 0.3, "a3_a": -0.012, "delta_phi_m3": 1.1,
                                  "a4_a": 0.008, "delta_phi_m4": 2.0}),
        ("EPL_MULTIPOLE_M1M3M4", {"theta_E": 0.9, "gamma": 1.9, "e1": -0.3, "e2": 0.25,
                                  "center_x": 0.0, "center_y": 0.0, "a1_a": -0.02,
                                  "delta_phi_m1": 2.9, "a3_a": 0.005, "delta_phi_m3": 0.2,
                                  "a4_a": -0.015, "delta_phi_m4": 0.7}),
    ]
    for name, kw in lens_cases:
        x, y = _points(rng, 64)
        lm = LensModel([name])
        ax, ay = lm.alpha(x, y, [kw])
        cases.append({"kind": "lens", "name": name, "kwargs": kw, "x": x, "y": y,
                      "out": np.stack([np.asarray(ax), np.asarray(ay)])})
    light_cases = [
        ("SERSIC", {"amp": 31.0, "R_sersic": 0.1, "n_sersic": 2.0, "center_x": 0.0,
                    "center_y": 0.0}),
        ("SERSIC_ELLIPSE", {"amp": 23.0, "R_sersic": 0.6, "n_sersic": 7.0, "e1": 0.05,
                            "e2": 0.03, "center_x": 0.0, "center_y": 0.0}),
        ("SERSIC_ELLIPSE", {"amp": 55.0, "R_sersic": 0.25, "n_sersic": 1.3, "e1": -0.12,
                            "e2": 0.08, "center_x": 0.07, "center_y": -0.04}),
        ("SERSIC_ELLIPSE", {"amp": 12.0, "R_sersic": 0.00005, "n_sersic": 4.0, "e1": 0.0,
                            "e2": 0.0, "center_x": 0.0, "center_y": 0.0}),
    ]
    for name, kw in light_cases:
        x, y = _points(rng, 64, -3.0, 3.0)
        lm = LightModel([name])
        out = lm.surface_brightness(x, y, [kw])
        cases.append({"kind": "light", "name": name, "kwargs": kw, "x": x, "y": y,
                      "out": np.asarray(out)[None, :]})
    # exact Hessians of the profiles with position derivatives (kind "hessian")
    for name, kw in [lens_cases[0], lens_cases[2], lens_cases[3], lens_cases[5],
                     lens_cases[6], lens_cases[7]] + [c for c in lens_cases if c[0] == "EPL"][:8:3]:
        x, y = _points(rng, 64)
        x[:4] = x[:4] + 0.3  # away from the centre floors
        out = np.stack([np.asarray(v) for v in LensModel([name]).hessian(x, y, [kw])])
        cases.append({"kind": "hessian", "name": name, "kwargs": kw, "x": x, "y": y,
                      "out": out})
    for kw in ({"kappa": -0.03, "ra_0": 0.2, "dec_0": -0.1}, {"kappa": 0.12}):
        x, y = _points(rng, 64)
        ax, ay = LensModel(["CONVERGENCE"]).alpha(x, y, [kw])
        cases.append({"kind": "lens", "name": "CONVERGENCE", "kwargs": kw, "x": x, "y": y,
                      "out": np.stack([np.asarray(ax), np.asarray(ay)])})
    return cases


def gen_hyp2f1():
    from jaxtronomy.Util.hyp2f1_util import hyp2f1_lopez_temme_8
    # the reference's own test points, test/test_Util/test_hyp2f1_util.py:87-112
    a, b, c = 0.3, 0.7, 2.2
    pts = [(complex(0.3, 0.5), 75), (complex(0.5, 2.1), 75), (complex(-0.6, 0.1), 75),
           (complex(0.2, -1.6), 75), (complex(-3.2, 1.1), 75), (complex(0.99, 0.001), 200),
           (complex(-10.99, 0.001), 75)]
    z = np.array([p[0] for p in pts])
    nmax = np.array([p[1] for p in pts])
    out = np.array([complex(np.asarray(hyp2f1_lopez_temme_8(a, b, c, zz, nmax=int(n))))
                    for zz, n in zip(z, nmax)])
    return {"a": a, "b": b, "c": c, "z": z, "nmax": nmax, "out": out}


def _image_model(num_pix, delta_pix, s, psf_kwargs, lens_list, src_list, ll_list,
                 data=None, bkg=0.01, exp_time=1000.0, flux_scaling=1, deflection_scaling=None,
                 convolution_type="fft", numerics=None):
    from jaxtronomy.Data.imaging_data import ImageData
    from jaxtronomy.ImSim.image_model import ImageModel
    from jaxtronomy.LensModel.lens_model import LensModel
    from jaxtronomy.LightModel.light_model import LightModel
    from jaxtronomy_gb300.workloads import grid_kwargs

    g = grid_kwargs(num_pix, delta_pix)
    if data is None:
        data = np.zeros((num_pix, num_pix))
    data_class = ImageData(image_data=data, exposure_time=exp_time, background_rms=bkg,
                           ra_at_xy_0=g["ra_at_xy_0"], dec_at_xy_0=g["dec_at_xy_0"],
                           transform_pix2angle=g["transform_pix2angle"],
                           flux_scaling=flux_scaling)
    psf = refshim.PSF(**psf_kwargs)
    return ImageModel(data_class, psf, LensModel(lens_list),
                      LightModel(src_list, deflection_scaling_list=deflection_scaling),
                      LightModel(ll_list),
                      kwargs_numerics=dict({"supersampling_factor": s,
                                            "convolution_type": convolution_type},
                                           **(numerics or {})))


def gen_images():
    from jaxtronomy_gb300 import workloads as W

    scenes = []
    # 1) the single-image workload, 60x60, s=1, 11x11 Gaussian PIXEL kernel
    model, lens, src, ll, kern = W.single_sie(seed=1000, batch=2)
    for i in range(2):
        kl, ks, kll = W.instance(lens, i), W.instance(src, i), W.instance(ll, i)
        im = _image_model(60, 0.05, 1, {"psf_type": "PIXEL", "kernel_point_source": kern[i]},
                          model["lens_model_list"], model["source_light_model_list"],
                          model["lens_light_model_list"])
        scenes.append({"tag": "single_sie_%d" % i, "num_pix": 60, "delta_pix": 0.05, "s": 1,
                       "psf_type": "PIXEL", "kernel": kern[i], "lens": model["lens_model_list"],
                       "src": model["source_light_model_list"],
                       "ll": model["lens_light_model_list"], "kwargs_lens": kl,
                       "kwargs_source": ks, "kwargs_lens_light": kll,
                       "image": np.asarray(im.image(kl, ks, kll))})
    # 2) EPL+SHEAR batch workload at a reduced grid (40x40, s=3, 11x11 Moffat)
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=3, num_pix=40, kernel_size=11)
    for i in range(3):
        kl, ks, kll = W.instance(lens, i), W.instance(src, i), W.instance(ll, i)
        im = _image_model(40, 0.04, 3, {"psf_type": "PIXEL", "kernel_point_source": kern[i]},
                          model["lens_model_list"], model["source_light_model_list"],
                          model["lens_light_model_list"])
        scenes.append({"tag": "batch_epl_%d" % i, "num_pix": 40, "delta_pix": 0.04, "s": 3,
                       "psf_type": "PIXEL", "kernel": kern[i], "lens": model["lens_model_list"],
                       "src": model["source_light_model_list"],
                       "ll": model["lens_light_model_list"], "kwargs_lens": kl,
                       "kwargs_source": ks, "kwargs_lens_light": kll,
                       "image": np.asarray(im.image(kl, ks, kll))})
    # 3) GAUSSIAN psf type (edge-padded Gaussian convolution), s=2, NFW+SHEAR lens,
    #    two sources with deflection scaling, flux scaling 1.7
    kl = [{"Rs": 1.2, "alpha_Rs": 0.9, "center_x": 0.05, "center_y": -0.02},
          {"gamma1": 0.02, "gamma2": -0.03}]
    ks = [{"amp": 40.0, "R_sersic": 0.2, "n_sersic": 1.5, "e1": 0.1, "e2": -0.05,
           "center_x": 0.1, "center_y": 0.05},
          {"amp": 15.0, "R_sersic": 0.3, "n_sersic": 2.5, "center_x": -0.2, "center_y": 0.1}]
    kll = [{"amp": 30.0, "R_sersic": 0.8, "n_sersic": 3.0, "e1": 0.05, "e2": 0.02,
            "center_x": 0.05, "center_y": -0.02}]
    im = _image_model(32, 0.08, 2, {"psf_type": "GAUSSIAN", "fwhm": 0.2, "truncation": 4},
                      ["NFW", "SHEAR"], ["SERSIC_ELLIPSE", "SERSIC"], ["SERSIC_ELLIPSE"],
                      flux_scaling=1.7, deflection_scaling=[1.0, 0.6])
    scenes.append({"tag": "gaussian_psf", "num_pix": 32, "delta_pix": 0.08, "s": 2,
                   "psf_type": "GAUSSIAN", "fwhm": 0.2, "truncation": 4.0,
                   "lens": ["NFW", "SHEAR"], "src": ["SERSIC_ELLIPSE", "SERSIC"],
                   "ll": ["SERSIC_ELLIPSE"], "flux_scaling": 1.7,
                   "deflection_scaling": [1.0, 0.6], "kwargs_lens": kl, "kwargs_source": ks,
                   "kwargs_lens_light": kll, "image": np.asarray(im.image(kl, ks, kll))})
    # 4) no PSF, TNFW+EPL+SHEAR, s=4, plus unconvolved / partial-component calls
    kl = [{"theta_E": 1.0, "gamma": 1.95, "e1": 0.15, "e2": -0.1, "center_x": 0.0,
           "center_y": 0.0},
          {"Rs": 0.1, "alpha_Rs": 0.01, "r_trunc": 1.0, "center_x": 0.6, "center_y": 0.5},
          {"gamma1": 0.01, "gamma2": 0.04}]
    ks = [{"amp": 70.0, "R_sersic": 0.15, "n_sersic": 3.5, "e1": -0.1, "e2": 0.2,
           "center_x": 0.02, "center_y": 0.03}]
    kll = []
    im = _image_model(24, 0.1, 4, {"psf_type": "NONE"}, ["EPL", "TNFW", "SHEAR"],
                      ["SERSIC_ELLIPSE"], [])
    scenes.append({"tag": "no_psf", "num_pix": 24, "delta_pix": 0.1, "s": 4,
                   "psf_type": "NONE", "lens": ["EPL", "TNFW", "SHEAR"],
                   "src": ["SERSIC_ELLIPSE"], "ll": [], "kwargs_lens": kl,
                   "kwargs_source": ks, "kwargs_lens_light": kll,
                   "image": np.asarray(im.image(kl, ks, kll))})
    # 5) serving-stream lens stacks: EPL_MULTIPOLE_M1M3M4 + SHEAR with two sources,
    #    NFW_ELLIPSE_CSE + SHEAR, both 36x36 at 0.08"/pix, s=2, 11x11 Gaussian kernel
    kern_g = W.gaussian_pixel_kernel(0.2, 0.08, 11)
    ks2 = [{"amp": 60.0, "R_sersic": 0.25, "n_sersic": 2.5, "e1": 0.05, "e2": 0.1,
            "center_x": 0.05, "center_y": -0.05},
           {"amp": 20.0, "R_sersic": 0.4, "n_sersic": 1.2, "e1": -0.1, "e2": 0.0,
            "center_x": -0.15, "center_y": 0.1}]
    kll2 = [{"amp": 35.0, "R_sersic": 1.0, "n_sersic": 3.5, "e1": 0.08, "e2": -0.04,
             "center_x": 0.0, "center_y": 0.0}]
    for tag, lens_list, kl in [
        ("multipole", ["EPL_MULTIPOLE_M1M3M4", "SHEAR"],
         [{"theta_E": 1.1, "gamma": 2.1, "e1": 0.12, "e2": -0.06, "center_x": 0.0,
           "center_y": 0.0, "a1_a": 0.008, "delta_phi_m1": 0.4, "a3_a": -0.01,
           "delta_phi_m3": 2.2, "a4_a": 0.012, "delta_phi_m4": 1.3},
          {"gamma1": 0.03, "gamma2": 0.01}]),
        ("nfw_cse", ["NFW_ELLIPSE_CSE", "SHEAR"],
         [{"Rs": 12.0, "alpha_Rs": 1.6, "e1": 0.1, "e2": 0.05, "center_x": 0.0,
           "center_y": 0.0}, {"gamma1": -0.02, "gamma2": 0.04}]),
    ]:
        im = _image_model(36, 0.08, 2, {"psf_type": "PIXEL", "kernel_point_source": kern_g},
                          lens_list, ["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"], ["SERSIC_ELLIPSE"])
        scenes.append({"tag": tag, "num_pix": 36, "delta_pix": 0.08, "s": 2,
                       "psf_type": "PIXEL", "kernel": kern_g, "lens": lens_list,
                       "src": ["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"], "ll": ["SERSIC_ELLIPSE"],
                       "kwargs_lens": kl, "kwargs_source": ks2, "kwargs_lens_light": kll2,
                       "image": np.asarray(im.image(kl, ks2, kll2))})
    # 7) convolution on the supersampled grid (SubgridKernelConvolution with the
    #    supersampled kernel given to the PSF; GaussianConvolution with
    #    supersampling_convolution), EPL+SHEAR, s = 3 and 2
    model, lens, src, ll, _ = W.batch_epl(seed=1005, batch=1, num_pix=30, kernel_size=11)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    for tag, side, cks, ssk in [("ssc_pixel_split", 27, None, 3),
                                ("ssc_pixel", 15, None, None),
                                ("ssc_pixel_cut", 27, 5, 1)]:
        k_super = W.moffat_pixel_kernel(0.12, 3.0, 0.05 / 3, side)
        num = {"supersampling_convolution": True, "supersampling_kernel_size": ssk}
        if cks is not None:
            num["convolution_kernel_size"] = cks
        im = _image_model(30, 0.05, 3, {"psf_type": "PIXEL", "kernel_point_source": k_super,
                                        "point_source_supersampling_factor": 3},
                          model["lens_model_list"], model["source_light_model_list"],
                          model["lens_light_model_list"], numerics=num)
        scenes.append({"tag": tag, "num_pix": 30, "delta_pix": 0.05, "s": 3,
                       "psf_type": "PIXEL", "kernel": k_super, "ssc": True, "cks": cks,
                       "ssk": ssk, "lens": model["lens_model_list"],
                       "src": model["source_light_model_list"],
                       "ll": model["lens_light_model_list"], "kwargs_lens": kl,
                       "kwargs_source": ks, "kwargs_lens_light": kll,
                       "image": np.asarray(im.image(kl, ks, kll))})
    im = _image_model(32, 0.08, 2, {"psf_type": "GAUSSIAN", "fwhm": 0.2, "truncation": 4},
                      model["lens_model_list"], model["source_light_model_list"],
                      model["lens_light_model_list"], numerics={"supersampling_convolution": True})
    scenes.append({"tag": "ssc_gaussian", "num_pix": 32, "delta_pix": 0.08, "s": 2,
                   "psf_type": "GAUSSIAN", "fwhm": 0.2, "truncation": 4.0, "ssc": True,
                   "lens": model["lens_model_list"], "src": model["source_light_model_list"],
                   "ll": model["lens_light_model_list"], "kwargs_lens": kl, "kwargs_source": ks,
                   "kwargs_lens_light": kll, "image": np.asarray(im.image(kl, ks, kll))})
    # 8) flux_evaluate_indexes (NumericsSubFrame): a disc mask whose bounding box
    #    (rows 6..22, columns 11..27) is off the diagonal, s = 2, PIXEL 7x7
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=1, num_pix=30, kernel_size=7)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    yy, xx = np.mgrid[0:30, 0:30]
    mask = (yy - 14) ** 2 + (xx - 19) ** 2 <= 64
    im = _image_model(30, 0.04, 2, {"psf_type": "PIXEL", "kernel_point_source": kern[0]},
                      model["lens_model_list"], model["source_light_model_list"],
                      model["lens_light_model_list"], numerics={"flux_evaluate_indexes": mask})
    scenes.append({"tag": "subframe", "num_pix": 30, "delta_pix": 0.04, "s": 2,
                   "psf_type": "PIXEL", "kernel": kern[0], "fei": mask.astype(int).tolist(),
                   "lens": model["lens_model_list"], "src": model["source_light_model_list"],
                   "ll": model["lens_light_model_list"], "kwargs_lens": kl, "kwargs_source": ks,
                   "kwargs_lens_light": kll, "image": np.asarray(im.image(kl, ks, kll))})
    # 6) likelihood on the first single-image scene with noisy data
    rng = np.random.default_rng(77)
    base = scenes[0]
    clean = base["image"]
    data = clean + rng.normal(0, 0.01, clean.shape) \
        + rng.poisson(np.clip(clean, 0, None) * 1000) / 1000 - np.clip(clean, 0, None)
    im = _image_model(60, 0.05, 1, {"psf_type": "PIXEL", "kernel_point_source": base["kernel"]},
                      base["lens"], base["src"], base["ll"], data=data, bkg=0.01,
                      exp_time=1000.0)
    logl = float(np.asarray(im.likelihood_data_given_model(
        base["kwargs_lens"], base["kwargs_source"], base["kwargs_lens_light"])))
    return scenes, {"data": data, "logL": logl, "bkg": 0.01, "exp_time": 1000.0,
                    "scene": base["tag"]}


def gen_bulk(rng):
    """LensModelBulk (single plane) on a substructure scene and a mixed list."""
    from jaxtronomy.LensModel.lens_model_bulk import LensModelBulk

    cases = []
    # main EPL + SHEAR plus TNFW subhalos drawn like the 1000^2-ray workload,
    # padded with NULL deflectors through num_deflectors
    n_sub = 60
    lens_list = ["EPL", "SHEAR"] + ["TNFW"] * n_sub
    kw = [{"theta_E": 1.2, "gamma": 2.05, "e1": 0.08, "e2": -0.05, "center_x": 0.01,
           "center_y": -0.02},
          {"gamma1": 0.03, "gamma2": -0.02}]
    cx = rng.uniform(-2.5, 2.5, n_sub)
    cy = rng.uniform(-2.5, 2.5, n_sub)
    rs = rng.uniform(0.01, 0.1, n_sub)
    ars = 10 ** rng.uniform(-4, -2, n_sub)
    for i in range(n_sub):
        kw.append({"Rs": float(rs[i]), "alpha_Rs": float(ars[i]), "r_trunc": float(10 * rs[i]),
                   "center_x": float(cx[i]), "center_y": float(cy[i])})
    x, y = _points(rng, 500)
    # rays on and next to subhalo centres (the R floors)
    x[4:10] = cx[:6] + np.array([0.0, 1e-6, 0.0, 3e-3, -0.02, 0.05])
    y[4:10] = cy[:6] + np.array([0.0, 0.0, -2e-5, 0.0, 0.01, -0.03])
    unique = ["EPL", "SHEAR", "TNFW"]
    bulk = LensModelBulk(unique, multi_plane=False)
    rk = bulk.prepare_ray_shooting_kwargs(lens_list, kw, num_deflectors=len(lens_list) + 5)
    bx, by = bulk.ray_shooting(x, y, rk)
    cases.append({"unique": unique, "lens_list": lens_list, "kwargs": kw,
                  "num_deflectors": len(lens_list) + 5, "x": x, "y": y,
                  "bx": np.asarray(bx), "by": np.asarray(by)})
    # every profile type through the bulk switch, in mixed order
    unique = ["TNFW", "NFW", "SIE", "EPL_MULTIPOLE_M1M3M4", "NFW_ELLIPSE_CSE", "SHEAR", "NIE"]
    lens_list = ["SIE", "TNFW", "NFW", "TNFW", "EPL_MULTIPOLE_M1M3M4", "NFW_ELLIPSE_CSE",
                 "SHEAR", "NIE", "NFW"]
    kw = [{"theta_E": 0.9, "e1": 0.1, "e2": 0.05, "center_x": 0.1, "center_y": 0.0},
          {"Rs": 0.05, "alpha_Rs": 0.003, "r_trunc": 0.4, "center_x": -0.5, "center_y": 0.7},
          {"Rs": 0.3, "alpha_Rs": 0.05, "center_x": 1.1, "center_y": -0.4},
          {"Rs": 0.02, "alpha_Rs": 0.0008, "r_trunc": 0.2, "center_x": 0.9, "center_y": 0.9},
          {"theta_E": 0.4, "gamma": 1.9, "e1": -0.1, "e2": 0.12, "center_x": -1.0,
           "center_y": -1.0, "a1_a": 0.01, "delta_phi_m1": 0.3, "a3_a": -0.005,
           "delta_phi_m3": 1.1, "a4_a": 0.008, "delta_phi_m4": 2.4},
          {"Rs": 6.0, "alpha_Rs": 0.7, "e1": 0.05, "e2": -0.08, "center_x": 0.0,
           "center_y": 0.2},
          {"gamma1": -0.02, "gamma2": 0.04, "ra_0": 0.1, "dec_0": 0.2},
          {"theta_E": 0.2, "e1": 0.0, "e2": 0.1, "s_scale": 0.01, "center_x": 1.5,
           "center_y": 1.5},
          {"Rs": 0.1, "alpha_Rs": 0.01}]
    x, y = _points(rng, 300)
    bulk = LensModelBulk(unique, multi_plane=False)
    rk = bulk.prepare_ray_shooting_kwargs(lens_list, kw)
    bx, by = bulk.ray_shooting(x, y, rk)
    cases.append({"unique": unique, "lens_list": lens_list, "kwargs": kw,
                  "num_deflectors": None, "x": x, "y": y,
                  "bx": np.asarray(bx), "by": np.asarray(by)})
    return cases


def gen_point_sources(rng):
    """ImageModel with point sources (PointSource LENSED_POSITION + UNLENSED,
    PointSourceRendering): images, the point-source term alone and a likelihood."""
    from jaxtronomy.Data.imaging_data import ImageData
    from jaxtronomy.ImSim.image_model import ImageModel
    from jaxtronomy.LensModel.lens_model import LensModel
    from jaxtronomy.LightModel.light_model import LightModel
    from jaxtronomy.PointSource.point_source import PointSource
    from jaxtronomy_gb300 import workloads as W

    lens = [{"theta_E": 1.0, "gamma": 2.05, "e1": 0.06, "e2": -0.03, "center_x": 0.01,
             "center_y": 0.0}, {"gamma1": 0.02, "gamma2": -0.01}]
    src = [{"amp": 4.0, "R_sersic": 0.15, "n_sersic": 1.5, "e1": 0.05, "e2": 0.0,
            "center_x": 0.03, "center_y": -0.02}]
    ll = [{"amp": 6.0, "R_sersic": 0.7, "n_sersic": 3.0, "center_x": 0.0, "center_y": 0.0}]
    out = []

    def scene(tag, n, dpix, s, psf_kwargs, ps_kwargs, numerics=None, special=None,
              unconvolved=False, flux_scaling=1.0, fixed=None):
        g = W.grid_kwargs(n, dpix)
        rng_d = np.random.default_rng(len(out) + 7)
        data = rng_d.normal(0, 0.01, (n, n))
        data_class = ImageData(image_data=data, exposure_time=800.0, background_rms=0.01,
                               ra_at_xy_0=g["ra_at_xy_0"], dec_at_xy_0=g["dec_at_xy_0"],
                               transform_pix2angle=g["transform_pix2angle"],
                               flux_scaling=flux_scaling)
        num = dict({"supersampling_factor": s}, **(numerics or {}))
        im = ImageModel(data_class, refshim.PSF(**psf_kwargs), LensModel(["EPL", "SHEAR"]),
                        LightModel(["SERSIC_ELLIPSE"]), LightModel(["SERSIC"]),
                        point_source_class=PointSource(["LENSED_POSITION", "UNLENSED"],
                                                       fixed_magnification_list=fixed),
                        kwargs_numerics=num)
        image = np.asarray(im.image(lens, src, ll, ps_kwargs, kwargs_special=special,
                                    unconvolved=unconvolved))
        ps1 = np.asarray(im.point_source(ps_kwargs, lens, kwargs_special=special, k=1))
        logl = float(im.likelihood_data_given_model(lens, src, ll, ps_kwargs,
                                                    kwargs_special=special))
        rec = {"tag": tag, "n": n, "dpix": dpix, "s": s, "numerics": numerics or {},
               "psf": {k: v for k, v in psf_kwargs.items() if k != "kernel_point_source"},
               "ps": ps_kwargs, "special": special, "unconvolved": unconvolved,
               "flux_scaling": flux_scaling, "logL": logl, "image": image, "ps1": ps1,
               "data": data, "lens": lens, "src": src, "ll": ll, "fixed": fixed}
        if "kernel_point_source" in psf_kwargs:
            rec["kernel"] = np.asarray(psf_kwargs["kernel_point_source"], float)
        out.append(rec)

    k11 = W.gaussian_pixel_kernel(0.12, 0.08, 11)
    # four lensed images (one near the field edge, one on a pixel centre), one
    # unlensed image and one outside the field
    ps = [{"ra_image": [1.02, -0.55, 0.31, -1.52], "dec_image": [0.11, 0.87, -0.98, -1.49],
           "point_amp": [3.0, 2.2, 1.7, 0.9]},
          {"ra_image": [0.4, 2.1], "dec_image": [1.2, 0.0], "point_amp": [1.3, 5.0]}]
    scene("pixel_psf_s2", 40, 0.08, 2, {"psf_type": "PIXEL", "kernel_point_source": k11}, ps)
    scene("pixel_psf_s2_shifted", 40, 0.08, 2, {"psf_type": "PIXEL", "kernel_point_source": k11},
          ps, special={"delta_x_image": [0.013, -0.02], "delta_y_image": [0.007, 0.011]},
          flux_scaling=1.3)
    scene("pixel_psf_unconvolved", 40, 0.08, 1, {"psf_type": "PIXEL", "kernel_point_source": k11},
          ps, unconvolved=True)
    scene("none_psf", 36, 0.1, 1, {"psf_type": "NONE"}, ps)
    # supersampled rendering: the supersampled kernel given, convolution on the
    # supersampled grid, point_source_supersampling_factor 3
    k33 = W.gaussian_pixel_kernel(0.12, 0.08 / 3, 33)
    scene("supersampled_rendering_s3", 30, 0.08, 3,
          {"psf_type": "PIXEL", "kernel_point_source": k33,
           "point_source_supersampling_factor": 3}, ps,
          numerics={"supersampling_convolution": True, "supersampling_kernel_size": None,
                    "point_source_supersampling_factor": 3})
    # fixed magnification: amplitudes source_amp * |mag| from the EPL + SHEAR Hessian
    ps_fixed = [{"ra_image": [1.02, -0.55, 0.31], "dec_image": [0.11, 0.87, -0.98],
                 "source_amp": 1.7}, ps[1]]
    scene("fixed_magnification", 40, 0.08, 2, {"psf_type": "PIXEL", "kernel_point_source": k11},
          ps_fixed, fixed=[True, False])
    return out


def gen_multi_plane(rng):
    """LensModelBulk (multi-plane, MultiPlaneBulk) through redshift-spread deflectors:
    the prepared kwargs (sorting, fillers, distance lists) and beta.  Distances come
    from refshim's flat Lambda-CDM Background (H0 = 70, Om0 = 0.3, no radiation)."""
    from jaxtronomy.LensModel.lens_model_bulk import LensModelBulk

    cosmo = refshim.FlatLCDM(70.0, 0.3)
    cases = []

    def run(tag, unique, lens_list, kw, z, z_source, num_deflectors, x, y):
        bulk = LensModelBulk(unique, multi_plane=True, cosmo=cosmo)
        rk = bulk.prepare_ray_shooting_kwargs(lens_list, kw, z_source=z_source,
                                              lens_redshift_list=z,
                                              num_deflectors=num_deflectors)
        # the reference updates its scan carry with augmented assignments, which act
        # in place on the shim's NumPy arrays (JAX arrays are immutable): pass copies
        bx, by = bulk.ray_shooting(np.array(x), np.array(y), rk)
        prep = {"index_list": np.asarray(rk["index_list"]),
                "T_ij_list": np.asarray(rk["T_ij_list"], dtype=float),
                "T_z_list": np.asarray(rk["T_z_list"], dtype=float),
                "reduced2physical_factor": np.asarray(rk["reduced2physical_factor"],
                                                      dtype=float)}
        for k, v in rk["all_kwargs"].items():
            prep["kw_" + k] = np.asarray(v, dtype=float)
        cases.append({"tag": tag, "unique": unique, "lens_list": lens_list, "kwargs": kw,
                      "z": [float(v) for v in z], "z_source": z_source,
                      "num_deflectors": num_deflectors, "x": x, "y": y,
                      "bx": np.asarray(bx), "by": np.asarray(by), "prep": prep})

    # substructure-like: TNFW halos on 8 planes, a negative CONVERGENCE sheet per
    # plane, NULL fillers; rays on and next to halo centres
    planes = np.round(np.linspace(0.1, 2.3, 8), 2)
    lens_list, kw, z = [], [], []
    for zp in planes:
        for _ in range(6):
            rs = rng.uniform(0.02, 0.15)
            lens_list.append("TNFW")
            kw.append({"Rs": float(rs), "alpha_Rs": float(10 ** rng.uniform(-3.5, -2)),
                       "r_trunc": float(rs * rng.uniform(5, 20)),
                       "center_x": float(rng.uniform(-2.5, 2.5)),
                       "center_y": float(rng.uniform(-2.5, 2.5))})
            z.append(float(zp))
        lens_list.append("CONVERGENCE")
        kw.append({"kappa": float(-rng.uniform(0.001, 0.01))})
        z.append(float(zp))
    perm = rng.permutation(len(lens_list))
    lens_list = [lens_list[i] for i in perm]
    kw = [kw[i] for i in perm]
    z = [z[i] for i in perm]
    x, y = _points(rng, 400, -3.0, 3.0)
    cent = [(k["center_x"], k["center_y"]) for k in kw if "center_x" in k][:4]
    x[4:8] = [c[0] + d for c, d in zip(cent, (0.0, 1e-4, -3e-3, 0.02))]
    y[4:8] = [c[1] + d for c, d in zip(cent, (0.0, 0.0, 2e-3, -0.01))]
    run("halos", ["TNFW", "CONVERGENCE"], lens_list, kw, z, 2.5, len(lens_list) + 9, x, y)

    # main deflector (EPL + SHEAR on one plane) with halos before, on and behind it
    unique = ["EPL", "SHEAR", "TNFW", "NFW", "CONVERGENCE", "SIE"]
    lens_list = ["TNFW", "EPL", "NFW", "SHEAR", "TNFW", "CONVERGENCE", "SIE", "TNFW"]
    kw = [{"Rs": 0.05, "alpha_Rs": 0.004, "r_trunc": 0.6, "center_x": 0.9, "center_y": -0.4},
          {"theta_E": 1.1, "gamma": 2.08, "e1": 0.07, "e2": -0.04, "center_x": 0.01,
           "center_y": -0.02},
          {"Rs": 0.4, "alpha_Rs": 0.05, "center_x": -0.8, "center_y": 1.2},
          {"gamma1": 0.03, "gamma2": -0.015},
          {"Rs": 0.08, "alpha_Rs": 0.006, "r_trunc": 0.9, "center_x": -1.0, "center_y": -0.7},
          {"kappa": 0.02, "ra_0": 0.1, "dec_0": -0.1},
          {"theta_E": 0.15, "e1": 0.1, "e2": 0.0, "center_x": 1.3, "center_y": 0.6},
          {"Rs": 0.03, "alpha_Rs": 0.002, "r_trunc": 0.3, "center_x": 0.2, "center_y": 1.0}]
    z = [0.3, 0.5, 0.2, 0.5, 0.5, 0.9, 1.4, 0.9]
    x, y = _points(rng, 400)
    run("main_lens", unique, lens_list, kw, z, 2.0, None, x, y)

    # one deflector, the source step only after it
    x, y = _points(rng, 50)
    run("single", ["SIE"], ["SIE"], [{"theta_E": 0.8, "e1": 0.05, "e2": 0.1}], [0.4], 1.2, 1,
        x, y)
    return cases


def gen_linear():
    """ImageLinearFit (image_linear_solve.py) on small scenes: amplitudes, model
    image, inverse normal matrix (source_marg) and logL."""
    import copy

    from jaxtronomy.ImSim.image_linear_solve import ImageLinearFit
    from jaxtronomy.Data.imaging_data import ImageData
    from jaxtronomy.LensModel.lens_model import LensModel
    from jaxtronomy.LightModel.light_model import LightModel
    from jaxtronomy_gb300 import workloads as W

    rng = np.random.default_rng(20240603)
    out = []
    sie = [{"theta_E": 1.0, "e1": 0.1, "e2": -0.05, "center_x": 0.02, "center_y": 0.0},
           {"gamma1": 0.02, "gamma2": -0.01}]
    epl = [{"theta_E": 1.1, "gamma": 2.05, "e1": -0.08, "e2": 0.06, "center_x": 0.0,
            "center_y": 0.03}, {"gamma1": -0.015, "gamma2": 0.025}]
    src = {"amp": 3.0, "R_sersic": 0.2, "n_sersic": 2.0, "e1": 0.05, "e2": 0.1,
           "center_x": 0.05, "center_y": -0.02}
    src2 = {"amp": 1.0, "R_sersic": 0.12, "n_sersic": 1.2, "e1": -0.1, "e2": 0.0,
            "center_x": -0.1, "center_y": 0.08}
    ll_s = {"amp": 5.0, "R_sersic": 0.8, "n_sersic": 3.0, "center_x": 0.0, "center_y": 0.0}
    ll_e = {"amp": 4.0, "R_sersic": 0.9, "n_sersic": 3.5, "e1": 0.05, "e2": 0.02,
            "center_x": 0.01, "center_y": 0.0}
    cases = [
        dict(tag="sie_gauss_s2", n=30, dpix=0.08, s=2, lens=["SIE", "SHEAR"], kl=sie,
             src=["SERSIC_ELLIPSE"], ks=[src], ll=["SERSIC"], kll=[ll_s],
             psf={"psf_type": "GAUSSIAN", "fwhm": 0.15, "truncation": 3}, mask=False,
             marg=False, pos=False, sign=1.0),
        dict(tag="epl_pixel_two_sources_mask_marg", n=36, dpix=0.06, s=1, lens=["EPL", "SHEAR"],
             kl=epl, src=["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"], ks=[src, src2],
             ll=["SERSIC_ELLIPSE"], kll=[ll_e], dsl=[1.0, 0.7],
             psf={"psf_type": "PIXEL", "kernel_point_source": W.gaussian_pixel_kernel(0.12, 0.06, 7)},
             mask=True, marg=True, pos=False, sign=1.0),
        dict(tag="sie_negative_source_positive_check", n=30, dpix=0.08, s=2, lens=["SIE", "SHEAR"],
             kl=sie, src=["SERSIC_ELLIPSE"], ks=[src], ll=["SERSIC"], kll=[ll_s],
             psf={"psf_type": "GAUSSIAN", "fwhm": 0.15, "truncation": 3}, mask=False,
             marg=False, pos=True, sign=-1.0),
        dict(tag="degenerate_two_identical_sources", n=24, dpix=0.1, s=1, lens=["SIE", "SHEAR"],
             kl=sie, src=["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"], ks=[src, dict(src)],
             ll=["SERSIC"], kll=[ll_s], psf={"psf_type": "NONE"}, mask=False, marg=True,
             pos=False, sign=1.0),
        dict(tag="sie_point_sources_marg", n=40, dpix=0.08, s=2, lens=["SIE", "SHEAR"], kl=sie,
             src=["SERSIC_ELLIPSE"], ks=[src], ll=["SERSIC"], kll=[ll_s],
             psf={"psf_type": "PIXEL", "kernel_point_source": W.gaussian_pixel_kernel(0.12, 0.08, 11)},
             mask=False, marg=True, pos=True, sign=1.0,
             ps_types=["LENSED_POSITION", "UNLENSED"],
             ps=[{"ra_image": [1.05, -0.62, 0.35, -0.2], "dec_image": [0.2, 0.8, -0.95, -0.1],
                  "point_amp": [3.0, 2.5, 1.5, 0.8]},
                 {"ra_image": [0.9], "dec_image": [-1.2], "point_amp": [2.0]}]),
        dict(tag="epl_fixed_magnification", n=40, dpix=0.08, s=2, lens=["EPL", "SHEAR"], kl=epl,
             src=["SERSIC_ELLIPSE"], ks=[src], ll=["SERSIC_ELLIPSE"], kll=[ll_e],
             psf={"psf_type": "PIXEL", "kernel_point_source": W.gaussian_pixel_kernel(0.12, 0.08, 11)},
             mask=False, marg=True, pos=False, sign=1.0, ps_types=["LENSED_POSITION"],
             ps_fixed=[True],
             ps=[{"ra_image": [1.05, -0.62, 0.35], "dec_image": [0.2, 0.8, -0.95],
                  "source_amp": 2.5}]),
    ]
    for c in cases:
        g = W.grid_kwargs(c["n"], c["dpix"])
        # data: the model with the given amplitudes (the source scaled by `sign`) + noise
        sim = _image_model(c["n"], c["dpix"], c["s"], c["psf"], c["lens"], c["src"], c["ll"],
                           deflection_scaling=c.get("dsl"))
        ks_sim = copy.deepcopy(c["ks"])
        ks_sim[0]["amp"] = ks_sim[0]["amp"] * c["sign"]
        img = np.asarray(sim.image(c["kl"], ks_sim, c["kll"]))
        if c.get("ps"):
            ra = np.concatenate([np.asarray(p["ra_image"], float) for p in c["ps"]])
            dec = np.concatenate([np.asarray(p["dec_image"], float) for p in c["ps"]])
            if c.get("ps_fixed"):
                amp = c["ps"][0]["source_amp"] * np.abs(np.asarray(
                    LensModel(c["lens"]).magnification(ra, dec, c["kl"])))
            else:
                amp = np.concatenate([np.asarray(p["point_amp"], float) for p in c["ps"]])
            img = img + np.asarray(sim.ImageNumerics.point_source_rendering(ra, dec, amp))
        data = img + rng.normal(0, 0.02, img.shape)
        mask = np.ones((c["n"], c["n"]))
        if c["mask"]:
            yy, xx = np.mgrid[:c["n"], :c["n"]]
            mask = (((xx - c["n"] / 2) ** 2 + (yy - c["n"] / 2) ** 2) < (0.42 * c["n"]) ** 2
                    ).astype(float)
        data_class = ImageData(image_data=data, exposure_time=500.0, background_rms=0.02, **g)
        pcls = None
        if c.get("ps"):
            from jaxtronomy.PointSource.point_source import PointSource
            pcls = PointSource(c["ps_types"], fixed_magnification_list=c.get("ps_fixed"))
        im = ImageLinearFit(data_class, refshim.PSF(**c["psf"]), LensModel(c["lens"]),
                            LightModel(c["src"], deflection_scaling_list=c.get("dsl")),
                            LightModel(c["ll"]), point_source_class=pcls,
                            kwargs_numerics={"supersampling_factor": c["s"]},
                            likelihood_mask=mask)
        kl, ks, kll = copy.deepcopy(c["kl"]), copy.deepcopy(c["ks"]), copy.deepcopy(c["kll"])
        kps = copy.deepcopy(c.get("ps", []))
        model, _, cov, param = im.image_linear_solve(kl, ks, kll, kwargs_ps=kps,
                                                     inv_bool=c["marg"])
        kl, ks, kll = copy.deepcopy(c["kl"]), copy.deepcopy(c["ks"]), copy.deepcopy(c["kll"])
        kps = copy.deepcopy(c.get("ps", []))
        logl, _ = im.likelihood_data_given_model(kl, ks, kll, kwargs_ps=kps,
                                                 source_marg=c["marg"],
                                                 check_positive_flux=c["pos"])
        rec = {k: c[k] for k in ("tag", "n", "dpix", "s", "lens", "kl", "src", "ks", "ll", "kll",
                                 "marg", "pos")}
        rec["dsl"] = c.get("dsl")
        rec["ps_types"], rec["ps"] = c.get("ps_types", []), c.get("ps", [])
        rec["ps_fixed"] = c.get("ps_fixed")
        rec["psf"] = {k: v for k, v in c["psf"].items() if k != "kernel_point_source"}
        rec["logL"] = float(logl)
        rec["bkg"], rec["exp_time"] = 0.02, 500.0
        rec["data"], rec["mask"], rec["model"] = data, mask, np.asarray(model)
        rec["param"] = np.asarray(param, float)
        rec["cov"] = None if cov is None else np.asarray(cov, float)
        if c["psf"]["psf_type"] == "PIXEL":
            rec["kernel"] = np.asarray(c["psf"]["kernel_point_source"])
        out.append(rec)
    return out


def gen_serving_scenes():
    """ImageModel.image of the four serving lens stacks, each with two
    SERSIC_ELLIPSE sources and a SERSIC_ELLIPSE lens light, drawn by the serving
    stream's generator and rendered at its largest supersampling factor and PSF
    (100x100 at 0.05"/pix, s = 4, a 41x41 Moffat kernel)."""
    from jaxtronomy_gb300 import workloads as W

    reqs, psfs = W.serving_stream(seed=1002, n=400)
    scenes = []
    for stack in W.SERVING_STACKS:
        r = next(q for q in reqs if q["key"][3] == stack and q["key"][4] == 2)
        kern = psfs[41][r["psf"]]
        lens = stack.split("+")
        src = ["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"]
        ll = ["SERSIC_ELLIPSE"]
        im = _image_model(100, 0.05, 4, {"psf_type": "PIXEL", "kernel_point_source": kern},
                          lens, src, ll)
        kl, ks, kll = r["kwargs_lens"], r["kwargs_source"], r["kwargs_lens_light"]
        scenes.append({"tag": stack, "num_pix": 100, "delta_pix": 0.05, "s": 4,
                       "psf_type": "PIXEL", "kernel": kern, "lens": lens, "src": src, "ll": ll,
                       "kwargs_lens": kl, "kwargs_source": ks, "kwargs_lens_light": kll,
                       "image": np.asarray(im.image(kl, ks, kll))})
    return scenes


def gen_hessians():
    """LensModel.hessian of the profiles whose exact Hessian comes from the
    adjoint's dual numbers beyond the round-one set: EPL_MULTIPOLE_M1M3M4 (the
    reference's analytic EPL + multipole Hessians), NFW_ELLIPSE_CSE (its
    analytic CSE Hessian) and CONVERGENCE, at seeded points away from the
    centre."""
    from jaxtronomy.LensModel.lens_model import LensModel

    rng = np.random.default_rng(20240607)
    cases = []
    for name, kw in [
        ("EPL_MULTIPOLE_M1M3M4", {"theta_E": 1.2, "gamma": 2.05, "e1": 0.1, "e2": 0.05,
                                  "center_x": 0.02, "center_y": -0.01, "a1_a": 0.01,
                                  "delta_phi_m1": 0.3, "a3_a": -0.012, "delta_phi_m3": 1.1,
                                  "a4_a": 0.008, "delta_phi_m4": 2.0}),
        ("EPL_MULTIPOLE_M1M3M4", {"theta_E": 0.9, "gamma": 1.9, "e1": -0.3, "e2": 0.25,
                                  "center_x": 0.0, "center_y": 0.0, "a1_a": -0.02,
                                  "delta_phi_m1": 2.9, "a3_a": 0.005, "delta_phi_m3": 0.2,
                                  "a4_a": -0.015, "delta_phi_m4": 0.7}),
        ("NFW_ELLIPSE_CSE", {"Rs": 8.0, "alpha_Rs": 1.3, "e1": 0.1, "e2": -0.2,
                             "center_x": 0.1, "center_y": 0.0}),
        ("NFW_ELLIPSE_CSE", {"Rs": 0.5, "alpha_Rs": 0.2, "e1": -0.05, "e2": 0.02,
                             "center_x": -0.3, "center_y": 0.4}),
        ("CONVERGENCE", {"kappa": 0.07, "ra_0": 0.1, "dec_0": -0.2}),
    ]:
        x = rng.uniform(-2.5, 2.5, 64)
        y = rng.uniform(-2.5, 2.5, 64)
        out = np.stack([np.asarray(v) for v in LensModel([name]).hessian(x, y, [kw])])
        cases.append({"name": name, "kwargs": kw, "x": x, "y": y, "out": out})
    return cases


def _rows_order(lens, src, ll):
    """(list index, profile index, parameter name) in the row layout of
    ImageModel.pack_params: lens, source, lens-light profiles in order, each
    profile's parameters in param_names order."""
    from jaxtronomy_gb300 import profiles as P

    out = []
    for li, (names, table) in enumerate(((lens, P.LENS_PARAMS), (src, P.LIGHT_PARAMS),
                                         (ll, P.LIGHT_PARAMS))):
        for pi, n in enumerate(names):
            out += [(li, pi, k) for k in table[n]]
    return out


def gen_grad_fd():
    """Finite differences of the reference's likelihood_data_given_model
    (image_model.py:163-221) with respect to every parameter, in the row order of
    ImageModel.pack_params: a five-point stencil (step 1e-4, truncation ~1e-13
    relative) and the central difference with step 1e-6 of the gradient workload.
    Data are the reference's own image at parameters 1 % off in theta_E (or Rs),
    plus seeded Gaussian and Poisson noise."""
    import copy

    from jaxtronomy_gb300 import workloads as W

    scenes = []
    # the gradient workload's first system: 120x120, s = 2, 21x21 Moffat
    model, lens, src, ll, kern = W.gradient_batch(seed=1003, batch=1)
    scenes.append({"tag": "epl_shear_120_s2_psf21", "num_pix": 120, "delta_pix": 0.05, "s": 2,
                   "psf": {"psf_type": "PIXEL", "kernel_point_source": kern[0]},
                   "lens": model["lens_model_list"], "src": model["source_light_model_list"],
                   "ll": model["lens_light_model_list"], "kwargs_lens": W.instance(lens, 0),
                   "kwargs_source": W.instance(src, 0), "kwargs_lens_light": W.instance(ll, 0)})
    ks1 = [{"amp": 40.0, "R_sersic": 0.3, "n_sersic": 2.2, "e1": 0.06, "e2": -0.04,
            "center_x": 0.03, "center_y": 0.02}]
    ks2 = ks1 + [{"amp": 15.0, "R_sersic": 0.2, "n_sersic": 1.5, "e1": -0.05, "e2": 0.08,
                  "center_x": -0.12, "center_y": 0.07}]
    kll = [{"amp": 30.0, "R_sersic": 0.8, "n_sersic": 3.0, "e1": 0.05, "e2": 0.02,
            "center_x": 0.01, "center_y": -0.01}]
    moffat = W.moffat_pixel_kernel(0.12, 3.0, 0.06, 11)
    scenes.append({"tag": "nfw_cse_gaussian_psf", "num_pix": 40, "delta_pix": 0.06, "s": 2,
                   "psf": {"psf_type": "GAUSSIAN", "fwhm": 0.15, "truncation": 3.0},
                   "lens": ["NFW_ELLIPSE_CSE", "SHEAR"], "src": ["SERSIC_ELLIPSE"],
                   "ll": ["SERSIC_ELLIPSE"],
                   "kwargs_lens": [{"Rs": 9.0, "alpha_Rs": 1.4, "e1": 0.12, "e2": -0.07,
                                    "center_x": 0.02, "center_y": -0.01},
                                   {"gamma1": 0.02, "gamma2": -0.03, "ra_0": 0.0,
                                    "dec_0": 0.0}],
                   "kwargs_source": ks1, "kwargs_lens_light": kll})
    scenes.append({"tag": "multipole_two_sources", "num_pix": 40, "delta_pix": 0.06, "s": 2,
                   "psf": {"psf_type": "PIXEL", "kernel_point_source": moffat},
                   "lens": ["EPL_MULTIPOLE_M1M3M4", "SHEAR"],
                   "src": ["SERSIC_ELLIPSE", "SERSIC_ELLIPSE"], "ll": ["SERSIC_ELLIPSE"],
                   "kwargs_lens": [{"theta_E": 1.05, "gamma": 2.08, "e1": 0.1, "e2": -0.05,
                                    "center_x": 0.02, "center_y": 0.01, "a1_a": 0.01,
                                    "delta_phi_m1": 0.5, "a3_a": -0.012,
                                    "delta_phi_m3": 1.9, "a4_a": 0.009, "delta_phi_m4": 0.8},
                                   {"gamma1": -0.01, "gamma2": 0.03, "ra_0": 0.0,
                                    "dec_0": 0.0}],
                   "kwargs_source": ks2, "kwargs_lens_light": kll})
    scenes.append({"tag": "sie_convergence_no_psf", "num_pix": 32, "delta_pix": 0.07, "s": 3,
                   "psf": {"psf_type": "NONE"},
                   "lens": ["SIE", "CONVERGENCE", "SHEAR"], "src": ["SERSIC_ELLIPSE"],
                   "ll": ["SERSIC_ELLIPSE"],
                   "kwargs_lens": [{"theta_E": 0.95, "e1": -0.08, "e2": 0.11,
                                    "center_x": -0.02, "center_y": 0.03},
                                   {"kappa": 0.04, "ra_0": 0.1, "dec_0": -0.05},
                                   {"gamma1": 0.03, "gamma2": 0.01, "ra_0": 0.0,
                                    "dec_0": 0.0}],
                   "kwargs_source": ks1, "kwargs_lens_light": kll})
    k_super = W.moffat_pixel_kernel(0.12, 3.0, 0.06 / 3, 27)
    scenes.append({"tag": "epl_supersampled_convolution", "num_pix": 30, "delta_pix": 0.06,
                   "s": 3, "psf": {"psf_type": "PIXEL", "kernel_point_source": k_super,
                                   "point_source_supersampling_factor": 3},
                   "numerics": {"supersampling_convolution": True,
                                "supersampling_kernel_size": 3},
                   "lens": ["EPL", "SHEAR"], "src": ["SERSIC_ELLIPSE"], "ll": ["SERSIC_ELLIPSE"],
                   "kwargs_lens": [{"theta_E": 1.0, "gamma": 1.95, "e1": -0.06, "e2": 0.09,
                                    "center_x": 0.0, "center_y": 0.02},
                                   {"gamma1": 0.02, "gamma2": 0.02, "ra_0": 0.0,
                                    "dec_0": 0.0}],
                   "kwargs_source": ks1, "kwargs_lens_light": kll})
    scenes.append({"tag": "epl_gaussian_supersampled_convolution", "num_pix": 28,
                   "delta_pix": 0.07, "s": 2,
                   "psf": {"psf_type": "GAUSSIAN", "fwhm": 0.16, "truncation": 3.0},
                   "numerics": {"supersampling_convolution": True},
                   "lens": ["EPL", "SHEAR"], "src": ["SERSIC_ELLIPSE"], "ll": ["SERSIC_ELLIPSE"],
                   "kwargs_lens": [{"theta_E": 0.9, "gamma": 2.12, "e1": 0.07, "e2": 0.03,
                                    "center_x": -0.01, "center_y": 0.0},
                                   {"gamma1": -0.02, "gamma2": 0.01, "ra_0": 0.0,
                                    "dec_0": 0.0}],
                   "kwargs_source": ks1, "kwargs_lens_light": kll})

    out = []
    for i, sc in enumerate(scenes):
        kl, ks, kl2 = sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"]
        # simulated data: the reference's image at parameters 1 % off, plus noise
        truth = copy.deepcopy(kl)
        main = "theta_E" if "theta_E" in truth[0] else "Rs"
        truth[0][main] *= 1.01
        im0 = _image_model(sc["num_pix"], sc["delta_pix"], sc["s"], sc["psf"], sc["lens"],
                           sc["src"], sc["ll"], numerics=sc.get("numerics"))
        clean = np.asarray(im0.image(truth, ks, kl2))
        data = W.noisy_data(clean[None], seed=3000 + i)[0]
        im = _image_model(sc["num_pix"], sc["delta_pix"], sc["s"], sc["psf"], sc["lens"],
                          sc["src"], sc["ll"], data=data, numerics=sc.get("numerics"))
        order = _rows_order(sc["lens"], sc["src"], sc["ll"])
        lists = [kl, ks, kl2]

        def logl(li, pi, name, delta):
            kw = copy.deepcopy(lists)
            kw[li][pi][name] = kw[li][pi][name] + delta
            return float(np.asarray(im.likelihood_data_given_model(kw[0], kw[1], kw[2])))

        g5, g2 = [], []
        for li, pi, name in order:
            lists[li][pi].setdefault(name, 0.0)
        for li, pi, name in order:
            h = 1e-4
            f = [logl(li, pi, name, d * h) for d in (-2, -1, 1, 2)]
            g5.append((f[0] - 8 * f[1] + 8 * f[2] - f[3]) / (12 * h))
            g2.append((logl(li, pi, name, 1e-6) - logl(li, pi, name, -1e-6)) / 2e-6)
        logl0 = float(np.asarray(im.likelihood_data_given_model(kl, ks, kl2)))
        rec = {k: v for k, v in sc.items() if k != "psf"}
        psf = dict(sc["psf"])
        rec["kernel"] = psf.pop("kernel_point_source", None)
        rec["psf_kwargs"] = psf
        rec.update({"data": data, "logL": logl0, "grad_5pt": np.array(g5),
                    "grad_central_1e-6": np.array(g2),
                    "param_order": [[li, pi, n] for li, pi, n in order]})
        out.append(rec)
        print("grad_fd", sc["tag"], "logL", logl0, "params", len(order))
    return out


def _save(path, arrays, meta):
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **arrays)


def main(reference_root, only=None):
    refshim.install(reference_root)
    if only:
        for name in only:
            if name not in EXTRA:
                raise SystemExit("unknown golden file %s (choose from %s)"
                                 % (name, ", ".join(sorted(EXTRA))))
            EXTRA[name]()
        return
    for fn in EXTRA.values():
        fn()
    rng = np.random.default_rng(20240601)
    cases = gen_profiles(rng)
    arrays, meta = {}, []
    for i, c in enumerate(cases):
        arrays["x_%d" % i] = c["x"]
        arrays["y_%d" % i] = c["y"]
        arrays["out_%d" % i] = c["out"]
        meta.append({"kind": c["kind"], "name": c["name"], "kwargs": c["kwargs"]})
    _save(os.path.join(HERE, "profiles.npz"), arrays, meta)

    h = gen_hyp2f1()
    _save(os.path.join(HERE, "hyp2f1.npz"), {"z": h["z"], "nmax": h["nmax"], "out": h["out"]},
          {"a": h["a"], "b": h["b"], "c": h["c"]})

    scenes, like = gen_images()
    arrays, meta = {}, []
    for i, sc in enumerate(scenes):
        arrays["image_%d" % i] = sc.pop("image")
        if "kernel" in sc:
            arrays["kernel_%d" % i] = sc.pop("kernel")
        meta.append(sc)
    arrays["like_data"] = like.pop("data")
    _save(os.path.join(HERE, "images.npz"), arrays, {"scenes": meta, "likelihood": like})

    bulk = gen_bulk(np.random.default_rng(20240602))
    arrays, meta = {}, []
    for i, c in enumerate(bulk):
        for k in ("x", "y", "bx", "by"):
            arrays["%s_%d" % (k, i)] = c.pop(k)
        meta.append(c)
    _save(os.path.join(HERE, "bulk.npz"), arrays, meta)
    pts = gen_point_sources(np.random.default_rng(20240605))
    arrays, meta = {}, []
    for i, c in enumerate(pts):
        for k in ("image", "ps1", "data", "kernel"):
            v = c.pop(k, None)
            if v is not None:
                arrays["%s_%d" % (k, i)] = v
        meta.append(c)
    _save(os.path.join(HERE, "point_sources.npz"), arrays, meta)
    mp = gen_multi_plane(np.random.default_rng(20240604))
    arrays, meta = {}, []
    for i, c in enumerate(mp):
        for k in ("x", "y", "bx", "by"):
            arrays["%s_%d" % (k, i)] = c.pop(k)
        for k, v in c.pop("prep").items():
            arrays["prep_%d_%s" % (i, k)] = v
        meta.append(c)
    _save(os.path.join(HERE, "multiplane.npz"), arrays, meta)
    lin = gen_linear()
    arrays, meta = {}, []
    for i, c in enumerate(lin):
        for k in ("data", "mask", "model", "param", "cov", "kernel"):
            v = c.pop(k, None)
            if v is not None:
                arrays["%s_%d" % (k, i)] = v
        meta.append(c)
    _save(os.path.join(HERE, "linear.npz"), arrays, meta)
    print("wrote", len(cases), "profile cases,", len(scenes), "image scenes,", len(bulk),
          "bulk cases,", len(mp), "multi-plane cases,", len(lin), "linear-solve cases")


def write_serving_scenes():
    arrays, meta = {}, []
    for i, sc in enumerate(gen_serving_scenes()):
        arrays["image_%d" % i] = sc.pop("image")
        arrays["kernel_%d" % i] = sc.pop("kernel")
        meta.append(sc)
    _save(os.path.join(HERE, "serving_scenes.npz"), arrays, meta)


def write_grad_fd():
    arrays, meta = {}, []
    for i, sc in enumerate(gen_grad_fd()):
        for k in ("data", "kernel", "grad_5pt", "grad_central_1e-6"):
            v = sc.pop(k)
            if v is not None:
                arrays["%s_%d" % (k, i)] = np.asarray(v)
        meta.append(sc)
    _save(os.path.join(HERE, "grad_fd.npz"), arrays, meta)


def write_hessians():
    arrays, meta = {}, []
    for i, c in enumerate(gen_hessians()):
        for k in ("x", "y", "out"):
            arrays["%s_%d" % (k, i)] = c.pop(k)
        meta.append(c)
    _save(os.path.join(HERE, "hessians.npz"), arrays, meta)


# golden files that can be regenerated one at a time
EXTRA = {"serving_scenes.npz": write_serving_scenes, "grad_fd.npz": write_grad_fd,
         "hessians.npz": write_hessians}


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("JAXTRONOMY_SOURCE")
    if not root:
        raise SystemExit("usage: make_golden.py <jaxtronomy source tree> [file ...] "
                         "(or set JAXTRONOMY_SOURCE)")
    main(root, sys.argv[2:])
