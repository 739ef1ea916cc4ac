"""Readers for the committed golden fixtures (tests/golden/*.npz) and the
scene dicts the oracle consumes."""

import json
import os

import numpy as np

from jaxtronomy_gb300.workloads import grid_kwargs
from oracle import numerics as onum

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    d = np.load(os.path.join(GOLDEN, name), allow_pickle=False)
    return d, json.loads(str(d["meta"]))


def profile_cases():
    d, meta = load("profiles.npz")
    out = []
    for i, m in enumerate(meta):
        out.append(dict(m, x=d["x_%d" % i], y=d["y_%d" % i], out=d["out_%d" % i]))
    return out


def image_scenes():
    d, meta = load("images.npz")
    scenes = []
    for i, sc in enumerate(meta["scenes"]):
        sc = dict(sc)
        sc["image"] = d["image_%d" % i]
        sc["kernel"] = d["kernel_%d" % i] if ("kernel_%d" % i) in d.files else None
        scenes.append(sc)
    like = dict(meta["likelihood"])
    like["data"] = d["like_data"]
    return scenes, like


def oracle_scene(sc):
    """Scene dict of the oracle (oracle.image) for a golden image scene."""
    g = grid_kwargs(sc["num_pix"], sc["delta_pix"])
    kernel = sc.get("kernel")
    if kernel is not None:
        kernel = kernel / kernel.sum()
        if sc.get("ssc") and sc.get("cks") is not None:
            size = sc["cks"] * sc["s"]
            kernel = onum.cut_psf(kernel, size if size % 2 else size + 1)
    extra = {}
    if sc.get("fei") is not None:
        extra["flux_evaluate_indexes"] = np.asarray(sc["fei"], dtype=bool)
    if sc.get("ssc"):
        extra = {"supersampling_convolution": True,
                 "supersampling_kernel_size": sc.get("ssk")}
    return dict(nx=sc["num_pix"], ny=sc["num_pix"], supersampling_factor=sc["s"], **extra,
                psf_type=sc["psf_type"], kernel=kernel, fwhm=sc.get("fwhm"),
                truncation=sc.get("truncation", 5.0), lens_model_list=sc["lens"],
                source_light_model_list=sc["src"], lens_light_model_list=sc["ll"],
                flux_scaling=sc.get("flux_scaling", 1.0),
                deflection_scaling_list=sc.get("deflection_scaling"), **g)


def bulk_cases():
    d, meta = load("bulk.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("x", "y", "bx", "by"):
            c[k] = d["%s_%d" % (k, i)]
        out.append(c)
    return out


def multi_plane_cases():
    """MultiPlaneBulk cases: unique list, lens list, kwargs, redshifts, rays, the
    reference's prepared kwargs (``prep``) and beta.  Distances of the reference run:
    flat Lambda-CDM, H0 = 70, Om0 = 0.3, no radiation."""
    d, meta = load("multiplane.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("x", "y", "bx", "by"):
            c[k] = d["%s_%d" % (k, i)]
        pre = "prep_%d_" % i
        prep = {k[len(pre):]: d[k] for k in d.files if k.startswith(pre)}
        c["prep"] = {"all_kwargs": {k[3:]: v for k, v in prep.items() if k.startswith("kw_")},
                     **{k: v for k, v in prep.items() if not k.startswith("kw_")}}
        out.append(c)
    return out


def point_source_cases():
    """ImageModel scenes with LENSED_POSITION + UNLENSED point sources: kwargs,
    data, the reference's image, its point-source term of model 1 and logL
    (exposure 800 s, background rms 0.01)."""
    d, meta = load("point_sources.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("image", "ps1", "data", "kernel"):
            key = "%s_%d" % (k, i)
            c[k] = d[key] if key in d.files else None
        out.append(c)
    return out


def point_source_scene(c):
    """Oracle scene dict of a point-source case (its extended-light part)."""
    g = grid_kwargs(c["n"], c["dpix"])
    num = c.get("numerics") or {}
    kernel = None if c["kernel"] is None else c["kernel"] / c["kernel"].sum()
    extra = {}
    if num.get("supersampling_convolution"):
        extra = {"supersampling_convolution": True,
                 "supersampling_kernel_size": num.get("supersampling_kernel_size")}
    return dict(nx=c["n"], ny=c["n"], supersampling_factor=c["s"], psf_type=c["psf"]["psf_type"],
                kernel=kernel, lens_model_list=["EPL", "SHEAR"],
                source_light_model_list=["SERSIC_ELLIPSE"], lens_light_model_list=["SERSIC"],
                flux_scaling=c["flux_scaling"], **extra, **g)


def linear_cases():
    """ImageLinearFit cases: kwargs, data, mask and the reference's amplitudes,
    model image, inverse normal matrix (source_marg) and logL."""
    d, meta = load("linear.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("data", "mask", "model", "param", "cov", "kernel"):
            key = "%s_%d" % (k, i)
            c[k] = d[key] if key in d.files else None
        out.append(c)
    return out


def linear_scene(c):
    """The oracle scene of a linear-solve case."""
    g = grid_kwargs(c["n"], c["dpix"])
    sc = dict(nx=c["n"], ny=c["n"], supersampling_factor=c["s"], psf_type=c["psf"]["psf_type"],
              lens_model_list=c["lens"], source_light_model_list=c["src"],
              lens_light_model_list=c["ll"], deflection_scaling_list=c["dsl"], **g)
    if c["psf"]["psf_type"] == "PIXEL":
        sc["kernel"] = c["kernel"]
        sc["ps_kernel"] = c["kernel"] / c["kernel"].sum()
    elif c["psf"]["psf_type"] == "GAUSSIAN":
        sc["fwhm"] = c["psf"]["fwhm"]
        sc["truncation"] = c["psf"]["truncation"]
    return sc


def serving_scenes():
    """The four serving lens stacks with two sources at 100x100, s = 4, 41x41
    kernel: the reference's image per scene (tag = lens stack)."""
    d, meta = load("serving_scenes.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        c["image"] = d["image_%d" % i]
        c["kernel"] = d["kernel_%d" % i]
        out.append(c)
    return out


def grad_fd_cases():
    """Finite-difference gradients of the reference's likelihood (grad_fd.npz):
    scene, data, PSF, the five-point and the step-1e-6 central differences in
    the row order of ImageModel.pack_params."""
    d, meta = load("grad_fd.npz")
    out = []
    for i, m in enumerate(meta):
        c = dict(m)
        for k in ("data", "kernel", "grad_5pt", "grad_central_1e-6"):
            key = "%s_%d" % (k, i)
            c[k] = d[key] if key in d.files else None
        out.append(c)
    return out


def hessian_cases():
    """The reference's LensModel.hessian of EPL_MULTIPOLE_M1M3M4, NFW_ELLIPSE_CSE
    and CONVERGENCE at seeded points (hessians.npz): f_xx, f_xy, f_yx, f_yy."""
    d, meta = load("hessians.npz")
    return [dict(m, x=d["x_%d" % i], y=d["y_%d" % i], out=d["out_%d" % i])
            for i, m in enumerate(meta)]
