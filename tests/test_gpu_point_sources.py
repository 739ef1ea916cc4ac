"""Point sources on the GPU (lensgb_point_sources_add, lensgb_loglike_image
through the C ABI) against the reference golden vectors and the oracle.

Tolerances: FP64 images and the point-source term 1e-10 relative (absolute
floor 1e-10 of the image maximum), logL 1e-10 relative; FP32 images within
1e-5 of the image maximum.
"""

import numpy as np
import pytest
import torch

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model(case, precision="fp64"):
    g = W.grid_kwargs(case["n"], case["dpix"])
    data = J.ImageData(case["data"], exposure_time=800.0, background_rms=0.01,
                       flux_scaling=case["flux_scaling"], **g)
    pk = dict(case["psf"])
    if case["kernel"] is not None:
        pk["kernel_point_source"] = case["kernel"]
    num = dict({"supersampling_factor": case["s"], "precision": precision},
               **(case.get("numerics") or {}))
    return J.ImageModel(data, J.PSF(**pk), J.LensModel(["EPL", "SHEAR"]),
                        J.LightModel(["SERSIC_ELLIPSE"]), J.LightModel(["SERSIC"]),
                        point_source_class=J.PointSource(
                            ["LENSED_POSITION", "UNLENSED"],
                            fixed_magnification_list=case.get("fixed")),
                        kwargs_numerics=num)


@pytest.mark.parametrize("case", golden_io.point_source_cases(), ids=lambda c: c["tag"])
def test_point_source_image_matches_reference(cuda, case):
    im = _model(case)
    got = im.image(case["lens"], case["src"], case["ll"], case["ps"],
                   kwargs_special=case["special"], unconvolved=case["unconvolved"])
    tol = 1e-10 * np.abs(case["image"]).max()
    np.testing.assert_allclose(got, case["image"], rtol=1e-10, atol=tol)
    if not case["unconvolved"]:
        ps1 = im.point_source(case["ps"], case["lens"], kwargs_special=case["special"], k=1)
        np.testing.assert_allclose(ps1, case["ps1"], rtol=1e-10, atol=tol)
        logl = im.likelihood_data_given_model(case["lens"], case["src"], case["ll"], case["ps"],
                                              kwargs_special=case["special"])
        assert abs(logl - case["logL"]) <= 1e-10 * abs(case["logL"])
    im32 = _model(case, "fp32")
    got32 = im32.image(case["lens"], case["src"], case["ll"], case["ps"],
                       kwargs_special=case["special"], unconvolved=case["unconvolved"])
    assert np.abs(got32 - case["image"]).max() <= 1e-5 * np.abs(case["image"]).max()


def test_point_source_batch_equals_single(cuda):
    """(B, n_images) point-source kwargs in one batched call equal B single calls,
    bit for bit; per-system PSF kernels reach the rendering too."""
    case = golden_io.point_source_cases()[0]
    im = _model(case)
    rng = np.random.default_rng(5)
    B = 5
    ps = [{k: np.asarray(v, float)[None] + (rng.normal(0, 0.05, (B, len(v))) if k != "point_amp"
                                            else np.zeros((B, len(v))))
           for k, v in case["ps"][0].items()},
          {k: np.broadcast_to(np.asarray(v, float), (B, len(v))).copy()
           for k, v in case["ps"][1].items()}]
    lens = [{k: np.full(B, v) for k, v in kw.items()} for kw in case["lens"]]
    src = [{k: np.full(B, v) for k, v in kw.items()} for kw in case["src"]]
    ll = [{k: np.full(B, v) for k, v in kw.items()} for kw in case["ll"]]
    batch = im.image_batch(lens, src, ll, kwargs_ps=ps).cpu().numpy()
    for b in range(B):
        one = im.image(case["lens"], case["src"], case["ll"],
                       [{k: v[b] for k, v in m.items()} for m in ps])
        np.testing.assert_array_equal(batch[b], one)
    # per-system kernels: the model kernel repeated gives the same images
    kern = case["kernel"] / case["kernel"].sum()
    kk = np.repeat(kern[None], B, axis=0)
    again = im.image_batch(lens, src, ll, kwargs_ps=ps, psf_kernels=kk).cpu().numpy()
    np.testing.assert_allclose(again, batch, rtol=1e-13, atol=1e-14 * np.abs(batch).max())
    # point_source_add=False drops them
    bare = im.image_batch(lens, src, ll, kwargs_ps=ps, point_source_add=False).cpu().numpy()
    assert np.abs(batch - bare).max() > 0.1


def test_point_source_options_raise(cuda):
    case = golden_io.point_source_cases()[0]
    g = W.grid_kwargs(case["n"], case["dpix"])
    data = J.ImageData(case["data"], exposure_time=800.0, background_rms=0.01, **g)
    with pytest.raises(ValueError):
        J.PointSource(["SOURCE_POSITION"])
    with pytest.raises(ValueError):
        J.PointSource(["UNLENSED"], save_cache=True)
    with pytest.raises(ValueError):
        J.ImageModel(data, J.PSF("GAUSSIAN", fwhm=0.1), J.LensModel(["SIE"]),
                     J.LightModel(["SERSIC"]), J.LightModel([]),
                     point_source_class=J.PointSource(["UNLENSED"]))
    im = _model(case)
    with pytest.raises(ValueError):
        im.image(case["lens"], case["src"], case["ll"], None)
    with pytest.raises(ValueError):
        im.likelihood_grad_batch(case["lens"], case["src"], case["ll"])


def test_fixed_magnification_batch_equals_single(cuda):
    """Batched lens kwargs with fixed-magnification point sources: one Hessian launch
    for the batch gives each system its own magnifications."""
    case = [c for c in golden_io.point_source_cases() if c["tag"] == "fixed_magnification"][0]
    im = _model(case)
    B = 3
    lens = [{k: np.full(B, v) * (1 + 0.01 * np.arange(B)) if k == "theta_E" else np.full(B, v)
             for k, v in kw.items()} for kw in case["lens"]]
    src = [{k: np.full(B, v) for k, v in kw.items()} for kw in case["src"]]
    ll = [{k: np.full(B, v) for k, v in kw.items()} for kw in case["ll"]]
    batch = im.image_batch(lens, src, ll, kwargs_ps=case["ps"]).cpu().numpy()
    for b in range(B):
        one = im.image([{k: float(v[b]) for k, v in kw.items()} for kw in lens], case["src"],
                       case["ll"], case["ps"])
        np.testing.assert_allclose(batch[b], one, rtol=1e-13, atol=1e-13 * np.abs(one).max())
