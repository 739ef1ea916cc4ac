"""ImageLinearFit on the GPU (component images through lensgb_image, the solve in
lensgb_linear_solve) against the reference's ImageLinearFit golden vectors:
amplitudes, model image, inverse normal matrix and logL at 1e-10 relative
(FP64); batched solves equal single ones; the FP32 model's amplitudes within
1e-5 of FP64."""

import copy

import numpy as np
import pytest

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W
from jaxtronomy_gb300.image_linear_solve import ImageLinearFit

pytestmark = pytest.mark.gpu


def _fit(c, precision="fp64"):
    g = W.grid_kwargs(c["n"], c["dpix"])
    data = J.ImageData(c["data"], exposure_time=c["exp_time"], background_rms=c["bkg"], **g)
    p = c["psf"]
    if p["psf_type"] == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=c["kernel"])
    elif p["psf_type"] == "GAUSSIAN":
        psf = J.PSF("GAUSSIAN", fwhm=p["fwhm"], truncation=p["truncation"])
    else:
        psf = J.PSF("NONE")
    pcls = (J.PointSource(c["ps_types"], fixed_magnification_list=c.get("ps_fixed"))
            if c.get("ps_types") else None)
    return ImageLinearFit(data, psf, J.LensModel(c["lens"]),
                          J.LightModel(c["src"], deflection_scaling_list=c["dsl"]),
                          J.LightModel(c["ll"]), point_source_class=pcls,
                          kwargs_numerics={"supersampling_factor": c["s"], "precision": precision},
                          likelihood_mask=c["mask"])


@pytest.mark.parametrize("case", golden_io.linear_cases(), ids=lambda c: c["tag"])
def test_linear_fit_matches_reference(cuda, case):
    im = _fit(case)
    kl, ks, kll, kps = (copy.deepcopy(case.get(k) or []) for k in ("kl", "ks", "kll", "ps"))
    logl, param = im.likelihood_data_given_model(kl, ks, kll, kps, source_marg=case["marg"],
                                                 check_positive_flux=case["pos"])
    assert abs(logl - case["logL"]) <= 1e-10 * abs(case["logL"]), (logl, case["logL"])
    np.testing.assert_allclose(param, case["param"], rtol=1e-10, atol=1e-12)
    # the amplitudes are written into the kwargs, as the reference does
    assert ks[0]["amp"] == param[0]
    if kps:
        # point_amp (or source_amp with fixed magnification) written back too
        n_ext = len(case["src"]) + len(case["ll"])
        if case.get("ps_fixed"):
            assert kps[0]["source_amp"] == param[n_ext]
        else:
            np.testing.assert_array_equal(kps[0]["point_amp"], param[n_ext:n_ext + 4])
    kl, ks, kll, kps = (copy.deepcopy(case.get(k) or []) for k in ("kl", "ks", "kll", "ps"))
    model, err, cov, p2 = im.image_linear_solve(kl, ks, kll, kps, inv_bool=case["marg"])
    np.testing.assert_array_equal(p2, param)
    np.testing.assert_allclose(model, case["model"], rtol=1e-10,
                               atol=1e-12 * np.abs(case["model"]).max())
    if case["cov"] is not None:
        np.testing.assert_allclose(cov, case["cov"], rtol=1e-9, atol=1e-14)
    A = im.linear_response_matrix(kl, ks, kll, kps)
    n_ps = (1 if case.get("ps_fixed") else
            sum(len(p["ra_image"]) for p in (case.get("ps") or [])))
    assert A.shape == (len(case["src"]) + len(case["ll"]) + n_ps, int(np.sum(case["mask"])))


def test_batched_solve_equals_single_and_fp32(cuda):
    case = golden_io.linear_cases()[1]  # two sources + lens light, mask, source_marg
    im = _fit(case)
    im32 = _fit(case, "fp32")
    rng = np.random.default_rng(3)
    B = 6
    kl = [{k: v * (1 + 0.01 * rng.standard_normal(B)) if k in ("theta_E", "gamma") else v
           for k, v in kw.items()} for kw in case["kl"]]
    ks, kll = case["ks"], case["kll"]
    logl, param, image, cov = im.likelihood_linear_batch(kl, ks, kll, source_marg=True)
    logl32, param32, _, _ = im32.likelihood_linear_batch(kl, ks, kll, source_marg=True)
    for i in range(B):
        kli = [{k: float(v[i]) if np.ndim(v) else v for k, v in kw.items()} for kw in kl]
        l1, p1 = im.likelihood_data_given_model(kli, copy.deepcopy(ks), copy.deepcopy(kll),
                                                source_marg=True)
        assert l1 == float(logl[i])
        np.testing.assert_array_equal(p1, param[i].cpu().numpy())
    p64 = param.cpu().numpy()
    np.testing.assert_allclose(param32.cpu().numpy(), p64, rtol=1e-5, atol=1e-5 * np.abs(p64).max())
