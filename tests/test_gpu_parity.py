"""CUDA path (liblensgb.so via the C ABI) against the reference golden vectors
and the FP64 oracle.

Tolerances:
  * FP64 kernels: 1e-10 relative per pixel / per value (the plain-FP64 bar).
  * FP32-split kernels: 1e-5 relative per pixel on pixels above 1e-3 of the
    image maximum, and 1e-5 of the image maximum everywhere.
"""

import warnings

import numpy as np
import pytest
import torch

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W
from oracle import image as oimage

warnings.filterwarnings("ignore", category=RuntimeWarning)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 1e-5


def rel_err(got, ref, floor_frac=1e-3):
    got = np.asarray(got, float)
    ref = np.asarray(ref, float)
    scale = np.abs(ref).max()
    sig = np.abs(ref) >= floor_frac * scale
    per_pix = np.abs(got - ref)[sig] / np.abs(ref)[sig]
    return float(per_pix.max()), float(np.abs(got - ref).max() / scale)


def build_model(sc, precision="fp64", kernel=None):
    g = W.grid_kwargs(sc["num_pix"], sc["delta_pix"])
    data = J.ImageData(np.zeros((sc["num_pix"], sc["num_pix"])), exposure_time=1000.0,
                       background_rms=0.01, flux_scaling=sc.get("flux_scaling", 1), **g)
    numerics = {"supersampling_factor": sc["s"], "precision": precision}
    if sc.get("fei") is not None:
        numerics["flux_evaluate_indexes"] = np.asarray(sc["fei"], dtype=bool)
    ssf = 1
    if sc.get("ssc"):
        numerics["supersampling_convolution"] = True
        numerics["supersampling_kernel_size"] = sc.get("ssk")
        if sc.get("cks") is not None:
            numerics["convolution_kernel_size"] = sc["cks"]
        ssf = sc["s"]
    if sc["psf_type"] == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=sc["kernel"] if kernel is None else kernel,
                    point_source_supersampling_factor=ssf)
    elif sc["psf_type"] == "GAUSSIAN":
        psf = J.PSF("GAUSSIAN", fwhm=sc["fwhm"], truncation=sc["truncation"])
    else:
        psf = J.PSF("NONE")
    return J.ImageModel(data, psf, J.LensModel(sc["lens"]),
                        J.LightModel(sc["src"], deflection_scaling_list=sc.get("deflection_scaling")),
                        J.LightModel(sc["ll"]), kwargs_numerics=numerics)


SCENES, LIKE = golden_io.image_scenes()


@pytest.mark.parametrize("sc", SCENES, ids=lambda s: s["tag"])
def test_fp64_image_matches_reference(cuda, sc):
    im = build_model(sc, "fp64")
    got = im.image(sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    pp, mx = rel_err(got, sc["image"], floor_frac=1e-8)
    assert pp < FP64_RTOL and mx < FP64_RTOL, (pp, mx)


@pytest.mark.parametrize("sc", SCENES, ids=lambda s: s["tag"])
def test_fp32_image_matches_reference(cuda, sc):
    im = build_model(sc, "fp32")
    got = im.image(sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    pp, mx = rel_err(got, sc["image"])
    assert pp < FP32_RTOL and mx < FP32_RTOL, (pp, mx)


@pytest.mark.parametrize("case", golden_io.profile_cases(),
                         ids=lambda c: "%s-%s" % (c["kind"], c["name"]))
def test_profiles_match_reference(cuda, case):
    if case["kind"] == "hessian":
        # exact second derivatives vs the reference's analytic Hessians
        lm = J.LensModel([case["name"]])
        got = np.array(lm.hessian(case["x"], case["y"], [case["kwargs"]]))
        ref = case["out"]
        if case["name"] in ("SIE", "NIE"):
            # the reference's NIE Hessian is a one-sided difference of its deflection
            # with step 1e-10 (nie.py:298-312): ~1e-6 relative error of its own
            np.testing.assert_allclose(got, ref, rtol=0, atol=5e-6 * np.abs(ref).max())
        else:
            np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
        # derived quantities (lens_model.py:417-526)
        f_xx, f_xy, f_yx, f_yy = ref
        g_xx, g_xy, g_yx, g_yy = got
        np.testing.assert_allclose(lm.kappa(case["x"], case["y"], [case["kwargs"]]),
                                   (g_xx + g_yy) / 2, rtol=1e-14, atol=1e-15)
        mag = 1.0 / ((1 - g_xx) * (1 - g_yy) - g_xy * g_yx)
        np.testing.assert_allclose(lm.magnification(case["x"], case["y"], [case["kwargs"]]),
                                   mag, rtol=1e-12)
        fd = np.array(lm.hessian(case["x"], case["y"], [case["kwargs"]], diff=1e-5))
        np.testing.assert_allclose(fd, ref, rtol=1e-4, atol=1e-5 * np.abs(ref).max())
        return
    if case["kind"] == "lens":
        lm = J.LensModel([case["name"]])
        ax, ay = lm.alpha(case["x"], case["y"], [case["kwargs"]])
        got = np.array([ax, ay])
        bx, by = lm.ray_shooting(case["x"], case["y"], [case["kwargs"]])
        np.testing.assert_allclose(bx, case["x"] - case["out"][0], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(by, case["y"] - case["out"][1], rtol=1e-12, atol=1e-12)
    else:
        got = J.LightModel([case["name"]]).surface_brightness(case["x"], case["y"],
                                                              [case["kwargs"]])[None]
    ref = case["out"]
    # 1e-10 relative per value; the absolute floor (1e-12 of the case maximum)
    # covers values the reference formula itself computes through a cancellation
    # (e.g. TNFW at R << Rs, tnfw.py:339-348), where two correct FP64
    # evaluations differ by ~cond * eps
    np.testing.assert_allclose(got, ref, rtol=FP64_RTOL, atol=1e-12 * np.abs(ref).max())


def test_likelihood_matches_reference(cuda):
    sc = [s for s in SCENES if s["tag"] == LIKE["scene"]][0]
    g = W.grid_kwargs(sc["num_pix"], sc["delta_pix"])
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-5)):
        data = J.ImageData(LIKE["data"], exposure_time=LIKE["exp_time"],
                           background_rms=LIKE["bkg"], **g)
        im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=sc["kernel"]),
                          J.LensModel(sc["lens"]), J.LightModel(sc["src"]), J.LightModel(sc["ll"]),
                          kwargs_numerics={"precision": precision})
        got = im.likelihood_data_given_model(sc["kwargs_lens"], sc["kwargs_source"],
                                             sc["kwargs_lens_light"])
        assert abs(got - LIKE["logL"]) <= tol * abs(LIKE["logL"]), (precision, got, LIKE["logL"])


def _oracle_images(model, lens, src, ll, kern, n, s, dpix, idx):
    g = W.grid_kwargs(n, dpix)
    out = []
    for i in idx:
        scene = dict(nx=n, ny=n, supersampling_factor=s, psf_type="PIXEL", kernel=kern[i],
                     lens_model_list=model["lens_model_list"],
                     source_light_model_list=model["source_light_model_list"],
                     lens_light_model_list=model["lens_light_model_list"], **g)
        out.append(oimage.image(scene, W.instance(lens, i), W.instance(src, i),
                                W.instance(ll, i)))
    return out


def _batch_model(model, kern0, n, dpix, s, precision):
    g = W.grid_kwargs(n, dpix)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    return J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern0),
                        J.LensModel(model["lens_model_list"]),
                        J.LightModel(model["source_light_model_list"]),
                        J.LightModel(model["lens_light_model_list"]),
                        kwargs_numerics={"supersampling_factor": s, "precision": precision})


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_single_image_workload_batch(cuda, precision):
    model, lens, src, ll, kern = W.single_sie(seed=1000, batch=6)
    im = _batch_model(model, kern[0], 60, 0.05, 1, precision)
    got = im.image_batch(lens, src, ll, psf_kernels=kern).double().cpu().numpy()
    refs = _oracle_images(model, lens, src, ll, kern, 60, 1, 0.05, range(6))
    tol = FP64_RTOL if precision == "fp64" else FP32_RTOL
    for i, ref in enumerate(refs):
        pp, mx = rel_err(got[i], ref, 1e-8 if precision == "fp64" else 1e-3)
        assert pp < tol and mx < tol, (i, pp, mx)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_epl_batch_workload_reduced_grid(cuda, precision):
    # the 1024 x 180^2 / s=3 / 31x31 workload at a size the oracle finishes fast
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=4, num_pix=48, kernel_size=31)
    im = _batch_model(model, kern[0], 48, 0.04, 3, precision)
    got = im.image_batch(lens, src, ll, psf_kernels=kern).double().cpu().numpy()
    refs = _oracle_images(model, lens, src, ll, kern, 48, 3, 0.04, range(4))
    tol = FP64_RTOL if precision == "fp64" else FP32_RTOL
    for i, ref in enumerate(refs):
        pp, mx = rel_err(got[i], ref, 1e-8 if precision == "fp64" else 1e-3)
        assert pp < tol and mx < tol, (i, pp, mx)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_flags_and_components(cuda, precision):
    sc = SCENES[2]  # batch_epl_0, s=3
    im = build_model(sc, precision)
    args = (sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    scene = golden_io.oracle_scene(sc)
    tol = FP64_RTOL if precision == "fp64" else FP32_RTOL
    floor = 1e-8 if precision == "fp64" else 1e-3
    for kw in [dict(unconvolved=True), dict(source_add=False), dict(lens_light_add=False)]:
        got = im.image(*args, **kw)
        ref = oimage.image(scene, *args, **kw)
        pp, mx = rel_err(got, ref, floor)
        assert pp < tol and mx < tol, (kw, pp, mx)
    src = im.source_surface_brightness(sc["kwargs_source"], sc["kwargs_lens"])
    ll = im.lens_surface_brightness(sc["kwargs_lens_light"])
    full = im.image(*args)
    np.testing.assert_allclose(src + ll, full, rtol=1e-4 if precision == "fp32" else 1e-12)


def test_fp32_refinement_fixes_steep_source_cusp(cuda):
    # system 207 of the 1024-system workload: an n=3.85, R_sersic=0.10" source whose
    # centre images near the Einstein ring, where beta = theta - alpha cancels and
    # the FP32 deflection error is amplified; the FP64 refine pass must bring the
    # image within 1e-5 of FP64
    # (the generator draws each parameter for the whole batch, so the batch size
    # must be the workload's 1024 for system 207 to be the same system)
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=1024)
    one = [W.subset(k, [207]) for k in (lens, src, ll)]
    psf = kern[207]
    g = W.grid_kwargs(180, 0.04)

    def make(**kn):
        data = J.ImageData(np.zeros((180, 180)), exposure_time=1000.0, background_rms=0.01, **g)
        return J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=psf),
                            J.LensModel(model["lens_model_list"]),
                            J.LightModel(model["source_light_model_list"]),
                            J.LightModel(model["lens_light_model_list"]),
                            kwargs_numerics=dict(supersampling_factor=3, **kn))

    ref = make(precision="fp64").image_batch(*one, psf_kernels=psf)[0].cpu().numpy()
    off = make(precision="fp32", fp32_refine_tol=0.0)
    on = make(precision="fp32")
    e_off = rel_err(off.image_batch(*one, psf_kernels=psf)[0].double().cpu().numpy(), ref)[0]
    e_on = rel_err(on.image_batch(*one, psf_kernels=psf)[0].double().cpu().numpy(), ref)[0]
    assert on.refined_pixels() > 0
    assert e_off > FP32_RTOL  # the case really is ill-conditioned in plain FP32
    assert e_on < FP32_RTOL, (e_off, e_on)


def test_batch_equals_single_bitwise_and_deterministic(cuda):
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=5, num_pix=40, kernel_size=11)
    for precision in ("fp64", "fp32"):
        im = _batch_model(model, kern[0], 40, 0.04, 3, precision)
        a = im.image_batch(lens, src, ll, psf_kernels=kern)
        b = im.image_batch(lens, src, ll, psf_kernels=kern)
        assert torch.equal(a, b)
        for i in range(5):
            one = im.image_batch(*[W.instance(k, i) for k in (lens, src, ll)],
                                 psf_kernels=kern[i])
            assert torch.equal(one[0], a[i])


def test_fp64_ray_per_thread_launch_equals_pixel_per_thread_launch(cuda):
    """A single 180x180, s = 3 system runs the FP64 kernel with one thread per
    ray (a per-pixel launch would fill less than one wave); a batch of eight runs
    one thread per pixel.  Both combine each pixel's rays in the same order, and
    the small-launch convolution tiles sum in the same order as the large ones:
    the images must agree bit for bit."""
    model, lens, src, ll, kern = W.batch_epl(seed=1001, batch=8, num_pix=180, kernel_size=31)
    im = _batch_model(model, kern[0], 180, 0.04, 3, "fp64")
    a = im.image_batch(lens, src, ll, psf_kernels=kern)
    for i in (0, 5):
        one = im.image_batch(*[W.instance(k, i) for k in (lens, src, ll)], psf_kernels=kern[i])
        assert torch.equal(one[0], a[i])


def test_empty_batch_and_edge_profiles(cuda):
    model, lens, src, ll, kern = W.batch_epl(seed=5, batch=3, num_pix=24, kernel_size=5)
    im = _batch_model(model, kern[0], 24, 0.04, 2, "fp64")
    empty = W.subset(lens, []), W.subset(src, []), W.subset(ll, [])
    rows = im.pack_params(*empty)
    assert rows.shape[0] == 0 or rows.shape[0] == 1
    out = im.image_batch(rows=np.zeros((0, rows.shape[1])))
    assert tuple(out.shape) == (0, 24, 24)
    # round EPL (f == 0 branch) and a very elliptical one (nmax = 500)
    kl = W.instance(lens, 0)
    for e1, e2 in [(0.0, 0.0), (0.95, 0.0)]:
        kl[0]["e1"], kl[0]["e2"] = e1, e2
        got = im.image(kl, W.instance(src, 0), W.instance(ll, 0))
        scene = dict(nx=24, ny=24, supersampling_factor=2, psf_type="PIXEL", kernel=kern[0],
                     lens_model_list=model["lens_model_list"],
                     source_light_model_list=model["source_light_model_list"],
                     lens_light_model_list=model["lens_light_model_list"],
                     **W.grid_kwargs(24, 0.04))
        ref = oimage.image(scene, kl, W.instance(src, 0), W.instance(ll, 0))
        pp, mx = rel_err(got, ref, 1e-8)
        assert pp < FP64_RTOL and mx < FP64_RTOL, (e1, pp, mx)


@pytest.mark.parametrize("name", ["NFW_ELLIPSE_CSE", "EPL_MULTIPOLE_M1M3M4"])
def test_exact_hessian_of_cse_and_multipole_matches_differences(cuda, name):
    """lensgb_hessian for NFW_ELLIPSE_CSE and EPL_MULTIPOLE_M1M3M4 (the
    adjoint's dual-number deflections) against the reference's square finite
    differences of alpha (lens_model.py:617-650) with step 1e-6, away from the
    centre."""
    for case in [c for c in golden_io.profile_cases() if c["kind"] == "lens" and c["name"] == name]:
        lm = J.LensModel([name])
        x, y = case["x"][4:], case["y"][4:]
        got = np.array(lm.hessian(x, y, [case["kwargs"]]))
        fd = np.array(lm.hessian(x, y, [case["kwargs"]], diff=1e-6))
        np.testing.assert_allclose(got, fd, rtol=1e-5, atol=1e-6 * np.abs(fd).max())


@pytest.mark.parametrize("case", golden_io.hessian_cases(),
                         ids=lambda c: "%s-%g" % (c["name"], c["kwargs"].get("e1", 0.0)))
def test_exact_hessian_matches_reference_hessian(cuda, case):
    """lensgb_hessian against the reference's own Hessians (analytic EPL +
    multipole, analytic CSE sum, constant CONVERGENCE)."""
    got = np.array(J.LensModel([case["name"]]).hessian(case["x"], case["y"], [case["kwargs"]]))
    ref = case["out"]
    np.testing.assert_allclose(got, ref, rtol=1e-8, atol=1e-10 * np.abs(ref).max())
