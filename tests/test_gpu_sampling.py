"""The sampler-facing likelihood on the GPU: LikelihoodModule.logL_batch over an
ensemble of parameter vectors (one batched lensgb_loglike launch) against the
per-vector likelihood of the same ImageModel (bit for bit: batching does not
change a system's arithmetic) and against the FP64 oracle (1e-10 relative);
bounds, Gaussian priors and prepare_logL_func."""

import numpy as np
import pytest

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import sampling as S, workloads as W
from oracle import image as oimage

pytestmark = pytest.mark.gpu

N, DPIX, SS, K = 48, 0.06, 2, 9
MODEL = {"lens_model_list": ["EPL", "SHEAR"], "source_light_model_list": ["SERSIC_ELLIPSE"],
         "lens_light_model_list": ["SERSIC_ELLIPSE"]}


def _setup(n_walkers=64, seed=5):
    model, lens, src, ll, kern = W.gradient_batch(seed=seed, batch=1, num_pix=N, delta_pix=DPIX,
                                                  supersampling=SS, kernel_size=K)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    g = W.grid_kwargs(N, DPIX)
    im0 = J.ImageModel(J.ImageData(np.zeros((N, N)), exposure_time=1000.0, background_rms=0.01,
                                   **g),
                       J.PSF("PIXEL", kernel_point_source=kern[0]), J.LensModel(MODEL["lens_model_list"]),
                       J.LightModel(MODEL["source_light_model_list"]),
                       J.LightModel(MODEL["lens_light_model_list"]),
                       kwargs_numerics={"supersampling_factor": SS})
    data = W.noisy_data(im0.image(kl, ks, kll))
    kwargs_data = {"image_data": data, "background_rms": 0.01, "exposure_time": 1000.0, **g}
    kwargs_psf = {"psf_type": "PIXEL", "kernel_point_source": kern[0]}
    kwargs_numerics = {"supersampling_factor": SS}
    joint = {"multi_band_list": [[kwargs_data, kwargs_psf, kwargs_numerics]],
             "multi_band_type": "single-band"}
    param = S.Param(MODEL, kwargs_fixed_lens=[{}, {"ra_0": 0.0, "dec_0": 0.0}],
                    linear_solver=False)
    truth = param.kwargs2args(kl, ks, kll)
    rng = np.random.default_rng(seed + 1)
    args = truth + 1e-3 * rng.standard_normal((n_walkers, truth.size))
    im = J.ImageModel(J.ImageData(data, exposure_time=1000.0, background_rms=0.01, **g),
                      J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(MODEL["lens_model_list"]),
                      J.LightModel(MODEL["source_light_model_list"]),
                      J.LightModel(MODEL["lens_light_model_list"]),
                      kwargs_numerics=kwargs_numerics)
    return joint, param, args, im, data, kern[0], g


def test_batch_equals_per_vector_likelihood_and_oracle(cuda):
    joint, param, args, im, data, kern, g = _setup()
    lm = S.LikelihoodModule(joint, MODEL, param)
    got = lm.logL_batch(args)
    ref = np.array([im.likelihood_data_given_model(**{k: v for k, v in param.args2kwargs(a).items()
                                                      if k in ("kwargs_lens", "kwargs_source",
                                                               "kwargs_lens_light")})
                    for a in args])
    np.testing.assert_array_equal(got, ref)
    assert lm.logL(args[3]) == got[3]
    # the FP64 oracle on a few walkers
    for j in (0, 17, 63):
        kw = param.args2kwargs(args[j])
        scene = dict(nx=N, ny=N, supersampling_factor=SS, psf_type="PIXEL", kernel=kern, **MODEL,
                     **g)
        model = oimage.image(scene, kw["kwargs_lens"], kw["kwargs_source"], kw["kwargs_lens_light"])
        o = oimage.log_likelihood(model, data, np.ones_like(data), 0.01, exposure_time=1000.0)
        assert abs(got[j] - o) <= 1e-10 * abs(o), (j, got[j], o)


def test_bounds_priors_and_prepare_logl_func(cuda):
    joint, param, args, im, data, kern, g = _setup(n_walkers=16)
    prior_lens = [[0, "theta_E", 1.1, 0.05], [0, "gamma", 2.0, 0.1]]
    lm = S.LikelihoodModule(joint, MODEL, param, prior_lens=prior_lens)
    plain = S.LikelihoodModule(joint, MODEL, param)
    a = args.copy()
    a[5, 1] = 3.0            # EPL gamma above its upper bound 2.5
    got = lm.logL_batch(a)
    base = plain.logL_batch(a)
    assert got[5] == -1e18 and base[5] == -1e18
    keep = np.arange(16) != 5
    kw = param.args2kwargs(a)
    prior = (-(kw["kwargs_lens"][0]["theta_E"] - 1.1) ** 2 / 0.05 ** 2 / 2
             - (kw["kwargs_lens"][0]["gamma"] - 2.0) ** 2 / 0.1 ** 2 / 2)
    np.testing.assert_allclose(got[keep], (base + prior)[keep], rtol=1e-14)
    f = S.prepare_logL_func("gpu", lm.logL)
    np.testing.assert_array_equal(f(a), got)
    # the image likelihood can be switched off: priors only
    priors_only = S.LikelihoodModule(joint, MODEL, param, image_likelihood=False,
                                     prior_lens=prior_lens)
    np.testing.assert_allclose(priors_only.logL_batch(a)[keep], prior[keep], rtol=1e-14)


def test_image_likelihood_wrapper(cuda):
    joint, param, args, im, data, kern, g = _setup(n_walkers=4)
    il = S.ImageLikelihood(joint["multi_band_list"], "single-band", MODEL, linear_solver=False)
    kw = param.args2kwargs(args[0])
    logl, lin = il.logL(kw["kwargs_lens"], kw["kwargs_source"], kw["kwargs_lens_light"])
    assert lin is None
    assert logl == im.likelihood_data_given_model(kw["kwargs_lens"], kw["kwargs_source"],
                                                  kw["kwargs_lens_light"])
    assert il.num_data == N * N


def test_linear_solver_likelihood_module(cuda):
    """linear_solver=True (the reference's default): amplitudes are solved per
    walker; the batched logL equals ImageLinearFit per vector (bit for bit) and the
    oracle's linear solve (1e-10)."""
    from jaxtronomy_gb300.image_linear_solve import ImageLinearFit
    from oracle import linear as olinear

    joint, _, args, im, data, kern, g = _setup(n_walkers=8)
    param = S.Param(MODEL, kwargs_fixed_lens=[{}, {"ra_0": 0.0, "dec_0": 0.0}])
    n = param.num_param()[0]
    rng = np.random.default_rng(9)
    lo, hi = param.param_limits()
    truth = param.kwargs2args(*[[{k: v for k, v in kw.items() if k != "amp"} for kw in lst]
                                for lst in _truth_kwargs()])
    a = truth + 1e-3 * rng.standard_normal((8, n))
    lm = S.LikelihoodModule(joint, MODEL, param, source_marg=True)
    got = lm.logL_batch(a)
    fit = ImageLinearFit(J.ImageData(data, exposure_time=1000.0, background_rms=0.01, **g),
                         J.PSF("PIXEL", kernel_point_source=kern),
                         J.LensModel(MODEL["lens_model_list"]),
                         J.LightModel(MODEL["source_light_model_list"]),
                         J.LightModel(MODEL["lens_light_model_list"]),
                         kwargs_numerics={"supersampling_factor": SS})
    for j in range(8):
        kw = param.args2kwargs(a[j])
        l1, _ = fit.likelihood_data_given_model(kw["kwargs_lens"], kw["kwargs_source"],
                                                kw["kwargs_lens_light"], source_marg=True)
        assert got[j] == l1
    kw = param.args2kwargs(a[2])
    scene = dict(nx=N, ny=N, supersampling_factor=SS, psf_type="PIXEL", kernel=kern, **MODEL, **g)
    o, _, _, _ = olinear.likelihood(scene, kw["kwargs_lens"], kw["kwargs_source"],
                                    kw["kwargs_lens_light"], data, np.ones_like(data), 0.01,
                                    exposure_time=1000.0, source_marg=True)
    assert abs(got[2] - o) <= 1e-10 * abs(o), (got[2], o)


def _truth_kwargs():
    _, lens, src, ll, _ = W.gradient_batch(seed=5, batch=1, num_pix=N, delta_pix=DPIX,
                                           supersampling=SS, kernel_size=K)
    kl = W.instance(lens, 0)
    return kl, W.instance(src, 0), W.instance(ll, 0)


@pytest.mark.parametrize("linear", [False, True])
def test_point_source_ensemble_equals_per_vector(cuda, linear):
    """point_source_model_list in the sampler path: sampled image positions (and,
    without the linear solver, amplitudes) of a LENSED_POSITION model; the
    ensemble's logL equals each vector's ImageModel / ImageLinearFit likelihood."""
    from jaxtronomy_gb300.image_linear_solve import ImageLinearFit
    joint, _, _, _, data, kern, g = _setup()
    model = dict(MODEL, point_source_model_list=["LENSED_POSITION"])
    ra0, dec0 = np.array([1.0, -0.6, 0.3]), np.array([0.2, 0.8, -0.9])
    lo = {"ra_image": ra0 - 0.1, "dec_image": dec0 - 0.1, "point_amp": np.zeros(3)}
    hi = {"ra_image": ra0 + 0.1, "dec_image": dec0 + 0.1, "point_amp": np.full(3, 10.0)}
    param = S.Param(model, kwargs_fixed_lens=[{}, {"ra_0": 0.0, "dec_0": 0.0}],
                    kwargs_lower_ps=[lo], kwargs_upper_ps=[hi], num_point_source_list=[3],
                    linear_solver=linear)
    lo_all, hi_all = param.param_limits()
    rng = np.random.default_rng(9)
    model0, lens, src, ll, _ = W.gradient_batch(seed=5, batch=1, num_pix=N, delta_pix=DPIX,
                                                supersampling=SS, kernel_size=K)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    kps = [{"ra_image": ra0, "dec_image": dec0, "point_amp": np.array([2.0, 1.5, 1.0])}]
    truth = param.kwargs2args(kl, ks, kll, kps)
    args = np.clip(truth + 1e-3 * rng.standard_normal((16, truth.size)), lo_all, hi_all)
    lm = S.LikelihoodModule(joint, model, param)
    got = lm.logL_batch(args)
    cls = ImageLinearFit if linear else J.ImageModel
    im = cls(J.ImageData(data, exposure_time=1000.0, background_rms=0.01, **g),
             J.PSF("PIXEL", kernel_point_source=kern), J.LensModel(MODEL["lens_model_list"]),
             J.LightModel(MODEL["source_light_model_list"]),
             J.LightModel(MODEL["lens_light_model_list"]),
             point_source_class=J.PointSource(["LENSED_POSITION"]),
             kwargs_numerics={"supersampling_factor": SS})
    ref = []
    for a in args:
        kw = param.args2kwargs(a)
        r = im.likelihood_data_given_model(kw["kwargs_lens"], kw["kwargs_source"],
                                           kw["kwargs_lens_light"], kw["kwargs_ps"])
        ref.append(r[0] if linear else r)
    np.testing.assert_allclose(got, np.array(ref), rtol=1e-12, atol=0)
