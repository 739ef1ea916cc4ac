"""Host logic of the sampler-facing layer (no GPU): parameter bookkeeping of
Param, bounds, and the construction-time errors of LikelihoodModule /
ImageLikelihood / prepare_logL_func."""

import numpy as np
import pytest

from jaxtronomy_gb300 import sampling as S

MODEL = {"lens_model_list": ["EPL", "SHEAR"], "source_light_model_list": ["SERSIC_ELLIPSE"],
         "lens_light_model_list": ["SERSIC"]}
FIXED_LENS = [{"center_x": 0.0, "center_y": 0.0}, {"ra_0": 0.0, "dec_0": 0.0}]


def _param(**kw):
    return S.Param(MODEL, kwargs_fixed_lens=FIXED_LENS, linear_solver=False, **kw)


def test_param_order_and_limits():
    p = _param()
    n, names = p.num_param()
    # EPL: theta_E gamma e1 e2 (centre fixed); SHEAR: gamma1 gamma2; Sersic ellipse 7; Sersic 5
    assert n == 4 + 2 + 7 + 5
    assert names[:6] == ["theta_E_lens0", "gamma_lens0", "e1_lens0", "e2_lens0", "gamma1_lens1",
                         "gamma2_lens1"]
    lo, hi = p.param_limits()
    assert lo[1] == 1.5 and hi[1] == 2.5          # EPL gamma (epl.py:51-66)
    assert lo[6] == 0.0 and hi[6] == 100.0        # Sersic amp (sersic_ellipse.py:26-43)
    assert lo[8] == 0.5 and hi[8] == 8.0          # n_sersic


def test_param_round_trip_single_and_batched():
    p = _param(kwargs_lower_lens=[{"theta_E": 0.5}, {}], kwargs_upper_lens=[{"theta_E": 2.0}, {}])
    lo, hi = p.param_limits()
    assert (lo[0], hi[0]) == (0.5, 2.0)
    rng = np.random.default_rng(0)
    a = rng.uniform(lo, np.minimum(hi, lo + 1.0), size=(7, p.num_param()[0]))
    kw = p.args2kwargs(a)
    assert kw["kwargs_lens"][0]["center_x"] == 0.0            # fixed values stay scalars
    assert np.shape(kw["kwargs_lens"][0]["theta_E"]) == (7,)  # sampled values become arrays
    for j in range(7):
        kj = p.args2kwargs(a[j])
        np.testing.assert_array_equal(p.kwargs2args(kj["kwargs_lens"], kj["kwargs_source"],
                                                    kj["kwargs_lens_light"]), a[j])


def test_linear_solver_leaves_amplitudes_to_the_solve():
    p = S.Param(MODEL, kwargs_fixed_lens=FIXED_LENS)  # linear_solver=True, as in lenstronomy
    n, names = p.num_param()
    assert n == 4 + 2 + 6 + 4 and not any(nm.startswith("amp_") for nm in names)
    kw = p.args2kwargs(np.zeros(n))
    assert kw["kwargs_source"][0]["amp"] == 1.0 and kw["kwargs_lens_light"][0]["amp"] == 1.0


def test_param_rejects_unsupported():
    with pytest.raises(ValueError):
        S.Param(MODEL, linear_solver=False, kwargs_fixed_ps=[{"ra_image": [0.0]}])
    with pytest.raises(ValueError):
        S.Param(MODEL, linear_solver=False, joint_lens_with_light=[[0, 0, ["center_x"]]])
    with pytest.raises(ValueError):
        S.Param({"lens_model_list": ["SPEMD"]}, linear_solver=False)
    with pytest.raises(ValueError):
        _param().args2kwargs(np.zeros(3))


def test_check_bounds_and_prepare_errors():
    pen, hit = S.LikelihoodModule.check_bounds([0.0, 2.0], [0.0, 0.0], [1.0, 1.0])
    assert hit and pen == 1e5
    pen, hit = S.LikelihoodModule.check_bounds([0.5], [0.0], [1.0])
    assert not hit and pen == 0.0
    with pytest.raises(ValueError):
        S.prepare_logL_func("tpu", lambda a: 0.0)
    with pytest.raises(ValueError):
        S.prepare_logL_func("cpu", lambda a: 0.0)
    with pytest.raises(ValueError):
        S.prepare_logL_func("gpu", lambda a: 0.0)


def test_likelihood_module_rejects_unsupported_terms():
    p = _param()
    with pytest.raises(ValueError):
        S.LikelihoodModule({}, MODEL, p, time_delay_likelihood=True)
    with pytest.raises(ValueError):
        S.LikelihoodModule({}, MODEL, p, prior_lens_kde=[[0, "theta_E", [1.0]]])
    with pytest.raises(ValueError):
        S.ImageLikelihood([[{}, {}, {}]], "multi-linear", MODEL, linear_solver=False)
    with pytest.raises(ValueError):
        S.ImageLikelihood([[{}, {}, {}]], "single-band", MODEL, linear_prior=1.0)
    with pytest.raises(ValueError):
        S.ImageLikelihood([[{}, {}, {}]], "single-band", MODEL, source_marg=True,
                          linear_solver=False)


def test_param_point_sources_round_trip():
    """Point-source arguments (ra_image, dec_image per image; point_amp left to the
    linear solve) after the light profiles; batched args give (n, n_images) arrays."""
    from jaxtronomy_gb300.sampling import Param
    km = {"lens_model_list": ["SIE"], "source_light_model_list": ["SERSIC"],
          "lens_light_model_list": [], "point_source_model_list": ["LENSED_POSITION"]}
    lo = [{"ra_image": [-2.0] * 4, "dec_image": [-2.0] * 4}]
    hi = [{"ra_image": [2.0] * 4, "dec_image": [2.0] * 4}]
    p = Param(km, kwargs_fixed_lens=[{"center_x": 0.0, "center_y": 0.0}],
              kwargs_lower_ps=lo, kwargs_upper_ps=hi, num_point_source_list=[4])
    n, names = p.num_param()
    assert n == 3 + 4 + 8 and names[-8:] == ["ra_image"] * 4 + ["dec_image"] * 4
    a = np.random.default_rng(0).uniform(-1, 1, (3, n))
    kw = p.args2kwargs(a)
    assert kw["kwargs_ps"][0]["ra_image"].shape == (3, 4)
    np.testing.assert_array_equal(kw["kwargs_ps"][0]["point_amp"], np.ones(4))
    one = p.args2kwargs(a[1])
    np.testing.assert_array_equal(p.kwargs2args(one["kwargs_lens"], one["kwargs_source"],
                                                one["kwargs_lens_light"], one["kwargs_ps"]), a[1])
    lo_all, hi_all = p.param_limits()
    assert lo_all[-1] == -2.0 and hi_all[-1] == 2.0
    with pytest.raises(ValueError):
        Param(km, num_point_source_list=[4])          # sampled ps arrays need bounds
    p2 = Param(km, linear_solver=False, kwargs_lower_ps=[dict(lo[0], point_amp=[0.0] * 4)],
               kwargs_upper_ps=[dict(hi[0], point_amp=[10.0] * 4)], num_point_source_list=[4])
    assert p2.num_param()[0] == 5 + 5 + 12
