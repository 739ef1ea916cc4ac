"""Host-side logic without a GPU: kwargs packing, validation mirroring the
reference's construction-time errors, PSF kernels and workload generation."""

import numpy as np
import pytest

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import profiles, workloads as W


def _image_model(psf=None, numerics=None, lens=("EPL", "SHEAR"), src=("SERSIC_ELLIPSE",),
                 ll=("SERSIC_ELLIPSE",), n=32):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=100.0, background_rms=0.01, **g)
    psf = psf or J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, 0.05, 11))
    return J.ImageModel(data, psf, J.LensModel(list(lens)), J.LightModel(list(src)),
                        J.LightModel(list(ll)), kwargs_numerics=numerics)


def test_pack_params_layout_matches_header_order():
    im = _image_model()
    kl = [{"theta_E": 1.1, "gamma": 2.05, "e1": 0.1, "e2": -0.1, "center_x": 0.01,
           "center_y": 0.02}, {"gamma1": 0.03, "gamma2": -0.02}]
    ks = [{"amp": 10.0, "R_sersic": 0.2, "n_sersic": 2.0, "e1": 0.0, "e2": 0.1,
           "center_x": 0.0, "center_y": 0.05}]
    kll = [{"amp": 20.0, "R_sersic": 0.7, "n_sersic": 3.0, "e1": 0.05, "e2": 0.0,
            "center_x": 0.01, "center_y": 0.02}]
    rows = im.pack_params(kl, ks, kll)
    assert rows.shape == (1, 24)
    np.testing.assert_array_equal(rows[0, :6], [1.1, 2.05, 0.1, -0.1, 0.01, 0.02])
    np.testing.assert_array_equal(rows[0, 6:10], [0.03, -0.02, 0.0, 0.0])  # ra_0, dec_0 default
    np.testing.assert_array_equal(rows[0, 10:17], [10.0, 0.2, 2.0, 0.0, 0.1, 0.0, 0.05])


def test_pack_params_batched_kwargs():
    model, lens, src, ll, _ = W.batch_epl(batch=5, num_pix=20, kernel_size=5)
    im = _image_model()
    rows = im.pack_params(lens, src, ll)
    assert rows.shape == (5, 24)
    for i in range(5):
        r1 = im.pack_params(*[W.instance(k, i) for k in (lens, src, ll)])
        np.testing.assert_array_equal(rows[i], r1[0])


def test_missing_required_parameter_raises():
    im = _image_model()
    with pytest.raises(ValueError):
        im.pack_params([{"gamma": 2.0, "e1": 0, "e2": 0}, {"gamma1": 0, "gamma2": 0}],
                       [{"amp": 1, "R_sersic": 1, "n_sersic": 1, "e1": 0, "e2": 0}],
                       [{"amp": 1, "R_sersic": 1, "n_sersic": 1, "e1": 0, "e2": 0}])


def test_inconsistent_batch_raises():
    with pytest.raises(ValueError):
        profiles.batch_size([{"a": np.zeros(3)}, {"b": np.zeros(4)}])


def test_check_parameters_mirrors_reference():
    lm = J.LensModel(["SIE"])
    lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0, "center_y": 0}])
    with pytest.raises(ValueError):
        lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0}])
    with pytest.raises(ValueError):
        lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0, "center_y": 0,
                              "gamma": 2}])
    with pytest.raises(ValueError):
        J.LightModel(["SERSIC"]).check_parameters([])


def test_unsupported_profiles_and_options_raise_at_construction():
    with pytest.raises(ValueError):
        J.LensModel(["PEMD"])
    with pytest.raises(ValueError):
        J.LightModel(["SHAPELETS"])
    with pytest.raises(ValueError):
        J.LensModel(["SIE"], multi_plane=True)
    with pytest.raises(ValueError):
        _image_model(numerics={"compute_mode": "adaptive"})
    with pytest.raises(TypeError):
        _image_model(numerics={"supersampling_factor": 2.0})
    with pytest.raises(TypeError):
        _image_model(numerics={"not_a_key": 1})
    with pytest.raises(ValueError):
        _image_model(numerics={"precision": "fp16"})
    with pytest.raises(ValueError):
        J.PSF("PIXEL", kernel_point_source=np.ones((4, 4)))
    with pytest.raises(ValueError):
        J.PSF("GAUSSIAN")


def test_pixel_psf_is_normalised_and_gaussian_kernel_follows_reference_size():
    k = np.ones((5, 5))
    assert abs(J.PSF("PIXEL", kernel_point_source=k).kernel_point_source.sum() - 1) < 1e-15
    from jaxtronomy_gb300.image_model import gaussian_kernel
    # radius = max(round(sigma * truncation), 1), convolution.py:204-206
    assert gaussian_kernel(0.8493, 5.0).shape == (9, 9)
    assert gaussian_kernel(0.1, 2.0).shape == (3, 3)
    assert abs(gaussian_kernel(1.7, 4.0).sum() - 1) < 1e-14


def test_image_data_grid_attributes():
    g = W.grid_kwargs(60, 0.05)
    d = J.ImageData(np.zeros((60, 60)), exposure_time=100.0, background_rms=0.01, **g)
    assert d.num_pixel_axes == (60, 60)
    assert abs(d.pixel_width - 0.05) < 1e-15
    cx, cy = d.center
    assert abs(cx) < 1e-12 and abs(cy) < 1e-12
    x, y = d.map_coord2pix(*d.map_pix2coord(3.0, 7.0))
    assert abs(x - 3) < 1e-12 and abs(y - 7) < 1e-12
    # exposure floor (image_noise.py:52-54)
    d2 = J.ImageData(np.zeros((4, 4)), exposure_time=0.0, background_rms=0.1)
    assert d2.exposure_map == 1e-10


def test_workloads_are_seeded_and_shaped():
    a = W.batch_epl(batch=8, num_pix=20, kernel_size=5)
    b = W.batch_epl(batch=8, num_pix=20, kernel_size=5)
    np.testing.assert_array_equal(a[1][0]["theta_E"], b[1][0]["theta_E"])
    assert a[4].shape == (8, 5, 5)
    np.testing.assert_allclose(a[4].sum(axis=(1, 2)), 1.0, rtol=1e-14)
    sie = W.single_sie(batch=500)[1][0]
    assert np.hypot(sie["e1"], sie["e2"]).max() < 0.4
