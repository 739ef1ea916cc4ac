"""The launch-shape autotuner (lensgb_model_autotune): it times every candidate
shape, keeps the fastest, and no shape changes any pixel (bit for bit)."""

import numpy as np
import pytest

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _model(precision, n=72, K=21):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    _, lens, src, ll, kern = W.batch_epl(seed=31, batch=48, num_pix=n, kernel_size=K)
    im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": 2, "precision": precision})
    return im, lens, src, ll, kern


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_autotune_keeps_results_and_picks_a_candidate(cuda, precision):
    im, lens, src, ll, kern = _model(precision)
    before = im.image_batch(lens, src, ll, psf_kernels=kern).cpu().numpy()
    res = im.autotune(lens, src, ll, psf_kernels=kern)
    assert res["ppt"] in (0, 1, 2, 4, 8)
    assert res["conv_tile_rows"] in ([0] + list(range(32, 65, 4)))
    if precision == "fp64":
        assert res["conv_tile_rows"] == 0
    assert 0 < res["ray_ms"] <= res["ray_ms_builtin"]
    assert 0 < res["conv_ms"] <= res["conv_ms_builtin"]
    after = im.image_batch(lens, src, ll, psf_kernels=kern).cpu().numpy()
    np.testing.assert_array_equal(after, before)


def test_every_launch_shape_gives_the_same_pixels(cuda):
    im, lens, src, ll, kern = _model("fp32", n=61, K=31)
    ref = im.image_batch(lens, src, ll, psf_kernels=kern).cpu().numpy()
    for ppt, rows in ((1, 32), (2, 44), (4, 60), (8, 64), (0, 0)):
        im.set_tuning(ppt, rows)
        got = im.image_batch(lens, src, ll, psf_kernels=kern).cpu().numpy()
        np.testing.assert_array_equal(got, ref)
    with pytest.raises(Exception):
        im.set_tuning(3, 0)
