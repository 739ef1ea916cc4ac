"""Systems on different pixel grids and PSF sizes in one launch sequence
(lensgb_image_mixed through the C ABI): every image must equal that system
computed alone by its own ImageModel: bit for bit in FP64; in FP32 within the
FP32 bar, 1e-5 of the image maximum, because the mixed launch runs its own
compiled instantiation of the FP32 ray kernel, whose FMA contractions may round
a few pixels differently by an ulp or two (and so flip a pixel's FP64
refinement).  Within the mixed path a
system's image does not depend on what else shares the launch: bit for bit in
both precisions."""

import numpy as np
import pytest

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W
from jaxtronomy_gb300.image_model import image_mixed

pytestmark = pytest.mark.gpu


def _model(n, dpix, K, s, precision, psf_type="PIXEL", lens=("EPL", "SHEAR")):
    g = W.grid_kwargs(n, dpix)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    if psf_type == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, dpix, K))
    elif psf_type == "GAUSSIAN":
        psf = J.PSF("GAUSSIAN", fwhm=0.02 * K, truncation=3)
    else:
        psf = J.PSF("NONE")
    return J.ImageModel(data, psf, J.LensModel(list(lens)), J.LightModel(["SERSIC_ELLIPSE"]),
                        J.LightModel(["SERSIC_ELLIPSE"]),
                        kwargs_numerics={"supersampling_factor": s, "precision": precision})


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("psf_type", ["PIXEL", "GAUSSIAN", "NONE"])
@pytest.mark.parametrize("mixed_s", [False, True])
def test_mixed_batch_equals_alone(cuda, precision, psf_type, mixed_s):
    """mixed_s: the systems also differ in supersampling (the run-time-s ray
    kernel and the per-pixel refine pass)."""
    shapes = [(24, 0.05, 5), (40, 0.04, 11), (33, 0.06, 21), (17, 0.05, 41), (64, 0.03, 9),
              (40, 0.04, 11)]
    sups = [1, 2, 3, 4, 2, 1] if mixed_s else [2] * len(shapes)
    _, lens, src, ll, _ = W.batch_epl(seed=21, batch=len(shapes), num_pix=24, kernel_size=5)
    reqs, alone = [], []
    rng = np.random.default_rng(4)
    for i, (n, d, K) in enumerate(shapes):
        im = _model(n, d, K, sups[i], precision, psf_type)
        kl, ks, kll = W.instance(lens, i), W.instance(src, i), W.instance(ll, i)
        psf = None
        if psf_type == "PIXEL" and i % 2:
            psf = W.moffat_pixel_kernel(0.1 + 0.01 * rng.random(), 3.0, d, K)
        req = (im, kl, ks, kll) if psf is None else (im, kl, ks, kll, psf)
        reqs.append(req)
        alone.append(im.image_batch(kl, ks, kll, psf_kernels=psf)[0].cpu().numpy())
    got = image_mixed(reqs)
    assert len(got) == len(shapes)
    for g, a, (n, _, _) in zip(got, alone, shapes):
        assert g.shape == (n, n)
        g = g.cpu().numpy()
        if precision == "fp64":
            np.testing.assert_array_equal(g, a)
        else:
            np.testing.assert_allclose(g, a, rtol=0, atol=1e-5 * np.abs(a).max())
    # each system alone through the mixed path: the same bits as in the mix
    for req, g in zip(reqs, got):
        np.testing.assert_array_equal(image_mixed([req])[0].cpu().numpy(), g.cpu().numpy())


def test_mixed_rejects_different_stacks(cuda):
    a = _model(24, 0.05, 5, 2, "fp32")
    b = _model(24, 0.05, 5, 2, "fp32", lens=("SIE", "SHEAR"))
    _, lens, src, ll, _ = W.batch_epl(seed=1, batch=1, num_pix=24, kernel_size=5)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    kls = [{"theta_E": 1.0, "e1": 0.0, "e2": 0.0, "center_x": 0.0, "center_y": 0.0}, kl[1]]
    with pytest.raises(ValueError):
        image_mixed([(a, kl, ks, kll), (b, kls, ks, kll)])
