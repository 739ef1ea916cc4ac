"""Accuracy of the serving workload's lens stacks at its largest sizes.

The serving stream draws grids up to 300x300, supersampling up to 4 and PSF
kernels up to 41x41 over four lens stacks (SIE, EPL, EPL_MULTIPOLE_M1M3M4 and
NFW_ELLIPSE_CSE, each + SHEAR) with one or two sources.  Here:

  * the reference's own images of the four stacks with two sources at 100x100,
    s = 4, K = 41 (tests/golden/serving_scenes.npz) against the FP64 kernels
    (1e-10 relative per pixel) and against the FP32-split kernels, uniform and
    served through the mixed-grid server (1e-5 relative per pixel on pixels
    above 1e-3 of the image maximum, and 1e-5 of the maximum everywhere);
  * requests of every stack at 300x300, s = 4, K = 41 in FP32-split against
    the same requests in FP64 on the GPU, with the same FP32 bar.
"""

import numpy as np
import pytest

import golden_io
from jaxtronomy_gb300 import serving, workloads as W

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_RTOL = 1e-5
SCENES = golden_io.serving_scenes()


def rel_err(got, ref, floor_frac=1e-3):
    got = np.asarray(got, float)
    ref = np.asarray(ref, float)
    scale = np.abs(ref).max()
    sig = np.abs(ref) >= floor_frac * scale
    return (float((np.abs(got - ref)[sig] / np.abs(ref)[sig]).max()),
            float(np.abs(got - ref).max() / scale))


def _key(sc, side=None):
    return (side or sc["num_pix"], sc["s"], sc["kernel"].shape[0], sc["tag"], len(sc["src"]))


def _image(sc, precision, kernel=None):
    im = W.serving_model(_key(sc), precision=precision)
    out = im.image_batch(sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"],
                         psf_kernels=sc["kernel"] if kernel is None else kernel)
    return out[0].double().cpu().numpy()


@pytest.mark.parametrize("sc", SCENES, ids=lambda s: s["tag"])
def test_fp64_matches_reference_at_s4_k41(cuda, sc):
    pp, mx = rel_err(_image(sc, "fp64"), sc["image"], floor_frac=1e-8)
    assert pp < FP64_RTOL and mx < FP64_RTOL, (pp, mx)


@pytest.mark.parametrize("sc", SCENES, ids=lambda s: s["tag"])
def test_fp32_matches_reference_at_s4_k41(cuda, sc):
    pp, mx = rel_err(_image(sc, "fp32"), sc["image"])
    assert pp < FP32_RTOL and mx < FP32_RTOL, (pp, mx)


def test_served_fp32_matches_reference(cuda):
    """All four scenes served together through mixed-grid buckets."""
    with serving.Server(n_streams=2, max_batch=8, mixed_grids=2) as srv:
        built = []
        for sc in SCENES:
            im = W.serving_model(_key(sc), precision="fp32")
            built.append(srv.request(im, sc["kwargs_lens"], sc["kwargs_source"],
                                     sc["kwargs_lens_light"], psf_kernel=sc["kernel"]))
        tickets = srv.submit_requests(built)
        srv.drain(120)
        for sc, t in zip(SCENES, tickets):
            pp, mx = rel_err(t.result(), sc["image"])
            assert pp < FP32_RTOL and mx < FP32_RTOL, (sc["tag"], pp, mx)


@pytest.mark.parametrize("stack", W.SERVING_STACKS)
def test_fp32_vs_fp64_at_300_s4_k41(cuda, stack):
    reqs, psfs = W.serving_stream(seed=1002, n=2000)
    sample = [r for r in reqs if r["key"][3] == stack][:3]
    for r in sample:
        key = (300, 4, 41, stack, r["key"][4])
        kern = psfs[41][r["psf"]]
        imgs = {}
        for prec in ("fp32", "fp64"):
            im = W.serving_model(key, precision=prec)
            imgs[prec] = im.image_batch(r["kwargs_lens"], r["kwargs_source"],
                                        r["kwargs_lens_light"],
                                        psf_kernels=kern)[0].double().cpu().numpy()
        pp, mx = rel_err(imgs["fp32"], imgs["fp64"])
        assert pp < FP32_RTOL and mx < FP32_RTOL, (stack, r["key"], pp, mx)
