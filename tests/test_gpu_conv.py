"""PSF convolution kernels through the C ABI (lensgb_convolve).

The FP32 zero-padded convolution stages its halo tiles with a TMA copy where the
images allow it (row pitch a multiple of 16 bytes, K <= 48) and with plain loads
otherwise; both sum every output's products in the same order, so the two paths
must agree bit for bit.  Both are checked against the FP64 direct convolution
(1e-5 of the image maximum: FP32 rounding of K^2-term sums of heavy-tailed test images) and against
scipy.signal.fftconvolve(mode="same"), the reference's operation
(convolution.py:74-86).  No CTA may give up its bounded wait for the copy.
"""

import ctypes

import numpy as np
import pytest
import scipy.signal
import torch

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import _device, _lib, workloads as W

pytestmark = pytest.mark.gpu


def _model(n, K, precision):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    kern = W.moffat_pixel_kernel(0.12, 3.0, 0.05, K)
    psf = J.PSF("PIXEL", kernel_point_source=kern)
    im = J.ImageModel(data, psf, J.LensModel(["SIE"]),
                      J.LightModel(["SERSIC"]), J.LightModel([]),
                      kwargs_numerics={"supersampling_factor": 1, "precision": precision})
    return im, im._model(range(1), range(1), range(0))


def _convolve(m, img, psf, K):
    out = torch.empty_like(img)
    _lib.check(_lib.load().lensgb_convolve(m.handle, _device.ptr(img), img.shape[0],
                                           _device.ptr(psf), K * K, _device.ptr(out),
                                           _device.stream_handle()))
    torch.cuda.synchronize()
    return out


@pytest.mark.parametrize("n,K", [(180, 31), (180, 11), (100, 21), (60, 41), (300, 41),
                                 (64, 5), (90, 31), (45, 9)])
def test_tma_and_plain_halo_fill_agree_bitwise(cuda, n, K):
    lib = _lib.load()
    rng = np.random.default_rng(n * 100 + K)
    B = 5
    img64 = rng.random((B, n, n)) * np.exp(rng.normal(0, 3, (B, n, n)))
    kern = np.stack([W.moffat_pixel_kernel(rng.uniform(0.08, 0.15), rng.uniform(2.5, 4.5),
                                           0.05, K) for _ in range(B)])
    _, m32 = _model(n, K, "fp32")
    img = torch.as_tensor(img64, dtype=torch.float32).cuda().contiguous()
    psf = torch.as_tensor(kern, dtype=torch.float32).cuda().contiguous()
    try:
        lib.lensgb_set_conv_tma(1)
        a = _convolve(m32, img, psf, K)
        lib.lensgb_set_conv_tma(0)
        b = _convolve(m32, img, psf, K)
    finally:
        lib.lensgb_set_conv_tma(1)
    assert torch.equal(a, b)
    # against the FP64 kernel and against the reference's operation
    _, m64 = _model(n, K, "fp64")
    c = _convolve(m64, torch.as_tensor(img.double()).contiguous(),
                  torch.as_tensor(kern).cuda().contiguous(), K).cpu().numpy()
    a = a.double().cpu().numpy()
    for i in range(B):
        ref = scipy.signal.fftconvolve(img[i].double().cpu().numpy(), kern[i], mode="same")
        scale = np.abs(ref).max()
        assert np.abs(c[i] - ref).max() <= 1e-12 * scale
        assert np.abs(a[i] - c[i]).max() <= 1e-5 * scale
    cnt = ctypes.c_uint(0)
    _lib.check(lib.lensgb_wait_timeouts(ctypes.byref(cnt)))
    assert cnt.value == 0
