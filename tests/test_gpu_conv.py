"""PSF convolution kernels through the C ABI (lensgb_convolve).

The FP32 zero-padded convolution stages its halo tiles with a TMA copy where the
images allow it (row pitch a multiple of 16 bytes, K <= 48) and with plain loads
otherwise; both sum every output's products in the same order, so the two paths
must agree bit for bit.  Both are checked against the FP64 direct convolution
(1e-5 of the image maximum: FP32 rounding of K^2-term sums of heavy-tailed test images) and against
scipy.signal.fftconvolve(mode="same"), the reference's operation
(convolution.py:74-86).  No CTA may give up its bounded wait for the copy.

The FP64 FFT path (convolution_method "fft"; under "auto" where a kernel is
too wide for the direct kernels' tile) is checked against fftconvolve, with
zero and with edge padding, and against the direct kernels on whole images.
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


def _method_model(n, K, precision, method, psf_type="PIXEL"):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    if psf_type == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=W.moffat_pixel_kernel(0.12, 3.0, 0.05, K))
    else:  # a GAUSSIAN model convolves with edge padding; K = 2 round(3 sigma) + 1
        psf = J.PSF("GAUSSIAN", fwhm=2.3548 * 0.05 * (K // 2) / 3.0, truncation=3.0)
    im = J.ImageModel(data, psf, J.LensModel(["SIE"]), J.LightModel(["SERSIC"]),
                      J.LightModel([]),
                      kwargs_numerics={"supersampling_factor": 1, "precision": precision,
                                       "convolution_method": method})
    return im._model(range(1), range(1), range(0))


@pytest.mark.parametrize("n,K", [(60, 11), (180, 31), (300, 41), (120, 61), (200, 99),
                                 (600, 165), (97, 7)])
@pytest.mark.parametrize("psf_type", ["PIXEL", "GAUSSIAN"])
def test_fft_convolution_matches_fftconvolve(cuda, n, K, psf_type):
    """The FP64 FFT path (fftconv.cu) against scipy.signal.fftconvolve(mode="same"),
    the reference's operation (after edge padding for a GAUSSIAN model,
    convolution.py:215-235), per-system kernels and one shared kernel, in both
    precisions (FP64: 1e-12 of the image maximum; FP32 images: 1e-6, their own
    rounding)."""
    rng = np.random.default_rng(n + K)
    B = 3
    img = rng.random((B, n, n)) * np.exp(rng.normal(0, 2, (B, n, n)))
    kern = np.stack([W.moffat_pixel_kernel(rng.uniform(0.08, 0.15) * K / 11,
                                           rng.uniform(2.5, 4.5), 0.05, K) for _ in range(B)])
    for prec, tol in (("fp64", 1e-12), ("fp32", 1e-6)):
        m = _method_model(n, K, prec, "fft", psf_type)
        assert m.desc.kernel_size == K
        dt = torch.float64 if prec == "fp64" else torch.float32
        x = torch.as_tensor(img, dtype=dt).cuda().contiguous()
        xs = x.double().cpu().numpy()
        for shared in (False, True):
            ks = kern[:1] if shared else kern
            k = torch.as_tensor(ks, dtype=dt).cuda().contiguous()
            out = torch.empty_like(x)
            _lib.check(_lib.load().lensgb_convolve(m.handle, _device.ptr(x), B, _device.ptr(k),
                                                   0 if shared else K * K, _device.ptr(out),
                                                   _device.stream_handle()))
            got = out.double().cpu().numpy()
            kd = k.double().cpu().numpy()
            for i in range(B):
                src = xs[i] if psf_type == "PIXEL" else np.pad(xs[i], K // 2, mode="edge")
                ref = scipy.signal.fftconvolve(src, kd[0 if shared else i], mode="same")
                if psf_type != "PIXEL":
                    ref = ref[K // 2:K // 2 + n, K // 2:K // 2 + n]
                assert np.abs(got[i] - ref).max() <= tol * np.abs(ref).max(), (prec, shared, i)


def test_fft_and_direct_images_agree(cuda):
    """Whole images (EPL + SHEAR, 120x120, s = 3, 31x31 kernels) by FFT and by the
    direct kernels: FP64 within 1e-10 per pixel above 1e-8 of the maximum,
    FP32 within the FP32 bar."""
    model, lens, src, ll, kern = W.batch_epl(seed=21, batch=4, num_pix=120, kernel_size=31)
    g = W.grid_kwargs(120, 0.04)
    for prec, tol, floor in (("fp64", 1e-10, 1e-8), ("fp32", 1e-5, 1e-3)):
        imgs = []
        for method in ("direct", "fft"):
            data = J.ImageData(np.zeros((120, 120)), exposure_time=1000.0, background_rms=0.01,
                               **g)
            im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                              J.LensModel(model["lens_model_list"]),
                              J.LightModel(model["source_light_model_list"]),
                              J.LightModel(model["lens_light_model_list"]),
                              kwargs_numerics={"supersampling_factor": 3, "precision": prec,
                                               "convolution_method": method})
            imgs.append(im.image_batch(lens, src, ll, psf_kernels=kern).double().cpu().numpy())
        a, b = imgs
        for i in range(4):
            scale = np.abs(a[i]).max()
            sig = np.abs(a[i]) >= floor * scale
            assert (np.abs(b[i] - a[i])[sig] / np.abs(a[i])[sig]).max() < tol, (prec, i)


def test_auto_convolution_uses_fft_where_direct_cannot_run(cuda):
    """A 165-pixel supersampled kernel (41 pixels at s = 4) does not fit the
    direct kernels' shared-memory tile: "direct" refuses it with a clear error,
    "auto" convolves it by FFT."""
    n, K = 300, 165
    rng = np.random.default_rng(3)
    x = torch.as_tensor(rng.random((1, n, n)), dtype=torch.float32).cuda().contiguous()
    k = torch.as_tensor(W.moffat_pixel_kernel(0.6, 3.0, 0.05, K)[None],
                        dtype=torch.float32).cuda().contiguous()
    out = torch.empty_like(x)
    lib = _lib.load()
    m = _method_model(n, K, "fp32", "direct")
    rc = lib.lensgb_convolve(m.handle, _device.ptr(x), 1, _device.ptr(k), 0, _device.ptr(out),
                             _device.stream_handle())
    assert rc == _lib.ERR_CUDA and b"shared-memory" in lib.lensgb_last_error()
    m = _method_model(n, K, "fp32", "auto")
    _lib.check(lib.lensgb_convolve(m.handle, _device.ptr(x), 1, _device.ptr(k), 0,
                                   _device.ptr(out), _device.stream_handle()))
    ref = scipy.signal.fftconvolve(x[0].double().cpu().numpy(), k[0].double().cpu().numpy(),
                                   mode="same")
    assert np.abs(out[0].double().cpu().numpy() - ref).max() <= 1e-6 * np.abs(ref).max()
