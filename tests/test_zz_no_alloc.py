"""lensgb_image_noalloc: the image entry point that allocates no device memory.

Callers that cannot allocate on the call path -- e.g. a handler running inside
an XLA/JAX program, where XLA has reserved most of the GPU memory for its own
pool -- use this variant; its scratch is a fixed array inside the library.
These tests call it through the C ABI and check that two calls in a row give
the same images as lensgb_image (within the parity tolerances used by the
other GPU tests), also when the second call has fewer systems and other
parameters than the first (nothing of the first call may leak into it), that a
call needing more scratch than the fixed array is refused with a clear error,
and that the two refused model kinds (convolution on the supersampled grid,
sub-frames) are refused with LENSGB_ERR_UNSUPPORTED, while an unconvolved call
of a supersampled-convolution model still works.

This file is named so that pytest collects it last.
"""

import ctypes

import numpy as np
import pytest
import torch

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import _device, _lib, workloads as W

pytestmark = pytest.mark.gpu


def _setup(precision, batch, num_pix=60, s=3, K=21, seed=33):
    model, lens, src, ll, kern = W.batch_epl(seed=seed, batch=batch, num_pix=num_pix,
                                             supersampling=s, kernel_size=K)
    g = W.grid_kwargs(num_pix, 0.04)
    data = J.ImageData(np.zeros((num_pix, num_pix)), exposure_time=1000.0, background_rms=0.01,
                       **g)
    im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(model["lens_model_list"]),
                      J.LightModel(model["source_light_model_list"]),
                      J.LightModel(model["lens_light_model_list"]),
                      kwargs_numerics={"supersampling_factor": s, "precision": precision})
    dtype = torch.float64 if precision == "fp64" else torch.float32
    rows = torch.as_tensor(im.pack_params(lens, src, ll)).cuda()
    psf = torch.as_tensor(kern, dtype=dtype).cuda().contiguous()
    m = im._model(range(2), range(1), range(1))
    return im, m, rows, psf, dtype, K


def _call(fn, m, rows, psf, K, out):
    B = rows.shape[0]
    _lib.check(fn(m.handle, _device.ptr(rows), B, _device.ptr(psf), K * K, _device.ptr(out), 0,
                  _device.stream_handle()))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_noalloc_matches_image_on_two_calls(cuda, precision, tol):
    lib = _lib.load()
    im, m, rows, psf, dtype, K = _setup(precision, batch=6)
    B, n = rows.shape[0], 60
    ref = torch.empty((B, n, n), dtype=dtype, device="cuda")
    _call(lib.lensgb_image, m, rows, psf, K, ref)
    for _ in range(2):
        out = torch.full((B, n, n), float("nan"), dtype=dtype, device="cuda")
        _call(lib.lensgb_image_noalloc, m, rows, psf, K, out)
        torch.cuda.synchronize()
        a = out.double().cpu().numpy()
        b = ref.double().cpu().numpy()
        assert np.all(np.isfinite(a))
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= tol, err


def test_noalloc_refuses_oversized_call(cuda):
    lib = _lib.load()
    # FP64 180x180 needs ~268 KB of scratch per system: 300 systems exceed 64 MiB
    im, m, rows, psf, dtype, K = _setup("fp64", batch=1, num_pix=180, s=1, K=5)
    rows_big = rows.repeat(300, 1).contiguous()
    out = torch.empty((300, 180, 180), dtype=dtype, device="cuda")
    rc = lib.lensgb_image_noalloc(m.handle, _device.ptr(rows_big), 300, _device.ptr(psf), 0,
                                  _device.ptr(out), 0, _device.stream_handle())
    assert rc == _lib.ERR_INVALID
    msg = lib.lensgb_last_error().decode()
    assert "bytes of scratch" in msg and str(64 << 20) in msg


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_noalloc_second_call_smaller_with_other_parameters(cuda, precision, tol):
    """Six systems, then three systems of another seed: the second call must
    match lensgb_image on its own inputs (records, EPL tables and the FP32
    refine list of the first call must not leak into it)."""
    lib = _lib.load()
    n = 60
    for batch, seed in ((6, 33), (3, 77)):
        im, m, rows, psf, dtype, K = _setup(precision, batch=batch, seed=seed)
        ref = torch.empty((batch, n, n), dtype=dtype, device="cuda")
        _call(lib.lensgb_image, m, rows, psf, K, ref)
        out = torch.full((batch, n, n), float("nan"), dtype=dtype, device="cuda")
        _call(lib.lensgb_image_noalloc, m, rows, psf, K, out)
        torch.cuda.synchronize()
        a = out.double().cpu().numpy()
        b = ref.double().cpu().numpy()
        assert np.all(np.isfinite(a))
        err = np.abs(a - b).max() / np.abs(b).max()
        assert err <= tol, (batch, seed, err)


def _model_with(numerics, precision="fp64", num_pix=30, s=3):
    model, lens, src, ll, kern = W.batch_epl(seed=5, batch=2, num_pix=num_pix,
                                             supersampling=s, kernel_size=9)
    g = W.grid_kwargs(num_pix, 0.05)
    data = J.ImageData(np.zeros((num_pix, num_pix)), exposure_time=1000.0,
                       background_rms=0.01, **g)
    if numerics.get("supersampling_convolution"):
        psf = J.PSF("PIXEL", kernel_point_source=W.moffat_pixel_kernel(0.12, 3.0, 0.05 / s, 15),
                    point_source_supersampling_factor=s)
    else:
        psf = J.PSF("PIXEL", kernel_point_source=kern[0])
    im = J.ImageModel(data, psf, J.LensModel(model["lens_model_list"]),
                      J.LightModel(model["source_light_model_list"]),
                      J.LightModel(model["lens_light_model_list"]),
                      kwargs_numerics=dict({"supersampling_factor": s, "precision": precision},
                                           **numerics))
    rows = torch.as_tensor(im.pack_params(lens, src, ll)).cuda()
    psf_t = im._kernel_tensor()
    return im, im._model(range(2), range(1), range(1)), rows, psf_t


def test_noalloc_refuses_supersampled_convolution_and_subframes(cuda):
    lib = _lib.load()
    yy, xx = np.mgrid[0:30, 0:30]
    fei = (yy - 14) ** 2 + (xx - 15) ** 2 <= 64
    for numerics in ({"supersampling_convolution": True}, {"flux_evaluate_indexes": fei}):
        im, m, rows, psf = _model_with(numerics)
        out = torch.empty((2, 30, 30), dtype=torch.float64, device="cuda")
        rc = lib.lensgb_image_noalloc(m.handle, _device.ptr(rows), 2, _device.ptr(psf), 0,
                                      _device.ptr(out), 0, _device.stream_handle())
        assert rc == _lib.ERR_UNSUPPORTED, numerics
        msg = lib.lensgb_last_error().decode()
        assert "supersampled convolution" in msg and "sub-frames" in msg


def test_noalloc_unconvolved_call_of_supersampled_convolution_model(cuda):
    lib = _lib.load()
    im, m, rows, psf = _model_with({"supersampling_convolution": True})
    ref = torch.empty((2, 30, 30), dtype=torch.float64, device="cuda")
    out = torch.full((2, 30, 30), float("nan"), dtype=torch.float64, device="cuda")
    for fn, o in ((lib.lensgb_image, ref), (lib.lensgb_image_noalloc, out)):
        _lib.check(fn(m.handle, _device.ptr(rows), 2, ctypes.c_void_p(0), 0, _device.ptr(o),
                      _lib.UNCONVOLVED, _device.stream_handle()))
    torch.cuda.synchronize()
    a, b = out.cpu().numpy(), ref.cpu().numpy()
    assert np.all(np.isfinite(a))
    assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
