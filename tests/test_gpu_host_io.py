"""lensgb_image_host (host rows / PSFs / images, chunked compute with the image
copies overlapped on a second stream): every image equals lensgb_image's, bit
for bit, for any chunking, PSF layout, precision and pinned or pageable
buffers."""

import ctypes

import numpy as np
import pytest
import torch

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def _model(precision, psf_type="PIXEL", n=40, K=11, s=2, ssc=False):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
    _, lens, src, ll, kern = W.batch_epl(seed=41, batch=7, num_pix=n, kernel_size=K)
    if psf_type == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=kern[0])
    elif psf_type == "GAUSSIAN":
        psf = J.PSF("GAUSSIAN", fwhm=0.12, truncation=3)
    else:
        psf = J.PSF("NONE")
    kn = {"supersampling_factor": s, "precision": precision}
    if ssc:
        kn.update(supersampling_convolution=True, supersampling_kernel_size=3)
        psf = J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, 0.05 / s, K * s + 1 - (K * s) % 2),
                    point_source_supersampling_factor=s)
    im = J.ImageModel(data, psf, J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      J.LightModel(["SERSIC_ELLIPSE"]), kwargs_numerics=kn)
    return im, im.pack_params(lens, src, ll), kern


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("psf_mode", ["default", "shared", "per_system", "gaussian", "none"])
@pytest.mark.parametrize("pinned", [True, False])
def test_host_call_equals_device_call(cuda, precision, psf_mode, pinned):
    psf_type = {"gaussian": "GAUSSIAN", "none": "NONE"}.get(psf_mode, "PIXEL")
    im, rows, kern = _model(precision, psf_type)
    dt = torch.float32 if precision == "fp32" else torch.float64
    kk = {"default": None, "shared": kern[3], "per_system": kern}.get(psf_mode)
    ref = im.image_batch(rows=rows, psf_kernels=None if kk is None else torch.as_tensor(kk).cuda())
    out = torch.empty((7, 40, 40), dtype=dt, pin_memory=pinned)
    rows_h = torch.as_tensor(rows)
    rows_h = rows_h.pin_memory() if pinned else rows_h
    k_h = None if kk is None else torch.as_tensor(kk)
    im.image_batch(rows=rows_h, psf_kernels=k_h, out=out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.numpy(), ref.cpu().numpy())


@pytest.mark.parametrize("n_chunks", [1, 2, 3, 7, 16])
def test_any_chunking_gives_the_same_images(cuda, n_chunks):
    im, rows, kern = _model("fp32")
    ref = im.image_batch(rows=rows, psf_kernels=torch.as_tensor(kern).cuda()).cpu().numpy()
    out = torch.empty((7, 40, 40), dtype=torch.float32, pin_memory=True)
    k_h = torch.as_tensor(kern, dtype=torch.float32).contiguous()
    rows_h = torch.as_tensor(rows).contiguous()
    model = im._model(range(2), range(1), range(1))
    stream = torch.cuda.current_stream()
    _lib.check(_lib.load().lensgb_image_host(
        model.handle, ctypes.c_void_p(rows_h.data_ptr()), 7, ctypes.c_void_p(k_h.data_ptr()),
        11 * 11, ctypes.c_void_p(out.data_ptr()), 0, n_chunks, ctypes.c_void_p(stream.cuda_stream)))
    _lib.check(_lib.load().lensgb_image_host_wait(model.handle, ctypes.c_void_p(stream.cuda_stream)))
    stream.synchronize()
    np.testing.assert_array_equal(out.numpy(), ref)


def test_back_to_back_host_calls_keep_every_result(cuda):
    """Calls whose copies overlap the next call: alternate device slots keep each
    call's images intact until they have been copied."""
    im, rows, kern = _model("fp32")
    refs, outs = [], []
    for j in range(5):
        r = rows.copy()
        r[:, 0] *= 1.0 + 0.01 * j   # a different theta_E per call
        refs.append(im.image_batch(rows=r).cpu().numpy())
        outs.append(torch.empty((7, 40, 40), dtype=torch.float32, pin_memory=True))
    for j in range(5):
        r = rows.copy()
        r[:, 0] *= 1.0 + 0.01 * j
        im.image_batch(rows=torch.as_tensor(r).pin_memory(), out=outs[j])
    im.host_wait()
    torch.cuda.current_stream().synchronize()
    for j in range(5):
        np.testing.assert_array_equal(outs[j].numpy(), refs[j])


def test_host_call_supersampled_convolution(cuda):
    im, rows, _ = _model("fp32", ssc=True, K=5, s=3)
    ref = im.image_batch(rows=rows).cpu().numpy()
    out = torch.empty((7, 40, 40), dtype=torch.float32, pin_memory=True)
    im.image_batch(rows=torch.as_tensor(rows), out=out)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.numpy(), ref)
