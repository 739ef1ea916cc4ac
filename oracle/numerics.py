"""PSF convolution classes of the numerics layer (oracle, FP64).

Follows ``jaxtronomy/ImSim/Numerics/convolution.py`` and
``jaxtronomy/ImSim/Numerics/numerics.py:102-177``.  ``jax.scipy.signal``'s
``fftconvolve(mode="same")`` / ``convolve2d(mode="same")`` (called at
``convolution.py:81,85``) are replaced by their SciPy equivalents, which share
the same "same"-mode centring and zero boundary.
"""

import numpy as np
from scipy import signal


def fwhm2sigma(fwhm):
    """``jaxtronomy/Util/util.py:56-63``."""
    return fwhm / (2 * np.sqrt(2 * np.log(2)))


def pixel_convolve(image, kernel, convolution_type="fft"):
    """``PixelKernelConvolution.convolution2d`` ``convolution.py:74-86``."""
    if convolution_type in ("fft", "fft_static"):
        return signal.fftconvolve(image, kernel, mode="same")
    if convolution_type == "grid":
        return signal.convolve2d(image, kernel, mode="same")
    raise ValueError("convolution_type %s not supported!" % convolution_type)


def gaussian_kernel(sigma_pix, truncation):
    """Kernel built by ``GaussianConvolution.__init__`` / ``pixel_kernel``
    (``convolution.py:199-206,254-273``): side 2*r+1 with
    r = max(round(sigma*truncation), 1), a unit-amplitude circular Gaussian on
    the centred integer grid, normalised to unit sum."""
    radius = max(round(sigma_pix * truncation), 1)
    num_pix = 2 * radius + 1
    c = np.arange(num_pix) - (num_pix - 1) / 2.0
    xx, yy = np.meshgrid(c, c)
    k = np.exp(-(xx ** 2 + yy ** 2) / (2 * sigma_pix ** 2)) / (2 * np.pi * sigma_pix ** 2)
    return k / np.sum(k), int(radius)


def gaussian_convolve(image, kernel, pad_width):
    """``GaussianConvolution.convolution2d`` ``convolution.py:215-235``: edge
    padding, FFT convolution, crop."""
    padded = np.pad(image, pad_width=pad_width, mode="edge")
    conv = signal.fftconvolve(padded, kernel, mode="same")
    return conv[pad_width:-pad_width, pad_width:-pad_width]


def normalize_pixel_kernel(kernel):
    """lenstronomy ``PSF`` (PIXEL) stores the kernel normalised to unit sum and
    requires odd axis lengths."""
    kernel = np.asarray(kernel, dtype=float)
    if kernel.shape[0] % 2 == 0 or kernel.shape[1] % 2 == 0:
        raise ValueError("kernel needs to have odd axis number")
    return kernel / np.sum(kernel)
