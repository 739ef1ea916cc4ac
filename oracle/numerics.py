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


def cut_psf(kernel, size):
    """Centred odd-size cut without renormalisation (lenstronomy
    ``kernel_util.cut_psf(..., normalisation=False)``, called at numerics.py:210)."""
    n = kernel.shape[0]
    if size >= n:
        return np.array(kernel, dtype=float)
    c = n // 2
    h = size // 2
    return np.array(kernel[c - h:c + h + 1, c - h:c + h + 1], dtype=float)


def split_kernel(kernel_super, supersampling_kernel_size, supersampling_factor):
    """Split of a supersampled kernel into the part convolved on the supersampled
    grid and the part convolved on the pixel grid (the role of lenstronomy's
    ``kernel_util.split_kernel``, called at convolution.py:123-127; restated
    here from that role, not from lenstronomy's code, so parity with lenstronomy
    itself is unpinned):

    * high-resolution part: the central n x n block of the supersampled kernel,
      n = supersampling_kernel_size * s (made odd, at most the kernel side);
    * pixel-scale part: the supersampled kernel with that block set to zero,
      summed over s x s blocks aligned on the kernel centre (the kernel is
      zero-padded symmetrically to a whole number of blocks).

    Both parts keep the supersampled kernel's normalisation, so together they
    carry its total weight.  Odd supersampling factors only (an even factor
    puts the kernel centre on a block boundary)."""
    s = int(supersampling_factor)
    if s <= 1:
        raise ValueError("a kernel split needs supersampling_factor > 1")
    if s % 2 == 0:
        raise ValueError("a kernel split needs an odd supersampling factor")
    k = np.asarray(kernel_super, dtype=float)
    n_super = k.shape[0]
    n_sub = supersampling_kernel_size * s
    if n_sub % 2 == 0:
        n_sub += 1
    n_sub = min(n_sub, n_super)
    i0 = (n_super - n_sub) // 2
    high = k[i0:i0 + n_sub, i0:i0 + n_sub].copy()
    hole = k.copy()
    hole[i0:i0 + n_sub, i0:i0 + n_sub] = 0.0
    n_low = -(-n_super // s)
    if n_low % 2 == 0:
        n_low += 1
    pad = (n_low * s - n_super) // 2
    big = np.zeros((n_low * s, n_low * s))
    big[pad:pad + n_super, pad:pad + n_super] = hole
    low = big.reshape(n_low, s, n_low, s).sum(axis=(1, 3))
    return low, high
