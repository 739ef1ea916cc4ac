"""Point-source rendering (oracle, FP64; test infrastructure).

Restates ``PointSourceRendering.point_source_rendering``
(``jaxtronomy/ImSim/Numerics/point_source_rendering.py:34-77``) with
``image_util.add_layer2image`` (``Util/image_util.py:9-40``) and
``image_util.re_size`` (``:78-98``), and ``ImageModel._displace_astrometry``
(``ImSim/image_model.py:652-676``).  The sub-pixel shift is
``jax.scipy.ndimage.map_coordinates`` with order 1 and mode ``"constant"``,
which JAX evaluates as linear interpolation with every corner outside the
kernel read as 0 (SciPy calls that mode ``"grid-constant"``); it is written
out here in that form.
"""

import numpy as np


def map_coordinates_linear(kernel, rows, cols):
    """Order-1 interpolation of ``kernel`` at (rows, cols), corners outside it = 0."""
    k = np.asarray(kernel, float)
    nr, nc = k.shape
    r0 = np.floor(rows)
    c0 = np.floor(cols)
    wr1 = rows - r0
    wc1 = cols - c0
    wr0 = 1 - wr1
    wc0 = 1 - wc1
    r0 = r0.astype(int)
    c0 = c0.astype(int)
    out = np.zeros(np.shape(rows))
    for dr, wr in ((0, wr0), (1, wr1)):
        for dc, wc in ((0, wc0), (1, wc1)):
            r = r0 + dr
            c = c0 + dc
            ok = (r >= 0) & (r < nr) & (c >= 0) & (c < nc)
            val = np.where(ok, k[np.clip(r, 0, nr - 1), np.clip(c, 0, nc - 1)], 0.0)
            out = out + wr * wc * val
    return out


def pixel_position(ra, dec, transform_pix2angle, ra_at_xy_0, dec_at_xy_0):
    """``util.map_coord2pix`` with lenstronomy ``PixelGrid``'s Ma2pix and the pixel
    position of (ra, dec) = (0, 0)."""
    M = np.linalg.inv(np.asarray(transform_pix2angle, float))
    x0, y0 = M.dot(np.array([-ra_at_xy_0, -dec_at_xy_0]))
    x, y = M.dot(np.array([np.asarray(ra, float), np.asarray(dec, float)]))
    return x + x0, y + y0


def render(nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0, ra, dec, amp, kernel,
           subgrid=1):
    """The (nx, ny) image of point images (ra, dec, amp), kernel at factor ``subgrid``."""
    x, y = pixel_position(ra, dec, transform_pix2angle, ra_at_xy_0, dec_at_xy_0)
    x = np.atleast_1d(x)
    y = np.atleast_1d(y)
    amp = np.atleast_1d(np.asarray(amp, float))
    p = int(subgrid)
    xs = x * p + (p - 1) / 2.0
    ys = y * p + (p - 1) / 2.0
    k = np.asarray(kernel, float)
    kr, kc = k.shape
    grid = np.zeros((nx * p, ny * p))
    n_row, n_col = grid.shape
    for i in range(len(x)):
        xr = np.arange(n_col) + kc // 2 - xs[i]
        yr = np.arange(n_row) + kr // 2 - ys[i]
        xg, yg = np.meshgrid(xr, yr)
        grid = map_coordinates_linear(amp[i] * k, yg, xg) + grid
    small = grid.reshape(nx, p, ny, p).mean(3).mean(1)
    return small * p ** 2


def displace_astrometry(ra, dec, kwargs_special=None):
    """``ImageModel._displace_astrometry``: add delta_x_image / delta_y_image to the
    first images."""
    ra = np.asarray(ra, float)
    dec = np.asarray(dec, float)
    if kwargs_special is not None and "delta_x_image" in kwargs_special:
        dx = np.zeros(len(ra))
        dy = np.zeros(len(dec))
        d = np.asarray(kwargs_special["delta_x_image"], float)
        dx[:len(d)] = d
        d = np.asarray(kwargs_special["delta_y_image"], float)
        dy[:len(d)] = d
        ra = ra + dx
        dec = dec + dy
    return ra, dec
