"""Pixel grid, supersampled ray grid and re-binning (oracle, FP64).

Follows ``jaxtronomy/ImSim/Numerics/grid.py:22-148`` and
``jaxtronomy/Util/image_util.py:79-98``.  The grid construction itself lives in
lenstronomy (``Coordinates1D.coordinate_grid`` and ``util.make_subgrid``, called
at ``grid.py:48,60``); it is restated here from lenstronomy's documented
behaviour:

* pixel (row i, column j) sits at
  ``ra = ra_at_xy_0 + j*M[0,0] + i*M[0,1]``,
  ``dec = dec_at_xy_0 + j*M[1,0] + i*M[1,1]``; arrays are flattened row-major
  (column index fastest);
* sub-pixel (si, sj) of a pixel is displaced by
  ``(-1/2 + (2*sj+1)/(2*s))`` columns and ``(-1/2 + (2*si+1)/(2*s))`` rows,
  i.e. the supersampled array position (I, J) = (i*s+si, j*s+sj) sits at
  ``ra_at_xy_0 + M[0,0]*((J+1/2)/s - 1/2) + M[0,1]*((I+1/2)/s - 1/2)``.
"""

import numpy as np


def pixel_coordinates(nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0):
    """1d ra/dec of the pixel centres, row-major (lenstronomy
    ``Coordinates1D.coordinate_grid``, called at ``grid.py:48``)."""
    m = np.asarray(transform_pix2angle, dtype=float)
    j, i = np.meshgrid(np.arange(nx), np.arange(ny))
    j = j.ravel().astype(float)
    i = i.ravel().astype(float)
    ra = j * m[0, 0] + i * m[0, 1] + ra_at_xy_0
    dec = j * m[1, 0] + i * m[1, 1] + dec_at_xy_0
    return ra, dec


def supersampled_coordinates(nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0, s):
    """1d ra/dec of the (ny*s, nx*s) supersampled ray grid, row-major
    (``RegularGrid.__init__`` ``grid.py:48-64`` with lenstronomy
    ``util.make_subgrid``).  For s == 1 this is the pixel grid itself."""
    ra, dec = pixel_coordinates(nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0)
    if s == 1:
        return ra, dec
    m = np.asarray(transform_pix2angle, dtype=float)
    ra2 = ra.reshape(ny, nx)
    dec2 = dec.reshape(ny, nx)
    out_ra = np.zeros((ny * s, nx * s))
    out_dec = np.zeros((ny * s, nx * s))
    for si in range(s):
        fy = -0.5 + 1.0 / (2.0 * s) + si / float(s)
        for sj in range(s):
            fx = -0.5 + 1.0 / (2.0 * s) + sj / float(s)
            out_ra[si::s, sj::s] = ra2 + m[0, 0] * fx + m[0, 1] * fy
            out_dec[si::s, sj::s] = dec2 + m[1, 0] * fx + m[1, 1] * fy
    return out_ra.ravel(), out_dec.ravel()


def array2image(array, nx, ny):
    """``jaxtronomy/Util/util.py:19-37`` (reshape to (ny, nx))."""
    return np.reshape(array, (ny, nx))


def re_size(image, factor):
    """s x s block mean, ``jaxtronomy/Util/image_util.py:79-98``: reshape to
    [n/f, f, m/f, f], mean over axis 3, then axis 1."""
    if factor < 1:
        raise ValueError("scaling factor in re-sizing %s < 1" % factor)
    if factor == 1:
        return image
    f = int(factor)
    nx, ny = image.shape
    if nx % f or ny % f:
        raise ValueError("scaling with factor %s is not possible with grid size %s, %s" % (f, nx, ny))
    return image.reshape([nx // f, f, ny // f, f]).mean(3).mean(1)


def pixel_width(transform_pix2angle):
    """lenstronomy ``PixelGrid.pixel_width``: sqrt(|det M|)."""
    m = np.asarray(transform_pix2angle, dtype=float)
    return float(np.sqrt(abs(np.linalg.det(m))))
