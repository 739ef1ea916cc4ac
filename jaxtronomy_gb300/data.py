"""Data and PSF classes with the attributes ImageModel uses.

``ImageData`` mirrors ``jaxtronomy/Data/imaging_data.py:50-182`` together with
the lenstronomy ``PixelGrid`` attributes it inherits (pixel_width,
num_pixel_axes, transform_pix2angle, radec_at_xy_0, center, width,
map_pix2coord) and ``ImageNoise`` (``jaxtronomy/Data/image_noise.py:16-137``).
``PSF`` mirrors the lenstronomy PSF attributes read at ``numerics.py:78,104,118,128-132``
and ``image_model.py:64,132``.  These are host-side containers; the likelihood
itself is evaluated on the GPU by :class:`jaxtronomy_gb300.ImageModel`.
"""

import numpy as np


class PixelGrid:
    """Regular pixel grid: pixel (x=column, y=row) maps to
    ``ra = ra_at_xy_0 + M[0,0] x + M[0,1] y``, ``dec = dec_at_xy_0 + M[1,0] x + M[1,1] y``."""

    def __init__(self, nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0,
                 antenna_primary_beam=None):
        self._nx = int(nx)
        self._ny = int(ny)
        self._M = np.asarray(transform_pix2angle, dtype=float)
        self._Minv = np.linalg.inv(self._M)
        self._ra_at_xy_0 = float(ra_at_xy_0)
        self._dec_at_xy_0 = float(dec_at_xy_0)
        self._pb = antenna_primary_beam

    @property
    def num_pixel_axes(self):
        return self._nx, self._ny

    @property
    def num_pixel(self):
        return self._nx * self._ny

    @property
    def transform_pix2angle(self):
        return self._M

    @property
    def transform_angle2pix(self):
        return self._Minv

    @property
    def radec_at_xy_0(self):
        return self._ra_at_xy_0, self._dec_at_xy_0

    @property
    def pixel_width(self):
        return float(np.sqrt(abs(np.linalg.det(self._M))))

    @property
    def width(self):
        return self.pixel_width * np.array([self._nx, self._ny])

    def map_pix2coord(self, x, y):
        ra = x * self._M[0, 0] + y * self._M[0, 1] + self._ra_at_xy_0
        dec = x * self._M[1, 0] + y * self._M[1, 1] + self._dec_at_xy_0
        return ra, dec

    def map_coord2pix(self, ra, dec):
        d = np.array([np.asarray(ra) - self._ra_at_xy_0, np.asarray(dec) - self._dec_at_xy_0])
        x, y = np.tensordot(self._Minv, d, axes=1)
        return x, y

    @property
    def center(self):
        return self.map_pix2coord((self._nx - 1) / 2.0, (self._ny - 1) / 2.0)

    @property
    def primary_beam(self):
        return self._pb

    def pixel_coordinates(self):
        """2d ra, dec arrays of the pixel centres, shape (ny, nx)."""
        x, y = np.meshgrid(np.arange(self._nx), np.arange(self._ny))
        return self.map_pix2coord(x.astype(float), y.astype(float))


def covariance_matrix(data, background_rms, exposure_map):
    """``image_noise.py:115-137``."""
    d_pos = np.where(data >= 0, data, 0)
    return d_pos / exposure_map + background_rms ** 2


class ImageData(PixelGrid):
    """Imaging data: grid, pixel values and noise model (``imaging_data.py:50-133``)."""

    def __init__(self, image_data, exposure_time=None, background_rms=None, noise_map=None,
                 gradient_boost_factor=None, ra_at_xy_0=0, dec_at_xy_0=0,
                 transform_pix2angle=None, ra_shift=0, dec_shift=0, phi_rot=0,
                 log_likelihood_constant=0, antenna_primary_beam=None,
                 likelihood_method="diagonal", flux_scaling=1):
        if antenna_primary_beam is not None:
            raise ValueError("primary beam is not supported")
        image_data = np.asarray(image_data, dtype=float)
        nx, ny = np.shape(image_data)
        if transform_pix2angle is None:
            transform_pix2angle = np.array([[1, 0], [0, 1]])
        cos_phi, sin_phi = np.cos(phi_rot), np.sin(phi_rot)
        rot = np.array([[cos_phi, -sin_phi], [sin_phi, cos_phi]])
        PixelGrid.__init__(self, nx, ny, np.dot(transform_pix2angle, rot),
                           ra_at_xy_0 + ra_shift, dec_at_xy_0 + dec_shift)
        # ImageNoise (image_noise.py:16-97)
        if exposure_time is None:
            if noise_map is None:
                raise ValueError("Exposure map has not been specified in Noise() class!")
            self.exposure_map = None
        else:
            et = np.asarray(exposure_time, dtype=float)
            self.exposure_map = np.where(et <= 10 ** (-10), 10 ** (-10), et)
        if background_rms is None:
            if noise_map is None:
                raise ValueError("rms background value as 'background_rms' not specified!")
            self.background_rms = float(np.median(noise_map))
        else:
            self.background_rms = background_rms
        if gradient_boost_factor is not None:
            raise ValueError("gradient_boost_factor is not supported")
        self.data = image_data
        self.flux_scaling = flux_scaling
        if noise_map is not None:
            assert np.shape(noise_map) == np.shape(image_data)
            self._noise_map = np.asarray(noise_map, dtype=float)
            self.C_D = self._noise_map ** 2
        else:
            self._noise_map = None
            self.C_D = covariance_matrix(self.data, self.background_rms, self.exposure_map)
        if likelihood_method not in ("diagonal", "interferometry_natwt"):
            raise ValueError("likelihood_method %s not supported! likelihood_method can only be "
                             "'diagonal' or 'interferometry_natwt'!" % likelihood_method)
        if likelihood_method != "diagonal":
            raise ValueError("only the 'diagonal' likelihood method is supported")
        self._logL_method = likelihood_method
        self._logL_constant = log_likelihood_constant

    @property
    def noise_map(self):
        return self._noise_map

    def C_D_model(self, model):
        """``image_noise.py:100-110``."""
        if self._noise_map is not None:
            return self._noise_map ** 2
        return covariance_matrix(np.asarray(model), self.background_rms, self.exposure_map)

    def likelihood_method(self):
        return self._logL_method


class PSF:
    """Point spread function description (lenstronomy ``PSF`` attributes).

    PIXEL kernels are normalised to unit sum and must have odd axes."""

    def __init__(self, psf_type="NONE", fwhm=None, truncation=5, kernel_point_source=None,
                 psf_variance_map=None, point_source_supersampling_factor=1,
                 kernel_point_source_init=None, kernel_point_source_normalisation=True):
        if psf_type not in ("NONE", "GAUSSIAN", "PIXEL"):
            raise ValueError("psf_type %s not supported!" % psf_type)
        self.psf_type = psf_type
        self._fwhm = fwhm
        self._truncation = truncation
        self._kernel = None
        self._pixel_size = None
        self.point_source_supersampling_factor = point_source_supersampling_factor
        if psf_type == "GAUSSIAN" and fwhm is None:
            raise ValueError("fwhm must be set for GAUSSIAN psf type!")
        if psf_type == "PIXEL":
            if kernel_point_source is None:
                raise ValueError("kernel_point_source needs to be specified for PIXEL PSF type!")
            k = np.asarray(kernel_point_source, dtype=float)
            if k.ndim != 2 or k.shape[0] % 2 == 0 or k.shape[1] % 2 == 0 or k.shape[0] != k.shape[1]:
                raise ValueError("kernel needs to have odd axis number, not %s" % (k.shape,))
            self._kernel = k / np.sum(k) if kernel_point_source_normalisation else k
        self._psf_variance_map = psf_variance_map

    @property
    def kernel_point_source(self):
        if self.psf_type == "PIXEL" and self.point_source_supersampling_factor > 1:
            raise NotImplementedError(
                "the pixel-scale kernel of a supersampled PSF (lenstronomy "
                "kernel_util.degrade_kernel) is not provided; use it with "
                "supersampling_convolution=True")
        return self._kernel

    def kernel_point_source_supersampled(self, supersampling_factor, updata_cache=False):
        """The supersampled PIXEL kernel: the kernel given at construction when
        ``point_source_supersampling_factor`` equals ``supersampling_factor``."""
        if self.psf_type != "PIXEL":
            raise ValueError("kernel_point_source_supersampled needs a PIXEL PSF")
        if supersampling_factor == self.point_source_supersampling_factor and supersampling_factor > 1:
            return self._kernel
        raise NotImplementedError(
            "building a supersampled kernel from a pixel-scale one (lenstronomy "
            "kernel_util.subgrid_kernel) is not provided; pass the supersampled kernel with "
            "point_source_supersampling_factor = supersampling_factor")

    @property
    def fwhm(self):
        return self._fwhm

    @property
    def truncation(self):
        return self._truncation

    @property
    def psf_variance_map_bool(self):
        return self._psf_variance_map is not None

    def set_pixel_size(self, deltaPix):
        self._pixel_size = deltaPix
