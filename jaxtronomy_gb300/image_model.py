"""``ImageModel``: lensed-source + lens-light image simulation on the GPU.

Drop-in for ``jaxtronomy.ImSim.image_model.ImageModel`` (``image_model.py:27-492``)
for the analytic-profile path without point sources, with the numerics of
``Numerics`` / ``NumericsSubFrame`` (``ImSim/Numerics/numerics.py:24-177``,
``numerics_subframe.py:20-100``) in regular compute mode.

Besides the reference's one-system calls (``image``, ``source_surface_brightness``,
``lens_surface_brightness``, ``likelihood_data_given_model``) it offers batched
calls (``image_batch``, ``likelihood_batch``) that take kwargs whose values are
arrays of length B -- the layout ``jax.vmap`` gives the reference -- and run
the whole batch in one launch sequence.

``kwargs_numerics`` accepts the reference keys plus ``precision``:
``"fp64"`` (default; plain FP64 throughout) or ``"fp32"`` (FP32 bulk arithmetic
with FP64 set-up, FP64-accurate coordinate offsets and an FP64 likelihood
reduction).
"""

import copy
import ctypes

import numpy as np
import torch

from . import _device, _lib, profiles
from .data import PSF
from .lens_model import LensModel
from .light_model import LightModel
from .point_source import PointSource

_NUMERICS_KEYS = {
    "supersampling_factor", "compute_mode", "supersampling_convolution",
    "supersampling_kernel_size", "flux_evaluate_indexes", "supersampled_indexes",
    "compute_indexes", "point_source_supersampling_factor", "convolution_kernel_size",
    "convolution_type", "truncation_conv", "precision", "fp32_refine_tol", "fp32_refine_kappa",
    "convolution_method", "gradient_precision",
}


def _delta_kernel():
    """The 3x3 kernel of an unconvolved point source (point_source_rendering.py:59-61) and
    of a NONE PSF."""
    k = np.zeros((3, 3))
    k[1, 1] = 1.0
    return k


def fwhm2sigma(fwhm):
    """``jaxtronomy/Util/util.py:56-63``."""
    return fwhm / (2 * np.sqrt(2 * np.log(2)))


def gaussian_kernel(sigma_pix, truncation):
    """Kernel of ``GaussianConvolution`` (``convolution.py:199-206,254-273``):
    side 2r+1 with r = max(round(sigma*truncation), 1), normalised to unit sum."""
    radius = max(round(sigma_pix * truncation), 1)
    n = 2 * radius + 1
    c = np.arange(n) - (n - 1) / 2.0
    xx, yy = np.meshgrid(c, c)
    k = np.exp(-(xx ** 2 + yy ** 2) / (2 * sigma_pix ** 2)) / (2 * np.pi * sigma_pix ** 2)
    return k / np.sum(k)


def cut_psf(kernel, size):
    """Centred odd-size cut of a kernel without renormalisation (lenstronomy
    ``kernel_util.cut_psf(..., normalisation=False)``, used at numerics.py:196-213)."""
    n = kernel.shape[0]
    if size >= n:
        return kernel
    c = n // 2
    h = size // 2
    return kernel[c - h:c + h + 1, c - h:c + h + 1]


def split_kernel(kernel_super, supersampling_kernel_size, supersampling_factor):
    """(pixel-scale part, supersampled part) of a supersampled kernel for
    ``SubgridKernelConvolution`` (the role of lenstronomy
    ``kernel_util.split_kernel`` at convolution.py:123-127, defined here from
    that role): the supersampled part is the central n x n block,
    n = supersampling_kernel_size * s made odd (at most the kernel side); the
    pixel-scale part is the rest of the kernel summed over s x s blocks aligned
    on its centre.  Odd s only."""
    s = int(supersampling_factor)
    if s <= 1 or s % 2 == 0:
        raise ValueError("a kernel split (supersampling_kernel_size) needs an odd "
                         "supersampling factor > 1; pass supersampling_kernel_size=None")
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
    return big.reshape(n_low, s, n_low, s).sum(axis=(1, 3)), high


class ImageModel:
    """Lens image simulation (``image_model.py:27-150``)."""

    def __init__(self, data_class, psf_class, lens_model_class=None, source_model_class=None,
                 lens_light_model_class=None, point_source_class=None, extinction_class=None,
                 kwargs_numerics=None, likelihood_mask=None, psf_error_map_bool_list=None,
                 kwargs_pixelbased=None):
        self.type = "single-band"
        self.num_bands = 1
        self.PSF = psf_class
        self.Data = data_class
        self._flux_scaling = getattr(data_class, "flux_scaling", 1)
        self.PSF.set_pixel_size(self.Data.pixel_width)
        kn = dict(kwargs_numerics or {})
        unknown = set(kn) - _NUMERICS_KEYS
        if unknown:
            raise TypeError("unexpected kwargs_numerics keys %s" % sorted(unknown))
        precision = kn.pop("precision", "fp64")
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self._precision = _lib.FP64 if precision == "fp64" else _lib.FP32_SPLIT
        self._dtype = torch.float64 if precision == "fp64" else torch.float32
        # FP32 path: per-ray predicted relative error above which a pixel is
        # recomputed in FP64 (<= 0 disables), and the FP32 deflection error bound
        self._refine = (float(kn.pop("fp32_refine_tol", 2e-5)),
                        float(kn.pop("fp32_refine_kappa", 3e-7)))
        # Numerics.__init__ checks (numerics.py:68-146)
        compute_mode = kn.get("compute_mode", "regular")
        if compute_mode != "regular":
            raise ValueError("compute_mode %s not supported; only 'regular'" % compute_mode)
        s = kn.get("supersampling_factor", 1)
        if not isinstance(s, (int, np.integer)) or isinstance(s, bool):
            raise TypeError("supersampling_factor needs to be an integer! Current type is %s"
                            % type(s))
        s = int(s)
        if s < 1:
            raise ValueError("supersampling_factor must be >= 1")
        ssc = bool(kn.get("supersampling_convolution", False))
        if s == 1:
            ssc = False  # numerics.py:84-85
        self._ssc = ssc
        # numerics.py:31: the supersampled kernel is split unless this is None
        self._ssk = kn.get("supersampling_kernel_size", 5) if ssc else None
        self._subframe = None
        fei = kn.get("flux_evaluate_indexes")
        if fei is not None:
            # NumericsSubFrame._init_sub_frame (numerics_subframe.py:151-163)
            fei = np.asarray(fei, dtype=bool)
            if fei.shape != tuple(data_class.num_pixel_axes) or not fei.any():
                raise ValueError("flux_evaluate_indexes must be a non-empty boolean image")
            rows, cols = np.where(fei)
            x0, x1, y0, y1 = rows.min(), rows.max(), cols.min(), cols.max()
            if x1 - x0 != y1 - y0:
                # the reference's sub-frame grid has the transposed shape of the
                # slice it fills (numerics_subframe.py:134-149,176-200)
                raise ValueError("flux_evaluate_indexes needs a square bounding box")
            self._subframe = (int(x0), int(y0), fei[x0:x1 + 1, y0:y1 + 1].copy())
        conv_type = kn.get("convolution_type", "fft")
        if conv_type not in ("fft", "grid", "fft_static"):
            raise ValueError("convolution_type %s not supported!" % conv_type)
        # how the GPU convolves (an option of this library; every convolution_type
        # of the reference gives the same image up to rounding): "auto" (the
        # direct halo-tile kernels, and the FP64 FFT where a kernel is too wide
        # for their shared-memory tile), "direct" or "fft" (FP64 FFT always; the
        # faster choice for FP64 models from K ~ 21)
        method = kn.get("convolution_method", "auto")
        if method not in _lib.CONV_METHODS:
            raise ValueError("convolution_method must be one of %s" % sorted(_lib.CONV_METHODS))
        self._conv_method = _lib.CONV_METHODS[method]
        # arithmetic of the adjoint's ray derivatives (an option of this library):
        # "fp64" (default) or "fp32" (FP32 dual numbers from FP64-accurate
        # offsets with an FP64 re-pass of ill-conditioned pixels; FP64 forward
        # image, weights and reduction)
        gp = kn.get("gradient_precision", "fp64")
        if gp not in ("fp64", "fp32"):
            raise ValueError("gradient_precision must be 'fp64' or 'fp32'")
        self._grad_precision = _lib.FP64 if gp == "fp64" else _lib.FP32_SPLIT
        self._s = s
        self._kwargs_numerics = dict(kwargs_numerics or {})
        if kwargs_pixelbased is not None:
            raise ValueError("pixelbased solver not supported")
        if extinction_class is not None and getattr(extinction_class, "_profile_type_list", []):
            raise ValueError("extinction is not supported")
        if point_source_class is None:
            point_source_class = PointSource([], lens_model=lens_model_class)
        if not isinstance(point_source_class, PointSource):
            raise ValueError("point_source_class must be a jaxtronomy_gb300.PointSource")
        self.PointSource = point_source_class
        self._n_ps = len(point_source_class.point_source_type_list)
        if data_class.primary_beam is not None:
            raise ValueError("primary beam not supported")
        self.LensModel = lens_model_class if lens_model_class is not None else LensModel([])
        if self.PointSource._lens_model is None:
            # image_model.py:80-92: the point sources get the image's lens model
            self.PointSource = copy.copy(self.PointSource)
            self.PointSource._lens_model = self.LensModel
        self.SourceModel = source_model_class if source_model_class is not None else LightModel([])
        self.LensLightModel = (lens_light_model_class if lens_light_model_class is not None
                               else LightModel([]))
        nx, ny = data_class.num_pixel_axes
        if nx != ny:
            raise ValueError("ImageModel needs a square pixel grid (got %d x %d)" % (nx, ny))
        self._nx, self._ny = int(nx), int(ny)
        if likelihood_mask is None:
            likelihood_mask = np.ones((self._nx, self._ny))
        self.likelihood_mask = np.array(likelihood_mask, dtype=bool)
        self.num_data_evaluate = int(np.sum(self.likelihood_mask))
        self._psf_error_map = self.PSF.psf_variance_map_bool

        # PSF kernel for the convolution step (numerics.py:102-139)
        pt = psf_class.psf_type
        if pt == "PIXEL":
            cks = kn.get("convolution_kernel_size")
            if ssc:
                # numerics.py:104-115,196-213: supersampled kernel, cut to
                # convolution_kernel_size * s (made odd)
                kernel = np.asarray(psf_class.kernel_point_source_supersampled(s), dtype=float)
                if cks is not None:
                    size = cks * s
                    kernel = cut_psf(kernel, size if size % 2 == 1 else size + 1)
            else:
                kernel = np.asarray(psf_class.kernel_point_source, dtype=float)
                if cks is not None:
                    size = cks if cks % 2 == 1 else cks + 1
                    kernel = cut_psf(kernel, size)
            self._psf_type = _lib.PSF_PIXEL
        elif pt == "GAUSSIAN":
            trunc = kn.get("truncation_conv")
            if trunc is None:
                trunc = psf_class.truncation
            sigma = fwhm2sigma(psf_class.fwhm) / data_class.pixel_width
            if ssc:
                sigma *= s  # convolution.py:194-195
            kernel = gaussian_kernel(sigma, trunc)
            self._psf_type = _lib.PSF_GAUSSIAN
        elif pt == "NONE":
            kernel = None
            self._psf_type = _lib.PSF_NONE
        else:
            raise ValueError("psf_type %s not valid! Chose either NONE, GAUSSIAN or PIXEL." % pt)
        self._kernel = kernel
        self._kernel_size = 0 if kernel is None else int(kernel.shape[0])
        self._low_kernel_size = 0
        if ssc and pt == "PIXEL" and self._ssk is not None:
            lo, hi = split_kernel(kernel, self._ssk, s)
            self._kernel_size = int(hi.shape[0])
            self._low_kernel_size = int(lo.shape[0])
        self._kernel_dev = None
        self._models = {}
        # point-source rendering kernel (numerics.py:147-151, point_source_rendering.py:14-32)
        self._ps_sub = int(kn.get("point_source_supersampling_factor", 1))
        self._ps_kernel = None
        if self._n_ps:
            if self._subframe is not None:
                raise ValueError("point sources with flux_evaluate_indexes are not supported")
            if self.PSF.psf_variance_map_bool:
                raise ValueError("PSF variance maps (point-source error maps) are not supported")
            if self._ps_sub < 1:
                raise ValueError("point_source_supersampling_factor must be >= 1")
            if pt == "PIXEL":
                ps_k = (psf_class.kernel_point_source if self._ps_sub == 1
                        else psf_class.kernel_point_source_supersampled(self._ps_sub))
            elif pt == "NONE":
                ps_k = _delta_kernel()
            else:
                raise ValueError("point sources need a PIXEL or NONE PSF (the pixelised "
                                 "GAUSSIAN kernel of lenstronomy's PSF is not provided)")
            self._ps_kernel = np.ascontiguousarray(ps_k, dtype=np.float64)

    # ------------------------------------------------------------------ models
    def _desc(self, lens_idx, src_idx, ll_idx, lensed=True, precision=None):
        d = _lib.ModelDesc()
        lm = self.LensModel.lens_model_list
        d.n_lens = len(lens_idx) if lensed else 0
        for j, i in enumerate(lens_idx if lensed else []):
            d.lens_codes[j] = _lib.LENS_CODES[lm[i]]
        sm = self.SourceModel.profile_type_list
        dsl = self.SourceModel.deflection_scaling_list
        d.n_source = len(src_idx)
        for j, i in enumerate(src_idx):
            d.source_codes[j] = _lib.LIGHT_CODES[sm[i]]
            d.deflection_scaling[j] = 1.0 if dsl is None else float(dsl[i])
        llm = self.LensLightModel.profile_type_list
        d.n_lens_light = len(ll_idx)
        for j, i in enumerate(ll_idx):
            d.lens_light_codes[j] = _lib.LIGHT_CODES[llm[i]]
        d.nx, d.ny = self._ny, self._nx  # columns, rows of an (nx, ny)-shaped array
        d.supersampling = self._s
        d.transform_pix2angle[:] = list(np.asarray(self.Data.transform_pix2angle, float).ravel())
        ra0, dec0 = self.Data.radec_at_xy_0
        d.ra_at_xy_0, d.dec_at_xy_0 = float(ra0), float(dec0)
        d.flux_scaling = float(self._flux_scaling)
        d.alpha_scaling = float(getattr(self.LensModel, "alpha_scaling", 1.0))
        d.psf_type = self._psf_type
        d.kernel_size = self._kernel_size
        d.precision = self._precision if precision is None else precision
        d.supersampling_convolution = 1 if self._ssc else 0
        d.low_res_kernel_size = self._low_kernel_size
        return d

    def _model(self, lens_idx, src_idx, ll_idx, lensed=True, precision=None):
        prec = self._precision if precision is None else precision
        key = (tuple(lens_idx), tuple(src_idx), tuple(ll_idx), lensed, prec)
        if key not in self._models:
            refine = self._refine if prec == _lib.FP32_SPLIT else None
            self._models[key] = _lib.Model(self._desc(lens_idx, src_idx, ll_idx, lensed, prec),
                                           refine, self._subframe, self._conv_method)
        return self._models[key]

    def refined_pixels(self, stream=None):
        """Pixels the last batched FP32 image call recomputed in FP64 (synchronizes)."""
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        return model.refined_pixels(_device.stream_handle(stream))

    def autotune(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                 psf_kernels=None, rows=None, stream=None):
        """Times the batched image call on these (batched) kwargs with every ray-kernel
        pixels-per-thread and convolution tile height (``lensgb_model_autotune``)
        and keeps the fastest for this model's later calls.  Returns the chosen
        shapes and their times next to the built-in ones (ms)."""
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        if rows is None:
            rows = self.pack_params(kwargs_lens, kwargs_source, kwargs_lens_light)
        rows_dev = _device.to_device_f64(rows)
        B = rows_dev.shape[0]
        out = torch.empty((B, self._nx, self._ny), dtype=self._dtype, device="cuda")
        kt, kstride, keep = self._psf_arg(psf_kernels, B)
        kptr = ctypes.c_void_p(0) if kt is None else _device.ptr(kt)
        res = _lib.TuneResult()
        _lib.check(_lib.load().lensgb_model_autotune(
            model.handle, _device.ptr(rows_dev), B, kptr, kstride, _device.ptr(out),
            _device.stream_handle(stream), ctypes.byref(res)))
        del keep
        return {n: getattr(res, n) for n, _ in _lib.TuneResult._fields_}

    def set_tuning(self, ppt=0, conv_tile_rows=0):
        """Launch shapes of this model's image calls (0: the built-in choice)."""
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        _lib.check(_lib.load().lensgb_model_set_tuning(model.handle, int(ppt),
                                                       int(conv_tile_rows)))

    def psf_elements(self):
        """PSF values per system in the C-ABI layout (0 for psf_type NONE)."""
        if self._kernel is None:
            return 0
        return self._kernel_size ** 2 + self._low_kernel_size ** 2

    def pack_psf(self, kernel):
        """One PSF kernel (the model's convolution-kernel shape: the supersampled
        kernel when convolving on the supersampled grid) as the flat array the
        C ABI takes: the kernel itself, or a split kernel's supersampled part
        followed by its pixel-scale part."""
        k = np.asarray(kernel, dtype=float)
        if self._low_kernel_size:
            lo, hi = split_kernel(k, self._ssk, self._s)
            return np.concatenate([hi.ravel(), lo.ravel()])
        return k.ravel()

    def _kernel_tensor(self):
        if self._kernel_dev is None and self._kernel is not None:
            self._kernel_dev = torch.as_tensor(self.pack_psf(self._kernel),
                                               dtype=self._dtype).cuda().contiguous()
        return self._kernel_dev

    # ------------------------------------------------------------------ packing
    def pack_params(self, kwargs_lens, kwargs_source, kwargs_lens_light, lens_idx=None,
                    src_idx=None, ll_idx=None, lensed=True):
        """(B, param_count) float64 rows for the given (possibly batched) kwargs."""
        lm = self.LensModel.lens_model_list
        sm = self.SourceModel.profile_type_list
        llm = self.LensLightModel.profile_type_list
        lens_idx = list(range(len(lm))) if lens_idx is None else lens_idx
        src_idx = list(range(len(sm))) if src_idx is None else src_idx
        ll_idx = list(range(len(llm))) if ll_idx is None else ll_idx
        kl = [kwargs_lens[i] for i in lens_idx] if (lensed and lens_idx) else []
        ks = [kwargs_source[i] for i in src_idx] if src_idx else []
        kll = [kwargs_lens_light[i] for i in ll_idx] if ll_idx else []
        B = profiles.batch_size(kl, ks, kll)
        names_l = [lm[i] for i in lens_idx] if lensed else []
        names_s = [sm[i] for i in src_idx]
        names_ll = [llm[i] for i in ll_idx]
        P = (profiles.n_params(names_l, profiles.LENS_PARAMS)
             + profiles.n_params(names_s, profiles.LIGHT_PARAMS)
             + profiles.n_params(names_ll, profiles.LIGHT_PARAMS))
        rows = np.zeros((B, P), dtype=np.float64)
        c = profiles.pack(names_l, profiles.LENS_PARAMS, kl, rows, 0, "Lens")
        c = profiles.pack(names_s, profiles.LIGHT_PARAMS, ks, rows, c, "Source")
        profiles.pack(names_ll, profiles.LIGHT_PARAMS, kll, rows, c, "Lens light")
        return rows

    def _psf_arg(self, psf_kernels, B, dtype=None):
        if self._psf_type == _lib.PSF_NONE:
            return None, 0, None
        dtype = self._dtype if dtype is None else dtype
        if psf_kernels is None:
            if dtype == self._dtype:
                k = self._kernel_tensor()
            else:  # the FP64 twin of an FP32 model: the kernel at full precision
                k = torch.as_tensor(self.pack_psf(self._kernel), dtype=dtype).cuda().contiguous()
            return k, 0, k
        k = psf_kernels
        K = int(self._kernel.shape[0])
        if self._low_kernel_size:
            # split each supersampled kernel on the host into the ABI layout
            arr = k.cpu().numpy() if isinstance(k, torch.Tensor) else np.asarray(k, float)
            if arr.shape[-2:] != (K, K) or arr.ndim not in (2, 3):
                raise ValueError("psf kernels must be %dx%d (supersampled)" % (K, K))
            arr = arr[None] if arr.ndim == 2 else arr
            packed = np.stack([self.pack_psf(a) for a in arr])
            t = torch.as_tensor(packed).to(device="cuda", dtype=dtype).contiguous()
            return t, (0 if packed.shape[0] == 1 else self.psf_elements()), t
        if not isinstance(k, torch.Tensor):
            k = torch.as_tensor(np.ascontiguousarray(k))
        k = k.to(device="cuda", dtype=dtype).contiguous()
        if k.dim() == 2:
            if tuple(k.shape) != (K, K):
                raise ValueError("psf kernel must be %dx%d" % (K, K))
            return k, 0, k
        if tuple(k.shape) != (B, K, K):
            raise ValueError("per-system psf kernels must have shape (%d, %d, %d)" % (B, K, K))
        return k, K * K, k

    # ------------------------------------------------------------------ launches
    def _launch(self, model, rows_dev, B, flags, psf_kernels=None, out=None, stream=None):
        _device.require_cuda()
        if out is None:
            out = torch.empty((B, self._nx, self._ny), dtype=self._dtype, device="cuda")
        elif out.dtype != self._dtype or not out.is_contiguous() or out.numel() < B * self._nx * self._ny:
            raise ValueError("out must be a contiguous %s tensor of shape (B, %d, %d)"
                             % (self._dtype, self._nx, self._ny))
        kt, kstride, keep = self._psf_arg(psf_kernels, B)
        kptr = ctypes.c_void_p(0) if kt is None else _device.ptr(kt)
        _lib.check(_lib.load().lensgb_image(
            model.handle, _device.ptr(rows_dev), B, kptr, kstride, _device.ptr(out), flags,
            _device.stream_handle(stream)))
        del keep
        return out

    # ------------------------------------------------------------------ point sources
    def point_source_rows(self, kwargs_ps, kwargs_special=None, B=None, k=None,
                          kwargs_lens=None):
        """(B, n_images, 3) FP64 rows (ra, dec, amp): PointSource.point_source_list
        (point_source.py:255-284) after ImageModel._displace_astrometry
        (image_model.py:652-676), broadcast over a batch of B systems."""
        ra, dec, amp = self.PointSource.point_source_list(kwargs_ps, kwargs_lens, k=k)
        ra, dec, amp = (np.atleast_2d(np.asarray(a, dtype=float)) for a in (ra, dec, amp))
        n = ra.shape[-1]
        if kwargs_special is not None and "delta_x_image" in kwargs_special:
            shifts = []
            for key in ("delta_x_image", "delta_y_image"):
                d = np.atleast_2d(np.asarray(kwargs_special[key], dtype=float))[..., :n]
                pad = np.zeros(d.shape[:-1] + (n - d.shape[-1],))
                shifts.append(np.concatenate([d, pad], axis=-1))
            ra, dec = ra + shifts[0], dec + shifts[1]
        ra, dec, amp = np.broadcast_arrays(ra, dec, amp)
        Bp = ra.shape[0]
        if B is None:
            B = Bp
        if Bp not in (1, B):
            raise ValueError("point-source kwargs have %d systems, the call %d" % (Bp, B))
        rows = np.stack([ra, dec, amp], axis=-1)
        return np.array(np.broadcast_to(rows, (B, n, 3)), dtype=np.float64)

    def _add_point_sources(self, out, B, kwargs_ps, kwargs_special=None, unconvolved=False,
                           psf_kernels=None, stream=None, k=None, kwargs_lens=None):
        """Adds ImageModel.point_source (image_model.py:396-429) to the (B, ny, nx)
        images ``out`` on the GPU (``lensgb_point_sources_add``)."""
        if not self._n_ps:
            return out
        if kwargs_ps is None:
            raise ValueError("kwargs_ps is needed for the point-source models %s"
                             % self.PointSource.point_source_type_list)
        rows = self.point_source_rows(kwargs_ps, kwargs_special, B, k=k, kwargs_lens=kwargs_lens)
        return self._render_point_rows(out, rows, unconvolved, psf_kernels, stream)

    def _render_point_rows(self, out, rows, unconvolved=False, psf_kernels=None, stream=None):
        """Adds the (B, n_images, 3) point rows (ra, dec, amp) to ``out``."""
        B, n = rows.shape[0], rows.shape[1]
        if n == 0:
            return out
        ps = _device.to_device_f64(rows)
        kstride = 0
        if unconvolved:
            kern = _delta_kernel()
        elif (psf_kernels is not None and self._ps_sub == 1 and self._psf_type == _lib.PSF_PIXEL
              and not self._ssc):
            # per-system pixel-scale kernels (supersampled ones, of a model convolving on
            # the supersampled grid, are not the rendering kernel)
            kern = psf_kernels.cpu().numpy() if isinstance(psf_kernels, torch.Tensor) \
                else np.asarray(psf_kernels, dtype=float)
            if kern.ndim == 3 and kern.shape[0] > 1:
                kstride = kern.shape[1] * kern.shape[2]
            kern = kern.reshape((-1,) + kern.shape[-2:])[0] if kstride == 0 else kern
        else:
            kern = self._ps_kernel
        kt = _device.to_device_f64(np.ascontiguousarray(kern, dtype=np.float64))
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        _lib.check(_lib.load().lensgb_point_sources_add(
            model.handle, _device.ptr(ps), n, B, _device.ptr(kt), int(kern.shape[-1]), kstride,
            self._ps_sub, _device.ptr(out),
            _device.stream_handle(stream)))
        self._ps_keep = (ps, kt)
        return out

    def host_wait(self, stream=None):
        """Makes ``stream`` wait for every image copy of earlier host-output calls."""
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        _lib.check(_lib.load().lensgb_image_host_wait(model.handle,
                                                      _device.stream_handle(stream)))

    def _launch_host(self, model, rows, flags, psf_kernels, out, stream, n_chunks=0):
        # host rows / PSFs / images: lensgb_image_host copies the images of each
        # chunk back while the next chunk is computed
        rows_h = rows if isinstance(rows, torch.Tensor) else torch.as_tensor(
            np.ascontiguousarray(rows, dtype=np.float64))
        if rows_h.device.type != "cpu":
            raise ValueError("host output needs host parameter rows")
        rows_h = rows_h.to(torch.float64).contiguous()
        B = rows_h.shape[0]
        if (out.dtype != self._dtype or not out.is_contiguous()
                or out.numel() < B * self._nx * self._ny):
            raise ValueError("out must be a contiguous %s tensor of shape (B, %d, %d)"
                             % (self._dtype, self._nx, self._ny))
        kh, kstride = None, 0
        if self._psf_type != _lib.PSF_NONE:
            K = int(self._kernel.shape[0])
            if psf_kernels is None:
                kh = torch.as_tensor(self.pack_psf(self._kernel))
            else:
                arr = psf_kernels if isinstance(psf_kernels, torch.Tensor) else torch.as_tensor(
                    np.asarray(psf_kernels))
                if arr.device.type != "cpu":
                    raise ValueError("host output needs host PSF kernels")
                if tuple(arr.shape[-2:]) != (K, K) or arr.dim() not in (2, 3) or (
                        arr.dim() == 3 and arr.shape[0] != B):
                    raise ValueError("psf kernels must have shape (%d, %d) or (%d, %d, %d)"
                                     % (K, K, B, K, K))
                per_system = arr.dim() == 3
                if self._low_kernel_size:
                    a3 = arr.double().numpy().reshape(-1, K, K)
                    arr = torch.as_tensor(np.stack([self.pack_psf(a) for a in a3]))
                kh = arr
                kstride = self.psf_elements() if per_system else 0
            kh = kh.to(self._dtype).contiguous()
        kptr = ctypes.c_void_p(0) if kh is None else ctypes.c_void_p(kh.data_ptr())
        _lib.check(_lib.load().lensgb_image_host(
            model.handle, ctypes.c_void_p(rows_h.data_ptr()), B, kptr, kstride,
            ctypes.c_void_p(out.data_ptr()), flags, int(n_chunks),
            _device.stream_handle(stream)))
        # the host buffers must outlive the copies queued on the stream (two
        # calls may be in flight)
        self._host_keep = (getattr(self, "_host_keep", (None,))[-1], (rows_h, kh))
        return out

    def image_batch(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                    unconvolved=False, source_add=True, lens_light_add=True, psf_kernels=None,
                    out=None, stream=None, rows=None, kwargs_ps=None, kwargs_special=None,
                    point_source_add=True):
        """Batched ``image``: kwargs values are arrays of length B (or scalars).
        Returns a (B, ny, nx) CUDA tensor in the model precision.  ``psf_kernels``
        may give one (K, K) kernel or one per system (B, K, K) in place of the
        model PSF (normalised by the caller).  ``rows`` may pass pre-packed
        parameter rows (host array or CUDA tensor, see :meth:`pack_params`).
        With a host tensor ``out`` (and host rows / PSFs) the call runs
        ``lensgb_image_host``: the images are copied back on a second stream,
        overlapping the next call's work (page-locked buffers give the overlap);
        ``out`` is complete after :meth:`host_wait` and a synchronization of the
        stream (or a device synchronization).  Point sources (``kwargs_ps``, values
        of shape (n_images,) or (B, n_images)) are rendered on the GPU and added
        after the convolution, as ``ImageModel.image`` adds ``point_source``."""
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        if rows is None:
            rows = self.pack_params(kwargs_lens, kwargs_source, kwargs_lens_light)
        flags = ((_lib.UNCONVOLVED if unconvolved else 0)
                 | (0 if source_add else _lib.NO_SOURCE)
                 | (0 if lens_light_add else _lib.NO_LENS_LIGHT))
        with_ps = bool(self._n_ps) and point_source_add
        host_out = isinstance(out, torch.Tensor) and out.device.type == "cpu"
        if host_out and not with_ps:
            return self._launch_host(model, rows, flags, psf_kernels, out, stream)
        rows_dev = _device.to_device_f64(rows)
        B = rows_dev.shape[0]
        dev_out = self._launch(model, rows_dev, B, flags, psf_kernels,
                               None if host_out else out, stream)
        if with_ps:
            self._add_point_sources(dev_out, B, kwargs_ps, kwargs_special, unconvolved,
                                    psf_kernels, stream, kwargs_lens=kwargs_lens)
        if host_out:
            out.copy_(dev_out)
            return out
        return dev_out

    # ------------------------------------------------------------------ reference API
    def image(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None, kwargs_ps=None,
              kwargs_extinction=None, kwargs_special=None, unconvolved=False, source_add=True,
              lens_light_add=True, point_source_add=True):
        """``image_model.py:432-492``: 2d array of the simulated image."""
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        im = self.image_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                              unconvolved=unconvolved, source_add=source_add,
                              lens_light_add=lens_light_add, kwargs_ps=kwargs_ps,
                              kwargs_special=kwargs_special, point_source_add=point_source_add)
        return im[0].cpu().numpy().astype(np.float64, copy=False)

    def source_surface_brightness(self, kwargs_source, kwargs_lens=None, kwargs_extinction=None,
                                  kwargs_special=None, unconvolved=False, de_lensed=False, k=None,
                                  update_pixelbased_mapping=True):
        """``image_model.py:224-266``."""
        sm = self.SourceModel.profile_type_list
        if len(sm) == 0:
            return np.zeros((self._nx, self._ny))
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        src_idx = self.SourceModel._select(k)
        lens_idx = list(range(len(self.LensModel.lens_model_list)))
        lensed = not de_lensed
        model = self._model(lens_idx, src_idx, [], lensed)
        rows = self.pack_params(kwargs_lens, kwargs_source, None, lens_idx=lens_idx,
                                src_idx=src_idx, ll_idx=[], lensed=lensed)
        flags = (_lib.UNCONVOLVED if unconvolved else 0) | _lib.NO_LENS_LIGHT
        im = self._launch(model, _device.to_device_f64(rows), rows.shape[0], flags)
        return im[0].cpu().numpy().astype(np.float64, copy=False)

    def lens_surface_brightness(self, kwargs_lens_light, unconvolved=False, k=None):
        """``image_model.py:371-393``."""
        llm = self.LensLightModel.profile_type_list
        if len(llm) == 0:
            return np.zeros((self._nx, self._ny))
        ll_idx = self.LensLightModel._select(k)
        model = self._model([], [], ll_idx)
        rows = self.pack_params(None, None, kwargs_lens_light, lens_idx=[], src_idx=[],
                                ll_idx=ll_idx)
        flags = (_lib.UNCONVOLVED if unconvolved else 0) | _lib.NO_SOURCE
        im = self._launch(model, _device.to_device_f64(rows), rows.shape[0], flags)
        return im[0].cpu().numpy().astype(np.float64, copy=False)

    def _noise_tensors(self, data=None):
        """Device copies of data, mask and noise model (cached for the model's own
        data; ``data`` may pass a (B, ny, nx) batch instead)."""
        if data is None:
            if getattr(self, "_noise_cache", None) is None:
                self._noise_cache = self._make_noise(self.Data.data)
            return self._noise_cache
        return self._make_noise(data)

    def _make_noise(self, data):
        D = self.Data
        t = {}
        dt = data if isinstance(data, torch.Tensor) else torch.as_tensor(np.asarray(data, float))
        dt = dt.to(device="cuda", dtype=torch.float64).contiguous()
        t["data"] = dt
        t["data_stride"] = self._nx * self._ny if dt.dim() == 3 else 0
        t["mask"] = torch.as_tensor(self.likelihood_mask.astype(np.float64)).cuda()
        nm = D.noise_map
        t["noise"] = None if nm is None else torch.as_tensor(np.asarray(nm, float)).cuda()
        em = D.exposure_map
        if nm is None and em is not None and np.ndim(em) > 0:
            t["expo"] = torch.as_tensor(np.broadcast_to(np.asarray(em, float),
                                                        (self._nx, self._ny)).copy()).cuda()
            t["expo_t"] = 1.0
        else:
            t["expo"] = None
            t["expo_t"] = float(em) if em is not None else 1.0
        return t

    def _noise_desc(self, nt):
        nd = _lib.NoiseDesc()
        nd.data_dev = nt["data"].data_ptr()
        nd.data_stride = nt["data_stride"]
        nd.mask_dev = nt["mask"].data_ptr()
        nd.noise_map_dev = 0 if nt["noise"] is None else nt["noise"].data_ptr()
        nd.noise_stride = 0
        nd.exposure_map_dev = 0 if nt["expo"] is None else nt["expo"].data_ptr()
        nd.exposure_stride = 0
        nd.exposure_time = nt["expo_t"]
        nd.background_rms = float(self.Data.background_rms)
        nd.error_map_dev = 0
        nd.mask_stride = 0
        return nd

    def likelihood_batch(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                         data=None, psf_kernels=None, rows=None, image_out=None, stream=None,
                         kwargs_ps=None, kwargs_special=None):
        """Batched ``likelihood_data_given_model``: (B,) FP64 CUDA tensor of
        log-likelihoods; ``data`` optionally gives one (ny, nx) image per system.
        With point-source models the model image (extended light + rendered point
        sources) is made first and ``lensgb_loglike_image`` scores it."""
        if self._n_ps:
            im = self.image_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                  psf_kernels=psf_kernels, out=image_out, stream=stream,
                                  rows=rows, kwargs_ps=kwargs_ps, kwargs_special=kwargs_special)
            nt = self._noise_tensors(data)
            nd = self._noise_desc(nt)
            logl = torch.empty((im.shape[0],), dtype=torch.float64, device="cuda")
            _lib.check(_lib.load().lensgb_loglike_image(
                self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list))).handle,
                _device.ptr(im), im.shape[0], ctypes.byref(nd), _device.ptr(logl),
                _device.stream_handle(stream)))
            return logl
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)))
        if rows is None:
            rows = self.pack_params(kwargs_lens, kwargs_source, kwargs_lens_light)
        rows_dev = _device.to_device_f64(rows)
        B = rows_dev.shape[0]
        nt = self._noise_tensors(data)
        nd = self._noise_desc(nt)
        if image_out is None:
            image_out = torch.empty((B, self._nx, self._ny), dtype=self._dtype, device="cuda")
        logl = torch.empty((B,), dtype=torch.float64, device="cuda")
        kt, kstride, keep = self._psf_arg(psf_kernels, B)
        kptr = ctypes.c_void_p(0) if kt is None else _device.ptr(kt)
        _lib.check(_lib.load().lensgb_loglike(
            model.handle, _device.ptr(rows_dev), B, kptr, kstride, ctypes.byref(nd),
            _device.ptr(image_out), _device.ptr(logl), _device.stream_handle(stream)))
        del keep
        return logl

    def likelihood_grad_batch(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                              data=None, psf_kernels=None, rows=None, image_out=None,
                              stream=None):
        """logL and d logL / d params for B systems: ((B,) logL, (B, param_count)
        gradient rows) as FP64 CUDA tensors, by the adjoint kernel
        (``lensgb_loglike_grad``).  The gradient has the layout of
        :meth:`pack_params`; :meth:`unpack_params` turns it into kwargs lists.
        This is ``jax.grad`` of the reference's ``likelihood_data_given_model``
        (``image_model.py:163-221``) for lens stacks of EPL,
        EPL_MULTIPOLE_M1M3M4, SIE, NIE, NFW, TNFW, NFW_ELLIPSE_CSE, CONVERGENCE
        and SHEAR with Sersic light, every PSF type, convolution on the pixel or
        the supersampled grid and sub-frames (``flux_evaluate_indexes``).  The
        gradient, its logL and ``image_out`` (float64) are computed in FP64
        whatever the model's precision: an FP32 model differentiates through
        its FP64 twin, because the gradient's sums over pixels mix signs.
        ``kwargs_numerics["gradient_precision"] = "fp32"`` runs the per-ray
        derivatives in FP32 (the forward image, weights and reduction stay FP64;
        pixels whose FP32 derivatives are predicted ill-conditioned are
        recomputed in FP64), within 1e-4 of the FP64 adjoint."""
        if self._n_ps:
            raise ValueError("likelihood gradients with point sources are not supported")
        model = self._model(range(len(self.LensModel.lens_model_list)),
                            range(len(self.SourceModel.profile_type_list)),
                            range(len(self.LensLightModel.profile_type_list)),
                            precision=_lib.FP64)
        _lib.check(_lib.load().lensgb_model_set_grad_precision(model.handle,
                                                                self._grad_precision))
        if rows is None:
            rows = self.pack_params(kwargs_lens, kwargs_source, kwargs_lens_light)
        rows_dev = _device.to_device_f64(rows)
        B = rows_dev.shape[0]
        nt = self._noise_tensors(data)
        nd = self._noise_desc(nt)
        if image_out is None:
            image_out = torch.empty((B, self._nx, self._ny), dtype=torch.float64, device="cuda")
        logl = torch.empty((B,), dtype=torch.float64, device="cuda")
        grad = torch.empty((B, model.param_count), dtype=torch.float64, device="cuda")
        kt, kstride, keep = self._psf_arg(psf_kernels, B, dtype=torch.float64)
        kptr = ctypes.c_void_p(0) if kt is None else _device.ptr(kt)
        _lib.check(_lib.load().lensgb_loglike_grad(
            model.handle, _device.ptr(rows_dev), B, kptr, kstride, ctypes.byref(nd),
            _device.ptr(image_out), _device.ptr(logl), _device.ptr(grad),
            _device.stream_handle(stream)))
        del keep
        return logl, grad

    def unpack_params(self, rows):
        """Inverse of :meth:`pack_params`: (kwargs_lens, kwargs_source,
        kwargs_lens_light) with one array of length B per parameter."""
        rows = rows.cpu().numpy() if isinstance(rows, torch.Tensor) else np.asarray(rows)
        rows = rows.reshape(-1, rows.shape[-1])
        out, c = [], 0
        for names, table in ((self.LensModel.lens_model_list, profiles.LENS_PARAMS),
                             (self.SourceModel.profile_type_list, profiles.LIGHT_PARAMS),
                             (self.LensLightModel.profile_type_list, profiles.LIGHT_PARAMS)):
            kws = []
            for n in names:
                kws.append({p: rows[:, c + j].copy() for j, p in enumerate(table[n])})
                c += len(table[n])
            out.append(kws)
        return tuple(out)

    def likelihood_data_given_model(self, kwargs_lens=None, kwargs_source=None,
                                    kwargs_lens_light=None, kwargs_ps=None,
                                    kwargs_extinction=None, kwargs_special=None,
                                    source_marg=False, linear_prior=None,
                                    check_positive_flux=False):
        """``image_model.py:163-221``: log-likelihood of the data given the model."""
        if check_positive_flux:
            raise ValueError("check positive flux is not supported")
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        return float(self.likelihood_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                           kwargs_ps=kwargs_ps,
                                           kwargs_special=kwargs_special)[0].cpu())

    def point_source(self, kwargs_ps, kwargs_lens=None, kwargs_special=None, unconvolved=False,
                     k=None):
        """``image_model.py:396-429``: the rendered point sources alone (all models, or
        the k-th)."""
        if not self._n_ps:
            return np.zeros((self._nx, self._ny))
        rows = self.point_source_rows(kwargs_ps, kwargs_special, k=k, kwargs_lens=kwargs_lens)
        out = torch.zeros((rows.shape[0], self._nx, self._ny), dtype=self._dtype, device="cuda")
        self._render_point_rows(out, rows, unconvolved)
        return out[0].cpu().numpy().astype(np.float64, copy=False)

    def reduced_residuals(self, model, error_map=0):
        """(data - model) / sqrt(C_D_model + |error_map|) on the host."""
        model = np.asarray(model)
        c_d = self.Data.C_D_model(model)
        return (model - self.Data.data) / np.sqrt(c_d + np.abs(error_map)) * self.likelihood_mask

    def update_psf(self, psf_class):
        raise ValueError("Updating psf class not supported. Create a new instance of ImageModel "
                         "instead.")

    def update_data(self, data_class):
        raise ValueError("Updating data class not supported. Create a new instance of ImageModel "
                         "instead.")


__all__ = ["ImageModel", "PSF"]


def image_mixed(requests, stream=None):
    """Images of systems on different pixel grids, PSF sizes and supersampling
    factors in one launch sequence (``lensgb_image_mixed``).  ``requests``: list
    of (image_model, kwargs_lens, kwargs_source, kwargs_lens_light[, psf_kernel])
    with one system each; the image models must share their profile lists, PSF
    type and precision.  Returns one CUDA tensor per request, each equal to that
    model's ``image_batch`` of the request alone."""
    _device.require_cuda()
    if not requests:
        return []
    first = requests[0][0]
    key = None
    rows, grids, psfs, shapes = [], [], [], []
    for req in requests:
        im, kl, ks, kll = req[:4]
        psf = req[4] if len(req) > 4 else None
        d = im._desc(range(len(im.LensModel.lens_model_list)),
                     range(len(im.SourceModel.profile_type_list)),
                     range(len(im.LensLightModel.profile_type_list)))
        k = (tuple(d.lens_codes[:d.n_lens]), tuple(d.source_codes[:d.n_source]),
             tuple(d.deflection_scaling[:d.n_source]), tuple(d.lens_light_codes[:d.n_lens_light]),
             d.psf_type, d.precision, d.flux_scaling, d.alpha_scaling)
        if key is None:
            key = k
        elif k != key:
            raise ValueError("image_mixed needs models with the same profiles, PSF type, "
                             "precision and scalings")
        if im._ssc or im._subframe is not None:
            raise ValueError("image_mixed does not take supersampled convolution or sub-frames")
        r = im.pack_params(kl, ks, kll)
        if r.shape[0] != 1:
            raise ValueError("one system per request")
        rows.append(r[0])
        g = _lib.SystemGrid()
        g.nx, g.ny = d.nx, d.ny
        g.transform_pix2angle[:] = list(d.transform_pix2angle)
        g.ra_at_xy_0, g.dec_at_xy_0 = d.ra_at_xy_0, d.dec_at_xy_0
        g.kernel_size = d.kernel_size
        g.supersampling = d.supersampling
        grids.append(g)
        if im._psf_type != _lib.PSF_NONE:
            psfs.append(im.pack_psf(im._kernel if psf is None else psf))
        shapes.append((im._nx, im._ny))
    model = first._model(range(len(first.LensModel.lens_model_list)),
                         range(len(first.SourceModel.profile_type_list)),
                         range(len(first.LensLightModel.profile_type_list)))
    rows_dev = _device.to_device_f64(np.stack(rows))
    dtype = first._dtype
    psf_dev = (torch.as_tensor(np.concatenate(psfs)).to(device="cuda", dtype=dtype)
               if psfs else None)
    total = sum(a * b for a, b in shapes)
    out = torch.empty(total, dtype=dtype, device="cuda")
    arr = (_lib.SystemGrid * len(grids))(*grids)
    _lib.check(_lib.load().lensgb_image_mixed(
        model.handle, _device.ptr(rows_dev), len(grids), arr,
        ctypes.c_void_p(0) if psf_dev is None else _device.ptr(psf_dev), _device.ptr(out), 0,
        _device.stream_handle(stream)))
    res, o = [], 0
    for a, b in shapes:
        res.append(out[o:o + a * b].view(a, b))
        o += a * b
    return res
