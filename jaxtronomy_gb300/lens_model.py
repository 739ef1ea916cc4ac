"""``LensModel``: single-plane ray shooting through a list of lens profiles.

Drop-in for ``jaxtronomy.LensModel.lens_model.LensModel``
(``lens_model.py:25-252,353-381``) restricted to the single-plane path
(``SinglePlane``, ``single_plane.py:39-139``).  All evaluation runs in
liblensgb.so on the GPU in FP64.
"""

import numpy as np
import torch

from . import _device, _lib, profiles


def _as_out(t, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


class LensModel:
    """Class to handle an arbitrary list of single-plane lens models."""

    def __init__(self, lens_model_list, z_lens=None, z_source=None, lens_redshift_list=None,
                 cosmo=None, multi_plane=False, observed_convention_index=None,
                 z_source_convention=None, cosmo_interp=False, z_interp_stop=None,
                 num_z_interp=100, profile_kwargs_list=None, decouple_multi_plane=False,
                 kwargs_multiplane_model=None, distance_ratio_sampling=False,
                 cosmology_sampling=False, cosmology_model="FlatLambdaCDM"):
        if cosmology_sampling:
            raise ValueError("Cosmology sampling not supported")
        if distance_ratio_sampling:
            raise ValueError("Distance ratio sampling not supported")
        if multi_plane or decouple_multi_plane:
            raise ValueError("multi-plane lensing is not supported by this build")
        if observed_convention_index is not None:
            raise ValueError("observed_convention_index is not supported")
        if len(lens_model_list) > _lib.MAX_PROFILES:
            raise ValueError("at most %d lens profiles per model; use LensModelBulk for "
                             "many deflectors" % _lib.MAX_PROFILES)
        if z_source is not None and z_source_convention is not None and z_source != z_source_convention:
            raise ValueError("z_source != z_source_convention needs a cosmology and is not "
                             "supported by this build")
        for kw in profile_kwargs_list or []:
            if kw:
                raise ValueError("non-default profile_kwargs are not supported")
        profiles.check_names(lens_model_list, profiles.LENS_PARAMS, "Lens")
        self.lens_model_list = list(lens_model_list)
        self.z_lens = z_lens
        self.z_source = z_source
        self.redshift_list = lens_redshift_list
        self.multi_plane = False
        self.type = "SinglePlane"
        self.alpha_scaling = 1.0
        self.param_name_list = [profiles.LENS_PARAMS[n] for n in self.lens_model_list]
        self._models = {}

    def check_parameters(self, kwargs_list):
        profiles.check_parameters(self.lens_model_list, profiles.LENS_PARAMS, kwargs_list, "Lens")

    def _select(self, k):
        if k is None:
            return list(range(len(self.lens_model_list)))
        if isinstance(k, (int, np.integer)):
            return [int(k)]
        k = list(k)
        if len(k) and isinstance(k[0], (bool, np.bool_)):
            return [i for i, b in enumerate(k) if b]
        return [int(i) for i in k]

    def _model(self, idx):
        key = tuple(idx)
        if key not in self._models:
            d = _lib.ModelDesc()
            d.n_lens = len(idx)
            for j, i in enumerate(idx):
                d.lens_codes[j] = _lib.LENS_CODES[self.lens_model_list[i]]
            d.nx = d.ny = 1
            d.supersampling = 1
            d.transform_pix2angle[:] = [1.0, 0.0, 0.0, 1.0]
            d.flux_scaling = 1.0
            d.alpha_scaling = self.alpha_scaling
            d.psf_type = _lib.PSF_NONE
            d.precision = _lib.FP64
            self._models[key] = _lib.Model(d)
        return self._models[key]

    def _row(self, idx, kwargs):
        names = [self.lens_model_list[i] for i in idx]
        kws = [kwargs[i] for i in idx]
        row = np.zeros((1, profiles.n_params(names, profiles.LENS_PARAMS)))
        profiles.pack(names, profiles.LENS_PARAMS, kws, row, 0, "Lens")
        return row

    def _points(self, fn, x, y, kwargs, k):
        _device.require_cuda()
        idx = self._select(k)
        xt = _device.to_device_f64(x).reshape(-1)
        yt = _device.to_device_f64(y).reshape(-1)
        shape = np.shape(x) if not isinstance(x, torch.Tensor) else tuple(x.shape)
        ox = torch.empty_like(xt)
        oy = torch.empty_like(yt)
        if len(idx) == 0:
            if fn == "alpha":
                ox.zero_()
                oy.zero_()
            else:
                ox.copy_(xt)
                oy.copy_(yt)
        else:
            m = self._model(idx)
            p = _device.to_device_f64(self._row(idx, kwargs))
            f = getattr(_lib.load(), "lensgb_" + fn)
            _lib.check(f(m.handle, _device.ptr(p), _device.ptr(xt), _device.ptr(yt),
                         _device.ptr(ox), _device.ptr(oy), xt.numel(), _device.stream_handle()))
        return _as_out(ox.reshape(shape), x), _as_out(oy.reshape(shape), x)

    def ray_shooting(self, x, y, kwargs, k=None):
        """Maps image to source position, ``lens_model.py:237-252``."""
        return self._points("ray_shooting", x, y, kwargs, k)

    def alpha(self, x, y, kwargs, k=None):
        """Deflection angles, ``lens_model.py:353-381``."""
        return self._points("alpha", x, y, kwargs, k)

    def hessian(self, x, y, kwargs, k=None, diff=None, diff_method="square"):
        """``lens_model.py:384-414``: (f_xx, f_xy, f_yx, f_yy).  ``diff=None`` gives the
        exact second derivatives (``lensgb_hessian``: EPL, SIE, NIE, NFW, TNFW, SHEAR,
        CONVERGENCE); a step ``diff`` gives the reference's finite differences of
        ``alpha`` on a square or a cross (``:617-680``), for any profile."""
        if diff is not None:
            if diff_method == "square":
                return self._hessian_differential_square(x, y, kwargs, k, diff)
            if diff_method == "cross":
                return self._hessian_differential_cross(x, y, kwargs, k, diff)
            raise ValueError('diff_method %s not supported. Chose among "square" or "cross".'
                             % diff_method)
        _device.require_cuda()
        idx = self._select(k)
        xt = _device.to_device_f64(x).reshape(-1)
        yt = _device.to_device_f64(y).reshape(-1)
        shape = np.shape(x) if not isinstance(x, torch.Tensor) else tuple(x.shape)
        out = torch.zeros((4, xt.numel()), dtype=torch.float64, device=xt.device)
        if len(idx):
            m = self._model(idx)
            p = _device.to_device_f64(self._row(idx, kwargs))
            _lib.check(_lib.load().lensgb_hessian(
                m.handle, _device.ptr(p), 1, _device.ptr(xt), _device.ptr(yt), _device.ptr(out),
                xt.numel(), _device.stream_handle()))
        return tuple(_as_out(out[c].reshape(shape), x) for c in range(4))

    def hessian_batch(self, x, y, kwargs):
        """Exact Hessians of B systems in one launch: kwargs values of length B (or
        scalars), x and y of shape (B, n); returns four (B, n) arrays."""
        _device.require_cuda()
        idx = self._select(None)
        xa = np.asarray(x, dtype=float)
        ya = np.asarray(y, dtype=float)
        if xa.ndim != 2 or xa.shape != ya.shape:
            raise ValueError("x and y must have shape (B, n)")
        B, n = xa.shape
        names = [self.lens_model_list[i] for i in idx]
        rows = np.zeros((B, profiles.n_params(names, profiles.LENS_PARAMS)))
        profiles.pack(names, profiles.LENS_PARAMS, [kwargs[i] for i in idx], rows, 0, "Lens")
        out = torch.zeros((4, B * n), dtype=torch.float64, device="cuda")
        if len(idx):
            m = self._model(idx)
            p = _device.to_device_f64(rows)
            xt = _device.to_device_f64(xa).reshape(-1)
            yt = _device.to_device_f64(ya).reshape(-1)
            _lib.check(_lib.load().lensgb_hessian(
                m.handle, _device.ptr(p), B, _device.ptr(xt), _device.ptr(yt), _device.ptr(out),
                n, _device.stream_handle()))
        o = out.reshape(4, B, n).cpu().numpy()
        return o[0], o[1], o[2], o[3]

    def _hessian_differential_cross(self, x, y, kwargs, k=None, diff=0.00001):
        ax_dx, ay_dx = self.alpha(x + diff / 2, y, kwargs, k=k)
        ax_dy, ay_dy = self.alpha(x, y + diff / 2, kwargs, k=k)
        ax_dx_, ay_dx_ = self.alpha(x - diff / 2, y, kwargs, k=k)
        ax_dy_, ay_dy_ = self.alpha(x, y - diff / 2, kwargs, k=k)
        return ((ax_dx - ax_dx_) / diff, (ax_dy - ax_dy_) / diff, (ay_dx - ay_dx_) / diff,
                (ay_dy - ay_dy_) / diff)

    def _hessian_differential_square(self, x, y, kwargs, k=None, diff=0.00001):
        ax_pp, ay_pp = self.alpha(x + diff / 2, y + diff / 2, kwargs, k=k)
        ax_pn, ay_pn = self.alpha(x + diff / 2, y - diff / 2, kwargs, k=k)
        ax_np, ay_np = self.alpha(x - diff / 2, y + diff / 2, kwargs, k=k)
        ax_nn, ay_nn = self.alpha(x - diff / 2, y - diff / 2, kwargs, k=k)
        return ((ax_pp - ax_np + ax_pn - ax_nn) / diff / 2,
                (ax_pp - ax_pn + ax_np - ax_nn) / diff / 2,
                (ay_pp - ay_np + ay_pn - ay_nn) / diff / 2,
                (ay_pp - ay_pn + ay_np - ay_nn) / diff / 2)

    def kappa(self, x, y, kwargs, k=None, diff=None, diff_method="square"):
        """``lens_model.py:417-441``: convergence (f_xx + f_yy) / 2."""
        f_xx, _, _, f_yy = self.hessian(x, y, kwargs, k, diff, diff_method)
        return 1.0 / 2 * (f_xx + f_yy)

    def curl(self, x, y, kwargs, k=None, diff=None, diff_method="square"):
        """``lens_model.py:444-467``: f_xy - f_yx."""
        _, f_xy, f_yx, _ = self.hessian(x, y, kwargs, k, diff, diff_method)
        return f_xy - f_yx

    def gamma(self, x, y, kwargs, k=None, diff=None, diff_method="square"):
        """``lens_model.py:470-497``: shear (gamma1, gamma2)."""
        f_xx, f_xy, _, f_yy = self.hessian(x, y, kwargs, k, diff, diff_method)
        return 1.0 / 2 * (f_xx - f_yy), f_xy

    def magnification(self, x, y, kwargs, k=None, diff=None, diff_method="square"):
        """``lens_model.py:500-526``: 1 / det(1 - Hessian)."""
        f_xx, f_xy, f_yx, f_yy = self.hessian(x, y, kwargs, k, diff, diff_method)
        det_A = (1 - f_xx) * (1 - f_yy) - f_xy * f_yx
        return 1.0 / det_A
