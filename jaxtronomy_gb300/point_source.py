"""``PointSource`` with the point-source types JAXtronomy implements.

Drop-in for ``jaxtronomy.PointSource.point_source.PointSource``
(``PointSource/point_source.py:12-115``) with ``LENSED_POSITION``
(``Types/lensed_position.py``: image positions ``ra_image``, ``dec_image`` and
amplitudes ``point_amp`` given) and ``UNLENSED`` (``Types/unlensed.py``).  The
reference raises for ``SOURCE_POSITION``, for additional images (both need
the lens-equation solver) and for ``save_cache``; this library raises in the
same places.  ``fixed_magnification`` LENSED_POSITION models take
``source_amp`` and give each image ``source_amp * |magnification|``, the
magnification from the lens model's exact Hessian (``LensModel.magnification``).

Kwargs values may be arrays of shape (n_images,) for one system or
(B, n_images) for a batch.
"""

import numpy as np

_SUPPORTED_MODELS = ["LENSED_POSITION", "UNLENSED"]


class PointSource:
    """Point-source model list (``point_source.py:12-115``)."""

    def __init__(self, point_source_type_list, lens_model=None, fixed_magnification_list=None,
                 additional_images_list=None, flux_from_point_source_list=None,
                 magnification_limit=None, save_cache=False, kwargs_lens_eqn_solver=None,
                 index_lens_model_list=None, point_source_frame_list=None, redshift_list=None):
        if "LENSED_POSITION" in point_source_type_list:
            if index_lens_model_list is not None and point_source_frame_list is None:
                raise ValueError("with specified index_lens_model_list, a specified "
                                 "point_source_frame_list argument is required for "
                                 "LENSED_POSITION")
            if index_lens_model_list is None:
                point_source_frame_list = [None] * len(point_source_type_list)
        if save_cache:
            raise ValueError("saving cache is not supported in jaxtronomy")
        if index_lens_model_list is not None:
            raise ValueError("index_lens_model_list (multi-band lens subsets) is not supported")
        n = len(point_source_type_list)
        self._lens_model = lens_model
        self.point_source_type_list = list(point_source_type_list)
        self._fixed_magnification_list = (list(fixed_magnification_list)
                                          if fixed_magnification_list is not None else [False] * n)
        self._additional_images_list = (list(additional_images_list)
                                        if additional_images_list is not None else [False] * n)
        self._flux_from_point_source_list = (list(flux_from_point_source_list)
                                             if flux_from_point_source_list is not None
                                             else [True] * n)
        self._redshift_list = list(redshift_list) if redshift_list is not None else [None] * n
        self._index_lens_model_list = index_lens_model_list
        self._point_source_frame_list = point_source_frame_list
        self._magnification_limit = magnification_limit
        self._kwargs_lens_eqn_solver = kwargs_lens_eqn_solver or {}
        self._save_cache = save_cache
        for i, model in enumerate(self.point_source_type_list):
            if model == "SOURCE_POSITION":
                raise ValueError("source position not supported in jaxtronomy")
            if model not in _SUPPORTED_MODELS:
                raise ValueError("Point-source model %s not available. Supported models are %s ."
                                 % (model, _SUPPORTED_MODELS))

    def _check(self, kwargs_ps):
        if len(kwargs_ps) != len(self.point_source_type_list):
            raise ValueError("kwargs_ps needs one dict per point-source model")
        for i in range(len(kwargs_ps)):
            if self.point_source_type_list[i] == "LENSED_POSITION" and \
                    self._additional_images_list[i]:
                raise ValueError("additional images not supported in jaxtronomy")

    def image_position(self, kwargs_ps, kwargs_lens=None, k=None, original_position=False,
                       additional_images=False):
        """``point_source.py:205-253``: per model, the image positions (arrays)."""
        if additional_images:
            raise ValueError("additional images not supported in jaxtronomy")
        self._check(kwargs_ps)
        ra, dec = [], []
        for i, kw in enumerate(kwargs_ps):
            if k is None or k == i:
                ra.append(np.asarray(kw["ra_image"], dtype=float))
                dec.append(np.asarray(kw["dec_image"], dtype=float))
        return ra, dec

    def fixed_magnification(self, i):
        return (self.point_source_type_list[i] == "LENSED_POSITION"
                and bool(self._fixed_magnification_list[i]))

    def magnification(self, ra, dec, kwargs_lens):
        """|magnification| of the lens model at image positions of shape (n,) or
        (B, n); batched lens kwargs are evaluated system by system."""
        if self._lens_model is None:
            raise ValueError("fixed_magnification needs the lens model (PointSource(..., "
                             "lens_model=...) or an ImageModel)")
        ra = np.asarray(ra, dtype=float)
        dec = np.asarray(dec, dtype=float)
        sizes = [np.size(v) for kw in (kwargs_lens or []) for v in kw.values()]
        B = max(sizes + [1])
        if ra.ndim == 2:
            B = max(B, ra.shape[0])
        if B == 1 and ra.ndim == 1:
            return np.abs(np.asarray(self._lens_model.magnification(ra, dec, kwargs_lens)))
        ra2 = np.broadcast_to(np.atleast_2d(ra), (B, ra.shape[-1]))
        dec2 = np.broadcast_to(np.atleast_2d(dec), (B, dec.shape[-1]))
        # one Hessian launch for the batch (lensgb_hessian with B parameter rows)
        f_xx, f_xy, f_yx, f_yy = self._lens_model.hessian_batch(ra2, dec2, kwargs_lens)
        return np.abs(1.0 / ((1 - f_xx) * (1 - f_yy) - f_xy * f_yx))

    def image_amplitude(self, kwargs_ps, kwargs_lens=None, k=None):
        """``point_source.py:304-326``: per model, the image amplitudes (zeros where
        flux_from_point_source is False; ``source_amp * |mag|`` with fixed
        magnification, ``Types/lensed_position.py:134-177``)."""
        self._check(kwargs_ps)
        out = []
        for i, kw in enumerate(kwargs_ps):
            if k is None or k == i:
                if self.fixed_magnification(i):
                    mag = self.magnification(kw["ra_image"], kw["dec_image"], kwargs_lens)
                    sa = np.asarray(kw["source_amp"], dtype=float)
                    amp = (sa[..., None] if sa.ndim else sa) * mag
                else:
                    amp = np.asarray(kw["point_amp"], dtype=float)
                out.append(amp if self._flux_from_point_source_list[i] else np.zeros_like(amp))
        return out

    def source_amplitude(self, kwargs_ps, kwargs_lens=None):
        """Intrinsic amplitudes: ``point_amp`` of every model (``Types/unlensed.py``;
        LENSED_POSITION without fixed magnification returns its image amplitudes)."""
        self._check(kwargs_ps)
        return [np.asarray(kw["point_amp"], dtype=float) for kw in kwargs_ps]

    def point_source_list(self, kwargs_ps, kwargs_lens=None, k=None, with_amp=True):
        """``point_source.py:255-284``: (ra, dec, amp) of every image of the selected
        models, concatenated along the last axis (shape (n,) or (B, n))."""
        ra, dec = self.image_position(kwargs_ps, kwargs_lens, k=k)
        if with_amp:
            amp = self.image_amplitude(kwargs_ps, kwargs_lens, k=k)
        else:
            amp = [np.ones_like(r) for r in ra]
        if not ra:
            e = np.zeros(0)
            return e, e, e
        ra, dec, amp = np.broadcast_arrays(_cat(ra), _cat(dec), _cat(amp))
        return ra, dec, amp

    def num_basis(self, kwargs_ps, kwargs_lens=None):
        """``point_source.py:286-302``: number of linear amplitudes."""
        ra, _ = self.image_position(kwargs_ps, kwargs_lens)
        return int(sum((1 if self.fixed_magnification(i) else
                        (np.shape(r)[-1] if np.ndim(r) else 1))
                       for i, r in enumerate(ra) if self._flux_from_point_source_list[i]))

    def check_positive_flux(self, kwargs_ps):
        """``point_source.py:488-502``: True when no ``point_amp`` is negative."""
        return all(np.all(np.asarray(kw[key]) >= 0) for kw in kwargs_ps
                   for key in ("point_amp", "source_amp") if key in kw)


def _cat(arrays):
    """Concatenate per-model arrays of shape (n_i,) or (B, n_i) along the image axis."""
    arrays = [np.atleast_1d(np.asarray(a, dtype=float)) for a in arrays]
    if any(a.ndim == 2 for a in arrays):
        B = max(a.shape[0] for a in arrays if a.ndim == 2)
        arrays = [a if a.ndim == 2 and a.shape[0] == B else np.broadcast_to(a, (B, a.shape[-1]))
                  for a in arrays]
    return np.concatenate(arrays, axis=-1)
