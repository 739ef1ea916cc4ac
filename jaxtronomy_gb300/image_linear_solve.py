"""ImageModel with the linear amplitude solve (``ImSim/image_linear_solve.py:11-740``).

Every light profile of this library (SERSIC, SERSIC_ELLIPSE) has one linear
amplitude, ``amp``.  For a batch of systems the unit-amplitude convolved image
of each linear component is one ``lensgb_image`` launch of that component alone
(``linear_response_matrix``, ``image_linear_solve.py:362-456``); one
``lensgb_linear_solve`` launch then forms and solves the weighted least-squares
system of every system (``de_lens.get_param_WLS``, ``de_lens.py:8-38``), writes
the model images and their log-likelihoods (``likelihood_data_given_model``,
``:229-341``).  Point images (LENSED_POSITION / UNLENSED models whose flux comes
from the point source) add one response row each: the image rendered alone at
amp = 1 (``:440-456``), so their ``point_amp`` are solved too.
"""

import ctypes

import numpy as np
import torch

from . import _device, _lib
from .image_model import ImageModel


class ImageLinearFit(ImageModel):
    """Linear version of :class:`ImageModel` (``image_linear_solve.py:11-97``)."""

    def __init__(self, data_class, psf_class, lens_model_class=None, source_model_class=None,
                 lens_light_model_class=None, point_source_class=None, extinction_class=None,
                 kwargs_numerics=None, likelihood_mask=None, psf_error_map_bool_list=None,
                 kwargs_pixelbased=None):
        super().__init__(data_class, psf_class, lens_model_class, source_model_class,
                         lens_light_model_class, point_source_class, extinction_class,
                         kwargs_numerics, likelihood_mask, psf_error_map_bool_list,
                         kwargs_pixelbased)
        self._n_src = len(self.SourceModel.profile_type_list)
        self._n_ll = len(self.LensLightModel.profile_type_list)
        if self._n_src + self._n_ll > _lib.LINEAR_MAX:
            raise ValueError("at most %d linear light components are supported"
                             % _lib.LINEAR_MAX)

    def _ps_linear(self, kwargs_ps, kwargs_special=None, kwargs_lens=None):
        """Response rows of the point sources with linear amplitudes
        (``PointSource.linear_response_set``, point_source.py:347-384): one row per
        image (amp 1), or one row per fixed-magnification model (all its images,
        amp |mag|); positions shifted as ``point_source_linear_response_set`` does
        (``image_linear_solve.py:559-600``, image by image in row order).  Each row
        is [ra, dec, amp] arrays of shape (B or 1, n_row)."""
        if not self._n_ps:
            return []
        ps = self.PointSource
        ra, dec = ps.image_position(kwargs_ps)
        out = []
        for k, (r, d) in enumerate(zip(ra, dec)):
            if not ps._flux_from_point_source_list[k]:
                continue
            r = np.atleast_2d(r)
            d = np.atleast_2d(d)
            if ps.fixed_magnification(k):
                mag = np.atleast_2d(ps.magnification(kwargs_ps[k]["ra_image"],
                                                     kwargs_ps[k]["dec_image"], kwargs_lens))
                out.append([r.copy(), d.copy(), mag])
            else:
                for j in range(r.shape[-1]):
                    out.append([r[:, j:j + 1].copy(), d[:, j:j + 1].copy(),
                                np.ones((1, 1))])
        if kwargs_special is not None and "delta_x_image" in kwargs_special:
            dx = np.atleast_2d(np.asarray(kwargs_special["delta_x_image"], dtype=float))
            dy = np.atleast_2d(np.asarray(kwargs_special["delta_y_image"], dtype=float))
            q = 0
            for row in out:
                for j in range(row[0].shape[-1]):
                    if q >= dx.shape[-1]:
                        break
                    row[0] = row[0] + np.eye(row[0].shape[-1])[j] * dx[..., q:q + 1]
                    row[1] = row[1] + np.eye(row[1].shape[-1])[j] * dy[..., q:q + 1]
                    q += 1
        return out

    # ------------------------------------------------------------------ linear parameters
    def num_param_linear(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                         kwargs_ps=None):
        """``image_linear_solve.py:342-360``: one amplitude per light profile and per
        point image with flux from the point source."""
        n_ps = self.PointSource.num_basis(kwargs_ps) if self._n_ps and kwargs_ps else 0
        return self._n_src + self._n_ll + n_ps

    def linear_param_from_kwargs(self, kwargs_source, kwargs_lens_light, kwargs_ps=None):
        """``image_linear_solve.py:484-528``: the amplitudes, sources, lens light, then
        the point images' ``point_amp``."""
        out = [kw["amp"] for kw in (kwargs_source or [])] + [
            kw["amp"] for kw in (kwargs_lens_light or [])]
        for k, kw in enumerate(kwargs_ps or []):
            if self.PointSource._flux_from_point_source_list[k]:
                if self.PointSource.fixed_magnification(k):
                    out.append(kw["source_amp"])
                else:
                    out += list(np.atleast_1d(kw["point_amp"]))
        return out

    def update_linear_kwargs(self, param, kwargs_lens, kwargs_source, kwargs_lens_light,
                             kwargs_ps=None):
        """``image_linear_solve.py:458-482``: writes the amplitudes into the kwargs
        (in place, as the reference's LightModel.update_linear does) and returns them."""
        p = np.asarray(param, dtype=float)
        for i, kw in enumerate(kwargs_source or []):
            kw["amp"] = p[..., i]
        for i, kw in enumerate(kwargs_lens_light or []):
            kw["amp"] = p[..., self._n_src + i]
        c = self._n_src + self._n_ll
        for k, kw in enumerate(kwargs_ps or []):
            if self.PointSource._flux_from_point_source_list[k]:
                if self.PointSource.fixed_magnification(k):
                    kw["source_amp"] = p[..., c]
                    c += 1
                    continue
                n = np.shape(kw["ra_image"])[-1]
                kw["point_amp"] = p[..., c:c + n]
                c += n
        return kwargs_lens, kwargs_source, kwargs_lens_light, kwargs_ps

    def check_positive_flux(self, kwargs_source, kwargs_lens_light, kwargs_ps=None):
        """``image_linear_solve.py:598-618``: True when no amplitude is negative."""
        amps = np.asarray(self.linear_param_from_kwargs(kwargs_source, kwargs_lens_light),
                          dtype=float)
        ok = bool(np.all(amps >= 0))
        if self._n_ps and kwargs_ps:
            ok = ok and self.PointSource.check_positive_flux(kwargs_ps)
        return ok

    # ------------------------------------------------------------------ response
    def linear_response_batch(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                              unconvolved=False, psf_kernels=None, stream=None, kwargs_ps=None,
                              kwargs_special=None):
        """(n_linear, B, ny, nx) CUDA tensor of unit-amplitude component images:
        each source lensed alone, each lens-light profile alone, amp = 1, then each
        point image alone at amp = 1 without the flux scaling (image_linear_solve.py:
        440-456)."""
        ps_pos = self._ps_linear(kwargs_ps, kwargs_special, kwargs_lens)
        if self._n_src + self._n_ll + len(ps_pos) > _lib.LINEAR_MAX:
            raise ValueError("at most %d linear amplitudes are supported" % _lib.LINEAR_MAX)
        n_lens = len(self.LensModel.lens_model_list)
        unit = lambda kws: [dict(kw, amp=1.0) for kw in (kws or [])]  # noqa: E731
        ks, kll = unit(kwargs_source), unit(kwargs_lens_light)
        jobs = [((range(n_lens), [j], []), True) for j in range(self._n_src)]
        jobs += [(([], [], [j]), False) for j in range(self._n_ll)]
        flags = _lib.UNCONVOLVED if unconvolved else 0
        rows = [self.pack_params(kwargs_lens, ks, kll, lens_idx=list(li), src_idx=si,
                                 ll_idx=lli, lensed=lensed)
                for (li, si, lli), lensed in jobs]
        # the batch of the whole kwargs (a lens-light row alone does not see batched lens
        # kwargs): rows of one system are repeated
        B = max([r.shape[0] for r in rows] + [max(p[0].shape[0], p[2].shape[0]) for p in ps_pos]
                + [1])
        A = torch.empty((len(jobs) + len(ps_pos), B, self._nx, self._ny), dtype=self._dtype,
                        device="cuda")
        for c, ((li, si, lli), lensed) in enumerate(jobs):
            r = rows[c] if rows[c].shape[0] == B else np.repeat(rows[c], B, axis=0)
            model = self._model(li, si, lli, lensed=lensed)
            self._launch(model, _device.to_device_f64(r), B, flags, psf_kernels, A[c], stream)
        # the renderer applies the model's flux scaling; the response rows have none
        unit = 1.0 / self._flux_scaling
        for j, (ra, dec, amp) in enumerate(ps_pos):
            row = A[len(jobs) + j]
            row.zero_()
            m = ra.shape[-1]
            pts = np.stack([np.broadcast_to(ra, (B, m)), np.broadcast_to(dec, (B, m)),
                            np.broadcast_to(amp, (B, m)) * unit], axis=-1)
            self._render_point_rows(row, np.ascontiguousarray(pts), False, psf_kernels, stream)
        return A

    def linear_response_matrix(self, kwargs_lens, kwargs_source, kwargs_lens_light,
                               kwargs_ps=None, kwargs_extinction=None, kwargs_special=None,
                               unconvolved=False):
        """``image_linear_solve.py:362-456``: (num_param, num_data_evaluate) response
        of one system (the unit-amplitude images at the mask pixels)."""
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        A = self.linear_response_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                       unconvolved=unconvolved, kwargs_ps=kwargs_ps,
                                       kwargs_special=kwargs_special)
        a = A[:, 0].to(torch.float64).cpu().numpy()
        return np.nan_to_num(a[:, self.likelihood_mask])

    # ------------------------------------------------------------------ solve
    def likelihood_linear_batch(self, kwargs_lens=None, kwargs_source=None,
                                kwargs_lens_light=None, data=None, source_marg=False,
                                check_positive_flux=False, psf_kernels=None, stream=None,
                                kwargs_ps=None, kwargs_special=None):
        """Linear solve of B systems: ((B,) logL, (B, n) amplitudes, (B, ny, nx) model
        images, (B, n, n) inverse normal matrices or None) as CUDA tensors (FP64;
        images in the model precision)."""
        A = self.linear_response_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                       psf_kernels=psf_kernels, stream=stream,
                                       kwargs_ps=kwargs_ps, kwargs_special=kwargs_special)
        n, B = A.shape[0], A.shape[1]
        nt = self._noise_tensors(data)
        nd = self._noise_desc(nt)
        param = torch.empty((B, n), dtype=torch.float64, device="cuda")
        cov = torch.empty((B, n, n), dtype=torch.float64, device="cuda") if source_marg else None
        image = torch.empty((B, self._nx, self._ny), dtype=self._dtype, device="cuda")
        logl = torch.empty((B,), dtype=torch.float64, device="cuda")
        flags = ((_lib.LINEAR_INVERSE if source_marg else 0)
                 | (_lib.LINEAR_POSITIVE if check_positive_flux else 0))
        model = self._model(range(len(self.LensModel.lens_model_list)), range(self._n_src),
                            range(self._n_ll))
        _lib.check(_lib.load().lensgb_linear_solve(
            model.handle, _device.ptr(A), n, B, ctypes.byref(nd), flags, _device.ptr(param),
            ctypes.c_void_p(0) if cov is None else _device.ptr(cov), _device.ptr(image),
            _device.ptr(logl), _device.stream_handle(stream)))
        return logl, param, image, cov

    def image_linear_solve(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                           kwargs_ps=None, kwargs_extinction=None, kwargs_special=None,
                           inv_bool=False):
        """``image_linear_solve.py:98-228``: (model image, model error, covariance of
        the amplitudes or None, amplitudes); the amplitudes are written into the
        kwargs as the reference does."""
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        logl, param, image, cov = self.likelihood_linear_batch(
            kwargs_lens, kwargs_source, kwargs_lens_light, source_marg=inv_bool,
            kwargs_ps=kwargs_ps, kwargs_special=kwargs_special)
        p = param[0].cpu().numpy()
        self.update_linear_kwargs(p, kwargs_lens, kwargs_source, kwargs_lens_light, kwargs_ps)
        return (image[0].to(torch.float64).cpu().numpy(), 0,
                None if cov is None else cov[0].cpu().numpy(), p)

    def likelihood_data_given_model(self, kwargs_lens=None, kwargs_source=None,
                                    kwargs_lens_light=None, kwargs_ps=None,
                                    kwargs_extinction=None, kwargs_special=None,
                                    source_marg=False, linear_prior=None,
                                    check_positive_flux=False):
        """``image_linear_solve.py:229-341``: (logL, amplitudes) after the linear solve."""
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        if linear_prior is not None:
            raise ValueError("linear_prior (marginalization_new) is not supported; use "
                             "source_marg with flat priors")
        logl, param, _, _ = self.likelihood_linear_batch(
            kwargs_lens, kwargs_source, kwargs_lens_light, source_marg=source_marg,
            check_positive_flux=check_positive_flux, kwargs_ps=kwargs_ps,
            kwargs_special=kwargs_special)
        p = param[0].cpu().numpy()
        self.update_linear_kwargs(p, kwargs_lens, kwargs_source, kwargs_lens_light, kwargs_ps)
        return float(logl[0].cpu()), p
