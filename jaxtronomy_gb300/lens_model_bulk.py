"""``LensModelBulk``: single-plane ray shooting through many deflectors.

Drop-in for ``jaxtronomy.LensModel.lens_model_bulk.LensModelBulk``
(``lens_model_bulk.py:18-128``) in its single-plane mode, ``SinglePlaneBulk``
(``single_plane_bulk.py:20-131``).  ``prepare_ray_shooting_kwargs`` builds the
same ``{"all_kwargs": {name: array}, "index_list": array}`` dictionary as the
reference; ``ray_shooting`` packs it into one row of
``LENSGB_BULK_PARAM_STRIDE`` doubles per deflector and calls
``lensgb_bulk_ray_shooting``, which evaluates every (ray, deflector) pair on the
GPU without materialising the reference's [n_deflectors, n_rays] arrays.

Like the reference, each deflector's arrays are bound positionally in
``param_names`` order to the profile's ``derivatives`` signature
(``_select_kwargs``, ``profile_list_base.py:768-778``).  For
EPL_MULTIPOLE_M1M3M4 the two orders differ, so in the bulk path the reference
evaluates that profile with its centre values in (a1_a, delta_phi_m1), its
multipole values shifted by two slots and (a4_a, delta_phi_m4) as the centre;
``ray_shooting`` reproduces that binding so results match the reference.

``precision="fp64"`` (default) evaluates every term in FP64, like the
reference.  ``precision="fp32"`` evaluates deflectors whose deflection is
bounded by ``fp32_alpha_max`` arcsec (default 0.05: subhalos) in FP32 with
FP64 accumulation, and the others (main deflectors, shear) in FP64.
"""

import numpy as np
import torch

from . import _device, _lib, profiles

_NULL = "NULL"


def _as_out(t, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


class LensModelBulk:
    """Many-deflector single-plane lens model (``LensModelBulk`` with multi_plane=False)."""

    def __init__(self, unique_lens_model_list, multi_plane=False, profile_kwargs_list=None,
                 cosmo=None, cosmology_model="FlatLambdaCDM", precision="fp64",
                 fp32_alpha_max=None):
        if multi_plane:
            raise ValueError("multi-plane bulk ray shooting (MultiPlaneBulk) is not supported "
                             "by this build")
        unique = list(unique_lens_model_list)
        if len(unique) > _lib.BULK_MAX_UNIQUE:
            raise ValueError("at most %d unique lens models" % _lib.BULK_MAX_UNIQUE)
        names = [n for n in unique if n != _NULL]
        profiles.check_names(names, profiles.LENS_PARAMS, "Lens")
        if profile_kwargs_list is None:
            profile_kwargs_list = [{} for _ in range(len(unique))]
        for kw in profile_kwargs_list:
            if kw:
                raise ValueError("non-default profile_kwargs are not supported")
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.profile_kwargs_list = profile_kwargs_list
        self.unique_lens_model_list = unique
        self.type = "SinglePlaneBulk"
        self.precision = precision
        self.init_kwargs = {
            "unique_lens_model_list": unique_lens_model_list,
            "cosmo": cosmo,
            "multi_plane": multi_plane,
            "profile_kwargs_list": profile_kwargs_list,
            "cosmology_model": cosmology_model,
        }
        # param names per unique model, then the NULL filler (single_plane_bulk.py:33-39)
        self.param_name_list = [profiles.LENS_PARAMS[n] if n != _NULL else [] for n in unique]
        self.param_name_list.append([])
        self._codes = [_lib.LENS_CODES[n] if n != _NULL else _lib.LENS_NULL for n in unique]
        # row column (param_names slot read by the kernel) that receives the
        # k-th param_names array under the reference's positional binding
        self._columns = []
        for n, names in zip(unique, self.param_name_list):
            sig = profiles.DERIVATIVES_SIGNATURE.get(n, names)
            self._columns.append([names.index(sig[k]) for k in range(len(names))])
        self._fp32_alpha_max = fp32_alpha_max
        self._bulk = None

    def _handle(self):
        if self._bulk is None:
            prec = _lib.FP32_SPLIT if self.precision == "fp32" else _lib.FP64
            self._bulk = _lib.Bulk(self._codes, prec, self._fp32_alpha_max)
        return self._bulk

    def prepare_ray_shooting_kwargs(self, lens_model_list, kwargs_lens, z_source=None,
                                    lens_redshift_list=None, num_deflectors=None):
        """Index list and per-parameter arrays (single_plane_bulk.py:47-106)."""
        if len(lens_model_list) != len(kwargs_lens):
            raise ValueError(
                f"length of lens model list {len(lens_model_list)} and length of kwargs_lens "
                f"{len(kwargs_lens)} do not match")
        if num_deflectors is None:
            num_deflectors = len(lens_model_list)
        elif num_deflectors < len(lens_model_list):
            raise ValueError(
                f"The provided num_deflectors {num_deflectors} is smaller than the length of "
                f"lens_model_list {len(lens_model_list)}")
        num_filler = num_deflectors - len(kwargs_lens)
        index_list = [self.unique_lens_model_list.index(m) for m in lens_model_list]
        index_list += [len(self.unique_lens_model_list)] * num_filler
        index_list = np.array(index_list, dtype=np.int64)
        unique_kwargs = sorted(set(p for sub in self.param_name_list for p in sub))
        all_kwargs = {}
        for kwarg in unique_kwargs:
            vals = [kw.get(kwarg, 0) for kw in kwargs_lens] + [0] * num_filler
            all_kwargs[kwarg] = np.array(vals, dtype=np.float64)
        return {"all_kwargs": all_kwargs, "index_list": index_list}

    def _rows(self, all_kwargs, index_list):
        """One LENSGB_BULK_PARAM_STRIDE row per deflector, in param_names order."""
        on_dev = isinstance(index_list, torch.Tensor) or any(
            isinstance(v, torch.Tensor) for v in all_kwargs.values())
        n_unique = len(self.unique_lens_model_list)
        if on_dev:
            idx = _device.to_device(index_list, torch.int64).reshape(-1)
            n = idx.numel()
            rows = torch.zeros((n, _lib.BULK_PARAM_STRIDE), dtype=torch.float64, device=idx.device)
            k = idx.clamp(0, n_unique)
            for u, names in enumerate(self.param_name_list[:-1]):
                sel = k == u
                for j, p in zip(self._columns[u], names):
                    v = _device.to_device_f64(all_kwargs[p]).reshape(-1)
                    rows[:, j] = torch.where(sel, v, rows[:, j])
            return idx.to(torch.int32).contiguous(), rows
        idx, rows = self.pack_rows(all_kwargs, index_list)
        return _device.to_device(idx, torch.int32), _device.to_device_f64(rows)

    def pack_rows(self, all_kwargs, index_list):
        """Host packing: (int32 index list, [n_deflectors, LENSGB_BULK_PARAM_STRIDE] rows)."""
        idx = np.asarray(index_list, dtype=np.int64).reshape(-1)
        n = idx.size
        rows = np.zeros((n, _lib.BULK_PARAM_STRIDE))
        k = np.clip(idx, 0, len(self.unique_lens_model_list))
        for u, names in enumerate(self.param_name_list[:-1]):
            sel = k == u
            if not sel.any():
                continue
            for j, p in zip(self._columns[u], names):
                rows[sel, j] = np.asarray(all_kwargs[p], dtype=np.float64).reshape(-1)[sel]
        return idx.astype(np.int32), rows

    def ray_shooting(self, x, y, ray_shooting_kwargs):
        """beta = x - sum of all deflections (single_plane_bulk.py:109-131)."""
        _device.require_cuda()
        kw = ray_shooting_kwargs
        idx, rows = self._rows(kw["all_kwargs"], kw["index_list"])
        xt = _device.to_device_f64(x).reshape(-1)
        yt = _device.to_device_f64(y).reshape(-1)
        if xt.numel() != yt.numel():
            raise ValueError("x and y must have the same number of points")
        shape = np.shape(x) if not isinstance(x, torch.Tensor) else tuple(x.shape)
        bx = torch.empty_like(xt)
        by = torch.empty_like(yt)
        _lib.check(_lib.load().lensgb_bulk_ray_shooting(
            self._handle().handle, _device.ptr(idx), _device.ptr(rows), int(idx.numel()),
            _device.ptr(xt), _device.ptr(yt), _device.ptr(bx), _device.ptr(by), xt.numel(),
            _device.stream_handle()))
        return _as_out(bx.reshape(shape), x), _as_out(by.reshape(shape), x)
