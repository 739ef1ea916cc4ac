"""``LensModelBulk``: ray shooting through many deflectors, single- or multi-plane.

Drop-in for ``jaxtronomy.LensModel.lens_model_bulk.LensModelBulk``
(``lens_model_bulk.py:18-128``) with its two back ends:

* ``SinglePlaneBulk`` (``single_plane_bulk.py:20-131``):
  ``prepare_ray_shooting_kwargs`` builds the reference's
  ``{"all_kwargs": {name: array}, "index_list": array}`` dictionary;
  ``ray_shooting`` packs it into one row of ``LENSGB_BULK_PARAM_STRIDE``
  doubles per deflector and calls ``lensgb_bulk_ray_shooting``, which
  evaluates every (ray, deflector) pair on the GPU without materialising the
  reference's [n_deflectors, n_rays] arrays.
* ``MultiPlaneBulk`` (``multi_plane_bulk.py:11-272``):
  ``prepare_ray_shooting_kwargs`` sorts the deflectors by redshift, appends the
  source step and the NULL fillers and computes the distance lists
  (``T_ij_list``, ``T_z_list``, ``reduced2physical_factor``) from a background
  cosmology (:mod:`jaxtronomy_gb300.cosmology`) on the host, as the reference
  does outside ``jit``; ``ray_shooting`` calls
  ``lensgb_bulk_multi_plane_ray_shooting``, one thread per ray walking the
  redshift-ordered steps.

Like the reference, each deflector's arrays are bound positionally in
``param_names`` order to the profile's ``derivatives`` signature
(``_select_kwargs``, ``profile_list_base.py:768-778``).  For
EPL_MULTIPOLE_M1M3M4 the two orders differ, so in the bulk path the reference
evaluates that profile with its centre values in (a1_a, delta_phi_m1), its
multipole values shifted by two slots and (a4_a, delta_phi_m4) as the centre;
the row packing reproduces that binding so results match the reference.

``precision="fp64"`` (default) evaluates every term in FP64, like the
reference.  ``precision="fp32"`` evaluates deflectors whose deflection is
bounded by ``fp32_alpha_max`` arcsec (default 0.05: subhalos) in FP32 with
FP64-accurate accumulation, and the others (main deflectors, shear) in FP64;
in multi-plane calls CONVERGENCE sheets are evaluated as FP32-pair products.
"""

import numpy as np
import torch

from . import _device, _lib, cosmology, profiles

_NULL = "NULL"


def _as_out(t, like):
    return t if isinstance(like, torch.Tensor) else t.cpu().numpy()


class _BulkProfiles:
    """Unique profile list, kwargs row packing and the ``lensgb_bulk`` handle shared by
    the single- and multi-plane back ends (``ProfileListBase`` with the NULL filler)."""

    def __init__(self, unique_lens_model_list, profile_kwargs_list=None, precision="fp64",
                 fp32_alpha_max=None):
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
        self.precision = precision
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

    def _rows(self, all_kwargs, index_list):
        """One LENSGB_BULK_PARAM_STRIDE row per deflector, in param_names order."""
        on_dev = isinstance(index_list, torch.Tensor) or any(
            isinstance(v, torch.Tensor) for v in all_kwargs.values())
        n_unique = len(self.unique_lens_model_list)
        if on_dev:
            # one gather: S stacks the parameter arrays (plus a zero row), and
            # G[u, j] names the row of S that column j of profile u reads
            idx = _device.to_device(index_list, torch.int64).reshape(-1)
            n = idx.numel()
            names = sorted(set(q for sub in self.param_name_list for q in sub))
            S = torch.stack([_device.to_device_f64(all_kwargs[q]).reshape(-1) for q in names]
                            + [torch.zeros(n, dtype=torch.float64, device=idx.device)])
            G = np.full((n_unique + 1, _lib.BULK_PARAM_STRIDE), len(names), dtype=np.int64)
            for u, pn in enumerate(self.param_name_list[:-1]):
                for j, q in zip(self._columns[u], pn):
                    G[u, j] = names.index(q)
            G = torch.as_tensor(G, device=idx.device)
            k = idx.clamp(0, n_unique)
            rows = S.t().gather(1, G.index_select(0, k))
            return idx.to(torch.int32).contiguous(), rows.contiguous()
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

    def _coords(self, x, y):
        xt = _device.to_device_f64(x).reshape(-1)
        yt = _device.to_device_f64(y).reshape(-1)
        if xt.numel() != yt.numel():
            raise ValueError("x and y must have the same number of points")
        shape = np.shape(x) if not isinstance(x, torch.Tensor) else tuple(x.shape)
        return xt, yt, shape


class SinglePlaneBulk(_BulkProfiles):
    """``SinglePlaneBulk`` (``single_plane_bulk.py:20-131``) on the GPU."""

    def prepare_ray_shooting_kwargs(self, lens_model_list, kwargs_lens, num_deflectors=None):
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

    def ray_shooting(self, x, y, all_kwargs, index_list):
        """beta = x - sum of all deflections (single_plane_bulk.py:109-131)."""
        _device.require_cuda()
        idx, rows = self._rows(all_kwargs, index_list)
        xt, yt, shape = self._coords(x, y)
        bx = torch.empty_like(xt)
        by = torch.empty_like(yt)
        _lib.check(_lib.load().lensgb_bulk_ray_shooting(
            self._handle().handle, _device.ptr(idx), _device.ptr(rows), int(idx.numel()),
            _device.ptr(xt), _device.ptr(yt), _device.ptr(bx), _device.ptr(by), xt.numel(),
            _device.stream_handle()))
        return _as_out(bx.reshape(shape), x), _as_out(by.reshape(shape), x)


class MultiPlaneBulk(_BulkProfiles):
    """``MultiPlaneBulk`` (``multi_plane_bulk.py:11-272``) on the GPU.

    ``cosmo`` is an astropy cosmology or :class:`jaxtronomy_gb300.cosmology.FlatLambdaCDM`;
    ``None`` selects astropy's default cosmology as the reference does."""

    def __init__(self, unique_lens_model_list, profile_kwargs_list=None, cosmo=None,
                 cosmology_model="FlatLambdaCDM", precision="fp64", fp32_alpha_max=None):
        super().__init__(unique_lens_model_list, profile_kwargs_list, precision, fp32_alpha_max)
        self._cosmo_bkg = cosmology.default_background(cosmo, cosmology_model)

    def prepare_ray_shooting_kwargs(self, lens_model_list, kwargs_lens, z_source,
                                    lens_redshift_list, num_deflectors=None):
        """Redshift-sorted index list, per-parameter arrays and distance lists, the source
        step and the NULL fillers appended (multi_plane_bulk.py:57-150)."""
        if (len(lens_model_list) != len(kwargs_lens)
                or len(kwargs_lens) != len(lens_redshift_list)
                or len(lens_model_list) != len(lens_redshift_list)):
            raise ValueError(
                f"length of lens model list {len(lens_model_list)}, length of kwargs_lens "
                f"{len(kwargs_lens)}, and length of redshift list {len(lens_redshift_list)} "
                f"should match")
        if num_deflectors is None:
            num_deflectors = len(lens_model_list)
        elif num_deflectors < len(lens_model_list):
            raise ValueError(
                f"The provided num_deflectors {num_deflectors} is smaller than the length of "
                f"lens_model_list {len(lens_model_list)}")
        lens_model_list, lens_redshift_list, kwargs_lens = self._sort_lists_by_redshift(
            lens_model_list, lens_redshift_list, kwargs_lens)
        num_filler = num_deflectors - len(lens_model_list)
        index_list = [self.unique_lens_model_list.index(m) for m in lens_model_list]
        index_list += [len(self.unique_lens_model_list)] * (num_filler + 1)
        index_list = np.array(index_list, dtype=np.int64)
        unique_kwargs = sorted(set(p for sub in self.param_name_list for p in sub))
        all_kwargs = {}
        for kwarg in unique_kwargs:
            vals = [kw.get(kwarg, 0) for kw in kwargs_lens] + [0] * (num_filler + 1)
            all_kwargs[kwarg] = np.array(vals, dtype=np.float64)
        T_ij, T_z, r2p = self._set_T_zs_and_T_ijs(lens_redshift_list, z_source, self._cosmo_bkg)
        T_ij = np.array(T_ij + [0] * num_filler, dtype=np.float64)
        T_z = np.array(T_z + [T_z[-1]] * num_filler, dtype=np.float64)
        r2p = np.array(r2p + [0] * (num_filler + 1), dtype=np.float64)
        return {"all_kwargs": all_kwargs, "index_list": index_list, "T_ij_list": T_ij,
                "T_z_list": T_z, "reduced2physical_factor": r2p}

    def ray_shooting(self, alpha_x, alpha_y, all_kwargs, index_list, T_ij_list, T_z_list,
                     reduced2physical_factor):
        """Angles at the source plane of rays starting at angles (alpha_x, alpha_y)
        (multi_plane_bulk.py:152-200)."""
        _device.require_cuda()
        idx, rows = self._rows(all_kwargs, index_list)
        n_steps = int(idx.numel())
        dists = [_device.to_device_f64(v).reshape(-1)
                 for v in (T_ij_list, T_z_list, reduced2physical_factor)]
        if any(d.numel() != n_steps for d in dists):
            raise ValueError("T_ij_list, T_z_list and reduced2physical_factor need one entry "
                             "per index_list entry (%d)" % n_steps)
        xt, yt, shape = self._coords(alpha_x, alpha_y)
        bx = torch.empty_like(xt)
        by = torch.empty_like(yt)
        _lib.check(_lib.load().lensgb_bulk_multi_plane_ray_shooting(
            self._handle().handle, _device.ptr(idx), _device.ptr(rows), n_steps,
            _device.ptr(dists[0]), _device.ptr(dists[1]), _device.ptr(dists[2]),
            _device.ptr(xt), _device.ptr(yt), _device.ptr(bx), _device.ptr(by), xt.numel(),
            _device.stream_handle()))
        return _as_out(bx.reshape(shape), alpha_x), _as_out(by.reshape(shape), alpha_x)

    @staticmethod
    def _sort_lists_by_redshift(lens_model_list, lens_redshift_list, kwargs_lens):
        """Stable-order sort by increasing redshift (multi_plane_bulk.py:203-224)."""
        lens_redshift_list = np.array(lens_redshift_list)
        order = np.argsort(lens_redshift_list)
        return ([lens_model_list[i] for i in order], lens_redshift_list[order],
                [kwargs_lens[i] for i in order])

    @staticmethod
    def _set_T_zs_and_T_ijs(lens_redshift_list, z_source, cosmo_bkg):
        """Distance lists for a SORTED redshift array (multi_plane_bulk.py:226-272):
        T_ij from each step to the next (the source included), T_z from the observer,
        and the reduced-to-physical factors d_xy(0, z_s) / d_xy(z_i, z_s)."""
        z = np.asarray(lens_redshift_list, dtype=float)
        r2p = (cosmo_bkg.d_xy(0, z_source) / cosmo_bkg.d_xy(z, np.ones(z.shape) * z_source))
        T_ij, T_z = [], []
        z_before, tz = 0, 0
        for zi in np.append(z, z_source):
            if z_before == zi:
                dt = 0
            else:
                tz = cosmo_bkg.T_xy(0, zi)
                dt = cosmo_bkg.T_xy(z_before, zi)
            T_ij.append(dt)
            T_z.append(tz)
            z_before = zi
        return T_ij, T_z, np.asarray(r2p, dtype=float).reshape(-1).tolist()


class LensModelBulk:
    """Many-deflector lens model (``lens_model_bulk.py:10-128``): ``SinglePlaneBulk``
    or, with ``multi_plane=True``, ``MultiPlaneBulk``."""

    def __init__(self, unique_lens_model_list, multi_plane=False, profile_kwargs_list=None,
                 cosmo=None, cosmology_model="FlatLambdaCDM", precision="fp64",
                 fp32_alpha_max=None):
        if multi_plane:
            self.lens_model = MultiPlaneBulk(unique_lens_model_list, profile_kwargs_list, cosmo,
                                             cosmology_model, precision, fp32_alpha_max)
            self.type = "MultiPlaneBulk"
        else:
            self.lens_model = SinglePlaneBulk(unique_lens_model_list, profile_kwargs_list,
                                              precision, fp32_alpha_max)
            self.type = "SinglePlaneBulk"
        self.profile_kwargs_list = self.lens_model.profile_kwargs_list
        self.unique_lens_model_list = self.lens_model.unique_lens_model_list
        self.precision = precision
        self.init_kwargs = {
            "unique_lens_model_list": unique_lens_model_list,
            "cosmo": cosmo,
            "multi_plane": multi_plane,
            "profile_kwargs_list": profile_kwargs_list,
            "cosmology_model": cosmology_model,
        }

    def prepare_ray_shooting_kwargs(self, lens_model_list, kwargs_lens, z_source=None,
                                    lens_redshift_list=None, num_deflectors=None):
        """``lens_model_bulk.py:65-111``; multi-plane mode needs the redshifts."""
        if self.type == "MultiPlaneBulk":
            if lens_redshift_list is None:
                raise ValueError("In multi-plane lensing, you need to specify the redshifts of "
                                 "the lensing planes.")
            if z_source is None:
                raise ValueError("z_source needs to be set for multi-plane lens modelling.")
            return self.lens_model.prepare_ray_shooting_kwargs(
                lens_model_list, kwargs_lens, z_source, lens_redshift_list, num_deflectors)
        return self.lens_model.prepare_ray_shooting_kwargs(lens_model_list, kwargs_lens,
                                                           num_deflectors)

    def ray_shooting(self, x, y, ray_shooting_kwargs):
        """Source-plane positions of image-plane positions (x, y) (lens_model_bulk.py:113-128)."""
        return self.lens_model.ray_shooting(x, y, **ray_shooting_kwargs)

    def pack_rows(self, all_kwargs, index_list):
        """Host packing: (int32 index list, [n_deflectors, LENSGB_BULK_PARAM_STRIDE] rows)."""
        return self.lens_model.pack_rows(all_kwargs, index_list)
