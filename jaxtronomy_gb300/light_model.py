"""``LightModel``: surface brightness of a list of light profiles.

Drop-in for ``jaxtronomy.LightModel.light_model.LightModel``
(``light_model.py:9-51``, ``light_model_base.py:63-252``).  Evaluation runs in
liblensgb.so on the GPU in FP64.
"""

import numpy as np
import torch

from . import _device, _lib, profiles


class LightModel:
    """Class to handle source and lens light models."""

    def __init__(self, light_model_list, deflection_scaling_list=None, source_redshift_list=None,
                 profile_kwargs_list=None):
        if source_redshift_list is not None and source_redshift_list != []:
            raise ValueError("multi plane sources not supported, source_redshift_list must be None")
        if len(light_model_list) > _lib.MAX_PROFILES:
            raise ValueError("at most %d light profiles per model" % _lib.MAX_PROFILES)
        for kw in profile_kwargs_list or []:
            if kw:
                raise ValueError("non-default profile_kwargs are not supported")
        profiles.check_names(light_model_list, profiles.LIGHT_PARAMS, "Light")
        self.profile_type_list = list(light_model_list)
        self.deflection_scaling_list = deflection_scaling_list
        if deflection_scaling_list is not None and len(deflection_scaling_list) != len(light_model_list):
            raise ValueError("deflection_scaling_list must have one entry per light profile")
        self.redshift_list = source_redshift_list
        self.param_name_list = [profiles.LIGHT_PARAMS[n] for n in self.profile_type_list]
        self._models = {}

    def check_parameters(self, kwargs_list):
        profiles.check_parameters(self.profile_type_list, profiles.LIGHT_PARAMS, kwargs_list,
                                  "Light")

    def _select(self, k):
        if k is None:
            return list(range(len(self.profile_type_list)))
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
            d.n_source = len(idx)
            for j, i in enumerate(idx):
                d.source_codes[j] = _lib.LIGHT_CODES[self.profile_type_list[i]]
                d.deflection_scaling[j] = 1.0
            d.nx = d.ny = 1
            d.supersampling = 1
            d.transform_pix2angle[:] = [1.0, 0.0, 0.0, 1.0]
            d.flux_scaling = 1.0
            d.alpha_scaling = 1.0
            d.psf_type = _lib.PSF_NONE
            d.precision = _lib.FP64
            self._models[key] = _lib.Model(d)
        return self._models[key]

    def surface_brightness(self, x, y, kwargs_list, k=None):
        """``light_model_base.py:230-252``."""
        _device.require_cuda()
        idx = self._select(k)
        xt = _device.to_device_f64(x).reshape(-1)
        yt = _device.to_device_f64(y).reshape(-1)
        shape = np.shape(x) if not isinstance(x, torch.Tensor) else tuple(x.shape)
        out = torch.zeros_like(xt)
        if len(idx):
            names = [self.profile_type_list[i] for i in idx]
            row = np.zeros((1, profiles.n_params(names, profiles.LIGHT_PARAMS)))
            profiles.pack(names, profiles.LIGHT_PARAMS, [kwargs_list[i] for i in idx], row, 0,
                          "Light")
            m = self._model(idx)
            p = _device.to_device_f64(row)
            _lib.check(_lib.load().lensgb_surface_brightness(
                m.handle, 0, _device.ptr(p), _device.ptr(xt), _device.ptr(yt), _device.ptr(out),
                xt.numel(), _device.stream_handle()))
        out = out.reshape(shape)
        return out if isinstance(x, torch.Tensor) else out.cpu().numpy()
