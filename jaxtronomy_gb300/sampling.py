"""Batched likelihood for samplers.

The reference's sampling path evaluates one parameter vector per call --
``LikelihoodModule.logL`` (``Sampling/likelihood.py:294-372``) ->
``ImageLikelihood.logL`` (``Sampling/Likelihoods/image_likelihood.py:57-97``) ->
``ImageModel.likelihood_data_given_model`` (``ImSim/image_model.py:163-221``) --
and ``prepare_logL_func`` (``Sampling/sampler.py:215-250``) vectorises it with
``jax.vmap`` for an ensemble of walkers.  Here ``LikelihoodModule.logL_batch``
takes the whole ensemble and evaluates it as one batched ``lensgb_loglike``
launch; ``prepare_logL_func("gpu", module.logL)`` returns that batched function.

With the linear solver (the reference's default) ``ImageLikelihood`` runs
``ImageLinearFit``'s batched solve (``image_linear_solve.py``).

``Param`` restates the sampled-parameter bookkeeping of lenstronomy's ``Param``
(``lenstronomy/Sampling/parameters.py``, not vendored; the reference's
LikelihoodModule takes an instance of it, ``likelihood.py:147-148``) for the
lens, source and lens-light lists; the default bounds are the profiles'
``lower_limit_default`` / ``upper_limit_default``.
"""

import numpy as np
import torch

from .data import PSF, ImageData
from .image_linear_solve import ImageLinearFit
from .image_model import ImageModel
from .lens_model import LensModel
from .light_model import LightModel
from .point_source import PointSource
from . import profiles

_PI = np.pi

# lower_limit_default / upper_limit_default of each supported profile
# (LensModel/Profiles/sie.py:41-54, nie.py:20-35, epl.py:51-66, shear.py:17-18,
# convergence.py:16-17, nfw.py:49-50, tnfw.py:28-41, nfw_ellipse_cse.py:173-188,
# epl_multipole_m1m3m4.py:429-456; LightModel/Profiles/sersic.py:22-35,
# sersic_ellipse.py:26-43)
_C = {"center_x": (-100.0, 100.0), "center_y": (-100.0, 100.0)}
_E = {"e1": (-0.5, 0.5), "e2": (-0.5, 0.5)}
LIMITS = {
    "SIE": {"theta_E": (0.0, 100.0), **_E, **_C},
    "NIE": {"theta_E": (0.0, 10.0), **_E, "s_scale": (0.0, 100.0), **_C},
    "EPL": {"theta_E": (0.0, 100.0), "gamma": (1.5, 2.5), **_E, **_C},
    "SHEAR": {"gamma1": (-0.5, 0.5), "gamma2": (-0.5, 0.5), "ra_0": (-100.0, 100.0),
              "dec_0": (-100.0, 100.0)},
    "CONVERGENCE": {"kappa": (-10.0, 10.0), "ra_0": (-100.0, 100.0), "dec_0": (-100.0, 100.0)},
    "NFW": {"Rs": (0.0, 100.0), "alpha_Rs": (0.0, 10.0), **_C},
    "TNFW": {"Rs": (0.0, 100.0), "alpha_Rs": (0.0, 10.0), "r_trunc": (0.0, 100.0), **_C},
    "NFW_ELLIPSE_CSE": {"Rs": (0.0, 100.0), "alpha_Rs": (0.0, 10.0), **_E, **_C},
    "EPL_MULTIPOLE_M1M3M4": {"theta_E": (0.0, 100.0), "gamma": (1.5, 2.5), **_E, **_C,
                             "a1_a": (-0.2, 0.2), "delta_phi_m1": (-_PI, _PI),
                             "a3_a": (-0.2, 0.2), "delta_phi_m3": (-_PI / 6, _PI / 6),
                             "a4_a": (-0.2, 0.2), "delta_phi_m4": (-_PI / 8, _PI / 8)},
    "SERSIC": {"amp": (0.0, 100.0), "R_sersic": (0.0, 100.0), "n_sersic": (0.5, 8.0), **_C},
    "SERSIC_ELLIPSE": {"amp": (0.0, 100.0), "R_sersic": (0.0, 100.0), "n_sersic": (0.5, 8.0),
                       **_E, **_C},
}

_LISTS = (("lens", "lens_model_list", profiles.LENS_PARAMS),
          ("source", "source_light_model_list", profiles.LIGHT_PARAMS),
          ("lens_light", "lens_light_model_list", profiles.LIGHT_PARAMS))

_UNSUPPORTED_MODEL_KEYS = ("optical_depth_model_list", "tracer_source_model_list")

# parameters of the point-source types (PointSource/Types/{lensed_position,unlensed}.py),
# each an array of num_point_source_list[i] values
_PS_PARAMS = ["ra_image", "dec_image", "point_amp"]


def _model_lists(kwargs_model):
    for key in _UNSUPPORTED_MODEL_KEYS:
        if kwargs_model.get(key):
            raise ValueError("%s is not supported by this build" % key)
    out = {tag: list(kwargs_model.get(key, [])) for tag, key, _ in _LISTS}
    out["ps"] = list(kwargs_model.get("point_source_model_list", []))
    return out


class Param:
    """Sampled parameters of the lens, source and lens-light lists.

    Every ``param_names`` entry of every profile that is not in the profile's
    ``kwargs_fixed_*`` dict is one sampled argument, ordered by list (lens,
    source, lens light), then profile, then ``param_names``.  Bounds default to
    the profiles' ``lower_limit_default`` / ``upper_limit_default``; entries of
    ``kwargs_lower_*`` / ``kwargs_upper_*`` replace them.  With ``linear_solver``
    (the default, as in lenstronomy) every light profile's ``amp`` is left to the
    linear solve: it is not sampled and reads 1 unless fixed otherwise.  Point
    sources (``point_source_model_list`` with ``num_point_source_list``) follow:
    ``ra_image``, ``dec_image`` and, without the linear solver, ``point_amp``, one
    argument per image; their bounds come from ``kwargs_lower_ps`` /
    ``kwargs_upper_ps``, which a sampled point-source parameter needs."""

    def __init__(self, kwargs_model, kwargs_fixed_lens=None, kwargs_fixed_source=None,
                 kwargs_fixed_lens_light=None, kwargs_fixed_ps=None, kwargs_fixed_special=None,
                 kwargs_fixed_extinction=None, kwargs_lower_lens=None, kwargs_lower_source=None,
                 kwargs_lower_lens_light=None, kwargs_lower_ps=None, kwargs_lower_special=None,
                 kwargs_lower_extinction=None, kwargs_upper_lens=None, kwargs_upper_source=None,
                 kwargs_upper_lens_light=None, kwargs_upper_ps=None, kwargs_upper_special=None,
                 kwargs_upper_extinction=None, linear_solver=True, **constraints):
        for name, v in (("kwargs_fixed_special", kwargs_fixed_special),
                        ("kwargs_fixed_extinction", kwargs_fixed_extinction),
                        ("kwargs_lower_special", kwargs_lower_special),
                        ("kwargs_lower_extinction", kwargs_lower_extinction),
                        ("kwargs_upper_special", kwargs_upper_special),
                        ("kwargs_upper_extinction", kwargs_upper_extinction)):
            if v:
                raise ValueError("%s is not supported by this build" % name)
        num_point_source_list = constraints.pop("num_point_source_list", None)
        for name, v in constraints.items():
            if v:
                raise ValueError("parameter constraint %s is not supported by this build" % name)
        self.linear_solver = bool(linear_solver)
        self._lists = _model_lists(kwargs_model)
        fixed = {"lens": kwargs_fixed_lens, "source": kwargs_fixed_source,
                 "lens_light": kwargs_fixed_lens_light}
        lower = {"lens": kwargs_lower_lens, "source": kwargs_lower_source,
                 "lens_light": kwargs_lower_lens_light}
        upper = {"lens": kwargs_upper_lens, "source": kwargs_upper_source,
                 "lens_light": kwargs_upper_lens_light}
        self._fixed = {}
        self._slots = []   # (list tag, profile index, param name) per sampled argument
        lo, hi = [], []
        for tag, _, table in _LISTS:
            names = self._lists[tag]
            profiles.check_names(names, table, tag)
            fx = list(fixed[tag]) if fixed[tag] is not None else [{} for _ in names]
            lw = list(lower[tag]) if lower[tag] is not None else [{} for _ in names]
            up = list(upper[tag]) if upper[tag] is not None else [{} for _ in names]
            for what, lst in (("fixed", fx), ("lower", lw), ("upper", up)):
                if len(lst) != len(names):
                    raise ValueError("kwargs_%s_%s needs one dict per %s profile"
                                     % (what, tag, tag))
            self._fixed[tag] = [dict(d) for d in fx]
            if self.linear_solver and tag != "lens":
                for d in self._fixed[tag]:
                    d.setdefault("amp", 1.0)
            fx = self._fixed[tag]
            for i, name in enumerate(names):
                for p in table[name]:
                    if p in fx[i]:
                        continue
                    self._slots.append((tag, i, p, None))
                    lo.append(float(lw[i].get(p, LIMITS[name][p][0])))
                    hi.append(float(up[i].get(p, LIMITS[name][p][1])))
        # point sources: ra_image, dec_image, point_amp arrays of num_point_source_list[i]
        # values; point_amp is left to the linear solve; sampled arrays need their bounds
        ps = self._lists["ps"]
        npl = (list(num_point_source_list) if num_point_source_list is not None
               else [1] * len(ps))
        if len(npl) != len(ps):
            raise ValueError("num_point_source_list needs one entry per point-source model")
        fx = list(kwargs_fixed_ps) if kwargs_fixed_ps is not None else [{} for _ in ps]
        lw = list(kwargs_lower_ps) if kwargs_lower_ps is not None else [{} for _ in ps]
        up = list(kwargs_upper_ps) if kwargs_upper_ps is not None else [{} for _ in ps]
        for what, lst in (("fixed", fx), ("lower", lw), ("upper", up)):
            if len(lst) != len(ps):
                raise ValueError("kwargs_%s_ps needs one dict per point-source model" % what)
        self._fixed["ps"] = [dict(d) for d in fx]
        self._num_point_source_list = npl
        for i, name in enumerate(ps):
            if name not in ("LENSED_POSITION", "UNLENSED"):
                raise ValueError("point-source model %s is not supported" % name)
            if self.linear_solver:
                self._fixed["ps"][i].setdefault("point_amp", np.ones(npl[i]))
            for p in _PS_PARAMS:
                if p in self._fixed["ps"][i]:
                    continue
                if p not in lw[i] or p not in up[i]:
                    raise ValueError("sampled point-source parameter %s needs kwargs_lower_ps "
                                     "and kwargs_upper_ps entries" % p)
                lo_p = np.broadcast_to(np.asarray(lw[i][p], dtype=float), (npl[i],))
                hi_p = np.broadcast_to(np.asarray(up[i][p], dtype=float), (npl[i],))
                for j in range(npl[i]):
                    self._slots.append(("ps", i, p, j))
                    lo.append(float(lo_p[j]))
                    hi.append(float(hi_p[j]))
        self._lower = np.array(lo)
        self._upper = np.array(hi)

    def num_param(self):
        """(number of sampled arguments, their names as ``param_name_list-tag-index``)."""
        names = [p if tag == "ps" else "%s_%s%d" % (p, tag, i) for tag, i, p, _ in self._slots]
        return len(self._slots), names

    def num_param_linear(self):
        return 0

    def param_limits(self):
        return self._lower.copy(), self._upper.copy()

    def kwargs2args(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                    kwargs_ps=None, kwargs_special=None, kwargs_extinction=None,
                    kwargs_tracer_source=None):
        kw = {"lens": kwargs_lens, "source": kwargs_source, "lens_light": kwargs_lens_light,
              "ps": kwargs_ps}
        return np.array([float(kw[tag][i][p] if j is None else np.asarray(kw[tag][i][p])[j])
                         for tag, i, p, j in self._slots])

    def args2kwargs(self, args, bijective=False):
        """kwargs of one vector (d,) or, for an ensemble (n, d), kwargs whose
        sampled values are arrays of length n (the batched layout of
        ``ImageModel.pack_params``)."""
        a = np.asarray(args, dtype=float)
        if a.shape[-1] != len(self._slots):
            raise ValueError("expected %d arguments, got %d" % (len(self._slots), a.shape[-1]))
        out = {tag: [dict(d) for d in self._fixed[tag]] for tag in ("lens", "source",
                                                                     "lens_light", "ps")}
        arrays = {}
        for k, (tag, i, p, j) in enumerate(self._slots):
            if j is None:
                out[tag][i][p] = a[..., k]
            else:
                arrays.setdefault((i, p), []).append(a[..., k])
        for (i, p), cols in arrays.items():
            out["ps"][i][p] = np.stack(cols, axis=-1)
        return {"kwargs_lens": out["lens"], "kwargs_source": out["source"],
                "kwargs_lens_light": out["lens_light"], "kwargs_ps": out["ps"],
                "kwargs_special": {}, "kwargs_extinction": [], "kwargs_tracer_source": []}


class ImageLikelihood:
    """Imaging-data likelihood of one band (``image_likelihood.py:8-132``),
    evaluated on the GPU; ``logL_batch`` takes batched kwargs."""

    def __init__(self, multi_band_list, multi_band_type, kwargs_model, bands_compute=None,
                 image_likelihood_mask_list=None, source_marg=False, linear_prior=None,
                 check_positive_flux=False, kwargs_pixelbased=None, linear_solver=True,
                 precision="fp64"):
        if kwargs_pixelbased is not None:
            raise ValueError("pixelbased solver not supported in jaxtronomy")
        if multi_band_type != "single-band":
            raise ValueError("Type %s is not supported in JAXtronomy! Use lenstronomy instead."
                             % multi_band_type)
        if linear_prior is not None:
            raise ValueError("linear_prior (marginalization_new) is not supported; use "
                             "source_marg with flat priors")
        if (source_marg or check_positive_flux) and not linear_solver:
            raise ValueError("source_marg and check_positive_flux need the linear solver")
        self._linear = bool(linear_solver)
        self._source_marg = bool(source_marg)
        self._check_positive_flux = bool(check_positive_flux)
        lists = _model_lists(kwargs_model)
        kwargs_data, kwargs_psf, kwargs_numerics = multi_band_list[0][:3]
        data = ImageData(**kwargs_data)
        psf = PSF(**{k: v for k, v in kwargs_psf.items() if k != "pixel_size"})
        kn = dict(kwargs_numerics or {})
        kn.setdefault("precision", precision)
        mask = None if image_likelihood_mask_list is None else image_likelihood_mask_list[0]
        cls = ImageLinearFit if self._linear else ImageModel
        lens_model = LensModel(lists["lens"])
        self.imSim = cls(data, psf, lens_model, LightModel(lists["source"]),
                         LightModel(lists["lens_light"]),
                         point_source_class=PointSource(lists["ps"], lens_model=lens_model),
                         kwargs_numerics=kn, likelihood_mask=mask)
        self._model_type = self.imSim.type

    @property
    def num_data(self):
        return self.imSim.num_data_evaluate

    def logL_batch(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                   stream=None, kwargs_ps=None, kwargs_special=None, **kwargs):
        """(B,) FP64 log-likelihoods of batched kwargs, NaN replaced by -1e15
        (``image_likelihood.py:95``)."""
        if self._linear:
            logl, _, _, _ = self.imSim.likelihood_linear_batch(
                kwargs_lens, kwargs_source, kwargs_lens_light, source_marg=self._source_marg,
                check_positive_flux=self._check_positive_flux, stream=stream,
                kwargs_ps=kwargs_ps, kwargs_special=kwargs_special)
        else:
            logl = self.imSim.likelihood_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                               stream=stream, kwargs_ps=kwargs_ps,
                                               kwargs_special=kwargs_special)
        return torch.nan_to_num(logl, nan=-(10.0 ** 15))

    def logL(self, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None, kwargs_ps=None,
             kwargs_special=None, kwargs_extinction=None, **kwargs):
        """(logL, linear parameters) of one system (None without the linear solver)."""
        if kwargs_extinction:
            raise ValueError("Extinction is not implemented")
        if not self._linear:
            return float(self.logL_batch(kwargs_lens, kwargs_source, kwargs_lens_light,
                                         kwargs_ps=kwargs_ps,
                                         kwargs_special=kwargs_special)[0]), None
        logl, param, _, _ = self.imSim.likelihood_linear_batch(
            kwargs_lens, kwargs_source, kwargs_lens_light, source_marg=self._source_marg,
            check_positive_flux=self._check_positive_flux, kwargs_ps=kwargs_ps,
            kwargs_special=kwargs_special)
        return float(torch.nan_to_num(logl, nan=-(10.0 ** 15))[0]), param[0].cpu().numpy()


def _prior_terms(prior, kwargs_list):
    """Gaussian priors [[index, param_name, mean, sigma], ...]: -(x - mean)^2 / (2 sigma^2)
    summed (lenstronomy PriorLikelihood's Gaussian terms)."""
    total = 0.0
    for index, name, mean, sigma in prior or []:
        x = np.asarray(kwargs_list[index][name], dtype=float)
        total = total - (x - mean) ** 2 / sigma ** 2 / 2.0
    return total


class LikelihoodModule:
    """Log-likelihood of sampled parameter vectors (``Sampling/likelihood.py:19-372``):
    the image likelihood, Gaussian priors, hard bounds and an optional custom
    term.  ``logL`` takes one vector; ``logL_batch`` an (n, d) ensemble,
    evaluated as one batched GPU launch."""

    def __init__(self, kwargs_data_joint, kwargs_model, param_class, image_likelihood=True,
                 check_bounds=True, astrometric_likelihood=False,
                 image_position_likelihood=False, source_position_likelihood=None,
                 image_position_uncertainty=0.004, check_positive_flux=False,
                 source_position_tolerance=None, source_position_sigma=0.001,
                 force_no_add_image=False, source_marg=False, linear_prior=None,
                 restrict_image_number=False, max_num_images=None, bands_compute=None,
                 time_delay_likelihood=False, image_likelihood_mask_list=None,
                 flux_ratio_likelihood=False, kwargs_flux_compute=None, prior_lens=None,
                 prior_source=None, prior_extinction=None, prior_lens_light=None, prior_ps=None,
                 prior_special=None, prior_lens_kde=None, prior_source_kde=None,
                 prior_lens_light_kde=None, prior_ps_kde=None, prior_special_kde=None,
                 prior_extinction_kde=None, prior_lens_lognormal=None,
                 prior_source_lognormal=None, prior_extinction_lognormal=None,
                 prior_lens_light_lognormal=None, prior_ps_lognormal=None,
                 prior_special_lognormal=None, custom_logL_addition=None,
                 kwargs_pixelbased=None, kinematic_2d_likelihood=False, kin_lens_idx=0,
                 kin_lens_light_idx=0, tracer_likelihood=False, tracer_likelihood_mask=None,
                 precision="fp64"):
        if (time_delay_likelihood or tracer_likelihood or flux_ratio_likelihood
                or kinematic_2d_likelihood):
            raise ValueError("tracer, flux_ratio, and kinematic_2d likelihoods are not currently "
                             "supported and should be set to False.")
        if astrometric_likelihood or image_position_likelihood or source_position_likelihood:
            raise ValueError("astrometric, image-position and source-position likelihoods are "
                             "not supported by this build")
        for name, v in (("prior_ps", prior_ps), ("prior_special", prior_special),
                        ("prior_extinction", prior_extinction)):
            if v:
                raise ValueError("%s is not supported by this build" % name)
        for name, v in (("prior_lens_kde", prior_lens_kde), ("prior_source_kde", prior_source_kde),
                        ("prior_lens_light_kde", prior_lens_light_kde),
                        ("prior_ps_kde", prior_ps_kde), ("prior_special_kde", prior_special_kde),
                        ("prior_extinction_kde", prior_extinction_kde),
                        ("prior_lens_lognormal", prior_lens_lognormal),
                        ("prior_source_lognormal", prior_source_lognormal),
                        ("prior_lens_light_lognormal", prior_lens_light_lognormal),
                        ("prior_ps_lognormal", prior_ps_lognormal),
                        ("prior_special_lognormal", prior_special_lognormal),
                        ("prior_extinction_lognormal", prior_extinction_lognormal)):
            if v:
                raise ValueError("%s is not supported by this build (Gaussian priors are)" % name)
        self.param = param_class
        self._lower_limit, self._upper_limit = self.param.param_limits()
        self._check_bounds = check_bounds
        self._priors = (prior_lens, prior_source, prior_lens_light)
        self._custom_logL_addition = custom_logL_addition
        multi_band_list = kwargs_data_joint.get("multi_band_list", [])
        self._image_likelihood = bool(image_likelihood) and len(multi_band_list) > 0
        if self._image_likelihood:
            self.image_likelihood = ImageLikelihood(
                multi_band_list, kwargs_data_joint.get("multi_band_type", "single-band"),
                kwargs_model, bands_compute=bands_compute,
                image_likelihood_mask_list=image_likelihood_mask_list, source_marg=source_marg,
                linear_prior=linear_prior, check_positive_flux=check_positive_flux,
                kwargs_pixelbased=kwargs_pixelbased, linear_solver=self.param.linear_solver,
                precision=precision)

    def __call__(self, a):
        return self.logL(a)

    def logL(self, args, verbose=False):
        """Log-likelihood of one parameter vector (``likelihood.py:294-318``)."""
        return float(self.logL_batch(np.asarray(args, dtype=float)[None, :])[0])

    def logL_batch(self, args, stream=None):
        """(n,) log-likelihoods of an (n, d) ensemble: out-of-bounds vectors get
        -1e18 (``likelihood.py:308-316``); otherwise prior + image likelihood +
        custom term, NaN replaced by 1e-18 (``likelihood.py:320-372``)."""
        a = np.atleast_2d(np.asarray(args, dtype=float))
        kw = self.param.args2kwargs(a)
        n = a.shape[0]
        logl = np.zeros(n)
        if self._custom_logL_addition is not None:
            for j in range(n):
                kj = self.param.args2kwargs(a[j])
                logl[j] += float(self._custom_logL_addition(**kj))
        for prior, key in zip(self._priors, ("kwargs_lens", "kwargs_source",
                                              "kwargs_lens_light")):
            logl = logl + _prior_terms(prior, kw[key])
        if self._image_likelihood:
            img = self.image_likelihood.logL_batch(kw["kwargs_lens"], kw["kwargs_source"],
                                                   kw["kwargs_lens_light"], stream=stream,
                                                   kwargs_ps=kw["kwargs_ps"] or None)
            logl = logl + img.cpu().numpy()
        logl = np.nan_to_num(logl, nan=1e-18)
        if self._check_bounds:
            hit = np.any((a < self._lower_limit) | (a > self._upper_limit), axis=1)
            logl = np.where(hit, -(10.0 ** 18), logl)
        return logl

    @staticmethod
    def check_bounds(args, lowerLimit, upperLimit, verbose=False):
        """(penalty, bound_hit) as ``likelihood.py:374-400``."""
        a = np.atleast_1d(np.asarray(args, dtype=float))
        hit = bool(np.any((a < np.atleast_1d(lowerLimit)) | (a > np.atleast_1d(upperLimit))))
        return (10.0 ** 5 if hit else 0.0), hit


def prepare_logL_func(backend, logL_func, threadCount=1):
    """``sampler.py:215-250``: a function of an (n, d) ensemble.  backend
    "gpu" with a ``LikelihoodModule``'s ``logL`` (or the module itself) returns
    its one-launch ``logL_batch``; this build has no CPU backend."""
    if backend == "cpu":
        raise ValueError("this build evaluates the likelihood on the GPU; use backend='gpu'")
    if backend != "gpu":
        raise ValueError("backend must be either 'cpu' or 'gpu'")
    module = logL_func if isinstance(logL_func, LikelihoodModule) else getattr(
        logL_func, "__self__", None)
    if not isinstance(module, LikelihoodModule):
        raise ValueError("prepare_logL_func needs a LikelihoodModule or its logL method")

    def new_logL_func(args):
        return np.asarray(module.logL_batch(args)).flatten()

    return new_logL_func
