"""Stand-ins that let the JAXtronomy reference source run under plain NumPy.

Used only by ``make_golden.py`` in a container that holds the reference source
tree but neither ``jax`` nor ``lenstronomy``.  Nothing here is imported by the
library, the tests or the benchmark.

* ``jax`` is replaced by a NumPy-backed module: ``jit`` / ``custom_jvp`` become
  pass-throughs, ``lax`` control flow becomes Python loops, ``jax.numpy`` is
  NumPy with arrays that support the ``.at[...].set/get`` update syntax, and
  ``jax.scipy`` maps onto SciPy.  Running in FP64 mirrors the reference's
  ``JAX_ENABLE_X64=True`` test configuration.
* The few ``lenstronomy`` / ``astropy`` names the reference imports on the
  image path are restated from lenstronomy's documented behaviour (pixel-grid
  construction, supersampled sub-grid, single-plane source mapping, PSF
  normalisation).  These are the *unpinned* conventions: the same restatement
  appears in the oracle, so the golden vectors pin only the JAXtronomy-owned
  arithmetic.
"""

import sys
import types

import numpy as np
import scipy.ndimage
import scipy.signal
import scipy.special


# ---------------------------------------------------------------------------
# jax.numpy with .at[] support
# ---------------------------------------------------------------------------


class AtArray(np.ndarray):
    @property
    def at(self):
        return _At(self)


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self.arr, idx)


class _AtIdx:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = idx

    def set(self, v):
        out = np.array(self.arr).view(AtArray)
        out[self.idx] = v
        return out

    def add(self, v):
        out = np.array(self.arr).view(AtArray)
        out[self.idx] += v
        return out

    def get(self):
        return self.arr[self.idx]


def _wrap(fn):
    def inner(*a, **k):
        r = fn(*a, **k)
        if isinstance(r, np.ndarray):
            return r.view(AtArray)
        return r
    return inner


def _make_jnp():
    jnp = types.ModuleType("jax.numpy")
    for name in dir(np):
        if not name.startswith("__"):
            setattr(jnp, name, getattr(np, name))
    for name in ("array", "asarray", "zeros", "zeros_like", "ones", "ones_like", "full",
                 "full_like", "where", "arange", "reshape", "concatenate", "stack",
                 "atleast_1d", "pad", "empty", "meshgrid"):
        fn = getattr(np, name)
        if name == "meshgrid":
            setattr(jnp, name, lambda *a, **k: [x.view(AtArray) for x in np.meshgrid(*a, **k)])
        else:
            setattr(jnp, name, _wrap(fn))
    jnp.ndarray = np.ndarray
    # jax.numpy.linalg returns non-finite values for a singular matrix where
    # numpy raises; the reference filters them (de_lens.py:72-99)
    linalg = types.ModuleType("jax.numpy.linalg")
    for name in dir(np.linalg):
        if not name.startswith("__"):
            setattr(linalg, name, getattr(np.linalg, name))

    def _nan_on_singular(fn):
        def inner(a, *rest):
            try:
                return fn(a, *rest)
            except np.linalg.LinAlgError:
                shape = np.shape(rest[0]) if rest else np.shape(a)
                return np.full(shape, np.nan)
        return inner

    linalg.inv = _nan_on_singular(np.linalg.inv)
    linalg.solve = _nan_on_singular(np.linalg.solve)
    jnp.linalg = linalg
    return jnp


# ---------------------------------------------------------------------------
# jax, jax.lax, jax.scipy, jax.tree_util
# ---------------------------------------------------------------------------


def jit(fun=None, static_argnums=None, static_argnames=None, **kwargs):
    if fun is None:
        return lambda f: f
    return fun


class custom_jvp:
    def __init__(self, fun, nondiff_argnums=()):
        if isinstance(fun, staticmethod):
            fun = fun.__func__
        self.fun = fun

    def __call__(self, *args, **kwargs):
        return self.fun(*args, **kwargs)

    def defjvp(self, jvp_fn):
        return jvp_fn


def _tree_map(f, tree):
    if isinstance(tree, dict):
        return {k: _tree_map(f, v) for k, v in tree.items()}
    if isinstance(tree, (list, tuple)):
        return type(tree)(_tree_map(f, v) for v in tree)
    return f(tree)


def _make_lax():
    lax = types.ModuleType("jax.lax")

    def fori_loop(lower, upper, body, init):
        val = init
        for i in range(int(lower), int(upper)):
            val = body(i, val)
        return val

    def switch(index, branches, *operands):
        # lax.switch clamps the index into [0, len(branches) - 1]
        k = min(max(int(np.asarray(index)), 0), len(branches) - 1)
        return branches[k](*operands)

    def cond(pred, true_fun, false_fun, *operands):
        return true_fun(*operands) if bool(np.asarray(pred)) else false_fun(*operands)

    def lax_map(f, xs):
        leaves = []
        _tree_map(lambda a: leaves.append(np.asarray(a)), xs)
        n = leaves[0].shape[0]
        outs = [f(_tree_map(lambda a, i=i: np.asarray(a)[i], xs)) for i in range(n)]
        if isinstance(outs[0], (tuple, list)):
            return tuple(np.stack([o[j] for o in outs]) for j in range(len(outs[0])))
        return np.stack(outs)

    def scan(f, init, xs):
        carry = init
        ys = []
        leaves = []
        _tree_map(lambda a: leaves.append(np.asarray(a)), xs)
        n = leaves[0].shape[0]
        for i in range(n):
            carry, y = f(carry, _tree_map(lambda a, i=i: np.asarray(a)[i], xs))
            ys.append(y)
        return carry, ys

    def dynamic_slice(operand, start_indices, slice_sizes):
        sl = tuple(slice(int(s), int(s) + int(n)) for s, n in zip(start_indices, slice_sizes))
        return np.asarray(operand)[sl]

    lax.fori_loop = fori_loop
    lax.switch = switch
    lax.cond = cond
    lax.map = lax_map
    lax.scan = scan
    lax.dynamic_slice = dynamic_slice
    return lax


def install_jax():
    jax = types.ModuleType("jax")
    jnp = _make_jnp()
    lax = _make_lax()
    tree_util = types.ModuleType("jax.tree_util")
    tree_util.register_pytree_node = lambda *a, **k: None
    tree_util.tree_map = _tree_map
    jscipy = types.ModuleType("jax.scipy")
    special = types.ModuleType("jax.scipy.special")
    special.gamma = scipy.special.gamma
    special.gammainc = scipy.special.gammainc
    special.gammaln = scipy.special.gammaln
    special.factorial = scipy.special.factorial
    signal = types.ModuleType("jax.scipy.signal")
    signal.fftconvolve = lambda in1, in2, mode="full": np.asarray(
        scipy.signal.fftconvolve(in1, in2, mode=mode)).view(AtArray)
    signal.convolve2d = lambda in1, in2, mode="full": np.asarray(
        scipy.signal.convolve2d(in1, in2, mode=mode)).view(AtArray)
    ndimage = types.ModuleType("jax.scipy.ndimage")

    def _map_coordinates(input, coordinates, order, mode="constant", cval=0.0):
        # jax.scipy.ndimage.map_coordinates reads every interpolation corner outside
        # the input as cval ("constant"); SciPy calls that mode "grid-constant"
        m = {"constant": "grid-constant"}.get(mode, mode)
        return np.asarray(scipy.ndimage.map_coordinates(np.asarray(input, float),
                                                        np.asarray(coordinates, float),
                                                        order=order, mode=m, cval=cval,
                                                        prefilter=False)).view(AtArray)

    ndimage.map_coordinates = _map_coordinates
    jscipy.special = special
    jscipy.signal = signal
    jscipy.ndimage = ndimage
    config = types.SimpleNamespace(update=lambda *a, **k: None)
    experimental = types.ModuleType("jax.experimental")
    jax.numpy = jnp
    jax.lax = lax
    jax.tree_util = tree_util
    jax.scipy = jscipy
    jax.config = config
    jax.experimental = experimental
    jax.jit = jit
    jax.custom_jvp = custom_jvp
    jax.jvp = lambda *a, **k: (_ for _ in ()).throw(NotImplementedError("jvp"))
    jax.grad = lambda *a, **k: (_ for _ in ()).throw(NotImplementedError("grad"))
    jax.vmap = lambda f, *a, **k: f
    jax.Array = np.ndarray
    jax.devices = lambda *a, **k: ["cpu"]
    jax.debug = types.SimpleNamespace(print=lambda *a, **k: None)
    # names the lens-equation solver module imports (never called on these paths)
    jrandom = types.ModuleType("jax.random")
    optimize = types.ModuleType("jax.scipy.optimize")
    optimize.minimize = _Dummy()
    jscipy.optimize = optimize
    jax.random = jrandom
    mods = {
        "jax": jax, "jax.numpy": jnp, "jax.lax": lax, "jax.tree_util": tree_util,
        "jax.scipy": jscipy, "jax.scipy.special": special, "jax.scipy.signal": signal,
        "jax.scipy.ndimage": ndimage, "jax.experimental": experimental,
        "jax.random": jrandom, "jax.scipy.optimize": optimize,
    }
    sys.modules.update(mods)


# ---------------------------------------------------------------------------
# lenstronomy / astropy names on the image path
# ---------------------------------------------------------------------------


def _make_grid(numPix, deltapix, subgrid_res=1, left_lower=False):
    n = np.array([numPix, numPix], dtype=int) if np.isscalar(numPix) else np.asarray(numPix, int)
    n_eff = (n * subgrid_res).astype(int)
    d_eff = deltapix / float(subgrid_res)
    xg = np.tile(np.arange(n_eff[0]), n_eff[1]) * d_eff
    yg = np.repeat(np.arange(n_eff[1]), n_eff[0]) * d_eff
    if left_lower:
        shift = -1.0 / 2 + 1.0 / (2 * subgrid_res) * np.array([1, 1])
    else:
        shift = d_eff * (n_eff - 1) / 2
    return xg - shift[0], yg - shift[1]


def _array2image(array, nx=0, ny=0):
    # lenstronomy's util.array2image fills an (nx, ny) array row by row; the
    # reference relies on that order for non-square shapes (grid.py:127-130)
    array = np.asarray(array)
    if nx == 0 or ny == 0:
        n = int(np.sqrt(len(array)))
        nx = ny = n
    return array.reshape(int(nx), int(ny))


def _image2array(image):
    return np.asarray(image).reshape(-1)


def _make_subgrid(ra_coord, dec_coord, subgrid_res=2):
    ra = _array2image(ra_coord)
    dec = _array2image(dec_coord)
    n = len(ra)
    d_ra_x = ra[0][1] - ra[0][0]
    d_ra_y = ra[1][0] - ra[0][0]
    d_dec_x = dec[0][1] - dec[0][0]
    d_dec_y = dec[1][0] - dec[0][0]
    ra_new = np.zeros((n * subgrid_res, n * subgrid_res))
    dec_new = np.zeros((n * subgrid_res, n * subgrid_res))
    for i in range(subgrid_res):
        fy = -0.5 + 1.0 / (2.0 * subgrid_res) + i / float(subgrid_res)
        for j in range(subgrid_res):
            fx = -0.5 + 1.0 / (2.0 * subgrid_res) + j / float(subgrid_res)
            ra_new[i::subgrid_res, j::subgrid_res] = ra + d_ra_x * fx + d_ra_y * fy
            dec_new[i::subgrid_res, j::subgrid_res] = dec + d_dec_x * fx + d_dec_y * fy
    return _image2array(ra_new), _image2array(dec_new)


def _convert_bool_list(n, k=None):
    if k is None:
        return [True] * n
    if isinstance(k, (int, np.integer)):
        out = [False] * n
        out[k] = True
        return out
    k = list(k)
    if len(k) and isinstance(k[0], (bool, np.bool_)):
        return [bool(v) for v in k]
    out = [False] * n
    for i in k:
        out[i] = True
    return out


def _grid_from_transform(nx, ny, M, ra0, dec0):
    a = np.arange(nx)
    b = np.arange(ny)
    mat = np.dstack(np.meshgrid(a, b)).reshape(-1, 2)
    x, y = mat[:, 0], mat[:, 1]
    ra = x * M[0, 0] + y * M[0, 1] + ra0
    dec = x * M[1, 0] + y * M[1, 1] + dec0
    return ra, dec


class Coordinates1D:
    def __init__(self, transform_pix2angle, ra_at_xy_0, dec_at_xy_0):
        self._Mpix2a = np.asarray(transform_pix2angle, float)
        self._Ma2pix = np.linalg.inv(self._Mpix2a)
        self._ra_at_xy_0 = ra_at_xy_0
        self._dec_at_xy_0 = dec_at_xy_0
        self._x_at_radec_0, self._y_at_radec_0 = self._Ma2pix.dot(
            np.array([-ra_at_xy_0, -dec_at_xy_0]))

    @property
    def transform_pix2angle(self):
        return self._Mpix2a

    @property
    def radec_at_xy_0(self):
        return self._ra_at_xy_0, self._dec_at_xy_0

    @property
    def pixel_width(self):
        return float(np.sqrt(abs(np.linalg.det(self._Mpix2a))))

    def map_pix2coord(self, x, y):
        ra = x * self._Mpix2a[0, 0] + y * self._Mpix2a[0, 1] + self._ra_at_xy_0
        dec = x * self._Mpix2a[1, 0] + y * self._Mpix2a[1, 1] + self._dec_at_xy_0
        return ra, dec

    def coordinate_grid(self, nx, ny):
        return _grid_from_transform(nx, ny, self._Mpix2a, self._ra_at_xy_0, self._dec_at_xy_0)


class PixelGrid(Coordinates1D):
    def __init__(self, nx, ny, transform_pix2angle, ra_at_xy_0, dec_at_xy_0,
                 antenna_primary_beam=None):
        super().__init__(transform_pix2angle, ra_at_xy_0, dec_at_xy_0)
        self._nx = nx
        self._ny = ny
        self._pb = antenna_primary_beam

    @property
    def num_pixel_axes(self):
        return self._nx, self._ny

    @property
    def num_pixel(self):
        return self._nx * self._ny

    @property
    def width(self):
        return self.pixel_width * np.array([self._nx, self._ny])

    @property
    def center(self):
        return self.map_pix2coord((self._nx - 1) / 2.0, (self._ny - 1) / 2.0)

    @property
    def primary_beam(self):
        return self._pb


class PSF:
    def __init__(self, psf_type="NONE", fwhm=None, truncation=5, kernel_point_source=None,
                 psf_variance_map=None, point_source_supersampling_factor=1, **kw):
        self.psf_type = psf_type
        self._fwhm = fwhm
        self._truncation = truncation
        self._kernel = None
        if psf_type == "PIXEL":
            k = np.asarray(kernel_point_source, float)
            self._kernel = k / np.sum(k)
        elif psf_type == "NONE":
            # lenstronomy's PSF("NONE") carries a 3x3 delta kernel
            self._kernel = np.zeros((3, 3))
            self._kernel[1, 1] = 1.0
        self.psf_variance_map_bool = psf_variance_map is not None
        self._pixel_size = None
        self.point_source_supersampling_factor = point_source_supersampling_factor

    @property
    def kernel_point_source(self):
        return self._kernel

    @property
    def fwhm(self):
        return self._fwhm

    @property
    def truncation(self):
        return self._truncation

    def set_pixel_size(self, deltaPix):
        self._pixel_size = deltaPix

    def kernel_point_source_supersampled(self, supersampling_factor, updata_cache=False):
        # the kernel given at construction is the supersampled one when the
        # factors match; building one from a pixel-scale kernel is not restated.
        # Factor 1 is only requested by the point-source renderer, which these
        # scenes never use.
        if supersampling_factor in (self.point_source_supersampling_factor, 1):
            return self._kernel
        raise NotImplementedError("supersampled PSF kernels are not restated")


class Image2SourceMapping:
    """Single lens plane: source i is evaluated at theta - scale_i * alpha(theta)."""

    def __init__(self, lens_model, source_model):
        self._lens = lens_model
        self._source = source_model

    def image_flux_joint(self, x, y, kwargs_lens, kwargs_source, kwargs_special=None, k=None):
        scal = getattr(self._source, "deflection_scaling_list", None)
        if scal is None:
            bx, by = self._lens.ray_shooting(x, y, kwargs_lens)
            return self._source.surface_brightness(bx, by, kwargs_source, k=k)
        ax, ay = self._lens.alpha(x, y, kwargs_lens)
        flux = np.zeros_like(np.asarray(x, float))
        for i, func in enumerate(self._source.func_list):
            if k is None or k == i:
                flux = flux + func.function(x - scal[i] * ax, y - scal[i] * ay, **kwargs_source[i])
        return flux

    def image_flux_split(self, x, y, kwargs_lens, kwargs_source, kwargs_special=None):
        """Unit-amplitude response of every linear source component at its lensed
        position: the source model's functions_split at theta - scale_i * alpha."""
        scal = getattr(self._source, "deflection_scaling_list", None)
        if scal is None:
            bx, by = self._lens.ray_shooting(x, y, kwargs_lens)
            return self._source.functions_split(bx, by, kwargs_source)
        ax, ay = self._lens.alpha(x, y, kwargs_lens)
        response, n = [], 0
        for i in range(len(self._source.func_list)):
            r, m = self._source.functions_split(x - scal[i] * ax, y - scal[i] * ay, kwargs_source,
                                                k=i)
            response += r
            n += m
        return response, n


def _exporter():
    names = []

    def export(obj):
        names.append(obj.__name__)
        return obj

    return export, names


class _Dummy:
    def __init__(self, *a, **k):
        pass

    def __getattr__(self, name):
        return _Dummy()

    def __call__(self, *a, **k):
        return _Dummy()


class FlatLCDM:
    """Stand-in for an astropy ``FlatLambdaCDM(H0, Om0, Tcmb0=0)`` instance: only the
    two parameters, read by :class:`Background`."""

    def __init__(self, H0=70.0, Om0=0.3):
        self.H0 = H0
        self.Om0 = Om0


class Background:
    """lenstronomy's ``Cosmo.background.Background`` distances (lenstronomy >= 1.13.6):
    ``d_xy`` = astropy's ``angular_diameter_distance_z1z2`` in Mpc and
    ``T_xy = d_xy (1 + z_source)``, for a flat matter + Lambda cosmology without
    radiation: D_C = (c/H0) int dz / sqrt(Om0 (1+z)^3 + 1 - Om0) by adaptive
    quadrature (scipy ``quad``), D_A(z1, z2) = D_C(z1, z2) / (1 + z2)."""

    def __init__(self, cosmo):
        self._h0 = float(cosmo.H0)
        self._om = float(cosmo.Om0)

    def _dc(self, z1, z2):
        from scipy.integrate import quad
        f = lambda z: 1.0 / np.sqrt(self._om * (1 + z) ** 3 + 1 - self._om)  # noqa: E731
        val, _ = quad(f, float(z1), float(z2), epsabs=0, epsrel=1e-13, limit=200)
        return 299792.458 / self._h0 * val

    def d_xy(self, z_observer, z_source):
        zo = np.asarray(z_observer, dtype=float)
        zs = np.asarray(z_source, dtype=float)
        zo, zs = np.broadcast_arrays(zo, zs)
        out = np.array([self._dc(a, b) / (1 + b) for a, b in zip(zo.ravel(), zs.ravel())])
        return out.reshape(zo.shape) if zo.ndim else float(out[0])

    def T_xy(self, z_observer, z_source):
        return self.d_xy(z_observer, z_source) * (1 + np.asarray(z_source, dtype=float))


def install_lenstronomy():
    def mod(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    util = mod("lenstronomy.Util.util", make_grid=_make_grid, make_subgrid=_make_subgrid,
               array2image=_array2image, image2array=_image2array,
               convert_bool_list=_convert_bool_list, local_minima_2d=_Dummy(),
               selectBest=_Dummy(), fwhm2sigma=lambda f: f / (2 * np.sqrt(2 * np.log(2))),
               grid_from_coordinate_transform=_grid_from_transform)
    package_util = mod("lenstronomy.Util.package_util", exporter=_exporter)
    from oracle import numerics as _onum

    def _cut_psf(psf_data, psf_size, normalisation=True):
        k = _onum.cut_psf(np.asarray(psf_data, float), psf_size)
        return k / np.sum(k) if normalisation else k

    def _split_kernel(kernel_super, supersampling_kernel_size, supersampling_factor,
                      normalized=True):
        return _onum.split_kernel(np.asarray(kernel_super, float), supersampling_kernel_size,
                                  supersampling_factor)

    mod("lenstronomy.Util.image_util")
    mod("lenstronomy.LensModel.Solver.epl_shear_solver", solve_lenseq_pemd=_Dummy())
    mod("lenstronomy.LensModel.Solver")
    kernel_util = mod("lenstronomy.Util.kernel_util", cut_psf=_cut_psf,
                      split_kernel=_split_kernel)
    constants = mod("lenstronomy.Util.constants")
    cosmo_util = mod("lenstronomy.Util.cosmo_util", get_astropy_cosmology=_Dummy())
    mod("lenstronomy.Util", util=util, package_util=package_util, kernel_util=kernel_util,
        constants=constants, cosmo_util=cosmo_util)
    base_profile = mod("lenstronomy.LensModel.Profiles.base_profile",
                       LensProfileBase=type("LensProfileBase", (object,), {
                           "__init__": lambda self, *a, **k: None,
                           "set_static": lambda self, **k: None,
                           "set_dynamic": lambda self: None}))
    mod("lenstronomy.LensModel.Profiles", base_profile=base_profile)
    mp = mod("lenstronomy.LensModel.MultiPlane.multi_plane", MultiPlane=_Dummy)
    mod("lenstronomy.LensModel.MultiPlane", multi_plane=mp)
    mod("lenstronomy.LensModel")
    pg = mod("lenstronomy.Data.pixel_grid", PixelGrid=PixelGrid)
    ct = mod("lenstronomy.Data.coord_transforms", Coordinates1D=Coordinates1D)
    psf = mod("lenstronomy.Data.psf", PSF=PSF)
    mod("lenstronomy.Data", pixel_grid=pg, coord_transforms=ct, psf=psf)
    i2s = mod("lenstronomy.ImSim.image2source_mapping", Image2SourceMapping=Image2SourceMapping)
    de = mod("lenstronomy.ImSim.differential_extinction", DifferentialExtinction=_Dummy)
    mod("lenstronomy.ImSim", image2source_mapping=i2s, differential_extinction=de)
    cl = mod("lenstronomy.Conf.config_loader", conventions_conf=lambda: {})
    mod("lenstronomy.Conf", config_loader=cl)
    lc = mod("lenstronomy.Cosmo.lens_cosmo", LensCosmo=_Dummy)
    bg = mod("lenstronomy.Cosmo.background", Background=Background)
    mod("lenstronomy.Cosmo", lens_cosmo=lc, background=bg)
    mod("lenstronomy")
    cosmo = mod("astropy.cosmology", default_cosmology=_Dummy())
    cosmo.__all__ = ["default_cosmology"]
    mod("astropy", cosmology=cosmo)


def install(reference_root):
    install_jax()
    install_lenstronomy()
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
