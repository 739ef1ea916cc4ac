"""Seeded synthetic lens systems with the shapes of the benchmark workloads.

No public dataset is involved: every system is drawn from
``numpy.random.default_rng(seed)`` with the parameter distributions listed in
each function's docstring.  Batched kwargs use the "vmap" layout accepted by
:meth:`jaxtronomy_gb300.ImageModel.image_batch`: a list of dicts (one per
profile) whose values are float64 arrays of length B.  ``instance(kw, i)``
extracts the scalar kwargs of system ``i``.
"""

import numpy as np


def grid_kwargs(num_pix, delta_pix):
    """Pixel grid centred at 0 with a diagonal pix->angle transform (RA increasing
    with column index), the layout of lenstronomy's
    ``data_configure_simple(..., inverse=False)``."""
    c = (num_pix - 1) / 2.0
    return {
        "transform_pix2angle": np.array([[delta_pix, 0.0], [0.0, delta_pix]]),
        "ra_at_xy_0": -c * delta_pix,
        "dec_at_xy_0": -c * delta_pix,
    }


def gaussian_pixel_kernel(fwhm, delta_pix, size):
    """Circular Gaussian of the given FWHM sampled at pixel centres of a
    size x size stamp, normalised to unit sum."""
    sigma = fwhm / (2 * np.sqrt(2 * np.log(2))) / delta_pix
    c = np.arange(size) - (size - 1) / 2.0
    xx, yy = np.meshgrid(c, c)
    k = np.exp(-(xx ** 2 + yy ** 2) / (2 * sigma ** 2))
    return k / k.sum()


def moffat_pixel_kernel(fwhm, beta, delta_pix, size):
    """Moffat I ~ [1 + (r/alpha)^2]^-beta with alpha = FWHM / (2 sqrt(2^(1/beta)-1)),
    sampled at pixel centres of a size x size stamp, normalised to unit sum."""
    alpha = fwhm / (2 * np.sqrt(2 ** (1.0 / beta) - 1)) / delta_pix
    c = np.arange(size) - (size - 1) / 2.0
    xx, yy = np.meshgrid(c, c)
    k = (1 + (xx ** 2 + yy ** 2) / alpha ** 2) ** (-beta)
    return k / k.sum()


def _ellip(rng, sigma, n, clip=None):
    e1 = rng.normal(0, sigma, n)
    e2 = rng.normal(0, sigma, n)
    if clip is not None:
        e = np.hypot(e1, e2)
        scale = np.where(e >= clip, 0.999 * clip / np.maximum(e, 1e-300), 1.0)
        e1, e2 = e1 * scale, e2 * scale
    return e1, e2


def _sersic_source(rng, n):
    e1, e2 = _ellip(rng, 0.1, n)
    return {
        "amp": rng.uniform(10, 100, n), "R_sersic": rng.uniform(0.1, 0.5, n),
        "n_sersic": rng.uniform(1, 4, n), "e1": e1, "e2": e2,
        "center_x": rng.normal(0, 0.1, n), "center_y": rng.normal(0, 0.1, n),
    }


def _sersic_lens_light(rng, n, cx, cy):
    e1, e2 = _ellip(rng, 0.1, n)
    return {
        "amp": rng.uniform(10, 100, n), "R_sersic": rng.uniform(0.5, 1.5, n),
        "n_sersic": rng.uniform(2, 5, n), "e1": e1, "e2": e2,
        "center_x": cx.copy(), "center_y": cy.copy(),
    }


def _shear(rng, n):
    return {"gamma1": rng.normal(0, 0.05, n), "gamma2": rng.normal(0, 0.05, n)}


def single_sie(seed=1000, batch=1):
    """Single image: 60x60 at 0.05"/pix; SIE (theta_E~U(0.8,1.5), e1,e2~N(0,0.1)
    clipped to |e|<0.4, centre~N(0,0.05)) + SHEAR (gamma~N(0,0.05)); source
    SERSIC_ELLIPSE (amp~U(10,100), R~U(0.1,0.5), n~U(1,4), e~N(0,0.1),
    centre~N(0,0.1)); lens light SERSIC_ELLIPSE (R~U(0.5,1.5), n~U(2,5), at the
    lens centre); supersampling 1; 11x11 PIXEL kernel of a FWHM 0.1" Gaussian."""
    rng = np.random.default_rng(seed)
    n = batch
    e1, e2 = _ellip(rng, 0.1, n, clip=0.4)
    cx, cy = rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)
    lens = [{"theta_E": rng.uniform(0.8, 1.5, n), "e1": e1, "e2": e2,
             "center_x": cx, "center_y": cy}, _shear(rng, n)]
    src = [_sersic_source(rng, n)]
    ll = [_sersic_lens_light(rng, n, cx, cy)]
    model = dict(num_pix=60, delta_pix=0.05, supersampling_factor=1,
                 lens_model_list=["SIE", "SHEAR"], source_light_model_list=["SERSIC_ELLIPSE"],
                 lens_light_model_list=["SERSIC_ELLIPSE"])
    kernels = np.stack([gaussian_pixel_kernel(0.1, 0.05, 11)] * n)
    return model, lens, src, ll, kernels


def batch_epl(seed=1001, batch=1024, num_pix=180, delta_pix=0.04, supersampling=3,
              kernel_size=31):
    """Batch of EPL+SHEAR systems: 180x180 at 0.04"/pix, supersampling 3; EPL
    (theta_E~U(0.8,1.5), gamma~U(1.8,2.2), e1,e2~N(0,0.1)); light as
    :func:`single_sie`; one 31x31 Moffat kernel per system (beta~U(2.5,4.5),
    FWHM~U(0.08,0.15)")."""
    rng = np.random.default_rng(seed)
    n = batch
    e1, e2 = _ellip(rng, 0.1, n)
    cx, cy = rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)
    lens = [{"theta_E": rng.uniform(0.8, 1.5, n), "gamma": rng.uniform(1.8, 2.2, n),
             "e1": e1, "e2": e2, "center_x": cx, "center_y": cy}, _shear(rng, n)]
    src = [_sersic_source(rng, n)]
    ll = [_sersic_lens_light(rng, n, cx, cy)]
    betas = rng.uniform(2.5, 4.5, n)
    fwhms = rng.uniform(0.08, 0.15, n)
    kernels = np.stack([moffat_pixel_kernel(f, b, delta_pix, kernel_size)
                        for f, b in zip(fwhms, betas)])
    model = dict(num_pix=num_pix, delta_pix=delta_pix, supersampling_factor=supersampling,
                 lens_model_list=["EPL", "SHEAR"], source_light_model_list=["SERSIC_ELLIPSE"],
                 lens_light_model_list=["SERSIC_ELLIPSE"])
    return model, lens, src, ll, kernels


def instance(kwargs_list, i):
    """Scalar kwargs of system ``i`` from a batched (vmap-layout) kwargs list."""
    return [{k: float(np.asarray(v).reshape(-1)[i]) for k, v in kw.items()} for kw in kwargs_list]


def subset(kwargs_list, idx):
    """Batched kwargs restricted to the systems ``idx``."""
    return [{k: np.asarray(v)[idx] for k, v in kw.items()} for kw in kwargs_list]


def substructure(seed=1004, num_pix=1000, delta_pix=0.01, n_sub=2000):
    """Substructure ray shooting: a num_pix^2 grid of rays at delta_pix"/pix
    (1000^2 = 1M rays at 0.01") through EPL + SHEAR (as :func:`batch_epl`) plus
    n_sub TNFW subhalos (centres U(-2.5, 2.5)^2, Rs~U(0.01, 0.1), alpha_Rs
    log-uniform in [1e-4, 1e-2], r_trunc = 10 Rs), then a SERSIC_ELLIPSE source
    as in :func:`single_sie`.  Returns (x, y, lens_model_list, kwargs_lens,
    kwargs_source) with x, y the flattened ray grid."""
    rng = np.random.default_rng(seed)
    e1, e2 = _ellip(rng, 0.1, 1)
    cx, cy = rng.normal(0, 0.05, 1), rng.normal(0, 0.05, 1)
    lens = [{"theta_E": float(rng.uniform(0.8, 1.5)), "gamma": float(rng.uniform(1.8, 2.2)),
             "e1": float(e1[0]), "e2": float(e2[0]), "center_x": float(cx[0]),
             "center_y": float(cy[0])},
            {k: float(v[0]) for k, v in _shear(rng, 1).items()}]
    sx = rng.uniform(-2.5, 2.5, n_sub)
    sy = rng.uniform(-2.5, 2.5, n_sub)
    rs = rng.uniform(0.01, 0.1, n_sub)
    ars = 10.0 ** rng.uniform(-4, -2, n_sub)
    for i in range(n_sub):
        lens.append({"Rs": float(rs[i]), "alpha_Rs": float(ars[i]), "r_trunc": float(10 * rs[i]),
                     "center_x": float(sx[i]), "center_y": float(sy[i])})
    src = [{k: float(v[0]) for k, v in _sersic_source(rng, 1).items()}]
    g = grid_kwargs(num_pix, delta_pix)
    c = np.arange(num_pix) * delta_pix
    xx, yy = np.meshgrid(g["ra_at_xy_0"] + c, g["dec_at_xy_0"] + c)
    lens_list = ["EPL", "SHEAR"] + ["TNFW"] * n_sub
    return xx.reshape(-1), yy.reshape(-1), lens_list, lens, src


def line_of_sight_halos(seed=1005, num_pix=400, half_width=10.0, n_halos=5130, n_planes=126,
                        z_lens=0.5, z_source=2.5, cone_radius=2.75, num_deflectors=5500):
    """Multi-plane substructure ray shooting with the shapes of the reference's
    GPU notebook benchmark (a pyHalo CDM realisation: 400^2 rays on
    linspace(-10, 10) through 5130 TNFW halos and 126 CONVERGENCE sheets,
    z_lens = 0.5, z_source = 2.5, padded to 5500 deflectors), drawn here
    synthetically: n_planes planes at z = linspace(0.02, z_source - 0.02); 30%
    of the halos on the plane nearest z_lens (subhalos), the rest uniform over
    the planes; centres uniform in a disk of radius cone_radius arcsec; masses
    log10 m ~ dN/dlog m ∝ m^-0.9 on [6, 10] with Rs = 0.05 (m / 1e8)^(1/3)
    arcsec, alpha_Rs = 0.004 (m / 1e8)^(2/3) arcsec, r_trunc = U(5, 20) Rs; one
    negative CONVERGENCE sheet kappa ~ -U(0.001, 0.006) per plane.  Returns
    (x, y, lens_model_list, kwargs_lens, lens_redshift_list, z_source,
    num_deflectors) with x, y the flattened ray grid (x fastest, as the
    notebook's np.tile / np.repeat)."""
    rng = np.random.default_rng(seed)
    planes = np.linspace(0.02, z_source - 0.02, n_planes)
    main = int(np.argmin(np.abs(planes - z_lens)))
    n_sub = int(0.3 * n_halos)
    zi = np.concatenate([np.full(n_sub, main), rng.integers(0, n_planes, n_halos - n_sub)])
    # inverse-CDF draw of dN/dlog m ∝ m^-0.9 on [1e6, 1e10]
    u = rng.uniform(0, 1, n_halos)
    a = -0.9 * np.log(10.0)
    lm = 6.0 + np.log1p(u * np.expm1(a * 4.0)) / a
    m8 = 10.0 ** (lm - 8.0)
    r = cone_radius * np.sqrt(rng.uniform(0, 1, n_halos))
    ph = rng.uniform(0, 2 * np.pi, n_halos)
    rs = 0.05 * m8 ** (1.0 / 3.0)
    lens_list, kwargs, z = [], [], []
    for i in range(n_halos):
        lens_list.append("TNFW")
        kwargs.append({"Rs": float(rs[i]), "alpha_Rs": float(0.004 * m8[i] ** (2.0 / 3.0)),
                       "r_trunc": float(rs[i] * rng.uniform(5, 20)),
                       "center_x": float(r[i] * np.cos(ph[i])),
                       "center_y": float(r[i] * np.sin(ph[i]))})
        z.append(float(planes[zi[i]]))
    for k in range(n_planes):
        lens_list.append("CONVERGENCE")
        kwargs.append({"kappa": float(-rng.uniform(0.001, 0.006))})
        z.append(float(planes[k]))
    x = np.tile(np.linspace(-half_width, half_width, num_pix), num_pix)
    y = np.repeat(np.linspace(-half_width, half_width, num_pix), num_pix)
    return x, y, lens_list, kwargs, z, z_source, num_deflectors


SERVING_STACKS = ("SIE+SHEAR", "EPL+SHEAR", "EPL_MULTIPOLE_M1M3M4+SHEAR", "NFW_ELLIPSE_CSE+SHEAR")


def serving_stream(seed=1002, n=50000, sides=(60, 100, 180, 300), supersampling=(1, 2, 4),
                   kernel_sizes=(11, 21, 41), delta_pix=0.05, psf_pool=32):
    """Request stream of the serving workload: per request a grid side, a
    supersampling factor and a PSF size drawn uniformly from the given sets, a
    lens stack drawn uniformly from SIE+SHEAR, EPL+SHEAR,
    EPL_MULTIPOLE_M1M3M4+SHEAR (multipole amplitudes a{1,3,4}_a~N(0,0.01),
    angles delta_phi_m{1,3,4}~U(0,pi)) and NFW_ELLIPSE_CSE+SHEAR (Rs~U(5,20),
    alpha_Rs~U(0.5,2)); 1 or 2 SERSIC_ELLIPSE sources and a SERSIC_ELLIPSE lens
    light drawn as in :func:`single_sie` / :func:`batch_epl`.  PSFs are Moffat
    kernels (beta~U(2.5,4.5), FWHM~U(0.08,0.15)") taken from a seeded pool of
    ``psf_pool`` kernels per size.  Returns (requests, psfs): each request a dict
    with key (side, s, K, stack, n_sources), kwargs lists and a PSF index."""
    rng = np.random.default_rng(seed)
    psfs = {}
    for K in kernel_sizes:
        b = rng.uniform(2.5, 4.5, psf_pool)
        f = rng.uniform(0.08, 0.15, psf_pool)
        psfs[K] = np.stack([moffat_pixel_kernel(f[i], b[i], delta_pix, K) for i in range(psf_pool)])
    side = rng.choice(sides, n)
    ss = rng.choice(supersampling, n)
    ks = rng.choice(kernel_sizes, n)
    stack = rng.integers(0, len(SERVING_STACKS), n)
    nsrc = rng.integers(1, 3, n)
    pidx = rng.integers(0, psf_pool, n)
    e1, e2 = _ellip(rng, 0.1, n, clip=0.4)
    cx, cy = rng.normal(0, 0.05, n), rng.normal(0, 0.05, n)
    theta = rng.uniform(0.8, 1.5, n)
    gam = rng.uniform(1.8, 2.2, n)
    am = rng.normal(0, 0.01, (n, 3))
    phim = rng.uniform(0, np.pi, (n, 3))
    rs = rng.uniform(5, 20, n)
    ars = rng.uniform(0.5, 2, n)
    sh = _shear(rng, n)
    src1 = _sersic_source(rng, n)
    src2 = _sersic_source(rng, n)
    ll = _sersic_lens_light(rng, n, cx, cy)
    out = []
    for i in range(n):
        st = SERVING_STACKS[stack[i]]
        if st == "SIE+SHEAR":
            main = {"theta_E": theta[i], "e1": e1[i], "e2": e2[i], "center_x": cx[i],
                    "center_y": cy[i]}
        elif st == "NFW_ELLIPSE_CSE+SHEAR":
            main = {"Rs": rs[i], "alpha_Rs": ars[i], "e1": e1[i], "e2": e2[i],
                    "center_x": cx[i], "center_y": cy[i]}
        else:
            main = {"theta_E": theta[i], "gamma": gam[i], "e1": e1[i], "e2": e2[i],
                    "center_x": cx[i], "center_y": cy[i]}
            if st.startswith("EPL_MULTIPOLE"):
                main.update({"a1_a": am[i, 0], "delta_phi_m1": phim[i, 0], "a3_a": am[i, 1],
                             "delta_phi_m3": phim[i, 1], "a4_a": am[i, 2],
                             "delta_phi_m4": phim[i, 2]})
        kl = [{k: float(v) for k, v in main.items()},
              {"gamma1": float(sh["gamma1"][i]), "gamma2": float(sh["gamma2"][i])}]
        srcs = [src1, src2][:int(nsrc[i])]
        kss = [{k: float(v[i]) for k, v in s.items()} for s in srcs]
        kll = [{k: float(v[i]) for k, v in ll.items()}]
        out.append({"key": (int(side[i]), int(ss[i]), int(ks[i]), st, int(nsrc[i])),
                    "kwargs_lens": kl, "kwargs_source": kss, "kwargs_lens_light": kll,
                    "psf": int(pidx[i])})
    return out, psfs


def serving_model(key, delta_pix=0.05, precision="fp32", data=None, exposure_time=1000.0,
                  background_rms=0.01):
    """ImageModel of a serving request key (side, s, K, stack, n_sources)."""
    from . import ImageData, ImageModel, LensModel, LightModel, PSF
    side, s, K, stack, nsrc = key
    g = grid_kwargs(side, delta_pix)
    d = ImageData(np.zeros((side, side)) if data is None else data, exposure_time=exposure_time,
                  background_rms=background_rms, **g)
    psf = PSF("PIXEL", kernel_point_source=gaussian_pixel_kernel(0.1, delta_pix, K))
    return ImageModel(d, psf, LensModel(stack.split("+")),
                      LightModel(["SERSIC_ELLIPSE"] * nsrc), LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": s, "precision": precision})


def gradient_batch(seed=1003, batch=256, num_pix=120, delta_pix=0.05, supersampling=2,
                   kernel_size=21):
    """Gradient workload: EPL+SHEAR lens (as :func:`batch_epl`), SERSIC_ELLIPSE
    source and lens light (as :func:`single_sie`), 120x120 at 0.05"/pix,
    supersampling 2, one 21x21 Moffat PSF per system; 6 + 4 + 7 + 7 parameters
    per system (22 free when SHEAR's ra_0, dec_0 are held).  Data come from
    :func:`noisy_data` applied to the simulated images."""
    model, lens, src, ll, kern = batch_epl(seed=seed, batch=batch, num_pix=num_pix,
                                           delta_pix=delta_pix, supersampling=supersampling,
                                           kernel_size=kernel_size)
    return model, lens, src, ll, kern


def noisy_data(images, seed=2003, background_rms=0.01, exposure_time=1000.0):
    """image + N(0, background_rms^2) + Poisson(image t)/t - image, with the image
    clipped at 0 for the Poisson draw."""
    rng = np.random.default_rng(seed)
    img = np.asarray(images, dtype=float)
    counts = rng.poisson(np.clip(img, 0, None) * exposure_time)
    return img + rng.normal(0, background_rms, img.shape) + counts / exposure_time - np.clip(
        img, 0, None)
