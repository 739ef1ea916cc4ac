"""Adjoint likelihood gradient (lensgb_loglike_grad through the C ABI) against
central finite differences.

Tolerance: |g - g_fd| <= 1e-4 * (|g_fd| + 1e-3 * max_k |g_fd_k|) per component,
with FD step 1e-6 (central).  FD of the GPU FP64 likelihood covers the batch;
FD of the FP64 oracle (the reference's likelihood restated) covers one small
system, tying the adjoint to the reference's own likelihood.
"""

import numpy as np
import pytest
import torch

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import autograd, workloads as W
from oracle import image as oimage

pytestmark = pytest.mark.gpu

STEP = 1e-6
RTOL = 1e-4


def _model(num_pix, s, kern, precision="fp64"):
    g = W.grid_kwargs(num_pix, 0.05)
    data = J.ImageData(np.zeros((num_pix, num_pix)), exposure_time=1000.0, background_rms=0.01,
                       **g)
    return J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern), J.LensModel(["EPL", "SHEAR"]),
                        J.LightModel(["SERSIC_ELLIPSE"]), J.LightModel(["SERSIC_ELLIPSE"]),
                        kwargs_numerics={"supersampling_factor": s, "precision": precision})


def _setup(batch=4, num_pix=32, s=2, K=11, seed=1003):
    model, lens, src, ll, kern = W.gradient_batch(seed=seed, batch=batch, num_pix=num_pix,
                                                  supersampling=s, kernel_size=K)
    im = _model(num_pix, s, kern[0])
    rows = im.pack_params(lens, src, ll)
    # simulate at slightly shifted parameters so that the gradient is not ~0
    truth = rows.copy()
    truth[:, 0] *= 1.01
    img = im.image_batch(rows=truth, psf_kernels=kern).cpu().numpy()
    data = W.noisy_data(img)
    return im, rows, kern, data


def _fd(im, rows, kern, data):
    B, P = rows.shape
    pert = np.repeat(rows[:, None, :], 2 * P, axis=1)
    for k in range(P):
        pert[:, 2 * k, k] += STEP
        pert[:, 2 * k + 1, k] -= STEP
    pert = pert.reshape(B * 2 * P, P)
    d = np.repeat(data, 2 * P, axis=0)
    kk = None if kern is None else np.repeat(kern, 2 * P, axis=0)
    ll = im.likelihood_batch(rows=pert, data=d, psf_kernels=kk).cpu().numpy().reshape(B, P, 2)
    return (ll[..., 0] - ll[..., 1]) / (2 * STEP)


def _check(g, fd):
    scale = np.abs(fd).max(axis=1, keepdims=True)
    bound = RTOL * (np.abs(fd) + 1e-3 * scale)
    bad = np.abs(g - fd) > bound
    assert not bad.any(), (np.argwhere(bad), g[bad], fd[bad])


def test_adjoint_matches_central_differences(cuda):
    im, rows, kern, data = _setup()
    logl, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kern)
    ref = im.likelihood_batch(rows=rows, data=data, psf_kernels=kern)
    np.testing.assert_array_equal(logl.cpu().numpy(), ref.cpu().numpy())
    _check(grad.cpu().numpy(), _fd(im, rows, kern, data))


def test_adjoint_without_psf_and_with_noise_map_and_mask(cuda):
    model, lens, src, ll, kern = W.gradient_batch(batch=2, num_pix=24, supersampling=1,
                                                  kernel_size=5)
    g = W.grid_kwargs(24, 0.05)
    rng = np.random.default_rng(4)
    noise = 0.02 + 0.01 * rng.random((24, 24))
    mask = (rng.random((24, 24)) > 0.2).astype(float)
    data = J.ImageData(np.zeros((24, 24)), exposure_time=500.0, background_rms=0.02,
                       noise_map=noise, **g)
    im = J.ImageModel(data, J.PSF("NONE"), J.LensModel(["EPL", "SHEAR"]),
                      J.LightModel(["SERSIC_ELLIPSE"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": 1}, likelihood_mask=mask)
    rows = im.pack_params(lens, src, ll)
    d = W.noisy_data(im.image_batch(rows=rows).cpu().numpy() * 1.02)
    logl, grad = im.likelihood_grad_batch(rows=rows, data=d)
    B, P = rows.shape
    fd = np.zeros((B, P))
    for k in range(P):
        rp, rm = rows.copy(), rows.copy()
        rp[:, k] += STEP
        rm[:, k] -= STEP
        fd[:, k] = (im.likelihood_batch(rows=rp, data=d).cpu().numpy()
                    - im.likelihood_batch(rows=rm, data=d).cpu().numpy()) / (2 * STEP)
    _check(grad.cpu().numpy(), fd)


def test_adjoint_matches_oracle_likelihood_differences(cuda):
    """FD of the oracle's FP64 likelihood (the reference's algorithm) for one
    small system equals the adjoint gradient."""
    im, rows, kern, data = _setup(batch=1, num_pix=20, s=2, K=5)
    _, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kern)
    kl, ks, kll = im.unpack_params(rows)
    scene = dict(nx=20, ny=20, supersampling_factor=2, psf_type="PIXEL", kernel=kern[0],
                 convolution_type="grid", lens_model_list=["EPL", "SHEAR"],
                 source_light_model_list=["SERSIC_ELLIPSE"],
                 lens_light_model_list=["SERSIC_ELLIPSE"], **W.grid_kwargs(20, 0.05))

    def logl(r):
        a, b, c = im.unpack_params(r[None])
        kw = lambda lst: [{k: float(v[0]) for k, v in d.items()} for d in lst]  # noqa: E731
        model = oimage.image(scene, kw(a), kw(b), kw(c))
        return oimage.log_likelihood(model, data[0], np.ones((20, 20)), 0.01,
                                     exposure_time=1000.0)

    P = rows.shape[1]
    fd = np.zeros((1, P))
    for k in range(P):
        rp, rm = rows[0].copy(), rows[0].copy()
        rp[k] += STEP
        rm[k] -= STEP
        fd[0, k] = (logl(rp) - logl(rm)) / (2 * STEP)
    _check(grad.cpu().numpy(), fd)


def test_autograd_function(cuda):
    im, rows, kern, data = _setup(batch=3)
    r = torch.as_tensor(rows).cuda().requires_grad_(True)
    out = autograd.log_likelihood(r, im, data=data, psf_kernels=kern)
    w = torch.tensor([1.0, -2.0, 0.5], dtype=torch.float64, device="cuda")
    (out * w).sum().backward()
    _, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kern)
    np.testing.assert_array_equal(r.grad.cpu().numpy(), (w[:, None] * grad).cpu().numpy())


@pytest.mark.parametrize("lens", ["SIE", "NIE"])
def test_isothermal_lenses_match_central_differences(cuda, lens):
    """SIE / NIE + SHEAR: the NIE major-axis formula differentiated in (b, s, q,
    x1, y1) and chained to (theta_E, e1, e2, [s_scale,] centre)."""
    model, lens_kw, src, ll, kern = W.gradient_batch(seed=1009, batch=3, num_pix=32,
                                                     supersampling=2, kernel_size=11)
    main = {k: v for k, v in lens_kw[0].items() if k != "gamma"}
    if lens == "NIE":
        main = dict(main, s_scale=np.full(3, 0.05))
        main = {k: main[k] for k in ("theta_E", "e1", "e2", "s_scale", "center_x", "center_y")}
    g = W.grid_kwargs(32, 0.05)
    data_cls = J.ImageData(np.zeros((32, 32)), exposure_time=1000.0, background_rms=0.01, **g)
    im = J.ImageModel(data_cls, J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel([lens, "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": 2})
    rows = im.pack_params([main, lens_kw[1]], src, ll)
    truth = rows.copy()
    truth[:, 0] *= 1.01
    data = W.noisy_data(im.image_batch(rows=truth, psf_kernels=kern).cpu().numpy())
    logl, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kern)
    _check(grad.cpu().numpy(), _fd(im, rows, kern, data))


def test_nfw_halos_match_central_differences(cuda):
    """EPL + SHEAR + an NFW halo + a TNFW subhalo near the arc: the NFW / TNFW
    deflections differentiated in (Rs, alpha_Rs, [r_trunc,] centre)."""
    model, lens_kw, src, ll, kern = W.gradient_batch(seed=1013, batch=3, num_pix=32,
                                                     supersampling=2, kernel_size=11)
    rng = np.random.default_rng(7)
    nfw = {"Rs": rng.uniform(0.8, 1.5, 3), "alpha_Rs": rng.uniform(0.1, 0.3, 3),
           "center_x": rng.uniform(-0.1, 0.1, 3), "center_y": rng.uniform(-0.1, 0.1, 3)}
    tnfw = {"Rs": rng.uniform(0.1, 0.3, 3), "alpha_Rs": rng.uniform(0.02, 0.06, 3),
            "r_trunc": rng.uniform(0.3, 0.8, 3), "center_x": rng.uniform(0.4, 0.6, 3),
            "center_y": rng.uniform(-0.3, 0.3, 3)}
    g = W.grid_kwargs(32, 0.05)
    data_cls = J.ImageData(np.zeros((32, 32)), exposure_time=1000.0, background_rms=0.01, **g)
    im = J.ImageModel(data_cls, J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(["EPL", "SHEAR", "NFW", "TNFW"]),
                      J.LightModel(["SERSIC_ELLIPSE"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": 2})
    rows = im.pack_params(list(lens_kw) + [nfw, tnfw], src, ll)
    truth = rows.copy()
    truth[:, 0] *= 1.01
    data = W.noisy_data(im.image_batch(rows=truth, psf_kernels=kern).cpu().numpy())
    logl, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kern)
    _check(grad.cpu().numpy(), _fd(im, rows, kern, data))


def test_too_many_parameters_raise(cuda):
    """Rows above 64 parameters (here 12 + 4 + 7 x 7 = 65) are refused."""
    g = W.grid_kwargs(16, 0.05)
    data = J.ImageData(np.zeros((16, 16)), exposure_time=100.0, background_rms=0.01, **g)
    im = J.ImageModel(data, J.PSF("NONE"), J.LensModel(["EPL_MULTIPOLE_M1M3M4", "SHEAR"]),
                      J.LightModel(["SERSIC_ELLIPSE"] * 7), J.LightModel([]))
    kl = [{"theta_E": 1.0, "gamma": 2.0, "e1": 0.1, "e2": 0.0, "center_x": 0, "center_y": 0,
           "a1_a": 0.0, "delta_phi_m1": 0.0, "a3_a": 0.0, "delta_phi_m3": 0.0, "a4_a": 0.0,
           "delta_phi_m4": 0.0}, {"gamma1": 0.0, "gamma2": 0.0}]
    ks = [{"amp": 1.0, "R_sersic": 0.3, "n_sersic": 2, "e1": 0.0, "e2": 0.0, "center_x": 0,
           "center_y": 0}] * 7
    with pytest.raises(Exception):
        im.likelihood_grad_batch(kl, ks, [], data=np.zeros((16, 16)))


# ---------------------------------------------------------------------------
# against finite differences of the reference's own likelihood
# ---------------------------------------------------------------------------

FD_CASES = golden_io.grad_fd_cases()


def _fd_case_model(c, precision="fp64"):
    n = c["num_pix"]
    g = W.grid_kwargs(n, c["delta_pix"])
    data = J.ImageData(np.asarray(c["data"]), exposure_time=1000.0, background_rms=0.01, **g)
    pk = c["psf_kwargs"]
    if pk["psf_type"] == "PIXEL":
        psf = J.PSF("PIXEL", kernel_point_source=c["kernel"],
                    point_source_supersampling_factor=pk.get("point_source_supersampling_factor",
                                                             1))
    elif pk["psf_type"] == "GAUSSIAN":
        psf = J.PSF("GAUSSIAN", fwhm=pk["fwhm"], truncation=pk["truncation"])
    else:
        psf = J.PSF("NONE")
    numerics = dict(c.get("numerics") or {}, supersampling_factor=c["s"], precision=precision)
    return J.ImageModel(data, psf, J.LensModel(c["lens"]), J.LightModel(c["src"]),
                        J.LightModel(c["ll"]), kwargs_numerics=numerics)


@pytest.mark.parametrize("c", FD_CASES, ids=lambda c: c["tag"])
def test_adjoint_matches_reference_finite_differences(cuda, c):
    """The adjoint against finite differences of the reference's
    likelihood_data_given_model run through the NumPy stand-in for jax
    (tests/golden/grad_fd.npz): NFW_ELLIPSE_CSE with a GAUSSIAN PSF,
    EPL_MULTIPOLE_M1M3M4 with two sources, SIE + CONVERGENCE + SHEAR without a
    PSF, convolution on the supersampled grid with a split PIXEL kernel and
    with a GAUSSIAN kernel, and the gradient workload's first system.  A
    component passes when it matches the five-point stencil (step 1e-4) or the
    central difference (step 1e-6), whichever a kink of the likelihood (the
    Sersic core floor, max(m, 0) of the noise) spares."""
    im = _fd_case_model(c)
    rows = im.pack_params(c["kwargs_lens"], c["kwargs_source"], c["kwargs_lens_light"])
    logl, grad = im.likelihood_grad_batch(rows=rows)
    assert abs(float(logl[0]) - c["logL"]) <= 1e-10 * abs(c["logL"])
    g = grad.cpu().numpy()[0]
    g5, g2 = c["grad_5pt"], c["grad_central_1e-6"]
    scale = np.abs(g5).max()
    ok5 = np.abs(g - g5) <= RTOL * (np.abs(g5) + 1e-3 * scale)
    ok2 = np.abs(g - g2) <= RTOL * (np.abs(g2) + 1e-3 * scale)
    bad = ~(ok5 | ok2)
    assert not bad.any(), [(c["param_order"][k], g[k], g5[k], g2[k]) for k in np.where(bad)[0]]


def test_fp32_model_gradient_equals_fp64_model_gradient(cuda):
    """An FP32 model differentiates through its FP64 twin: same logL and
    gradient bits as the FP64 model."""
    c = FD_CASES[1]
    out = {}
    for prec in ("fp64", "fp32"):
        im = _fd_case_model(c, prec)
        rows = im.pack_params(c["kwargs_lens"], c["kwargs_source"], c["kwargs_lens_light"])
        out[prec] = [t.cpu().numpy() for t in im.likelihood_grad_batch(rows=rows)]
    np.testing.assert_array_equal(out["fp32"][0], out["fp64"][0])
    np.testing.assert_array_equal(out["fp32"][1], out["fp64"][1])


def _batch_fd_model(lens_list, extra_kw, psf, numerics, num_pix=30, seed=1017):
    model, lens_kw, src, ll, kern = W.gradient_batch(seed=seed, batch=3, num_pix=num_pix,
                                                     supersampling=2, kernel_size=9)
    g = W.grid_kwargs(num_pix, 0.05)
    data_cls = J.ImageData(np.zeros((num_pix, num_pix)), exposure_time=1000.0,
                           background_rms=0.01, **g)
    im = J.ImageModel(data_cls, psf(kern), J.LensModel(lens_list),
                      J.LightModel(["SERSIC_ELLIPSE"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics=dict({"supersampling_factor": 2}, **numerics))
    rows = im.pack_params(extra_kw(lens_kw), src, ll)
    truth = rows.copy()
    truth[:, 0] *= 1.01
    kk = None if im._psf_type != 1 or numerics.get("supersampling_convolution") else kern
    data = W.noisy_data(im.image_batch(rows=truth, psf_kernels=kk).cpu().numpy())
    return im, rows, kk, data


def test_cse_and_multipole_batches_match_central_differences(cuda):
    """Batches of three systems: NFW_ELLIPSE_CSE + SHEAR and
    EPL_MULTIPOLE_M1M3M4 + SHEAR against central differences of the GPU FP64
    likelihood."""
    rng = np.random.default_rng(11)
    cases = [
        (["NFW_ELLIPSE_CSE", "SHEAR"],
         lambda kw: [{"Rs": rng.uniform(5, 20, 3), "alpha_Rs": rng.uniform(0.5, 2, 3),
                      "e1": kw[0]["e1"], "e2": kw[0]["e2"], "center_x": kw[0]["center_x"],
                      "center_y": kw[0]["center_y"]}, kw[1]]),
        (["EPL_MULTIPOLE_M1M3M4", "SHEAR"],
         lambda kw: [dict(kw[0], a1_a=rng.normal(0, 0.01, 3),
                          delta_phi_m1=rng.uniform(0, np.pi, 3), a3_a=rng.normal(0, 0.01, 3),
                          delta_phi_m3=rng.uniform(0, np.pi, 3), a4_a=rng.normal(0, 0.01, 3),
                          delta_phi_m4=rng.uniform(0, np.pi, 3)), kw[1]]),
    ]
    for lens_list, extra in cases:
        im, rows, kk, data = _batch_fd_model(
            lens_list, extra, lambda k: J.PSF("PIXEL", kernel_point_source=k[0]), {})
        _, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kk)
        _check(grad.cpu().numpy(), _fd(im, rows, kk, data))


def test_subframe_gradient_matches_central_differences(cuda):
    """flux_evaluate_indexes (NumericsSubFrame): the full-frame residual cropped
    to the sub-frame, the transposed convolution there and the evaluation mask."""
    yy, xx = np.mgrid[0:30, 0:30]
    fei = (yy - 13) ** 2 + (xx - 16) ** 2 <= 90
    im, rows, kk, data = _batch_fd_model(
        ["EPL", "SHEAR"], lambda kw: list(kw),
        lambda k: J.PSF("PIXEL", kernel_point_source=k[0]), {"flux_evaluate_indexes": fei})
    _, grad = im.likelihood_grad_batch(rows=rows, data=data, psf_kernels=kk)
    _check(grad.cpu().numpy(), _fd(im, rows, kk, data))


# ---------------------------------------------------------------------------
# FP32 per-ray derivatives (gradient_precision "fp32")
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("c", FD_CASES, ids=lambda c: c["tag"])
def test_fp32_adjoint_matches_reference_finite_differences(cuda, c):
    """FP32 dual numbers from FP64-accurate offsets (FP64 forward image, weights
    and reduction) against the reference's finite differences: the same 1e-4
    bar as the FP64 adjoint."""
    c = dict(c, numerics=dict(c.get("numerics") or {}, gradient_precision="fp32"))
    im = _fd_case_model(c)
    rows = im.pack_params(c["kwargs_lens"], c["kwargs_source"], c["kwargs_lens_light"])
    logl, grad = im.likelihood_grad_batch(rows=rows)
    assert abs(float(logl[0]) - c["logL"]) <= 1e-10 * abs(c["logL"])
    g = grad.cpu().numpy()[0]
    g5, g2 = c["grad_5pt"], c["grad_central_1e-6"]
    scale = np.abs(g5).max()
    ok5 = np.abs(g - g5) <= RTOL * (np.abs(g5) + 1e-3 * scale)
    ok2 = np.abs(g - g2) <= RTOL * (np.abs(g2) + 1e-3 * scale)
    bad = ~(ok5 | ok2)
    assert not bad.any(), [(c["param_order"][k], g[k], g5[k], g2[k]) for k in np.where(bad)[0]]


def test_fp32_adjoint_batch_matches_fp64_adjoint(cuda):
    """The gradient workload's shapes (120x120, s = 2, 21x21): FP32 per-ray
    derivatives within 1e-4 of the FP64 adjoint (relative, floor 1e-3 of the
    largest component), and the same logL bits (the forward stays FP64)."""
    model, lens, src, ll, kern = W.gradient_batch(seed=1003, batch=8)
    out = {}
    for gp in ("fp64", "fp32"):
        g = W.grid_kwargs(120, 0.05)
        data = J.ImageData(np.zeros((120, 120)), exposure_time=1000.0, background_rms=0.01, **g)
        im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                          J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                          J.LightModel(["SERSIC_ELLIPSE"]),
                          kwargs_numerics={"supersampling_factor": 2, "gradient_precision": gp})
        rows = im.pack_params(lens, src, ll)
        truth = rows.copy()
        truth[:, 0] *= 1.01
        d = W.noisy_data(im.image_batch(rows=truth, psf_kernels=kern).cpu().numpy())
        out[gp] = [t.cpu().numpy() for t in im.likelihood_grad_batch(rows=rows, data=d,
                                                                     psf_kernels=kern)]
    np.testing.assert_array_equal(out["fp32"][0], out["fp64"][0])
    _check(out["fp32"][1], out["fp64"][1])
