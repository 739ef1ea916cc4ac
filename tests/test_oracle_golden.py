"""The oracle against golden vectors computed by the reference's own source
(tests/golden/make_golden.py) and against scipy at the reference's own
hyp2f1 test points (test/test_Util/test_hyp2f1_util.py:87-112)."""

import warnings

import numpy as np
import pytest
from scipy.special import hyp2f1 as hyp2f1_scipy

import golden_io
from oracle import image, lens, light

warnings.filterwarnings("ignore", category=RuntimeWarning)


@pytest.mark.parametrize("case", golden_io.profile_cases(),
                         ids=lambda c: "%s-%s" % (c["kind"], c["name"]))
def test_profiles_match_reference(case):
    if case["kind"] == "hessian":
        pytest.skip("Hessians have no oracle restatement; checked on the GPU")
    if case["kind"] == "lens":
        got = np.array(lens.deflection(case["name"], case["x"], case["y"], case["kwargs"]))
    else:
        got = light.profile(case["name"], case["x"], case["y"], case["kwargs"])[None]
    np.testing.assert_allclose(got, case["out"], rtol=1e-13, atol=1e-300)


def test_hyp2f1_reference_points():
    d, meta = golden_io.load("hyp2f1.npz")
    a, b, c = meta["a"], meta["b"], meta["c"]
    for z, nmax, ref in zip(d["z"], d["nmax"], d["out"]):
        got = lens.hyp2f1_lopez_temme_8(a, b, c, z, nmax=int(nmax))
        np.testing.assert_allclose(got, ref, rtol=1e-14)
        # the reference's own tolerances against scipy
        tol = 1e-5 if abs(z - (0.99 + 0.001j)) < 1e-12 else 1e-8
        np.testing.assert_allclose(got, hyp2f1_scipy(a, b, c, z), rtol=tol, atol=tol)


def test_hyp2f1_epl_domain_vs_scipy():
    # the EPL uses a=1, b=t/2, c=2-t/2 with |z| = f; the adaptive nmax must reach
    # 1e-8 of scipy across the whole f range (epl.py:311-319)
    rng = np.random.default_rng(3)
    for f in [0.05, 0.3, 0.5, 0.7, 0.8, 0.9, 0.95]:
        t = rng.uniform(0.6, 1.4)
        phi = rng.uniform(0, 2 * np.pi, 16)
        z = f * np.exp(1j * phi)
        got = lens.hyp2f1_lopez_temme_8(1.0, t / 2, 2 - t / 2, z, nmax=lens.epl_nmax(f))
        ref = hyp2f1_scipy(1.0, t / 2, 2 - t / 2, z)
        np.testing.assert_allclose(got, ref, rtol=1e-6)


@pytest.mark.parametrize("sc", golden_io.image_scenes()[0], ids=lambda s: s["tag"])
def test_images_match_reference(sc):
    scene = golden_io.oracle_scene(sc)
    got = image.image(scene, sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    ref = sc["image"]
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


@pytest.mark.parametrize("sc", golden_io.serving_scenes(), ids=lambda s: s["tag"])
def test_serving_scenes_match_reference(sc):
    """The four serving stacks with two sources at s = 4 and a 41x41 kernel."""
    scene = golden_io.oracle_scene(sc)
    got = image.image(scene, sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    ref = sc["image"]
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())


def test_likelihood_matches_reference():
    scenes, like = golden_io.image_scenes()
    sc = [s for s in scenes if s["tag"] == like["scene"]][0]
    scene = golden_io.oracle_scene(sc)
    model = image.image(scene, sc["kwargs_lens"], sc["kwargs_source"], sc["kwargs_lens_light"])
    mask = np.ones_like(model)
    got = image.log_likelihood(model, like["data"], mask, like["bkg"], like["exp_time"])
    np.testing.assert_allclose(got, like["logL"], rtol=1e-12)


def test_epl_gamma2_matches_sie_limit():
    # EPL with gamma=2 is the singular isothermal ellipsoid (epl.py docstring);
    # the reference SIE routes to NIE with s_scale=1e-10
    x = np.linspace(-2, 2, 41)
    y = np.linspace(-1.7, 1.9, 41)
    kw = dict(theta_E=1.1, e1=0.1, e2=-0.05, center_x=0.02, center_y=-0.01)
    a_epl = np.array(lens.epl(x, y, gamma=2.0, **kw))
    a_sie = np.array(lens.sie(x, y, **kw))
    np.testing.assert_allclose(a_epl, a_sie, rtol=1e-6, atol=1e-8)


def test_nfw_alpha_at_Rs():
    # alpha2rho0 normalises |alpha(R = Rs)| = alpha_Rs (nfw.py:386-395)
    ax, ay = lens.nfw(np.array([0.7]), np.array([0.0]), Rs=0.7, alpha_Rs=1.3)
    np.testing.assert_allclose(np.hypot(ax, ay), 1.3, rtol=1e-12)


def test_sersic_at_R_sersic_equals_amp():
    v = light.sersic(np.array([0.4]), np.array([0.0]), amp=7.0, R_sersic=0.4, n_sersic=3.0)
    np.testing.assert_allclose(v, 7.0, rtol=1e-14)


@pytest.mark.parametrize("case", golden_io.bulk_cases(), ids=lambda c: "+".join(c["unique"]))
def test_bulk_ray_shooting_matches_reference(case):
    """Oracle SinglePlaneBulk vs LensModelBulk run from the reference source."""
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        rk = lens.bulk_prepare(case["unique"], case["lens_list"], case["kwargs"],
                               case["num_deflectors"])
        bx, by = lens.bulk_ray_shooting(case["unique"], case["x"], case["y"], rk["all_kwargs"],
                                        rk["index_list"])
    np.testing.assert_allclose(bx, case["bx"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(by, case["by"], rtol=1e-12, atol=1e-14)


def test_bulk_equals_single_plane_sum():
    """Bulk ray shooting equals the LensModel sum over the same profile list
    (EPL + SHEAR + TNFW subhalos + NULL fillers)."""
    case = golden_io.bulk_cases()[0]
    rk = lens.bulk_prepare(case["unique"], case["lens_list"], case["kwargs"],
                           case["num_deflectors"])
    bx, by = lens.bulk_ray_shooting(case["unique"], case["x"], case["y"], rk["all_kwargs"],
                                    rk["index_list"])
    sx, sy = lens.ray_shooting(case["lens_list"], case["x"], case["y"], case["kwargs"])
    np.testing.assert_allclose(bx, sx, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(by, sy, rtol=1e-13, atol=1e-15)


def _ref_background():
    """The flat Lambda-CDM background the multi-plane goldens were made with."""
    import os
    import sys
    sys.path.insert(0, golden_io.GOLDEN)
    import refshim
    return refshim.Background(refshim.FlatLCDM(70.0, 0.3))


@pytest.mark.parametrize("case", golden_io.multi_plane_cases(), ids=lambda c: c["tag"])
def test_multi_plane_prepare_matches_reference(case):
    """Oracle MultiPlaneBulk.prepare_ray_shooting_kwargs: sorting, NULL source and
    filler steps, zero-filled arrays and distance lists, as the reference made them."""
    bg = _ref_background()
    rk = lens.multi_plane_prepare(case["unique"], case["lens_list"], case["kwargs"],
                                  case["z_source"], case["z"], bg.d_xy, bg.T_xy,
                                  case["num_deflectors"])
    ref = case["prep"]
    np.testing.assert_array_equal(rk["index_list"], ref["index_list"])
    assert set(rk["all_kwargs"]) == set(ref["all_kwargs"])
    for k, v in ref["all_kwargs"].items():
        np.testing.assert_array_equal(rk["all_kwargs"][k], v)
    for k in ("T_ij_list", "T_z_list", "reduced2physical_factor"):
        np.testing.assert_allclose(rk[k], ref[k], rtol=1e-14, atol=0)


@pytest.mark.parametrize("case", golden_io.multi_plane_cases(), ids=lambda c: c["tag"])
def test_multi_plane_ray_shooting_matches_reference(case):
    """Oracle MultiPlaneBulk.ray_shooting on the reference's prepared kwargs."""
    ref = case["prep"]
    bx, by = lens.multi_plane_ray_shooting(case["unique"], case["x"], case["y"],
                                           ref["all_kwargs"], ref["index_list"],
                                           ref["T_ij_list"], ref["T_z_list"],
                                           ref["reduced2physical_factor"])
    np.testing.assert_allclose(bx, case["bx"], rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(by, case["by"], rtol=1e-12, atol=1e-14)


def test_multi_plane_one_plane_equals_single_plane():
    """All deflectors on one plane: the multi-plane recurrence reduces to the
    single-plane sum scaled by r2p (D_s / D_ds) and T_ij/T_z (flat cosmology)."""
    case = golden_io.bulk_cases()[1]
    rk = lens.bulk_prepare(case["unique"], case["lens_list"], case["kwargs"])
    n = len(rk["index_list"])
    bg = _ref_background()
    zl, zs = 0.5, 2.0
    T_l, T_s = bg.T_xy(0, zl), bg.T_xy(0, zs)
    r2p = bg.d_xy(0, zs) / bg.d_xy(zl, zs)
    idx = np.append(rk["index_list"], len(case["unique"]))
    kw = {k: np.append(v, 0.0) for k, v in rk["all_kwargs"].items()}
    T_ij = np.array([T_l] + [0.0] * (n - 1) + [bg.T_xy(zl, zs)])
    T_z = np.array([T_l] * n + [T_s])
    r = np.array([r2p] * n + [0.0])
    bx, by = lens.multi_plane_ray_shooting(case["unique"], case["x"], case["y"], kw, idx, T_ij,
                                           T_z, r)
    sx, sy = lens.bulk_ray_shooting(case["unique"], case["x"], case["y"], rk["all_kwargs"],
                                    rk["index_list"])
    # beta = theta - alpha_red r2p D_ls T... ; with T_ij = T_s - T_l (flat):
    # beta = theta - (theta - s) r2p (T_s - T_l) / T_s where s = single-plane beta
    scale = r2p * bg.T_xy(zl, zs) / T_s
    np.testing.assert_allclose(bx, case["x"] - (case["x"] - sx) * scale, rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(by, case["y"] - (case["y"] - sy) * scale, rtol=1e-12, atol=1e-13)


@pytest.mark.parametrize("case", golden_io.linear_cases(), ids=lambda c: c["tag"])
def test_linear_solve_matches_reference(case):
    """oracle.linear against the reference's ImageLinearFit (amplitudes, model
    image, inverse normal matrix, logL incl. marginalisation and positivity)."""
    from oracle import linear

    if case.get("ps_fixed"):
        pytest.skip("fixed-magnification amplitudes need lens Hessians (checked on the GPU)")
    sc = golden_io.linear_scene(case)
    logl, param, model, cov = linear.likelihood(
        sc, case["kl"], case["ks"], case["kll"], case["data"], case["mask"], case["bkg"],
        exposure_time=case["exp_time"], source_marg=case["marg"], check_positive_flux=case["pos"],
        kwargs_ps=case.get("ps"))
    np.testing.assert_allclose(param, case["param"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(model, case["model"], rtol=1e-10, atol=1e-12 * np.abs(model).max())
    assert abs(logl - case["logL"]) <= 1e-10 * abs(case["logL"])
    if case["cov"] is not None:
        np.testing.assert_allclose(cov, case["cov"], rtol=1e-9, atol=1e-14)


def _ps_kernel(case):
    """The kernel the reference renders with: the 3x3 delta when unconvolved or for
    a NONE PSF, else the (supersampled) PIXEL kernel, normalised."""
    if case["unconvolved"] or case["psf"]["psf_type"] == "NONE":
        k = np.zeros((3, 3))
        k[1, 1] = 1.0
        return k
    return case["kernel"] / case["kernel"].sum()


def _ps_render(case, models):
    from oracle import point_source as ops
    from jaxtronomy_gb300.workloads import grid_kwargs
    g = grid_kwargs(case["n"], case["dpix"])
    ra = np.concatenate([np.asarray(case["ps"][m]["ra_image"], float) for m in models])
    dec = np.concatenate([np.asarray(case["ps"][m]["dec_image"], float) for m in models])
    amp = np.concatenate([np.asarray(case["ps"][m]["point_amp"], float) for m in models])
    ra, dec = ops.displace_astrometry(ra, dec, case["special"])
    p = (case.get("numerics") or {}).get("point_source_supersampling_factor", 1)
    img = ops.render(case["n"], case["n"], g["transform_pix2angle"], g["ra_at_xy_0"],
                     g["dec_at_xy_0"], ra, dec, amp, _ps_kernel(case), p)
    return img * case["flux_scaling"]


@pytest.mark.parametrize("case", golden_io.point_source_cases(), ids=lambda c: c["tag"])
def test_point_source_images_match_reference(case):
    """Oracle extended image + rendered point sources (LENSED_POSITION + UNLENSED,
    astrometric shifts, flux scaling, unconvolved, NONE PSF, supersampled
    rendering) against the reference's ImageModel, its point-source term of model
    1 and its likelihood."""
    if case.get("fixed") and any(case["fixed"]):
        pytest.skip("fixed-magnification amplitudes need lens Hessians (checked on the GPU)")
    sc = golden_io.point_source_scene(case)
    ext = image.image(sc, case["lens"], case["src"], case["ll"], unconvolved=case["unconvolved"])
    model = ext + _ps_render(case, [0, 1])
    tol = 1e-10 * np.abs(case["image"]).max()
    np.testing.assert_allclose(model, case["image"], rtol=1e-10, atol=tol)
    if case["unconvolved"]:
        return
    np.testing.assert_allclose(_ps_render(case, [1]), case["ps1"], rtol=1e-10, atol=tol)
    logl = image.log_likelihood(model, case["data"], np.ones_like(model), 0.01,
                                exposure_time=800.0)
    assert abs(logl - case["logL"]) <= 1e-10 * abs(case["logL"])
