"""Host-side logic without a GPU: kwargs packing, validation mirroring the
reference's construction-time errors, PSF kernels and workload generation."""

import numpy as np
import pytest

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import profiles, workloads as W


def _image_model(psf=None, numerics=None, lens=("EPL", "SHEAR"), src=("SERSIC_ELLIPSE",),
                 ll=("SERSIC_ELLIPSE",), n=32):
    g = W.grid_kwargs(n, 0.05)
    data = J.ImageData(np.zeros((n, n)), exposure_time=100.0, background_rms=0.01, **g)
    psf = psf or J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, 0.05, 11))
    return J.ImageModel(data, psf, J.LensModel(list(lens)), J.LightModel(list(src)),
                        J.LightModel(list(ll)), kwargs_numerics=numerics)


def test_pack_params_layout_matches_header_order():
    im = _image_model()
    kl = [{"theta_E": 1.1, "gamma": 2.05, "e1": 0.1, "e2": -0.1, "center_x": 0.01,
           "center_y": 0.02}, {"gamma1": 0.03, "gamma2": -0.02}]
    ks = [{"amp": 10.0, "R_sersic": 0.2, "n_sersic": 2.0, "e1": 0.0, "e2": 0.1,
           "center_x": 0.0, "center_y": 0.05}]
    kll = [{"amp": 20.0, "R_sersic": 0.7, "n_sersic": 3.0, "e1": 0.05, "e2": 0.0,
            "center_x": 0.01, "center_y": 0.02}]
    rows = im.pack_params(kl, ks, kll)
    assert rows.shape == (1, 24)
    np.testing.assert_array_equal(rows[0, :6], [1.1, 2.05, 0.1, -0.1, 0.01, 0.02])
    np.testing.assert_array_equal(rows[0, 6:10], [0.03, -0.02, 0.0, 0.0])  # ra_0, dec_0 default
    np.testing.assert_array_equal(rows[0, 10:17], [10.0, 0.2, 2.0, 0.0, 0.1, 0.0, 0.05])


def test_pack_params_batched_kwargs():
    model, lens, src, ll, _ = W.batch_epl(batch=5, num_pix=20, kernel_size=5)
    im = _image_model()
    rows = im.pack_params(lens, src, ll)
    assert rows.shape == (5, 24)
    for i in range(5):
        r1 = im.pack_params(*[W.instance(k, i) for k in (lens, src, ll)])
        np.testing.assert_array_equal(rows[i], r1[0])


def test_missing_required_parameter_raises():
    im = _image_model()
    with pytest.raises(ValueError):
        im.pack_params([{"gamma": 2.0, "e1": 0, "e2": 0}, {"gamma1": 0, "gamma2": 0}],
                       [{"amp": 1, "R_sersic": 1, "n_sersic": 1, "e1": 0, "e2": 0}],
                       [{"amp": 1, "R_sersic": 1, "n_sersic": 1, "e1": 0, "e2": 0}])


def test_inconsistent_batch_raises():
    with pytest.raises(ValueError):
        profiles.batch_size([{"a": np.zeros(3)}, {"b": np.zeros(4)}])


def test_check_parameters_mirrors_reference():
    lm = J.LensModel(["SIE"])
    lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0, "center_y": 0}])
    with pytest.raises(ValueError):
        lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0}])
    with pytest.raises(ValueError):
        lm.check_parameters([{"theta_E": 1, "e1": 0, "e2": 0, "center_x": 0, "center_y": 0,
                              "gamma": 2}])
    with pytest.raises(ValueError):
        J.LightModel(["SERSIC"]).check_parameters([])


def test_unsupported_profiles_and_options_raise_at_construction():
    with pytest.raises(ValueError):
        J.LensModel(["PEMD"])
    with pytest.raises(ValueError):
        J.LightModel(["SHAPELETS"])
    with pytest.raises(ValueError):
        J.LensModel(["SIE"], multi_plane=True)
    with pytest.raises(ValueError):
        _image_model(numerics={"compute_mode": "adaptive"})
    with pytest.raises(TypeError):
        _image_model(numerics={"supersampling_factor": 2.0})
    with pytest.raises(TypeError):
        _image_model(numerics={"not_a_key": 1})
    with pytest.raises(ValueError):
        _image_model(numerics={"precision": "fp16"})
    with pytest.raises(ValueError):
        J.PSF("PIXEL", kernel_point_source=np.ones((4, 4)))
    with pytest.raises(ValueError):
        J.PSF("GAUSSIAN")


def test_pixel_psf_is_normalised_and_gaussian_kernel_follows_reference_size():
    k = np.ones((5, 5))
    assert abs(J.PSF("PIXEL", kernel_point_source=k).kernel_point_source.sum() - 1) < 1e-15
    from jaxtronomy_gb300.image_model import gaussian_kernel
    # radius = max(round(sigma * truncation), 1), convolution.py:204-206
    assert gaussian_kernel(0.8493, 5.0).shape == (9, 9)
    assert gaussian_kernel(0.1, 2.0).shape == (3, 3)
    assert abs(gaussian_kernel(1.7, 4.0).sum() - 1) < 1e-14


def test_image_data_grid_attributes():
    g = W.grid_kwargs(60, 0.05)
    d = J.ImageData(np.zeros((60, 60)), exposure_time=100.0, background_rms=0.01, **g)
    assert d.num_pixel_axes == (60, 60)
    assert abs(d.pixel_width - 0.05) < 1e-15
    cx, cy = d.center
    assert abs(cx) < 1e-12 and abs(cy) < 1e-12
    x, y = d.map_coord2pix(*d.map_pix2coord(3.0, 7.0))
    assert abs(x - 3) < 1e-12 and abs(y - 7) < 1e-12
    # exposure floor (image_noise.py:52-54)
    d2 = J.ImageData(np.zeros((4, 4)), exposure_time=0.0, background_rms=0.1)
    assert d2.exposure_map == 1e-10


def test_workloads_are_seeded_and_shaped():
    a = W.batch_epl(batch=8, num_pix=20, kernel_size=5)
    b = W.batch_epl(batch=8, num_pix=20, kernel_size=5)
    np.testing.assert_array_equal(a[1][0]["theta_E"], b[1][0]["theta_E"])
    assert a[4].shape == (8, 5, 5)
    np.testing.assert_allclose(a[4].sum(axis=(1, 2)), 1.0, rtol=1e-14)
    sie = W.single_sie(batch=500)[1][0]
    assert np.hypot(sie["e1"], sie["e2"]).max() < 0.4


def test_bulk_prepare_mirrors_reference_layout():
    """prepare_ray_shooting_kwargs builds the reference's index list and
    per-parameter arrays (single_plane_bulk.py:47-106), including NULL fillers."""
    from oracle import lens as olens
    unique = ["EPL", "SHEAR", "TNFW"]
    lens_list = ["EPL", "TNFW", "SHEAR", "TNFW"]
    kw = [{"theta_E": 1.0, "gamma": 2.0, "e1": 0.1, "e2": 0.0, "center_x": 0.0, "center_y": 0.0},
          {"Rs": 0.05, "alpha_Rs": 0.01, "r_trunc": 0.5, "center_x": 1.0, "center_y": 2.0},
          {"gamma1": 0.01, "gamma2": 0.02},
          {"Rs": 0.02, "alpha_Rs": 0.002, "r_trunc": 0.2, "center_x": -1.0, "center_y": 0.5}]
    b = J.LensModelBulk(unique, multi_plane=False)
    rk = b.prepare_ray_shooting_kwargs(lens_list, kw, num_deflectors=6)
    ref = olens.bulk_prepare(unique, lens_list, kw, 6)
    assert list(rk["index_list"]) == [0, 2, 1, 2, 3, 3] == list(ref["index_list"])
    assert set(rk["all_kwargs"]) == set(ref["all_kwargs"])
    for k in ref["all_kwargs"]:
        np.testing.assert_array_equal(rk["all_kwargs"][k], ref["all_kwargs"][k])
    idx, rows = b.pack_rows(rk["all_kwargs"], rk["index_list"])
    assert idx.dtype == np.int32 and rows.shape == (6, 12)
    np.testing.assert_array_equal(rows[1, :5], [0.05, 0.01, 0.5, 1.0, 2.0])
    np.testing.assert_array_equal(rows[2, :4], [0.01, 0.02, 0.0, 0.0])
    assert not rows[4:].any()


def test_bulk_pack_reproduces_positional_binding():
    """EPL_MULTIPOLE_M1M3M4 in the bulk path: the reference binds the arrays in
    param_names order to the derivatives signature, so the kernel row (read in
    param_names order) receives the shifted values."""
    b = J.LensModelBulk(["EPL_MULTIPOLE_M1M3M4"])
    names = profiles.LENS_PARAMS["EPL_MULTIPOLE_M1M3M4"]
    kw = [{n: float(i + 1) for i, n in enumerate(names)}]
    rk = b.prepare_ray_shooting_kwargs(["EPL_MULTIPOLE_M1M3M4"], kw)
    _, rows = b.pack_rows(rk["all_kwargs"], rk["index_list"])
    sig = profiles.DERIVATIVES_SIGNATURE["EPL_MULTIPOLE_M1M3M4"]
    # the value the reference binds to parameter `p` is the param_names value at
    # p's position in the signature
    for col, p in enumerate(names):
        assert rows[0, col] == kw[0][names[sig.index(p)]]


def test_bulk_errors_mirror_reference():
    with pytest.raises(ValueError):
        J.LensModelBulk(["NOT_A_PROFILE"])
    b = J.LensModelBulk(["TNFW"])
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW", "TNFW"], [{}])
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW", "TNFW"], [{}, {}], num_deflectors=1)


def test_substructure_workload_shape():
    x, y, ll, kw, src = W.substructure(num_pix=50, n_sub=20)
    assert x.shape == (2500,) and len(ll) == len(kw) == 22
    assert ll[:2] == ["EPL", "SHEAR"] and set(ll[2:]) == {"TNFW"}
    assert np.isclose(x.max() - x.min(), 49 * 0.01)
    assert all(k["r_trunc"] == 10 * k["Rs"] for k in kw[2:])


def test_serving_stream_is_seeded_and_covers_the_grid():
    reqs, psfs = W.serving_stream(n=400, psf_pool=4)
    reqs2, _ = W.serving_stream(n=400, psf_pool=4)
    assert [r["key"] for r in reqs] == [r["key"] for r in reqs2]
    keys = {r["key"] for r in reqs}
    assert {k[0] for k in keys} == {60, 100, 180, 300}
    assert {k[1] for k in keys} == {1, 2, 4} and {k[2] for k in keys} == {11, 21, 41}
    assert {k[3] for k in keys} == set(W.SERVING_STACKS) and {k[4] for k in keys} == {1, 2}
    for K, p in psfs.items():
        assert p.shape == (4, K, K) and np.allclose(p.sum(axis=(1, 2)), 1.0)
    r = next(r for r in reqs if r["key"][3].startswith("EPL_MULTIPOLE"))
    assert set(r["kwargs_lens"][0]) == set(profiles.LENS_PARAMS["EPL_MULTIPOLE_M1M3M4"])
    im = W.serving_model(r["key"])
    rows = im.pack_params(r["kwargs_lens"], r["kwargs_source"], r["kwargs_lens_light"])
    assert rows.shape[0] == 1


def test_split_kernel_product_equals_oracle_and_keeps_weight():
    from jaxtronomy_gb300.image_model import split_kernel
    from oracle import numerics as onum
    k = W.moffat_pixel_kernel(0.12, 3.0, 0.05 / 3, 27)
    for ssk in (1, 3, 5, 9):
        lo, hi = split_kernel(k, ssk, 3)
        lo2, hi2 = onum.split_kernel(k, ssk, 3)
        np.testing.assert_array_equal(lo, lo2)
        np.testing.assert_array_equal(hi, hi2)
        assert np.isclose(lo.sum() + hi.sum(), k.sum())
        assert hi.shape[0] % 2 == 1 and lo.shape[0] % 2 == 1
    with pytest.raises(ValueError):
        split_kernel(k, 3, 2)


def test_supersampled_convolution_models():
    g = W.grid_kwargs(20, 0.05)
    data = J.ImageData(np.zeros((20, 20)), exposure_time=100.0, background_rms=0.01, **g)
    ks = W.moffat_pixel_kernel(0.12, 3.0, 0.05 / 3, 27)
    lm, sm = J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"])
    psf = J.PSF("PIXEL", kernel_point_source=ks, point_source_supersampling_factor=3)
    im = J.ImageModel(data, psf, lm, sm, kwargs_numerics={"supersampling_factor": 3,
                                                          "supersampling_convolution": True,
                                                          "supersampling_kernel_size": 3})
    d = im._desc(range(2), range(1), [])
    assert d.supersampling_convolution == 1 and d.kernel_size == 9 and d.low_res_kernel_size == 9
    assert im.pack_psf(ks).size == 81 + 81
    im2 = J.ImageModel(data, psf, lm, sm, kwargs_numerics={"supersampling_factor": 3,
                                                           "supersampling_convolution": True,
                                                           "supersampling_kernel_size": None})
    d2 = im2._desc(range(2), range(1), [])
    assert d2.kernel_size == 27 and d2.low_res_kernel_size == 0
    # an even factor cannot split; a pixel-scale PSF cannot be supersampled here
    psf2 = J.PSF("PIXEL", kernel_point_source=ks[1:-1, 1:-1][:25, :25],
                 point_source_supersampling_factor=2)
    with pytest.raises(ValueError):
        J.ImageModel(data, psf2, lm, sm, kwargs_numerics={"supersampling_factor": 2,
                                                          "supersampling_convolution": True})
    with pytest.raises(NotImplementedError):
        J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=ks), lm, sm,
                     kwargs_numerics={"supersampling_factor": 3,
                                      "supersampling_convolution": True})


def test_flux_evaluate_indexes_subframe():
    g = W.grid_kwargs(20, 0.05)
    data = J.ImageData(np.zeros((20, 20)), exposure_time=100.0, background_rms=0.01, **g)
    psf = J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, 0.05, 5))
    mask = np.zeros((20, 20), bool)
    mask[3:9, 10:16] = True
    mask[3, 10] = False
    im = J.ImageModel(data, psf, J.LensModel(["SIE"]), J.LightModel(["SERSIC"]),
                      kwargs_numerics={"flux_evaluate_indexes": mask})
    r0, c0, cut = im._subframe
    assert (r0, c0) == (3, 10) and cut.shape == (6, 6) and not cut[0, 0] and cut.sum() == 35
    bad = np.zeros((20, 20), bool)
    bad[2:5, 4:12] = True
    with pytest.raises(ValueError):
        J.ImageModel(data, psf, J.LensModel(["SIE"]), J.LightModel(["SERSIC"]),
                     kwargs_numerics={"flux_evaluate_indexes": bad})


@pytest.mark.parametrize("case", golden_io.multi_plane_cases(), ids=lambda c: c["tag"])
def test_multi_plane_prepare_matches_reference(case):
    """LensModelBulk(multi_plane=True).prepare_ray_shooting_kwargs against the
    reference's own output (multi_plane_bulk.py:57-150): redshift sort, NULL source
    and filler steps, zero-filled arrays; distance lists from FlatLambdaCDM(70, 0.3)
    against the goldens' independent quadrature."""
    b = J.LensModelBulk(case["unique"], multi_plane=True, cosmo=J.FlatLambdaCDM(70.0, 0.3))
    rk = b.prepare_ray_shooting_kwargs(case["lens_list"], case["kwargs"],
                                       z_source=case["z_source"], lens_redshift_list=case["z"],
                                       num_deflectors=case["num_deflectors"])
    ref = case["prep"]
    np.testing.assert_array_equal(rk["index_list"], ref["index_list"])
    assert set(rk["all_kwargs"]) == set(ref["all_kwargs"])
    for k, v in ref["all_kwargs"].items():
        np.testing.assert_array_equal(rk["all_kwargs"][k], v)
    for k in ("T_ij_list", "T_z_list", "reduced2physical_factor"):
        np.testing.assert_allclose(rk[k], ref[k], rtol=1e-12, atol=0)


def test_multi_plane_errors_mirror_reference():
    b = J.LensModelBulk(["TNFW"], multi_plane=True, cosmo=J.FlatLambdaCDM())
    kw = [{"Rs": 0.1, "alpha_Rs": 0.01, "r_trunc": 1.0}]
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW"], kw, z_source=2.0)
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW"], kw, lens_redshift_list=[0.5])
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW"], kw, z_source=2.0, lens_redshift_list=[0.5, 0.6])
    with pytest.raises(ValueError):
        b.prepare_ray_shooting_kwargs(["TNFW", "TNFW"], kw * 2, z_source=2.0,
                                      lens_redshift_list=[0.5, 0.6], num_deflectors=1)
    try:
        import astropy  # noqa: F401
    except ImportError:
        with pytest.raises(ValueError):
            J.LensModelBulk(["TNFW"], multi_plane=True)


def test_flat_lcdm_distances():
    """FlatLambdaCDM against closed forms: Einstein-de Sitter (Om0 = 1),
    D_C = 2 (c/H0) (1 - 1/sqrt(1+z)); de Sitter (Om0 = 0), D_C = (c/H0) z; and
    additivity of comoving distance (flat: T_xy(z1, z3) = T_xy(z1, z2) + T_xy(z2, z3))."""
    from jaxtronomy_gb300 import cosmology
    dh = cosmology.C_KM_S / 70.0
    for z in (0.1, 0.5, 2.5, 6.0):
        eds = J.FlatLambdaCDM(70.0, 1.0).comoving_distance(z)
        assert abs(eds - 2 * dh * (1 - 1 / np.sqrt(1 + z))) <= 1e-13 * eds
        ds = J.FlatLambdaCDM(70.0, 0.0).comoving_distance(z)
        assert abs(ds - dh * z) <= 1e-13 * ds
    bg = cosmology.Background(J.FlatLambdaCDM(67.0, 0.31))
    t13, t12, t23 = bg.T_xy(0.2, 2.4), bg.T_xy(0.2, 0.9), bg.T_xy(0.9, 2.4)
    assert abs(t13 - (t12 + t23)) <= 1e-12 * t13
    d = bg.d_xy(np.array([0.1, 0.5]), np.array([1.0, 1.0]))
    assert d.shape == (2,) and abs(d[1] - bg.d_xy(0.5, 1.0)) == 0


def test_point_source_rows_layout():
    """PointSource.point_source_list order (models concatenated), the astrometric
    shift of the first images (image_model.py:652-676) and batch broadcasting."""
    g = W.grid_kwargs(20, 0.1)
    data = J.ImageData(np.zeros((20, 20)), exposure_time=100.0, background_rms=0.01, **g)
    psf = J.PSF("PIXEL", kernel_point_source=W.gaussian_pixel_kernel(0.1, 0.1, 5))
    im = J.ImageModel(data, psf, J.LensModel(["SIE"]), J.LightModel(["SERSIC"]),
                      J.LightModel([]),
                      point_source_class=J.PointSource(["LENSED_POSITION", "UNLENSED"],
                                                       flux_from_point_source_list=[True, False]))
    ps = [{"ra_image": [0.1, 0.2], "dec_image": [0.3, 0.4], "point_amp": [1.0, 2.0]},
          {"ra_image": [0.5], "dec_image": [0.6], "point_amp": [3.0]}]
    rows = im.point_source_rows(ps, {"delta_x_image": [0.01], "delta_y_image": [0.02]}, B=3)
    assert rows.shape == (3, 3, 3)
    np.testing.assert_allclose(rows[0, :, 0], [0.11, 0.2, 0.5])
    np.testing.assert_allclose(rows[0, :, 1], [0.32, 0.4, 0.6])
    np.testing.assert_allclose(rows[2, :, 2], [1.0, 2.0, 0.0])  # flux_from_point_source False
    assert im.PointSource.num_basis(ps) == 2
    with pytest.raises(ValueError):
        im.point_source_rows([ps[0]])
