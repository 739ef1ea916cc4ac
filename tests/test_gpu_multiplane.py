"""MultiPlaneBulk on the GPU (lensgb_bulk_multi_plane_ray_shooting through the
C ABI) against the reference golden vectors and the FP64 oracle.

Tolerances:
  * FP64: 1e-10 relative per ray on beta (absolute floor 1e-12 of max |beta|).
  * FP32 (FP32-pair ray state, subhalo terms in FP32): |beta_fp32 - beta_fp64|
    <= 2e-7 arcsec per ray.
"""

import warnings

import numpy as np
import pytest
import torch

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W
from oracle import lens as olens

warnings.filterwarnings("ignore", category=RuntimeWarning)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_BETA_ATOL = 2e-7
COSMO = J.FlatLambdaCDM(70.0, 0.3)


def assert_beta_close(got, ref, rtol=FP64_RTOL):
    got = np.asarray(got, float)
    ref = np.asarray(ref, float)
    np.testing.assert_allclose(got, ref, rtol=rtol, atol=1e-12 * np.abs(ref).max())


def _bulk(unique, precision="fp64"):
    return J.LensModelBulk(unique, multi_plane=True, cosmo=COSMO, precision=precision)


@pytest.mark.parametrize("case", golden_io.multi_plane_cases(), ids=lambda c: c["tag"])
def test_multi_plane_fp64_matches_reference(cuda, case):
    """The reference's own prepared kwargs through the GPU ray shooting, and the
    whole call (this library's prepare with FlatLambdaCDM) against the reference's beta."""
    b = _bulk(case["unique"])
    bx, by = b.ray_shooting(case["x"], case["y"], case["prep"])
    assert_beta_close(bx, case["bx"])
    assert_beta_close(by, case["by"])
    rk = b.prepare_ray_shooting_kwargs(case["lens_list"], case["kwargs"],
                                       z_source=case["z_source"], lens_redshift_list=case["z"],
                                       num_deflectors=case["num_deflectors"])
    bx, by = b.ray_shooting(case["x"], case["y"], rk)
    assert_beta_close(bx, case["bx"])
    assert_beta_close(by, case["by"])


@pytest.mark.parametrize("case", golden_io.multi_plane_cases(), ids=lambda c: c["tag"])
def test_multi_plane_fp32_golden_cases(cuda, case):
    b = _bulk(case["unique"], "fp32")
    bx, by = b.ray_shooting(case["x"], case["y"], case["prep"])
    assert np.abs(bx - case["bx"]).max() <= FP32_BETA_ATOL
    assert np.abs(by - case["by"]).max() <= FP32_BETA_ATOL


def _halos(n_pix=100, n_halos=800, n_planes=40):
    x, y, ll, kw, z, zs, nd = W.line_of_sight_halos(seed=1006, num_pix=n_pix, n_halos=n_halos,
                                                    n_planes=n_planes, half_width=4.0,
                                                    num_deflectors=n_halos + n_planes + 11)
    return x, y, ll, kw, z, zs, nd


def test_multi_plane_line_of_sight_halos_fp64_vs_oracle_and_fp32(cuda):
    """The benchmark's kind of realisation at 10^4 rays x 851 steps: FP64 against
    the oracle, FP32 against FP64 (including the few halos above fp32_alpha_max
    that run in FP64, and 40 CONVERGENCE sheets)."""
    x, y, ll, kw, z, zs, nd = _halos()
    unique = ["TNFW", "CONVERGENCE"]
    b64 = _bulk(unique)
    rk = b64.prepare_ray_shooting_kwargs(ll, kw, z_source=zs, lens_redshift_list=z,
                                         num_deflectors=nd)
    bx, by = b64.ray_shooting(x, y, rk)
    ox, oy = olens.multi_plane_ray_shooting(unique, x, y, rk["all_kwargs"], rk["index_list"],
                                            rk["T_ij_list"], rk["T_z_list"],
                                            rk["reduced2physical_factor"])
    assert_beta_close(bx, ox)
    assert_beta_close(by, oy)
    fx, fy = _bulk(unique, "fp32").ray_shooting(x, y, rk)
    assert np.abs(fx - bx).max() <= FP32_BETA_ATOL
    assert np.abs(fy - by).max() <= FP32_BETA_ATOL
    # deflections are resolved: beta differs from theta far above the tolerance
    assert np.abs(bx - x).max() > 1e3 * FP32_BETA_ATOL


def test_multi_plane_main_lens_fp32_runs_strong_terms_in_fp64(cuda):
    """EPL + SHEAR on the main plane (tagged FP64 in FP32 mode), halos in front of
    and behind it, rays through the Einstein ring."""
    case = [c for c in golden_io.multi_plane_cases() if c["tag"] == "main_lens"][0]
    rng = np.random.default_rng(11)
    x = rng.uniform(-2, 2, 5003)
    y = rng.uniform(-2, 2, 5003)
    b64, b32 = _bulk(case["unique"]), _bulk(case["unique"], "fp32")
    bx, by = b64.ray_shooting(x, y, case["prep"])
    ox, oy = olens.multi_plane_ray_shooting(case["unique"], x, y, case["prep"]["all_kwargs"],
                                            case["prep"]["index_list"],
                                            case["prep"]["T_ij_list"], case["prep"]["T_z_list"],
                                            case["prep"]["reduced2physical_factor"])
    assert_beta_close(bx, ox)
    assert_beta_close(by, oy)
    fx, fy = b32.ray_shooting(x, y, case["prep"])
    assert np.abs(fx - bx).max() <= FP32_BETA_ATOL
    assert np.abs(fy - by).max() <= FP32_BETA_ATOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_multi_plane_edge_cases(cuda, precision):
    """No deflector (the source step only: beta = theta), NULL fillers only, all
    deflectors on one plane, torch inputs, and ray counts off the CTA size."""
    b = _bulk(["TNFW", "CONVERGENCE"], precision)
    x = np.linspace(-1, 1, 129)
    y = np.linspace(1, -1, 129)
    rk = b.prepare_ray_shooting_kwargs([], [], z_source=1.5, lens_redshift_list=[],
                                       num_deflectors=5)
    assert len(rk["index_list"]) == 6
    bx, by = b.ray_shooting(x, y, rk)
    np.testing.assert_allclose(bx, x, rtol=1e-15, atol=1e-15)
    np.testing.assert_allclose(by, y, rtol=1e-15, atol=1e-15)
    # every deflector at one redshift: oracle agreement
    kw = [{"Rs": 0.1, "alpha_Rs": 0.01, "r_trunc": 1.0, "center_x": 0.2, "center_y": -0.1},
          {"kappa": -0.004}, {"Rs": 0.05, "alpha_Rs": 0.003, "r_trunc": 0.4,
                              "center_x": -0.3, "center_y": 0.3}]
    ll = ["TNFW", "CONVERGENCE", "TNFW"]
    rk = b.prepare_ray_shooting_kwargs(ll, kw, z_source=1.5, lens_redshift_list=[0.6] * 3)
    xt = torch.tensor(x, device="cuda")
    yt = torch.tensor(y, device="cuda")
    bx, by = b.ray_shooting(xt, yt, rk)
    assert isinstance(bx, torch.Tensor) and bx.device.type == "cuda"
    ox, oy = olens.multi_plane_ray_shooting(["TNFW", "CONVERGENCE"], x, y, rk["all_kwargs"],
                                            rk["index_list"], rk["T_ij_list"], rk["T_z_list"],
                                            rk["reduced2physical_factor"])
    tol = FP64_RTOL if precision == "fp64" else None
    if tol:
        assert_beta_close(bx.cpu().numpy(), ox)
        assert_beta_close(by.cpu().numpy(), oy)
    else:
        assert np.abs(bx.cpu().numpy() - ox).max() <= FP32_BETA_ATOL
        assert np.abs(by.cpu().numpy() - oy).max() <= FP32_BETA_ATOL
    ex, ey = b.ray_shooting(np.zeros(0), np.zeros(0), rk)
    assert ex.shape == (0,) and ey.shape == (0,)


def test_multi_plane_abi_rejects_bad_arguments(cuda):
    from jaxtronomy_gb300 import _lib
    b = _bulk(["TNFW"])
    rk = b.prepare_ray_shooting_kwargs([], [], z_source=1.0, lens_redshift_list=[])
    with pytest.raises(ValueError):
        b.ray_shooting(np.zeros(3), np.zeros(3), dict(rk, T_z_list=np.ones(3)))
    h = b.lens_model._handle().handle
    d = torch.zeros(4, dtype=torch.float64, device="cuda")
    i = torch.zeros(1, dtype=torch.int32, device="cuda")
    p = d.data_ptr()
    rc = _lib.load().lensgb_bulk_multi_plane_ray_shooting(h, i.data_ptr(), p, 0, p, p, p, p, p,
                                                          p, p, 1, None)
    assert rc == 1


def test_multi_plane_benchmark_realisation_fp32_vs_fp64(cuda):
    """The benchmark's full workload (400^2 rays, 5130 TNFW + 126 CONVERGENCE on 126
    planes, 5501 steps): FP32 beta within 2e-7 arcsec of FP64 on every ray, and FP64
    within 1e-10 of the oracle on a ray sample."""
    x, y, ll, kw, z, zs, nd = W.line_of_sight_halos()
    unique = ["TNFW", "CONVERGENCE"]
    cosmo = J.FlatLambdaCDM(67.66, 0.30966)
    b64 = J.LensModelBulk(unique, multi_plane=True, cosmo=cosmo)
    b32 = J.LensModelBulk(unique, multi_plane=True, cosmo=cosmo, precision="fp32")
    rk = b64.prepare_ray_shooting_kwargs(ll, kw, z_source=zs, lens_redshift_list=z,
                                         num_deflectors=nd)
    xt = torch.as_tensor(x).cuda()
    yt = torch.as_tensor(y).cuda()
    bx, by = b64.ray_shooting(xt, yt, rk)
    fx, fy = b32.ray_shooting(xt, yt, rk)
    err = torch.maximum((fx - bx).abs(), (fy - by).abs())
    assert err.max().item() <= FP32_BETA_ATOL
    s = np.arange(0, x.size, x.size // 64)[:64]
    ox, oy = olens.multi_plane_ray_shooting(unique, x[s], y[s], rk["all_kwargs"], rk["index_list"],
                                            rk["T_ij_list"], rk["T_z_list"],
                                            rk["reduced2physical_factor"])
    assert_beta_close(bx.cpu().numpy()[s], ox)
    assert_beta_close(by.cpu().numpy()[s], oy)
