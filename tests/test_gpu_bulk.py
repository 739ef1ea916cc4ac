"""LensModelBulk on the GPU (lensgb_bulk_ray_shooting through the C ABI)
against the reference golden vectors and the FP64 oracle.

Tolerances:
  * FP64: 1e-10 relative per ray on beta (absolute floor 1e-12 of max |beta|).
  * FP32 (subhalo terms in FP32, FP64 accumulation): |beta_fp32 - beta_fp64|
    <= 2e-7 arcsec per ray, and the source surface brightness at beta within
    1e-5 relative on pixels above 1e-3 of the maximum.
"""

import warnings

import numpy as np
import pytest
import torch

import golden_io
import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W
from oracle import lens as olens
from oracle import light as olight

warnings.filterwarnings("ignore", category=RuntimeWarning)

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
FP32_BETA_ATOL = 2e-7


def assert_beta_close(got, ref, rtol=FP64_RTOL):
    got = np.asarray(got, float)
    ref = np.asarray(ref, float)
    atol = 1e-12 * np.abs(ref).max()
    np.testing.assert_allclose(got, ref, rtol=rtol, atol=atol)


@pytest.mark.parametrize("case", golden_io.bulk_cases(), ids=lambda c: "+".join(c["unique"]))
def test_bulk_fp64_matches_reference(cuda, case):
    b = J.LensModelBulk(case["unique"], multi_plane=False)
    rk = b.prepare_ray_shooting_kwargs(case["lens_list"], case["kwargs"],
                                       num_deflectors=case["num_deflectors"])
    bx, by = b.ray_shooting(case["x"], case["y"], rk)
    assert_beta_close(bx, case["bx"])
    assert_beta_close(by, case["by"])


def _substructure(num_pix=64, n_sub=300, seed=1004):
    x, y, ll, kw, src = W.substructure(seed=seed, num_pix=num_pix, n_sub=n_sub)
    # spread the small grid over the subhalo box so that rays meet subhalo cores
    return x * (5.0 / (num_pix * 0.01)), y * (5.0 / (num_pix * 0.01)), ll, kw, src


def test_bulk_fp64_matches_oracle_substructure(cuda):
    x, y, ll, kw, _ = _substructure()
    unique = ["EPL", "SHEAR", "TNFW"]
    b = J.LensModelBulk(unique)
    rk = b.prepare_ray_shooting_kwargs(ll, kw, num_deflectors=len(ll) + 7)
    bx, by = b.ray_shooting(x, y, rk)
    ox, oy = olens.bulk_ray_shooting(unique, x, y, rk["all_kwargs"], rk["index_list"])
    assert_beta_close(bx, ox)
    assert_beta_close(by, oy)


def test_bulk_fp32_deflection_and_image_error(cuda):
    x, y, ll, kw, src = _substructure(num_pix=96, n_sub=600)
    unique = ["EPL", "SHEAR", "TNFW"]
    b64 = J.LensModelBulk(unique, precision="fp64")
    b32 = J.LensModelBulk(unique, precision="fp32")
    rk = b64.prepare_ray_shooting_kwargs(ll, kw)
    x64, y64 = b64.ray_shooting(x, y, rk)
    x32, y32 = b32.ray_shooting(x, y, rk)
    err = np.maximum(np.abs(x32 - x64), np.abs(y32 - y64))
    assert err.max() <= FP32_BETA_ATOL, err.max()
    # the FP32 path really ran: not bit-identical to FP64
    assert err.max() > 0
    s64 = olight.surface_brightness(["SERSIC_ELLIPSE"], x64, y64, src)
    s32 = olight.surface_brightness(["SERSIC_ELLIPSE"], x32, y32, src)
    sig = np.abs(s64) >= 1e-3 * np.abs(s64).max()
    rel = np.abs(s32 - s64)[sig] / np.abs(s64)[sig]
    assert rel.max() <= 1e-5, rel.max()


def test_bulk_fp32_strong_deflectors_run_in_fp64(cuda):
    """With every deflection bound above fp32_alpha_max the FP32 handle
    evaluates everything in FP64 and agrees with the FP64 handle to rounding."""
    x, y, ll, kw, _ = _substructure(num_pix=32, n_sub=40)
    unique = ["EPL", "SHEAR", "TNFW"]
    b64 = J.LensModelBulk(unique)
    b32 = J.LensModelBulk(unique, precision="fp32", fp32_alpha_max=0.0)
    rk = b64.prepare_ray_shooting_kwargs(ll, kw)
    x64, y64 = b64.ray_shooting(x, y, rk)
    x32, y32 = b32.ray_shooting(x, y, rk)
    assert_beta_close(x32, x64, rtol=1e-14)
    assert_beta_close(y32, y64, rtol=1e-14)


def test_bulk_index_clamping_and_null(cuda):
    """Out-of-range indices clamp like lax.switch; NULL deflects nothing."""
    rng = np.random.default_rng(3)
    x, y = rng.uniform(-2, 2, 200), rng.uniform(-2, 2, 200)
    unique = ["TNFW", "SIE", "NULL"]
    b = J.LensModelBulk(unique)
    kw = [{"Rs": 0.1, "alpha_Rs": 0.01, "r_trunc": 1.0, "center_x": 0.3, "center_y": -0.2},
          {"theta_E": 1.0, "e1": 0.05, "e2": 0.02, "center_x": 0.0, "center_y": 0.0}]
    rk = b.prepare_ray_shooting_kwargs(["TNFW", "SIE"], kw, num_deflectors=4)
    rk["index_list"] = np.array([-5, 1, 2, 17])  # -> TNFW, SIE, NULL, filler NULL
    bx, by = b.ray_shooting(x, y, rk)
    ox, oy = olens.bulk_ray_shooting(unique, x, y, rk["all_kwargs"], rk["index_list"])
    assert_beta_close(bx, ox)
    assert_beta_close(by, oy)
    sx, sy = olens.ray_shooting(["TNFW", "SIE"], x, y, kw)
    assert_beta_close(bx, sx)


def test_bulk_no_deflectors_is_identity(cuda):
    x = np.linspace(-1, 1, 33)
    y = np.linspace(2, -2, 33)
    b = J.LensModelBulk(["TNFW"])
    rk = b.prepare_ray_shooting_kwargs([], [])
    bx, by = b.ray_shooting(x, y, rk)
    np.testing.assert_array_equal(bx, x)
    np.testing.assert_array_equal(by, y)


def test_bulk_device_kwargs_match_host_kwargs(cuda):
    x, y, ll, kw, _ = _substructure(num_pix=40, n_sub=50)
    unique = ["EPL", "SHEAR", "TNFW"]
    b = J.LensModelBulk(unique, precision="fp32")
    rk = b.prepare_ray_shooting_kwargs(ll, kw)
    bx, by = b.ray_shooting(x, y, rk)
    rk_dev = {"all_kwargs": {k: torch.as_tensor(v).cuda() for k, v in rk["all_kwargs"].items()},
              "index_list": torch.as_tensor(rk["index_list"]).cuda()}
    tx, ty = b.ray_shooting(torch.as_tensor(x).cuda(), torch.as_tensor(y).cuda(), rk_dev)
    assert isinstance(tx, torch.Tensor) and tx.is_cuda
    np.testing.assert_array_equal(tx.cpu().numpy(), bx)
    np.testing.assert_array_equal(ty.cpu().numpy(), by)


def test_bulk_matches_lens_model_for_short_lists(cuda):
    """Bulk and the per-model LensModel path agree on the same profile list."""
    rng = np.random.default_rng(5)
    x, y = rng.uniform(-2, 2, 500), rng.uniform(-2, 2, 500)
    ll = ["EPL", "SHEAR", "NFW_ELLIPSE_CSE", "TNFW"]
    kw = [{"theta_E": 1.1, "gamma": 2.1, "e1": 0.05, "e2": -0.1, "center_x": 0.0,
           "center_y": 0.1},
          {"gamma1": 0.02, "gamma2": 0.01, "ra_0": 0.0, "dec_0": 0.0},
          {"Rs": 8.0, "alpha_Rs": 0.9, "e1": 0.1, "e2": 0.0, "center_x": 0.0, "center_y": 0.0},
          {"Rs": 0.05, "alpha_Rs": 0.004, "r_trunc": 0.5, "center_x": 0.5, "center_y": 0.5}]
    b = J.LensModelBulk(ll)
    bx, by = b.ray_shooting(x, y, b.prepare_ray_shooting_kwargs(ll, kw))
    lx, ly = J.LensModel(ll).ray_shooting(x, y, kw)
    assert_beta_close(bx, lx, rtol=1e-13)
    assert_beta_close(by, ly, rtol=1e-13)


@pytest.mark.parametrize("tau", [0.1, 0.5, 3.0, 10.0, 40.0, 200.0])
def test_bulk_fp32_tnfw_near_and_far_field(cuda, tau):
    """FP32 subhalo deflections against FP64 from the core through the switch to
    the bracket polynomial (x = max(tau, 1)) and far beyond: |d alpha| <= 2e-6
    of max(|alpha|, alpha_Rs).  (Near the R = 0.001 Rs floor the reference
    formula, which the FP64 path follows, cancels to ~1e-5 relative; there alpha
    itself is below 1e-5 alpha_Rs.)"""
    Rs = 0.05
    s = max(tau, 1)
    xs = Rs * np.concatenate([np.geomspace(1e-4, 2.0, 40), np.geomspace(0.5, 4.0, 40) * s,
                              [s * (1 - 1e-6), s * (1 + 1e-6), 3 * s],
                              np.geomspace(5, 2000, 30), [1e5 * s]])
    ang = np.linspace(0, 2 * np.pi, xs.size)
    x, y = 0.3 + xs * np.cos(ang), -0.2 + xs * np.sin(ang)
    kw = [{"Rs": Rs, "alpha_Rs": 0.004, "r_trunc": tau * Rs, "center_x": 0.3, "center_y": -0.2}]
    b64 = J.LensModelBulk(["TNFW"])
    b32 = J.LensModelBulk(["TNFW"], precision="fp32")
    rk = b64.prepare_ray_shooting_kwargs(["TNFW"], kw)
    bx64, by64 = b64.ray_shooting(x, y, rk)
    bx32, by32 = b32.ray_shooting(x, y, rk)
    a64 = np.hypot(x - bx64, y - by64)
    err = np.hypot(bx32 - bx64, by32 - by64) / np.maximum(a64, 0.004)
    assert err.max() <= 2e-6, (err.max(), xs[np.argmax(err)] / Rs)
