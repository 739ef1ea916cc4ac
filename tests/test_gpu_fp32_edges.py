"""FP32-split images at the edges of the parameter space, against the FP64 path
(which matches the reference to 1e-10): very elliptical EPL (the 500-term
series, shortened in FP32), a round EPL (f = 0, no series), EPL at its slope
limits, SIE and NFW_ELLIPSE_CSE nearly round and very elliptical, small and
large CSE scale radii, strong multipoles, and a lens centre on a ray.

Bar: the FP32 bar of the other tests, 1e-5 relative per pixel on pixels above
1e-3 of the image maximum and 1e-5 of the maximum everywhere.
"""

import numpy as np
import pytest

import jaxtronomy_gb300 as J
from jaxtronomy_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SRC = [{"amp": 50.0, "R_sersic": 0.3, "n_sersic": 2.5, "e1": 0.05, "e2": -0.08,
        "center_x": 0.04, "center_y": 0.02}]
LL = [{"amp": 30.0, "R_sersic": 0.9, "n_sersic": 3.5, "e1": 0.06, "e2": 0.03,
       "center_x": 0.0, "center_y": 0.0}]
SHEAR = {"gamma1": 0.02, "gamma2": -0.03}

CASES = [
    ("EPL", {"theta_E": 1.1, "gamma": 2.0, "e1": 0.95 * np.cos(0.3), "e2": 0.95 * np.sin(0.3),
             "center_x": 0.0, "center_y": 0.0}),
    ("EPL", {"theta_E": 1.1, "gamma": 2.05, "e1": 0.0, "e2": 0.0, "center_x": 0.0,
             "center_y": 0.0}),
    ("EPL", {"theta_E": 0.8, "gamma": 1.55, "e1": 0.3, "e2": -0.2, "center_x": 0.02,
             "center_y": 0.0}),
    ("EPL", {"theta_E": 1.4, "gamma": 2.45, "e1": -0.25, "e2": 0.1, "center_x": 0.0,
             "center_y": 0.01}),
    ("EPL", {"theta_E": 1.0, "gamma": 2.0, "e1": 0.1, "e2": 0.05, "center_x": 0.02,
             "center_y": 0.02}),  # the centre sits on a pixel-centre ray (0.04"/pix grid)
    ("SIE", {"theta_E": 1.0, "e1": 1e-6, "e2": 0.0, "center_x": 0.0, "center_y": 0.0}),
    ("SIE", {"theta_E": 1.2, "e1": 0.6, "e2": -0.5, "center_x": 0.0, "center_y": 0.0}),
    ("NFW_ELLIPSE_CSE", {"Rs": 0.3, "alpha_Rs": 0.4, "e1": 0.01, "e2": 0.0, "center_x": 0.0,
                         "center_y": 0.0}),
    ("NFW_ELLIPSE_CSE", {"Rs": 30.0, "alpha_Rs": 2.5, "e1": 0.4, "e2": 0.3, "center_x": 0.0,
                         "center_y": 0.0}),
    ("EPL_MULTIPOLE_M1M3M4", {"theta_E": 1.1, "gamma": 2.0, "e1": 0.1, "e2": -0.1,
                              "center_x": 0.0, "center_y": 0.0, "a1_a": 0.05,
                              "delta_phi_m1": 0.9, "a3_a": 0.04, "delta_phi_m3": 2.5,
                              "a4_a": -0.05, "delta_phi_m4": 0.1}),
]


def _model(lens, precision):
    g = W.grid_kwargs(100, 0.04)
    data = J.ImageData(np.zeros((100, 100)), exposure_time=1000.0, background_rms=0.01, **g)
    return J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=W.moffat_pixel_kernel(
                            0.12, 3.0, 0.04, 21)),
                        J.LensModel([lens, "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                        J.LightModel(["SERSIC_ELLIPSE"]),
                        kwargs_numerics={"supersampling_factor": 3, "precision": precision})


@pytest.mark.parametrize("lens,kw", CASES, ids=["%s-%d" % (c[0], i) for i, c in enumerate(CASES)])
def test_fp32_split_matches_fp64_at_parameter_edges(cuda, lens, kw):
    kl = [kw, SHEAR]
    a = _model(lens, "fp64").image(kl, SRC, LL)
    b = _model(lens, "fp32").image(kl, SRC, LL)
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    scale = np.abs(a).max()
    sig = np.abs(a) >= 1e-3 * scale
    per = (np.abs(b - a)[sig] / np.abs(a)[sig]).max()
    mx = np.abs(b - a).max() / scale
    assert per < 1e-5 and mx < 1e-5, (per, mx)
