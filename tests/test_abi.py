"""C-ABI checks that need no GPU: the library loads, exports every entry point
declared in include/lensgb.h, and validates descriptors on the host."""

import ctypes
import os
import re

import numpy as np
import pytest

from jaxtronomy_gb300 import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "lensgb.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|long long|const char\*)\s+(lensgb_\w+)\s*\(",
                                 text, re.M)))


def test_header_lists_the_python_symbols():
    assert declared_functions() == sorted(_lib.SYMBOLS)


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert lib.lensgb_version() == 116


def _desc(**kw):
    d = _lib.ModelDesc()
    d.n_lens = 2
    d.lens_codes[0] = _lib.LENS_CODES["EPL"]
    d.lens_codes[1] = _lib.LENS_CODES["SHEAR"]
    d.n_source = 1
    d.source_codes[0] = _lib.LIGHT_CODES["SERSIC_ELLIPSE"]
    d.deflection_scaling[0] = 1.0
    d.n_lens_light = 1
    d.lens_light_codes[0] = _lib.LIGHT_CODES["SERSIC_ELLIPSE"]
    d.nx = d.ny = 32
    d.supersampling = 2
    d.transform_pix2angle[:] = [0.05, 0, 0, 0.05]
    d.ra_at_xy_0 = d.dec_at_xy_0 = -0.775
    d.flux_scaling = 1.0
    d.alpha_scaling = 1.0
    d.psf_type = _lib.PSF_PIXEL
    d.kernel_size = 11
    d.precision = _lib.FP32_SPLIT
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def _create(d):
    lib = _lib.load()
    h = ctypes.c_void_p()
    rc = lib.lensgb_model_create(ctypes.byref(d), ctypes.byref(h))
    return rc, h, lib.lensgb_last_error().decode()


def test_model_create_and_param_count():
    rc, h, _ = _create(_desc())
    assert rc == _lib.OK
    lib = _lib.load()
    assert lib.lensgb_model_param_count(h) == 6 + 4 + 7 + 7
    assert lib.lensgb_model_destroy(h) == _lib.OK


@pytest.mark.parametrize("kw,code,msg", [
    (dict(nx=0), _lib.ERR_INVALID, "grid"),
    (dict(supersampling=0), _lib.ERR_INVALID, "grid"),
    (dict(kernel_size=10), _lib.ERR_INVALID, "odd"),
    (dict(precision=7), _lib.ERR_UNSUPPORTED, "precision"),
    (dict(psf_type=9), _lib.ERR_UNSUPPORTED, "psf_type"),
    (dict(n_lens=9), _lib.ERR_INVALID, "profile count"),
])
def test_model_create_rejects_bad_descriptors(kw, code, msg):
    rc, h, err = _create(_desc(**kw))
    assert rc == code
    assert msg in err
    assert not h.value


def test_unknown_profile_code_is_rejected():
    d = _desc()
    d.lens_codes[0] = 99
    rc, _, err = _create(d)
    assert rc == _lib.ERR_UNSUPPORTED and "lens profile" in err


def test_null_arguments_are_rejected_without_a_gpu():
    lib = _lib.load()
    rc = lib.lensgb_image(None, None, 1, None, 0, None, 0, None)
    assert rc == _lib.ERR_INVALID
    rc, h, _ = _create(_desc())
    assert rc == _lib.OK
    # n_inst out of range and null pointers fail before any CUDA call
    assert lib.lensgb_image(h, None, -1, None, 0, None, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image(h, None, 70000, None, 0, None, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image(h, None, 2, None, 0, None, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image(h, None, 0, None, 0, None, 0, None) == _lib.OK
    assert lib.lensgb_ray_shooting(h, None, None, None, None, None, -5, None) == _lib.ERR_INVALID
    lib.lensgb_model_destroy(h)


def test_split_bits_is_exact_for_grid_indices():
    # host mirror of split_bits: hi has <= bits significant bits, so J*hi is exact
    # in FP32 for every supersampled index J < 2^(24-bits)
    step = 0.04 / 3
    bits = 24 - 10  # 540 rays per side < 2^10
    m, e = np.frexp(step)
    hi = np.ldexp(np.trunc(m * 2.0 ** bits) / 2.0 ** bits, e)
    hi32 = np.float32(hi)
    assert float(hi32) == hi
    J = np.arange(540, dtype=np.float32)
    assert np.all((J * hi32).astype(np.float64) == J.astype(np.float64) * hi)


def test_struct_sizes_match_the_header_layout():
    """ctypes mirrors of the public structs have the C layout (x86-64 / aarch64 LP64)."""
    assert ctypes.sizeof(_lib.NoiseDesc) == 11 * 8
    assert ctypes.sizeof(_lib.ServerConfig) == 4 + 4 + 8 + 4 + 4 + 4 + 4  # tail padding
    assert ctypes.sizeof(_lib.ServerStats) == 11 * 8
    assert ctypes.sizeof(_lib.Request) == ctypes.sizeof(_lib.ModelDesc) + 10 * 8


def test_bulk_and_server_handles_on_the_host():
    """Argument validation of the bulk and server entry points (no device work)."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    codes = (ctypes.c_int * 2)(_lib.LENS_CODES["TNFW"], 99)
    assert lib.lensgb_bulk_create(codes, 2, _lib.FP32_SPLIT, ctypes.byref(h)) == _lib.ERR_UNSUPPORTED
    assert b"99" in lib.lensgb_last_error()
    assert lib.lensgb_bulk_create(codes, 17, _lib.FP64, ctypes.byref(h)) == _lib.ERR_INVALID
    assert lib.lensgb_bulk_create(codes, 1, 7, ctypes.byref(h)) == _lib.ERR_UNSUPPORTED
    assert lib.lensgb_bulk_create(codes, 1, _lib.FP64, ctypes.byref(h)) == _lib.OK
    assert lib.lensgb_bulk_set_fp32_alpha_max(h, -1.0) == _lib.ERR_INVALID
    assert lib.lensgb_bulk_set_fp32_alpha_max(h, 0.1) == _lib.OK
    assert lib.lensgb_bulk_destroy(h) == _lib.OK
    cfg = _lib.ServerConfig(65, 0, 0, 0, 0)
    assert lib.lensgb_server_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.ERR_INVALID
    cfg = _lib.ServerConfig(4, 0, 0, 0, 0, 3)  # mixed_grids must be 0, 1 or 2
    assert lib.lensgb_server_create(ctypes.byref(cfg), ctypes.byref(h)) == _lib.ERR_INVALID


def test_tuning_arguments_are_validated_without_a_gpu():
    lib = _lib.load()
    assert ctypes.sizeof(_lib.TuneResult) == 2 * 4 + 4 * 8
    rc, h, _ = _create(_desc())
    assert rc == _lib.OK
    assert lib.lensgb_model_set_tuning(h, 3, 0) == _lib.ERR_INVALID
    assert lib.lensgb_model_set_tuning(h, 2, 30) == _lib.ERR_INVALID
    assert lib.lensgb_model_set_tuning(h, 2, 66) == _lib.ERR_INVALID
    assert lib.lensgb_model_set_tuning(h, 4, 60) == _lib.OK
    assert lib.lensgb_model_set_tuning(h, 0, 0) == _lib.OK
    res = _lib.TuneResult()
    assert lib.lensgb_model_autotune(h, None, 0, None, 0, None, None,
                                     ctypes.byref(res)) == _lib.ERR_INVALID
    assert lib.lensgb_model_autotune(h, None, 4, None, 0, None, None, None) == _lib.ERR_INVALID
    lib.lensgb_model_destroy(h)


def test_host_call_arguments_are_validated_without_a_gpu():
    lib = _lib.load()
    rc, h, _ = _create(_desc())
    assert rc == _lib.OK
    assert lib.lensgb_image_host(None, None, 1, None, 0, None, 0, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image_host(h, None, -1, None, 0, None, 0, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image_host(h, None, 2, None, 0, None, 0, 0, None) == _lib.ERR_INVALID
    assert lib.lensgb_image_host(h, None, 0, None, 0, None, 0, 0, None) == _lib.OK
    lib.lensgb_model_destroy(h)


def test_model_options_are_validated_without_a_gpu():
    """The adjoint-precision and convolution-method setters accept their
    documented values and refuse others with LENSGB_ERR_INVALID."""
    lib = _lib.load()
    rc, h, _ = _create(_desc(precision=_lib.FP64))
    assert rc == _lib.OK
    assert lib.lensgb_model_set_grad_precision(h, _lib.FP64) == _lib.OK
    assert lib.lensgb_model_set_grad_precision(h, _lib.FP32_SPLIT) == _lib.OK
    assert lib.lensgb_model_set_grad_precision(h, 7) == _lib.ERR_INVALID
    assert "precision" in lib.lensgb_last_error().decode()
    assert lib.lensgb_model_set_grad_precision(None, _lib.FP64) == _lib.ERR_INVALID
    for m in _lib.CONV_METHODS.values():
        assert lib.lensgb_model_set_convolution(h, m) == _lib.OK
    assert lib.lensgb_model_set_convolution(h, 99) == _lib.ERR_INVALID
    lib.lensgb_model_destroy(h)
