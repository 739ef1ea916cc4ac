"""ctypes binding of liblensgb.so (the C ABI declared in include/lensgb.h).

The library is the only compute path: if it is missing this module raises,
and there is no CPU fallback.
"""

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblensgb.so")

MAX_PROFILES = 8

# status codes
OK = 0
ERR_INVALID = 1
ERR_UNSUPPORTED = 2
ERR_OOM = 3
ERR_CUDA = 4

# profile codes
LENS_NULL = 0
BULK_MAX_UNIQUE = 16
BULK_PARAM_STRIDE = 12
LENS_CODES = {"SIE": 1, "NIE": 2, "EPL": 3, "SHEAR": 4, "NFW": 5, "TNFW": 6,
              "NFW_ELLIPSE_CSE": 7, "EPL_MULTIPOLE_M1M3M4": 8, "CONVERGENCE": 9}
LIGHT_CODES = {"SERSIC": 1, "SERSIC_ELLIPSE": 2}

PSF_NONE, PSF_PIXEL, PSF_GAUSSIAN = 0, 1, 2
FP64, FP32_SPLIT = 0, 1

CONV_METHODS = {"auto": 0, "direct": 1, "fft": 2}

UNCONVOLVED = 1
NO_SOURCE = 2
NO_LENS_LIGHT = 4

# exported symbols (must match include/lensgb.h)
SYMBOLS = [
    "lensgb_model_create", "lensgb_model_destroy", "lensgb_model_param_count",
    "lensgb_model_reserve", "lensgb_model_set_refine", "lensgb_model_refined_pixels",
    "lensgb_model_set_tuning", "lensgb_model_autotune", "lensgb_image_host",
    "lensgb_image_host_wait", "lensgb_linear_solve",
    "lensgb_model_set_subframe",
    "lensgb_image", "lensgb_image_noalloc", "lensgb_image_mixed", "lensgb_convolve",
    "lensgb_loglike",
    "lensgb_loglike_grad",
    "lensgb_ray_shooting", "lensgb_alpha",
    "lensgb_surface_brightness",
    "lensgb_bulk_create", "lensgb_bulk_destroy", "lensgb_bulk_set_fp32_alpha_max",
    "lensgb_bulk_ray_shooting", "lensgb_bulk_multi_plane_ray_shooting",
    "lensgb_loglike_image", "lensgb_point_sources_add", "lensgb_hessian",
    "lensgb_server_create", "lensgb_server_submit", "lensgb_server_poll", "lensgb_server_wait",
    "lensgb_server_cancel",
    "lensgb_server_drain", "lensgb_server_clock_ns", "lensgb_server_request_times",
    "lensgb_server_get_stats", "lensgb_server_destroy",
    "lensgb_fma_chain", "lensgb_set_conv_tma", "lensgb_wait_timeouts",
    "lensgb_model_set_convolution", "lensgb_model_set_grad_precision",
    "lensgb_last_error", "lensgb_version",
]


class ModelDesc(ctypes.Structure):
    _fields_ = [
        ("n_lens", ctypes.c_int),
        ("lens_codes", ctypes.c_int * MAX_PROFILES),
        ("n_source", ctypes.c_int),
        ("source_codes", ctypes.c_int * MAX_PROFILES),
        ("deflection_scaling", ctypes.c_double * MAX_PROFILES),
        ("n_lens_light", ctypes.c_int),
        ("lens_light_codes", ctypes.c_int * MAX_PROFILES),
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("supersampling", ctypes.c_int),
        ("transform_pix2angle", ctypes.c_double * 4),
        ("ra_at_xy_0", ctypes.c_double),
        ("dec_at_xy_0", ctypes.c_double),
        ("flux_scaling", ctypes.c_double),
        ("alpha_scaling", ctypes.c_double),
        ("psf_type", ctypes.c_int),
        ("kernel_size", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("supersampling_convolution", ctypes.c_int),
        ("low_res_kernel_size", ctypes.c_int),
    ]


class NoiseDesc(ctypes.Structure):
    _fields_ = [
        ("data_dev", ctypes.c_void_p),
        ("data_stride", ctypes.c_longlong),
        ("mask_dev", ctypes.c_void_p),
        ("noise_map_dev", ctypes.c_void_p),
        ("noise_stride", ctypes.c_longlong),
        ("exposure_map_dev", ctypes.c_void_p),
        ("exposure_stride", ctypes.c_longlong),
        ("exposure_time", ctypes.c_double),
        ("background_rms", ctypes.c_double),
        ("error_map_dev", ctypes.c_void_p),
        ("mask_stride", ctypes.c_longlong),
    ]


class TuneResult(ctypes.Structure):
    _fields_ = [
        ("ppt", ctypes.c_int),
        ("conv_tile_rows", ctypes.c_int),
        ("ray_ms", ctypes.c_double),
        ("conv_ms", ctypes.c_double),
        ("ray_ms_builtin", ctypes.c_double),
        ("conv_ms_builtin", ctypes.c_double),
    ]


class SystemGrid(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int),
        ("ny", ctypes.c_int),
        ("transform_pix2angle", ctypes.c_double * 4),
        ("ra_at_xy_0", ctypes.c_double),
        ("dec_at_xy_0", ctypes.c_double),
        ("kernel_size", ctypes.c_int),
        ("supersampling", ctypes.c_int),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("n_streams", ctypes.c_int),
        ("max_batch", ctypes.c_int),
        ("hbm_budget_bytes", ctypes.c_longlong),
        ("contexts_per_bucket", ctypes.c_int),
        ("use_graphs", ctypes.c_int),
        ("mixed_grids", ctypes.c_int),
    ]


class Request(ctypes.Structure):
    _fields_ = [
        ("desc", ModelDesc),
        ("params", ctypes.c_void_p),
        ("psf", ctypes.c_void_p),
        ("image_out", ctypes.c_void_p),
        ("data", ctypes.c_void_p),
        ("noise_map", ctypes.c_void_p),
        ("mask", ctypes.c_void_p),
        ("background_rms", ctypes.c_double),
        ("exposure_time", ctypes.c_double),
        ("logl_out", ctypes.c_void_p),
        ("release_ns", ctypes.c_longlong),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_longlong) for n in (
        "batches", "requests_launched", "requests_done", "graph_captures", "graph_launches",
        "evictions", "bytes_held", "peak_bytes", "host_launch_ns", "capture_ns",
        "mixed_batches")]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_FAILED, REQ_CANCELLED = 0, 1, 2, 3, 4

LINEAR_MAX, LINEAR_INVERSE, LINEAR_POSITIVE = 8, 1, 2


class LensgbError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("liblensgb error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load():
    """Load liblensgb.so once; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            "liblensgb.so is not built (%s); run `python -m jaxtronomy_gb300.build`" % LIB_PATH)
    lib = ctypes.CDLL(LIB_PATH)
    vp, dp, i, ll = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong
    lib.lensgb_model_create.argtypes = [ctypes.POINTER(ModelDesc), ctypes.POINTER(vp)]
    lib.lensgb_model_create.restype = i
    lib.lensgb_model_destroy.argtypes = [vp]
    lib.lensgb_model_destroy.restype = i
    lib.lensgb_model_param_count.argtypes = [vp]
    lib.lensgb_model_param_count.restype = i
    lib.lensgb_model_set_subframe.argtypes = [vp, i, i, i, vp]
    lib.lensgb_model_set_subframe.restype = i
    lib.lensgb_model_reserve.argtypes = [vp, i]
    lib.lensgb_model_reserve.restype = i
    lib.lensgb_model_set_refine.argtypes = [vp, ctypes.c_double, ctypes.c_double]
    lib.lensgb_model_set_refine.restype = i
    lib.lensgb_model_refined_pixels.argtypes = [vp, vp, ctypes.POINTER(ll)]
    lib.lensgb_model_refined_pixels.restype = i
    lib.lensgb_image_host.argtypes = [vp, vp, i, vp, ll, vp, i, i, vp]
    lib.lensgb_image_host.restype = i
    lib.lensgb_linear_solve.argtypes = [vp, vp, i, i, ctypes.POINTER(NoiseDesc), i, vp, vp, vp,
                                        vp, vp]
    lib.lensgb_linear_solve.restype = i
    lib.lensgb_image_host_wait.argtypes = [vp, vp]
    lib.lensgb_image_host_wait.restype = i
    lib.lensgb_model_set_tuning.argtypes = [vp, i, i]
    lib.lensgb_model_set_tuning.restype = i
    lib.lensgb_model_autotune.argtypes = [vp, dp, i, vp, ll, vp, vp, ctypes.POINTER(TuneResult)]
    lib.lensgb_model_autotune.restype = i
    lib.lensgb_image.argtypes = [vp, dp, i, vp, ll, vp, i, vp]
    lib.lensgb_image.restype = i
    lib.lensgb_image_mixed.argtypes = [vp, dp, i, ctypes.POINTER(SystemGrid), vp, vp, i, vp]
    lib.lensgb_image_mixed.restype = i
    lib.lensgb_image_noalloc.argtypes = [vp, dp, i, vp, ll, vp, i, vp]
    lib.lensgb_image_noalloc.restype = i
    lib.lensgb_convolve.argtypes = [vp, vp, i, vp, ll, vp, vp]
    lib.lensgb_convolve.restype = i
    lib.lensgb_loglike.argtypes = [vp, dp, i, vp, ll, ctypes.POINTER(NoiseDesc), vp, dp, vp]
    lib.lensgb_loglike.restype = i
    lib.lensgb_loglike_grad.argtypes = [vp, dp, i, vp, ll, ctypes.POINTER(NoiseDesc), vp, dp, dp,
                                        vp]
    lib.lensgb_loglike_grad.restype = i
    lib.lensgb_ray_shooting.argtypes = [vp, dp, dp, dp, dp, dp, ll, vp]
    lib.lensgb_ray_shooting.restype = i
    lib.lensgb_alpha.argtypes = [vp, dp, dp, dp, dp, dp, ll, vp]
    lib.lensgb_alpha.restype = i
    lib.lensgb_surface_brightness.argtypes = [vp, i, dp, dp, dp, dp, ll, vp]
    lib.lensgb_surface_brightness.restype = i
    lib.lensgb_bulk_create.argtypes = [ctypes.POINTER(ctypes.c_int), i, i, ctypes.POINTER(vp)]
    lib.lensgb_bulk_create.restype = i
    lib.lensgb_bulk_destroy.argtypes = [vp]
    lib.lensgb_bulk_destroy.restype = i
    lib.lensgb_bulk_set_fp32_alpha_max.argtypes = [vp, ctypes.c_double]
    lib.lensgb_bulk_set_fp32_alpha_max.restype = i
    lib.lensgb_bulk_ray_shooting.argtypes = [vp, vp, dp, i, dp, dp, dp, dp, ll, vp]
    lib.lensgb_bulk_ray_shooting.restype = i
    lib.lensgb_bulk_multi_plane_ray_shooting.argtypes = [vp, vp, dp, i, dp, dp, dp, dp, dp, dp,
                                                         dp, ll, vp]
    lib.lensgb_bulk_multi_plane_ray_shooting.restype = i
    lib.lensgb_loglike_image.argtypes = [vp, vp, i, ctypes.POINTER(NoiseDesc), dp, vp]
    lib.lensgb_loglike_image.restype = i
    lib.lensgb_point_sources_add.argtypes = [vp, dp, i, i, dp, i, ll, i, vp, vp]
    lib.lensgb_point_sources_add.restype = i
    lib.lensgb_fma_chain.argtypes = [i, i, i, vp, ctypes.POINTER(ll), vp]
    lib.lensgb_fma_chain.restype = i
    lib.lensgb_model_set_convolution.argtypes = [vp, i]
    lib.lensgb_model_set_convolution.restype = i
    lib.lensgb_model_set_grad_precision.argtypes = [vp, i]
    lib.lensgb_model_set_grad_precision.restype = i
    lib.lensgb_set_conv_tma.argtypes = [i]
    lib.lensgb_set_conv_tma.restype = i
    lib.lensgb_wait_timeouts.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    lib.lensgb_wait_timeouts.restype = i
    lib.lensgb_hessian.argtypes = [vp, dp, i, dp, dp, dp, ll, vp]
    lib.lensgb_hessian.restype = i
    lib.lensgb_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)]
    lib.lensgb_server_create.restype = i
    lib.lensgb_server_submit.argtypes = [vp, ctypes.POINTER(Request), i,
                                         ctypes.POINTER(ctypes.c_longlong)]
    lib.lensgb_server_submit.restype = i
    lib.lensgb_server_poll.argtypes = [vp, ll, ctypes.POINTER(i)]
    lib.lensgb_server_poll.restype = i
    lib.lensgb_server_wait.argtypes = [vp, ll, ctypes.c_double, ctypes.POINTER(i)]
    lib.lensgb_server_wait.restype = i
    lib.lensgb_server_cancel.argtypes = [vp, ll, ctypes.POINTER(i)]
    lib.lensgb_server_cancel.restype = i
    lib.lensgb_server_drain.argtypes = [vp, ctypes.c_double]
    lib.lensgb_server_drain.restype = i
    lib.lensgb_server_clock_ns.argtypes = [vp]
    lib.lensgb_server_clock_ns.restype = ll
    lib.lensgb_server_request_times.argtypes = [vp, ll, ctypes.POINTER(ll), ctypes.POINTER(ll),
                                                ctypes.POINTER(ll)]
    lib.lensgb_server_request_times.restype = i
    lib.lensgb_server_get_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    lib.lensgb_server_get_stats.restype = i
    lib.lensgb_server_destroy.argtypes = [vp]
    lib.lensgb_server_destroy.restype = i
    lib.lensgb_last_error.argtypes = []
    lib.lensgb_last_error.restype = ctypes.c_char_p
    lib.lensgb_version.argtypes = []
    lib.lensgb_version.restype = i
    _lib = lib
    return lib


def check(rc):
    if rc != OK:
        msg = load().lensgb_last_error().decode("utf-8", "replace")
        raise LensgbError(rc, msg)


class Model:
    """Owner of one lensgb_model handle."""

    def __init__(self, desc, refine=None, subframe=None, conv_method=0):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.lensgb_model_create(ctypes.byref(desc), ctypes.byref(h)))
        self._h = h
        if conv_method:
            check(lib.lensgb_model_set_convolution(h, int(conv_method)))
        self.desc = desc
        self.param_count = lib.lensgb_model_param_count(h)
        self.subframe = subframe
        if refine is not None:
            check(lib.lensgb_model_set_refine(h, float(refine[0]), float(refine[1])))
        if subframe is not None:
            r0, c0, mask = subframe
            m = (ctypes.c_ubyte * mask.size).from_buffer_copy(mask.astype("uint8").tobytes())
            check(lib.lensgb_model_set_subframe(h, int(r0), int(c0), int(mask.shape[0]), m))

    def refined_pixels(self, stream):
        n = ctypes.c_longlong(0)
        check(load().lensgb_model_refined_pixels(self._h, stream, ctypes.byref(n)))
        return int(n.value)

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            load().lensgb_model_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Bulk:
    """Owner of one lensgb_bulk handle (unique profile codes + scratch)."""

    def __init__(self, codes, precision, fp32_alpha_max=None):
        lib = load()
        arr = (ctypes.c_int * max(1, len(codes)))(*codes)
        h = ctypes.c_void_p()
        check(lib.lensgb_bulk_create(arr, len(codes), int(precision), ctypes.byref(h)))
        self._h = h
        if fp32_alpha_max is not None:
            check(lib.lensgb_bulk_set_fp32_alpha_max(h, float(fp32_alpha_max)))

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            load().lensgb_bulk_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
