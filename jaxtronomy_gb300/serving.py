"""Continuous-batching server for image and likelihood requests.

``Server`` wraps the ``lensgb_server_*`` entry points: a native worker thread
in liblensgb.so groups requests by bucket (the compiled model of their
``ImageModel`` plus noise options), keeps several batches in flight on
separate CUDA streams, admits new contexts within an HBM budget and replays
CUDA graphs for repeated launch shapes; with ``mixed_grids`` (default 2),
image requests that differ only in their grid, PSF size and supersampling
factor (``mixed_grids=1``: grid and PSF size) share a bucket and run through one
mixed-grid launch sequence.  Each result equals what
``ImageModel.image_batch`` / ``likelihood_batch`` returns for that request
alone.  The reference has no serving loop; requests here are single
``ImageModel.image`` / ``likelihood_data_given_model`` calls
(``image_model.py:163-221,432-492``).
"""

import ctypes

import numpy as np
import torch

from . import _device, _lib


class Ticket:
    """One submitted request: its ticket number and the host buffers it uses."""

    def __init__(self, server, ticket, image, logl, keep):
        self.server = server
        self.ticket = ticket
        self.image = image          # host array receiving the image
        self.logl = logl            # 1-element host array receiving logL (or None)
        self._keep = keep           # inputs that must stay alive until done

    def state(self):
        self.server._check_open()
        st = ctypes.c_int(0)
        _lib.check(_lib.load().lensgb_server_poll(self.server._h, self.ticket, ctypes.byref(st)))
        return st.value

    def done(self):
        return self.state() == _lib.REQ_DONE

    def cancel(self):
        """Withdraws the request if no batch has taken it yet; True if it will not
        run (state REQ_CANCELLED), False if it is already running or finished."""
        self.server._check_open()
        c = ctypes.c_int(0)
        _lib.check(_lib.load().lensgb_server_cancel(self.server._h, self.ticket,
                                                    ctypes.byref(c)))
        if c.value:
            self._keep = None
        return bool(c.value)

    def result(self, timeout=60.0):
        """Waits for the request; returns the image (and logL for likelihood requests)."""
        self.server._check_open()
        st = ctypes.c_int(0)
        _lib.check(_lib.load().lensgb_server_wait(self.server._h, self.ticket, float(timeout),
                                                  ctypes.byref(st)))
        if st.value == _lib.REQ_CANCELLED:
            raise RuntimeError("request %d was cancelled" % self.ticket)
        if st.value != _lib.REQ_DONE:
            raise TimeoutError("request %d not done after %.1f s" % (self.ticket, timeout))
        self._keep = None
        if self.logl is not None:
            return self.image, float(self.logl[0])
        return self.image

    def times(self):
        """(release, admit, done) in seconds on the server clock (-1: not reached)."""
        self.server._check_open()
        r, a, d = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_longlong()
        _lib.check(_lib.load().lensgb_server_request_times(
            self.server._h, self.ticket, ctypes.byref(r), ctypes.byref(a), ctypes.byref(d)))
        f = lambda v: v.value / 1e9 if v.value >= 0 else -1.0  # noqa: E731
        return f(r), f(a), f(d)


class Server:
    """Native serving loop (continuous batching) on the current CUDA device."""

    def __init__(self, n_streams=4, max_batch=256, hbm_budget_bytes=4 << 30,
                 contexts_per_bucket=2, use_graphs=True, mixed_grids=2):
        _device.require_cuda()
        # mixed_grids: 0 / False (exact-model buckets), 1 / True (grids and PSF
        # sizes share a bucket) or 2 (also supersampling factors; the default)
        cfg = _lib.ServerConfig(int(n_streams), int(max_batch), int(hbm_budget_bytes),
                                int(contexts_per_bucket), 1 if use_graphs else 0,
                                int(mixed_grids))
        h = ctypes.c_void_p()
        lib = _lib.load()
        _lib.check(lib.lensgb_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h

    def _check_open(self):
        if not self._h:
            raise RuntimeError("the server is closed; read results before closing it")

    def clock(self):
        """Server clock in seconds (the time base of ``release_s``)."""
        return _lib.load().lensgb_server_clock_ns(self._h) / 1e9

    def request(self, image_model, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
                psf_kernel=None, data=None, noise_map=None, mask=None, release_s=None,
                out=None):
        """Builds (without submitting) one request and the buffers it names.
        ``data`` makes it a likelihood request using the model's ImageData
        ``background_rms`` / ``exposure_time``.  ``psf_kernel``, ``data``,
        ``noise_map``, ``mask`` and ``out`` may be CUDA tensors on the server's
        device (contiguous, float64 for data / noise / mask, the model's dtype
        for the PSF -- already in :meth:`ImageModel.pack_psf` layout -- and the
        image): they stay resident and are read or written in place, with no
        host copy per batch.  Returns (Request, keep, image, logl)."""
        if getattr(image_model, "_n_ps", 0):
            raise ValueError("serving requests with point sources are not supported")
        if getattr(image_model, "_subframe", None) is not None:
            raise ValueError("the server does not take models with flux_evaluate_indexes")
        model = image_model._model(range(len(image_model.LensModel.lens_model_list)),
                                   range(len(image_model.SourceModel.profile_type_list)),
                                   range(len(image_model.LensLightModel.profile_type_list)))
        rows = image_model.pack_params(kwargs_lens, kwargs_source, kwargs_lens_light)
        if rows.shape[0] != 1:
            raise ValueError("a request holds one system; submit batched kwargs one by one")
        np_dtype = np.float64 if image_model._precision == _lib.FP64 else np.float32
        keep = [np.ascontiguousarray(rows[0])]
        req = _lib.Request()
        req.desc = model.desc
        req.params = keep[0].ctypes.data
        if image_model._psf_type != _lib.PSF_NONE:
            if isinstance(psf_kernel, torch.Tensor) and psf_kernel.is_cuda:
                tdt = torch.float64 if np_dtype == np.float64 else torch.float32
                if (psf_kernel.dtype != tdt or not psf_kernel.is_contiguous()
                        or psf_kernel.numel() != image_model.psf_elements()):
                    raise ValueError("a device PSF must be a contiguous %s tensor of %d values "
                                     "(ImageModel.pack_psf layout)"
                                     % (tdt, image_model.psf_elements()))
                keep.append(psf_kernel)
                req.psf = psf_kernel.data_ptr()
            else:
                k = image_model._kernel if psf_kernel is None else psf_kernel
                if np.shape(k) != image_model._kernel.shape:
                    raise ValueError("psf kernel must have shape %s"
                                     % (image_model._kernel.shape,))
                k = np.ascontiguousarray(image_model.pack_psf(k), dtype=np_dtype)
                keep.append(k)
                req.psf = k.ctypes.data
        shape = (image_model._nx, image_model._ny)
        if out is None:
            out = np.empty(shape, dtype=np_dtype)
        elif isinstance(out, torch.Tensor):
            tdt = torch.float64 if np_dtype == np.float64 else torch.float32
            if out.dtype != tdt or tuple(out.shape) != shape or not out.is_contiguous():
                raise ValueError("out must be a contiguous %s tensor of shape %s" % (tdt, shape))
        elif out.dtype != np_dtype or out.shape != shape or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous %s array of shape %s" % (np_dtype, shape))
        req.image_out = out.ctypes.data if isinstance(out, np.ndarray) else out.data_ptr()

        def plane(x, what):
            # a (ny, nx) float64 input: a resident CUDA tensor, or host memory
            if isinstance(x, torch.Tensor) and x.is_cuda:
                if x.dtype != torch.float64 or tuple(x.shape) != shape or not x.is_contiguous():
                    raise ValueError("%s must be a contiguous float64 tensor of shape %s"
                                     % (what, shape))
                keep.append(x)
                return x.data_ptr()
            a = np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype=np.float64), shape))
            keep.append(a)
            return a.ctypes.data
        logl = None
        if data is not None:
            if not (isinstance(data, torch.Tensor) and data.is_cuda) and np.shape(data) != shape:
                raise ValueError("data must have shape %s" % (shape,))
            req.data = plane(data, "data")
            D = image_model.Data
            if noise_map is None:
                noise_map = D.noise_map
            if mask is None and not np.all(image_model.likelihood_mask == 1):
                mask = image_model.likelihood_mask
            if noise_map is not None:
                req.noise_map = plane(noise_map, "noise_map")
            if mask is not None:
                req.mask = plane(mask, "mask")
            em = D.exposure_map
            if noise_map is None and em is None:
                raise ValueError("likelihood requests need an exposure time or a noise map")
            if noise_map is None and np.ndim(em) > 0:
                raise ValueError("server likelihood requests need a scalar exposure time or a "
                                 "noise map")
            req.background_rms = float(D.background_rms)
            req.exposure_time = float(em) if em is not None and np.ndim(em) == 0 else 1.0
            logl = np.zeros(1)
            keep.append(logl)
            req.logl_out = logl.ctypes.data
        req.release_ns = 0 if release_s is None else int(release_s * 1e9)
        return req, keep, out, logl

    def submit(self, image_model, kwargs_lens=None, kwargs_source=None, kwargs_lens_light=None,
               **kw):
        """Submits one request; returns its :class:`Ticket`."""
        req, keep, out, logl = self.request(image_model, kwargs_lens, kwargs_source,
                                            kwargs_lens_light, **kw)
        return self.submit_requests([(req, keep, out, logl)])[0]

    def submit_requests(self, built, array=None):
        """Submits requests built by :meth:`request` in one call (``array``: a
        ctypes array of their Request structs, e.g. kept between submissions)."""
        n = len(built)
        arr = (_lib.Request * n)(*[b[0] for b in built]) if array is None else array
        tickets = (ctypes.c_longlong * n)()
        _lib.check(_lib.load().lensgb_server_submit(self._h, arr, n, tickets))
        return [Ticket(self, tickets[i], built[i][2], built[i][3], built[i][1]) for i in range(n)]

    def drain(self, timeout=600.0):
        _lib.check(_lib.load().lensgb_server_drain(self._h, float(timeout)))

    def stats(self):
        st = _lib.ServerStats()
        _lib.check(_lib.load().lensgb_server_get_stats(self._h, ctypes.byref(st)))
        return {n: getattr(st, n) for n, _ in _lib.ServerStats._fields_}

    def close(self):
        if self._h:
            _lib.load().lensgb_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def pinned_empty(shape, dtype):
    """Page-locked host array (numpy view of a pinned torch tensor)."""
    t = torch.empty(shape, dtype=torch.float32 if dtype == np.float32 else torch.float64,
                    pin_memory=True)
    return t.numpy()
