"""Serving loop (lensgb_server_* through the C ABI) on the GPU.

Each served result must equal the same request computed alone by
ImageModel.image_batch / likelihood_batch.  The kernels compute every system
independently of the rest of its batch, so the stated tolerance -- 1e-5
relative on pixels above 1e-3 of the image maximum, the FP32 bar -- is met with
equality for exact-model buckets; the tests check bit equality there.  Mixed-grid
buckets (requests of different grids and PSF sizes in one batch) run the
mixed-launch instantiation of the FP32 ray kernel, whose FMA contractions may
round a few pixels by an ulp or two (which can also flip a pixel's FP64
refinement): against image_batch they are checked with the FP32 bar, 1e-5 of
the image maximum, and a request served alone and in a mix must agree bit for
bit in both modes.
"""

import ctypes

import numpy as np
import pytest
import torch

from jaxtronomy_gb300 import serving, workloads as W

pytestmark = pytest.mark.gpu

SIDES, SS, KS = (24, 40), (1, 2), (5, 11)


def _stream(n, seed=7):
    return W.serving_stream(seed=seed, n=n, sides=SIDES, supersampling=SS, kernel_sizes=KS,
                            psf_pool=4)


def _alone(models, r, psfs):
    im = models[r["key"]]
    out = im.image_batch(r["kwargs_lens"], r["kwargs_source"], r["kwargs_lens_light"],
                         psf_kernels=psfs[r["key"][2]][r["psf"]])
    return out[0].cpu().numpy()


def _check(got, ref, mixed_grids):
    if mixed_grids:
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    else:
        np.testing.assert_array_equal(got, ref)


def _models(reqs):
    return {k: W.serving_model(k) for k in {r["key"] for r in reqs}}


def _submit(srv, models, reqs, psfs, release=None, pinned=False):
    built = []
    for i, r in enumerate(reqs):
        im = models[r["key"]]
        out = serving.pinned_empty((r["key"][0],) * 2, np.float32) if pinned else None
        rel = None if release is None else release[i]
        built.append(srv.request(im, r["kwargs_lens"], r["kwargs_source"],
                                 r["kwargs_lens_light"], psf_kernel=psfs[r["key"][2]][r["psf"]],
                                 release_s=rel, out=out))
    return srv.submit_requests(built)


@pytest.mark.parametrize("mixed_grids", [False, True, 2])
def test_served_results_equal_alone_results(cuda, mixed_grids):
    base, psfs = _stream(60)
    reqs = [r for r in base for _ in range(2)]  # every request twice, released together
    models = _models(reqs)
    with serving.Server(n_streams=3, max_batch=16, mixed_grids=mixed_grids) as srv:
        t0 = srv.clock() + 0.01
        # staggered bursts: requests join batches while others are in flight
        gaps = np.random.default_rng(1).exponential(4e-4, len(base))
        release = t0 + np.repeat(np.cumsum(gaps), 2)
        tickets = _submit(srv, models, reqs, psfs, release=release)
        srv.drain(120)
        st = srv.stats()
        assert st["requests_done"] == len(reqs)
        assert st["batches"] < len(reqs)  # requests were batched
        assert (st["mixed_batches"] > 0) == bool(mixed_grids)
        for r, t in zip(reqs, tickets):
            got = t.result()
            _check(got, _alone(models, r, psfs), mixed_grids)
            rel, adm, done = t.times()
            assert 0 <= rel <= adm <= done


@pytest.mark.parametrize("mixed_grids", [False, True, 2])
def test_request_alone_and_in_mix_and_pinned_outputs(cuda, mixed_grids):
    reqs, psfs = _stream(60, seed=11)
    models = _models(reqs)
    probe = reqs[5]
    with serving.Server(n_streams=4, max_batch=8, mixed_grids=mixed_grids) as srv:
        alone = _submit(srv, models, [probe], psfs)[0].result()
    with serving.Server(n_streams=4, max_batch=8, mixed_grids=mixed_grids) as srv:
        tickets = _submit(srv, models, reqs, psfs, pinned=True)
        srv.drain(120)
        mixed = tickets[5].result()
        for r, t in zip(reqs, tickets):
            _check(t.result(), _alone(models, r, psfs), mixed_grids)
    np.testing.assert_array_equal(alone, mixed)


def test_graph_replay_matches_eager(cuda):
    reqs, psfs = _stream(200, seed=3)
    key = reqs[0]["key"]
    same = [r for r in reqs if r["key"] == key][:12] * 4
    models = _models(same)
    with serving.Server(n_streams=1, max_batch=4, contexts_per_bucket=1, use_graphs=True,
                        mixed_grids=False) as srv:
        tickets = []
        for i in range(0, len(same), 4):  # four equal batches of one bucket, one after another
            tickets += _submit(srv, models, same[i:i + 4], psfs)
            srv.drain(60)
        st = srv.stats()
        assert st["graph_captures"] >= 1 and st["graph_launches"] >= 1
        for r, t in zip(same, tickets):
            np.testing.assert_array_equal(t.result(), _alone(models, r, psfs))


@pytest.mark.parametrize("mixed_grids", [False, True])
def test_hbm_budget_evicts_idle_contexts(cuda, mixed_grids):
    reqs, psfs = _stream(80, seed=5)
    models = _models(reqs)
    # room for a handful of the ~40 small contexts (16 mixed ones) this stream needs
    budget = 512 << 10
    with serving.Server(n_streams=1, max_batch=4, hbm_budget_bytes=budget,
                        mixed_grids=mixed_grids) as srv:
        tickets = _submit(srv, models, reqs, psfs)
        srv.drain(120)
        st = srv.stats()
        assert st["evictions"] > 0
        assert st["peak_bytes"] <= budget
        for r, t in zip(reqs, tickets):
            _check(t.result(), _alone(models, r, psfs), mixed_grids)


def test_likelihood_requests_match_likelihood_batch(cuda):
    reqs, psfs = _stream(30, seed=9)
    rng = np.random.default_rng(2)
    models = _models(reqs)
    datas = []
    for i, r in enumerate(reqs):
        img = _alone(models, r, psfs).astype(np.float64)
        d = img + rng.normal(0, 0.01, img.shape)
        if i % 2:  # page-locked data is read by the device directly
            p = serving.pinned_empty(d.shape, np.float64)
            p[...] = d
            d = p
        datas.append(d)
    with serving.Server(n_streams=2, max_batch=8) as srv:
        built = [srv.request(models[r["key"]], r["kwargs_lens"], r["kwargs_source"],
                             r["kwargs_lens_light"], psf_kernel=psfs[r["key"][2]][r["psf"]],
                             data=d) for r, d in zip(reqs, datas)]
        tickets = srv.submit_requests(built)
        srv.drain(120)
        for r, d, t in zip(reqs, datas, tickets):
            img, logl = t.result()
            im = models[r["key"]]
            ref = im.likelihood_batch(r["kwargs_lens"], r["kwargs_source"],
                                      r["kwargs_lens_light"], data=d,
                                      psf_kernels=psfs[r["key"][2]][r["psf"]])
            ref = float(ref[0]) if hasattr(ref, "__len__") else float(ref)
            assert logl == ref
            np.testing.assert_array_equal(img, _alone(models, r, psfs))


def test_bad_request_is_rejected_at_submit(cuda):
    reqs, psfs = _stream(4)
    models = _models(reqs)
    with serving.Server() as srv:
        req, keep, out, logl = srv.request(models[reqs[0]["key"]], reqs[0]["kwargs_lens"],
                                           reqs[0]["kwargs_source"], reqs[0]["kwargs_lens_light"],
                                           psf_kernel=psfs[reqs[0]["key"][2]][0])
        req.desc.supersampling = 0
        with pytest.raises(Exception):
            srv.submit_requests([(req, keep, out, logl)])


# ---------------------------------------------------------------------------
# failure paths, cancellation and device-resident inputs
# ---------------------------------------------------------------------------

def test_request_over_the_hbm_budget_fails_with_oom(cuda):
    """A request whose context cannot fit hbm_budget_bytes, with nothing in flight
    and nothing left to evict, ends FAILED with LENSGB_ERR_OOM instead of
    waiting forever; a later request that fits is still served."""
    from jaxtronomy_gb300 import _lib
    reqs, psfs = W.serving_stream(seed=13, n=40, sides=(100,), supersampling=(2,),
                                  kernel_sizes=(11,), psf_pool=2)
    models = _models(reqs[:1])
    with serving.Server(n_streams=1, max_batch=4, hbm_budget_bytes=64 << 10,
                        mixed_grids=False) as srv:
        t = _submit(srv, models, reqs[:1], psfs)[0]
        st = ctypes.c_int(0)
        rc = _lib.load().lensgb_server_wait(srv._h, t.ticket, 30.0, ctypes.byref(st))
        assert rc == _lib.ERR_OOM and st.value == _lib.REQ_FAILED
        with pytest.raises(_lib.LensgbError):
            t.result()
        assert srv.stats()["requests_done"] == 1
    small, spsf = _stream(4)
    sm = _models(small)
    with serving.Server(n_streams=1, max_batch=4, hbm_budget_bytes=64 << 20) as srv:
        ok = _submit(srv, sm, small, spsf)
        for r, tk in zip(small, ok):
            _check(tk.result(), _alone(sm, r, spsf), True)


def test_wait_times_out_without_blocking_and_cancel(cuda):
    """A request released 30 s in the future: a wait with a 50 ms timeout returns
    (TimeoutError from Ticket.result) without blocking; cancelling it ends it
    CANCELLED before it ever runs, and the server drains at once.  A request
    that has finished cannot be cancelled."""
    import time as _time
    from jaxtronomy_gb300 import _lib
    reqs, psfs = _stream(3, seed=17)
    models = _models(reqs)
    with serving.Server(n_streams=1, max_batch=4) as srv:
        later = _submit(srv, models, reqs[:1], psfs, release=[srv.clock() + 30.0])[0]
        t0 = _time.perf_counter()
        with pytest.raises(TimeoutError):
            later.result(timeout=0.05)
        assert _time.perf_counter() - t0 < 2.0
        assert later.state() == _lib.REQ_QUEUED
        assert later.cancel() is True
        assert later.state() == _lib.REQ_CANCELLED
        with pytest.raises(RuntimeError):
            later.result(timeout=1.0)
        assert later.times()[1] == -1  # never admitted
        now = _submit(srv, models, reqs[1:2], psfs)[0]
        img = now.result()
        assert now.cancel() is False
        srv.drain(10.0)
        _check(img, _alone(models, reqs[1], psfs), True)
        assert srv.stats()["requests_done"] == 2


@pytest.mark.parametrize("on_device", ["psf", "data", "all"])
def test_device_resident_inputs_equal_host_inputs(cuda, on_device):
    """Likelihood requests whose PSF, data, noise map and mask (and output image)
    are CUDA tensors kept on the device: the gather kernels read them in place,
    and the results equal the host-buffer requests and likelihood_batch bit for
    bit."""
    reqs, psfs = _stream(12, seed=19)
    rng = np.random.default_rng(5)
    models = _models(reqs)
    host, dev = [], []
    for r in reqs:
        img = _alone(models, r, psfs).astype(np.float64)
        d = img + rng.normal(0, 0.01, img.shape)
        nm = np.full(img.shape, 0.012)
        mk = (rng.random(img.shape) > 0.1).astype(np.float64)
        host.append((d, nm, mk))
    with serving.Server(n_streams=2, max_batch=8) as srv:
        bh, bd = [], []
        for r, (d, nm, mk) in zip(reqs, host):
            im = models[r["key"]]
            kern = psfs[r["key"][2]][r["psf"]]
            bh.append(srv.request(im, r["kwargs_lens"], r["kwargs_source"],
                                  r["kwargs_lens_light"], psf_kernel=kern, data=d,
                                  noise_map=nm, mask=mk))
            dt = torch.float32
            kd = (torch.as_tensor(im.pack_psf(kern), dtype=dt).cuda().contiguous()
                  if on_device in ("psf", "all") else kern)
            dd, nmd, mkd = ((torch.as_tensor(x).cuda().contiguous() for x in (d, nm, mk))
                            if on_device in ("data", "all") else (d, nm, mk))
            out = (torch.empty((r["key"][0],) * 2, dtype=dt, device="cuda")
                   if on_device == "all" else None)
            bd.append(srv.request(im, r["kwargs_lens"], r["kwargs_source"],
                                  r["kwargs_lens_light"], psf_kernel=kd, data=dd, noise_map=nmd,
                                  mask=mkd, out=out))
        th = srv.submit_requests(bh)
        td = srv.submit_requests(bd)
        srv.drain(120)
        for r, (d, nm, mk), a, b in zip(reqs, host, th, td):
            ia, la = a.result()
            ib, lb = b.result()
            ib = ib.cpu().numpy() if isinstance(ib, torch.Tensor) else ib
            assert la == lb
            np.testing.assert_array_equal(ia, ib)
