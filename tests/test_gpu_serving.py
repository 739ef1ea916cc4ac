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
