#!/usr/bin/env python
"""Benchmark of the lens image-simulation path on GB300.

Workload (one "step"): a batch of 1024 EPL+SHEAR lens systems, 180x180 pixels at
0.04"/pix, supersampling 3 (540x540 rays per system), SERSIC_ELLIPSE source and
lens light, one 31x31 Moffat PSF per system -- simulated in ONE batched launch
sequence of the FP32-split kernels, inputs resident in HBM.

Reported beside it: the plain FP64 kernel at one request per launch, single-
request latency, FP32-vs-FP64 and FP64-vs-oracle errors, the end-to-end rate
through the public API with host buffers, the roofline of the dominant kernel,
and the CPU baseline (the FP64 oracle on the host cores).

``--impl reference`` times the reference's CPU path instead: the reference
itself (JAXtronomy on JAX) cannot be installed here, so this arm times the FP64
NumPy restatement of it (``oracle/``) on all host cores.
"""

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "images/s + p50/p99 latency, batched FP32-split vs plain FP64, rel err<=1e-5"
WORKLOAD = "batch_epl_180x180_s3_psf31"
N_PIX, DPIX, SS, KSIZE = 180, 0.04, 3, 31

# Algorithmic work per supersampled ray and per output pixel ("flop" = add, mul
# or compare with FMA = 2; "T" = one transcendental call), counted from the
# reference formulas: EPL 60 + 8 nmax flop / 7 T, SHEAR 8, SIE 20 / 5 T,
# SERSIC_ELLIPSE 15 / 4 T, s x s re-binning 1; direct convolution 2 K^2 per pixel.
FLOP_EPL_BASE, FLOP_EPL_PER_TERM, T_EPL = 60, 8, 7
FLOP_SHEAR = 8
FLOP_SERSIC, T_SERSIC = 15, 4
FLOP_REDUCE = 1


# ---------------------------------------------------------------------------
# CPU side (oracle port), run in spawn-started worker processes
# ---------------------------------------------------------------------------

_JOB_CACHE = {}


def _oracle_inputs(seed):
    if seed not in _JOB_CACHE:
        from jaxtronomy_gb300 import workloads as W
        model, lens, src, ll, kern = W.batch_epl(seed=seed, batch=8)
        g = W.grid_kwargs(N_PIX, DPIX)
        jobs = []
        for i in range(8):
            scene = dict(nx=N_PIX, ny=N_PIX, supersampling_factor=SS, psf_type="PIXEL",
                         kernel=kern[i], lens_model_list=model["lens_model_list"],
                         source_light_model_list=model["source_light_model_list"],
                         lens_light_model_list=model["lens_light_model_list"], **g)
            jobs.append((scene, W.instance(lens, i), W.instance(src, i), W.instance(ll, i)))
        _JOB_CACHE[seed] = jobs
    return _JOB_CACHE[seed]


def _oracle_job(args):
    seed, i = args
    import warnings
    warnings.simplefilter("ignore")
    from oracle import image as oimage
    scene, kl, ks, kll = _oracle_inputs(seed)[i % 8]
    t = time.perf_counter()
    oimage.image(scene, kl, ks, kll)
    return time.perf_counter() - t


def _spawn_pool(cores):
    for v in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
        os.environ[v] = "1"
    pool = mp.get_context("spawn").Pool(cores)
    pool.map(_oracle_job, [(2001, 0)] * cores, chunksize=1)  # imports + input cache
    return pool


def cpu_cores():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_cpu_sample(pool, cores, n_images, seed=2001):
    jobs = [(seed, i % 8) for i in range(n_images)]
    t0 = time.perf_counter()
    pool.map(_oracle_job, jobs, chunksize=1)
    return time.perf_counter() - t0


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu model")):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def reference_arm(args):
    """CPU reference path: the FP64 oracle over all host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cores = cpu_cores()
    per_step = 2 * cores
    pool = _spawn_pool(cores)
    try:
        for _ in range(args.warmup):
            run_cpu_sample(pool, cores, per_step)
        times = [run_cpu_sample(pool, cores, per_step) for _ in range(args.steps)]
    finally:
        pool.close()
    sec = statistics.mean(times)
    value = per_step / sec
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "images/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "batch_per_step": per_step, "grid": N_PIX,
                   "supersampling": SS, "psf": KSIZE},
        "cpu_baseline": {"value": value, "unit": "images/s", "cores": cores, "kind": "port",
                         "sample": "%d systems of the workload per step, one per worker "
                                   "process (spawn pool of %d), FP64 NumPy oracle; JAXtronomy "
                                   "itself needs jax, which is not installable offline"
                                   % (per_step, cores),
                         "cpu": cpu_model()},
        "e2e": {"value": value, "unit": "images/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------------------
# GPU side
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        # side files (the per-run clock samples) go to LENSGB_BENCH_OUT if set
        outdir = os.environ.get("LENSGB_BENCH_OUT") or tempfile.gettempdir()
        self.path = os.path.join(outdir, "clocks_rank%d.csv" % gpu_index)

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, v in zip(names[1:], p[5:9]):
                if v.lower() in ("active", "0x1") or v == "Active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def ray_work(lens, n_inst, nmax_list):
    rays = (N_PIX * SS) ** 2
    flop = 0
    tcount = 0
    for nm in nmax_list:
        flop += rays * (FLOP_EPL_BASE + FLOP_EPL_PER_TERM * nm + FLOP_SHEAR + 2 * FLOP_SERSIC
                        + FLOP_REDUCE)
        tcount += rays * (T_EPL + 2 * T_SERSIC)
    return flop, tcount


def epl_nmax(e1, e2):
    import numpy as np
    c = np.minimum(np.hypot(e1, e2), 0.9999)
    q = (1 - c) / (1 + c)
    f = (1 - q) / (1 + q)
    out = []
    for v in f:
        if v == 0:
            out.append(0)
        elif v < 0.12:
            out.append(10)
        elif v < 0.4:
            out.append(20)
        elif v < 0.6:
            out.append(35)
        elif v < 0.73:
            out.append(50)
        elif v < 0.86:
            out.append(100)
        elif v < 0.92:
            out.append(200)
        else:
            out.append(500)
    return out


def epl_fp32_series_length(lens):
    """Per system, the number of EPL series terms the FP32 kernel evaluates: the
    reference's nmax(f) shortened to where sum_{m>=k} |F_m| (f/(2-f))^m falls
    below 2^-27 (the prepare kernel's rule, restated for the count)."""
    import numpy as np
    e1, e2, gam = lens[0]["e1"], lens[0]["e2"], lens[0]["gamma"]
    out = []
    for nm, a, b, g in zip(epl_nmax(e1, e2), e1, e2, gam):
        c = min(np.hypot(a, b), 0.9999)
        q = (1 - c) / (1 + c)
        f = (1 - q) / (1 + q)
        if nm <= 1:
            out.append(nm)
            continue
        t = g - 1.0
        B, C = t / 2.0, 2.0 - t / 2.0
        F = [1.0, 1.0 - 2.0 * B / C]
        for n in range(2, nm):
            F.append(((n - 1.0) * F[n - 2] - (2.0 * B - C) * F[n - 1]) / (C + n - 1.0))
        wmax = f / (2.0 - f)
        tail, wp, n32 = 0.0, wmax ** (nm - 1), nm
        for m in range(nm - 1, 0, -1):
            tail += abs(F[m]) * wp
            if tail > 7.450580596923828e-09:
                break
            n32 = m
            wp /= wmax
        out.append(n32)
    return out


def fma_peaks(reps=5):
    """Measured FP32 and FP64 FMA rates (TFLOP/s) of this device: the project's
    FMA-chain kernel (lensgb_fma_chain, 8 CTAs of 256 threads per SM, 8
    independent chains per thread), best of `reps` launches timed with CUDA
    events on the launch stream after a warm-up."""
    import ctypes
    import torch
    from jaxtronomy_gb300 import _device, _lib
    lib = _lib.load()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks = 8 * sms
    out = {"sms": sms, "blocks": blocks, "threads_per_block": 256, "chains_per_thread": 8}
    stream = torch.cuda.current_stream()
    for name, prec, iters, dtype in (("fp32", _lib.FP32_SPLIT, 65536, torch.float32),
                                     ("fp32_pairs", 2, 32768, torch.float32),
                                     ("fp64", _lib.FP64, 1024, torch.float64)):
        buf = torch.empty(blocks * 256, dtype=dtype, device="cuda")
        flops = ctypes.c_longlong(0)
        best = None
        for k in range(reps + 1):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(lib.lensgb_fma_chain(prec, blocks, iters, _device.ptr(buf),
                                            ctypes.byref(flops), _device.stream_handle()))
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            if k > 0 and (best is None or ms < best):
                best = ms
        out[name + "_tflops"] = flops.value / (best / 1e3) / 1e12
        out[name + "_launch_ms"] = best
    return out


# Substructure ray shooting (LensModelBulk): 1000^2 rays at 0.01"/pix through
# EPL + SHEAR + 2000 TNFW subhalos.  Per (ray, TNFW) pair 35 flop and 8 T,
# counted from the reference formulas (tnfw.py:69-87,228-349).
FLOP_TNFW, T_TNFW = 35, 8
SUB_PIX, SUB_DPIX, SUB_N = 1000, 0.01, 2000


def substructure_section(steps, warmup, fp32_peak, flush):
    """FP32 bulk ray shooting rate, FP32-vs-FP64 deflection and image error,
    FP64-vs-oracle on a ray sample, and the oracle's CPU rate on a sample."""
    import numpy as np
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import workloads as W
    from oracle import lens as olens

    x, y, ll, kw, src = W.substructure(num_pix=SUB_PIX, delta_pix=SUB_DPIX, n_sub=SUB_N)
    unique = ["EPL", "SHEAR", "TNFW"]
    b32 = J.LensModelBulk(unique, precision="fp32")
    b64 = J.LensModelBulk(unique, precision="fp64")
    rk = b32.prepare_ray_shooting_kwargs(ll, kw)
    rk_dev = {"all_kwargs": {k: torch.as_tensor(v).cuda() for k, v in rk["all_kwargs"].items()},
              "index_list": torch.as_tensor(rk["index_list"]).cuda()}
    xt = torch.as_tensor(x).cuda()
    yt = torch.as_tensor(y).cuda()
    stream = torch.cuda.current_stream()
    for _ in range(max(warmup, 3)):
        b32.ray_shooting(xt, yt, rk_dev)
    torch.cuda.synchronize()
    times = []
    for _ in range(max(steps, 3)):
        flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bx32, by32 = b32.ray_shooting(xt, yt, rk_dev)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.mean(times)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    bx64, by64 = b64.ray_shooting(xt, yt, rk_dev)
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1)
    d = torch.maximum((bx32 - bx64).abs(), (by32 - by64).abs())
    lm = J.LightModel(["SERSIC_ELLIPSE"])
    s32 = lm.surface_brightness(bx32, by32, src)
    s64 = lm.surface_brightness(bx64, by64, src)
    sig = s64.abs() >= 1e-3 * s64.abs().max()
    rel = ((s32 - s64).abs()[sig] / s64.abs()[sig])
    # FP64 vs the oracle on a ray sample
    sample = np.arange(0, x.size, x.size // 256)[:256]
    ox, oy = olens.bulk_ray_shooting(unique, x[sample], y[sample], rk["all_kwargs"],
                                     rk["index_list"])
    g64x = bx64.cpu().numpy()[sample]
    g64y = by64.cpu().numpy()[sample]
    orc = max(np.max(np.abs(g64x - ox) / np.maximum(np.abs(ox), 1e-300)),
              np.max(np.abs(g64y - oy) / np.maximum(np.abs(oy), 1e-300)))
    # oracle CPU rate on a ray sample (1 core, vectorised over rays)
    cs = np.arange(0, x.size, x.size // 2000)[:2000]
    t0 = time.perf_counter()
    olens.bulk_ray_shooting(unique, x[cs], y[cs], rk["all_kwargs"], rk["index_list"])
    cpu_s = time.perf_counter() - t0
    n_pairs = x.size * len(ll)
    flop = x.size * SUB_N * FLOP_TNFW
    return {
        "workload": "substructure_1000x1000_epl_shear_2000tnfw",
        "rays": int(x.size), "deflectors": len(ll),
        "ms_per_call": ms, "rays_per_s": x.size / (ms / 1e3),
        "pairs_per_s": n_pairs / (ms / 1e3),
        "fp64_ms_per_call": ms64, "speedup_vs_fp64": ms64 / ms,
        "beta_err_fp32_vs_fp64_arcsec_max": d.max().item(),
        "beta_err_fp32_vs_fp64_arcsec_median": d.median().item(),
        "image_rel_err_fp32_vs_fp64_max": rel.max().item(),
        "image_rel_err_fp32_vs_fp64_median": rel.median().item(),
        "fp64_vs_oracle_rel_err_max": float(orc),
        "roofline": {"kernel": "bulk_ray_kernel<FP32>", "bound": "fp32", "unit": "TFLOP/s",
                     "achieved": flop / (ms / 1e3) / 1e12, "peak": fp32_peak,
                     "frac": flop / (ms / 1e3) / 1e12 / fp32_peak,
                     "algorithmic_gflop_per_launch": flop / 1e9,
                     "transcendentals_per_s": x.size * SUB_N * T_TNFW / (ms / 1e3)},
        "cpu_baseline": {"value": cs.size / cpu_s, "unit": "rays/s", "cores": 1, "kind": "port",
                         "sample": "%d rays x %d deflectors, FP64 NumPy oracle "
                                   "(SinglePlaneBulk restatement), vectorised over rays"
                                   % (cs.size, len(ll))},
        "timing": "CUDA events per call after %d warm-ups, L2 flushed before each" % max(warmup, 3),
    }


# Multi-plane substructure ray shooting (LensModelBulk, multi_plane=True): the
# shapes of the reference's GPU notebook benchmark (400^2 rays through 5130 TNFW
# halos and 126 CONVERGENCE sheets on 126 planes, z_s = 2.5, num_deflectors =
# 5500); published there: 47.93 s lenstronomy CPU, 0.468 s JAXtronomy GPU (FP64).
MP_PUBLISHED_S = {"lenstronomy_cpu": 47.93, "jaxtronomy_gpu_fp64": 0.468}


def multi_plane_section(steps, warmup, fp32_peak, flush):
    """FP32 and FP64 multi-plane ray shooting times, FP32-vs-FP64 and FP64-vs-oracle
    errors, and the oracle's CPU rate on a ray sample."""
    import numpy as np
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import workloads as W
    from oracle import lens as olens

    x, y, ll, kw, z, zs, nd = W.line_of_sight_halos()
    unique = ["TNFW", "CONVERGENCE"]
    cosmo = J.FlatLambdaCDM(67.66, 0.30966)
    b32 = J.LensModelBulk(unique, multi_plane=True, cosmo=cosmo, precision="fp32")
    b64 = J.LensModelBulk(unique, multi_plane=True, cosmo=cosmo, precision="fp64")
    t0 = time.perf_counter()
    rk = b32.prepare_ray_shooting_kwargs(ll, kw, z_source=zs, lens_redshift_list=z,
                                         num_deflectors=nd)
    prep_s = time.perf_counter() - t0
    rk_dev = {k: ({kk: torch.as_tensor(vv).cuda() for kk, vv in v.items()}
                  if isinstance(v, dict) else torch.as_tensor(v).cuda())
              for k, v in rk.items()}
    xt = torch.as_tensor(x).cuda()
    yt = torch.as_tensor(y).cuda()
    stream = torch.cuda.current_stream()

    def timed(b, n_rep):
        times = []
        for _ in range(n_rep):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = b.ray_shooting(xt, yt, rk_dev)
            e1.record(stream)
            torch.cuda.synchronize()
            times.append(e0.elapsed_time(e1))
        return statistics.mean(times), out

    for _ in range(max(warmup, 3)):
        b32.ray_shooting(xt, yt, rk_dev)
    torch.cuda.synchronize()
    ms, (bx32, by32) = timed(b32, max(steps, 3))
    b64.ray_shooting(xt, yt, rk_dev)
    ms64, (bx64, by64) = timed(b64, 1)
    d = torch.maximum((bx32 - bx64).abs(), (by32 - by64).abs())
    sample = np.arange(0, x.size, x.size // 256)[:256]
    ox, oy = olens.multi_plane_ray_shooting(unique, x[sample], y[sample], rk["all_kwargs"],
                                            rk["index_list"], rk["T_ij_list"], rk["T_z_list"],
                                            rk["reduced2physical_factor"])
    g64x = bx64.cpu().numpy()[sample]
    g64y = by64.cpu().numpy()[sample]
    orc = max(np.max(np.abs(g64x - ox) / np.maximum(np.abs(ox), 1e-300)),
              np.max(np.abs(g64y - oy) / np.maximum(np.abs(oy), 1e-300)))
    cs = np.arange(0, x.size, x.size // 2000)[:2000]
    t0 = time.perf_counter()
    olens.multi_plane_ray_shooting(unique, x[cs], y[cs], rk["all_kwargs"], rk["index_list"],
                                   rk["T_ij_list"], rk["T_z_list"], rk["reduced2physical_factor"])
    cpu_s = time.perf_counter() - t0
    n_tnfw = sum(1 for m in ll if m == "TNFW")
    flop = x.size * n_tnfw * FLOP_TNFW
    return {
        "workload": "multi_plane_400x400_5130tnfw_126convergence_126planes_5500steps",
        "rays": int(x.size), "deflectors": len(ll), "steps": int(len(rk["index_list"])),
        "ms_per_call": ms, "rays_per_s": x.size / (ms / 1e3),
        "pairs_per_s": x.size * len(rk["index_list"]) / (ms / 1e3),
        "fp64_ms_per_call": ms64, "speedup_vs_fp64": ms64 / ms,
        "published_s": MP_PUBLISHED_S,
        "speedup_vs_published_jaxtronomy_gpu": MP_PUBLISHED_S["jaxtronomy_gpu_fp64"] / (ms / 1e3),
        "fp64_speedup_vs_published_jaxtronomy_gpu":
            MP_PUBLISHED_S["jaxtronomy_gpu_fp64"] / (ms64 / 1e3),
        "host_prepare_s": prep_s,
        "beta_err_fp32_vs_fp64_arcsec_max": d.max().item(),
        "beta_err_fp32_vs_fp64_arcsec_median": d.median().item(),
        "fp64_vs_oracle_rel_err_max": float(orc),
        "roofline": {"kernel": "multi_plane_kernel<FP32>", "bound": "fp32", "unit": "TFLOP/s",
                     "achieved": flop / (ms / 1e3) / 1e12, "peak": fp32_peak,
                     "frac": flop / (ms / 1e3) / 1e12 / fp32_peak,
                     "algorithmic_gflop_per_launch": flop / 1e9,
                     "flop_model": "%d flop per (ray, TNFW) pair; CONVERGENCE, plane updates "
                                   "and FP32-pair state not counted" % FLOP_TNFW},
        "cpu_baseline": {"value": cs.size / cpu_s, "unit": "rays/s", "cores": 1, "kind": "port",
                         "sample": "%d rays x %d steps, FP64 NumPy oracle (MultiPlaneBulk "
                                   "restatement), vectorised over rays"
                                   % (cs.size, len(rk["index_list"]))},
        "timing": "CUDA events per call after %d warm-ups, L2 flushed before each; "
                  "distances from FlatLambdaCDM(67.66, 0.30966)" % max(warmup, 3),
    }


def single_image_section(n_calls=200, n_systems=16, seed=1000):
    """Plain single image (60x60 at 0.05", SIE+SHEAR, SERSIC_ELLIPSE source and
    lens light, s = 1, 11x11 PIXEL kernel of a FWHM 0.1" Gaussian): one
    ImageModel.image call per image.  Latency p50/p99 of the device work (CUDA
    events around one image_batch call with the row on the device) and of the
    whole public call ImageModel.image(kwargs...) -> numpy (host clock), and the
    per-pixel error of FP64 and FP32 against the FP64 oracle on n_systems systems
    (max and median, no floor)."""
    import warnings
    import numpy as np
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import workloads as W
    from oracle import image as oimage
    warnings.simplefilter("ignore")

    model, lens, src, ll, kern = W.single_sie(seed=seed, batch=max(n_systems, 1))
    n, dpix = model["num_pix"], model["delta_pix"]
    g = W.grid_kwargs(n, dpix)
    scene = dict(nx=n, ny=n, supersampling_factor=1, psf_type="PIXEL", kernel=kern[0],
                 lens_model_list=model["lens_model_list"],
                 source_light_model_list=model["source_light_model_list"],
                 lens_light_model_list=model["lens_light_model_list"], **g)
    refs = [oimage.image(scene, W.instance(lens, i), W.instance(src, i), W.instance(ll, i))
            for i in range(n_systems)]
    out = {"workload": "single_sie_60x60_s1_psf11", "calls": n_calls, "systems": n_systems}
    stream = torch.cuda.current_stream()
    for prec in ("fp64", "fp32"):
        data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0, background_rms=0.01, **g)
        im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                          J.LensModel(model["lens_model_list"]),
                          J.LightModel(model["source_light_model_list"]),
                          J.LightModel(model["lens_light_model_list"]),
                          kwargs_numerics={"supersampling_factor": 1, "precision": prec})
        errs = []
        for i in range(n_systems):
            got = im.image(W.instance(lens, i), W.instance(src, i), W.instance(ll, i))
            errs.append((np.abs(np.asarray(got, float) - refs[i]) / np.abs(refs[i])).ravel())
        errs = np.concatenate(errs)
        rows = torch.as_tensor(im.pack_params(lens, src, ll)).cuda()
        img = torch.empty((1, n, n), dtype=torch.float64 if prec == "fp64" else torch.float32,
                          device="cuda")
        for i in range(5):
            im.image_batch(rows=rows[i % n_systems:i % n_systems + 1], out=img)
        torch.cuda.synchronize()
        dev = []
        for i in range(n_calls):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            im.image_batch(rows=rows[i % n_systems:i % n_systems + 1], out=img)
            e1.record(stream)
            e1.synchronize()
            dev.append(e0.elapsed_time(e1))
        kws = [(W.instance(lens, i), W.instance(src, i), W.instance(ll, i))
               for i in range(n_systems)]
        host = []
        for i in range(n_calls):
            t0 = time.perf_counter()
            im.image(*kws[i % n_systems])
            host.append((time.perf_counter() - t0) * 1e3)
        out[prec] = {"device_latency_ms_p50": percentile(dev, 0.5),
                     "device_latency_ms_p99": percentile(dev, 0.99),
                     "image_call_latency_ms_p50": percentile(host, 0.5),
                     "image_call_latency_ms_p99": percentile(host, 0.99),
                     "images_per_s_one_per_call": 1e3 / statistics.mean(host),
                     "vs_oracle_rel_err_max": float(errs.max()),
                     "vs_oracle_rel_err_median": float(np.median(errs))}
    out["timing"] = ("device: CUDA events around image_batch(rows on the device) of one "
                     "system; image_call: host clock around ImageModel.image(kwargs) returning "
                     "a numpy image (parameter packing, upload, kernels, download)")
    return out


def serving_section(n_req, seed=1002, n_streams=32, max_batch=64, contexts_per_bucket=2,
                    use_graphs=True, loads=(0.5, 0.8, 0.95), mixed_grids=2,
                    sweep=(0.7, 0.85, 0.9, 1.0), repeats=3):
    """Serving stream: capacity (all requests released at once), then Poisson
    arrivals at fractions of it (0.5 .. 1.0, each repeated) with p50/p99 latency
    and the highest load served in full (sustained capacity); results of a
    sample checked against the same requests computed alone.  mixed_grids:
    requests of every grid and PSF size of one (profile stack, supersampling)
    share a bucket (2: of one profile stack); otherwise every exact model is a
    bucket of its own."""
    import numpy as np
    from jaxtronomy_gb300 import _lib, serving, workloads as W

    reqs, psfs = W.serving_stream(seed=seed, n=n_req)
    models = {k: W.serving_model(k) for k in sorted({r["key"] for r in reqs})}
    pool = {side: [serving.pinned_empty((side, side), np.float32) for _ in range(32)]
            for side in {k[0] for k in models}}
    srv = serving.Server(n_streams=n_streams, max_batch=max_batch, hbm_budget_bytes=16 << 30,
                         contexts_per_bucket=contexts_per_bucket, use_graphs=use_graphs,
                         mixed_grids=mixed_grids)
    built = []
    t_build = time.perf_counter()
    for i, r in enumerate(reqs):
        out = pool[r["key"][0]][i % 32]
        built.append(srv.request(models[r["key"]], r["kwargs_lens"], r["kwargs_source"],
                                 r["kwargs_lens_light"], psf_kernel=psfs[r["key"][2]][r["psf"]],
                                 out=out))
    t_build = time.perf_counter() - t_build

    arr = (_lib.Request * len(built))(*[b[0] for b in built])
    run_lead = [0.5]

    def run(offsets):
        # release times start after the submission call has surely returned
        t0 = srv.clock() + run_lead[0]
        rel = ((t0 + np.asarray(offsets)) * 1e9).astype(np.int64)
        for i in range(len(built)):
            arr[i].release_ns = int(rel[i])
        st0 = srv.stats()
        ts = time.perf_counter()
        tickets = srv.submit_requests(built, array=arr)
        run.submit_s = time.perf_counter() - ts
        run_lead[0] = 0.05 + 2 * run.submit_s
        srv.drain(900)
        st1 = srv.stats()
        run.captures = st1["graph_captures"] - st0["graph_captures"]
        run.capture_ms = (st1["capture_ns"] - st0["capture_ns"]) / 1e6
        times = np.array([t.times() for t in tickets])
        lat = (times[:, 2] - times[:, 0]) * 1e3
        span = times[:, 2].max() - times[:, 0].min()
        run.wait_ms = (times[:, 1] - times[:, 0]) * 1e3
        run.service_ms = (times[:, 2] - times[:, 1]) * 1e3
        return tickets, lat, span

    # warm-up: every bucket's contexts, graphs and kernels -- for the large
    # batches of a burst and the small ones of Poisson arrivals
    run(np.zeros(len(built)))
    _, lat_cap, span = run(np.zeros(len(built)))
    capacity = len(built) / span
    rng = np.random.default_rng(seed + 1)
    for f in (0.5, 0.95):
        run(np.cumsum(rng.exponential(1.0 / (f * capacity), len(built))))
    # Poisson loads as fractions of the burst capacity, each repeated; a load is
    # sustained when every repeat served >= 0.99 of the offered rate (offered =
    # requests / arrival span of that realisation)
    runs = {}
    for rep in range(repeats):
        for f in sorted(set(loads) | set(sweep)):
            lam = f * capacity
            offs = np.cumsum(rng.exponential(1.0 / lam, len(built)))
            tickets, lat, span = run(offs)
            offered = (len(built) - 1) / (offs[-1] - offs[0])
            runs.setdefault(f, []).append({
                "offered_per_s": offered, "served_per_s": len(built) / span,
                "latency_ms_p50": float(np.percentile(lat, 50)),
                "latency_ms_p99": float(np.percentile(lat, 99)),
                "queue_wait_ms_p50": float(np.percentile(run.wait_ms, 50)),
                "service_ms_p50": float(np.percentile(run.service_ms, 50)),
                "submit_call_s": run.submit_s,
                "graph_captures": run.captures, "capture_ms": run.capture_ms})
    med = lambda v: float(np.median(v))  # noqa: E731
    load_lines = []
    for f in sorted(runs):
        rr = runs[f]
        load_lines.append({"load": f, "arrival_rate_per_s": f * capacity,
                           "repeats": len(rr),
                           "served_over_offered_min": min(r["served_per_s"] / r["offered_per_s"]
                                                          for r in rr),
                           **{k: med([r[k] for r in rr]) for k in rr[0]},
                           "latency_ms_p99_repeats": [r["latency_ms_p99"] for r in rr],
                           "graph_captures_repeats": [r["graph_captures"] for r in rr]})
    ok = [ln for ln in load_lines if ln["served_over_offered_min"] >= 0.99]
    best = max(ok, key=lambda ln: ln["load"]) if ok else None
    sustained = None if best is None else {
        "load": best["load"], "requests_per_s": best["served_per_s"],
        "latency_ms_p50": best["latency_ms_p50"], "latency_ms_p99": best["latency_ms_p99"],
        "rule": "highest Poisson load (fraction of the burst capacity) at which all %d "
                "repeats served >= 0.99 x the offered rate; latencies: median over repeats"
                % repeats}
    # sample of results vs the same requests alone
    worst = 0.0
    for i in rng.choice(len(reqs), 24, replace=False):
        r = reqs[i]
        im = models[r["key"]]
        req, keep, out, _ = srv.request(im, r["kwargs_lens"], r["kwargs_source"],
                                        r["kwargs_lens_light"],
                                        psf_kernel=psfs[r["key"][2]][r["psf"]])
        served = srv.submit_requests([(req, keep, out, None)])[0].result()
        alone = im.image_batch(r["kwargs_lens"], r["kwargs_source"], r["kwargs_lens_light"],
                               psf_kernels=psfs[r["key"][2]][r["psf"]])[0].cpu().numpy()
        worst = max(worst, float(np.max(np.abs(served - alone))))
    st = srv.stats()
    srv.close()
    rays = np.mean([(r["key"][0] * r["key"][1]) ** 2 for r in reqs])
    return {
        "workload": "serving_stream_%d_requests" % len(reqs),
        "requests": len(reqs),
        "buckets": (len({(k[3], k[4]) for k in models}) if mixed_grids == 2 else
                    len({(k[1], k[3], k[4]) for k in models}) if mixed_grids else len(models)),
        "mixed_grids": mixed_grids,
        "capacity_requests_per_s": capacity,
        "capacity_latency_ms_p50": float(np.percentile(lat_cap, 50)),
        "capacity_latency_ms_p99": float(np.percentile(lat_cap, 99)),
        "poisson": load_lines,
        "sustained": sustained,
        "mean_rays_per_request": float(rays),
        "served_vs_alone_max_abs_diff": worst,
        "server": {"n_streams": n_streams, "max_batch": max_batch,
                   "contexts_per_bucket": contexts_per_bucket, "graphs": use_graphs,
                   "hbm_budget_bytes": 16 << 30, "batches": st["batches"],
                   "graph_launches": st["graph_launches"], "mixed_batches": st["mixed_batches"],
                   "evictions": st["evictions"],
                   "peak_bytes": st["peak_bytes"],
                   "worker_launch_s": st["host_launch_ns"] / 1e9,
                   "worker_capture_s": st["capture_ns"] / 1e9},
        "host_build_s": t_build,
        "timing": "server clock (host steady clock): latency = completion - release per "
                  "request; capacity = requests / makespan with all released at once",
    }


def convolution_section(reps=3):
    """Direct halo-tile convolution against the FP64 FFT convolution, per image,
    on the serving workload's grids and PSF sizes (pixel scale) and on a 4x
    supersampled 300x300 grid (1200x1200, kernels 4 K + 1): CUDA-event time of
    one lensgb_convolve call over a batch (L2 flushed before each), min of
    `reps`, and the FFT result's error against the FP64 direct result."""
    import numpy as np
    import scipy.signal
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import _device, _lib, workloads as W
    lib = _lib.load()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    cases = [(n, k) for n in (60, 180, 300) for k in (11, 21, 41)] + \
            [(1200, 45), (1200, 85), (1200, 165)]
    rows = []
    rng = np.random.default_rng(5)
    for n, K in cases:
        B = 64 if n <= 300 else 4
        img = rng.random((B, n, n)) * np.exp(rng.normal(0, 2, (B, n, n)))
        kern = np.stack([W.moffat_pixel_kernel(0.12 * K / 11, 3.0, 0.05, K)] * B)
        res = {"n": n, "K": K, "batch": B}
        outs = {}
        for prec in ("fp32", "fp64"):
            dt = torch.float32 if prec == "fp32" else torch.float64
            x = torch.as_tensor(img, dtype=dt).cuda().contiguous()
            k = torch.as_tensor(kern, dtype=dt).cuda().contiguous()
            for method in ("direct", "fft"):
                g = W.grid_kwargs(n, 0.05)
                data = J.ImageData(np.zeros((n, n)), exposure_time=1000.0,
                                   background_rms=0.01, **g)
                im = J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                                  J.LensModel(["SIE"]), J.LightModel(["SERSIC"]),
                                  J.LightModel([]),
                                  kwargs_numerics={"supersampling_factor": 1, "precision": prec,
                                                   "convolution_method": method})
                m = im._model(range(1), range(1), range(0))
                out = torch.empty_like(x)
                best = None
                for r in range(reps + 1):
                    flush.zero_()
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    rc = lib.lensgb_convolve(m.handle, _device.ptr(x), B, _device.ptr(k), K * K,
                                             _device.ptr(out), _device.stream_handle())
                    e1.record(stream)
                    torch.cuda.synchronize()
                    if rc != 0:
                        best = None
                        res["%s_%s" % (prec, method)] = "not possible: %s" % \
                            lib.lensgb_last_error().decode()
                        break
                    ms = e0.elapsed_time(e1)
                    if r > 0 and (best is None or ms < best):
                        best = ms
                if best is not None:
                    res["%s_%s_ms_per_image" % (prec, method)] = best / B
                    outs[(prec, method)] = out.double().cpu().numpy()
                m.close()
        ref = outs.get(("fp64", "direct"))
        if ref is None:
            ref = np.stack([scipy.signal.fftconvolve(img[i], kern[i], mode="same")
                            for i in range(2)])
        for prec in ("fp32", "fp64"):
            got = outs.get((prec, "fft"))
            if got is None:
                continue
            nb = ref.shape[0]
            scale = np.abs(ref).reshape(nb, -1).max(axis=1)[:, None, None]
            res["%s_fft_vs_fp64_direct_maxnorm" % prec] = float((np.abs(got[:nb] - ref)
                                                                 / scale).max())
        rows.append(res)
        del outs
    return {"cases": rows,
            "timing": "CUDA events around one lensgb_convolve call of `batch` images (L2 "
                      "flushed before each), min of %d, divided by the batch" % reps,
            "error": "max |fft - fp64 direct| / max |fp64 direct| (fftconvolve on the CPU "
                     "when the FP64 direct kernel cannot run)"}


def serving_accuracy_section(seed=1002, per_bucket=4):
    """FP32-split accuracy of served requests: for each serving bucket (lens
    stack x number of sources), per_bucket requests of the stream -- the first
    re-keyed to the largest case, 300x300 at s = 4 with a 41x41 kernel -- served
    together through the default server (mixed-grid buckets), each image compared
    per pixel with the same request computed in FP64 on the GPU."""
    import numpy as np
    from jaxtronomy_gb300 import serving, workloads as W

    reqs, psfs = W.serving_stream(seed=seed, n=4000)
    picked = []
    for stack in W.SERVING_STACKS:
        for nsrc in (1, 2):
            sel = [dict(r) for r in reqs if r["key"][3] == stack and r["key"][4] == nsrc]
            sel = sel[:per_bucket]
            sel[0]["key"] = (300, 4, 41, stack, nsrc)
            picked += sel
    models = {}
    with serving.Server(n_streams=4, max_batch=64) as srv:
        built = []
        for r in picked:
            if r["key"] not in models:
                models[r["key"]] = W.serving_model(r["key"])
            built.append(srv.request(models[r["key"]], r["kwargs_lens"], r["kwargs_source"],
                                     r["kwargs_lens_light"],
                                     psf_kernel=psfs[r["key"][2]][r["psf"]]))
        tickets = srv.submit_requests(built)
        srv.drain(300)
        served = [t.result().astype(np.float64) for t in tickets]
    buckets = {}
    for r, img in zip(picked, served):
        ref = W.serving_model(r["key"], precision="fp64").image_batch(
            r["kwargs_lens"], r["kwargs_source"], r["kwargs_lens_light"],
            psf_kernels=psfs[r["key"][2]][r["psf"]])[0].cpu().numpy()
        scale = np.abs(ref).max()
        sig = np.abs(ref) >= 1e-3 * scale
        d = np.abs(img - ref)
        per = d[sig] / np.abs(ref)[sig]
        b = buckets.setdefault("%s/%d_sources" % (r["key"][3], r["key"][4]),
                               {"requests": 0, "keys": [], "rel_err_max": 0.0, "_med": [],
                                "maxnorm_err_max": 0.0, "rel_err_max_unfloored": 0.0})
        b["requests"] += 1
        b["keys"].append("%dx%d s%d K%d" % (r["key"][0], r["key"][0], r["key"][1], r["key"][2]))
        b["rel_err_max"] = max(b["rel_err_max"], float(per.max()))
        b["_med"].append(per)
        b["maxnorm_err_max"] = max(b["maxnorm_err_max"], float(d.max() / scale))
        b["rel_err_max_unfloored"] = max(b["rel_err_max_unfloored"],
                                         float((d / np.maximum(np.abs(ref), 1e-300)).max()))
    for b in buckets.values():
        b["rel_err_median"] = float(np.median(np.concatenate(b.pop("_med"))))
    return {"buckets": buckets,
            "rel_err_max": max(b["rel_err_max"] for b in buckets.values()),
            "maxnorm_err_max": max(b["maxnorm_err_max"] for b in buckets.values()),
            "floor": "rel_err: per pixel over pixels >= 1e-3 of the image maximum; maxnorm: "
                     "|served - fp64| / max|fp64| over all pixels; unfloored: per pixel over "
                     "all pixels",
            "reference": "the same request in FP64 on the GPU (equal to the reference's own "
                         "images to 1e-10 on the golden serving scenes)"}


def sampler_section(steps, seed=1003, n_walkers=256, linear_solver=False):
    """Sampler ensemble: LikelihoodModule.logL_batch over n_walkers parameter
    vectors of the gradient workload's system (120^2, s=2, K=21, EPL+SHEAR,
    Sersic source and lens light; 22 sampled parameters, or 20 with the linear
    solver fitting the two amplitudes) -- one batched launch sequence -- against
    the same module called one vector at a time."""
    import numpy as np
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import sampling as S, workloads as W

    N, S2, K = 120, 2, 21
    model_lists = {"lens_model_list": ["EPL", "SHEAR"],
                   "source_light_model_list": ["SERSIC_ELLIPSE"],
                   "lens_light_model_list": ["SERSIC_ELLIPSE"]}
    _, lens, src, ll, kern = W.gradient_batch(seed=seed, batch=1, num_pix=N, supersampling=S2,
                                              kernel_size=K)
    kl, ks, kll = W.instance(lens, 0), W.instance(src, 0), W.instance(ll, 0)
    g = W.grid_kwargs(N, 0.05)
    im = J.ImageModel(J.ImageData(np.zeros((N, N)), exposure_time=1000.0, background_rms=0.01,
                                  **g),
                      J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(model_lists["lens_model_list"]),
                      J.LightModel(model_lists["source_light_model_list"]),
                      J.LightModel(model_lists["lens_light_model_list"]),
                      kwargs_numerics={"supersampling_factor": S2})
    data = W.noisy_data(im.image(kl, ks, kll))
    joint = {"multi_band_list": [[{"image_data": data, "background_rms": 0.01,
                                   "exposure_time": 1000.0, **g},
                                  {"psf_type": "PIXEL", "kernel_point_source": kern[0]},
                                  {"supersampling_factor": S2}]],
             "multi_band_type": "single-band"}
    param = S.Param(model_lists, kwargs_fixed_lens=[{}, {"ra_0": 0.0, "dec_0": 0.0}],
                    linear_solver=linear_solver)
    lm = S.LikelihoodModule(joint, model_lists, param)
    f = S.prepare_logL_func("gpu", lm.logL)
    truth = param.kwargs2args(kl, ks, kll)
    args = truth + 1e-3 * np.random.default_rng(seed).standard_normal((n_walkers, truth.size))
    for _ in range(3):
        f(args)
    t = []
    for _ in range(max(steps, 3)):
        t0 = time.perf_counter()
        f(args)
        t.append(time.perf_counter() - t0)
    batched = statistics.median(t)
    n1 = 16
    for j in range(3):
        lm.logL(args[j])
    t0 = time.perf_counter()
    for j in range(n1):
        lm.logL(args[j])
    single = (time.perf_counter() - t0) / n1
    return {
        "workload": "sampler_ensemble_epl_120x120_s2_psf21" + ("_linear_solve" if linear_solver
                                                                  else ""),
        "walkers": n_walkers, "sampled_params": int(truth.size),
        "ms_per_ensemble": batched * 1e3, "evaluations_per_s": n_walkers / batched,
        "one_vector_per_call_ms": single * 1e3, "one_vector_per_call_evaluations_per_s": 1.0 / single,
        "speedup": single * n_walkers / batched,
        "precision": "FP64 image and likelihood",
        "timing": "host wall clock of prepare_logL_func('gpu', LikelihoodModule.logL) on an "
                  "(n_walkers, 22) host array, result back on the host; median over calls",
    }


def gradient_section(steps, seed=1003, peaks=None):
    """Adjoint gradient of logL for 256 systems (120^2, s=2, PSF 21, EPL+SHEAR,
    Sersic source and lens light): time per batch, and the worst component
    error against central finite differences (step 1e-6) on a sample; then the
    same batch with FP32 per-ray derivatives (gradient_precision "fp32"), its
    time and its error against the FP64 adjoint."""
    import numpy as np
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import workloads as W

    B, N, S, K = 256, 120, 2, 21
    model, lens, src, ll, kern = W.gradient_batch(seed=seed, batch=B, num_pix=N,
                                                  supersampling=S, kernel_size=K)
    g = W.grid_kwargs(N, 0.05)
    data_cls = J.ImageData(np.zeros((N, N)), exposure_time=1000.0, background_rms=0.01, **g)
    im = J.ImageModel(data_cls, J.PSF("PIXEL", kernel_point_source=kern[0]),
                      J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                      J.LightModel(["SERSIC_ELLIPSE"]),
                      kwargs_numerics={"supersampling_factor": S, "precision": "fp64"})
    rows = im.pack_params(lens, src, ll)
    truth = rows.copy()
    truth[:, 0] *= 1.01
    data = W.noisy_data(im.image_batch(rows=truth, psf_kernels=kern).cpu().numpy())
    rows_d = torch.as_tensor(rows).cuda()
    data_d = torch.as_tensor(data).cuda()
    kern_d = torch.as_tensor(kern).cuda()
    for _ in range(2):
        im.likelihood_grad_batch(rows=rows_d, data=data_d, psf_kernels=kern_d)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n = max(steps, 3)
    e0.record(stream)
    for _ in range(n):
        logl, grad = im.likelihood_grad_batch(rows=rows_d, data=data_d, psf_kernels=kern_d)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n
    e0.record(stream)
    for _ in range(n):
        im.likelihood_batch(rows=rows_d, data=data_d, psf_kernels=kern_d)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_fwd = e0.elapsed_time(e1) / n
    # central differences on a sample of systems, all perturbations in one batch
    idx = np.array([0, 77, 191])
    P = rows.shape[1]
    pert = np.repeat(rows[idx][:, None, :], 2 * P, axis=1)
    for k in range(P):
        pert[:, 2 * k, k] += 1e-6
        pert[:, 2 * k + 1, k] -= 1e-6
    pert = pert.reshape(-1, P)
    lp = im.likelihood_batch(rows=pert, data=np.repeat(data[idx], 2 * P, axis=0),
                             psf_kernels=np.repeat(kern[idx], 2 * P, axis=0)).cpu().numpy()
    lp = lp.reshape(len(idx), P, 2)
    fd = (lp[..., 0] - lp[..., 1]) / 2e-6
    gs = grad.cpu().numpy()[idx]
    scale = np.abs(fd).max(axis=1, keepdims=True)
    sig = np.abs(fd) > 1e-3 * scale
    rel = np.abs(gs - fd)[sig] / np.abs(fd)[sig]
    # FP32 per-ray derivatives, flagged pixels recomputed in FP64
    im32 = J.ImageModel(data_cls, J.PSF("PIXEL", kernel_point_source=kern[0]),
                        J.LensModel(["EPL", "SHEAR"]), J.LightModel(["SERSIC_ELLIPSE"]),
                        J.LightModel(["SERSIC_ELLIPSE"]),
                        kwargs_numerics={"supersampling_factor": S, "precision": "fp64",
                                         "gradient_precision": "fp32"})
    for _ in range(2):
        im32.likelihood_grad_batch(rows=rows_d, data=data_d, psf_kernels=kern_d)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(n):
        logl32, grad32 = im32.likelihood_grad_batch(rows=rows_d, data=data_d, psf_kernels=kern_d)
    e1.record(stream)
    torch.cuda.synchronize()
    ms32 = e0.elapsed_time(e1) / n
    g64, g32 = grad.cpu().numpy(), grad32.cpu().numpy()
    floor = 1e-3 * np.abs(g64).max(axis=1, keepdims=True)
    rel32 = np.abs(g32 - g64) / (np.abs(g64) + floor)
    return {
        "workload": "gradient_epl_256x120x120_s2_psf21",
        "systems": B, "params_per_system": P,
        "ms_per_batch": ms, "systems_per_s": B / (ms / 1e3),
        "forward_loglike_ms_per_batch": ms_fwd, "grad_over_forward": ms / ms_fwd,
        "fd_rel_err_max": float(rel.max()), "fd_rel_err_median": float(np.median(rel)),
        "fd_components_checked": int(sig.sum()),
        "precision": "FP64 (forward image, adjoint and reduction)",
        "roofline": grad_roofline(B, N, S, K, P, ms, peaks, "fp64"),
        "timing": "CUDA events, mean over %d batches after 2 warm-ups" % n,
        "fp32_adjoint": {
            "ms_per_batch": ms32, "systems_per_s": B / (ms32 / 1e3),
            "speedup_over_fp64_adjoint": ms / ms32,
            "rel_err_vs_fp64_adjoint_max": float(rel32.max()),
            "rel_err_vs_fp64_adjoint_median": float(np.median(rel32)),
            "logL_bits_equal": bool(torch.equal(logl32, logl)),
            "err_floor": "per component over |fp64| + 1e-3 of the system's largest component",
            "precision": "FP32 dual numbers from FP64 offsets; pixels whose predicted FP32 "
                         "derivative error exceeds 1e-5 recomputed in FP64; forward image, "
                         "weights and reduction FP64",
            "roofline": grad_roofline(B, N, S, K, P, ms32, peaks, "fp32"),
        },
    }


def grad_roofline(B, N, S, K, P, ms, peaks=None, kind="fp64"):
    """Algorithmic work of one adjoint batch: every ray's EPL + SHEAR + two
    Sersic evaluation (~220 flop) carried with 5 tangent directions (~6x), plus
    the per-parameter accumulation (2 P flop per ray); the forward image and
    likelihood (ray work + 2 K^2 per pixel), and the transposed convolution
    (2 K^2 per pixel).  Peak: the FMA rate of the dominant kernel's arithmetic
    (FP64, or FP32 for FP32 per-ray derivatives), measured in this run by the
    FMA-chain kernel when available, else nominal."""
    rays = B * (N * S) ** 2
    flop = rays * (220 * 6 + 2 * P) + rays * 220 + 2 * (2 * K * K) * B * N * N
    key = "fp64_tflops" if kind == "fp64" else "fp32_tflops"
    if peaks and peaks.get(key):
        peak, src = peaks[key], "measured %s FMA rate of this device (fma_peaks, of measured)" \
            % kind.upper()
    else:
        peak = 1.25 if kind == "fp64" else 78.3
        src = "nominal %s rate (no FMA measurement in this run)" % kind.upper()
    achieved = flop / (ms / 1e3) / 1e12
    return {"kernel": "grad_ray_kernel (+ forward image, weights, transposed conv)",
            "bound": kind, "unit": "TFLOP/s", "algorithmic_gflop_per_batch": flop / 1e9,
            "achieved": achieved, "peak": peak, "frac": achieved / peak,
            "peak_source": src}


def max_over_ranks(ms, dist=None, device="cpu"):
    """Step time of the whole job: the maximum of the ranks' mean step times
    (an all-reduce of one float; nothing on the data path)."""
    if dist is None:
        return float(ms)
    import torch
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, world, ms):
    """Whole-job throughput: every rank processes units_per_rank per step
    (weak scaling), the job's step time is the slowest rank's."""
    return units_per_rank * world / (ms / 1e3)


def rank_seed(base, rank):
    """Each replica simulates its own seeded batch."""
    return base + rank


def percentile(v, q):
    v = sorted(v)
    k = (len(v) - 1) * q
    lo, hi = int(k), min(int(k) + 1, len(v) - 1)
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def gpu_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    cores = cpu_cores()
    pool = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # spawn the oracle pool before the first CUDA call
        pool = _spawn_pool(cores)

    import numpy as np
    import torch
    import jaxtronomy_gb300 as J
    from jaxtronomy_gb300 import _lib, workloads as W

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    B = args.batch
    model, lens, src, ll, kern = W.batch_epl(seed=rank_seed(1001, rank), batch=B, num_pix=N_PIX,
                                             delta_pix=DPIX, supersampling=SS, kernel_size=KSIZE)
    g = W.grid_kwargs(N_PIX, DPIX)

    def make(precision):
        data = J.ImageData(np.zeros((N_PIX, N_PIX)), exposure_time=1000.0, background_rms=0.01,
                           **g)
        return J.ImageModel(data, J.PSF("PIXEL", kernel_point_source=kern[0]),
                            J.LensModel(model["lens_model_list"]),
                            J.LightModel(model["source_light_model_list"]),
                            J.LightModel(model["lens_light_model_list"]),
                            kwargs_numerics={"supersampling_factor": SS, "precision": precision})

    im32 = make("fp32")
    im64 = make("fp64")
    rows_host = im32.pack_params(lens, src, ll)
    rows_dev = torch.as_tensor(rows_host).cuda()
    psf32 = torch.as_tensor(kern, dtype=torch.float32).cuda().contiguous()
    psf64 = torch.as_tensor(kern, dtype=torch.float64).cuda().contiguous()
    out32 = torch.empty((B, N_PIX, N_PIX), dtype=torch.float32, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step():
        im32.image_batch(rows=rows_dev, psf_kernels=psf32, out=out32)

    # launch shapes from the autotuner (timed on this workload before the run)
    tune = im32.autotune(rows=rows_dev, psf_kernels=psf32)
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier()
    t_wall = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()  # evict L2 between timed steps (outside the step events)
        starts[k].record(stream)
        step()
        ends[k].record(stream)
    barrier()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = statistics.mean(step_ms)
    ms = max_over_ranks(ms, dist, "cuda")
    value = job_rate(B, world, ms)

    extra = {}
    if rank == 0:
        # --- FP32 vs FP64 over the whole batch (FP64 batched, outside timing)
        out64 = im64.image_batch(rows=rows_dev, psf_kernels=psf64)
        a = out32.double()
        b = out64
        scale = b.abs().amax(dim=(1, 2), keepdim=True)
        sig = b.abs() >= 1e-3 * scale
        rel = ((a - b).abs() / b.abs().clamp_min(1e-300))[sig]
        extra["fp32_vs_fp64_rel_err_max"] = float(rel.max())
        extra["fp32_vs_fp64_rel_err_median"] = float(rel.median())
        extra["fp32_vs_fp64_maxnorm_err_max"] = float(((a - b).abs() / scale).amax())
        # per pixel with no floor, over the whole batch (pixels of order 1e-30 of
        # the maximum, far in a profile's wing, carry most of this figure)
        rel_all = (a - b).abs() / b.abs().clamp_min(1e-300)
        extra["fp32_vs_fp64_rel_err_max_unfloored"] = float(rel_all.max())
        extra["fp32_vs_fp64_rel_err_median_unfloored"] = float(rel_all.median())
        extra["fp32_vs_fp64_floor"] = ("rel_err_max / _median: per pixel over pixels >= 1e-3 "
                                       "of each image's maximum; maxnorm: |m - o| / max|o| over "
                                       "all pixels; unfloored: per pixel over all pixels")
        del rel_all
        # --- FP64 and FP32 against the oracle (max and median per pixel, no floor)
        import warnings
        warnings.simplefilter("ignore")
        from oracle import image as oimage
        e64, e32 = [], []
        n_or = args.oracle_systems
        for i in range(n_or):
            scene = dict(nx=N_PIX, ny=N_PIX, supersampling_factor=SS, psf_type="PIXEL",
                         kernel=kern[i], lens_model_list=model["lens_model_list"],
                         source_light_model_list=model["source_light_model_list"],
                         lens_light_model_list=model["lens_light_model_list"], **g)
            ref = oimage.image(scene, W.instance(lens, i), W.instance(src, i), W.instance(ll, i))
            e64.append(np.abs(out64[i].cpu().numpy() - ref) / np.abs(ref))
            e32.append(np.abs(out32[i].double().cpu().numpy() - ref) / np.abs(ref))
        e64, e32 = np.concatenate([e.ravel() for e in e64]), np.concatenate([e.ravel() for e in e32])
        extra["fp64_vs_oracle_rel_err_max"] = float(e64.max())
        extra["fp64_vs_oracle_rel_err_median"] = float(np.median(e64))
        extra["fp32_vs_oracle_rel_err_max"] = float(e32.max())
        extra["fp32_vs_oracle_rel_err_median"] = float(np.median(e32))
        extra["oracle_systems"] = n_or

        # --- plain FP64, one request per launch
        n_plain = args.plain_sample
        e0 = [torch.cuda.Event(enable_timing=True) for _ in range(n_plain)]
        e1 = [torch.cuda.Event(enable_timing=True) for _ in range(n_plain)]
        one64 = torch.empty((1, N_PIX, N_PIX), dtype=torch.float64, device="cuda")
        im64.image_batch(rows=rows_dev[:1], psf_kernels=psf64[0], out=one64)
        torch.cuda.synchronize()
        for i in range(n_plain):
            e0[i].record(stream)
            im64.image_batch(rows=rows_dev[i:i + 1], psf_kernels=psf64[i], out=one64)
            e1[i].record(stream)
        torch.cuda.synchronize()
        plain_ms = [a.elapsed_time(b) for a, b in zip(e0, e1)]
        plain_ips = 1e3 / statistics.mean(plain_ms)
        extra["fp64_plain_images_per_s"] = plain_ips
        extra["fp64_plain_latency_ms_p50"] = percentile(plain_ms, 0.5)
        extra["fp64_plain_latency_ms_p99"] = percentile(plain_ms, 0.99)
        extra["fp64_plain_launch"] = ("one system per call; FP64 ray kernel with one thread per "
                                      "supersampled ray (%d CTAs of 256 threads), convolution in "
                                      "8 x 16 tiles" % ((N_PIX * N_PIX + 256 // (SS * SS) - 1)
                                                        // (256 // (SS * SS))))
        extra["speedup_vs_fp64_plain"] = value / world / plain_ips
        # --- batched FP64 (the whole workload in one FP64 launch sequence)
        b64 = []
        for _ in range(3):
            flush.zero_()
            q0 = torch.cuda.Event(enable_timing=True)
            q1 = torch.cuda.Event(enable_timing=True)
            q0.record(stream)
            im64.image_batch(rows=rows_dev, psf_kernels=psf64, out=out64)
            q1.record(stream)
            torch.cuda.synchronize()
            b64.append(q0.elapsed_time(q1))
        b64_ips = B / (statistics.mean(b64[1:]) / 1e3)
        extra["fp64_batched_images_per_s"] = b64_ips
        extra["fp64_batched_ms_per_step"] = statistics.mean(b64[1:])
        extra["speedup_vs_fp64_batched"] = value / world / b64_ips
        extra["fp64_plain_over_batched_per_image"] = b64_ips / plain_ips

        # --- FP32 single-request latency (one system per launch)
        n1 = args.plain_sample * 2
        one32 = torch.empty((1, N_PIX, N_PIX), dtype=torch.float32, device="cuda")
        lat = []
        for i in range(n1):
            s0 = torch.cuda.Event(enable_timing=True)
            s1 = torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            im32.image_batch(rows=rows_dev[i:i + 1], psf_kernels=psf32[i], out=one32)
            s1.record(stream)
            s1.synchronize()
            lat.append(s0.elapsed_time(s1))
        extra["autotune"] = tune
        extra["fp32_single_request_latency_ms_p50"] = percentile(lat, 0.5)
        extra["fp32_single_request_latency_ms_p99"] = percentile(lat, 0.99)

        # --- stage timing for the roofline (L2 flushed before each rep)
        low = torch.empty_like(out32)
        lib = _lib.load()
        from jaxtronomy_gb300 import _device
        m32 = im32._model(range(2), range(1), range(1))
        reps = 5
        rt_ms, cv_ms = [], []
        for _ in range(reps):
            flush.zero_()
            a0 = torch.cuda.Event(enable_timing=True)
            a1 = torch.cuda.Event(enable_timing=True)
            a0.record(stream)
            im32.image_batch(rows=rows_dev, psf_kernels=psf32, out=low, unconvolved=True)
            a1.record(stream)
            flush.zero_()
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            _lib.check(lib.lensgb_convolve(m32.handle, _device.ptr(low), B, _device.ptr(psf32),
                                           KSIZE * KSIZE, _device.ptr(out32),
                                           _device.stream_handle()))
            c1.record(stream)
            torch.cuda.synchronize()
            rt_ms.append(a0.elapsed_time(a1))
            cv_ms.append(c0.elapsed_time(c1))
        nm = epl_nmax(lens[0]["e1"], lens[0]["e2"])
        n32 = epl_fp32_series_length(lens)
        flop_ray, t_ray = ray_work(lens, B, nm)
        flop_ray_exec, _ = ray_work(lens, B, n32)
        flop_conv = 2 * KSIZE * KSIZE * N_PIX * N_PIX * B
        rt = statistics.mean(rt_ms) / 1e3
        cv = statistics.mean(cv_ms) / 1e3
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        sm_mhz = clk.get("sm_mhz") or 2070.0
        fp32_nominal = sms * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s at the sampled clock
        peaks = fma_peaks()
        fp32_peak = peaks["fp32_tflops"]
        extra["fma_peaks"] = dict(peaks, source="measured in this run: lensgb_fma_chain "
                                  "(project FMA-chain kernel), best of 5 CUDA-event-timed "
                                  "launches; nominal FP32 at the sampled clock %.1f TFLOP/s"
                                  % fp32_nominal)
        extra["roofline"] = {
            "kernel": "raytrace_fp32_kernel (with prepare_kernel and refine_kernel)",
            "bound": "fp32", "unit": "TFLOP/s",
            "achieved": flop_ray / rt / 1e12, "peak": fp32_peak,
            "frac": flop_ray / rt / 1e12 / fp32_peak,
            "peak_source": "measured FP32 FMA rate of this device (fma_peaks, of measured)",
            "frac_of_nominal": flop_ray / rt / 1e12 / fp32_nominal,
            "algorithmic_gflop_per_launch": flop_ray / 1e9,
            "count": "reference formulas, EPL 60 + 8 nmax flop per ray at the reference's "
                     "nmax(f) (mean %.1f terms)" % (sum(nm) / len(nm)),
            "executed_gflop_per_launch": flop_ray_exec / 1e9,
            "executed_frac": flop_ray_exec / rt / 1e12 / fp32_peak,
            "executed_count": "as above with the FP32 kernel's shortened series (mean %.2f "
                              "terms per ray)" % (sum(n32) / len(n32)),
            "epl_series_terms_mean_reference": sum(nm) / len(nm),
            "epl_series_terms_mean_fp32": sum(n32) / len(n32),
            "transcendentals_per_s": t_ray / rt, "launch_ms": rt * 1e3,
            # DRAM bytes per 1024-system launch (read + write) of raytrace_fp32_kernel plus
            # refine_kernel: 0.83 + 74.0 MB and 0.75 + 0 MB.  Below the algorithmic
            # 132.7 MB image write because the image tail is still in L2 when the kernel ends.
            "traffic": 75.6e6 if B == 1024 else None,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one capture "
                              "of this workload (profiles/dram_traffic_raytrace_refine_conv_"
                              "batch_epl_180x180_s3_psf31.md), not measured in this run",
            "algorithmic_bytes_per_launch": B * N_PIX * N_PIX * 4 + rows_host.nbytes,
        }
        hbm_peak = 6784.5
        try:
            with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
                hbm_peak = float(json.load(f)["hbm_gbs"])
        except Exception:
            pass
        conv_bytes = B * N_PIX * N_PIX * 4 * 2 + B * KSIZE * KSIZE * 4
        extra["roofline_conv"] = {
            "kernel": "conv_f32_tma_kernel (TMA-staged halo tile, K <= 48: compile-time width)", "bound": "fp32", "unit": "TFLOP/s",
            "achieved": flop_conv / cv / 1e12, "peak": fp32_peak,
            "frac": flop_conv / cv / 1e12 / fp32_peak, "launch_ms": cv * 1e3,
            "peak_source": "measured FP32 FMA rate of this device (fma_peaks, of measured)",
            "frac_of_nominal": flop_conv / cv / 1e12 / fp32_nominal,
            "hbm_gbs": conv_bytes / cv / 1e9, "hbm_frac_of_measured": conv_bytes / cv / 1e9 / hbm_peak,
            # 136.7 MB read + 83.8 MB written per launch
            "traffic": 220.5e6 if B == 1024 else None,
            "traffic_source": "ncu capture of this workload (profiles/dram_traffic_raytrace_"
                              "refine_conv_batch_epl_180x180_s3_psf31.md), not measured in this "
                              "run",
            "algorithmic_bytes_per_launch": conv_bytes,
        }

        # --- end to end through the public API with host buffers
        rows_pin = torch.as_tensor(rows_host).pin_memory()
        psf_pin = torch.as_tensor(kern, dtype=torch.float32).pin_memory()
        out_pin = torch.empty((B, N_PIX, N_PIX), dtype=torch.float32).pin_memory()

        def e2e_step():
            # host rows / PSFs in, host images out: lensgb_image_host copies each
            # chunk's images back while the next chunk is computed
            im32.image_batch(rows=rows_pin, psf_kernels=psf_pin, out=out_pin)

        for _ in range(2):
            e2e_step()
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        im32.host_wait()  # the timed region ends after the last step's image copies
        f1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = f0.elapsed_time(f1) / args.steps
        h2d = rows_pin.numel() * 8 + psf_pin.numel() * 4
        d2h = out_pin.numel() * 4
        extra["e2e"] = {"value": B / (e2e_ms / 1e3), "unit": "images/s",
                        "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "ms_per_step": e2e_ms,
                        "path": "ImageModel.image_batch with pinned host rows / PSFs / output "
                                "-> lensgb_image_host (H2D and compute on the launch stream; "
                                "each step's D2H on a second stream, overlapping the next "
                                "step; the timed region ends after the last D2H)"}

        # --- direct vs FFT convolution
        if args.conv_table:
            extra["convolution"] = convolution_section()

        # --- plain single image (60x60, SIE+SHEAR, s=1, 11x11)
        extra["single_image"] = single_image_section()

        # --- substructure ray shooting (LensModelBulk, FP32 subhalo terms)
        if not args.no_sub:
            extra["substructure"] = substructure_section(args.steps, args.warmup, fp32_peak,
                                                         flush)
            extra["multi_plane"] = multi_plane_section(args.steps, args.warmup, fp32_peak,
                                                       flush)

        # --- adjoint likelihood gradient
        if not args.no_grad:
            extra["gradient"] = gradient_section(args.steps, peaks=peaks)
            extra["sampler"] = sampler_section(args.steps)
            extra["sampler_linear_solve"] = sampler_section(args.steps, linear_solver=True)

        # --- serving stream (continuous batching)
        if args.serve_requests > 0:
            extra["serving_accuracy"] = serving_accuracy_section()
            extra["serving"] = serving_section(args.serve_requests)
            extra["serving_grid_buckets"] = serving_section(args.serve_requests, mixed_grids=1)
            extra["serving_exact_buckets"] = serving_section(args.serve_requests,
                                                             mixed_grids=False)

        # --- CPU baseline (oracle port, bounded sample)
        if pool is not None:
            n_img = 4 * cores
            sec = run_cpu_sample(pool, cores, n_img)
            extra["cpu_baseline"] = {
                "value": n_img / sec, "unit": "images/s", "cores": cores, "kind": "port",
                "sample": "%d systems of the workload, FP64 NumPy oracle, spawn pool of %d "
                          "workers" % (n_img, cores), "cpu": cpu_model()}
            pool.close()

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "images/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch_per_gpu": B, "grid": N_PIX,
                       "delta_pix": DPIX, "supersampling": SS, "psf": KSIZE,
                       "lens": "EPL+SHEAR", "light": "SERSIC_ELLIPSE source + lens light",
                       "precision": "FP32 bulk, FP64 set-up / offsets / reductions",
                       "l2": "flushed between timed steps by a 512 MiB memset outside the "
                             "per-step CUDA events",
                       "timing": "per-step CUDA events on the launch stream, mean over steps, "
                                 "max over ranks"},
            "latency_ms_p50": percentile(step_ms, 0.5), "latency_ms_p99": percentile(step_ms, 0.99),
            "wall_s_timed_region": t_wall,
            "gpu_launches": 4 * args.steps,
            "clocks": clk,
        }
        line.update(extra)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def _free_port():
    import socket
    sk = socket.socket()
    sk.bind(("127.0.0.1", 0))
    port = sk.getsockname()[1]
    sk.close()
    return port


def _replica_entry(local_rank, world, port, worker, wargs):
    os.environ.update(RANK=str(local_rank), LOCAL_RANK=str(local_rank), WORLD_SIZE=str(world),
                      LOCAL_WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    rc = worker(*wargs)
    if rc:
        raise SystemExit(rc)


def launch_replicas(world, worker, *wargs):
    """Runs worker(*wargs) in `world` spawned processes, one per GPU, with the
    environment torchrun would give them (RANK, LOCAL_RANK, WORLD_SIZE,
    MASTER_ADDR 127.0.0.1, a free MASTER_PORT): `python bench.py --gpus N`
    without torchrun.  Each replica simulates its own seeded batch; the process
    group serves only the barrier and the max-over-ranks step time."""
    import torch.multiprocessing as tmp
    tmp.start_processes(_replica_entry, args=(world, _free_port(), worker, wargs), nprocs=world,
                        join=True, start_method="spawn")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--plain-sample", type=int, default=16)
    ap.add_argument("--oracle-systems", type=int, default=8)
    ap.add_argument("--no-conv-table", dest="conv_table", action="store_false")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-sub", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=50000)
    args = ap.parse_args()
    if args.impl == "reference":
        return reference_arm(args)
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return launch_replicas(args.gpus, gpu_arm, args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())
