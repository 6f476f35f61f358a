#!/usr/bin/env python
"""Throughput/latency benchmark of the Shack-Hartmann WFS step.

Workload (one GPU): the 74x74-subaperture ELT NGS sensor -- 39 m pupil with
0.28 central obstruction (3972 lit subapertures), phasesize 10, fftsize 20,
clipsize 20, nimg 10, 2-D Gaussian spot PSF of FWHM 1.5 FFT pixels, 500
photons/subaperture, Poisson shot noise, 3 e- read noise, sky 10 e-/px,
threshold 6 (2 sigma) -- on seeded synthetic von Karman phase screens
(r0 0.157 m at 500 nm, L0 25 m, lambda 589 nm, 740x740 px).

A step is one batch of F independent frames through the fused kernel with
the phase already in HBM (``value``).  ``e2e`` is the same metric through the
reference-facing call (``centcmod.run`` -> ``shwfs_run``) with host phase and
host outputs, one synchronous frame at a time, which also gives the per-frame
latency percentiles.  ``--impl reference`` times the reference's own
centmodule (cmod/src/centmodule.c, built unmodified into oracle/_ref with
FFT/GSL shims) on all host cores, through its own initialise/run calls.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

WORKLOAD = dict(name="elt74x74_ngs_psf_noisy", nsubx=74, p=10, N=20, C=20, m=10, ncen=10, obs=0.28, Dtel=39.0,
                r0=0.157, L0=25.0, wavelength=589.0, psf_fwhm=1.5, sig=500.0, addPoisson=1, readnoise=3.0,
                readbg=0.0, sky=10.0, floor=6.0, threshType=0)
METRIC = "SH WFS subap-frames/s (74x74 NGS, fftsize 20, Gaussian spot PSF, Poisson+read noise)"
UNIT = "subap-frames/s"
FPSTEP = 64  # frames per step


# ---------------------------------------------------------------- inputs

def make_pupil():
    from dasp_gb300.tel import Pupil
    w = WORKLOAD
    npup = w["nsubx"] * w["p"]
    return Pupil(npup, npup / 2.0, npup / 2.0 * w["obs"])


def make_screens(n, seed0=1000):
    from dasp_gb300.screens import von_karman_screen
    w = WORKLOAD
    npup = w["nsubx"] * w["p"]
    return [von_karman_screen(npup, w["Dtel"], w["r0"], w["L0"], seed0 + s, w["wavelength"]) for s in range(n)]


def make_frames(screens, nframes, seed):
    """nframes distinct frames from a few screens: flips, transposes, rolls."""
    rng = np.random.default_rng(seed)
    out = np.empty((nframes,) + screens[0].shape, np.float32)
    for f in range(nframes):
        s = screens[f % len(screens)]
        if rng.random() < 0.5:
            s = s[::-1]
        if rng.random() < 0.5:
            s = s.T
        out[f] = np.roll(s, (int(rng.integers(0, 740)), int(rng.integers(0, 740))), axis=(0, 1))
    return out


def make_engine(pup, phs, cents, bimg, noiseless=False):
    from dasp_gb300.centcmod import centcmod
    from dasp_gb300.screens import gaussian_psf
    w = WORKLOAD
    psf = gaussian_psf(w["C"], w["psf_fwhm"])
    return centcmod(8, w["nsubx"], w["ncen"], w["N"], w["C"], w["m"], w["p"],
                    0.0 if noiseless else w["readnoise"], w["readbg"], 0 if noiseless else w["addPoisson"],
                    w["floor"], w["sig"], w["sky"], 0, 1.0, 1, 0, 1234, phs, pup, psf, cents, bimg, 0.5, 0, None,
                    0, 0.0, None, None, w["threshType"], 0, 0, 1, 0, None)


# ---------------------------------------------------------------- algorithmic work

# DRAM bytes (read + write) per launch of the 64-frame step, from one ncu
# capture of each kernel (commands and figures in profiles/)
NCU_TRAFFIC = {"wfs_gemm_kernel": 161.5e6, "wfs_post_warp_kernel": 149.3e6}


def tensor_flops_per_subap():
    """Algorithmic tensor-core flops of one GEMM-DFT pass per lit subap-frame:
    2 (2c^2)(2p^2) for the cropped DFT plus 2 m^2 c^2 for the convolve+bin map
    (no padding counted)."""
    w = WORKLOAD
    c, p, m = w["N"], w["p"], w["m"]
    return float(2 * (2 * c * c) * (2 * p * p) + 2 * m * m * c * c)


def algorithmic_per_subap():
    """Per lit subap-frame: flops (F_alg) and bytes (B_alg).

    F_alg = 6p^2 + 10 N^2 log2 N + 3c^2 + [10 P^2 log2 P + 6 P (P/2+1)] + C^2 + 3 m^2
    B_alg = 4p^2 (phase in) + 4m^2 (image out) + 8 (centroids out)
    """
    w = WORKLOAD
    p, N, C, m, P = w["p"], w["N"], w["C"], w["m"], w["C"]
    c = min(N, P)
    F = 6 * p * p + 10 * N * N * np.log2(N) + 3 * c * c + 10 * P * P * np.log2(P) + 6 * P * (P // 2 + 1) \
        + C * C + 3 * m * m
    B = 4 * p * p + 4 * m * m + 8
    return float(F), float(B)


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- distributed

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def reduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU baseline

def cpu_sample(frames, nthreads=1, seed=0):
    """Time the CPU restatement of the path (the oracle) on ``frames`` frames."""
    from oracle.shwfs_oracle import CentOracle
    from dasp_gb300.screens import gaussian_psf
    w = WORKLOAD
    pup = make_pupil()
    nsx, p = w["nsubx"], w["p"]
    orc = CentOracle(nsubx=nsx, phasesize=p, fftsize=w["N"], clipsize=w["C"], nimg=w["m"], ncen=w["ncen"],
                     pupfn=pup.perSubap(nsx, 0), subflag=pup.getSubapFlag(nsx, 0.5),
                     fracSubArea=(pup.getSubarea(nsx) / (p * p)).astype(np.float32), sig=w["sig"],
                     readnoise=w["readnoise"], readbg=w["readbg"], addPoisson=w["addPoisson"],
                     noiseFloor=w["floor"], skybrightness=w["sky"], seed=1234 + seed, nthreads=nthreads,
                     spotpsf=gaussian_psf(w["C"], w["psf_fwhm"]), threshType=w["threshType"])
    screens = make_screens(2, 5000 + seed)
    cents = np.zeros(nsx * nsx * 2, np.float32)
    bimg = np.zeros((nsx * nsx, w["m"], w["m"]), np.float32)
    t0 = time.perf_counter()
    for f in range(frames):
        orc.run(screens[f % 2], cents, bimg)
    return time.perf_counter() - t0, int(orc.subflag.sum())


def _cpu_worker(args):
    frames, seed = args
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    dt, nlit = cpu_sample(frames, 1, seed)
    return dt, nlit, frames


def cpu_parallel(frames_per_worker, workers):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(workers) as pool:
        t0 = time.perf_counter()
        res = pool.map(_cpu_worker, [(frames_per_worker, i) for i in range(workers)])
        wall = time.perf_counter() - t0
    nlit = res[0][1]
    total = sum(r[2] for r in res)
    return wall, nlit, total


def accuracy_vs_fp64(eng_cents, phs):
    """Noiseless centroid error of the engine vs the float64 oracle (px)."""
    from oracle.shwfs_oracle import CentOracle
    from dasp_gb300.screens import gaussian_psf
    w = WORKLOAD
    pup = make_pupil()
    nsx, p = w["nsubx"], w["p"]
    orc = CentOracle(nsubx=nsx, phasesize=p, fftsize=w["N"], clipsize=w["C"], nimg=w["m"], ncen=w["ncen"],
                     pupfn=pup.perSubap(nsx, 0), subflag=pup.getSubapFlag(nsx, 0.5),
                     fracSubArea=(pup.getSubarea(nsx) / (p * p)).astype(np.float32), sig=w["sig"],
                     noiseFloor=w["floor"], skybrightness=w["sky"], spotpsf=gaussian_psf(w["C"], w["psf_fwhm"]),
                     threshType=w["threshType"], mode="f64")
    cents = np.zeros(nsx * nsx * 2, np.float32)
    bimg = np.zeros((nsx * nsx, w["m"], w["m"]), np.float32)
    orc.run(phs, cents, bimg)
    return float(np.abs(cents - eng_cents.reshape(-1)).max())


# ---------------------------------------------------------------- reference arm

def host_cores() -> int:
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)


class RefTimer:
    """The reference's own module (oracle/_ref: the unmodified
    cmod/src/centmodule.c, FFT/GSL shims) on the bench workload, driven
    through its own initialise/run entry points with ``nthreads`` worker
    threads.  Frames are written into the module's borrowed phase array
    between calls (as the simulation writes its phase in place) outside the
    timed region; each frame is timed around ``cent.run`` (wall clock) and by
    the module's own timer (py_run's elapsed seconds, centmodule.c:3203-3228)."""

    def __init__(self, nthreads, frames):
        from oracle.ref_cent import RefCent
        from dasp_gb300.screens import gaussian_psf
        w = WORKLOAD
        self.frames = frames
        self.phs = np.ascontiguousarray(frames[0]).copy()
        self.cents = np.zeros(w["nsubx"] ** 2 * 2, np.float32)
        self.bimg = np.zeros((w["nsubx"], w["nsubx"], w["m"], w["m"]), np.float32)
        pup = make_pupil()
        self.ref = RefCent(nthreads, w["nsubx"], w["ncen"], w["N"], w["C"], w["m"], w["p"], w["readnoise"],
                           w["readbg"], w["addPoisson"], w["floor"], w["sig"], w["sky"], 0, 1.0, 1, 0, 1234,
                           self.phs, pup, gaussian_psf(w["C"], w["psf_fwhm"]), self.cents, self.bimg, 0.5, 0, None,
                           0, 0.0, None, None, w["threshType"], 0, 0, 1, 0, None)
        self.nlit = int(pup.getSubapFlag(w["nsubx"], 0.5).sum())
        self.k = 0

    def step(self, nframes):
        """nframes frames; returns (wall seconds inside run, py_run seconds)."""
        wall = own = 0.0
        for _ in range(nframes):
            np.copyto(self.phs, self.frames[self.k % len(self.frames)])
            self.k += 1
            t0 = time.perf_counter()
            own += self.ref.run(0)
            wall += time.perf_counter() - t0
        return wall, own

    def free(self):
        self.ref.free()


def reference_available():
    try:
        from oracle import ref_cent
        ref_cent.module()
        return True, ""
    except Exception as e:  # the build needs the staged sources and gcc
        return False, str(e).splitlines()[0] if str(e) else type(e).__name__


def cpu_baseline_entry(frames_all=64, frames_one=4):
    """The reference module on a bounded sample of the bench workload: all
    host cores (the reference's nthreads) and one core."""
    ok, why = reference_available()
    if not ok:
        dt, nl = cpu_sample(16, 1)
        return {"value": nl * 16 / dt, "unit": UNIT, "cores": 1, "kind": "port",
                "sample": "16 noisy frames through the numpy/C restatement (reference module unavailable: %s)" % why}
    cores = host_cores()
    frames = make_frames(make_screens(4, 5000), frames_all, 7)
    rt = RefTimer(cores, frames)
    rt.step(2)
    wall, own = rt.step(frames_all)
    rt.free()
    rt1 = RefTimer(1, frames[:frames_one])
    rt1.step(1)
    wall1, _ = rt1.step(frames_one)
    rt1.free()
    return {"value": rt.nlit * frames_all / wall, "unit": UNIT, "cores": cores, "kind": "reference",
            "sample": "%d noisy frames of the same workload through the reference's own centmodule (oracle/_ref, "
                      "unmodified centmodule.c with FFT/GSL shims), nthreads=%d; %.2f s wall, py_run's own timer "
                      "%.2f s" % (frames_all, cores, wall, own),
            "single_thread": {"value": rt1.nlit * frames_one / wall1, "frames": frames_one, "seconds": wall1}}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    ok, why = reference_available()
    cores = host_cores()
    F = args.frames
    base = {"impl": "reference", "metric": METRIC, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded von Karman phase screens (r0 0.157 m @500 nm, L0 25 m, 589 nm)"}
    if ok:
        frames = make_frames(make_screens(16, 1000), F, 0)
        rt = RefTimer(cores, frames)
        for _ in range(args.warmup):
            rt.step(F)
        walls, owns = [], []
        for _ in range(args.steps):
            wl, ow = rt.step(F)
            walls.append(wl)
            owns.append(ow)
        rt.free()
        t = sum(walls)
        v = rt.nlit * F * args.steps / t
        kind = "reference"
        sample = ("%d frames per step through the reference's own centmodule (oracle/_ref: unmodified "
                  "cmod/src/centmodule.c built with FFT/GSL shims; nthreads=%d worker threads), each frame timed "
                  "around cent.run; py_run's own timer summed %.3f s over the timed steps" % (F, cores, sum(owns)))
    else:
        fpw = 1
        walls, total_sf = [], 0.0
        for _ in range(args.warmup):
            cpu_parallel(fpw, cores)
        for _ in range(args.steps):
            wall, nlit, total = cpu_parallel(fpw, cores)
            walls.append(wall)
            total_sf += nlit * total
        t = sum(walls)
        v = total_sf / t
        F = fpw * cores
        kind = "port"
        sample = ("%d frames per step through the numpy/C restatement (reference module unavailable: %s)"
                  % (F, why))
    line = dict(base, value=v, ms_per_step=1e3 * t / args.steps,
                config={"workload": WORKLOAD["name"], "frames_per_step": F},
                cpu_baseline={"value": v, "unit": UNIT, "cores": cores, "kind": kind, "sample": sample},
                e2e={"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- serving workload

def serving_systems(nsys=64, seed=5):
    """64 simulated AO systems: subaperture counts from {8,16,32,40,74,84}^2,
    fftsize 16-32 (phasesize N/2, nimg N/2), half NGS (Gaussian spot), half
    LGS (per-subaperture elongated spots), nintegrations 1-4, Poisson
    request rates 500-2000 Hz."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nsys):
        nsubx = int(rng.choice([8, 16, 32, 40, 74, 84]))
        N = int(rng.choice([16, 20, 24, 32]))
        out.append(dict(nsubx=nsubx, N=N, p=N // 2, m=N // 2, lgs=bool(rng.random() < 0.5),
                        nint=int(rng.integers(1, 5)), rate=float(rng.uniform(500.0, 2000.0)),
                        sig=float(rng.uniform(300.0, 2000.0)), rn=float(rng.uniform(1.0, 3.0)), seed=1000 + k))
    return out


def serving_kwargs(sysd, screens_cache):
    """centcmod arguments and device phase frames of one serving system."""
    import torch
    from dasp_gb300.screens import gaussian_psf, lgs_psfs, von_karman_screen
    from dasp_gb300.tel import Pupil
    nsubx, p, N, m = sysd["nsubx"], sysd["p"], sysd["N"], sysd["m"]
    npup = nsubx * p
    pup = Pupil(npup, npup / 2.0, npup / 2.0 * 0.2)
    if sysd["lgs"]:
        frac = pup.getSubarea(nsubx) / (p * p)
        psf = lgs_psfs(nsubx, N, 1.2, 6.0, subap_area=frac)
    else:
        psf = gaussian_psf(N, 1.5)
    if npup not in screens_cache:
        screens_cache[npup] = von_karman_screen(npup, nsubx * 0.5, 0.15, 30.0, 77 + npup, 640.0)
    base = screens_cache[npup]
    frames = [torch.from_numpy(np.ascontiguousarray(np.roll(base, (31 * j + sysd["seed"]) % npup, axis=j % 2)))
              .cuda() for j in range(2)]
    kw = dict(nthreads=8, nsubx=nsubx, ncen=m, fftsize=N, clipsize=N, nimg=m, phasesize=p, readnoise=sysd["rn"],
              readbg=0.0, addPoisson=1, noiseFloor=2 * sysd["rn"], sig=sysd["sig"], skybrightness=5.0, calsource=0,
              pxlPower=1.0, nintegrations=sysd["nint"], nlatency=0, seed=sysd["seed"], phs=base, pup=pup,
              spotpsf=psf, cents=np.zeros(nsubx * nsubx * 2, np.float32),
              bimg=np.zeros((nsubx * nsubx, m, m), np.float32), minarea=0.5, opticalBinning=0, centWeight=None,
              correlationCentroiding=0, corrThresh=0.0, corrPattern=None, corrimg=None, threshType=0, imageOnly=0,
              useBrightest=0, preBinningFactor=1, parabolicFit=0, gaussianFitVals=None)
    return kw, frames


def run_serving(args):
    """Serving loop on device-resident state: 64 systems, Poisson arrivals,
    HBM-budget admission; p50/p99 frame latency and subap-frames/s for the
    tensor-core (fp16) and FP32 forms."""
    import torch
    from dasp_gb300.serving import WfsServer, poisson_schedule, run_schedule
    torch.cuda.set_device(0)
    systems = serving_systems()
    cache = {}
    prepared = [serving_kwargs(sd, cache) for sd in systems]
    duration = float(args.serve_seconds)
    sched = poisson_schedule([sd["rate"] for sd in systems], duration, seed=11)
    budget = 120 << 30
    res = {}
    runs = [("fp16", "compat"), ("fp32", "compat"), ("fp16", "physical")]
    with ClockSampler(0) as clk:
        for form, integ in runs:
            # compat: the reference's integration (only readout frames form an
            # image); physical: every sub-exposure formed and averaged on the
            # device (nintegrations 1-4), about 2.5x the formation work
            srv = WfsServer(budget, max_inflight=args.serve_inflight, integration=integ)
            ids = [srv.add_system(form=form, **kw) for kw, _ in prepared]
            t_end = time.time() + 120
            while srv.stats()["admitted"] < len(ids) and time.time() < t_end:
                time.sleep(0.05)
            # warm-up: one frame per system
            for i, (_, fr) in zip(ids, prepared):
                srv.submit(i, fr[0])
            srv.drain(120)
            r = run_schedule(srv, ids, [fr for _, fr in prepared], sched)
            st = srv.stats()
            r["hbm_used_gb"] = st["used_bytes"] / 1e9
            res[form if integ == "compat" else form + "_physical"] = r
            srv.close()
    head = res["fp16"]
    lit = {}
    line = {
        "metric": "serving: p99 WFS-frame latency, 64 simulated AO systems (Poisson arrivals 500-2000 Hz)",
        "value": head["latency_ms"]["p99"], "unit": "ms", "n_gpus": 1, "steps": len(sched), "warmup": len(systems),
        "ms_per_step": head["latency_ms"]["mean"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "fp16 (GEMM-DFT; LGS systems with per-subaperture PSFs run FP32)",
        "data": "synthetic: seeded von Karman screens, Gaussian NGS and elongated LGS spots",
        "config": {"workload": "serving_64_systems", "systems": len(systems), "duration_s": duration,
                   "requests": len(sched), "hbm_budget_gb": budget / 2 ** 30, "max_inflight": args.serve_inflight,
                   "nsubx_choices": [8, 16, 32, 40, 74, 84], "fftsize_choices": [16, 20, 24, 32],
                   "lgs_systems": sum(sd["lgs"] for sd in systems),
                   "integration": "forms fp16/fp32: compat (the reference's: only the readout frame's phase "
                                  "reaches the image); fp16_physical: nintegrations 1-4 with every exposed "
                                  "sub-exposure formed and averaged on the device, noise and centroids at the "
                                  "readout -- every request then forms an image",
                   "offered_subap_frames_per_s": sum(sd["rate"] / sd["nint"] * sd["nsubx"] ** 2 * 0.75
                                                     for sd in systems)},
        "forms": res, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- precision sweep

PRECISION = dict(nsubx=40, Dtel=8.0, obs=0.2, L0=25.0, wavelength=500.0, cases=[(8, 16), (16, 32), (32, 64)],
                 r0s=[0.05, 0.1, 0.2, 0.3], sig=1e4, psf_fwhm=1.5)


_PREC = {}


def _prec_setup(p, N, bases):
    """Per process: the case's oracle inputs and base screens (pool initializer)."""
    from dasp_gb300.screens import gaussian_psf
    from dasp_gb300.tel import Pupil
    P = PRECISION
    nsx = P["nsubx"]
    npup = nsx * p
    pup = Pupil(npup, npup / 2.0, npup / 2.0 * P["obs"])
    _PREC.update(p=p, N=N, nsx=nsx, bases=bases, pupfn=pup.perSubap(nsx, 0), subflag=pup.getSubapFlag(nsx, 0.5),
                 frac=(pup.getSubarea(nsx) / (p * p)).astype(np.float32), psf=gaussian_psf(N, P["psf_fwhm"]))


def _prec_frame(bases, f, scale):
    """Frame f of a case: a flip/transpose/roll of one of the base screens
    (deterministic in f), scaled for r0."""
    npup = bases[0].shape[0]
    rng = np.random.default_rng(1000 + f)
    s_ = bases[f % len(bases)]
    s_ = s_[::-1] if rng.random() < 0.5 else s_
    s_ = s_.T if rng.random() < 0.5 else s_
    s_ = np.roll(s_, (int(rng.integers(0, npup)), int(rng.integers(0, npup))), axis=(0, 1))
    return np.ascontiguousarray(s_ * np.float32(scale), dtype=np.float32)


def _prec_ref(job):
    """float64 oracle of frames [f0, f1) at one r0 scale: lit centroids of
    every frame, lit images of frames below nimg_frames."""
    from oracle.shwfs_oracle import CentOracle
    f0, f1, scale, nimg_frames = job
    c_ = _PREC
    p, N, nsx = c_["p"], c_["N"], c_["nsx"]
    lit = c_["subflag"].reshape(-1) == 1
    orc = CentOracle(nsubx=nsx, phasesize=p, fftsize=N, clipsize=N, nimg=p, ncen=p, pupfn=c_["pupfn"],
                     subflag=c_["subflag"], fracSubArea=c_["frac"], sig=PRECISION["sig"], spotpsf=c_["psf"],
                     mode="f64")
    cents, imgs = [], []
    for f in range(f0, f1):
        c = np.zeros(nsx * nsx * 2, np.float32)
        b = np.zeros((nsx * nsx, p, p), np.float32)
        orc.run(_prec_frame(c_["bases"], f, scale), c, b)
        cents.append(c.reshape(-1, 2)[lit].astype(np.float64))
        if f < nimg_frames:
            imgs.append(b.reshape(nsx * nsx, -1)[lit].astype(np.float64))
    return f0, cents, imgs


def run_precision(args):
    """Noiseless centroid error (mean/max px over lit subapertures) and
    image-plane relative L2 error of every compute form against the float64
    oracle, on a 40x40-subaperture WFS, phasesize 8/16/32 with fftsize
    16/32/64 (2x padding, nimg = phasesize), r0 0.05-0.3 m on an 8 m pupil
    (peak-to-valley phase up to a few hundred rad).  --precision-frames
    frames per (phasesize, r0) case (phasesize 32, where only the FP32 form
    runs, at most 200), the float64 references computed by a pool of host
    processes over all cores; image errors on the first 16 frames."""
    import multiprocessing as mp
    from dasp_gb300.centcmod import centcmod
    from dasp_gb300.screens import gaussian_psf, von_karman_screen
    from dasp_gb300.tel import Pupil
    P = PRECISION
    nsx = P["nsubx"]
    FORMS = ("fp32", "tf32", "bf16", "fp16", "bf16x3")
    codes = {"fp32": 0, "bf16": 1, "bf16x3": 2, "fp16": 3, "tf32": 4}
    nimg_frames = 16
    cores = host_cores()
    out = []
    t0 = time.time()
    # references first (a spawn pool, before the GPU is touched)
    plan = []
    for p, N in P["cases"]:
        nfr = int(args.precision_frames) if p < 32 else min(int(args.precision_frames), 200)
        npup = nsx * p
        nb = 8 if p < 32 else 4
        bases = [von_karman_screen(npup, P["Dtel"], P["r0s"][0], P["L0"], 500 + 10 * p + k, P["wavelength"])
                 for k in range(nb)]
        refs = {}
        ctx = mp.get_context("spawn")
        per = max(1, (nfr + 4 * cores - 1) // (4 * cores))
        with ctx.Pool(cores, initializer=_prec_setup, initargs=(p, N, bases)) as pool:
            for r0 in P["r0s"]:
                scale = (P["r0s"][0] / r0) ** (5.0 / 6.0)
                jobs = [(f, min(nfr, f + per), scale, nimg_frames) for f in range(0, nfr, per)]
                cents, imgs = [None] * nfr, [None] * min(nfr, nimg_frames)
                for f0, cs, ims in pool.imap_unordered(_prec_ref, jobs):
                    for k, cc in enumerate(cs):
                        cents[f0 + k] = cc
                    for k, im in enumerate(ims):
                        imgs[f0 + k] = im
                refs[r0] = (scale, cents, imgs)
        plan.append((p, N, nfr, bases, refs))
    t_ref = time.time() - t0
    import torch
    torch.cuda.set_device(0)
    for p, N, nfr, bases, refs in plan:
        m = p
        npup = nsx * p
        pup = Pupil(npup, npup / 2.0, npup / 2.0 * P["obs"])
        psf = gaussian_psf(N, P["psf_fwhm"])
        lit = pup.getSubapFlag(nsx, 0.5).reshape(-1) == 1
        hp = np.zeros((npup, npup), np.float32)  # the engines' bound phase buffer
        hc = np.zeros(nsx * nsx * 2, np.float32)
        hb = np.zeros((nsx, nsx, m, m), np.float32)
        engines = {}
        for form in FORMS:
            e = centcmod(1, nsx, m, N, N, m, p, 0.0, 0.0, 0, 0.0, P["sig"], 0.0, 0, 1.0, 1, 0, 1, hp, pup, psf,
                         hc, hb, 0.5, 0, None, 0, 0.0, None, None, 0, 0, 0, 1, 0, None)
            e.set_form(form)
            if e.info()["form_active"] == codes[form]:
                engines[form] = e
            else:
                e.free()
        for r0 in P["r0s"]:
            scale, rcents, rimgs = refs[r0]
            case = {"phasesize": p, "fftsize": N, "nimg": m, "r0_m": r0, "frames": nfr,
                    "image_frames": len(rimgs), "lit_subaps": int(lit.sum()), "forms": {}}
            errs = {f: [] for f in engines}
            l2 = {f: [] for f in engines}
            pv = 0.0
            for f in range(nfr):
                hp[...] = _prec_frame(bases, f, scale)
                pv = max(pv, float(hp.max() - hp.min()))
                for form, e in engines.items():
                    e.run(0)
                    errs[form].append(np.abs(hc.reshape(-1, 2)[lit].astype(np.float64) - rcents[f]).ravel())
                    if f < len(rimgs):
                        eb = hb.reshape(nsx * nsx, -1)[lit].astype(np.float64)
                        l2[form].append(np.linalg.norm(eb - rimgs[f]) / np.linalg.norm(rimgs[f]))
            case["phase_pv_rad"] = round(pv, 1)
            for form in FORMS:
                if form not in engines:
                    case["forms"][form] = {"active": False,
                                           "note": "geometry outside the tensor-core kernel's limits; FP32 form runs"}
                    continue
                ee = np.concatenate(errs[form])
                case["forms"][form] = {"active": True, "mean_err_px": float(ee.mean()), "max_err_px": float(ee.max()),
                                       "p99_err_px": float(np.percentile(ee, 99)), "img_rel_l2": float(np.mean(l2[form]))}
            out.append(case)
            print(json.dumps({"case": case}), file=sys.stderr, flush=True)
        for e in engines.values():
            e.free()
    worst = {f: max((c["forms"][f]["max_err_px"] for c in out if c["forms"][f].get("active")), default=None)
             for f in FORMS}
    line = {
        "metric": "precision sweep: max centroid error vs FP64 oracle (px), noiseless, 40x40 subaps",
        "value": worst["fp16"], "unit": "px", "n_gpus": 1, "steps": sum(c["frames"] for c in out), "warmup": 0,
        "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "per form (fp32, tf32, bf16, fp16 with per-subaperture scaling, bf16x3)",
        "data": "synthetic: seeded von Karman screens (r0 %s m at 500 nm, L0 %g m, %g m pupil); frames are "
                "flips/transposes/rolls of 8 base screens per case (4 for phasesize 32)"
                % (P["r0s"], P["L0"], P["Dtel"]),
        "config": {"workload": "precision_sweep_40x40", "nsubx": nsx, "cases": P["cases"], "r0_m": P["r0s"],
                   "frames_per_case": {str(c[0]): c[2] for c in plan}, "image_error_frames": nimg_frames,
                   "reference": "float64 oracle on %d host processes" % cores},
        "max_err_px_by_form": worst, "cases": out, "wall_s": round(time.time() - t0, 1),
        "reference_wall_s": round(t_ref, 1),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- batched multi-WFS step

LGS_BATCH = dict(lgs=dict(count=6, nsubx=74, p=10, N=32, m=16, Dtel=39.0, obs=0.28),
                 ngs=[dict(nsubx=8, p=8, N=16, m=8), dict(nsubx=16, p=16, N=32, m=16),
                      dict(nsubx=24, p=32, N=64, m=16)])


def run_lgs_batch(args):
    """Batched uneven multi-WFS tomography step: 6 LGS WFS at 74x74 (p 10,
    fftsize 32, nimg 16, per-subaperture 32x32 elongated spots) and 3 NGS at
    8x8, 16x16, 24x24, all captured into one CUDA graph (one branch per WFS,
    the FP32 kernels' tiles picked by the autotuner) and replayed once per
    step; the same WFSs run one after another on one stream for comparison.
    NGS sensors run BF16x3 where the tensor-core geometry allows, LGS
    sensors (per-subaperture PSFs) the FP32 form.  L2 is flushed between
    timed steps."""
    import torch
    from dasp_gb300.batch import WfsBatch
    from dasp_gb300.centcmod import centcmod
    from dasp_gb300.screens import gaussian_psf, lgs_psfs, von_karman_screen
    from dasp_gb300.tel import Pupil
    torch.cuda.set_device(0)
    rng = np.random.default_rng(21)
    specs = []
    L = LGS_BATCH["lgs"]
    for k in range(L["count"]):
        specs.append(dict(L, lgs=True, sig=float(rng.uniform(300, 2000)), rn=float(rng.uniform(1, 3)),
                          theta=60.0 * k, seed=300 + k))
    for k, n in enumerate(LGS_BATCH["ngs"]):
        specs.append(dict(n, lgs=False, Dtel=n["nsubx"] * 0.5, obs=0.2, sig=float(rng.uniform(300, 2000)),
                          rn=float(rng.uniform(1, 3)), seed=400 + k))
    engines, lit, forms, tensors = [], 0, [], []
    screens = {}
    for sp in specs:
        nsx, p, N, m = sp["nsubx"], sp["p"], sp["N"], sp["m"]
        npup = nsx * p
        pup = Pupil(npup, npup / 2.0, npup / 2.0 * sp["obs"])
        if sp["lgs"]:
            frac = pup.getSubarea(nsx) / (p * p)
            psf = lgs_psfs(nsx, N, 1.2, 6.0, launch_theta_deg=sp["theta"], subap_area=frac)
        else:
            psf = gaussian_psf(N, 1.5)
        key = (npup, sp["Dtel"])
        if key not in screens:
            screens[key] = von_karman_screen(npup, sp["Dtel"], 0.157, 25.0, 900 + npup, 589.0)
        ph = np.ascontiguousarray(np.roll(screens[key], 37 * sp["seed"], axis=0))
        hc = np.zeros(nsx * nsx * 2, np.float32)
        hb = np.zeros((nsx, nsx, m, m), np.float32)
        eng = centcmod(1, nsx, m, N, N, m, p, sp["rn"], 0.0, 1, 2 * sp["rn"], sp["sig"], 5.0, 0, 1.0, 1, 0,
                       sp["seed"], ph, pup, psf, hc, hb, 0.5, 0, None, 0, 0.0, None, None, 0, 0, 0, 1, 0, None)
        if not sp["lgs"]:
            eng.set_form("bf16x3")
        if eng.info()["form_active"] == 0:
            eng.autotune()
        dp = torch.from_numpy(ph).cuda()
        dc = torch.zeros(nsx * nsx * 2, device="cuda")
        db = torch.zeros((nsx * nsx, m, m), device="cuda")
        eng.set_io(dp, dc, db)
        tensors.append((dp, dc, db))
        engines.append(eng)
        lit += eng.info()["nlit"]
        forms.append({0: "fp32", 1: "bf16", 2: "bf16x3", 3: "fp16", 4: "tf32"}[eng.info()["form_active"]])
    batch = WfsBatch(engines)
    stream = torch.cuda.Stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)  # L2 flush, outside the timed events
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
            stream.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts)), float(np.mean(ts))

    def run_graph():
        batch.run(stream)

    def run_seq():
        for eng, (dp, dc, db) in zip(engines, tensors):
            eng.run_batch(dp.unsqueeze(0), dc.unsqueeze(0), db.unsqueeze(0), stream=stream)

    with ClockSampler(0) as clk:
        g_med, g_mean = timed(run_graph)
        s_med, s_mean = timed(run_seq)
        # the same graph with the FP32-form LGS sensors as one multi-handle kernel
        batch.set_multi(True)
        multi = batch.multi_launches()
        m_med, _ = timed(run_graph)
    batch.free()
    for e in engines:
        e.free()
    line = {
        "metric": "batched multi-WFS step: subap-frames/s (6 LGS 74x74 + 3 NGS, one CUDA graph)",
        "value": lit / (g_med / 1e3), "unit": "subap-frames/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": g_med, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "per WFS: " + ", ".join(forms),
        "data": "synthetic: seeded von Karman screens, elongated LGS and Gaussian NGS spots",
        "config": {"workload": "lgs_batch_6x74_3ngs",
                   "multi_handle": {"launches": multi, "ms_per_step": m_med},
                   "wfs": [{k: v for k, v in sp.items() if k != "obs"} for sp in specs],
                   "lit_subaps_per_step": lit, "l2": "flushed between timed steps (256 MB write, untimed)"},
        "sequential_ms_per_step": s_med, "graph_speedup_vs_sequential": s_med / g_med,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- reconstructor step

def run_recon(args):
    """The centroids' consumer: tomoRecon's decay + reconstructor MVM on
    the device for an ELT-scale system (5,316 actuators x the 7,944 slopes
    of the 74x74 sensor; R 169 MB, larger than L2, read once per step)."""
    import torch
    from dasp_gb300.recon import Reconstructor
    torch.cuda.set_device(0)
    nacts, ncents = 5316, 7944
    rng = np.random.default_rng(2)
    R = torch.from_numpy(rng.standard_normal((nacts, ncents), dtype=np.float32)).cuda()
    rec = Reconstructor(R, 0.5, 0.99)
    xs = [torch.from_numpy(rng.standard_normal(ncents, dtype=np.float32)).cuda() for _ in range(4)]
    stream = torch.cuda.Stream()
    for k in range(max(args.warmup, 3)):
        rec.step(xs[k % 4], stream=stream)
    stream.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(0) as clk:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                ev[k][0].record(stream)
                rec.step(xs[k % 4], stream=stream)
                ev[k][1].record(stream)
        stream.synchronize()
    ms = float(np.median([a.elapsed_time(b) for a, b in ev]))
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    bytes_step = 4.0 * nacts * ncents + 4.0 * ncents + 8.0 * nacts
    gbs = bytes_step / (ms / 1e3) / 1e9
    line = {
        "metric": "reconstructor steps/s (5316 actuators x 7944 slopes, decay + MVM)", "value": 1e3 / ms,
        "unit": "steps/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded normal reconstructor and slopes",
        "config": {"workload": "recon_mvm_5316x7944", "l2": "R (169 MB) larger than L2, read once per step"},
        "roofline": {"bound": "hbm", "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                     "traffic": None, "kernel": "mvm_update_kernel",
                     "algorithmic_bytes_per_step": bytes_step},
        "clocks": clk.summary(), "gpu_launches": args.steps,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- AO loop on the device

ATMOS = dict(layers=[  # Cn2 fraction, wind (pixels of 0.0527 m per frame: 10, 20, 30, 50 m/s at 1 kHz)
    dict(frac=0.5, wind=0.19, seed=51), dict(frac=0.2, wind=0.38, seed=52),
    dict(frac=0.2, wind=0.57, seed=53), dict(frac=0.1, wind=0.95, seed=54)], nacts=5316)


def run_atmos(args):
    """One AO-loop frame on the device, end to end, for the 74x74 sensor:
    four frozen-flow layers advanced by their wind (infScrn's column
    extrusion, science/infScrn.py:747-791, each layer's screen 741 x 742 px
    in HBM), the sensor's 740x740 pupil phase from them (infAtmos'
    createPupilPhs for a source at infinity, util/atmos.py:678-833: each
    layer's window with linearshift's sub-pixel shift, piston removed,
    scaled to 589 nm), the WFS frame in the FP16 form with Poisson and read
    noise, and the reconstructor step (decay + MVM, 5,316 actuators over the
    engine's 10,952-slope centroid vector, R 233 MB).  Every stage is queued
    on one stream; nothing crosses the host link.  The loop rate is frames
    over the events around the timed frames; the per-stage medians are
    event intervals on the same stream (they include any wait for the
    host's launches)."""
    import torch
    from dasp_gb300.infscreen import DeviceScreen, extrusion_matrices, phase_covariance, pupil_phase
    from dasp_gb300.recon import Reconstructor
    from dasp_gb300.screens import von_karman_screen
    torch.cuda.set_device(0)
    w = WORKLOAD
    pup = make_pupil()
    npup = w["nsubx"] * w["p"]
    nsub = w["nsubx"] ** 2
    ny, nx = npup + 1, npup + 2
    scale = w["Dtel"] / npup
    t0 = time.time()
    ay, by = extrusion_matrices(ny, phase_covariance(ny, w["L0"], scale))
    setup_s = time.time() - t0
    layers = []
    for ly in ATMOS["layers"]:
        r0 = w["r0"] * ly["frac"] ** (-3. / 5)
        init = von_karman_screen(nx, nx * scale, r0, w["L0"], ly["seed"], 500.0)[:ny, :nx]
        layers.append(dict(ly, r0=r0, pos=0.0, screen=DeviceScreen(init, w["L0"], ay=ay, by=by, seed=ly["seed"])))
    pupil_t = torch.from_numpy(pup.fn.astype(np.float32)).cuda()
    area = float(pup.fn.sum())
    dp = torch.zeros((npup, npup), device="cuda")
    dc = torch.zeros(nsub * 2, device="cuda")
    db = torch.zeros((nsub, w["m"], w["m"]), device="cuda")
    hc = np.zeros(nsub * 2, np.float32)
    hb = np.zeros((w["nsubx"], w["nsubx"], w["m"], w["m"]), np.float32)
    eng = make_engine(pup, np.zeros((npup, npup), np.float32), hc, hb)
    eng.set_form("fp16")
    form = {0: "fp32", 1: "bf16", 2: "bf16x3", 3: "fp16", 4: "tf32"}[eng.info()["form_active"]]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        pupil_phase([(ly["screen"], 0, 0, 0.0, 0.0) for ly in layers], pupil_t, dp, pupil_area=area,
                    wavelength=w["wavelength"], stream=stream)
    stream.synchronize()
    eng.set_io(dp, dc, db)
    eng.autotune()
    rng = np.random.default_rng(2)
    R = torch.from_numpy(rng.standard_normal((ATMOS["nacts"], nsub * 2), dtype=np.float32) * 1e-3).cuda()
    rec = Reconstructor(R, 0.5, 0.99)
    ncols = 0

    def frame(ev=None):
        nonlocal ncols
        if ev:
            ev[0].record(stream)
        wins = []
        for ly in layers:
            ly["pos"] += ly["wind"]
            k = int(ly["pos"])
            if k:
                ly["screen"].add_columns(k, ly["r0"], stream=stream)
                ly["pos"] -= k
                ncols += k
            wins.append((ly["screen"], 0, 0, 0.0, float(ly["pos"])))
        if ev:
            ev[1].record(stream)
        pupil_phase(wins, pupil_t, dp, pupil_area=area, wavelength=w["wavelength"], stream=stream)
        if ev:
            ev[2].record(stream)
        eng.run_batch(dp.unsqueeze(0), dc.unsqueeze(0), db.unsqueeze(0), stream=stream)
        if ev:
            ev[3].record(stream)
        rec.step(dc, stream=stream)
        if ev:
            ev[4].record(stream)

    nframes = max(args.steps * 50, 500)
    for _ in range(max(args.warmup, 3) * 10):
        frame()
    stream.synchronize()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(nframes)]
    ncols = 0
    tq = []
    with ClockSampler(0) as clk:
        with torch.cuda.stream(stream):
            t0 = time.perf_counter()
            for k in range(nframes):
                frame(evs[k])
                if k < 33:
                    tq.append(time.perf_counter())
            stream.synchronize()
            wall = time.perf_counter() - t0
    # the host's time to queue one frame, over the first frames (before the
    # launch queue fills and the host waits for the device): below the
    # frame's event interval the device sets the rate, at it the host does
    host_ms = float(np.median(np.diff(tq))) * 1e3
    span_ms = evs[0][0].elapsed_time(evs[-1][4])
    stage = lambda a, b: float(np.median([e[a].elapsed_time(e[b]) for e in evs]))  # noqa: E731
    stages = {"screens_ms": stage(0, 1), "pupil_phase_ms": stage(1, 2), "wfs_ms": stage(2, 3),
              "reconstructor_ms": stage(3, 4), "frame_ms": stage(0, 4)}
    # a sanity check of the loop's output: finite slopes and commands
    ok = bool(torch.isfinite(dc).all().item() and torch.isfinite(rec.act).all().item())
    nlit = eng.info()["nlit"]
    for ly in layers:
        ly["screen"].free()
    eng.free()
    line = {
        "metric": "AO-loop frames/s on the device (4 layers -> 74x74 pupil phase -> WFS -> reconstructor)",
        "value": nframes / (span_ms / 1e3), "unit": "frames/s", "n_gpus": 1, "steps": nframes,
        "warmup": max(args.warmup, 3) * 10, "ms_per_step": span_ms / nframes, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "screens f64 extrusion, f32 phase; WFS " + form,
        "data": "synthetic: seeded von Karman layers (r0 0.157 m total, L0 25 m), seeded normal reconstructor",
        "config": {"workload": "atmos_loop_74x74", "layers": [{k: ly[k] for k in ("frac", "wind", "r0")}
                                                            for ly in layers],
                   "screen_px": [ny, nx], "npup": npup, "lit_subaps": nlit, "nacts": ATMOS["nacts"],
                   "columns_extruded": ncols, "matrix_setup_s": setup_s,
                   "l2": "screens' extrusion matrices (53 MB) L2-resident; R (233 MB) larger than L2"},
        "stages_median": stages, "host_enqueue_ms_per_frame": host_ms, "wall_frames_per_s": nframes / wall,
        "finite": ok,
        "clocks": clk.summary(), "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


def run_corr(args):
    """Correlation centroiding on the 74x74 sensor (noisy, Gaussian spot
    PSF): mode 1 (FFT correlation with a 20x20 pattern made by
    transform_psf from a reference spot, as util/centroid.py does) and mode
    5 (brute-force correlation with the spot itself), FP16 and FP32 forms.
    Correlation runs one frame per call: each frame goes through
    centcmod.set_io + run_async with host numpy phase/cents/bimg (copies;
    the correlation images are not bound), timed between CUDA events on the
    launch stream."""
    import torch
    from dasp_gb300.centcmod import centcmod
    from dasp_gb300.correlation import transform_psf
    from dasp_gb300.screens import gaussian_psf
    torch.cuda.set_device(0)
    w = WORKLOAD
    pup = make_pupil()
    nsx, m = w["nsubx"], w["m"]
    nsub = nsx * nsx
    screens = make_screens(4)
    frames = [np.ascontiguousarray(f) for f in make_frames(screens, 8, 21)]
    cs = 2 * m
    y, x = np.mgrid[0:cs, 0:cs] - (cs - 1) / 2.0
    spot = (50.0 * np.exp(-(x * x + y * y) / (2 * 1.5 ** 2))).astype(np.float32)
    spots = np.ascontiguousarray(np.broadcast_to(spot, (nsx, nsx, cs, cs)))
    psf = gaussian_psf(w["C"], w["psf_fwhm"])
    nframes = max(args.steps * 10, 100)
    results = {}
    with ClockSampler(0) as clk:
        for mode in (1, 5):
            pattern = transform_psf(spots) if mode == 1 else spots.copy()
            for form in ("fp16", "fp32"):
                hc = np.zeros(nsub * 2, np.float32)
                hb = np.zeros((nsx, nsx, m, m), np.float32)
                e = centcmod(8, nsx, w["ncen"], w["N"], w["C"], m, w["p"], w["readnoise"], w["readbg"],
                             w["addPoisson"], w["floor"], w["sig"], w["sky"], 0, 1.0, 1, 0, 1234, frames[0], pup,
                             psf, hc, hb, 0.5, 0, None, mode, 0.0, pattern, None, w["threshType"], 0, 0, 1, 0, None)
                e.set_form(form)
                st = torch.cuda.Stream()
                for k in range(max(args.warmup, 3)):
                    e.set_io(phs=frames[k % 8])
                    e.run_async(st)
                st.synchronize()
                lat = []
                for k in range(nframes):
                    e.set_io(phs=frames[k % 8])
                    ea = torch.cuda.Event(enable_timing=True)
                    eb = torch.cuda.Event(enable_timing=True)
                    ea.record(st)
                    e.run_async(st)
                    eb.record(st)
                    st.synchronize()
                    lat.append(ea.elapsed_time(eb))
                nlit = e.info()["nlit"]
                p50 = float(np.percentile(lat, 50))
                results["mode%d_%s" % (mode, form)] = {
                    "ms_p50": p50, "ms_p99": float(np.percentile(lat, 99)),
                    "subap_frames_per_s": nlit / (p50 / 1e3), "form_active": e.info()["form_active"]}
                e.free()
    head = results["mode1_fp16"]
    line = {
        "metric": "correlation-centroiding subap-frames/s (74x74 NGS, mode 1 FFT correlation, one frame per call)",
        "value": head["subap_frames_per_s"], "unit": "subap-frames/s", "n_gpus": 1, "steps": nframes,
        "warmup": max(args.warmup, 3), "ms_per_step": head["ms_p50"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp16 (per-subap scaled, f32 accumulate); correlation f32",
        "data": "synthetic: seeded von Karman phase screens; Gaussian reference spot (sigma 1.5 px, 20x20)",
        "config": {"workload": "elt74x74_ngs_correlation", "corrsize": cs, "modes": [1, 5],
                   "io": "host numpy phase/cents/bimg, copies (correlation keeps the copying path)"},
        "results": results, "clocks": clk.summary(), "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


def run_slope(args):
    """Image input (centroidsFromImage through runSlope, the real-camera
    path): the 74x74 sensor's 740x740 detector frame -- the noisy images of a
    phase-mode frame laid out as the detector sees them -- centroided one
    frame per call from a pinned host numpy array into host cents/bimg,
    with zero-copy host I/O (default) and with copies.  Latency from the
    call's entry to the centroids on the host."""
    import time
    import torch
    torch.cuda.set_device(0)
    w = WORKLOAD
    pup = make_pupil()
    nsx, m = w["nsubx"], w["m"]
    nsub = nsx * nsx
    screens = make_screens(2)
    # detector frame: one noisy phase-mode frame's images, tiled
    hc = np.zeros(nsub * 2, np.float32)
    hb = np.zeros((nsx, nsx, m, m), np.float32)
    ph = np.ascontiguousarray(make_frames(screens, 1, 3)[0])
    e0 = make_engine(pup, ph, hc, hb)
    e0.run(0)
    det = np.ascontiguousarray(hb.transpose(0, 2, 1, 3).reshape(nsx * m, nsx * m))
    e0.free()
    results = {}
    with ClockSampler(0) as clk:
        for name, outputs, inp in (("zero_copy", True, True), ("copies", False, False)):
            img = det.copy()
            c2 = np.zeros(nsub * 2, np.float32)
            b2 = np.zeros((nsx, nsx, m, m), np.float32)
            from dasp_gb300.centcmod import centcmod
            from dasp_gb300.screens import gaussian_psf
            e = centcmod(8, nsx, w["ncen"], w["N"], w["C"], m, w["p"], w["readnoise"], w["readbg"],
                         w["addPoisson"], w["floor"], w["sig"], w["sky"], 0, 1.0, 1, 0, 1234, ph, pup,
                         gaussian_psf(w["C"], w["psf_fwhm"]), c2, b2, 0.5, 0, None, 0, 0.0, None, None,
                         w["threshType"], 0, 0, 1, 0, None, img)
            e.set_host_io(outputs=outputs, phase=inp)
            for k in range(max(args.warmup, 3)):
                e.runSlope(0)
            lat = []
            n = max(args.e2e_frames, 100)
            t0 = time.perf_counter()
            for k in range(n):
                t1 = time.perf_counter()
                e.runSlope(0)
                lat.append((time.perf_counter() - t1) * 1e3)
            wall = time.perf_counter() - t0
            nlit = e.info()["nlit"]
            results[name] = {"latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))},
                             "subap_frames_per_s": nlit * n / wall, "host_io_direct": e.info()["host_io_direct"]}
            e.free()
    head = results["zero_copy"]
    line = {
        "metric": "image-input centroiding subap-frames/s (74x74 NGS, 740x740 detector frame, runSlope, one "
                  "frame per call, host arrays)",
        "value": head["subap_frames_per_s"], "unit": "subap-frames/s", "n_gpus": 1, "steps": max(args.e2e_frames, 100),
        "warmup": max(args.warmup, 3), "ms_per_step": head["latency_ms"]["p50"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: the noisy images of a seeded von Karman phase frame, tiled as a 740x740 detector frame",
        "config": {"workload": "elt74x74_ngs_image_input", "detector": [nsx * m, nsx * m],
                   "e2e": {"h2d_bytes_per_step": int(nsx * m * nsx * m * 4),
                           "d2h_bytes_per_step": int(nsub * 2 * 4 + nsub * m * m * 4)}},
        "results": results, "clocks": clk.summary(), "gpu_launches": None,
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- our arm

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--frames", type=int, default=FPSTEP, help="frames per step")
    ap.add_argument("--e2e-frames", type=int, default=1000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="ngs74",
                    choices=["ngs74", "serving", "precision", "lgs_batch", "recon", "corr", "slope", "atmos"],
                    help="ngs74: the headline 74x74 NGS sensor; serving: 64 AO systems through the serving loop; "
                         "precision: per-form centroid error sweep vs the float64 oracle; "
                         "lgs_batch: 6 LGS + 3 NGS sensors in one CUDA graph; recon: the reconstructor step; "
                         "corr: correlation centroiding (modes 1 and 5) on the 74x74 sensor; "
                         "slope: image input (runSlope) from a 740x740 detector frame; "
                         "atmos: the AO loop on the device (layers, pupil phase, WFS, reconstructor)")
    ap.add_argument("--form", default=None, choices=["fp32", "fp16", "bf16x3", "tf32", "bf16"],
                    help="headline form (and the end-to-end run's) instead of the fastest within 1e-3 px; for "
                         "profiling runs, whose timings cannot choose")
    ap.add_argument("--staging", type=int, default=None,
                    help="with --form: that form's GEMM staging index instead of the autotuner's choice "
                         "(profiling runs)")
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    ap.add_argument("--precision-frames", type=int, default=8)
    ap.add_argument("--serve-inflight", type=int, default=16)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.workload in ("serving", "precision", "lgs_batch", "recon", "corr", "slope", "atmos") and args.impl == "ours":
        if rank == 0:
            from dasp_gb300 import build
            build.build()
            {"serving": run_serving, "precision": run_precision, "lgs_batch": run_lgs_batch,
             "recon": run_recon, "corr": run_corr, "slope": run_slope, "atmos": run_atmos}[args.workload](args)
        return

    if args.impl == "reference":
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(args, ws, rank)
        return

    import torch
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    from dasp_gb300 import build
    build.build()

    w = WORKLOAD
    pup = make_pupil()
    nsx = w["nsubx"]
    W = nsx * w["p"]
    nsub = nsx * nsx
    screens = make_screens(16, 1000 + 97 * rank)
    F = args.frames
    batches = [torch.from_numpy(make_frames(screens, F, 10 * rank + b)).cuda() for b in range(2)]
    dc = torch.zeros((F, nsub * 2), device="cuda")
    db = torch.zeros((F, nsub, w["m"], w["m"]), device="cuda")

    # engine bound to a host phase frame and host outputs (reference-facing path)
    host_phs = np.ascontiguousarray(screens[0])
    host_c = np.zeros(nsub * 2, np.float32)
    host_b = np.zeros((nsx, nsx, w["m"], w["m"]), np.float32)
    eng = make_engine(pup, host_phs, host_c, host_b)
    info = eng.info()
    nlit = info["nlit"]

    stream = torch.cuda.Stream()

    FORM_CODES = {"fp32": 0, "bf16": 1, "bf16x3": 2, "fp16": 3, "tf32": 4}
    PASSES = {"bf16x3": 3}

    def time_form(form):
        """Warm up and time args.steps batched steps of one compute form; for
        the tensor-core forms also the image-formation kernel alone (an event
        the engine records between it and the noise/centroid kernel)."""
        eng.set_form(form)
        if eng.info()["form_active"] != FORM_CODES[form]:
            return None
        # the engine's own autotuner picks the launch shape on this handle's
        # phase (results do not depend on it): the FP32 kernel's tile size,
        # the GEMM kernel's staging (--staging fixes the headline form's for
        # profiling runs, which then launch no tuning kernels)
        if args.staging is not None and form == args.form and form != "fp32":
            from dasp_gb300.centcmod import GEMMSTAGING
            eng.update(GEMMSTAGING, args.staging)
            ts = eng.info()["tile_subaps"]
        else:
            ts = eng.autotune()
        inf = eng.info()
        staging = {k: inf["gemm_" + k] for k in ("cw", "kcb", "nw", "nk", "dbuf")} if form != "fp32" else {"tile": ts}
        with torch.cuda.stream(stream):
            for k in range(args.warmup):
                eng.run_batch(batches[k % 2], dc, db, stream=stream)
        stream.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        mid = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        split = form != "fp32" and hasattr(mid[0], "cuda_event")
        if split:
            with torch.cuda.stream(stream):
                for m_ in mid:
                    m_.record(stream)  # creates the CUDA event
            stream.synchronize()
        t_start = torch.cuda.Event(enable_timing=True)
        t_end = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            t_start.record(stream)
            for k in range(args.steps):
                if split:
                    eng.set_split_event(mid[k])
                ev[k][0].record(stream)
                eng.run_batch(batches[k % 2], dc, db, stream=stream)
                ev[k][1].record(stream)
            t_end.record(stream)
        stream.synchronize()
        torch.cuda.synchronize()
        if split:
            eng.set_split_event(None)
        barrier(ws)
        tot = reduce_max(t_start.elapsed_time(t_end), ws)
        out = {"total_ms": tot, "ms_per_step": tot / args.steps,
               "per_launch_ms": float(np.mean([a.elapsed_time(b) for a, b in ev])),
               "value": ws * nlit * F * args.steps / (tot / 1e3)}
        if split:
            out["formation_ms"] = float(np.mean([a.elapsed_time(m_) for (a, _), m_ in zip(ev, mid)]))
            out["post_ms"] = float(np.mean([m_.elapsed_time(b) for (_, b), m_ in zip(ev, mid)]))
        out["tuned"] = staging
        return out

    with ClockSampler(local) as clk:
        forms = {f: time_form(f) for f in ("fp32", "fp16", "bf16x3", "tf32", "bf16")}
    forms = {f: r for f, r in forms.items() if r}

    # accuracy of a noiseless frame of every form vs the float64 oracle
    # (the oracle only checks; the tensor-core headline must meet 1e-3 px)
    errs = {}
    if rank == 0:
        nph = np.ascontiguousarray(screens[3])
        nc = np.zeros(nsub * 2, np.float32)
        nb = np.zeros((nsx, nsx, w["m"], w["m"]), np.float32)
        e2 = make_engine(pup, nph, nc, nb, noiseless=True)
        for f in forms:
            e2.set_form(f)
            e2.run(0)
            errs[f] = accuracy_vs_fp64(nc, nph)
        e2.free()
    ok_forms = [f for f in forms if f != "fp32" and errs.get(f, 1.0) <= 1e-3]
    head = max(ok_forms, key=lambda f: forms[f]["value"]) if ok_forms else "fp32"
    if args.form:  # profiling runs: timings under a profiler cannot choose
        if args.form not in forms:
            raise SystemExit("--form %s is not active on this workload" % args.form)
        head = args.form
    if ws > 1:
        import torch.distributed as dist
        hl = [head]
        dist.broadcast_object_list(hl, 0)
        head = hl[0]
    eng.set_form(head)
    total_ms = forms[head]["total_ms"]
    per_launch_ms = forms[head]["per_launch_ms"]
    ms_per_step = forms[head]["ms_per_step"]
    value = forms[head]["value"]

    # e2e through the reference-facing call (headline form): host phase in,
    # host cents/bimg out.  Eight host phase frames, each bound (and pinned)
    # once during the warm-up; each step binds the next one and runs, as a
    # simulation that writes its phase into one of a few buffers would
    host_frames = [np.ascontiguousarray(f) for f in make_frames(screens, 8, 99 + rank)]
    lat = []
    for k in range(8):
        eng.set_io(phs=host_frames[k])
        eng.run(0)
    barrier(ws)
    t0 = time.perf_counter()
    for k in range(args.e2e_frames):
        t1 = time.perf_counter()
        eng.set_io(phs=host_frames[k % 8])
        eng.run(0)
        lat.append(time.perf_counter() - t1)
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s, ws)
    e2e_value = ws * nlit * args.e2e_frames / e2e_s
    lat_ms = np.array(lat) * 1e3
    # device-side latency of the same frames (run_async between two events on
    # one stream: phase H2D from pinned memory, kernels, centroid/image D2H)
    dev_lat = []
    s_async = torch.cuda.Stream()
    for k in range(min(args.e2e_frames, 1000)):
        eng.set_io(phs=host_frames[k % 8])
        ea = torch.cuda.Event(enable_timing=True)
        eb = torch.cuda.Event(enable_timing=True)
        ea.record(s_async)
        eng.run_async(s_async)
        eb.record(s_async)
        s_async.synchronize()
        dev_lat.append(ea.elapsed_time(eb))
    dev_lat = np.array(dev_lat)

    F_alg, B_alg = algorithmic_per_subap()
    T_alg = tensor_flops_per_subap()
    B_post = 8 * w["m"] * w["m"] + 8  # pre-noise image in, final image out, centroids out
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
        peak_src = "measured"
    except Exception:
        peak_src = "fallback"
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    bf16_peak = float(peaks.get("bf16_tflops", 1900.0))
    sm_count = torch.cuda.get_device_properties(0).multi_processor_count
    clocks = clk.summary()
    fp32_peak_tf = sm_count * 128 * 2 * (clocks["sm_max_mhz"] or 2070.0) * 1e6 / 1e12
    units = nlit * F  # subap-frames per launch

    def tensor_peak(form):
        # tf32 runs at half the 16-bit rate (nominal 1.1 vs 2.25 PFLOP/s dense)
        return bf16_peak / 2 if form == "tf32" else bf16_peak

    def rooflines(form, r):
        t = r["per_launch_ms"] / 1e3
        out = {"hbm_gbs": B_alg * units / t / 1e9, "hbm_frac": B_alg * units / t / 1e9 / hbm_peak,
               "fp32_tflops": F_alg * units / t / 1e12, "fp32_frac": F_alg * units / t / 1e12 / fp32_peak_tf}
        if form != "fp32":
            tk = r.get("formation_ms", r["per_launch_ms"]) / 1e3
            tf = T_alg * PASSES.get(form, 1) * units / tk / 1e12
            out.update({"tensor_tflops": tf, "tensor_frac": tf / tensor_peak(form),
                        "tensor_peak_tflops": tensor_peak(form),
                        "formation_kernel_ms": r.get("formation_ms"), "post_kernel_ms": r.get("post_ms")})
        return out

    form_report = {}
    for f, r in forms.items():
        if r:
            form_report[f] = {"value": r["value"], "ms_per_step": r["ms_per_step"],
                              "kernel_ms_per_launch": r["per_launch_ms"], **rooflines(f, r)}
            form_report[f]["tuned"] = r["tuned"]
    if rank != 0:
        eng.free()
        return
    rl = rooflines(head, forms[head])
    if head == "fp32":
        roof = {"bound": "hbm", "achieved": rl["hbm_gbs"], "peak": hbm_peak, "unit": "GB/s", "frac": rl["hbm_frac"],
                "traffic": None, "peak_source": peak_src, "algorithmic_bytes_per_subap_frame": B_alg}
    else:
        # the two kernels of the tensor-core form, each against its own
        # roofline; "roofline" is the one that takes longer
        gemm = {"bound": "tensor", "achieved": rl["tensor_tflops"], "peak": tensor_peak(head), "unit": "TFLOP/s",
                "frac": rl["tensor_frac"], "traffic": NCU_TRAFFIC.get("wfs_gemm_kernel"),
                "peak_source": peak_src + (" (bf16 burst / 2 for tf32)" if head == "tf32" else " (bf16 burst)"),
                "algorithmic_flops_per_subap_frame": T_alg * PASSES.get(head, 1),
                "kernel": "wfs_gemm_kernel (image formation); timed between engine-recorded events",
                "kernel_ms": rl["formation_kernel_ms"]}
        post_s = rl["post_kernel_ms"] / 1e3
        post_gbs = B_post * units / post_s / 1e9
        post = {"bound": "hbm", "achieved": post_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": post_gbs / hbm_peak,
                "traffic": NCU_TRAFFIC.get("wfs_post_warp_kernel"), "peak_source": peak_src + " (copy bandwidth)",
                "algorithmic_bytes_per_subap_frame": B_post,
                "kernel": "wfs_post_warp_kernel (noise, threshold, centroids); timed between engine-recorded events",
                "kernel_ms": rl["post_kernel_ms"],
                "note": "issue-bound on the Philox/Poisson/normal samplers, far below its HBM roofline"}
        roof = dict(post if rl["post_kernel_ms"] > rl["formation_kernel_ms"] else gemm)
        roof["kernels"] = {"wfs_gemm_kernel": gemm, "wfs_post_warp_kernel": post}
    roof["step_ms_per_launch"] = per_launch_ms
    roof["units_per_launch"] = units
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp32": "f32", "bf16x3": "bf16x3 (split products, f32 accumulate)", "bf16": "bf16 (f32 accumulate)",
                  "fp16": "fp16 (per-subap scaled, f32 accumulate)", "tf32": "tf32 (f32 accumulate)"}[head],
        "data": "synthetic: seeded von Karman phase screens (r0 0.157 m @500 nm, L0 25 m, 589 nm)",
        "config": {"workload": w["name"], "nsubx": nsx, "lit_subaps": nlit, "phasesize": w["p"], "fftsize": w["N"],
                   "clipsize": w["C"], "nimg": w["m"], "psf": "2-D Gaussian FWHM 1.5 px (20x20)",
                   "noise": "Poisson + 3 e- read noise, sky 10, floor 6 (counter-based streams)",
                   "form": head, "frames_per_step": F, "replicas": ws,
                   "l2": "inputs larger than L2: two rotating %d-frame phase batches of %.0f MB"
                         % (F, F * W * W * 4 / 1e6)},
        "roofline": roof,
        "forms": form_report,
        "fp32_compute": {"achieved_tflops": form_report["fp32"]["fp32_tflops"], "peak_tflops": fp32_peak_tf,
                         "frac": form_report["fp32"]["fp32_frac"], "algorithmic_flops_per_subap_frame": F_alg,
                         "peak_basis": "SMs x 128 FP32 lanes x 2 x max SM clock", "form": "fp32"},
        # zero-copy host I/O (the engine's default): the image-formation
        # kernel reads the lit subapertures' phase from the pinned host array,
        # the noise/centroid kernel writes every centroid and the lit
        # subapertures' final images into the pinned host arrays
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(nlit * w["p"] * w["p"] * 4),
                "d2h_bytes_per_step": int(nsub * 2 * 4 + nlit * w["m"] * w["m"] * 4),
                "path": "centcmod.set_io + centcmod.run -> shwfs_run (%s form), pinned host numpy phase in, host "
                        "cents/bimg out, one synchronous frame per step; zero-copy host I/O (kernels read the "
                        "host phase and write the host outputs through their device aliases)" % head,
                "frames": args.e2e_frames},
        "latency_ms": {"p50": float(np.percentile(lat_ms, 50)), "p99": float(np.percentile(lat_ms, 99)),
                       "mean": float(lat_ms.mean()), "frames": len(lat_ms),
                       "path": "run() entry to centroids on the host (sync, host I/O)"},
        "latency_ms_device": {"p50": float(np.percentile(dev_lat, 50)) if len(dev_lat) else None,
                              "p99": float(np.percentile(dev_lat, 99)) if len(dev_lat) else None,
                              "frames": len(dev_lat),
                              "path": "run_async between CUDA events: phase in, kernels, outputs back"},
        "clocks": clocks,
        # per step: formation + noise/centroid kernels (tensor-core forms;
        # the latter also zeroes the unlit centroids), or fused + unlit (FP32)
        "gpu_launches": 2 * args.steps,
        "centroid_err_px_vs_fp64": errs,
        "head_rule": "fastest tensor-core form whose noiseless centroid error vs the float64 oracle is <= 1e-3 px",
    }
    if ws == 1 and not args.no_cpu_baseline:
        # the reference's own module on a bounded sample (64 frames on all
        # host cores, 4 on one core)
        line["cpu_baseline"] = cpu_baseline_entry()
    eng.free()
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
