#!/usr/bin/env python
"""Benchmark: chi2 evaluations per second of galario's chi2Profile on the
nxy=4096, 2M-visibility workload (double-ring profile, inc 40 deg, PA 70 deg).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one chi2Profile evaluation of one model over all 2M visibilities.
Prints ONE JSON line (rank 0).  Under torchrun (N > 1) every rank evaluates
its own replica of the workload (the path has no data exchange), the time is
the max over ranks and `value` counts the evaluations of all ranks.

--impl ours (default)
  value        device-resident plain FP64 chi2Profile (galario_gb300 C ABI,
               inputs already in HBM, L2 flushed between steps, the flush
               outside the CUDA-event-timed region)
  e2e          the same through the public Python API (galario_gb300.double.
               chi2Profile) with inputs in pinned host memory: every step copies
               intensity, u, v, Re, Im, w to the device and reads chi2 back
  single       the same for the FP32 module (galario_gb300.single)
  roofline     dominant kernel: algorithmic bytes / mean CUDA-event duration
  cpu_baseline the CPU oracle (C restatement of the reference CPU path) timed
               on a bounded sample on this host's cores
  batched      B=64 models of the workload, FP32 with double-float index and
               phase, chi2 and the gradient w.r.t. every profile sample and
               (inc, PA, dRA, dDec), one call per step (galario_gb300.batch)
  batched_sets B=256 single-ring profiles against 8 uneven visibility sets
               (nxy=2048), chi2 per set, with and without the gradient
  batched_images B=16 free-form 2048^2 images against the same 8 sets, chi2
               and the gradient w.r.t. every pixel and (PA, dRA, dDec)
--part plain|batched
  run only the plain (FP64/FP32 single-model) or only the batched
  measurements and print their own JSON line (for profiling runs)
--impl reference
  the reference's CPU implementation of the path (the reference build in
  oracle/_ref when present, else the C restatement oracle/_build), on all
  host cores, same workload, same metric.
"""
from __future__ import annotations

import argparse
import csv
import datetime
import io
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("chi2 evals/s, nxy=4096, 2M vis: plain FP64 vs batched FP32+grad, ≤1e-6 rel chi2")
UNIT = "evals/s"
ARCSEC = 4.84813681109536e-06
DEG = 0.017453292519943295


# ---------------------------------------------------------------------------
# workload: nxy=4096, dxy=3e-3", double-ring profile (r0 0.2"/0.6", sigma
# 0.03"/0.08", amplitudes 1:0.4, total flux 0.1 Jy), Rmin=1e-4", dR=2.5e-4"
# (the reference's central-pixel check rejects dR=1e-3" at this dxy),
# nr=4096, inc=40 deg, PA=70 deg, dRA/dDec ~ U[-0.05, 0.05]", Nvis=2e6 with
# radius log-uniform in [1e4, 4e6] wavelengths and uniform angle; noise
# sigma ~ U[0.5, 1.5] mJy on Re and Im, w = 1/sigma^2; seed 0.  Synthetic.
# ---------------------------------------------------------------------------
class Workload:
    nxy = 4096
    dxy = 3e-3 * ARCSEC
    nr = 4096
    Rmin = 1e-4 * ARCSEC
    dR = 2.5e-4 * ARCSEC
    inc = 40 * DEG
    PA = 70 * DEG
    nd = 2_000_000

    def __init__(self, seed=0):
        rng = np.random.default_rng(seed)
        R = self.Rmin + self.dR * np.arange(self.nr)
        ring = (np.exp(-0.5 * ((R - 0.2 * ARCSEC) / (0.03 * ARCSEC)) ** 2) +
                0.4 * np.exp(-0.5 * ((R - 0.6 * ARCSEC) / (0.08 * ARCSEC)) ** 2))
        trap = getattr(np, "trapezoid", None) or np.trapz
        flux = trap(ring * 2 * np.pi * R, R)
        self.intensity_scale = 0.1 / flux          # Jy/sr per unit profile
        self.intensity = ring * self.intensity_scale
        self.dRA, self.dDec = rng.uniform(-0.05, 0.05, 2) * ARCSEC
        r = np.exp(rng.uniform(np.log(1e4), np.log(4e6), self.nd))
        th = rng.uniform(0, 2 * np.pi, self.nd)
        self.u, self.v = r * np.cos(th), r * np.sin(th)
        self.sigma = rng.uniform(0.5e-3, 1.5e-3, self.nd)
        self.noise_re = rng.normal(0, self.sigma)
        self.noise_im = rng.normal(0, self.sigma)
        self.w = 1. / self.sigma ** 2

    @property
    def duv(self):
        return 1. / (self.dxy * self.nxy)

    def kw(self):
        return dict(dRA=float(self.dRA), dDec=float(self.dDec), PA=self.PA, inc=self.inc)

    def args(self):
        return (self.intensity, self.Rmin, self.dR, self.nxy, self.dxy)

    def config(self):
        return {"workload": "chi2Profile nxy=4096 dxy=3e-3\" Nvis=2e6 double-ring nr=4096 dR=2.5e-4\" "
                            "inc=40deg PA=70deg (config 1)",
                "nxy": self.nxy, "nvis": self.nd, "nr": self.nr, "global_batch": 1,
                "parallelism": "replicas", "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def window(self):
        """The part of the spectrum the kernels touch (same rule as the library)."""
        N = self.nxy
        ext = np.sqrt(np.max(self.u ** 2 + self.v ** 2)) / self.duv * (1 + 2e-6) + 1e-6
        K = min(N // 2 + 1, int(np.floor(ext)) + 2)
        kv = int(np.ceil(ext))
        r0, r1 = max(0, N // 2 - kv - 1), min(N, N // 2 + kv + 3)
        rmax = min(int(np.ceil((self.Rmin + self.nr * self.dR) / self.dxy)), N // 2)
        return K, r1 - r0, 2 * rmax


def algorithmic_bytes(wl: Workload, s: int):
    """Algorithmic HBM bytes per launch of each stage, s = bytes per real."""
    K, W, R = wl.window()
    N, nd = wl.nxy, wl.nd
    return {
        "extent": nd * 2 * s,                                  # read u, v
        "rows": R * K * 2 * s + wl.nr * s,                     # sweep fused: write R x K complex, read profile
        "cols": K * R * 2 * s + K * W * 2 * s,                 # read band rows, write window rows
        "vis": nd * 5 * s,                                     # read u, v, Re, Im, w (gathers hit L2)
        "quad": K * W * 3 * s + K * W * 16 * s,                # read window + moduli, write cell records
    }, {"K": K, "W": W, "R_rows": R}


# ---------------------------------------------------------------------------
# the large single-model image workload: chi2Image, nxy=8192, dxy=1.5e-3",
# three Gaussian rings (r0 0.2"/0.5"/0.9", sigma 0.03"/0.05"/0.08") and a
# Gaussian blob (sigma 0.02") at a seeded position within 0.5" of the centre,
# the four of equal flux, 0.1 Jy in total; Nvis=1e7 with radius log-uniform in
# [1e4, 1.5e7] wavelengths; noise as above; dRA=0.05", dDec=-0.03", PA=0;
# seed 2.  Synthetic.
# ---------------------------------------------------------------------------
class ImageWorkload:
    nxy = 8192
    dxy = 1.5e-3 * ARCSEC
    nd = 10_000_000

    def __init__(self, seed=2):
        rng = np.random.default_rng(seed)
        N = self.nxy
        x = (np.arange(N) - N / 2) * self.dxy
        r2 = x[None, :] ** 2 + x[:, None] ** 2
        rad = np.sqrt(r2)
        img = np.zeros((N, N))
        for r0, sig in ((0.2, 0.03), (0.5, 0.05), (0.9, 0.08)):
            ring = np.exp(-0.5 * ((rad - r0 * ARCSEC) / (sig * ARCSEC)) ** 2)
            img += ring * (0.025 / ring.sum())
        del rad
        rb, tb = 0.5 * np.sqrt(rng.uniform()) * ARCSEC, rng.uniform(0, 2 * np.pi)
        bx, by = rb * np.cos(tb), rb * np.sin(tb)
        blob = np.exp(-0.5 * ((x[None, :] - bx) ** 2 + (x[:, None] - by) ** 2) / (0.02 * ARCSEC) ** 2)
        img += blob * (0.025 / blob.sum())
        del blob, r2
        self.image = img
        r = np.exp(rng.uniform(np.log(1e4), np.log(1.5e7), self.nd))
        th = rng.uniform(0, 2 * np.pi, self.nd)
        self.u, self.v = r * np.cos(th), r * np.sin(th)
        sigma = rng.uniform(0.5e-3, 1.5e-3, self.nd)
        self.noise_re = rng.normal(0, sigma)
        self.noise_im = rng.normal(0, sigma)
        self.w = 1. / sigma ** 2

    @property
    def duv(self):
        return 1. / (self.dxy * self.nxy)

    def kw(self):
        return dict(dRA=0.05 * ARCSEC, dDec=-0.03 * ARCSEC, PA=0.0)

    def describe(self):
        return ("chi2Image nxy=8192 dxy=1.5e-3\" 3 rings + blob, Nvis=1e7 radius log-uniform [1e4, 1.5e7] "
                "(config 2), device-resident inputs, L2 flushed between steps")

    def algorithmic_bytes(self, s: int):
        """Algorithmic HBM bytes per launch of each kernel, s = bytes per real."""
        N, nd = self.nxy, self.nd
        ext = np.sqrt(np.max(self.u ** 2 + self.v ** 2)) / self.duv * (1 + 2e-6) + 1e-6
        K = min(N // 2 + 1, int(np.floor(ext)) + 2)
        kv = int(np.ceil(ext))
        r0, r1 = max(0, N // 2 - kv - 1), min(N, N // 2 + kv + 3)
        W = r1 - r0
        return {
            "extent": nd * 2 * s,                        # read u, v
            "rows": N * N * s + N * K * 2 * s,           # read the image, write N x K complex
            "cols": K * N * 2 * s + K * W * 3 * s,       # read K columns, write window + moduli
            "quad": K * W * 3 * s + K * W * 16 * s,      # read window + moduli, write cell records
            "vis": nd * 5 * s,                           # read u, v, Re, Im, w (gathers hit L2)
        }, {"K": K, "W": W, "R_rows": N}


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling every 20 ms from start() to stop(); summary() keeps
    the samples whose timestamps fall inside the marked timed regions."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.out = ""
        self.windows = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(0.5)  # let the first samples come in before a timed region starts
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def mark(self, t0, t1):
        """A timed region, as two datetime.now() values."""
        self.windows.append((t0, t1))

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()
            self.proc = None

    def summary(self):
        """Median SM clock and throttle reasons over the timed regions.  A
        region shorter than the sampling interval may hold no sample: it then
        takes the nearest sample within 0.25 s of it (the clock a few ms away
        from a region that ran at full load)."""
        if not self.out:
            return None
        rows = []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for row in csv.reader(io.StringIO(self.out)):
            if len(row) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(row[0].strip(), "%Y/%m/%d %H:%M:%S.%f")
                clk, cmax = float(row[2]), float(row[3])
            except ValueError:
                continue
            act = [n for n, val in zip(names, row[6:10]) if val.strip().lower() == "active"]
            rows.append((ts, clk, cmax, act))
        if not rows:
            return None
        picked, inside, nearest = {}, 0, 0
        for a, b in self.windows:
            got = [i for i, r in enumerate(rows) if a <= r[0] <= b]
            if got:
                inside += len(got)
            else:
                mid = a + (b - a) / 2
                i = min(range(len(rows)), key=lambda j: abs((rows[j][0] - mid).total_seconds()))
                if abs((rows[i][0] - mid).total_seconds()) <= 0.25 + (b - a).total_seconds() / 2:
                    got = [i]
                    nearest += 1
            for i in got:
                picked[i] = rows[i]
        if not picked:
            return None
        sel = list(picked.values())
        return {"sm_mhz": statistics.median(r[1] for r in sel), "sm_max_mhz": max(r[2] for r in sel),
                "sm_mhz_min": min(r[1] for r in sel), "samples": len(sel), "samples_inside": inside,
                "regions_nearest_sample": nearest, "regions": len(self.windows),
                "reasons": sorted({n for r in sel for n in r[3]}),
                "how": "nvidia-smi every 20 ms; samples inside the timed loops (all legs), or the nearest one"}


def profiled_traffic(stage: str, precision: str):
    """DRAM bytes per launch of a kernel from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 3 and not line.startswith("#") and parts[0] == stage and parts[1] == precision:
                return float(parts[2])
    return None


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_fp64_work(kernel: str):
    """(FP64 flops, FP64-pipe thread instructions) per visibility of a kernel
    from the committed ncu summary (flops = 2 DFMA + DADD + DMUL; the pipe
    count adds conversions and compares), or None."""
    p = os.path.join(ROOT, "profiles", "fp64_work.txt")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        for line in f:
            parts = line.split()
            if len(parts) == 3 and not line.startswith("#") and parts[0] == kernel:
                return float(parts[1]), float(parts[2])
    return None


def step_stats(ms):
    """Per-step times (ms) of a timed loop: mean, median, min, max."""
    return {"ms_mean": sum(ms) / len(ms), "ms_median": statistics.median(ms), "ms_min": min(ms),
            "ms_max": max(ms), "steps": len(ms)}


# ---------------------------------------------------------------------------
# CPU baseline (the oracle) -- only here and in --impl reference
# ---------------------------------------------------------------------------
def cpu_chi2_profile_rate(wl: Workload, re, im, steps: int, prefer_ref: bool = True):
    from oracle import oracle as O
    kind = "port"
    if prefer_ref and O.have_ref():
        impl, kind = O.get("ref", "double"), "reference"
    else:
        O.build_port()
        impl = O.get("port", "double")
    cores = len(os.sched_getaffinity(0))
    impl.threads(cores)
    args = wl.args()
    impl.chi2Profile(*args, wl.u, wl.v, re, im, wl.w, **wl.kw())  # first call dropped (speed_benchmark.py:170-172)
    t0 = time.perf_counter()
    chi2 = None
    for _ in range(steps):
        chi2 = impl.chi2Profile(*args, wl.u, wl.v, re, im, wl.w, **wl.kw())
    dt = time.perf_counter() - t0
    return steps / dt, kind, cores, chi2, dt


# ---------------------------------------------------------------------------
def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    wl = Workload()
    from oracle import oracle as O
    if not O.have_ref():
        O.build_port()
    impl = O.get("ref", "double") if O.have_ref() else O.get("port", "double")
    impl.threads(len(os.sched_getaffinity(0)))
    model = impl.sampleProfile(*wl.args(), wl.u, wl.v, **wl.kw())
    re, im = model.real + wl.noise_re, model.imag + wl.noise_im
    for _ in range(max(args.warmup, 1)):
        impl.chi2Profile(*wl.args(), wl.u, wl.v, re, im, wl.w, **wl.kw())
    rate, kind, cores, chi2, dt = cpu_chi2_profile_rate(wl, re, im, args.steps)
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": wl.config(),
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": "%d full chi2Profile evaluations (galario.double CPU path, FFT from the "
                                       "project's C FFT in place of FFTW)" % args.steps},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "chi2": chi2}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import ctypes as C

    import torch

    import galario_gb300 as g
    from galario_gb300 import _lib

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    g.double.use_gpu(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    wl = Workload(seed=0)
    L = _lib.lib()
    dev = torch.device("cuda", local)
    clock_sampler = ClockSampler(local).start()
    # a dedicated stream: the library's kernels, the L2 flush and the timing
    # events are all ordered on it
    stream = torch.cuda.Stream(dev)
    sptr = C.c_void_p(stream.cuda_stream)

    # observations: model from the product itself plus noise
    model = g.double.sampleProfile(*wl.args(), wl.u, wl.v, **wl.kw())
    re = model.real + wl.noise_re
    im = model.imag + wl.noise_im

    def to_dev(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)

    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(fn, steps, barrier=False):
        """W warm-up calls, then `steps` calls each bracketed by CUDA events on
        the library's stream, the L2 flush between them outside the events.
        Returns the per-step milliseconds and the last output."""
        out = None
        with torch.cuda.stream(stream):
            for _ in range(args.warmup):
                flush.zero_()
                out = fn()
            torch.cuda.synchronize()
            evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            if barrier and dist is not None:
                dist.barrier()
            torch.cuda.synchronize()
            d0 = datetime.datetime.now()
            for a, b in evs:
                flush.zero_()
                a.record(stream)
                out = fn()
                b.record(stream)
            torch.cuda.synchronize()
            clock_sampler.mark(d0, datetime.datetime.now())
        if barrier and dist is not None:
            dist.barrier()
        return [a.elapsed_time(b) for a, b in evs], out

    def stage_times_begin():
        _lib.check(L.galario_stage_timing(1))
        _lib.check(L.galario_stage_times((C.c_double * 8)(), (C.c_int * 8)(), 8))  # discard earlier records

    def stage_times_end():
        ms_sum = (C.c_double * 8)()
        cnt = (C.c_int * 8)()
        _lib.check(L.galario_stage_times(ms_sum, cnt, 8))
        _lib.check(L.galario_stage_timing(0))
        err = C.c_uint(0)
        _lib.check(L.galario_device_status(C.byref(err)))
        if err.value:
            raise RuntimeError("device error bits %d" % err.value)
        return {L.galario_stage_name(i).decode(): (ms_sum[i] / cnt[i] if cnt[i] else 0.0) for i in range(8)
                if cnt[i]}

    def device_rate(precision):
        dt = torch.float64 if precision == "double" else torch.float32
        R = C.c_double if precision == "double" else C.c_float
        npdt = np.float64 if precision == "double" else np.float32
        I_host = np.ascontiguousarray(wl.intensity, dtype=npdt)
        I_d = to_dev(wl.intensity, dt)
        u_d, v_d, re_d, im_d, w_d = (to_dev(x, dt) for x in (wl.u, wl.v, re, im, wl.w))
        chi2_d = torch.zeros(1, dtype=torch.float64, device=dev)
        fn = _lib.fn("chi2_profile_device", precision)
        kw = wl.kw()
        cargs = (wl.nr, I_host.ctypes.data, I_d.data_ptr(), R(wl.Rmin), R(wl.dR), R(wl.dxy), wl.nxy, R(kw["inc"]),
                 R(kw["dRA"]), R(kw["dDec"]), R(wl.duv), R(kw["PA"]), wl.nd, u_d.data_ptr(), v_d.data_ptr(),
                 re_d.data_ptr(), im_d.data_ptr(), w_d.data_ptr(), chi2_d.data_ptr(), sptr)

        def step():
            _lib.check(fn(*cargs))

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        # the rate without instrumentation; the per-stage breakdown (CUDA
        # events around every stage) from a second, shorter loop
        ms, _ = timed(step, args.steps, barrier=True)
        stage_times_begin()
        timed(step, max(3, min(args.steps, 50)))
        stages = stage_times_end()
        return ms, stages, float(chi2_d.item())

    if args.part == "batched":  # profiling runs of the batched path: the FP64 chi2 from one public call
        chi2_64 = g.double.chi2Profile(wl.intensity, wl.Rmin, wl.dR, wl.nxy, wl.dxy, wl.u, wl.v, re, im, wl.w,
                                       **wl.kw())
    elif args.part in ("all", "plain"):
        ms64_l, stages64, chi2_64 = device_rate("double")
        ms32_l, stages32, chi2_32 = device_rate("single")
        ms64, ms32 = sum(ms64_l), sum(ms32_l)
    if args.part == "plain":
        if rank == 0:
            print(json.dumps({"part": "plain", "f64_evals_per_s": world * args.steps / (ms64 / 1e3),
                              "f32_evals_per_s": world * args.steps / (ms32 / 1e3), "stages_f64": stages64,
                              "stages_f32": stages32, "f64_steps": step_stats(ms64_l),
                              "f32_steps": step_stats(ms32_l)}), flush=True)
        return 0

    # the large single-model image workload (chi2Image, nxy=8192, 1e7
    # visibilities), FP64 and FP32, with per-kernel times and HBM GB/s
    def image8192():
        iw = ImageWorkload()
        model = g.double.sampleImage(iw.image, iw.dxy, iw.u, iw.v, **iw.kw())
        ire, iim = model.real + iw.noise_re, model.imag + iw.noise_im
        del model
        out = {"workload": iw.describe(), "steps": max(20, min(args.steps, 50))}
        for precision, s in (("double", 8), ("single", 4)):
            dt = torch.float64 if precision == "double" else torch.float32
            R = C.c_double if precision == "double" else C.c_float
            img_d = to_dev(iw.image, dt)
            u_d, v_d, re_d, im_d, w_d = (to_dev(x, dt) for x in (iw.u, iw.v, ire, iim, iw.w))
            chi2_d = torch.zeros(1, dtype=torch.float64, device=dev)
            fn = _lib.fn("chi2_image_device", precision)
            kw = iw.kw()
            cargs = (iw.nxy, iw.nxy, img_d.data_ptr(), R(1.0), R(kw["dRA"]), R(kw["dDec"]), R(iw.duv), R(kw["PA"]),
                     iw.nd, u_d.data_ptr(), v_d.data_ptr(), re_d.data_ptr(), im_d.data_ptr(), w_d.data_ptr(),
                     chi2_d.data_ptr(), sptr)

            def step():
                _lib.check(fn(*cargs))

            step()
            torch.cuda.synchronize()
            ms, _ = timed(step, out["steps"])
            stage_times_begin()
            timed(step, max(3, min(out["steps"], 20)))
            stages = stage_times_end()
            alg, win = iw.algorithmic_bytes(s)
            per = {}
            for k, t in stages.items():
                if k in alg:
                    per[k] = {"ms": round(t, 4), "bytes": alg[k], "GBs": alg[k] / (t * 1e-3) / 1e9,
                              "hbm_frac": alg[k] / (t * 1e-3) / 1e9 / peaks()[0]}
            out["f64" if s == 8 else "f32"] = dict(
                {"evals_per_s": len(ms) / (sum(ms) / 1e3), "chi2": float(chi2_d.item()), "kernels": per}, **step_stats(ms))
            out["window"] = win
            del img_d, u_d, v_d, re_d, im_d, w_d
        out["rel_chi2_f32_vs_f64"] = abs(out["f32"]["chi2"] - out["f64"]["chi2"]) / abs(out["f64"]["chi2"])
        return out

    if args.part == "image8192":
        if rank == 0:
            print(json.dumps({"part": "image8192", "image8192": image8192()}), flush=True)
        return 0

    # batched FP32 + gradient: B models (model 0 = the workload's parameters,
    # the others perturbed) on the same dataset, every step computes the B
    # chi2 values and their gradients w.r.t. the 4096 profile samples and
    # (inc, PA, dRA, dDec)
    def batched_rate(B=64):
        from galario_gb300.batch import Dataset, chi2_profile_batch
        ds = Dataset(wl.u, wl.v, re, im, wl.w)
        rng = np.random.default_rng(1)
        kw = wl.kw()
        p0 = np.array([kw["inc"], kw["PA"], kw["dRA"], kw["dDec"]])
        prm = np.tile(p0, (B, 1))
        prm[1:, 0] += rng.uniform(-0.2, 0.2, B - 1)
        prm[1:, 1] += rng.uniform(-0.5, 0.5, B - 1)
        prm[1:, 2:] += rng.uniform(-0.02, 0.02, (B - 1, 2)) * ARCSEC
        scale = 1 + np.r_[0, rng.uniform(-0.1, 0.1, B - 1)]
        tI = torch.tensor(np.outer(scale, wl.intensity), dtype=torch.float32, device=dev)
        tp = torch.tensor(prm, dtype=torch.float32, device=dev)
        ms, out = timed(lambda: chi2_profile_batch(ds, tI, tp, wl.Rmin, wl.dR, wl.dxy, wl.nxy, grad=True),
                        max(20, args.steps))
        chi2_b = out[0].double().cpu().numpy()
        ds.close()
        # every model's FP32 chi2 against the FP64 module on the same inputs:
        # the dataset (stored as float32), the profiles, parameters and
        # geometry rounded to float32 as the batched call receives them
        prm32, I32 = tp.double().cpu().numpy(), tI.double().cpu().numpy()
        f32 = lambda a: np.asarray(a, dtype=np.float32).astype(np.float64)  # noqa: E731
        u32, v32, re32, im32, w32 = (f32(x) for x in (wl.u, wl.v, re, im, wl.w))
        Rmin32, dR32, dxy32 = (float(np.float32(x)) for x in (wl.Rmin, wl.dR, wl.dxy))
        # chi2's own condition number kappa = sum 2 w |r| |V| / chi2 (r the
        # residual): a relative error e common to the visibilities moves chi2
        # by up to e kappa; with strong signals (|V| >> noise) kappa is large
        def accuracy(chi2_gpu, I_rows, prm_rows):
            rel, ratio, kap = [], [], []
            for b in range(len(chi2_gpu)):
                kw_b = dict(inc=prm_rows[b, 0], PA=prm_rows[b, 1], dRA=prm_rows[b, 2], dDec=prm_rows[b, 3])
                V = g.double.sampleProfile(I_rows[b], Rmin32, dR32, wl.nxy, dxy32, u32, v32, **kw_b)
                r = np.abs(V - (re32 + 1j * im32))
                ref = float(np.sum(w32 * r * r))
                k = float(np.sum(2 * w32 * r * np.abs(V))) / ref
                rel.append(abs(chi2_gpu[b] - ref) / ref)
                kap.append(k)
                ratio.append(rel[-1] / (2.0 ** -24 * k))
            return {"max_rel_chi2_vs_f64": max(rel), "median_rel_chi2_vs_f64": float(np.median(rel)),
                    "kappa_chi2_range": [min(kap), max(kap)], "max_rel_over_2^-24_kappa": max(ratio)}
        acc_far = accuracy(chi2_b, I32, prm32)
        # walkers within 1e-3 of the observations' parameters (a fit near its optimum)
        prm_n = np.tile(p0, (B, 1)) * (1 + rng.uniform(-1e-3, 1e-3, (B, 4)))
        I_n = np.outer(1 + rng.uniform(-1e-3, 1e-3, B), wl.intensity)
        tIn = torch.tensor(I_n, dtype=torch.float32, device=dev)
        tpn = torch.tensor(prm_n, dtype=torch.float32, device=dev)
        ds = Dataset(wl.u, wl.v, re, im, wl.w)
        chi2_n = chi2_profile_batch(ds, tIn, tpn, wl.Rmin, wl.dR, wl.dxy, wl.nxy).double().cpu().numpy()
        ds.close()
        acc_near = accuracy(chi2_n, tIn.double().cpu().numpy(), tpn.double().cpu().numpy())
        return dict({"value": B * len(ms) / (sum(ms) * 1e-3), "unit": UNIT, "B": B, "dtype": "f32",
                     "gradient": "chi2 and dchi2/d(4096 profile samples, inc, PA, dRA, dDec) per model",
                     "ms_per_step": sum(ms) / len(ms),
                     "max_rel_chi2_vs_f64_all_models": acc_far["max_rel_chi2_vs_f64"],
                     "accuracy_timed_models": dict(acc_far, models="model 0 at the observations' parameters, "
                                                   "63 with inc +-0.2 rad, PA +-0.5 rad, offsets +-0.02\", "
                                                   "scale +-10 %"),
                     "accuracy_near_optimum": dict(acc_near, models="64 walkers within 1e-3 (relative) of the "
                                                   "observations' parameters"),
                     # model setup, fold/rows, two products or cols, vis, finalize, cell adjoint, two products
                     # or colsT/rowsT, sweep adjoint + its reduction (tensor-core path), central, params
                     "gpu_launches_per_step": 13 if os.environ.get("GALARIO_TC", "1") != "0" else 10},
                    **step_stats(ms))

    # the multi-dataset workload: B single-ring profiles, nxy=2048, dxy=5e-3",
    # Rmin=1e-4", dR=4e-4", nr=4096; 8 visibility sets with nd_k ~ U[2e5, 3e6],
    # radius log-uniform in [1e4, 2e6] wavelengths, seed 1000 + k
    def sets_workload():
        sets = []
        for k in range(8):
            r = np.random.default_rng(1000 + k)
            n = int(r.uniform(2e5, 3e6))
            rad = np.exp(r.uniform(np.log(1e4), np.log(2e6), n))
            th = r.uniform(0, 2 * np.pi, n)
            sig = r.uniform(0.5e-3, 1.5e-3, n)
            sets.append((rad * np.cos(th), rad * np.sin(th), r.normal(0, sig), r.normal(0, sig), 1 / sig ** 2))
        return sets

    def batched_sets_rate(ds, B=256):
        from galario_gb300.batch import chi2_profile_batch
        nxy, dxy, Rmin, dR, nr = 2048, 5e-3 * ARCSEC, 1e-4 * ARCSEC, 4e-4 * ARCSEC, 4096
        r = np.random.default_rng(7)
        R = Rmin + dR * np.arange(nr)
        r0, sig = r.uniform(0.1, 0.8, B) * ARCSEC, r.uniform(0.01, 0.1, B) * ARCSEC
        flux = r.uniform(0.05, 0.2, B)
        prof = np.exp(-0.5 * ((R[None, :] - r0[:, None]) / sig[:, None]) ** 2)
        prof *= (flux / (2 * np.pi * (prof * R[None, :]).sum(axis=1) * dR))[:, None]  # Jy/sr
        prm = np.c_[r.uniform(0, 70, B) * DEG, r.uniform(0, 180, B) * DEG, np.zeros(B), np.zeros(B)]
        tI = torch.tensor(prof, dtype=torch.float32, device=dev)
        tp = torch.tensor(prm, dtype=torch.float32, device=dev)
        out = {"B": B, "nsets": ds.nsets, "nvis": ds.nd, "nxy": nxy, "unit": UNIT}
        for grad in (False, True):
            ms, _ = timed(lambda: chi2_profile_batch(ds, tI, tp, Rmin, dR, dxy, nxy, grad=grad, per_set=True),
                          max(20, min(args.steps, 40)))
            out["grad" if grad else "forward"] = dict({"value": B * len(ms) / (sum(ms) * 1e-3),
                                                       "ms_per_step": sum(ms) / len(ms)}, **step_stats(ms))
        return out

    def batched_images_rate(ds, B=16):
        from galario_gb300.batch import chi2_image_batch
        nxy, dxy = 2048, 5e-3 * ARCSEC
        r = np.random.default_rng(8)
        x = (np.arange(nxy) - nxy / 2) * dxy
        X, Y = np.meshgrid(x, x)
        rad = np.hypot(X, Y)
        imgs = torch.empty((B, nxy, nxy), dtype=torch.float32, device=dev)
        for b in range(B):
            ring = np.exp(-0.5 * ((rad - r.uniform(0.2, 0.8) * ARCSEC) / (r.uniform(0.03, 0.1) * ARCSEC)) ** 2)
            ring += r.normal(0, 1e-4, ring.shape)
            imgs[b] = torch.from_numpy(ring * (0.1 / ring.sum()))
        tp = torch.tensor(np.c_[r.uniform(0, np.pi, B), r.uniform(-0.05, 0.05, (B, 2)) * ARCSEC],
                          dtype=torch.float32, device=dev)
        ms, _ = timed(lambda: chi2_image_batch(ds, imgs, tp, dxy, grad=True), max(20, min(args.steps, 40)))
        return dict({"value": B * len(ms) / (sum(ms) * 1e-3), "unit": UNIT, "B": B, "nxy": nxy, "nsets": ds.nsets,
                     "nvis": ds.nd, "ms_per_step": sum(ms) / len(ms),
                     "gradient": "chi2 and dchi2/d(every pixel, PA, dRA, dDec) per image"}, **step_stats(ms))

    batched = batched_rate()
    from galario_gb300.batch import Dataset as _Dataset
    _sets = sets_workload()
    ds_sets = _Dataset(*[[st[i] for st in _sets] for i in range(5)])
    del _sets
    batched_sets = batched_sets_rate(ds_sets)
    batched_images = batched_images_rate(ds_sets)
    ds_sets.close()
    if args.part == "batched":
        if rank == 0:
            print(json.dumps({"part": "batched", "batched": batched, "batched_sets": batched_sets,
                              "batched_images": batched_images}), flush=True)
        return 0
    img8192 = image8192()

    # max over ranks of the timed region
    t_local = ms64 / 1e3
    if dist is not None:
        t = torch.tensor([t_local], dtype=torch.float64, device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_local = float(t.item())
    value = world * args.steps / t_local

    # e2e: public API, host inputs, H2D + D2H inside every step; pinned
    # (page-locked) host arrays, and plain (pageable) numpy arrays as a
    # drop-in caller passes them
    def pinned(a, dt):
        t = torch.empty(len(a), dtype=dt, pin_memory=True)
        arr = t.numpy()
        arr[:] = a
        return t, arr

    def e2e_rate(host):
        chi2 = None
        for _ in range(max(1, min(args.warmup, 3))):
            chi2 = g.double.chi2Profile(host["I"], wl.Rmin, wl.dR, wl.nxy, wl.dxy, host["u"], host["v"], host["re"],
                                        host["im"], host["w"], **wl.kw())
        if dist is not None:
            dist.barrier()
        d0 = datetime.datetime.now()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            chi2 = g.double.chi2Profile(host["I"], wl.Rmin, wl.dR, wl.nxy, wl.dxy, host["u"], host["v"],
                                        host["re"], host["im"], host["w"], **wl.kw())
        dt = time.perf_counter() - t0
        clock_sampler.mark(d0, datetime.datetime.now())
        if dist is not None:
            t = torch.tensor([dt], dtype=torch.float64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dt = float(t.item())
        return world * args.steps / dt, chi2

    keep = []
    host = {}
    for name, a in (("I", wl.intensity), ("u", wl.u), ("v", wl.v), ("re", re), ("im", im), ("w", wl.w)):
        t, arr = pinned(a, torch.float64)
        keep.append(t)
        host[name] = arr
    e2e_value, e2e_chi2 = e2e_rate(host)
    e2e_pageable, _ = e2e_rate({"I": wl.intensity, "u": wl.u, "v": wl.v, "re": re, "im": im, "w": wl.w})
    clock_sampler.stop()
    clocks = clock_sampler.summary()
    h2d_bytes = 8 * (wl.nr + 5 * wl.nd)
    d2h_bytes = 64  # device state block carrying chi2 and the error bits

    line = None
    if rank == 0:
        hbm, peak_kind = peaks()
        alg, win = algorithmic_bytes(wl, 8)
        dom = max((k for k in stages64 if k in alg), key=lambda k: stages64[k])
        achieved = alg[dom] / (stages64[dom] * 1e-3) / 1e9
        fp64_peak = C.c_double(0.0)
        _lib.check(L.galario_measure_fp64_peak(C.byref(fp64_peak)))
        work = profiled_fp64_work("vis_kernel_f64_profile") if dom == "vis" else None
        rate_cpu, kind, cores, chi2_cpu, dt_cpu = cpu_chi2_profile_rate(wl, re, im, steps=2)
        alg32, _ = algorithmic_bytes(wl, 4)
        roof = {"kernel": dom, "algorithmic_bytes": alg[dom],
                "traffic": profiled_traffic(dom, "f64"),
                "traffic_source": "profiles/dram_traffic.txt (ncu dram__bytes_read+write of one launch)",
                "hbm": {"achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                        "peak_source": peak_kind + " (MEASURED_PEAKS.json hbm_gbs)"}}
        if work is not None:
            # the FP64 pipe binds this kernel: its fraction is the primary one.
            # achieved = FP64-pipe thread instructions per second (ncu count per
            # visibility x visibilities / live event time); peak = the measured
            # FP64 FMA rate in instructions per second (flops / 2)
            flops_pv, inst_pv = work
            t = stages64[dom] * 1e-3
            roof.update({"bound": "fp64", "achieved": inst_pv * wl.nd / t / 1e9, "peak": fp64_peak.value / 2,
                         "unit": "G FP64-pipe instr/s", "frac": inst_pv * wl.nd / t / 1e9 / (fp64_peak.value / 2),
                         "fp64_gflops": flops_pv * wl.nd / t / 1e9, "fp64_peak_gflops": fp64_peak.value,
                         "peak_source": "measured in this run (galario_measure_fp64_peak: FP64 FMA chains)",
                         "per_vis": {"fp64_flops": flops_pv, "fp64_pipe_instr": inst_pv},
                         "work_source": "profiles/fp64_work.txt (ncu FP64 thread instructions of one launch "
                                        "/ visibilities)"})
        else:
            roof.update({"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                         "fp64_peak_gflops": fp64_peak.value})
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms64 / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": wl.config(),
            "step_stats": step_stats(ms64_l),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes,
                    "d2h_bytes_per_step": d2h_bytes, "api": "galario_gb300.double.chi2Profile, pinned numpy inputs",
                    "pageable": {"value": e2e_pageable, "api": "the same call with plain (pageable) numpy inputs"}},
            "roofline": roof,
            "stages_ms": {k: round(v, 4) for k, v in stages64.items()},
            "window": win,
            "single": {"value": world * args.steps / (ms32 / 1e3), "unit": UNIT, "dtype": "f32",
                       "ms_per_step": ms32 / args.steps, "stages_ms": {k: round(v, 4) for k, v in stages32.items()},
                       "rel_chi2_vs_f64": abs(chi2_32 - chi2_64) / abs(chi2_64),
                       "vis_GBs": alg32["vis"] / (stages32.get("vis", 1e9) * 1e-3) / 1e9},
            "batched": dict(batched, ratio_vs_plain_f64=batched["value"] / value),
            "batched_sets": batched_sets,
            "batched_images": batched_images,
            "image8192": img8192,
            "cpu_baseline": {"value": rate_cpu, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": "2 full chi2Profile evaluations (FP64, FFT from the project's C FFT in place "
                                       "of FFTW), first call dropped"},
            "parity": {"chi2_f64": chi2_64, "chi2_e2e": e2e_chi2, "chi2_cpu": chi2_cpu,
                       "rel_f64_vs_cpu": abs(chi2_64 - chi2_cpu) / abs(chi2_cpu)},
            # per FP64 step (ncu launch list): extent, the sweep's digits, two
            # tensor-core products with the pass between them, the window,
            # the cell records, vis; with GALARIO_TC=0: extent, rows, cols,
            # cell records, vis
            "gpu_launches": (8 if os.environ.get("GALARIO_TC", "1") != "0" else 5) * args.steps,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--part", choices=["all", "plain", "batched", "image8192"], default="all")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
