"""Benchmark of the ERA / DM reconstruction loop on one GB300 (or N replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload c1|c0]

Workload c1 (default, the headline): 1024 frames of 256 x 256 on a 32 x 32
raster (step 24 px, +-3 px seeded jitter), object 1024 x 1024 (Gaussian-filtered
random amplitude 0.5-1 and phase +-pi/2), probe a 64 px aperture with an 8 px
Gaussian edge and quadratic phase, initial probe with that phase coefficient
x1.2, additive background 0.01 mean(I) x smooth blob, Poisson noise at 1e6
photons per frame, mask = 12 px beamstop + 0.5 % dead pixels.  All synthetic
and seeded.  One step = one ERA iteration (method 6: object + probe +
background) followed by one DM iteration (method 6) over all 1024 frames.
Workload c0: 100 frames of 128 x 128, object 320 x 320, noise free, ERA method 1.

Metric: frame-iterations per second (n_frames x iterations / s).  `value` is
timed with CUDA events around device-resident steps; `e2e` runs the public
pty.ERA / pty.DM calls on host arrays.  The exit waves (537 MB at c1) exceed the
126 MB L2, so no L2 flush is needed between steps.

--impl reference times the CPU oracle (a NumPy port of the reference's
era.py / dm.py) on the host cores: one process per core, each on its own
disjoint shard of frames (no all-reduce), every step a bounded sample.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)


# --------------------------------------------------------------------------- workloads
def _smooth01(rng, shape, sigma=4.0):
    import scipy.ndimage as ndi
    a = ndi.gaussian_filter(rng.random(shape), sigma)
    return (a - a.min()) / (a.max() - a.min())


def make_object(rng, U):
    return (0.5 + 0.5 * _smooth01(rng, (U, U))) * np.exp(1j * np.pi * (_smooth01(rng, (U, U)) - 0.5))


def make_probe(N, radius, edge, quad):
    y, x = np.mgrid[:N, :N] - N / 2
    r = np.sqrt(x ** 2 + y ** 2)
    amp = np.exp(-np.clip(r - radius, 0, None) ** 2 / (2 * edge ** 2)) * (r < radius + 3 * edge)
    return amp * np.exp(1j * quad * r ** 2)


def raster(rng, side, step, jitter, N, U, offset=4):
    pos = np.arange(side) * step + offset
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = R + rng.integers(-jitter, jitter + 1, R.shape)
    return np.clip(R, -(U - N), 0).astype(np.int64)


class Workload:
    pass


def workload_c1(exits_fn, frames=None):
    """The 256^2 / 1024-frame job; `exits_fn(O, P, R)` returns |FFT2(P O[R])|^2 per frame."""
    rng = np.random.default_rng(1)
    N, U, side = 256, 1024, 32
    w = Workload()
    w.name = "c1"
    w.O_true = make_object(rng, U)
    w.P_true = make_probe(N, 64, 8, 0.0005)
    w.P0 = make_probe(N, 64, 8, 0.0006)
    w.R = raster(rng, side, 24, 3, N, U)
    if frames is not None:
        w.R = w.R[frames]
    I = exits_fn(w.O_true, w.P_true, w.R)                      # unshifted |F|^2
    y, x = np.mgrid[:N, :N] - N / 2
    blob = np.fft.ifftshift(np.exp(-(x ** 2 + y ** 2) / (2 * 40.0 ** 2)))
    I = I + 0.01 * I.mean() * blob
    I = I * (1e6 / I.sum(axis=(1, 2), keepdims=True))
    I = rng.poisson(I).astype(np.float32)
    w.I = np.fft.fftshift(I, axes=(-2, -1))                    # centred, as recorded
    M = np.ones((N, N), bool)
    M[np.sqrt(x ** 2 + y ** 2) < 12] = False
    M[rng.random((N, N)) < 0.005] = False
    w.M = M
    w.method = 6
    w.N, w.U = N, U
    return w


def workload_c0(exits_fn):
    rng = np.random.default_rng(0)
    N, U = 128, 320
    w = Workload()
    w.name = "c0"
    w.O_true = make_object(rng, U)
    w.P_true = make_probe(N, 32, 4, 0.002)
    w.P0 = w.P_true
    w.R = raster(rng, 10, 16, 2, N, U, offset=16)
    w.I = np.fft.fftshift(exits_fn(w.O_true, w.P_true, w.R), axes=(-2, -1)).astype(np.float32)
    w.M = np.ones((N, N), bool)
    w.method = 1
    w.N, w.U = N, U
    return w


class DeviceWorkload:
    """The 512^2 / 4096-frame job, generated and kept on the device.

    64 x 64 raster, step 36 px, +-4 px jitter, object 2816 x 2816 built like the
    other workloads, 128 px aperture probe with a 16 px edge (initial probe: its
    quadratic phase coefficient x1.2), background 0.01 mean(I) x smooth blob,
    Poisson noise at 1e8 photons per frame (torch's seeded sampler, data
    generation only), beamstop + 0.5 % dead-pixel mask.  The background buffer
    is initialised from the known blob (DM method 6 with a given background).
    """

    def __init__(self, dev, frames=None):
        import torch
        from ptychography_gb300 import _native
        rng = np.random.default_rng(4)
        N, U, side = 512, 2816, 64
        self.name, self.method, self.N, self.U = "c4", 6, N, U
        self.O_true = make_object(rng, U)
        self.P_true = make_probe(N, 128, 16, 0.0001)
        self.P0 = make_probe(N, 128, 16, 0.00012)
        self.R = raster(rng, side, 36, 4, N, U)
        if frames:      # the first frames of the scan (profiling a smaller case)
            self.R = self.R[:frames]
        lib = _native.load()
        n = len(self.R)
        plan = ctypes.c_void_p()
        R64 = np.ascontiguousarray(self.R, dtype=np.int64)
        _native.check(lib.pty_plan_create(ctypes.byref(_native.Geometry(n, N, N, U, U)),
                                          R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                          ctypes.byref(plan)))
        p = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
        sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        O_d = torch.from_numpy(self.O_true.astype(np.complex64)).to(dev)
        P_d = torch.from_numpy(self.P_true.astype(np.complex64)).to(dev)
        I = torch.empty((n, N, N), dtype=torch.float32, device=dev)
        _native.check(lib.pty_intensities(plan, p(O_d), p(P_d), p(I), sp))   # centred |F|^2
        lib.pty_plan_destroy(plan)
        y, x = np.mgrid[:N, :N] - N / 2
        blob = torch.from_numpy(np.exp(-(x ** 2 + y ** 2) / (2 * 80.0 ** 2)).astype(np.float32)).to(dev)
        I += 0.01 * I.mean() * blob
        I *= 1e8 / I.sum(dim=(1, 2), keepdim=True)
        gen = torch.Generator(device=dev)
        gen.manual_seed(4)
        self.I_dev = torch.poisson(I, generator=gen)
        del I
        M = np.ones((N, N), bool)
        M[np.sqrt(x ** 2 + y ** 2) < 12] = False
        M[rng.random((N, N)) < 0.005] = False
        self.M = M
        self.B = (0.01 * float(self.I_dev.mean()) * blob).cpu().numpy()   # known background


def numpy_intensities(O, P, R):
    """|FFT2(P O[R])|^2 on the host (used only where no GPU is involved)."""
    N = P.shape[0]
    rows = (np.arange(N)[None, :] - R[:, 0:1])
    cols = (np.arange(N)[None, :] - R[:, 1:2])
    out = np.empty((len(R), N, N))
    for i in range(0, len(R), 64):
        ex = O[rows[i:i + 64, :, None], cols[i:i + 64, None, :]] * P
        out[i:i + 64] = np.abs(np.fft.fft2(ex)) ** 2
    return out


def gpu_intensities(O, P, R):
    from ptychography_gb300.forward_models import diffraction_intensities
    I = diffraction_intensities(O, P, R)                       # fftshift(|F|^2)
    return np.fft.ifftshift(I, axes=(-2, -1))


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi's start-up (NVML initialisation) must not fall inside
            # the timed region: wait for its first sample (it stalled a
            # 3-step timing by ~1 s otherwise)
            t0 = time.perf_counter()
            while not self.rows and self.proc.poll() is None and time.perf_counter() - t0 < 10.0:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 5 + i and r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# --------------------------------------------------------------------------- GPU arm
class DeviceJob:
    """Device-resident ERA/DM state of a workload, driven through the C ABI."""

    def __init__(self, w, dev):
        import torch
        from ptychography_gb300 import _engine, _native
        self.torch, self.lib, self.native = torch, _native.load(), _native
        self.w, self.dev = w, dev
        if isinstance(w, DeviceWorkload):
            self._init_device(w, dev)
            return
        np.random.seed(12)
        pre = _engine.Preamble(w.I, w.R.copy(), w.P0, None, 1, w.M, None, w.method, "single")
        self.pre = pre
        n, N0, N1 = pre.n, pre.N0, pre.N1
        U, V = pre.O.shape
        self.n, self.N, self.U, self.V = n, N0, U, V
        R64 = np.ascontiguousarray(pre.R[:, :2], dtype=np.int64)
        self.plan = ctypes.c_void_p()
        _native.check(self.lib.pty_plan_create(ctypes.byref(_native.Geometry(n, N0, N1, U, V)),
                                               R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                               ctypes.byref(self.plan)))
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
        I_d = t(pre.I.astype(np.float32))
        self.amp = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
        _native.check(self.lib.pty_amp_from_intensity(self.plan, self.p(I_d), 0, self.p(self.amp),
                                                      self.sp()))
        del I_d
        self.O0 = pre.O.astype(np.complex64)
        self.O = t(self.O0)
        self.P = t(pre.P.astype(np.complex64))
        self.psi = torch.empty((n, N0, N1), dtype=torch.complex64, device=dev)
        self.mask = t(pre.mask) if pre.mask is not None else None
        self.bg = t(pre.background) if pre.background is not None else None
        self.bmean = torch.zeros((N0, N1), dtype=torch.float32, device=dev)
        self.heat = torch.zeros((U, V), dtype=torch.float64, device=dev)
        self.emod = torch.zeros(4096, dtype=torch.float64, device=dev)
        self.econ = torch.zeros(4096, dtype=torch.float64, device=dev)
        self.I_norm = pre.I_norm

    def _init_device(self, w, dev):
        """Preamble of era.py:435-548 on device-resident intensities (no host copy)."""
        torch, nat, lib = self.torch, self.native, self.lib
        n, N, U = len(w.R), w.N, w.U
        R = w.R.copy()
        R[:, 0] -= R[:, 0].max()
        R[:, 1] -= R[:, 1].max()
        U = N + int(R[:, 0].max() - R[:, 0].min())
        V = N + int(R[:, 1].max() - R[:, 1].min())
        self.n, self.N, self.U, self.V = n, N, U, V
        R64 = np.ascontiguousarray(R, dtype=np.int64)
        self.plan = ctypes.c_void_p()
        nat.check(lib.pty_plan_create(ctypes.byref(nat.Geometry(n, N, N, U, V)),
                                      R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      ctypes.byref(self.plan)))
        self.amp = torch.empty((n, N, N), dtype=torch.float32, device=dev)
        nat.check(lib.pty_amp_from_intensity(self.plan, self.p(w.I_dev), 0, self.p(self.amp), self.sp()))
        mask_c = torch.from_numpy(w.M.astype(np.float32)).to(dev)
        self.I_norm = float((w.I_dev * mask_c).sum(dtype=torch.float64))
        self.O0 = np.ones((U, V), np.complex64)
        self.O = torch.from_numpy(self.O0).to(dev)
        self.P = torch.from_numpy(w.P0.astype(np.complex64)).to(dev)
        self.psi = torch.empty((n, N, N), dtype=torch.complex64, device=dev)
        self.mask = torch.from_numpy(np.fft.ifftshift(w.M).astype(np.uint8)).to(dev)
        b = torch.from_numpy(np.sqrt(np.fft.ifftshift(w.B)).astype(np.float32)).to(dev)
        self.bg = b.expand(n, N, N).contiguous()
        self.start = (self.P.clone(), b)          # the initial probe and background (reset())
        self.bmean = torch.zeros((N, N), dtype=torch.float32, device=dev)
        self.heat = torch.zeros((U, V), dtype=torch.float64, device=dev)
        self.emod = torch.zeros(4096, dtype=torch.float64, device=dev)
        self.econ = torch.zeros(4096, dtype=torch.float64, device=dev)

    def p(self, x):
        return ctypes.c_void_p(x.data_ptr()) if x is not None else None

    def sp(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def run(self, kind, method, iters):
        nat = self.native
        buf = nat.Buffers(self.p(self.O), self.p(self.P), self.p(self.psi), self.p(self.amp),
                          self.p(self.mask), self.p(self.bg), None, self.p(self.bmean),
                          self.p(self.heat), None, self.p(self.emod), self.p(self.econ))
        opt = nat.Options(method, 1, 1, 0, 0, 1, 1e-10, self.I_norm)
        hv = ctypes.c_int32(0)
        fn = self.lib.pty_era if kind == "era" else self.lib.pty_dm
        nat.check(fn(self.plan, ctypes.byref(buf), ctypes.byref(opt), iters, ctypes.byref(hv), self.sp()))

    def reset(self, O_init):
        """Back to the workload's start (initial probe and background, device
        workloads only) with the object O_init."""
        self.O.copy_(O_init)
        P0, b = self.start
        self.P.copy_(P0)
        self.bg.copy_(b.expand_as(self.bg))

    def step(self):
        if self.w.name == "c4":
            self.run("dm", 6, 1)
        elif self.w.method == 6:
            self.run("era", 6, 1)
            self.run("dm", 6, 1)
        else:
            self.run("era", self.w.method, 1)

    def frames_per_step(self):
        return self.n * (2 if self.w.name == "c1" else 1)

    def close(self):
        self.lib.pty_plan_destroy(self.plan)


class BatchJob:
    """64 independent ERA reconstructions of uneven size, run together.

    Per problem (seeded): frame size N drawn from {64, 128, 192, 256}, scan
    count from 50..2000 positions on a jittered square raster whose step gives
    40-60 % probe overlap, probe an N/4-radius aperture with an N/32 edge and a
    quadratic phase scaled to the aperture (initial probe: coefficient x1.2),
    object cropped from one large Gaussian-filtered random object, Poisson
    noise at 10^U(5,7) photons per frame, FP32.  Intensities are formed and
    kept on the device.  Each reconstruction is ERA method 3 (object + probe)
    from an object of ones.  A step is `iters` iterations of all 64
    reconstructions in one pty_run_batch call: one CUDA-graph launch holding
    one branch per reconstruction.
    """

    def __init__(self, dev, count=64, iters=10, seed=2):
        import torch
        from ptychography_gb300 import _native
        self.torch, self.nat, self.lib, self.dev = torch, _native, _native.load(), dev
        self.iters, self.count = iters, count
        rng = np.random.default_rng(seed)
        specs = []
        for _ in range(count):
            N = int(rng.choice([64, 128, 192, 256]))
            n = int(rng.integers(50, 2001))
            ov = float(rng.uniform(0.4, 0.6))
            rad = N / 4
            step = max(1, int(round(2 * rad * (1 - ov))))
            side = int(math.ceil(math.sqrt(n)))
            jit = max(1, step // 8)
            U = N + step * (side - 1) + 2 * jit + 8
            specs.append((N, n, rad, step, side, jit, U, 10 ** rng.uniform(5, 7)))
        Umax = max(sp[6] for sp in specs)
        master = make_object(rng, Umax)
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        self.jobs, self.frames, self.sizes = [], 0, []
        sp_ = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
        self.p = p
        for (N, n, rad, step, side, jit, U, photons) in specs:
            quad = 0.002 * (32.0 / rad) ** 2
            P_true = make_probe(N, rad, N / 32, quad)
            P0 = make_probe(N, rad, N / 32, 1.2 * quad)
            R = raster(rng, side, step, jit, N, U, offset=jit + 4)[:n]
            o0 = int(rng.integers(0, Umax - U + 1))
            O_true = master[o0:o0 + U, o0:o0 + U]
            R = R - R.max(axis=0)
            Ur = N + int(R[:, 0].max() - R[:, 0].min())
            Vr = N + int(R[:, 1].max() - R[:, 1].min())
            R64 = np.ascontiguousarray(R, dtype=np.int64)
            plan = ctypes.c_void_p()
            _native.check(self.lib.pty_plan_create(
                ctypes.byref(_native.Geometry(n, N, N, Ur, Vr)),
                R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ctypes.byref(plan)))
            Ot = torch.from_numpy(np.ascontiguousarray(O_true[:Ur, :Vr]).astype(np.complex64)).to(dev)
            Pt = torch.from_numpy(P_true.astype(np.complex64)).to(dev)
            I = torch.empty((n, N, N), dtype=torch.float32, device=dev)
            _native.check(self.lib.pty_intensities(plan, p(Ot), p(Pt), p(I), sp_))
            I *= photons / I.sum(dim=(1, 2), keepdim=True)
            I = torch.poisson(I, generator=gen)
            amp = torch.empty_like(I)
            _native.check(self.lib.pty_amp_from_intensity(plan, p(I), 0, p(amp), sp_))
            I_norm = float(I.sum(dtype=torch.float64))
            del I, Ot
            j = dict(plan=plan, amp=amp, n=n, N=N,
                     O=torch.ones((Ur, Vr), dtype=torch.complex64, device=dev),
                     P=torch.from_numpy(P0.astype(np.complex64)).to(dev),
                     psi=torch.empty((n, N, N), dtype=torch.complex64, device=dev),
                     heat=torch.zeros((Ur, Vr), dtype=torch.float64, device=dev),
                     emod=torch.zeros(iters, dtype=torch.float64, device=dev),
                     econ=torch.zeros(iters, dtype=torch.float64, device=dev), I_norm=I_norm)
            self.jobs.append(j)
            self.frames += n
            self.sizes.append(N)
        torch.cuda.synchronize()
        k = len(self.jobs)
        self.plans = (ctypes.c_void_p * k)(*[j["plan"].value for j in self.jobs])
        self.bufs = (_native.Buffers * k)(*[self.buffers(j) for j in self.jobs])
        self.opts = (_native.Options * k)(*[_native.Options(3, 1, 1, 0, 0, 1, 1e-10, j["I_norm"])
                                            for j in self.jobs])
        self.hv = (ctypes.c_int32 * k)()

    def buffers(self, j):
        p = self.p
        return self.nat.Buffers(p(j["O"]), p(j["P"]), p(j["psi"]), p(j["amp"]), None, None, None,
                                None, p(j["heat"]), None, p(j["emod"]), p(j["econ"]))

    def sp(self):
        return ctypes.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def step(self):
        self.nat.check(self.lib.pty_run_batch(0, self.plans, self.bufs, self.opts, len(self.jobs),
                                              self.iters, self.hv, self.sp()))

    def step_one_by_one(self):
        """The same iterations as separate per-reconstruction pty_era calls (graph each)."""
        hv = ctypes.c_int32(0)
        for r in range(len(self.jobs)):
            self.nat.check(self.lib.pty_era(self.plans[r], ctypes.byref(self.bufs[r]),
                                            ctypes.byref(self.opts[r]), self.iters,
                                            ctypes.byref(hv), self.sp()))

    def frames_per_step(self):
        return self.frames * self.iters

    def close(self):
        for j in self.jobs:
            self.lib.pty_plan_destroy(j["plan"])


def batched_rate(dev, steps=20):
    """Batched form: 64 reconstructions x 200 iterations (20 steps of 10)."""
    import torch
    t0 = time.perf_counter()
    job = BatchJob(dev)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    job.step()                                   # capture + first launch
    torch.cuda.synchronize()
    capture_s = time.perf_counter() - t0
    for _ in range(2):
        job.step()
    t = event_time(torch, job.step, steps)
    job.step_one_by_one()                        # capture the per-problem graphs
    t_seq = event_time(torch, job.step_one_by_one, 2)
    eml = [float(j["emod"][job.iters - 1]) for j in job.jobs]
    out = {"workload": "64 ERA-m3 reconstructions, frames %s, %d frames in all, %d iterations"
                       % ({N: job.sizes.count(N) for N in sorted(set(job.sizes))}, job.frames,
                          job.iters * steps),
           "frame_iters_per_s": round(job.frames_per_step() * steps / t, 1),
           "seconds": round(t, 3),
           "one_by_one_frame_iters_per_s": round(job.frames_per_step() * 2 / t_seq, 1),
           "graph_capture_s": round(capture_s, 3), "data_generation_s": round(gen_s, 1),
           "final_eMod_median": round(statistics.median(eml), 5)}
    # algorithmic bytes per frame-iteration of ERA method 3: the fused frame
    # pass reads the amplitudes (4 N^2) and writes the exit waves (8 N^2; the
    # object window and probe come from L2), the object and probe gathers
    # read the exit waves once each (8 N^2 + 8 N^2)
    byts = 28.0 * sum(j["n"] * j["N"] * j["N"] for j in job.jobs) * job.iters * steps
    pk, kind = peaks()
    out["roofline"] = {"bound": "hbm", "achieved": round(byts / t / 1e9, 1), "peak": pk, "unit": "GB/s",
                       "frac": round(byts / t / 1e9 / pk, 4), "peak_kind": kind,
                       "algorithmic_bytes_per_frame_iter": "28 N^2 (amplitudes 4, exit waves written 8, "
                                                           "read by the object and probe gathers 8 + 8)"}
    job.close()
    return out


def event_time(torch, fn, reps):
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / 1e3


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def roofline_pmod7(job, torch, tile, sm_max_mhz, reps=20):
    """Fused frame kernel (Pmod_7 form, the DM m6 modulus step) alone, event-timed.

    Algorithmic bytes per frame: psi read 8 N^2 + psi write 8 N^2 + amp 4 N^2 +
    background read 4 N^2 + background write 4 N^2 = 28 N^2.
    """
    lib, p = job.lib, job.p
    job.lib.pty_make_exits(job.plan, p(job.O), p(job.P), p(job.psi), job.sp())
    bg = job.bg if job.bg is not None else torch.ones_like(job.amp)
    fn = lambda: lib.pty_pmod_7(job.plan, p(job.amp), p(bg), p(job.psi), p(job.mask), 1e-10, None,  # noqa: E731
                                job.sp())
    for _ in range(3):
        fn()
    t = event_time(torch, fn, reps) / reps
    bytes_ = 28.0 * job.N * job.N * job.n
    # DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one ncu
    # capture, scaled by frames, for the two tiles the benchmark workloads run
    # on: the 256^2 8-CTA tile (880.7 MB for 512 frames) and the staged 512^2
    # tile's three launches (3864.6 MB for 256 frames)
    traffic = None
    if job.N == 256 and tile == 8:
        traffic = round(880.7e6 * job.n / 512)
    elif job.N == 512 and tile == 264:
        traffic = round(3864.6e6 * job.n / 256)
    if tile > 200:      # staged: row, column and row launches through a frame scratch
        kname = "staged_rows_kernel<PSI7> + staged_cols_kernel<PSI7> + staged_rows_kernel<PSI7>"
    elif tile > 100:    # three-stage line transforms
        kname = "line3_cluster_kernel<PSI7>" if job.N == 256 else "line3_512_kernel<PSI7>"
    elif tile > 1:
        kname = "cluster_frame_kernel<%d,%d,PSI7>" % (job.N, tile)
    else:
        kname = "frame_kernel<%d,%d,PSI7>" % (job.N, job.N)
    pk, kind = peaks()
    gbs = bytes_ / t / 1e9
    # FP32 side: 5 N^2 log2(N^2) flops per 2-D transform, forward + inverse,
    # against 2 flops x 128 FP32 lanes x SMs x the SM clock
    flops = 10.0 * job.N * job.N * math.log2(job.N * job.N) * job.n
    props = torch.cuda.get_device_properties(job.dev)
    fp32_peak = 2 * 128 * props.multi_processor_count * sm_max_mhz * 1e6
    return {"kernel": kname,
            "bound": "hbm", "achieved": round(gbs, 1), "peak": pk, "unit": "GB/s",
            "frac": round(gbs / pk, 4), "peak_kind": kind, "traffic": traffic,
            "launch_ms": round(t * 1e3, 4), "algorithmic_bytes": bytes_,
            "fp32": {"flops_per_launch": flops, "achieved_tflops": round(flops / t / 1e12, 2),
                     "peak_tflops": round(fp32_peak / 1e12, 1),
                     "frac": round(flops / t / fp32_peak, 4),
                     "peak_kind": "nominal: 2 x 128 lanes x %d SMs x %d MHz"
                                  % (props.multi_processor_count, sm_max_mhz)}}


def era_m1_rate(job, torch, K):
    """Plain FP32 ERA (method 1, object only) on the same frames: rate and HBM fraction.

    Algorithmic bytes per iteration: 20 N^2 per frame (amp 4, psi write 8,
    psi read by the object gather 8) + 24 U V (object read, write, denominator).
    """
    job.O.copy_(torch.from_numpy(job.O0).to(job.dev))
    for _ in range(3):
        job.run("era", 1, 1)
    t = event_time(torch, lambda: job.run("era", 1, 1), K) / K
    bytes_ = 20.0 * job.N * job.N * job.n + 24.0 * job.U * job.V
    pk, _ = peaks()
    return {"frame_iters_per_s": round(job.n / t, 1), "ms_per_iter": round(t * 1e3, 4),
            "hbm_gbs": round(bytes_ / t / 1e9, 1), "hbm_frac": round(bytes_ / t / 1e9 / pk, 4)}


def nmse(O, O_true, heat, rel_thresh=1e-3):
    """Object error over the illuminated region (heat > 1e-3 max) after removing
    the global complex scale c = <O_true, O> / |O|^2."""
    m = heat > rel_thresh * heat.max()
    a, t = O[m].astype(np.complex128), O_true[m].astype(np.complex128)
    c = np.vdot(a, t) / np.vdot(a, a)
    return float(np.sum(np.abs(c * a - t) ** 2) / np.sum(np.abs(t) ** 2))


def _era_to_nmse(torch, job, O_init, O_true, heat, target, max_iters):
    """ERA from O_init, one iteration at a time, until the object NMSE is at
    most `target`; device time of the iterations."""
    job.O.copy_(O_init)
    total, it = 0.0, 0
    err0 = err = nmse(job.O.cpu().numpy(), O_true, heat)
    while it < max_iters and err > target:
        total += event_time(torch, lambda: job.run("era", 1, 1), 1)
        it += 1
        err = nmse(job.O.cpu().numpy(), O_true, heat)
    return {"iterations": it, "seconds": round(total, 5), "nmse": err, "initial_nmse": err0,
            "reached": bool(err <= target)}


def workload_nmse_c1(exits_fn):
    """The 256^2 / 1024-frame job of workload_c1 -- the same object, probe,
    32 x 32 raster and Poisson noise at 1e6 photons per frame -- without the
    additive background and the mask, reconstructed with the true probe (ERA
    method 1).  With the background and probe retrieval of the full job no
    start reaches object NMSE 1e-3 against the ground truth (ERA method 4
    from the known background floors at 1.0e-3), and with the beamstop the
    unconstrained lowest spatial frequencies drift, so every pixel is used."""
    rng = np.random.default_rng(1)
    N, U, side = 256, 1024, 32
    w = Workload()
    w.name = "c1n"
    w.O_true = make_object(rng, U)
    w.P_true = make_probe(N, 64, 8, 0.0005)
    w.P0 = w.P_true
    w.R = raster(rng, side, 24, 3, N, U)
    I = exits_fn(w.O_true, w.P_true, w.R)
    I = I * (1e6 / I.sum(axis=(1, 2), keepdims=True))
    I = rng.poisson(I).astype(np.float32)
    w.I = np.fft.fftshift(I, axes=(-2, -1))
    w.M = np.ones((N, N), bool)
    w.method = 1
    w.N, w.U = N, U
    return w


def workload_heldout(exits_fn, seed=7):
    """A held-out 20 x 20 scan of 128^2 frames (the warm start's frame size):
    an object and a probe drawn like its training frames' (smooth random
    object, aperture radius 24-40 px, quadratic phase 0.001-0.004) from a
    seed its training never uses; step 16 px, +-2 px jitter, noise free,
    known probe (ERA method 1)."""
    rng = np.random.default_rng(seed)
    N, side, step = 128, 20, 16
    U = N + step * (side - 1) + 8
    w = Workload()
    w.name = "heldout"
    w.O_true = make_object(rng, U)
    w.P_true = make_probe(N, rng.uniform(24, 40), 4, rng.uniform(0.001, 0.004))
    w.P0 = w.P_true
    w.R = raster(rng, side, step, 2, N, U)
    w.I = np.fft.fftshift(exits_fn(w.O_true, w.P_true, w.R), axes=(-2, -1)).astype(np.float32)
    w.M = np.ones((N, N), bool)
    w.method = 1
    w.N, w.U = N, U
    return w


def _nmse_leg(torch, dev, net, w, target, max_iters):
    """Plain FP32 ERA from the reference's default object of ones
    (era.py:480-486) against ERA from the learned warm start, both to object
    NMSE <= target against the synthetic ground truth."""
    from ptychography_gb300 import warmstart as ws
    job = DeviceJob(w, dev)
    job.run("era", 1, 1)                         # heatmap of the known probe
    torch.cuda.synchronize()
    heat = job.heat.cpu().numpy()
    # ground truth on the reconstruction's grid: the preamble shifts R so that
    # its maximum is 0, i.e. the object window starts at -R.max(axis=0)
    r0, r1 = (-w.R.max(axis=0)).tolist()
    U, V = heat.shape
    O_true = w.O_true[r0:r0 + U, r1:r1 + V]
    ones = torch.from_numpy(job.O0).to(dev)
    for _ in range(3):                           # warm the graph cache
        job.O.copy_(ones)
        job.run("era", 1, 1)
    plain = _era_to_nmse(torch, job, ones, O_true, heat, target, max_iters)
    I_dev = torch.from_numpy(np.ascontiguousarray(w.I, dtype=np.float32)).to(dev)
    R_sh = w.R - w.R.max(axis=0)
    # set-up (the coarse probe, plan and buffers), like the main plan: untimed
    st = ws.DownsampledStart(net, I_dev.shape[0], w.N, w.N, w.P0, R_sh)
    st.run(I_dev, U, V)                          # first call: kernels, tiles, tensor maps
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    O_ws = st.run(I_dev, U, V)
    torch.cuda.synchronize()
    stitch_s = time.perf_counter() - t0
    warm = _era_to_nmse(torch, job, O_ws, O_true, heat, target, max_iters)
    warm["frames_through_network"] = int(len(st.frames))
    st.close()
    warm["inference_stitch_seconds"] = round(stitch_s, 5)
    warm["seconds_total"] = round(stitch_s + warm["seconds"], 5)
    job.close()
    return {"plain_era": plain, "warm_start": warm,
            "iterations": plain["iterations"], "seconds": plain["seconds"], "reached": plain["reached"],
            "nmse": plain["nmse"],
            "warm_start_speedup": round(plain["seconds"] / warm["seconds_total"], 3)
            if warm["seconds_total"] > 0 and warm["reached"] else None}


def train_warm_start(torch, dev, warm_steps=20000, warm_frames=50000):
    """The warm start's network (128^2 frames) trained on the GPU: warm_steps
    Adam steps of 32 frames from warm_frames simulated frames (random objects
    with smoothing widths 2-4 px, random probes, Poisson noise at 1e5-1e7
    photons).  Returns the network and a description of its training."""
    from ptychography_gb300 import warmstart as ws
    net = ws.WarmStartNet(128, 128, seed=0, device=dev)
    t0 = time.perf_counter()
    data = ws.make_training_set(net, warm_frames, seed=1, sigma=(2.0, 4.0), photons=(1e5, 1e7))
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    losses = ws.train(net, data, warm_steps, batch=32, lr=3e-4)
    t2 = time.perf_counter()
    del data
    torch.cuda.empty_cache()
    info = {"steps": warm_steps, "batch": 32, "frames": warm_frames,
            "data_seconds": round(t1 - t0, 2), "train_seconds": round(t2 - t1, 2),
            "loss_first_20": float(np.mean(losses[:20])), "loss_last_20": float(np.mean(losses[-20:])),
            "input": "back-projection ifftn(sqrt(I) exp(i angle fftn P)) conj(P), (Re, Im)",
            "target": "object phase under the probe (cos, sin), weights |P|^2",
            "kernels": "inference and the training forward pass: tcgen05 implicit-GEMM convolutions "
                       "(layers 1-4), direct CUDA-core convolutions (layers 0, 5); training backward: "
                       "input gradients as tcgen05 convolutions with flipped weights (layers 1-4; "
                       "layer 5 direct), weight gradients as tcgen05 GEMMs over the pixels (layers "
                       "1-5; layer 0 im2col + mma.sync)"}
    return net, info


def time_to_nmse(torch, dev, net, training, target=1e-3, max_iters=400):
    """Time to object NMSE <= target (illuminated region, global complex scale
    removed, against the synthetic ground truth): plain FP32 GPU ERA from
    ones against ERA from the learned warm start's stitched object.

    Two scans are reconstructed with the trained network (train_warm_start):
    the 256^2 / 1024-frame geometry (workload_nmse_c1; the network sees a
    covering subset of the frames at half resolution, the central 128^2 of
    each pattern, and the stitched object is upsampled) and a held-out
    20 x 20 scan of 128^2 frames (workload_heldout).  The warm start's
    inference + stitching is wall clock (host work included) and counts
    towards its time; its training time is reported beside it."""
    c1 = _nmse_leg(torch, dev, net, workload_nmse_c1(gpu_intensities), target, max_iters)
    held = _nmse_leg(torch, dev, net, workload_heldout(gpu_intensities), target, max_iters)
    out = {"workload": "ERA m1 (known probe), 1024 frames 256x256, object 1006x1006 (1024x1024 truth), "
                       "32x32 raster step 24 +-3, Poisson 1e6, no background, no mask",
           "reference_object": "synthetic ground truth (illuminated region, global scale removed)",
           "target": target}
    out.update(c1)
    out["warm_start"]["downsampling"] = "network at 128x128: central 128^2 of each 256^2 pattern, object upsampled x2"
    out["warm_start"]["training"] = training
    out["warm_start"]["timing"] = ("inference + stitching + upsampling wall clock after an untimed set-up of "
                                   "the coarse plan (as the main plan is set up untimed)")
    held["workload"] = "held-out 20x20 scan, 400 frames 128x128, ERA m1 (known probe), noise free"
    out["heldout_20x20"] = held
    return out


def c4_rate(torch, dev, steps=5, warmup=2, net=None, warm_iters=10):
    """The 4096-frame 512 x 512 DM method-6 job (DeviceWorkload) timed beside
    the headline: device-resident iterations, CUDA events.  Its error against
    the chunked FP64 oracle is checked by tests/test_gpu_c4_fp64.py.  With a
    trained warm-start network, the per-frame warm start (each 512^2 frame
    seen at 128^2) is timed, its object's NMSE against the synthetic truth
    is compared with that of ones, and warm_iters DM iterations from each
    report the reference's own error metric (eMod): with the probe and
    background retrieved, DM's early iterates wander from the truth
    (object NMSE ~1 after 10 iterations from either start), so the object
    error after a few iterations says nothing about the start."""
    w = DeviceWorkload(dev)
    job = DeviceJob(w, dev)
    for _ in range(warmup):
        job.step()
    t = event_time(torch, job.step, steps) / steps
    out = {"workload": workload_config("c4")["workload"], "frame_iters_per_s": round(job.n / t, 1),
           "ms_per_iter": round(t * 1e3, 3), "steps": steps, "warmup": warmup,
           "error_vs_fp64": "tests/test_gpu_c4_fp64.py: 3 DM iterations against the chunked FP64 oracle; "
                            "O (illuminated) / P / background within 3e-5"}
    if net is not None:
        out["warm_start"] = _c4_warm_start(torch, dev, w, job, net, warm_iters)
    job.close()
    del job, w
    torch.cuda.empty_cache()
    return out


def _c4_warm_start(torch, dev, w, job, net, iters):
    from ptychography_gb300 import warmstart as ws
    torch.cuda.synchronize()
    heat = job.heat.cpu().numpy()
    r0, r1 = (-w.R.max(axis=0)).tolist()
    U, V = job.U, job.V
    O_true = w.O_true[r0:r0 + U, r1:r1 + V]
    R_sh = w.R - w.R.max(axis=0)
    st = ws.DownsampledStart(net, job.n, w.N, w.N, w.P0, R_sh)
    st.run(w.I_dev, U, V)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    O_ws = st.run(w.I_dev, U, V)
    torch.cuda.synchronize()
    t_ws = time.perf_counter() - t0
    ones = torch.ones((U, V), dtype=torch.complex64, device=dev)
    res = {"frames_through_network": int(len(st.frames)), "downsampling": "512^2 -> 128^2 (central crop), x4 upsampling",
           "inference_stitch_seconds": round(t_ws, 5)}
    for name, O0 in (("ones", ones), ("warm_start", O_ws)):
        job.reset(O0)
        e0 = nmse(O0.cpu().numpy(), O_true, heat)
        t = event_time(torch, lambda: job.run("dm", 6, iters), 1)
        em = job.emod[:iters].cpu().numpy()
        res[name] = {"initial_object_nmse": e0, "eMod_after_%d" % iters: float(em[-1]),
                     "eMod_first": float(em[0]), "dm_seconds": round(t, 4)}
    st.close()
    return res


def e2e_public_api(w, K):
    """The public API on host arrays: ERA (K iterations) then DM (K iterations),
    after one untimed pair of 1-iteration calls (the process's first public
    calls load kernels and set up the generator's jump tables and the
    page-locked output pool, once)."""
    import torch
    import ptychography_gb300 as pty

    def api_calls(k):
        if w.method == 6:
            O, P, info = pty.ERA(w.I, w.R.copy(), w.P0, None, k, mask=w.M, method=6)
            O, P, info2 = pty.DM(w.I, w.R.copy(), P, O, k, mask=w.M, method=6,
                                 background=info["background"])
            return (O, P, info2["eMod"][-1])
        O, info = pty.ERA(w.I, w.R.copy(), w.P0, None, k, mask=w.M, method=w.method)
        return (O, info["eMod"][-1])

    np.random.seed(13)
    api_calls(1)
    torch.cuda.synchronize()
    np.random.seed(13)
    t0 = time.perf_counter()
    api_calls(1)
    torch.cuda.synchronize()
    dt1 = time.perf_counter() - t0
    np.random.seed(13)
    t0 = time.perf_counter()
    res = api_calls(K)
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    # wall time = fixed + K x per-iteration, from the 1- and K-iteration calls
    per_iter = (dt - dt1) / (K - 1) if K > 1 else None
    fixed = dt1 - per_iter if per_iter is not None else None
    n, N = w.I.shape[0], w.I.shape[1]
    U = w.U
    calls = 2 if w.method == 6 else 1
    # per call up: I (float32), O (complex64), P (complex64), mask (uint8); the DM
    # call also one background pattern (float32; ERA's random background is drawn
    # on the device).  Down: O, P, info['I'] (float32), heatmap (float64), the
    # eMod / eCon histories and, for methods 4-6, the mean background.
    h2d = calls * (n * N * N * 4 + U * U * 8 + N * N * 9) + (N * N * 4 if w.method >= 4 else 0)
    d2h = calls * (U * U * 8 + N * N * 8 + n * N * N * 4 + U * U * 8 + 16 * K
                   + (N * N * 4 if w.method >= 4 else 0))
    frames = n * K * calls
    return {"value": round(frames / dt, 1), "unit": "frame-iters/s",
            "h2d_bytes_per_step": int(h2d / K), "d2h_bytes_per_step": int(d2h / K),
            "wall_s": round(dt, 3), "final_eMod": float(res[-1]),
            "fixed_cost_s": round(fixed, 4) if fixed is not None else None,
            "per_iteration_s": round(per_iter, 6) if per_iter is not None else None,
            "fixed_cost": "wall time of the public calls that does not grow with the iteration count "
                          "(host preamble, copies, plan set-up, result download), from a 1-iteration "
                          "and a K-iteration call",
            "warmup": "one untimed ERA + DM pair of 1 iteration each"}


# --------------------------------------------------------------------------- CPU oracle
_SHARD_CACHE = {}


def _oracle_shard(args):
    """One worker of the CPU baseline: oracle ERA m6 + DM m6, one iteration each.

    The shard's data are generated once per process and cached; only the
    reconstruction is timed."""
    shard, seed_frames, method = args
    sys.path.insert(0, ROOT)
    from oracle import ptycho_oracle as orc
    key = (method, tuple(np.asarray(seed_frames).tolist()))
    if key not in _SHARD_CACHE:
        _SHARD_CACHE.clear()
        _SHARD_CACHE[key] = (workload_c1(numpy_intensities, frames=seed_frames) if method == 6
                             else workload_c0(numpy_intensities))
    w = _SHARD_CACHE[key]
    np.random.seed(shard)
    t0 = time.perf_counter()
    if method == 6:
        O, P, info = orc.ERA(w.I, w.R.copy(), w.P0, None, 1, mask=w.M, method=6, dtype="single")
        orc.DM(w.I, w.R.copy(), P, O, 1, mask=w.M, method=6, dtype="single",
               background=info["background"], full_output=False)
        n_fi = 2 * len(w.R)
    else:
        orc.ERA(w.I, w.R.copy(), w.P0, None, 1, mask=w.M, method=1, dtype="single", full_output=False)
        n_fi = len(w.R)
    return n_fi, time.perf_counter() - t0


def cpu_oracle_rate(method, shard_frames, cores, pool=None):
    """Frame-iterations per second of the oracle on `cores` disjoint shards."""
    chunks = [(i, np.arange(i * shard_frames, (i + 1) * shard_frames) % 1024, method)
              for i in range(cores)]
    if pool is None:
        res = [_oracle_shard(c) for c in chunks]
    else:
        res = pool.map(_oracle_shard, chunks)
    # the shards run in parallel: a step lasts as long as its slowest shard
    wall = max(r[1] for r in res)
    return sum(r[0] for r in res) / wall, wall


# --------------------------------------------------------------------------- main
def max_over_ranks(torch, t, world, dev):
    """The slowest rank's time (every rank gets it); t itself for one rank."""
    if world <= 1:
        return t
    tt = torch.tensor([t], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    return float(tt.item())


def job_rate(frames_per_step, steps, world, t):
    """Whole-job frame-iterations per second: every rank runs its own replica
    of the workload (weak scaling), so the job does world x the frames."""
    return frames_per_step * steps * world / t


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), \
        int(os.environ.get("LOCAL_RANK", 0))


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    method = 6 if args.workload == "c1" else 1
    shard = 16 if method == 6 else 100
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            cpu_oracle_rate(method, shard, cores, pool)
        rates, walls = [], []
        for _ in range(args.steps):
            r, wll = cpu_oracle_rate(method, shard, cores, pool)
            rates.append(r)
            walls.append(wll)
    total_fi = (2 if method == 6 else 1) * shard * cores * args.steps
    value = total_fi / sum(walls)
    line = {
        "impl": "reference", "metric": "frame-iters/s", "value": round(value, 2),
        "unit": "frame-iters/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(walls) / args.steps, 2), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args.workload),
        "cpu_baseline": {"value": round(value, 2), "unit": "frame-iters/s", "cores": cores,
                         "kind": "port",
                         "sample": "%d processes x %d disjoint frames, ERA m6 + DM m6 one iteration "
                                   "each per step (oracle NumPy port, no all-reduce)" % (cores, shard)
                         if method == 6 else "%d processes x 100 frames, ERA m1 one iteration" % cores},
        "e2e": {"value": round(value, 2), "unit": "frame-iters/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def workload_config(name, frames=None):
    cfg = _workload_config(name)
    if frames and name in ("c1", "c4"):     # a profiling case: the first frames of the scan
        cfg = dict(cfg, n_frames=min(frames, cfg["n_frames"]),
                   workload="first %d frames of: %s" % (min(frames, cfg["n_frames"]), cfg["workload"]))
    return cfg


def _workload_config(name):
    if name == "c1":
        return {"workload": "ERA m6 then DM m6 (object+probe+background), 1024 frames 256x256, "
                            "object 1024x1024, Poisson 1e6, beamstop+dead-pixel mask",
                "n_frames": 1024, "frame": [256, 256], "object": [1024, 1024],
                "step": "1 ERA-m6 iteration + 1 DM-m6 iteration over all frames",
                "l2": "working set (psi 537 MB) larger than L2; no flush"}
    if name == "c4":
        return {"workload": "DM m6 (object+probe+background), 4096 frames 512x512, object 2816x2816, "
                            "Poisson 1e8, beamstop+dead-pixel mask",
                "n_frames": 4096, "frame": [512, 512], "object": [2816, 2816],
                "step": "1 DM-m6 iteration over all frames",
                "l2": "working set (psi 8.6 GB) larger than L2; no flush"}
    return {"workload": "ERA m1 (object only), 100 frames 128x128, object 320x320, noise free",
            "n_frames": 100, "frame": [128, 128], "object": [320, 320],
            "step": "1 ERA-m1 iteration over all frames",
            "l2": "working set 20 MB fits in L2: reported as an L2-resident case"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c1", choices=["c1", "c0", "c4"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-nmse", action="store_true")
    ap.add_argument("--no-c4", action="store_true",
                    help="skip the 4096-frame 512x512 DM measurement")
    ap.add_argument("--no-batch", action="store_true",
                    help="skip the 64-reconstruction batched measurement")
    ap.add_argument("--warm-steps", type=int, default=20000,
                    help="training steps of the warm start's network in the time-to-NMSE measurement")
    ap.add_argument("--frame-tile", type=int, default=0,
                    help="force this frame tile (CTAs per frame; see pty_set_frame_tile) for profiling")
    ap.add_argument("--frames", type=int, default=None,
                    help="use only the first F frames of the c1 or c4 raster (profiling captures)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from ptychography_gb300 import _native
    lib = _native.load()

    if args.workload == "c1":
        w = workload_c1(gpu_intensities, frames=np.arange(args.frames) if args.frames else None)
    elif args.workload == "c4":
        w = DeviceWorkload(dev, frames=args.frames)
    else:
        w = workload_c0(gpu_intensities)
    if args.frame_tile:     # profiling one tile: forced for both op families
        for fam in (0, 1):
            _native.check(lib.pty_set_frame_tile(w.N, w.N, fam, args.frame_tile))
    job = DeviceJob(w, dev)
    for _ in range(args.warmup):
        job.step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    launches0 = lib.pty_launch_count()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        s.record()
        for _ in range(args.steps):
            job.step()
        e.record()
        torch.cuda.synchronize()
    barrier()
    launches = lib.pty_launch_count() - launches0
    t = max_over_ranks(torch, s.elapsed_time(e) / 1e3, world, dev)
    value = job_rate(job.frames_per_step(), args.steps, world, t)

    tiles = []
    for fam in (0, 1):                       # plain / background op families
        t_ = ctypes.c_int32(0)
        _native.check(lib.pty_get_frame_tile(job.N, job.N, fam, ctypes.byref(t_)))
        tiles.append(int(t_.value))
    roof = roofline_pmod7(job, torch, tiles[1], clk.summary()["sm_max_mhz"] or 2070)
    m1 = era_m1_rate(job, torch, max(args.steps, 10)) if args.workload == "c1" else None
    job.close()
    if rank != 0:
        return 0

    e2e = None if (args.no_e2e or args.workload == "c4") else e2e_public_api(w, args.steps)
    cpu = None
    if not args.no_cpu_baseline and args.workload != "c4":
        method = w.method
        # about 10 s of single-core work: every frame of the workload once
        shard = 1024 if method == 6 else 100
        r, wall = cpu_oracle_rate(method, shard, 1)
        cpu = {"value": round(r, 2), "unit": "frame-iters/s", "cores": 1, "host_cpus": os.cpu_count(), "kind": "port",
               "sample": ("ERA m6 + DM m6, one iteration each, on all %d frames "
                          "(oracle NumPy port, single process), %.1f s" % (shard, wall))
               if method == 6 else "ERA m1 one iteration on the 100 frames, %.1f s" % wall}
    line = {
        "metric": "frame-iters/s", "value": round(value, 1), "unit": "frame-iters/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * t / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(workload_config(args.workload, args.frames),
                       parallelism="replicas" if world > 1 else "1 GPU",
                       frame_tile_ctas={"plain": tiles[0], "background": tiles[1]}),
        "gpu_launches": int(launches), "clocks": clk.summary(), "roofline": roof,
        "cpu_baseline": cpu, "e2e": e2e,
        "error_vs_fp64": ({"test": "tests/test_gpu_geometry_c1.py",
                           "bound": "one ERA m6 and one DM m6 iteration on this geometry (1024 frames 256x256) "
                                    "within 1e-5 relative of the FP64 oracle on O, P, background and eMod"}
                          if args.workload == "c1" else
                          {"test": "tests/test_gpu_c4_fp64.py",
                           "bound": "3 DM m6 iterations within 3e-5 of the chunked FP64 oracle (lit object, "
                                    "probe, background, eMod)"} if args.workload == "c4" else
                          {"test": "tests/test_gpu_parity_c0.py", "bound": "1e-5 relative per iteration"}),
    }
    if m1:
        line["era_m1"] = m1
    net = None
    if not args.no_nmse:
        net, training = train_warm_start(torch, dev, warm_steps=args.warm_steps)
        line["time_to_nmse"] = time_to_nmse(torch, dev, net, training)
    if args.workload == "c1" and not args.no_batch:
        line["batched"] = batched_rate(dev)
    if args.workload == "c1" and not args.no_c4:
        line["c4"] = c4_rate(torch, dev, net=net)
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
