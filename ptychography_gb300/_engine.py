"""Host side of the drop-in ERA / DM: the reference's preamble, device upload,
one C-ABI call for the whole loop, and the reference's return values.

Host work mirrors ``preamble`` (ptychography/era.py:435-548): the method and
update choice, the dtype rule, the default object of ones, the random initial
probe drawn from NumPy's global RNG, and the in-place shift of ``R``.  The
random initial background (era.py:539-540) is the next draw of that same
generator; on the public path it is drawn on the GPU from the generator's state
(``device_random_background``), which is then advanced exactly as the host
draw would have advanced it.  ``I_norm`` (era.py:495) is summed on the GPU in
the pass that forms the amplitudes.  Everything else (exit waves, FFTs,
projections, metrics) runs on the GPU in libptycho_gb300.  Bulk arithmetic is
complex64; ``dtype='double'`` only sets the dtype of the returned arrays.
"""
import atexit
import ctypes
import math
import threading

import numpy as np

from . import _native

_UPDATE = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("ptychography_gb300 runs on a CUDA GPU; none is available")
    return torch


def choose_method(method, O, P, background):
    """era.py:440-456."""
    if method is None:
        if O is None and P is None:
            method = 3
        elif O is None:
            method = 1
        elif P is None:
            method = 2
        else:
            raise ValueError("method=None needs O or P to be None (era.py:440-449)")
        if background is not None:
            method += 3
    if method not in _UPDATE:
        raise ValueError("method must be one of 1..6, got %r" % (method,))
    return method


def pmod_probe_count(Pmod_probe, iters):
    """Number of leading iterations i with ``i < Pmod_probe`` (era.py:193)."""
    if Pmod_probe is None or Pmod_probe is False:
        return 0
    x = float(Pmod_probe)
    if math.isinf(x):
        return iters if x > 0 else 0
    return max(0, min(iters, int(math.ceil(x))))


class Preamble:
    """Host set-up shared by ERA and DM (era.py:435-548), without exit waves."""

    def __init__(self, I, R, P, O, OP_iters, mask, background, method, dtype,
                 host_background_draw=True, host_norm=True):
        I = np.asarray(I)
        if I.ndim != 3:
            raise ValueError("I must be (n_frames, N0, N1)")
        R = np.asarray(R) if not isinstance(R, np.ndarray) else R
        if R.ndim != 2 or R.shape[0] != I.shape[0] or R.shape[1] < 2:
            raise ValueError("R must be (n_frames, 2)")
        self.method = choose_method(method, O, P, background)
        self.update = _UPDATE[self.method]
        if isinstance(OP_iters, (int, np.integer)):
            OP_iters = (int(OP_iters), 1)
        self.OP_iters = (int(OP_iters[0]), int(OP_iters[1]))
        if dtype is None:
            dtype = "single" if I.dtype == np.float32 else "double"
        if dtype not in ("single", "double"):
            raise ValueError("dtype must be None, 'single' or 'double'")
        self.rdt, self.cdt = ((np.float32, np.complex64) if dtype == "single"
                              else (np.float64, np.complex128))
        n, N0, N1 = I.shape
        if O is None:
            O = np.ones((N0 + R[:, 0].max() - R[:, 0].min(), N1 + R[:, 1].max() - R[:, 1].min()),
                        dtype=self.cdt)
        if P is None:
            P = np.random.random(I[0].shape) + 1J * np.random.random(I[0].shape)
        # the reference's astype copies (era.py:492-493) only shield the
        # caller's arrays from its in-place updates; these are read once, to
        # upload, so a matching dtype is not copied
        self.P = np.asarray(P, dtype=self.cdt)
        self.O = np.asarray(O, dtype=self.cdt)
        if self.P.shape != (N0, N1):
            raise ValueError("P must have the frame shape %s" % ((N0, N1),))
        scalar_mask = np.ndim(mask) == 0
        # I_norm (era.py:495); with host_norm=False and a 0/1 mask it is left to
        # the device (None here, norm_scale the scalar mask's value)
        self.norm_scale = 1.0
        if scalar_mask:
            mask_arr = None
            if host_norm:
                self.I_norm = float(np.sum(mask * I, dtype=np.float64))
            else:
                self.I_norm, self.norm_scale = None, float(mask)
        else:
            mask = np.asarray(mask)
            if mask.shape != (N0, N1):
                raise ValueError("mask must have the frame shape %s" % ((N0, N1),))
            binary = mask.dtype == np.bool_ or bool(np.all((mask == 0) | (mask == 1)))
            self.I_norm = None if (binary and not host_norm) else float(np.sum(mask * I))
            mask_arr = np.ascontiguousarray(np.fft.ifftshift(mask) != 0).astype(np.uint8)
        self.mask = mask_arr
        self.I = I
        R[:, 0] -= R[:, 0].max()                                  # era.py:504-505
        R[:, 1] -= R[:, 1].max()
        self.R = R
        self.n, self.N0, self.N1 = n, N0, N1
        self.background = None
        self.background_pattern = None
        self.random_background = False
        if self.method in (4, 5, 6):                              # era.py:539-544
            if background is None and not host_background_draw:
                # drawn later on the device from the same generator state
                # (device_random_background), the next draw of the global RNG
                self.random_background = True
            elif background is None:
                self.background = (np.random.random((n, N0, N1)).astype(self.rdt) + 0.1).astype(np.float32)
            else:
                b = np.sqrt(np.fft.ifftshift(np.asarray(background, dtype=np.float64)))
                if host_background_draw:
                    self.background = np.ascontiguousarray(
                        np.broadcast_to(b.astype(np.float32), (n, N0, N1)))
                else:
                    # one frame's pattern; copied to every frame on the device
                    self.background_pattern = np.ascontiguousarray(b.astype(np.float32))
        self.user_background = background
        self._Pamp = None

    @property
    def Pamp(self):
        """|fftn(P)| of the initial probe (era.py:546-547), formed on first
        use: only the far-field probe constraint (Pmod_probe) reads it."""
        if self._Pamp is None:
            F = np.fft.fftn(self.P, axes=(-2, -1))
            self._Pamp = np.sqrt((F.conj() * F).real).astype(np.float32)
        return self._Pamp


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def device_random_background(lib, out, rdt, sp):
    """np.random.random(out.shape).astype(rdt) + 0.1 (as float32) into the
    device tensor `out`, drawn on the GPU from NumPy's global legacy generator,
    which is then advanced exactly as the host draw would have advanced it."""
    st = np.random.get_state()
    if st[0] != "MT19937":
        raise RuntimeError("NumPy's global generator is not MT19937")
    key = np.ascontiguousarray(st[1], dtype=np.uint32)
    key_out = np.empty(624, dtype=np.uint32)
    pos_out = ctypes.c_int32(0)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    # scratch (2 words per double) from the library's stream-ordered pool: a
    # block this large from torch's caching allocator would displace the
    # blocks the run's own large buffers reuse
    _native.check(lib.pty_legacy_random_background(
        key.ctypes.data_as(u32p), int(st[2]), int(out.numel()), int(rdt == np.float64),
        _ptr(out), None, key_out.ctypes.data_as(u32p), ctypes.byref(pos_out), sp))
    np.random.set_state((st[0], key_out, int(pos_out.value), st[3], st[4]))


_SIDE = {}


def _side_stream(dev):
    torch = _torch()
    s = _SIDE.get(dev.index)
    if s is None:
        s = _SIDE[dev.index] = torch.cuda.Stream(device=dev)
    return s


def device_random_background_async(lib, out, rdt, main):
    """device_random_background on a side stream that starts after `main`'s
    work so far, overlapping the caller's next uploads.  Returns (event,
    finish): `main` must wait for the event before reading `out`, and
    finish() -- called once the event has passed, e.g. after a stream
    synchronisation -- hands the generator's new state to NumPy."""
    torch = _torch()
    st = np.random.get_state()
    if st[0] != "MT19937":
        raise RuntimeError("NumPy's global generator is not MT19937")
    key = np.ascontiguousarray(st[1], dtype=np.uint32)
    key_out = torch.empty(624, dtype=torch.int32, pin_memory=True)     # written by the stream
    pos_out = ctypes.c_int32(0)
    u32p = ctypes.POINTER(ctypes.c_uint32)
    side = _side_stream(out.device)
    side.wait_stream(main)
    _native.check(lib.pty_legacy_random_background_async(
        key.ctypes.data_as(u32p), int(st[2]), int(out.numel()), int(rdt == np.float64), _ptr(out), None,
        ctypes.cast(key_out.data_ptr(), u32p), ctypes.byref(pos_out), ctypes.c_void_p(side.cuda_stream)))
    out.record_stream(side)
    ev = torch.cuda.Event()
    ev.record(side)
    pos = int(pos_out.value)

    def finish():
        ev.synchronize()
        np.random.set_state((st[0], key_out.numpy().view(np.uint32).copy(), pos, st[3], st[4]))
    return ev, finish


# The plan of the last public call, kept for the next call with the same
# geometry and scan (ERA then DM on the same data, or repeated calls): its
# set-up (tile lists, device scratch) and, when the next call's buffers land at
# the same addresses, its captured loop are reused.  Only plans of at most
# 2^27 frame pixels are kept (about 100-300 MB of plan scratch); the tensors a
# call allocates are torch's and go back to its allocator as usual.
_PLAN_CACHE = {"key": None, "plan": None}
_PLAN_LOCK = threading.Lock()
_PLAN_CACHE_MAX_PIXELS = 1 << 27


def release_plan_cache():
    """Destroy the plan kept from the last public call (frees its device memory)."""
    with _PLAN_LOCK:
        plan, _PLAN_CACHE["plan"], _PLAN_CACHE["key"] = _PLAN_CACHE["plan"], None, None
    if plan:
        _native.load().pty_plan_destroy(plan)


atexit.register(lambda: _PLAN_CACHE.update(plan=None, key=None))   # the context may be gone at exit


def _plan_key(dev, geom, R64):
    return (dev.index, geom.n_frames, geom.N0, geom.N1, geom.U, geom.V, R64.tobytes())


def _take_plan(lib, dev, geom, R64):
    key = _plan_key(dev, geom, R64)
    with _PLAN_LOCK:
        if _PLAN_CACHE["key"] == key and _PLAN_CACHE["plan"]:
            plan = _PLAN_CACHE["plan"]
            _PLAN_CACHE["plan"], _PLAN_CACHE["key"] = None, None
            return plan, key
    plan = ctypes.c_void_p()
    _native.check(lib.pty_plan_create(ctypes.byref(geom), R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                      ctypes.byref(plan)))
    return plan, key


def _return_plan(lib, key, plan):
    """Keep a plan for the next call (when small enough), destroying the one kept before."""
    if key[1] * key[2] * key[3] > _PLAN_CACHE_MAX_PIXELS:
        lib.pty_plan_destroy(plan)
        return
    with _PLAN_LOCK:
        old, _PLAN_CACHE["plan"], _PLAN_CACHE["key"] = _PLAN_CACHE["plan"], plan, key
    if old:
        lib.pty_plan_destroy(old)


class _Job:
    """One reconstruction's plan and device buffers (era.py:435-548 set-up on the GPU)."""

    def __init__(self, lib, dev, sp, kind, I, R, P, O, iters, OP_iters, mask, background, method,
                 Pmod_probe, probe_centering, alpha, dtype, full_output, use_graph, reuse_plan=False,
                 overlap_draw=False):
        torch = _torch()
        self.lib, self.kind, self.full_output = lib, kind, full_output
        self.reuse_plan, self.plan_key, self.ok = reuse_plan, None, False
        self.draw_event, self.finish_draw = None, None
        pre = self.pre = Preamble(I, R, P, O, OP_iters, mask, background, method, dtype,
                                  host_background_draw=False, host_norm=False)
        self.iters = iters = int(iters)
        n, N0, N1 = pre.n, pre.N0, pre.N1
        U, V = pre.O.shape
        geom = _native.Geometry(n, N0, N1, U, V)
        R64 = np.ascontiguousarray(pre.R[:, :2], dtype=np.int64)
        if reuse_plan:
            self.plan, self.plan_key = _take_plan(lib, dev, geom, R64)
        else:
            self.plan = ctypes.c_void_p()
            _native.check(lib.pty_plan_create(ctypes.byref(geom),
                                              R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              ctypes.byref(self.plan)))
        try:
            bg_d = None
            if pre.random_background and overlap_draw:              # era.py:539-540
                # drawn on a side stream while the intensities upload
                bg_d = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
                self.draw_event, self.finish_draw = device_random_background_async(
                    lib, bg_d, pre.rdt, torch.cuda.current_stream(dev))
            Iin = pre.I
            if Iin.dtype not in (np.float32, np.float64):
                Iin = Iin.astype(np.float64)
            I_d = torch.from_numpy(np.ascontiguousarray(Iin)).to(dev, non_blocking=False)
            amp = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
            mask_d = torch.from_numpy(pre.mask).to(dev) if pre.mask is not None else None
            if pre.I_norm is None:
                # amplitudes and I_norm = sum(mask * I) in one pass over I
                norm_d = torch.zeros(1, dtype=torch.float64, device=dev)
                _native.check(lib.pty_amp_and_norm(self.plan, _ptr(I_d), int(Iin.dtype == np.float64),
                                                   _ptr(mask_d), _ptr(amp), _ptr(norm_d), sp))
                pre.I_norm = float(norm_d.cpu()[0]) * pre.norm_scale
            else:
                _native.check(lib.pty_amp_from_intensity(self.plan, _ptr(I_d),
                                                         int(Iin.dtype == np.float64), _ptr(amp), sp))
            del I_d
            self.O_d = torch.from_numpy(np.ascontiguousarray(pre.O, dtype=np.complex64)).to(dev)
            self.P_d = torch.from_numpy(np.ascontiguousarray(pre.P, dtype=np.complex64)).to(dev)
            psi = torch.empty((n, N0, N1), dtype=torch.complex64, device=dev)
            if pre.background is not None:
                bg_d = torch.from_numpy(pre.background).to(dev)
            if pre.background_pattern is not None:
                bg_d = torch.from_numpy(pre.background_pattern).to(dev).expand(n, N0, N1).contiguous()
            if pre.random_background and not overlap_draw:          # era.py:539-540
                bg_d = torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
                device_random_background(lib, bg_d, pre.rdt, sp)
            npm = pmod_probe_count(Pmod_probe, iters)
            Pamp_d = torch.from_numpy(pre.Pamp).to(dev) if npm > 0 else None
            self.bmean = (torch.zeros((N0, N1), dtype=torch.float32, device=dev)
                          if bg_d is not None else None)
            self.heat = torch.zeros((U, V), dtype=torch.float64, device=dev)
            self.inten = (torch.empty((n, N0, N1), dtype=torch.float32, device=dev)
                          if full_output and iters > 0 else None)
            self.emod = torch.zeros(max(iters, 1), dtype=torch.float64, device=dev)
            self.econ = torch.zeros(max(iters, 1), dtype=torch.float64, device=dev)
            # keep every buffer the library writes alive for the job's lifetime
            self._keep = (amp, psi, mask_d, bg_d, Pamp_d)
            self.buf = _native.Buffers(_ptr(self.O_d), _ptr(self.P_d), _ptr(psi), _ptr(amp),
                                       _ptr(mask_d), _ptr(bg_d), _ptr(Pamp_d), _ptr(self.bmean),
                                       _ptr(self.heat), _ptr(self.inten), _ptr(self.emod),
                                       _ptr(self.econ))
            self.opt = _native.Options(pre.method, pre.OP_iters[0], pre.OP_iters[1], npm,
                                       int(bool(probe_centering)), int(bool(use_graph)),
                                       float(alpha), pre.I_norm)
        except BaseException:
            self.settle_draw()
            self.close()
            raise
        self.heat_valid = 0
        self.inten_host = None

    def stage_outputs(self):
        """Page-locked host memory for the model intensities (info['I'], n x N0 x
        N1 float32), allocated while the GPU runs the loop: a fresh host array
        of that size spends most of its download in page faults, which this
        moves off the critical path (a 268 MB download: ~15 ms -> ~2 ms)."""
        if self.inten is not None and self.pre.rdt == np.float32:
            torch = _torch()
            self.inten_host = torch.empty(tuple(self.inten.shape), dtype=torch.float32, pin_memory=True)

    def outputs(self):
        """The reference's return value (era.py:300-332 / dm.py:300-333)."""
        pre, kind, iters = self.pre, self.kind, self.iters
        # astype(copy=False): no host copy when the dtype already matches
        O_out = self.O_d.cpu().numpy().astype(pre.cdt, copy=False)
        P_out = self.P_d.cpu().numpy().astype(pre.cdt, copy=False)
        upd = pre.update
        if not self.full_output:
            return O_out if upd == "O" else P_out if upd == "P" else (O_out, P_out)
        rt = pre.rdt
        info = {
            "I": self._intensities(rt),
            "eMod": [rt(x) for x in self.emod.cpu().numpy()[:iters]],
            "eCon": [rt(x) for x in self.econ.cpu().numpy()[:iters]],
            # rounded to rt on the device: half the bytes to copy, no host pass
            "heatmap": ((self.heat.to(_torch().float32) if rt == np.float32 else self.heat).cpu().numpy()
                        if (self.heat_valid and upd != "P") else None),
        }
        if self.bmean is not None:
            info["background"] = (np.fft.fftshift(self.bmean.cpu().numpy()) ** 2).astype(rt)
        elif kind == "era" and pre.user_background is not None:
            b = np.asarray(pre.user_background)                   # era.py:311-314
            info["background"] = np.fft.fftshift(b[0] if b.ndim == 3 else b) ** 2
        if upd == "O":
            return O_out, info
        if upd == "P":
            return P_out, info
        return O_out, P_out, info

    def _intensities(self, rt):
        if self.inten is None:
            return None
        if self.inten_host is not None:
            self.inten_host.copy_(self.inten)
            return self.inten_host.numpy()
        return self.inten.cpu().numpy().astype(rt, copy=False)

    def settle_draw(self):
        """Wait for an overlapped background draw and hand NumPy the
        generator state it leaves (the reference has drawn it by now)."""
        if self.finish_draw is not None:
            fin, self.finish_draw = self.finish_draw, None
            fin()

    def close(self):
        if self.plan:
            if self.reuse_plan and self.ok:
                _return_plan(self.lib, self.plan_key, self.plan)
            else:
                self.lib.pty_plan_destroy(self.plan)
            self.plan = ctypes.c_void_p()


def run(kind, I, R, P, O, iters, OP_iters, mask, background, method, Pmod_probe,
        probe_centering, alpha, dtype, full_output, use_graph=True):
    """Run ERA (kind='era') or DM (kind='dm') on the GPU; return the reference's outputs."""
    torch = _torch()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    job = _Job(lib, dev, sp, kind, I, R, P, O, iters, OP_iters, mask, background, method,
               Pmod_probe, probe_centering, alpha, dtype, full_output, use_graph, reuse_plan=True,
               overlap_draw=True)
    try:
        if job.draw_event is not None:
            stream.wait_event(job.draw_event)
        hv = ctypes.c_int32(0)
        fn = lib.pty_era if kind == "era" else lib.pty_dm
        _native.check(fn(job.plan, ctypes.byref(job.buf), ctypes.byref(job.opt), job.iters,
                         ctypes.byref(hv), sp))
        job.stage_outputs()            # host work overlapping the GPU loop
        stream.synchronize()
        job.heat_valid = hv.value
        out = job.outputs()
        job.ok = True                  # a plan is kept for the next call only after a clean run
        return out
    finally:
        job.settle_draw()
        job.close()


_PROBLEM_KEYS = ("I", "R", "P", "O", "mask", "background", "method", "OP_iters", "Pmod_probe",
                 "probe_centering", "alpha", "dtype")


def run_batch(kind, problems, iters, defaults):
    """Many independent reconstructions in one graph launch (pty_run_batch).

    ``problems``: a sequence of dicts with the per-problem arguments of ERA/DM
    (``I``, ``R``, ``P``, ``O`` and optionally any of ``mask``, ``background``,
    ``method``, ``OP_iters``, ``Pmod_probe``, ``probe_centering``, ``alpha``,
    ``dtype``), or of ``(I, R, P, O)`` tuples.  ``defaults`` supplies the
    arguments a problem leaves out.  Preambles run in list order, so NumPy's
    global RNG is drawn exactly as by the same ERA/DM calls made one after
    another; ``R`` arrays are shifted in place as the single call does.
    Returns the list of per-problem return values.
    """
    torch = _torch()
    lib = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(dev)
    sp = ctypes.c_void_p(stream.cuda_stream)
    jobs = []
    try:
        for prob in problems:
            if not isinstance(prob, dict):
                I, R, P, O = prob
                prob = {"I": I, "R": R, "P": P, "O": O}
            unknown = set(prob) - set(_PROBLEM_KEYS)
            if unknown:
                raise ValueError("unknown problem keys: %s" % sorted(unknown))
            a = dict(defaults)
            a.update(prob)
            jobs.append(_Job(lib, dev, sp, kind, a["I"], a["R"], a.get("P"), a.get("O"), iters,
                             a["OP_iters"], a["mask"], a["background"], a["method"],
                             a["Pmod_probe"], a["probe_centering"], a["alpha"], a["dtype"],
                             a["full_output"], True))
        if not jobs:
            return []
        nrec = len(jobs)
        plans = (ctypes.c_void_p * nrec)(*[j.plan.value for j in jobs])
        bufs = (_native.Buffers * nrec)(*[j.buf for j in jobs])
        opts = (_native.Options * nrec)(*[j.opt for j in jobs])
        hv = (ctypes.c_int32 * nrec)()
        _native.check(lib.pty_run_batch(0 if kind == "era" else 1, plans, bufs, opts, nrec,
                                        int(iters), hv, sp))
        for j in jobs:
            j.stage_outputs()
        stream.synchronize()
        out = []
        for j, h in zip(jobs, hv):
            j.heat_valid = h
            out.append(j.outputs())
        return out
    finally:
        for j in jobs:
            j.close()
