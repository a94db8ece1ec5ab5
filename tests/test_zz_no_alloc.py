"""pty_psup_P_noalloc: the probe update for callers that cannot allocate.

Some callers cannot call cudaMalloc (an application that owns the whole device
budget, an allocator that forbids foreign allocations, a loop that must not
block).  This entry point needs no plan and allocates nothing; its partial sums
and the device copy of the scan offsets live in fixed arrays inside the
library.  The test compares it with the plan-based pty_psup_P and with the
oracle's psup_P (era.py:371-400) on two calls in a row with different inputs
(so leftover contents of the shared arrays from the first call would show up
in the second), and checks that the second call leaves the device's free
memory unchanged.  Probe shapes 128 x 128, 256 x 256 and 128 x 512 run the
three probe-gather kernels (tiled, 256-wide rows, 512-wide rows) on the fixed
scratch.  The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest
import torch

from gpu_util import Plan, ptr, rel, stream, to_dev
from oracle import ptycho_oracle as orc
from ptychography_gb300 import _native

pytestmark = pytest.mark.gpu

# (n, N0, N1, U, V); 128 x 512 has no frame kernel, so no plan: oracle only
SHAPES = [(40, 128, 128, 200, 184), (24, 256, 256, 330, 300), (16, 128, 512, 180, 600)]


def case(seed, n, N0, N1, U, V):
    rng = np.random.default_rng(seed)
    R = np.stack([-rng.integers(0, U - N0 + 1, n), -rng.integers(0, V - N1 + 1, n)], 1).astype(np.int64)
    c = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)  # noqa: E731
    return R, c(n, N0, N1), c(U, V)


def psup_P_reference_entry(R, ex, O):
    n, N0, N1 = ex.shape
    U, V = O.shape
    plan = Plan(n, N0, N1, U, V, R)
    psi, Od = to_dev(ex, np.complex64), to_dev(O, np.complex64)
    heat = torch.zeros((N0, N1), dtype=torch.float64, device=psi.device)
    P = torch.empty((N0, N1), dtype=torch.complex64, device=psi.device)
    plan.call("pty_psup_P", ptr(psi), ptr(Od), ptr(heat), 1, 1e-10, ptr(P))
    plan.close()
    return P.cpu().numpy(), heat.cpu().numpy()


def psup_P_noalloc(R, ex, O):
    lib = _native.load()
    n, N0, N1 = ex.shape
    U, V = O.shape
    geom = _native.Geometry(n, N0, N1, U, V)
    psi, Od = to_dev(ex, np.complex64), to_dev(O, np.complex64)
    heat = torch.zeros((N0, N1), dtype=torch.float64, device=psi.device)
    P = torch.empty((N0, N1), dtype=torch.complex64, device=psi.device)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    R64 = np.ascontiguousarray(R, dtype=np.int64)
    rc = lib.pty_psup_P_noalloc(ctypes.byref(geom), R64.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                ptr(psi), ptr(Od), ptr(heat), 1, 1e-10, ptr(P), stream())
    _native.check(rc)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return P.cpu().numpy(), heat.cpu().numpy(), free0 - free1


@pytest.mark.parametrize("shape", SHAPES, ids=["128x128", "256x256", "128x512"])
def test_noalloc_matches_plan_entry_and_oracle_on_two_calls(shape):
    used = []
    for seed in (1, 2):
        R, ex, O = case(seed, *shape)
        P_na, h_na, d_free = psup_P_noalloc(R, ex, O)
        used.append(d_free)
        if shape[1:3] != (128, 512):
            P_ref, h_ref = psup_P_reference_entry(R, ex, O)
            # same kernels, different frame chunking: FP32 partial-sum order only
            assert rel(P_na, P_ref) < 1e-6
            assert rel(h_na, h_ref) < 1e-7
        # the oracle in float64 from the same complex64-rounded inputs
        ex32 = ex.astype(np.complex64).astype(np.complex128)
        O32 = O.astype(np.complex64).astype(np.complex128)
        P_orc, h_orc = orc.psup_P(ex32, O32, R, alpha=1e-10)
        assert rel(P_na, P_orc) < 3e-6
        assert rel(h_na, h_orc) < 1e-7
    assert used[1] == 0, "the second call changed the device's free memory"


def test_noalloc_rejects_oversize_and_bad_offsets():
    lib = _native.load()
    dummy = torch.zeros(4, dtype=torch.complex64, device="cuda")
    heat = torch.zeros(4, dtype=torch.float64, device="cuda")
    for geom, msg in ((_native.Geometry(2, 512, 512, 600, 600), b"N0 * N1 > 65536"),
                      (_native.Geometry(20000, 32, 32, 64, 64), b"n_frames > 16384")):
        Rg = np.zeros((geom.n_frames, 2), dtype=np.int64)
        rc = lib.pty_psup_P_noalloc(ctypes.byref(geom), Rg.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                    ptr(dummy), ptr(dummy), ptr(heat), 1, 1e-10, ptr(dummy), stream())
        assert rc == 3 and msg in lib.pty_last_error()
    R = np.array([[0, 0], [-40, 0]], dtype=np.int64)       # rows 40..72 > U = 64
    geom = _native.Geometry(2, 32, 32, 64, 64)
    rc = lib.pty_psup_P_noalloc(ctypes.byref(geom), R.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                ptr(dummy), ptr(dummy), ptr(heat), 1, 1e-10, ptr(dummy), stream())
    assert rc == 3 and b"outside the object" in lib.pty_last_error()


def test_noalloc_offsets_beyond_one_parameter_batch():
    # 5000 frames: three offset-copy launches of up to 2048 frames each
    n, N0, N1, U, V = 5000, 32, 32, 96, 80
    R, ex, O = case(3, n, N0, N1, U, V)
    P_ref, h_ref = psup_P_reference_entry(R, ex, O)
    P_na, h_na, _ = psup_P_noalloc(R, ex, O)
    assert rel(P_na, P_ref) < 1e-6
    assert rel(h_na, h_ref) < 1e-7
