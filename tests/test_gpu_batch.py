"""Batched reconstructions (pty_run_batch / ERA_batch / DM_batch).

Every reconstruction of a batch runs the same kernels in the same order as a
separate call, on its own graph branch, and the engine has no floating-point
atomics, so each result must equal the separate call's bit for bit -- including
problems whose preamble draws a random probe from NumPy's global RNG, which the
batch draws in list order.
"""
import numpy as np
import pytest

import ptychography_gb300 as pty
from test_gpu_cluster192 import small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def problems():
    # frame sizes of the batched workload (64, 128, 192, 256), small scans
    return [small_problem(N, seed=10 + k, side=3) for k, N in enumerate((64, 128, 192, 256))]


def _same(a, b):
    if isinstance(a, tuple):
        assert len(a) == len(b)
        for x, y in zip(a, b):
            _same(x, y)
    elif isinstance(a, dict):
        assert a.keys() == b.keys()
        for k in a:
            _same(a[k], b[k])
    elif a is None:
        assert b is None
    else:
        np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_era_batch_equals_separate_calls(problems):
    probs = []
    for k, (I, R, P, O, M) in enumerate(problems):
        # problem 1 draws its probe from the global RNG; problem 3 updates O only
        probs.append(dict(I=I, R=R.copy(), P=None if k == 1 else P * np.exp(0.2j), O=None, mask=M,
                          method=1 if k == 3 else 3))
    np.random.seed(5)
    got = pty.ERA_batch([dict(p, R=p["R"].copy()) for p in probs], 4, dtype="single")
    np.random.seed(5)
    want = [pty.ERA(p["I"], p["R"].copy(), p["P"], p["O"], 4, mask=p["mask"], method=p["method"],
                    dtype="single") for p in probs]
    assert len(got) == len(want)
    for g, w in zip(got, want):
        _same(g, w)


def test_dm_batch_method6_equals_separate_calls(problems):
    probs = []
    for I, R, P, O, M in problems:
        b = np.full(I.shape[1:], 0.5, np.float32)
        probs.append(dict(I=I, R=R.copy(), P=P * np.exp(0.2j), O=None, mask=M, background=b))
    got = pty.DM_batch([dict(p, R=p["R"].copy()) for p in probs], 3, method=6)
    want = [pty.DM(p["I"], p["R"].copy(), p["P"], p["O"], 3, mask=p["mask"],
                   background=p["background"], method=6) for p in probs]
    for g, w in zip(got, want):
        _same(g, w)


def test_batch_tuple_form_and_empty(problems):
    I, R, P, O, M = problems[0]
    assert pty.ERA_batch([], 2) == []
    (o1, i1), = pty.ERA_batch([(I, R.copy(), P, None)], 2, mask=M, method=1)
    o2, i2 = pty.ERA(I, R.copy(), P, None, 2, mask=M, method=1)
    _same((o1, i1), (o2, i2))


def test_batch_graph_replay_matches_separate_runs(problems):
    """A repeated pty_run_batch call replays the cached graph; results stay exact."""
    import ctypes
    import torch
    from ptychography_gb300 import _engine, _native
    lib = _native.load()
    dev = torch.device("cuda", 0)
    sp = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)

    def jobs():
        out = []
        for I, R, P, O, M in problems[:3]:
            np.random.seed(3)
            out.append(_engine._Job(lib, dev, sp, "era", I, R.copy(), P * np.exp(0.2j), None, 2, 1,
                                    M, None, 3, False, False, 1e-10, "single", True, True))
        return out

    a, b = jobs(), jobs()
    try:
        k = len(a)
        plans = (ctypes.c_void_p * k)(*[j.plan.value for j in a])
        bufs = (_native.Buffers * k)(*[j.buf for j in a])
        opts = (_native.Options * k)(*[j.opt for j in a])
        hv = (ctypes.c_int32 * k)()
        before = lib.pty_launch_count()
        _native.check(lib.pty_run_batch(0, plans, bufs, opts, k, 2, hv, sp))
        first = lib.pty_launch_count() - before
        _native.check(lib.pty_run_batch(0, plans, bufs, opts, k, 2, hv, sp))
        assert lib.pty_launch_count() - before == 2 * first      # replay counted the same
        h = ctypes.c_int32(0)
        for j in b:
            for _ in range(2):
                _native.check(lib.pty_era(j.plan, ctypes.byref(j.buf), ctypes.byref(j.opt), 2,
                                          ctypes.byref(h), sp))
        torch.cuda.synchronize()
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x.O_d.cpu().numpy(), y.O_d.cpu().numpy())
            np.testing.assert_array_equal(x.P_d.cpu().numpy(), y.P_d.cpu().numpy())
            np.testing.assert_array_equal(x.emod.cpu().numpy(), y.emod.cpu().numpy())
    finally:
        for j in a + b:
            j.close()
