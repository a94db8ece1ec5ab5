"""Whole ERA / DM runs on the GPU against the reference's recorded runs.

The recorded runs (tests/golden/runs.npz) are the reference itself, four
iterations, FP64 and FP32.  The engine computes in complex64, so after four
iterations of a nonlinear map the expected gap to the reference is a few
times FP32 rounding of the FFT round trips.  The bound is 1e-4 relative
(norm-wise) on O / P and every eMod / eCon entry, or ten times the gap between
the reference's own FP32 and FP64 runs of the case when that is larger (the
difference map amplifies rounding: its reference FP32/FP64 gap reaches 2e-4).  One case is excluded: the
reference's own FP32 run ERA_m6_opiters_single diverges (eCon ~ 400), so any
FP32 comparison of it is ill-conditioned.
"""
import os

import numpy as np
import pytest

import ptychography_gb300 as pty
from cases import ITERS, initial_guess, run_cases
from gpu_util import rel

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-4
UNSTABLE = {"ERA_m6_opiters_single"}


@pytest.fixture(scope="module")
def problem():
    d = np.load(os.path.join(GOLD, "forward_sim.npz"))
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="module")
def runs():
    return np.load(os.path.join(GOLD, "runs.npz"))


def gpu_run(case, p, **extra):
    name, drv, m, dt, kw = case
    O0, P0, bg = initial_guess(m, p["O"], p["P"], p["B"], p["I"], p["R"])
    if kw.get("probe_centering"):
        P0 = np.roll(P0, (3, -2), axis=(0, 1))
    Rc = p["R"].copy()
    np.random.seed(99)
    f = pty.ERA if drv == "ERA" else pty.DM
    I = p["I"].astype(np.float32) if dt == "single" else p["I"]
    res = f(I, Rc, P0, O0, ITERS, mask=p["M"], method=m, background=bg, dtype=dt,
            full_output=True, **kw, **extra)
    return res, Rc


def case_tol(name, runs):
    """max(1e-4, 10 x the reference's own FP32-vs-FP64 gap for this case)."""
    base = name.rsplit("_", 1)[0]
    gaps = []
    for k in ("O", "P"):
        a, b = base + "_single/" + k, base + "_double/" + k
        if a in runs.files and b in runs.files:
            gaps.append(rel(runs[a], runs[b]))
    return max([TOL] + [10 * g for g in gaps])


@pytest.mark.parametrize("case", [c for c in run_cases() if c[0] not in UNSTABLE],
                         ids=lambda c: c[0])
def test_run_matches_reference(case, problem, runs):
    name, drv, m, dt, kw = case
    tol = case_tol(name, runs)
    res, Rc = gpu_run(case, problem)
    info = res[-1]
    g = lambda k: runs[name + "/" + k]  # noqa: E731
    assert np.array_equal(Rc, g("R_after"))
    upd = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}[m]
    keys = {"O": ["O"], "P": ["P"], "OP": ["O", "P"]}[upd]
    for arr, k in zip(res[:-1], keys):
        assert arr.dtype == g(k).dtype and arr.shape == g(k).shape
        assert rel(arr, g(k)) < tol, (k, rel(arr, g(k)), tol)
    np.testing.assert_allclose(np.array(info["eMod"], float), g("eMod"), rtol=tol)
    np.testing.assert_allclose(np.array(info["eCon"], float), g("eCon"), rtol=tol, atol=1e-7)
    assert rel(info["I"], g("I_f32")) < tol
    if name + "/heatmap" in runs.files:
        assert info["heatmap"] is not None and rel(info["heatmap"], g("heatmap")) < 1e-6
    else:
        assert info["heatmap"] is None
    if name + "/background" in runs.files:
        assert rel(info["background"], g("background")) < tol


def test_bitwise_repeatable(problem):
    """Same inputs, same bits: the gathers use fixed orders, no float atomics."""
    case = ("DM_m6_double", "DM", 6, "double", {})
    a, _ = gpu_run(case, problem)
    b, _ = gpu_run(case, problem)
    for x, y in zip(a[:-1], b[:-1]):
        assert np.array_equal(x, y)
    assert a[-1]["eMod"] == b[-1]["eMod"] and a[-1]["eCon"] == b[-1]["eCon"]
    assert np.array_equal(a[-1]["I"], b[-1]["I"])


def test_graph_and_stream_paths_agree(problem):
    """The CUDA-graph capture of the loop launches exactly the stream-ordered work."""
    case = ("ERA_m3_double", "ERA", 3, "double", {})
    from ptychography_gb300 import _engine
    p = problem
    O0, P0, _ = initial_guess(3, p["O"], p["P"], p["B"], p["I"], p["R"])
    outs = []
    for g in (True, False):
        np.random.seed(5)
        outs.append(_engine.run("era", p["I"], p["R"].copy(), P0, O0, ITERS, 1, p["M"], None, 3,
                                False, False, 1e-10, "double", True, use_graph=g))
    for x, y in zip(outs[0][:-1], outs[1][:-1]):
        assert np.array_equal(x, y)
