"""The CPU oracle against golden fixtures recorded from the reference itself.

FP64 runs must agree to rounding (the oracle follows the reference's operation
order); FP32 runs use NumPy complex64 exactly as the reference does.
"""
import os

import numpy as np
import pytest

from oracle import ptycho_oracle as orc
from cases import ITERS, initial_guess, run_cases

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(GOLD, name), allow_pickle=False)


@pytest.fixture(scope="module")
def problem():
    d = _load("forward_sim.npz")
    return {k: d[k] for k in d.files}


@pytest.fixture(scope="module")
def runs():
    return _load("runs.npz")


def _rel(a, b):
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300)


def test_forward_sim_matches_reference(problem):
    """forward_sim with the reference's object: probe, scan, RNG draws, I, mask, B."""
    p = problem
    np.random.seed(int(p["seed"]))
    I, R, M, P, O, B = orc.forward_sim_from_object(
        p["O"], shape_P=(32, 32), A=9, defocus=0.02, photons_pupil=100.0, ny=3, nx=3,
        random_offset=3, background=2, mask=12, counting_statistics=False)
    assert np.array_equal(R, p["R"])
    assert np.array_equal(M, p["M"])
    assert np.array_equal(B, p["B"])
    np.testing.assert_allclose(P, p["P"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(I, p["I"], rtol=1e-12, atol=1e-9)


def test_forward_sim_rect_poisson():
    d = _load("forward_sim_rect.npz")
    np.random.seed(int(d["seed"]))
    I, R, M, P, O, B = orc.forward_sim_from_object(
        d["O"], shape_P=(32, 64), A=10, defocus=0.01, photons_pupil=50.0, ny=3, nx=2,
        random_offset=4, background=3, mask=8, counting_statistics=True)
    assert I.dtype == d["I"].dtype == np.int64
    assert np.array_equal(R, d["R"]) and np.array_equal(M, d["M"])
    assert np.array_equal(B, d["B"])
    # Poisson draws depend on lam to the last bit; equal draws pin the intensities
    assert np.array_equal(I, d["I"])


@pytest.fixture(scope="module")
def ops():
    d = _load("ops.npz")
    return {k: d[k] for k in d.files}


def test_ops_match_reference(ops):
    o = ops
    R, O, P, ex, amp, bg, mask = (o[k] for k in ("R", "O", "P", "exits", "amp", "bg", "mask"))
    a = 1.0e-10
    assert np.array_equal(orc.make_exits(O, P, R), o["make_exits"])
    assert np.array_equal(orc.multiroll(O, [-7, 13]), o["multiroll"])
    e1, em1 = orc.pmod_1(amp, ex.copy(), mask, a, True)
    np.testing.assert_allclose(e1, o["pmod_1"], rtol=1e-13, atol=1e-13)
    assert em1 == pytest.approx(float(o["pmod_1_eMod"]), rel=1e-13)
    e7, b7, em7 = orc.pmod_7(amp, bg.copy(), ex.copy(), mask, a, True)
    np.testing.assert_allclose(e7, o["pmod_7"], rtol=1e-13, atol=1e-13)
    np.testing.assert_allclose(b7, o["pmod_7_bg"], rtol=1e-13, atol=1e-13)
    assert em7 == pytest.approx(float(o["pmod_7_eMod"]), rel=1e-13)
    np.testing.assert_allclose(orc.Pmod_P(o["Pamp"], P.copy(), mask, a), o["Pmod_P"],
                               rtol=1e-13, atol=1e-13)
    Oo, hP = orc.psup_O(ex, P, R, O.shape, None, a)
    assert np.array_equal(hP, o["P_heatmap"])
    assert np.array_equal(Oo, o["psup_O"])
    Pp, hO = orc.psup_P(ex, O, R, None, a)
    assert np.array_equal(hO, o["O_heatmap"])
    assert np.array_equal(Pp, o["psup_P"])
    assert orc.model_error_1(amp, ex, mask, bg) == pytest.approx(float(o["model_error_1"]), rel=1e-13)
    assert orc.model_error_1(amp, ex, mask) == pytest.approx(float(o["model_error_1_nobg"]), rel=1e-13)


def run_oracle(case, problem):
    name, drv, m, dt, kw = case
    p = problem
    O0, P0, bg = initial_guess(m, p["O"], p["P"], p["B"], p["I"], p["R"])
    if kw.get("probe_centering"):
        P0 = np.roll(P0, (3, -2), axis=(0, 1))
    Rc = p["R"].copy()
    np.random.seed(99)
    f = orc.ERA if drv == "ERA" else orc.DM
    I = p["I"].astype(np.float32) if dt == "single" else p["I"]
    res = f(I, Rc, P0, O0, ITERS, mask=p["M"], method=m, background=bg, dtype=dt,
            full_output=True, **kw)
    return res, Rc


@pytest.mark.parametrize("case", run_cases(), ids=lambda c: c[0])
def test_runs_match_reference(case, problem, runs):
    name, drv, m, dt, kw = case
    res, Rc = run_oracle(case, problem)
    info = res[-1]
    g = lambda k: runs[name + "/" + k]  # noqa: E731
    tol = 1e-9 if dt == "double" else 2e-5
    assert np.array_equal(Rc, g("R_after"))
    upd = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}[m]
    outs = {"O": [res[0]], "P": [res[0]], "OP": [res[0], res[1]]}[upd]
    keys = {"O": ["O"], "P": ["P"], "OP": ["O", "P"]}[upd]
    for arr, k in zip(outs, keys):
        assert arr.dtype == g(k).dtype
        assert _rel(arr, g(k)) < tol, (k, _rel(arr, g(k)))
    np.testing.assert_allclose(info["eMod"], g("eMod"), rtol=tol * 10)
    np.testing.assert_allclose(info["eCon"], g("eCon"), rtol=tol * 10, atol=tol)
    assert _rel(info["I"], g("I_f32")) < max(tol, 1e-6)
    if name + "/heatmap" in runs.files:
        assert _rel(info["heatmap"], g("heatmap")) < tol
    if name + "/background" in runs.files:
        assert _rel(info["background"], g("background")) < tol


def test_back_projection_matches_reference(problem):
    d = _load("back_projection.npz")
    p = problem
    Rc = p["R"].copy()
    O, info = orc.Back_projection(p["I"], Rc, d["P"], None, mask=p["M"])
    assert np.array_equal(Rc, d["R_after"])
    assert _rel(O, d["O"]) < 1e-12
    assert _rel(info["exits"], d["exits"]) < 1e-12
    assert _rel(info["heatmap"], d["heatmap"]) < 1e-12
