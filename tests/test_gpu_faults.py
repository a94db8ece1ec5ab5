"""Failure handling made on the host (no GPU fault, trap or hang):

* NaN in the intensities propagates as the reference's NumPy arithmetic does
  (the eMod history holds NaN; no exception, no error status), and the next
  call on clean data is unaffected (the context and the library state stay
  usable);
* a device allocation that fails part-way through a call's set-up raises to
  the caller and the call's plan is still destroyed (no leaked plan);
* a scan window outside the object is rejected before any launch with
  ValueError (the reference fails later with a NumPy broadcast error).
"""
import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from oracle import ptycho_oracle as orc
from ptychography_gb300 import _engine, _native

pytestmark = pytest.mark.gpu


def _small():
    d = np.load(__file__.rsplit("/", 1)[0] + "/golden/forward_sim.npz")
    return d["I"], d["R"], d["M"], d["P"]


def _start(I, R):
    # ones plus seeded noise: with this band-limited probe, ones alone leaves
    # |FFT(P O)| at rounding level outside the pupil (FP32 vs FP64 ill-conditioned)
    rng = np.random.default_rng(11)
    shp = (I.shape[1] + R[:, 0].max() - R[:, 0].min(), I.shape[2] + R[:, 1].max() - R[:, 1].min())
    return np.ones(shp) + 0.1 * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp))


def test_nan_intensity_propagates_like_the_reference():
    I, R, M, P = _small()
    O0 = _start(I, R)
    Ib = I.astype(np.float64).copy()
    Ib[3, 5, 7] = np.nan
    O, info = pty.ERA(Ib, R.copy(), P, O0, 2, mask=M, method=1)
    O_o, info_o = orc.ERA(Ib, R.copy(), P, O0, 2, mask=M, method=1, dtype="double")
    assert np.isnan(info["eMod"]).all() == np.isnan(info_o["eMod"]).all()
    assert np.isnan(info["eMod"][0])
    # a clean call afterwards (on the plan the NaN call left) matches the oracle as usual
    O2, info2 = pty.ERA(I, R.copy(), P, O0, 2, mask=M, method=1)
    O2o, info2o = orc.ERA(I, R.copy(), P, O0, 2, mask=M, method=1, dtype="double")
    assert np.isfinite(info2["eMod"]).all()
    np.testing.assert_allclose(info2["eMod"], info2o["eMod"], rtol=1e-4)


def test_failed_allocation_raises_and_frees_the_plan(monkeypatch):
    I, R, M, P = _small()
    lib = _native.load()
    destroyed = []
    real_destroy = lib.pty_plan_destroy
    monkeypatch.setattr(lib, "pty_plan_destroy", lambda p: destroyed.append(p) or real_destroy(p))
    real_empty = torch.empty
    calls = {"n": 0}

    def failing_empty(*a, **k):
        calls["n"] += 1
        if calls["n"] == 2:       # the second device buffer of the set-up
            raise torch.cuda.OutOfMemoryError("simulated allocation failure")
        return real_empty(*a, **k)

    monkeypatch.setattr(_engine, "_torch", lambda: _FakeTorch(torch, failing_empty))
    with pytest.raises(torch.cuda.OutOfMemoryError):
        pty.ERA(I, R.copy(), P, None, 1, mask=M, method=1)
    assert len(destroyed) == 1
    monkeypatch.undo()
    O, info = pty.ERA(I, R.copy(), P, None, 1, mask=M, method=1)
    assert np.isfinite(info["eMod"]).all()


class _FakeTorch:
    """torch with one function replaced (the engine reads torch through _torch())."""

    def __init__(self, real, empty):
        self._real, self.empty = real, empty

    def __getattr__(self, k):
        return getattr(self._real, k)


def test_window_outside_object_is_rejected_before_launch():
    I, R, M, P = _small()
    O_small = np.ones((I.shape[1] + 2, I.shape[2] + 2), np.complex128)
    before = int(_native.load().pty_launch_count())
    with pytest.raises(ValueError):
        pty.ERA(I, R.copy(), P, O_small, 1, mask=M, method=1)
    assert int(_native.load().pty_launch_count()) == before


def test_plan_kept_between_calls_gives_the_same_results():
    """The public calls keep the last plan for the next call with the same
    geometry and scan: ERA then DM on the same data reuse it, a call on another
    scan replaces it, and results equal those of calls on fresh plans."""
    from ptychography_gb300 import _engine
    I, R, M, P = _small()
    lib = _native.load()
    pty.release_plan_cache()
    O1, i1 = pty.ERA(I, R.copy(), P, None, 2, mask=M, method=1)
    kept = _engine._PLAN_CACHE["plan"]
    assert kept
    O2, i2 = pty.ERA(I, R.copy(), P, None, 2, mask=M, method=1)      # reuses the kept plan
    assert _engine._PLAN_CACHE["plan"].value == kept.value
    np.testing.assert_array_equal(O1, O2)
    np.testing.assert_array_equal(i1["eMod"], i2["eMod"])
    pty.release_plan_cache()
    assert _engine._PLAN_CACHE["plan"] is None
    O3, i3 = pty.ERA(I, R.copy(), P, None, 2, mask=M, method=1)      # a fresh plan
    np.testing.assert_array_equal(O1, O3)
    R2 = R.copy()
    R2[0] += 1
    pty.ERA(I, R2, P, None, 1, mask=M, method=1)                    # another scan: replaced
    assert _engine._PLAN_CACHE["plan"].value != kept.value
    pty.release_plan_cache()
    assert lib is _native.load()
