"""One ERA and one DM iteration (method 6: object + probe + background) on the
full 256 x 256 / 1024-frame benchmark geometry, against the oracle.

The benchmark's own data (bench.workload_c1: 32 x 32 jittered raster, object
1024 x 1024, background, Poisson 1e6, beamstop + dead-pixel mask) and its own
plan geometry (1024 frames, object 1006 x 1006 after the preamble's shift) run
the per-tile frame lists, the K-chunk probe reduction and the error-slot layout
at the size the headline is measured on.  The start is a near-converged FP64
state: the true object under the shifted scan, times 1 + 5 % noise, the
benchmark's perturbed probe and the true background shape.  Contract: one
iteration within 1e-5 relative on O, P, the background and eMod
(era.py:220-291, dm.py:165-294).
"""
import numpy as np
import pytest

import bench
import ptychography_gb300 as pty
from gpu_util import rel
from oracle import ptycho_oracle as orc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def state():
    w = bench.workload_c1(bench.numpy_intensities)
    N = w.N
    d = w.R.max(axis=0)                              # the preamble's shift (era.py:504-505)
    U = N + int(w.R[:, 0].max() - w.R[:, 0].min())
    V = N + int(w.R[:, 1].max() - w.R[:, 1].min())
    rng = np.random.default_rng(77)
    O = w.O_true[-d[0]:-d[0] + U, -d[1]:-d[1] + V]
    O = O * (1 + 0.05 * (rng.standard_normal(O.shape) + 1j * rng.standard_normal(O.shape)))
    y, x = np.mgrid[:N, :N] - N / 2
    B = 0.01 * float(w.I.mean()) * np.exp(-(x ** 2 + y ** 2) / (2 * 40.0 ** 2))
    return w, O, B


def _compare(res_g, res_o):
    O_g, P_g, ig = res_g
    O_o, P_o, io = res_o
    assert O_g.shape == O_o.shape == (1006, 1006)
    assert rel(O_g, O_o) < 1e-5
    assert rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
    assert ig["eCon"][0] == pytest.approx(io["eCon"][0], rel=1e-4)
    assert rel(ig["background"], io["background"]) < 1e-5


def test_era_m6_one_step_full_geometry(state):
    w, O, B = state
    kw = dict(mask=w.M, method=6, background=B, dtype="double")
    res_o = orc.ERA(w.I, w.R.copy(), w.P0, O, 1, **kw)
    res_g = pty.ERA(w.I, w.R.copy(), w.P0, O, 1, **kw)
    _compare(res_g, res_o)


def test_dm_m6_one_step_full_geometry(state):
    w, O, B = state
    kw = dict(mask=w.M, method=6, background=B, dtype="double")
    res_o = orc.DM(w.I, w.R.copy(), w.P0, O, 1, **kw)
    res_g = pty.DM(w.I, w.R.copy(), w.P0, O, 1, **kw)
    _compare(res_g, res_o)
