"""Probe centring and the far-field probe constraint at the large-frame scale:
1024 frames of 512 x 512 (the first 1024 positions of the 4096-frame scan of
bench.DeviceWorkload, on the staged 512^2 tile), ERA and DM method 3 (object
and probe) with probe centring and / or Pmod_probe=2, three iterations,
through the public API, against the chunked FP64 oracle (oracle/chunked_fp64.py,
pinned to the NumPy oracle by tests/test_chunked_oracle_cpu.py).  The initial
probe is off centre, so the centring rolls the probe, the object and (DM) the
exit waves.  Bound: 1e-4 relative on the probe, on the object where the probe
lights it and on every eMod, as for the reference's recorded runs
(tests/test_gpu_runs.py)."""
import numpy as np
import pytest
import torch

import bench
import ptychography_gb300 as pty
from oracle import chunked_fp64 as ck

pytestmark = pytest.mark.gpu
ITERS = 3
TOL = 1e-4


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def data():
    dev = torch.device("cuda", 0)
    w = bench.DeviceWorkload(dev, frames=1024)
    P0 = np.roll(w.P0, (5, -3), axis=(0, 1))
    return w, P0, dev


# DM with Pmod_P is left out here: from this probe (a smooth aperture with a
# small defocus, whose far field is at rounding level over most of the
# detector) the probe's far-field constraint makes DM ill-conditioned in FP32:
# the NumPy oracle's own FP32 and FP64 runs of a 128^2 version of this job
# (DM method 3, Pmod_probe=2, ones or ones + noise to start) differ by 4-5 % on
# the probe and 3-9x on eMod, so no FP32 engine can be held to FP64 there.
# DM + Pmod_P parity rests on the reference-recorded DM_m3_opiters_double run
# (tests/test_gpu_runs.py), whose bound includes the reference's own FP32/FP64 gap.
@pytest.mark.parametrize("algo,cent,pmod", [("ERA", True, 2), ("ERA", False, 2), ("DM", False, 0),
                                           ("DM", True, 0)])
def test_centring_and_probe_modulus_512(algo, cent, pmod, data):
    w, P0, dev = data
    I = w.I_dev.cpu().numpy()
    f = pty.ERA if algo == "ERA" else pty.DM
    O_g, P_g, info_g = f(I, w.R.copy(), P0.copy(), None, ITERS, mask=w.M, method=3,
                         probe_centering=cent, Pmod_probe=pmod)
    pb = ck.Problem(w.I_dev, w.R, P0, None, w.M, None, dev, chunk=256)
    O_o, P_o, info_o = getattr(ck, algo)(pb, ITERS, 3, probe_centering=cent, Pmod_probe=pmod)
    O_o, P_o = O_o.cpu().numpy(), P_o.cpu().numpy()
    heat = np.zeros(O_o.shape)
    Rs = w.R - w.R.max(axis=0)
    p2 = np.abs(P_o) ** 2
    for r0, r1 in Rs:
        heat[-r0:-r0 + 512, -r1:-r1 + 512] += p2
    lit = heat > 1e-3 * heat.max()
    eP, eO = _rel(P_g, P_o), _rel(O_g[lit], O_o[lit])
    print("%s m3 centring %s Pmod_probe %d, 1024 x 512^2: P %.2e O (lit) %.2e eMod %s" % (
        algo, cent, pmod, eP, eO, np.abs(np.array(info_g["eMod"]) / np.array(info_o["eMod"]) - 1)))
    assert eP < TOL and eO < TOL
    np.testing.assert_allclose(np.array(info_g["eMod"], float), info_o["eMod"], rtol=TOL)
    if not cent:
        return
    # the probe was moved back to the middle
    a = np.abs(P_g) ** 2
    com = (np.arange(512) @ a.sum(axis=1) / a.sum(), np.arange(512) @ a.sum(axis=0) / a.sum())
    assert abs(com[0] - 256) <= 1.0 and abs(com[1] - 256) <= 1.0
