"""The 4096-frame 512 x 512 reconstruction (DM method 6: object, probe and
background) against the chunked FP64 oracle.

The benchmark's own data (bench.DeviceWorkload: 64 x 64 raster, step 36 +-4,
object 2816 x 2816, Poisson 1e8, beamstop + dead-pixel mask, known
background) and start (object of ones, the perturbed probe) run three DM
iterations on the engine (FP32 bulk, float-float reductions) and in the
chunked float64 restatement of dm.py:165-294 (oracle/chunked_fp64.py, pinned
to the NumPy oracle by tests/test_chunked_oracle_cpu.py).  After three
iterations the object over the illuminated region (P_heatmap > 1e-3 of its
maximum, the region the object error is reported on), the probe, the
background and every eMod must agree within 3e-5 relative (1e-5 per
iteration, compounded).  Over the whole object the FP32 rounding of the
barely illuminated border, where the overlap update divides tiny sums by
tiny heatmaps, is larger; it is bounded at 1e-3.
"""
import numpy as np
import pytest
import torch

import bench
from oracle import chunked_fp64 as ck

pytestmark = pytest.mark.gpu
ITERS = 3


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_c4_dm_m6_against_chunked_fp64_oracle():
    dev = torch.device("cuda", 0)
    w = bench.DeviceWorkload(dev)
    job = bench.DeviceJob(w, dev)
    job.run("dm", 6, ITERS)
    torch.cuda.synchronize()
    O_g, P_g = job.O.cpu().numpy(), job.P.cpu().numpy()
    emod_g = job.emod[:ITERS].cpu().numpy()
    b_g = np.fft.fftshift(job.bmean.cpu().numpy().astype(np.float64)) ** 2
    U, V = job.U, job.V
    job.close()
    del job
    torch.cuda.empty_cache()
    pb = ck.Problem(w.I_dev, w.R, w.P0, np.ones((U, V), np.complex128), w.M, w.B, dev, chunk=256)
    O_o, P_o, info = ck.DM(pb, ITERS, 6)
    O_o = O_o.cpu().numpy()
    heat = info["heatmap"].cpu().numpy()
    lit = heat > 1e-3 * heat.max()
    eO, eP = _rel(O_g, O_o), _rel(P_g, P_o.cpu().numpy())
    eO_lit = _rel(O_g[lit], O_o[lit])
    eb = _rel(b_g, info["background"].cpu().numpy())
    print("c4 DM m6 x%d vs FP64: O %.2e (illuminated %.2e, %.1f%% of pixels) P %.2e background %.2e "
          "eMod %s" % (ITERS, eO, eO_lit, 100.0 * lit.mean(), eP, eb,
                       np.abs(emod_g / np.array(info["eMod"]) - 1)))
    assert eO_lit < 3e-5 and eP < 3e-5 and eb < 3e-5
    assert eO < 1e-3
    np.testing.assert_allclose(emod_g, info["eMod"], rtol=3e-5)
