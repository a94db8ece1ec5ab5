"""512 x 512 frames: every tile against the oracle on whole iterations, and
the staged tile's multi-group path.

* Each 512^2 tile (264: staged row / column / row launches; 116: 16-CTA
  clusters with the same three-stage line transforms; 16: 16-CTA clusters with
  16 x 32 line transforms), forced in turn, runs one DM method-6 iteration
  (DM7 recursion, PSI7, the model error) and one ERA method-1 iteration
  (EXIT1) from the oracle's FP64 state on a 16-frame problem shaped like the
  4096-frame benchmark: within 1e-5 relative of the oracle (dm.py:165-294,
  era.py:220-291).
* The staged tile's scratch holds 1024 frames of 512^2; longer launches run
  group by group.  1100 frames through pty_pmod_7 on tile 264 must equal tile
  116 bit for bit (same line transforms and per-pixel code), and frames around
  the group boundary must match the oracle's pmod_7 (era.py:574-595).
"""
import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from gpu_util import Plan, ptr, rel
from oracle import ptycho_oracle as orc
from test_gpu_cluster512 import c4_small
from test_gpu_tiles import candidates, forced_tile

pytestmark = pytest.mark.gpu
N = 512


@pytest.fixture(scope="module")
def c4s():
    I, R, P, O, M = c4_small(seed=14, side=4)
    np.random.seed(19)
    O_k, P_k, info = orc.ERA(I, R.copy(), P * np.exp(0.1j), None, 1, mask=M, method=6, dtype="double")
    return I, R, P, M, O_k, P_k, info["background"]


@pytest.mark.parametrize("tile", [264, 116, 16])
def test_dm_m6_one_step_each_512_tile(c4s, tile):
    assert tile in candidates(N)
    I, R, P, M, O_k, P_k, b = c4s
    kw = dict(mask=M, method=6, background=b, dtype="double")
    O_o, P_o, io = orc.DM(I, R.copy(), P_k, O_k, 1, **kw)
    with forced_tile(N, tile):
        O_g, P_g, ig = pty.DM(I, R.copy(), P_k, O_k, 1, **kw)
    assert rel(O_g, O_o) < 1e-5 and rel(P_g, P_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)
    assert rel(ig["background"], io["background"]) < 1e-5


@pytest.mark.parametrize("tile", [264, 116, 16])
def test_era_m1_one_step_each_512_tile(c4s, tile):
    I, R, P, M, O_k, P_k, b = c4s
    O_o, io = orc.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=1, dtype="double")
    with forced_tile(N, tile):
        O_g, ig = pty.ERA(I, R.copy(), P_k, O_k, 1, mask=M, method=1, dtype="double")
    assert rel(O_g, O_o) < 1e-5
    assert ig["eMod"][0] == pytest.approx(io["eMod"][0], rel=1e-5)


def test_staged_multi_group_matches_cluster_tile_and_oracle():
    n, U = 1100, 600
    gen = torch.Generator(device="cuda")
    gen.manual_seed(1100)
    dev = torch.device("cuda", 0)
    rng = np.random.default_rng(1100)
    R = np.stack([-rng.integers(0, U - N + 1, n), -rng.integers(0, U - N + 1, n)], 1)
    ex = torch.randn((n, N, N), dtype=torch.complex64, device=dev, generator=gen)
    amp = torch.randn((n, N, N), dtype=torch.float32, device=dev, generator=gen).abs_() * 50
    bg = torch.randn((n, N, N), dtype=torch.float32, device=dev, generator=gen).abs_()
    mask_np = rng.random((N, N)) > 0.05
    mask = torch.from_numpy(mask_np.astype(np.uint8)).to(dev)
    outs = {}
    for tile in (264, 116):
        with forced_tile(N, tile):
            plan = Plan(n, N, N, U, U, R)
            try:
                psi, b = ex.clone(), bg.clone()
                e = torch.zeros(1, dtype=torch.float64, device=dev)
                plan.call("pty_pmod_7", ptr(amp), ptr(b), ptr(psi), ptr(mask), 1e-10, ptr(e))
                outs[tile] = (psi, b, float(e.cpu()[0]))
            finally:
                plan.close()
    assert torch.equal(outs[264][0], outs[116][0])
    assert torch.equal(outs[264][1], outs[116][1])
    assert outs[264][2] == pytest.approx(outs[116][2], rel=1e-9)
    sub = slice(1020, 1030)          # frames on both sides of the 1024-frame group boundary
    ref, bref = orc.pmod_7(amp[sub].cpu().numpy().astype(np.float64),
                           bg[sub].cpu().numpy().astype(np.float64),
                           ex[sub].cpu().numpy().astype(np.complex128), mask_np, 1e-10)
    assert rel(outs[264][0][sub].cpu().numpy(), ref) < 4e-6
    assert rel(outs[264][1][sub].cpu().numpy(), bref) < 2e-5
