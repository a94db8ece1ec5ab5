"""Frame tiles: every tile built for a shape gives the same exit waves.

128 x 128 frames have a single-CTA kernel and a 2-CTA cluster kernel, 256 x 256
frames 8- and 4-CTA cluster kernels (16 x 16 line transforms) and an 8-CTA
kernel with three-stage 8 x 8 x 4 line transforms (tile 108), 512 x 512
frames the staged row / column / row launches with three-stage 16 x 8 x 4
line transforms (tile 264), a 16-CTA kernel with the same transforms (tile
116) and one with 16 x 32 line transforms (tile 16).  Each tile,
forced in turn, must match the oracle.  Tiles running the same line transforms
give bit-identical exit waves, object and probe (only the error sums, whose
per-CTA partials are grouped differently, may differ in rounding); tiles with
other line transforms agree to FP32 rounding.
"""
import ctypes

import numpy as np
import pytest
import torch

import ptychography_gb300 as pty
from gpu_util import Plan, ptr, rel, to_dev
from oracle import ptycho_oracle as orc
from ptychography_gb300 import _native
from test_gpu_cluster192 import small_problem

pytestmark = pytest.mark.gpu


# tiles sharing a line decomposition (bit-identical results), per frame size
SAME_LINES = {128: [(1, 2)], 256: [(8, 4), (108,)], 512: [(16,), (116, 264)]}


def same_lines(N, t0, t1):
    return any(t0 in grp and t1 in grp for grp in SAME_LINES[N])


def candidates(N):
    lib = _native.load()
    buf = (ctypes.c_int32 * 4)()
    cnt = ctypes.c_int32(0)
    _native.check(lib.pty_frame_tile_candidates(N, N, buf, 4, ctypes.byref(cnt)))
    return [buf[i] for i in range(cnt.value)]


class forced_tile:
    def __init__(self, N, tile):
        self.N, self.tile, self.lib = N, tile, _native.load()

    def __enter__(self):
        for fam in (0, 1):       # plain and background op families
            _native.check(self.lib.pty_set_frame_tile(self.N, self.N, fam, self.tile))

    def __exit__(self, *a):
        for fam in (0, 1):
            self.lib.pty_set_frame_tile(self.N, self.N, fam, 0)


@pytest.mark.parametrize("N", [128, 256, 512])
def test_tiles_listed_and_chosen(N):
    lib = _native.load()
    c = candidates(N)
    assert len(c) == {128: 2, 256: 3, 512: 3}[N]
    for fam in (0, 1):
        t = ctypes.c_int32(0)
        _native.check(lib.pty_get_frame_tile(N, N, fam, ctypes.byref(t)))
        assert t.value in c
    assert lib.pty_set_frame_tile(N, N, 0, 3) == 1    # PTY_ERR_ARG: tile not built
    assert lib.pty_set_frame_tile(N, N, 2, c[0]) == 1  # no such family


def test_mixed_family_tiles_keep_error_sums():
    """Plain and background ops on different tiles in one run: eMod unchanged."""
    N = 256
    I, R, P, O, M = small_problem(N, seed=5, side=3)
    b = np.full((N, N), 0.3, np.float32)
    lib = _native.load()
    try:
        # reference: both families on the 8-CTA tile
        for fam in (0, 1):
            _native.check(lib.pty_set_frame_tile(N, N, fam, 8))
        np.random.seed(4)
        ref = pty.ERA(I, R.copy(), P * np.exp(0.2j), None, 2, mask=M, method=6, background=b)
        # the background family's kernel (EXIT7 here) on 4 CTAs per frame with
        # 8 error slots per frame: slots 4-7 must come back zero
        _native.check(lib.pty_set_frame_tile(N, N, 1, 4))
        np.random.seed(4)
        got = pty.ERA(I, R.copy(), P * np.exp(0.2j), None, 2, mask=M, method=6, background=b)
    finally:
        for fam in (0, 1):
            lib.pty_set_frame_tile(N, N, fam, 0)
    np.testing.assert_array_equal(got[0], ref[0])
    np.testing.assert_array_equal(got[1], ref[1])
    np.testing.assert_allclose(got[2]["eMod"], ref[2]["eMod"], rtol=1e-6)


@pytest.mark.parametrize("N", [128, 256, 512])
def test_pmod_7_every_tile(N):
    rng = np.random.default_rng(N + 7)
    n, U = 5, N + 40
    R = np.stack([-rng.integers(0, U - N + 1, n), -rng.integers(0, U - N + 1, n)], 1)
    ex = rng.standard_normal((n, N, N)) + 1j * rng.standard_normal((n, N, N))
    amp = np.abs(rng.standard_normal((n, N, N))) * 50
    bg = np.abs(rng.standard_normal((n, N, N)))
    mask = rng.random((N, N)) > 0.05
    ref, bref, em = orc.pmod_7(amp, bg.copy(), ex.copy(), mask, 1e-10, True)
    # FP32 rounding of an N^2 transform pair grows with N (b * f weights the
    # small-|F| pixels most)
    tp, tb = (4e-6, 2e-5) if N == 512 else (3e-6, 1e-5)
    outs = []
    for tile in candidates(N):
        with forced_tile(N, tile):
            plan = Plan(n, N, N, U, U, R)
            try:
                psi = to_dev(ex, np.complex64)
                b = to_dev(bg, np.float32)
                # device inputs held by name until the call has synchronised
                amp_d, mask_d = to_dev(amp, np.float32), to_dev(mask, np.uint8)
                e = torch.zeros(1, dtype=torch.float64, device=psi.device)
                plan.call("pty_pmod_7", ptr(amp_d), ptr(b), ptr(psi), ptr(mask_d), 1e-10, ptr(e))
            finally:
                plan.close()
        p = psi.cpu().numpy()
        assert rel(p, ref) < tp, tile
        assert rel(b.cpu().numpy(), bref) < tb, tile
        assert float(e.cpu()[0]) == pytest.approx(em, rel=1e-5)
        outs.append((tile, p, b.cpu().numpy()))
    t0, p0, b0 = outs[0]
    for t, p, b in outs[1:]:
        if same_lines(N, t0, t):
            np.testing.assert_array_equal(p, p0)
            np.testing.assert_array_equal(b, b0)
        else:   # other line transforms: agreement to FP32 rounding
            assert rel(p, p0) < tp and rel(b, b0) < tb


@pytest.mark.parametrize("N", [128, 256, 512])
def test_era_m3_every_tile(N):
    I, R, P, O, M = small_problem(N, seed=N, side=3)
    res = []
    tiles = candidates(N)
    for tile in tiles:
        with forced_tile(N, tile):
            res.append(pty.ERA(I, R.copy(), P * np.exp(0.2j), None, 3, mask=M, method=3))
    for t, (O_t, P_t, info) in zip(tiles[1:], res[1:]):
        if same_lines(N, tiles[0], t):
            np.testing.assert_array_equal(O_t, res[0][0])
            np.testing.assert_array_equal(P_t, res[0][1])
            np.testing.assert_allclose(info["eMod"], res[0][2]["eMod"], rtol=1e-6)
        else:
            # two FP32 rounding paths through three iterations on noisy data
            # (each operator agrees with the FP64 oracle to 3e-6)
            assert rel(O_t, res[0][0]) < 5e-5 and rel(P_t, res[0][1]) < 5e-5
            np.testing.assert_allclose(info["eMod"], res[0][2]["eMod"], rtol=2e-5)


def test_staged_tile_unaligned_amplitudes():
    """Tile 264 copies amplitude rows in 16-byte pieces; an amplitude array
    that is not 16-byte aligned runs through tile 116 (same line transforms):
    the same exit waves and background bit for bit."""
    N, n, U = 512, 3, 560
    rng = np.random.default_rng(11)
    R = np.stack([-rng.integers(0, U - N + 1, n), -rng.integers(0, U - N + 1, n)], 1)
    ex = rng.standard_normal((n, N, N)) + 1j * rng.standard_normal((n, N, N))
    amp = (np.abs(rng.standard_normal((n, N, N))) * 50).astype(np.float32)
    bg = np.abs(rng.standard_normal((n, N, N))).astype(np.float32)
    mask = rng.random((N, N)) > 0.05
    outs = []
    with forced_tile(N, 264):
        plan = Plan(n, N, N, U, U, R)
        try:
            for off in (0, 1):      # amplitudes at a 16-byte boundary, then 4 bytes past one
                psi = to_dev(ex, np.complex64)
                b = to_dev(bg, np.float32)
                buf = torch.zeros(n * N * N + 4, dtype=torch.float32, device=psi.device)
                buf[off:off + n * N * N] = to_dev(amp.ravel())
                amp_d = buf[off:off + n * N * N]
                mask_d = to_dev(mask, np.uint8)
                plan.call("pty_pmod_7", ptr(amp_d), ptr(b), ptr(psi), ptr(mask_d), 1e-10, None)
                outs.append((psi.cpu().numpy(), b.cpu().numpy()))
        finally:
            plan.close()
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
