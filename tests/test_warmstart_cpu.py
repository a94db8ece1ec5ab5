"""Host-side pieces of the learned warm start (no GPU): the simulated objects
and probes of its training set and the C ABI's argument checks."""
import ctypes

import numpy as np

from ptychography_gb300 import _native
from ptychography_gb300 import warmstart as ws


def test_random_object_and_probe_ranges():
    rng = np.random.default_rng(0)
    O = ws.random_object(rng, 96)
    a, ph = np.abs(O), np.angle(O)
    assert O.shape == (96, 96)
    assert a.min() >= 0.5 - 1e-12 and a.max() <= 1.0 + 1e-12
    assert ph.min() >= -np.pi / 2 - 1e-12 and ph.max() <= np.pi / 2 + 1e-12
    P = ws.aperture_probe(64, 20, 3.0, 0.002)
    y, x = np.mgrid[:64, :64] - 32
    r = np.sqrt(x ** 2 + y ** 2)
    assert np.all(np.abs(P[r < 20]) > 0.999)
    assert np.all(P[r >= 20 + 9] == 0)
    np.testing.assert_allclose(np.angle(P[32, 32 + 5]), 0.002 * 25)


def test_network_layout():
    # six 3 x 3 convolutions, channels 32-128, (cos, sin) output
    # input: (Re, Im) of the back-projected object estimate
    assert len(ws.LAYERS) == 6 and ws.LAYERS[0][0] == 2 and ws.LAYERS[-1][1] == 2
    assert max(c for _, c, _, _ in ws.LAYERS) == 128
    assert [l for _, _, _, l in ws.LAYERS] == [0, 1, 2, 1, 0, 0]


def test_c_abi_rejects_bad_arguments_without_a_gpu():
    lib = _native.load()
    assert lib.pty_ws_gemm(0, 4, 4, None, 1, 1, None, 1, 1, None, 1, 1, 1, None, None) != 0
    assert lib.pty_ws_im2col(1, 0, 4, 4, None, None, None) != 0
    assert lib.pty_ws_pool2(1, 5, 4, 4, None, None, None) != 0        # odd side
    assert lib.pty_ws_act_bwd_scratch(0, 4) == -1
    assert lib.pty_ws_act_bwd_scratch(1000, 4) == 4 * 4                 # ceil(1000 / 256) blocks x C
    assert lib.pty_ws_adam(10, None, None, None, None, None, 1e-3, 0.9, 0.999, 1e-8, 1, None) != 0
    assert lib.pty_ws_prep_bp(1, 0, 8, None, None, 1, None, None) != 0
    one = ctypes.c_void_p(16)                                          # never dereferenced: rejected first
    assert lib.pty_ws_prep_bp(1, 8, 7, one, one, 1, one, None) != 0     # odd side with the sign correction
    assert b"even" in lib.pty_last_error()


def test_covering_frames_lights_every_pixel():
    """The warm start's frame subset: on a dense jittered raster (step 12 px,
    probe radius ~36 px at the network's sampling) it keeps well under half
    the frames, and every pixel the full scan lights gets at least 30 % of
    the best |P|^2 any frame gives it from some kept frame."""
    rng = np.random.default_rng(2)
    side, step, N = 32, 12, 128
    pos = np.arange(side) * step
    R = -np.stack(np.meshgrid(pos, pos, indexing="ij"), -1).reshape(-1, 2)
    R = R + rng.integers(-1, 2, R.shape)
    R = R - R.max(axis=0)
    P = ws.aperture_probe(N, 32, 4.0, 0.002)
    sel = ws.covering_frames(R, P)
    assert 0 < len(sel) < 0.45 * len(R)
    assert np.all(np.diff(sel) > 0)
    p2 = np.abs(P) ** 2
    U, V = N + int(R[:, 0].max() - R[:, 0].min()), N + int(R[:, 1].max() - R[:, 1].min())
    heat, best_all, best = np.zeros((U, V)), np.zeros((U, V)), np.zeros((U, V))
    for f, (r0, r1) in enumerate(R):
        w = (slice(-r0, -r0 + N), slice(-r1, -r1 + N))
        heat[w] += p2
        best_all[w] = np.maximum(best_all[w], p2)
        if f in set(sel.tolist()):
            best[w] = np.maximum(best[w], p2)
    lit = heat > 1e-2 * heat.max()
    assert np.all(best[lit] >= 0.3 * best_all[lit])
