"""Case definitions shared by the golden-fixture generator and the tests.

The ERA / DM runs recorded in ``runs.npz`` are the product of these cases; the
oracle tests and the GPU parity tests rebuild the same inputs from them.
"""
import numpy as np


ITERS = 4


def run_cases():
    """(name, driver, method, dtype, extra kwargs, initial O?, initial P?, background mode)."""
    cases = []
    for drv in ("ERA", "DM"):
        for m in range(1, 7):
            for dt in ("double", "single"):
                cases.append(("%s_m%d_%s" % (drv, m, dt), drv, m, dt, {}))
    cases += [
        ("ERA_m3_centre_double", "ERA", 3, "double", dict(probe_centering=True, OP_iters=(2, 2))),
        ("ERA_m3_pmodP_double", "ERA", 3, "double", dict(Pmod_probe=2)),
        ("ERA_m6_opiters_single", "ERA", 6, "single", dict(OP_iters=(1, 3), Pmod_probe=np.inf)),
        ("DM_m3_centre_double", "DM", 3, "double", dict(probe_centering=True)),
        ("DM_m3_opiters_double", "DM", 3, "double", dict(OP_iters=(2, 2), Pmod_probe=1)),
        ("DM_m6_centre_single", "DM", 6, "single", dict(probe_centering=True, Pmod_probe=np.inf)),
    ]
    return cases


def default_object_shape(I, R):
    """The preamble's default object shape (era.py:484-486)."""
    return (I.shape[1] + R[:, 0].max() - R[:, 0].min(), I.shape[2] + R[:, 1].max() - R[:, 1].min())


def initial_guess(method, O_true, P_true, B, I=None, R=None):
    """Initial O, P, background for a method.

    Methods 4 and 6 start from the reference's default object (O=None: ones).
    Methods 1 and 3 start from ones plus seeded noise: with forward_sim's
    band-limited pupil probe, O = ones makes |FFT(P O)| exactly zero outside the
    pupil, Pmod_1 (no background term) then scales rounding noise up to the
    measured amplitude, and the reference's own FP32 and FP64 runs disagree by
    O(1) -- a comparison of any FP32 engine with FP64 would be meaningless.
    """
    upd_O = method in (1, 3, 4, 6)
    upd_P = method in (2, 3, 5, 6)
    O0 = None if upd_O else O_true
    if method in (1, 3) and I is not None:
        rng = np.random.default_rng(11)
        shp = default_object_shape(I, R)
        O0 = np.ones(shp) + 0.1 * (rng.standard_normal(shp) + 1j * rng.standard_normal(shp))
    P0 = (P_true * np.exp(0.3j) * 0.9) if upd_P else P_true
    bg = None
    if method == 5:
        bg = B.astype(np.float64) + 1.0
    return O0, P0, bg
