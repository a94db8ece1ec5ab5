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


def initial_guess(method, O_true, P_true, B):
    """Initial O, P, background for a method: O from ones when O is updated."""
    upd_O = method in (1, 3, 4, 6)
    upd_P = method in (2, 3, 5, 6)
    O0 = None if upd_O else O_true
    P0 = (P_true * np.exp(0.3j) * 0.9) if upd_P else P_true
    bg = None
    if method == 5:
        bg = B.astype(np.float64) + 1.0
    return O0, P0, bg


