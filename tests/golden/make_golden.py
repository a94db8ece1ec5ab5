"""Generate the golden fixtures from the reference implementation itself.

Run from the repository root with ``PTY_REFERENCE_ROOT`` naming the root of a
reference checkout (the directory holding ``ptychography/era.py``)::

    PTY_REFERENCE_ROOT=<reference checkout> python tests/golden/make_golden.py

It loads the reference's own ``era``/``dm``/``forward_models`` through
``reference_loader`` (Python-2 spellings rewritten at load time, single-rank MPI)
and records, for small seeded problems:

* ``forward_sim.npz``    -- forward_sim outputs (forward_models.py:12-203)
* ``ops.npz``            -- each hot-path operator on seeded inputs (era.py:336-610,
                            dm.py:337-341)
* ``runs.npz``           -- full ERA / DM runs, methods 1-6, FP64 and FP32, with
                            the options that change control flow (OP_iters,
                            probe_centering, Pmod_probe)

The fixtures are what pins the CPU oracle (``oracle/ptycho_oracle.py``) to the
reference; the GPU tests then compare the CUDA engine with the oracle.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import reference_loader  # noqa: E402
from cases import ITERS, initial_guess, run_cases  # noqa: E402

def base_problem(ref, seed=1234, shape_P=(32, 32), shape_O=(56, 56), ny=3, nx=3):
    np.random.seed(seed)
    I, R, M, P, O, B = ref.forward_models.forward_sim(
        shape_P=shape_P, shape_O=shape_O, A=9, defocus=0.02, photons_pupil=100.0,
        ny=ny, nx=nx, random_offset=3, background=2, mask=12, counting_statistics=False)
    return I, R, M, P, O, B


def make_runs(ref, I, R, M, P, O, B):
    out = {}
    for name, drv, m, dt, kw in run_cases():
        O0, P0, bg = initial_guess(m, O, P, B, I, R)
        if kw.get("probe_centering"):
            P0 = np.roll(P0, (3, -2), axis=(0, 1))   # give the centring a shift to undo
        Rc = R.copy()
        np.random.seed(99)
        f = ref.era.ERA if drv == "ERA" else ref.dm.DM
        Iin = I.astype(np.float32) if dt == "single" else I
        res = f(Iin, Rc, P0, O0, ITERS, mask=M, method=m, background=bg, dtype=dt,
                full_output=True, **kw)
        info = res[-1]
        upd = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}[m]
        if upd == "O":
            out[name + "/O"] = res[0]
        elif upd == "P":
            out[name + "/P"] = res[0]
        else:
            out[name + "/O"] = res[0]
            out[name + "/P"] = res[1]
        out[name + "/eMod"] = np.array(info["eMod"], dtype=np.float64)
        out[name + "/eCon"] = np.array(info["eCon"], dtype=np.float64)
        out[name + "/R_after"] = Rc
        Iout = np.asarray(info["I"])
        out[name + "/I_f32"] = Iout.astype(np.float32)
        out[name + "/I_sum"] = np.array([Iout.astype(np.float64).sum(),
                                         (Iout.astype(np.float64) ** 2).sum()])
        if info.get("heatmap") is not None:
            out[name + "/heatmap"] = info["heatmap"]
        if "background" in info:
            out[name + "/background"] = info["background"]
        print("  %-26s eMod[-1]=%.6e eCon[-1]=%.6e" % (name, info["eMod"][-1], info["eCon"][-1]))
    return out


def make_ops(ref):
    era, dm = ref.era, ref.dm
    rng = np.random.default_rng(7)
    n, N0, N1, U, V = 4, 32, 64, 56, 88
    R = np.stack([-rng.integers(0, U - N0 + 1, n), -rng.integers(0, V - N1 + 1, n)], 1)
    O = rng.standard_normal((U, V)) + 1j * rng.standard_normal((U, V))
    P = rng.standard_normal((N0, N1)) + 1j * rng.standard_normal((N0, N1))
    ex = rng.standard_normal((n, N0, N1)) + 1j * rng.standard_normal((n, N0, N1))
    amp = np.abs(rng.standard_normal((n, N0, N1))) * 5
    bg = np.abs(rng.standard_normal((n, N0, N1)))
    mask = rng.random((N0, N1)) > 0.1
    alpha = 1.0e-10
    d = dict(R=R, O=O, P=P, exits=ex, amp=amp, bg=bg, mask=mask)
    d["make_exits"] = era.make_exits(O, P, R)
    e1, em1 = era.pmod_1(amp, ex.copy(), mask, alpha=alpha, eMod_calc=True)
    d["pmod_1"], d["pmod_1_eMod"] = e1, np.array(em1)
    e7, b7, em7 = era.pmod_7(amp, bg.copy(), ex.copy(), mask, alpha=alpha, eMod_calc=True)
    d["pmod_7"], d["pmod_7_bg"], d["pmod_7_eMod"] = e7, b7, np.array(em7)
    Pamp = np.abs(np.fft.fftn(P)) * 1.3
    d["Pamp"] = Pamp
    d["Pmod_P"] = era.Pmod_P(Pamp, P.copy(), mask, alpha)
    Oo, hP = era.psup_O(ex, P, R, O.shape, None, alpha)
    d["psup_O"], d["P_heatmap"] = Oo, hP
    Pp, hO = era.psup_P(ex, O, R, None, alpha)
    d["psup_P"], d["O_heatmap"] = Pp, hO
    d["model_error_1"] = np.array(dm.model_error_1(amp, ex, mask, bg))
    d["model_error_1_nobg"] = np.array(dm.model_error_1(amp, ex, mask))
    d["multiroll"] = era.multiroll(O, [-7, 13])
    return d


def main():
    ref = reference_loader.load_reference()
    I, R, M, P, O, B = base_problem(ref)
    np.savez_compressed(os.path.join(HERE, "forward_sim.npz"), I=I, R=R, M=M, P=P, O=O, B=B,
                        seed=1234)
    # a second forward_sim with Poisson statistics and a rectangular probe
    np.random.seed(4321)
    I2, R2, M2, P2, O2, B2 = ref.forward_models.forward_sim(
        shape_P=(32, 64), shape_O=(80, 96), A=10, defocus=0.01, photons_pupil=50.0,
        ny=3, nx=2, random_offset=4, background=3, mask=8, counting_statistics=True)
    np.savez_compressed(os.path.join(HERE, "forward_sim_rect.npz"), I=I2, R=R2, M=M2, P=P2,
                        O=O2, B=B2, seed=4321)
    # Back_projection (back_projection.py:4-88) on the base problem.  The probe
    # is perturbed by seeded noise: forward_sim's band-limited pupil has exact
    # spectral zeros whose angle() is rounding noise, which would make the
    # back-projected phases depend on the FFT library's rounding.
    rng = np.random.default_rng(21)
    Pb = P * (1 + 0.1 * (rng.standard_normal(P.shape) + 1j * rng.standard_normal(P.shape)))
    Rb = R.copy()
    Ob, info_b = ref.back_projection.Back_projection(I, Rb, Pb, None, mask=M, alpha=1e-10)
    np.savez_compressed(os.path.join(HERE, "back_projection.npz"), O=Ob, heatmap=info_b["heatmap"],
                        exits=info_b["exits"], R_after=Rb, P=Pb)
    print("ops ...")
    np.savez_compressed(os.path.join(HERE, "ops.npz"), **make_ops(ref))
    print("runs ...")
    np.savez_compressed(os.path.join(HERE, "runs.npz"), **make_runs(ref, I, R, M, P, O, B))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print("%-22s %8.1f KB" % (f, os.path.getsize(os.path.join(HERE, f)) / 1024))


if __name__ == "__main__":
    main()
