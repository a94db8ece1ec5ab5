"""CPU oracle for the ERA / DM ptychography hot path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: the tests, the smoke
check and the CPU-baseline leg of ``bench.py`` call it to produce expected
results.  The shipped engine (``ptychography_gb300``) never imports it, and has
no CPU fallback through it.

It is a NumPy restatement of the reference's algorithm (andyofmelbourne/
Ptychography, ``ptychography/era.py`` and ``ptychography/dm.py``), written to
follow the reference's arithmetic order so that FP64 runs agree with the
reference to rounding, and FP32 runs (``dtype='single'``) use the same
complex64 NumPy arithmetic the reference uses.  The fixtures under
``tests/golden`` were produced by running the reference itself; the CPU test
suite pins this restatement against them.

Every function cites the reference lines it restates.  MPI is absent: the
reference's collectives over one rank are identities, so a single process is
the reference's ``mpirun -n 1`` behaviour.
"""
import numpy as np
import scipy.ndimage

__all__ = [
    "multiroll", "make_exits", "pmod_1", "Pmod_1", "pmod_7", "Pmod_7", "Pmod_P",
    "psup_O", "psup_P", "make_P_heatmap", "make_O_heatmap", "model_error_1",
    "preamble", "probe_shift", "ERA", "DM", "forward_sim_from_object", "Back_projection",
]


# --------------------------------------------------------------------------
# elementary operators
# --------------------------------------------------------------------------
def multiroll(x, shift):
    """Periodic shift of every axis (era.py:631-740): y[i] = x[i - shift]."""
    x = np.asarray(x)
    return np.roll(x, tuple(int(s) for s in shift), axis=tuple(range(x.ndim)))


def _window_index(R, N0, N1, U, V):
    """Object row/col indices of every frame pixel: (a - r0) mod U, (b - r1) mod V."""
    rows = (np.arange(N0)[None, :] - R[:, 0:1]) % U
    cols = (np.arange(N1)[None, :] - R[:, 1:2]) % V
    return rows, cols


def make_exits(O, P, R, exits=None):
    """psi_i = roll(O, R_i)[:N0, :N1] * P (era.py:426-433)."""
    N0, N1 = P.shape
    rows, cols = _window_index(np.asarray(R), N0, N1, O.shape[0], O.shape[1])
    ex = O[rows[:, :, None], cols[:, None, :]] * P
    if exits is None:
        return ex
    exits[...] = ex
    return exits


def Pmod_1(amp, F, mask=1, alpha=1.0e-10, eMod_calc=False):
    """Amplitude replacement, masked pixels kept (era.py:560-572)."""
    Mag = np.sqrt((F.conj() * F).real) + alpha
    eMod = np.sum((Mag - amp) ** 2 * mask) if eMod_calc else None
    fac = amp / Mag
    if not (isinstance(mask, int) and mask == 1):
        bad = np.asarray(mask) == 0
        if bad.any():
            fac[:, bad] = 1.0
    F *= fac
    return F, eMod


def pmod_1(amp, exits, mask=1, alpha=1.0e-10, eMod_calc=False):
    """FFT -> Pmod_1 -> IFFT over the frame axes (era.py:550-558)."""
    F = np.fft.fftn(exits, axes=(-2, -1))
    F, eMod = Pmod_1(amp, F, mask, alpha, eMod_calc)
    out = np.fft.ifftn(F, axes=(-2, -1))
    return (out, eMod) if eMod_calc else out


def Pmod_7(amp, background, F, mask=1, alpha=1.0e-10, eMod_calc=False):
    """Amplitude replacement with incoherent background (era.py:583-595).

    Masked pixels are zeroed in both the wave and the background (the factor is
    ``mask * amp / Mag``); the reference's ``mask is 1`` branch never runs for an
    array mask.
    """
    Mag = np.sqrt((F.conj() * F).real + background ** 2 + alpha)
    eMod = np.sum((Mag - amp) ** 2 * mask) if eMod_calc else None
    fac = mask * amp / Mag
    F *= fac
    background *= fac
    return F, background, eMod


def pmod_7(amp, background, exits, mask=1, alpha=1.0e-10, eMod_calc=False):
    """FFT -> Pmod_7 -> IFFT (era.py:574-581)."""
    F = np.fft.fftn(exits, axes=(-2, -1))
    F, background, eMod = Pmod_7(amp, background, F, mask, alpha, eMod_calc)
    out = np.fft.ifftn(F, axes=(-2, -1))
    if eMod_calc:
        return out, background, eMod
    return out, background


def Pmod_P(amp, P, mask=1, alpha=1.0e-10):
    """Far-field probe modulus constraint (era.py:597-610)."""
    F = np.fft.fftn(P, axes=(-2, -1))
    Mag = np.sqrt((F.conj() * F).real) + alpha
    fac = amp / Mag
    if not (isinstance(mask, int) and mask == 1):
        bad = np.asarray(mask) == 0
        if bad.any():
            fac[bad] = 1.0
    F *= fac
    return np.fft.ifftn(F, axes=(-2, -1))


def make_P_heatmap(P, R, shape):
    """sum_i |P|^2 placed at each scan window (era.py:402-410), frames in order."""
    heat = np.zeros(shape, dtype=P.real.dtype)
    p2 = (P.conj() * P).real
    N0, N1 = P.shape
    for r0, r1 in np.asarray(R):
        heat[-r0:N0 - r0, -r1:N1 - r1] += p2
    return heat


def make_O_heatmap(O, R, shape):
    """sum_i |O[R_i window]|^2 (era.py:412-417), frames in order."""
    o2 = (O * O.conj()).real
    acc = np.zeros(O.shape, dtype=O.real.dtype)
    for r0, r1 in np.asarray(R):
        acc += multiroll(o2, (r0, r1))
    return np.ascontiguousarray(acc[:shape[0], :shape[1]])


def psup_O(exits, P, R, O_shape, P_heatmap=None, alpha=1.0e-10):
    """Object overlap projection (era.py:336-369)."""
    if P_heatmap is None:
        P_heatmap = make_P_heatmap(P, R, O_shape)
    num = np.zeros(O_shape, dtype=P.dtype)
    Pc = P.conj()
    N0, N1 = P.shape
    for (r0, r1), ex in zip(np.asarray(R), exits):
        num[-r0:N0 - r0, -r1:N1 - r1] += ex * Pc
    return num / (P_heatmap + alpha), P_heatmap


def psup_P(exits, O, R, O_heatmap=None, alpha=1.0e-10):
    """Probe overlap projection (era.py:371-400)."""
    N0, N1 = exits.shape[1:]
    if O_heatmap is None:
        O_heatmap = make_O_heatmap(O, R, (N0, N1))
    num = np.zeros((N0, N1), dtype=exits.dtype)
    Oc = O.conj()
    for (r0, r1), ex in zip(np.asarray(R), exits):
        num += ex * Oc[-r0:N0 - r0, -r1:N1 - r1]
    return num / (O_heatmap + alpha), O_heatmap


def model_error_1(amp, exits, mask, background=0):
    """sum mask (sqrt(|F psi|^2 + b^2) - amp)^2, no alpha (dm.py:337-341)."""
    F = np.fft.fftn(exits, axes=(-2, -1))
    Mag = np.sqrt((F.conj() * F).real + background ** 2)
    return np.sum(mask * (Mag - amp) ** 2)


def probe_shift(P):
    """Integer shift that centres |P|^2 (era.py:172-176): rint(com) - shape//2."""
    a = (P.conj() * P).real
    com = scipy.ndimage.center_of_mass(a)
    return np.rint(com).astype(int) - np.array(a.shape) // 2


# --------------------------------------------------------------------------
# set-up shared by ERA and DM (era.py:435-548)
# --------------------------------------------------------------------------
def preamble(I, R, P, O, OP_iters, mask, background, method, dtype):
    """Host set-up of era.py:435-548 for one rank.

    Mutates ``R`` in place (era.py:504-505) and draws the random initial probe
    (era.py:488-490) and background (era.py:539-540) from NumPy's global RNG in
    the reference's order.
    """
    if method is None:
        if O is None and P is None:
            method = 3
        elif O is None:
            method = 1
        elif P is None:
            method = 2
        if background is not None:
            method += 3
    update = {1: "O", 4: "O", 2: "P", 5: "P", 3: "OP", 6: "OP"}[method]
    if isinstance(OP_iters, int):
        OP_iters = (OP_iters, 1)

    if dtype is None:
        dtype = "single" if I.dtype == np.float32 else "double"
    rdt, cdt = ((np.float32, np.complex64) if dtype == "single"
                else (np.float64, np.complex128))

    if O is None:
        shape = (I.shape[1] + R[:, 0].max() - R[:, 0].min(),
                 I.shape[2] + R[:, 1].max() - R[:, 1].min())
        O = np.ones(shape, dtype=cdt)
    if P is None:
        P = np.random.random(I[0].shape) + 1J * np.random.random(I[0].shape)
    P = P.astype(cdt)
    O = O.astype(cdt)

    I_norm = np.sum(mask * I)
    amp = np.fft.ifftshift(np.sqrt(I).astype(rdt), axes=(-2, -1))
    mask = np.fft.ifftshift(mask)
    R[:, 0] -= R[:, 0].max()
    R[:, 1] -= R[:, 1].max()

    exits = make_exits(O, P, R)
    if background is None and method in (4, 5, 6):
        background = np.random.random(exits.shape).astype(rdt) + 0.1
    elif method in (4, 5, 6):
        b = np.empty(exits.shape, dtype=rdt)
        b[:] = np.sqrt(np.fft.ifftshift(background))
        background = b

    Pamp = np.fft.fftn(P, axes=(-2, -1))
    Pamp = np.sqrt((Pamp.conj() * Pamp).real)
    return dict(method=method, update=update, dtype=rdt, c_dtype=cdt, OP_iters=OP_iters,
                O=O, P=P, amp=amp, Pamp=Pamp, background=background, R=R, mask=mask,
                I_norm=I_norm, exits=exits)


def _snapshot(update, O, P):
    if update == "O":
        return O.copy()
    if update == "P":
        return P.copy()
    return np.hstack((O.ravel().copy(), P.ravel().copy()))


def _econ(bak, update, O, P):
    cur = O if update == "O" else P if update == "P" else np.hstack((O.ravel(), P.ravel()))
    bak -= cur
    return np.sqrt(np.sum((bak * bak.conj()).real) / np.sum((cur * cur.conj()).real))


def _op_round(exits, O, P, R, OP_iters, alpha):
    for _ in range(OP_iters[0]):
        O, Ph = psup_O(exits, P, R, O.shape, None, alpha)
        P, Oh = psup_P(exits, O, R, None, alpha)
    return O, P, Ph, Oh


# --------------------------------------------------------------------------
# ERA (era.py:13-332)
# --------------------------------------------------------------------------
def ERA(I, R, P, O, iters, OP_iters=1, mask=1, background=None, method=None,
        Pmod_probe=False, probe_centering=False, hardware="cpu", alpha=1.0e-10,
        dtype=None, full_output=True):
    """Error-reduction loop, methods 1-6 (era.py:13-332)."""
    s = preamble(I, R, P, O, OP_iters, mask, background, method, dtype)
    method, update, OP_iters = s["method"], s["update"], s["OP_iters"]
    O, P, amp, Pamp, bg, R, mask, I_norm, exits = (
        s["O"], s["P"], s["amp"], s["Pamp"], s["background"], s["R"], s["mask"],
        s["I_norm"], s["exits"])
    use_bg = method in (4, 5, 6)
    P_heatmap = O_heatmap = None
    eMods, eCons = [], []
    for i in range(iters):
        bak = _snapshot(update, O, P)
        if use_bg:                                            # era.py:230
            exits, bg, eMod = pmod_7(amp, bg, exits, mask, alpha, True)
        else:                                                 # era.py:160
            exits, eMod = pmod_1(amp, exits, mask, alpha, True)
        if update == "O":                                     # era.py:163/233
            O, P_heatmap = psup_O(exits, P, R, O.shape, P_heatmap, alpha)
        elif update == "P":                                   # era.py:164/234
            P, O_heatmap = psup_P(exits, O, R, O_heatmap, alpha)
        else:
            if i % OP_iters[1] == 0:                          # era.py:166-186
                O, P, P_heatmap, O_heatmap = _op_round(exits, O, P, R, OP_iters, alpha)
                if probe_centering:
                    cm = probe_shift(P)
                    P = multiroll(P, -cm)
                    O = multiroll(O, -cm)
                    P_heatmap = O_heatmap = None
            else:                                             # era.py:188-189
                O, P_heatmap = psup_O(exits, P, R, O.shape, P_heatmap, alpha)
        if Pmod_probe is not None and i < Pmod_probe:         # era.py:193-194
            P = Pmod_P(Pamp, P, mask, alpha)
        if use_bg:                                            # era.py:265-270
            bg[:] = np.mean(bg, axis=0)
        exits = make_exits(O, P, R, exits)                    # era.py:196/272
        eCons.append(_econ(bak, update, O, P))                # era.py:201-208
        eMods.append(np.sqrt(eMod / I_norm))                  # era.py:210
    b2d = None
    if bg is not None:                                        # era.py:311-314
        b2d = bg[0] if np.ndim(bg) == 3 else bg
    return _finish(update, O, P, exits, eMods, eCons, P_heatmap, b2d, full_output)


def _finish(update, O, P, exits, eMods, eCons, P_heatmap, b2d, full_output):
    """Outputs of era.py:293-332 / dm.py:296-333."""
    if not full_output:
        return O if update == "O" else P if update == "P" else (O, P)
    info = {
        "I": np.fft.fftshift(np.abs(np.fft.fftn(exits, axes=(-2, -1))) ** 2, axes=(-2, -1)),
        "eMod": eMods,
        "eCon": eCons,
        "heatmap": P_heatmap,
    }
    if b2d is not None:
        info["background"] = np.fft.fftshift(b2d) ** 2
    if update == "O":
        return O, info
    if update == "P":
        return P, info
    return O, P, info


# --------------------------------------------------------------------------
# DM (dm.py:13-333)
# --------------------------------------------------------------------------
def DM(I, R, P, O, iters, OP_iters=1, mask=1, background=None, Pmod_probe=False,
       probe_centering=False, method=None, hardware="cpu", alpha=1.0e-10, dtype=None,
       full_output=True):
    """Difference map, methods 1-6 (dm.py:13-333)."""
    s = preamble(I, R, P, O, OP_iters, mask, background, method, dtype)
    method, update, OP_iters = s["method"], s["update"], s["OP_iters"]
    O, P, amp, Pamp, bg, R, mask, I_norm, exits = (
        s["O"], s["P"], s["amp"], s["Pamp"], s["background"], s["R"], s["mask"],
        s["I_norm"], s["exits"])
    use_bg = method in (4, 5, 6)
    P_heatmap = O_heatmap = None
    eMods, eCons = [], []
    bak = _snapshot(update, O, P)                             # dm.py:35-38
    ex_0 = np.empty_like(exits)
    b_0 = np.empty_like(bg) if use_bg else None
    Os = Ps = None
    for i in range(iters):
        if use_bg:                                            # dm.py:171
            exits, bg = pmod_7(amp, bg, exits, mask, alpha)
        # main consistency projection (dm.py:56-85 / 174-202)
        if update == "O":
            O, P_heatmap = psup_O(exits, P, R, O.shape, P_heatmap, alpha)
        elif update == "P":
            P, O_heatmap = psup_P(exits, O, R, O_heatmap, alpha)
        else:
            if i % OP_iters[1] == 0:
                O, P, P_heatmap, O_heatmap = _op_round(exits, O, P, R, OP_iters, alpha)
                if probe_centering:
                    cm = probe_shift(P)
                    P = multiroll(P, -cm)
                    O = multiroll(O, -cm)
                    P_heatmap = O_heatmap = None
                    exits = multiroll(exits, (0, -cm[0], -cm[1]))
            else:
                O, P_heatmap = psup_O(exits, P, R, O.shape, P_heatmap, alpha)
        if Pmod_probe is not None and i < Pmod_probe:         # dm.py:88-89
            P = Pmod_P(Pamp, P, mask, alpha)
        # difference-map update (dm.py:91-97 / 208-224)
        if use_bg:
            b_0[:] = np.mean(bg, axis=0)
        ex_0 = make_exits(O, P, R, ex_0)
        exits -= ex_0
        ex_0 -= exits
        if use_bg:
            bg -= b_0
            b_0 -= bg
            ex_0, b_0 = pmod_7(amp, b_0, ex_0, mask, alpha)
            exits += ex_0
            bg += b_0
        else:
            ex_0 = pmod_1(amp, ex_0, mask, alpha)
            exits += ex_0
        # metric projection (dm.py:104-137 / 231-271)
        Os = O.copy()
        Ps = P.copy()
        if update == "O":
            Os, P_heatmap = psup_O(exits, Ps, R, O.shape, P_heatmap, alpha)
        elif update == "P":
            Ps, O_heatmap = psup_P(exits, Os, R, O_heatmap, alpha)
        else:
            if i % OP_iters[1] == 0:
                Os, Ps, _, _ = _op_round(exits, Os, Ps, R, OP_iters, alpha)
                if probe_centering:
                    cm = probe_shift(Ps)
                    Ps = multiroll(Ps, -cm)
                    Os = multiroll(Os, -cm)
            else:
                Os, P_heatmap = psup_O(exits, P, R, O.shape, P_heatmap, alpha)
        if Pmod_probe is not None and i < Pmod_probe:
            Ps = Pmod_P(Pamp, Ps, mask, alpha)
        if use_bg:
            b_0[:] = np.mean(bg, axis=0)
        ex_0 = make_exits(Os, Ps, R, ex_0)
        eMod = model_error_1(amp, ex_0, mask, b_0) if use_bg else model_error_1(amp, ex_0, mask)
        eCons.append(_econ(bak, update, Os, Ps))              # dm.py:142-149
        eMods.append(np.sqrt(eMod / I_norm))
        bak = _snapshot(update, Os, Ps)                       # dm.py:158-160
    if full_output:
        exits = make_exits(Os, Ps, R, exits)                  # dm.py:298
    return _finish(update, O, P, exits, eMods, eCons, P_heatmap,
                   b_0[0] if use_bg else None, full_output)


# --------------------------------------------------------------------------
# forward model (forward_models.py:119-203), with the object supplied
# --------------------------------------------------------------------------
def forward_probe(shape_P, A, defocus, photons_pupil):
    """Defocused circular-pupil probe (forward_models.py:124-138)."""
    f0 = np.fft.fftfreq(shape_P[0], 1 / float(shape_P[0]))
    f1 = np.fft.fftfreq(shape_P[1], 1 / float(shape_P[1]))
    i, j = np.meshgrid(f0, f1, indexing="ij")
    q2 = np.fft.fftshift(i ** 2 + j ** 2)
    P = (q2 < A ** 2).astype(np.complex128) * np.sqrt(photons_pupil)
    P *= np.exp(-1.0J * np.pi * defocus * q2)
    return np.fft.fftshift(np.fft.ifftn(np.fft.ifftshift(P)))


def forward_sim_from_object(O, shape_P=(32, 64), A=14, defocus=0., photons_pupil=1,
                            ny=10, nx=10, random_offset=None, background=None,
                            mask=None, counting_statistics=False):
    """forward_sim (forward_models.py:12-203) for a given object ``O``.

    The reference builds ``O`` from two bundled test images
    (forward_models.py:142-144); every later step, including the order of the
    global-RNG draws, is restated here.
    """
    shape_O = O.shape
    P = forward_probe(shape_P, A, defocus, photons_pupil)
    ys = np.rint(np.linspace(0, shape_P[0] - shape_O[0], ny)).astype(int)
    xs = np.rint(np.linspace(0, shape_P[1] - shape_O[1], nx)).astype(int)
    ys, xs = np.meshgrid(ys, xs, indexing="ij")
    R = np.stack([ys.ravel(), xs.ravel()], axis=1)
    if random_offset is not None:                             # forward_models.py:155-160
        R += (np.random.random(R.shape) * int(random_offset)).astype(int)
        R[R > 0] = 0
        R[:, 0][R[:, 0] < shape_P[0] - shape_O[0]] = shape_P[0] - shape_O[0]
        R[:, 1][R[:, 1] < shape_P[1] - shape_O[1]] = shape_P[1] - shape_O[1]
    R[:, 0] -= R[:, 0].max()
    R[:, 1] -= R[:, 1].max()
    F = np.fft.fftn(make_exits(O, P, R), axes=(-2, -1))        # forward_models.py:167-171
    I = np.fft.ifftshift((F.conj() * F).real, axes=(-2, -1))
    if background is not None:                                # forward_models.py:174-179
        B = np.rint(np.random.random(I[0].shape) * background)
        I += B
    else:
        B = 0
    if mask is not None:                                      # forward_models.py:182-188
        ss = (np.random.random(mask) * I.shape[1]).astype(int)
        fs = (np.random.random(mask) * I.shape[2]).astype(int)
        M = np.ones(I[0].shape, dtype=bool)
        M[ss, fs] = False
    else:
        M = 1
    if counting_statistics:                                   # forward_models.py:191-192
        I = np.random.poisson(lam=I)
    if not (isinstance(B, int) and B == 0):
        B = B.astype(I.dtype)
    return I, R, M, P, O, B


# --------------------------------------------------------------------------
# Back_projection (back_projection.py:4-88)
# --------------------------------------------------------------------------
def Back_projection(I, R, P, O, mask=1, alpha=1.0e-10, full_output=True):
    """Back projection with the probe's far-field phases (back_projection.py:4-88).

    The reference calls the nonexistent ``era.psup_O_1``; the object update it
    means is ``psup_O`` (era.py:336-369), used here.  ``sqrt(I)`` and ``mask``
    are used in the given (centred) order against the unshifted fftn(P) phases.
    """
    if O is None:
        O = np.ones((I.shape[1] + R[:, 0].max() - R[:, 0].min(),
                     I.shape[2] + R[:, 1].max() - R[:, 1].min()), dtype=P.dtype)
    R[:, 0] -= R[:, 0].max()
    R[:, 1] -= R[:, 1].max()
    amp = np.sqrt(I.astype(np.float64))
    exits = mask * amp * np.exp(1J * np.angle(np.fft.fftn(P)))
    exits = np.fft.ifftn(exits, axes=(-2, -1))
    O, heat = psup_O(exits, P, R, O.shape, None, alpha)
    if full_output:
        return O, {"exits": exits, "heatmap": heat}
    return O
