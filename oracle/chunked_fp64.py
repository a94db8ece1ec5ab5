"""Chunked FP64 oracle for reconstructions too large for the NumPy oracle.

TEST INFRASTRUCTURE ONLY.  Like ``ptycho_oracle`` this module is a checker:
only the tests call it.  The shipped engine never imports it.

It restates the reference's ERA and DM loops (``ptychography/era.py:13-332``,
``ptychography/dm.py:13-333``, with the set-up of ``era.py:435-548``) in
float64 / complex128 torch arithmetic on a torch device, the transforms run
on chunks of frames so that their temporaries stay bounded.  At 4096 frames
of 512 x 512 the reference's complex128 state (exit waves and their update
copy, 17 GB each, plus the per-frame background and amplitudes) exceeds what
NumPy can hold and process on one host core in reasonable time; on a GPU the
same arithmetic takes seconds per iteration.

Operation order follows the reference step by step (the NumPy oracle's
order), and the overlap sums add the frames one after another in scan order,
as era.py:355-360 and 386-390 do, so results agree with the NumPy oracle to
float64 rounding of the transforms (tests/test_chunked_oracle_cpu.py pins
that on small problems).

Supported: methods 1-6 (object, probe, or object and probe, without or with
a known background), OP_iters = k or (k, m) (k object / probe rounds every
m-th iteration, the object alone in between, with the reference's cached
heatmaps: era.py:163-189, dm.py:56-85 / 104-134), with or without probe
centring (era.py:172-186, dm.py:65-82 / 115-127) and the far-field probe
constraint Pmod_P (era.py:597-610) for the first Pmod_probe iterations.
Anything else raises NotImplementedError.
"""
import numpy as np


def _torch():
    import torch
    return torch


class Problem:
    """The set-up of era.py:435-548 for one reconstruction, on `device`.

    I: (n, N0, N1) centred intensities (NumPy or torch, any float dtype);
    R: (n, >=2) scan offsets (copied, then shifted so that their maximum is
    0, as era.py:504-505 does in place); P, O: complex arrays (O None: ones
    of the preamble's default shape, era.py:480-486); mask: centred (N0, N1)
    bool array or None (all valid); background: the centred (N0, N1)
    background intensity for methods 4 and 6 (era.py:541-544), or None.
    """

    def __init__(self, I, R, P, O, mask, background, device, chunk=256):
        torch = _torch()
        self.dev, self.chunk = device, int(chunk)
        I = I if isinstance(I, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(I))
        self.I = I.to(device)
        self.n, self.N0, self.N1 = (int(s) for s in I.shape)
        R = np.array(R, dtype=np.int64)[:, :2].copy()
        R -= R.max(axis=0)
        self.R = R
        if O is None:
            O = np.ones((self.N0 + int(R[:, 0].max() - R[:, 0].min()),
                         self.N1 + int(R[:, 1].max() - R[:, 1].min())), np.complex128)
        self.O0 = self._c(O)
        self.P0 = self._c(P)
        self.U, self.V = (int(s) for s in self.O0.shape)
        if (-R[:, 0]).max() + self.N0 > self.U or (-R[:, 1]).max() + self.N1 > self.V:
            raise ValueError("a scan window lies outside the object")
        m = np.ones((self.N0, self.N1), bool) if mask is None else np.asarray(mask, bool)
        mc = torch.as_tensor(m.astype(np.float64), device=device)
        self.mask = torch.fft.ifftshift(mc)                           # era.py:499
        # era.py:495: I_norm = sum(mask * I), accumulated here in float64
        self.I_norm = float(sum(float((self.I[s:e].to(torch.float64) * mc).sum()) for s, e in self.chunks()))
        F = torch.fft.fftn(self.P0)                                   # era.py:546-547
        self.Pamp = torch.sqrt((F.conj() * F).real)
        self.bg2d = None
        if background is not None:                                    # era.py:541-544
            b = torch.as_tensor(np.ascontiguousarray(background), device=device).to(torch.float64)
            self.bg2d = torch.sqrt(torch.fft.ifftshift(b))

    def _c(self, a):
        torch = _torch()
        if isinstance(a, torch.Tensor):
            return a.to(device=self.dev, dtype=torch.complex128).clone()
        return torch.as_tensor(np.ascontiguousarray(a)).to(device=self.dev, dtype=torch.complex128)

    def chunks(self):
        for s in range(0, self.n, self.chunk):
            yield s, min(self.n, s + self.chunk)

    def amp(self, s, e):
        """sqrt(I) in the input's precision, then float64, unshifted (era.py:497)."""
        torch = _torch()
        return torch.fft.ifftshift(torch.sqrt(self.I[s:e]).to(torch.float64), dim=(-2, -1))

    # ------------------------------------------------------------ operators
    def window(self, f):
        """Object slice of frame f (era.py:355-358: O[-r0:N0-r0, -r1:N1-r1])."""
        r0, r1 = int(-self.R[f, 0]), int(-self.R[f, 1])
        return slice(r0, r0 + self.N0), slice(r1, r1 + self.N1)

    def make_exits(self, O, P, s, e):
        """psi_f = O[window_f] * P for frames s..e-1 (era.py:426-433)."""
        torch = _torch()
        return torch.stack([O[self.window(f)] for f in range(s, e)]) * P

    def psup_O(self, exits, P):
        """O = sum_f psi_f conj(P) / (sum_f |P|^2 + alpha) over the windows,
        frames added in scan order (era.py:336-369, heatmap era.py:402-410)."""
        torch = _torch()
        num = torch.zeros((self.U, self.V), dtype=torch.complex128, device=self.dev)
        heat = torch.zeros((self.U, self.V), dtype=torch.float64, device=self.dev)
        Pc = P.conj()
        p2 = (P.conj() * P).real
        for s, e in self.chunks():
            prod = exits[s:e] * Pc
            for f in range(s, e):
                w = self.window(f)
                num[w] += prod[f - s]
                heat[w] += p2
        return num, heat

    def psup_P(self, exits, O):
        """P = sum_f psi_f conj(O[window_f]) / (sum_f |O[window_f]|^2 + alpha)
        (era.py:371-400, heatmap era.py:412-417)."""
        torch = _torch()
        num = torch.zeros((self.N0, self.N1), dtype=torch.complex128, device=self.dev)
        heat = torch.zeros((self.N0, self.N1), dtype=torch.float64, device=self.dev)
        Oc = O.conj()
        o2 = (O * O.conj()).real
        for f in range(self.n):
            w = self.window(f)
            num += exits[f] * Oc[w]
            heat += o2[w]
        return num, heat


def _pmod_1(pb, psi, amp, alpha):
    """fftn -> amplitude replacement, masked pixels kept -> ifftn, and the
    frames' eMod sum (era.py:550-572)."""
    torch = _torch()
    F = torch.fft.fftn(psi, dim=(-2, -1))
    Mag = torch.sqrt((F.conj() * F).real) + alpha
    emod = float(((Mag - amp) ** 2 * pb.mask).sum())
    fac = torch.where(pb.mask == 0, torch.ones_like(Mag), amp / Mag)
    return torch.fft.ifftn(F * fac, dim=(-2, -1)), emod


def _pmod_7(pb, psi, bg, amp, alpha):
    """fftn -> amplitude replacement with the incoherent background -> ifftn
    (era.py:574-595); masked pixels zeroed in wave and background."""
    torch = _torch()
    F = torch.fft.fftn(psi, dim=(-2, -1))
    Mag = torch.sqrt((F.conj() * F).real + bg ** 2 + alpha)
    emod = float(((Mag - amp) ** 2 * pb.mask).sum())
    fac = pb.mask * amp / Mag
    return torch.fft.ifftn(F * fac, dim=(-2, -1)), bg * fac, emod


def _model_error(pb, ex, b, amp):
    """sum mask (sqrt(|fftn psi|^2 + b^2) - amp)^2, no alpha (dm.py:337-341)."""
    torch = _torch()
    F = torch.fft.fftn(ex, dim=(-2, -1))
    Mag = torch.sqrt((F.conj() * F).real + b ** 2)
    return float((pb.mask * (Mag - amp) ** 2).sum())


def _pmod_P(pb, P, alpha):
    """Far-field probe modulus |fftn P| -> Pamp, masked pixels kept (era.py:597-610)."""
    torch = _torch()
    F = torch.fft.fftn(P)
    Mag = torch.sqrt((F.conj() * F).real) + alpha
    fac = torch.where(pb.mask == 0, torch.ones_like(Mag), pb.Pamp / Mag)
    return torch.fft.ifftn(F * fac)


def _probe_shift(P):
    """rint(centre of mass of |P|^2) - shape // 2 (era.py:172-176)."""
    torch = _torch()
    a = (P.conj() * P).real
    tot = a.sum()
    i = torch.arange(a.shape[0], dtype=torch.float64, device=a.device)
    j = torch.arange(a.shape[1], dtype=torch.float64, device=a.device)
    c0 = float((a.sum(dim=1) * i).sum() / tot)
    c1 = float((a.sum(dim=0) * j).sum() / tot)
    return int(np.rint(c0)) - a.shape[0] // 2, int(np.rint(c1)) - a.shape[1] // 2


def _roll2(x, s):
    """Periodic shift of the last two axes by s (multiroll, era.py:631-740)."""
    torch = _torch()
    return torch.roll(x, shifts=(int(s[0]), int(s[1])), dims=(-2, -1))


def _pmod_count(Pmod_probe, iters):
    """The iterations i with i < Pmod_probe (era.py:193)."""
    if Pmod_probe is None or Pmod_probe is False:
        return 0
    x = float(Pmod_probe)
    return iters if x == float("inf") else max(0, min(iters, int(np.ceil(x))))


_UPDATE = {1: "O", 2: "P", 3: "OP", 4: "O", 5: "P", 6: "OP"}   # era.py:451-456


def _check(method):
    if method not in _UPDATE:
        raise NotImplementedError("the chunked oracle restates methods 1-6")


def _econ(bak, cur):
    """sqrt(|bak - cur|^2 / |cur|^2) on the snapshot vector (era.py:201-208)."""
    torch = _torch()
    d = bak - cur
    return float(torch.sqrt((d.conj() * d).real.sum() / (cur.conj() * cur).real.sum()))


def _snap(update, O, P):
    torch = _torch()
    if update == "O":
        return O.reshape(-1).clone()
    if update == "P":
        return P.reshape(-1).clone()
    return torch.cat((O.reshape(-1), P.reshape(-1)))


def _mean_frames(pb, bg):
    """np.mean(background, axis=0) (era.py:265-270, dm.py:203-207): a sum of
    the frames in order, divided by their count."""
    acc = bg[0].clone()
    for f in range(1, pb.n):
        acc += bg[f]
    return acc / pb.n


def _op_iters(OP_iters):
    """(rounds, every) from an int k or a pair (era.py:458-463)."""
    if isinstance(OP_iters, (int, np.integer)):
        return int(OP_iters), 1
    k, m = (int(x) for x in OP_iters)
    if k < 1 or m < 1:
        raise NotImplementedError("OP_iters must be positive")
    return k, m


def _psup_O(pb, exits, P, P_heat, alpha):
    """psup_O with the reference's heatmap cache: a given P_heat is used as
    it is, even when P has changed since (era.py:336-369)."""
    num, heat = pb.psup_O(exits, P)
    P_heat = heat if P_heat is None else P_heat
    return num / (P_heat + alpha), P_heat


def _psup_P(pb, exits, O, O_heat, alpha):
    """psup_P with the reference's heatmap cache (era.py:371-400)."""
    num, heat = pb.psup_P(exits, O)
    O_heat = heat if O_heat is None else O_heat
    return num / (O_heat + alpha), O_heat


def _op_round(pb, exits, O, P, rounds, alpha):
    """`rounds` alternating object and probe projections, heatmaps recomputed
    each time; returns the last round's heatmaps (the object's from the probe
    before its update), as era.py:166-171 leaves them."""
    for _ in range(rounds):
        O, Ph = _psup_O(pb, exits, P, None, alpha)
        P, Oh = _psup_P(pb, exits, O, None, alpha)
    return O, P, Ph, Oh


def ERA(pb, iters, method, alpha=1e-10, probe_centering=False, Pmod_probe=False, OP_iters=1):
    """Error reduction (era.py:13-332) for methods 1-6.  Returns (O, P, info)
    with info keys eMod, eCon, heatmap and, for methods 4-6, background
    (fftshift(b)^2 of the frames' common background)."""
    torch = _torch()
    _check(method)
    update = _UPDATE[method]
    use_bg = method >= 4
    if use_bg and pb.bg2d is None:
        raise NotImplementedError("methods 4-6 need the known background here")
    rounds, every = _op_iters(OP_iters)
    O, P = pb.O0.clone(), pb.P0.clone()
    exits = torch.empty((pb.n, pb.N0, pb.N1), dtype=torch.complex128, device=pb.dev)
    for s, e in pb.chunks():
        exits[s:e] = pb.make_exits(O, P, s, e)                  # era.py:536
    bg = pb.bg2d.expand(pb.n, pb.N0, pb.N1).clone() if use_bg else None
    P_heat = O_heat = None
    npm = _pmod_count(Pmod_probe, iters)
    eMods, eCons = [], []
    for i in range(iters):
        bak = _snap(update, O, P)
        emod = 0.0
        for s, e in pb.chunks():                                # era.py:160 / 230
            if use_bg:
                exits[s:e], bg[s:e], em = _pmod_7(pb, exits[s:e], bg[s:e], pb.amp(s, e), alpha)
            else:
                exits[s:e], em = _pmod_1(pb, exits[s:e], pb.amp(s, e), alpha)
            emod += em
        if update == "O":                                       # era.py:163 / 233
            O, P_heat = _psup_O(pb, exits, P, P_heat, alpha)
        elif update == "P":                                     # era.py:164 / 234
            P, O_heat = _psup_P(pb, exits, O, O_heat, alpha)
        elif i % every == 0:                                    # era.py:166-186
            O, P, P_heat, O_heat = _op_round(pb, exits, O, P, rounds, alpha)
            if probe_centering:
                cm = _probe_shift(P)
                P, O = _roll2(P, (-cm[0], -cm[1])), _roll2(O, (-cm[0], -cm[1]))
                P_heat = O_heat = None
        else:                                                   # era.py:188-189
            O, P_heat = _psup_O(pb, exits, P, P_heat, alpha)
        if i < npm:                                             # era.py:193-194
            P = _pmod_P(pb, P, alpha)
        if use_bg:                                              # era.py:265-270
            bg[:] = _mean_frames(pb, bg)
        for s, e in pb.chunks():                                # era.py:196 / 272
            exits[s:e] = pb.make_exits(O, P, s, e)
        eCons.append(_econ(bak, _snap(update, O, P)))
        eMods.append(float(np.sqrt(emod / pb.I_norm)))
    info = {"eMod": eMods, "eCon": eCons, "heatmap": P_heat}
    if use_bg:
        info["background"] = torch.fft.fftshift(bg[0]) ** 2
    return O, P, info


def DM(pb, iters, method, alpha=1e-10, probe_centering=False, Pmod_probe=False, OP_iters=1):
    """Difference map (dm.py:13-333) for methods 1-6.  Returns (O, P, info)
    like ERA; info's background is the frames' mean of the last metric
    projection (dm.py:308-318)."""
    torch = _torch()
    _check(method)
    update = _UPDATE[method]
    use_bg = method >= 4
    if use_bg and pb.bg2d is None:
        raise NotImplementedError("methods 4-6 need the known background here")
    rounds, every = _op_iters(OP_iters)
    O, P = pb.O0.clone(), pb.P0.clone()
    exits = torch.empty((pb.n, pb.N0, pb.N1), dtype=torch.complex128, device=pb.dev)
    for s, e in pb.chunks():
        exits[s:e] = pb.make_exits(O, P, s, e)                  # era.py:536
    bg = pb.bg2d.expand(pb.n, pb.N0, pb.N1).clone() if use_bg else None
    P_heat = O_heat = None
    b0 = None
    npm = _pmod_count(Pmod_probe, iters)
    eMods, eCons = [], []
    bak = _snap(update, O, P)                                   # dm.py:35-38
    for i in range(iters):
        if use_bg:                                              # dm.py:171
            for s, e in pb.chunks():
                exits[s:e], bg[s:e], _ = _pmod_7(pb, exits[s:e], bg[s:e], pb.amp(s, e), alpha)
        # main consistency projection (dm.py:56-85 / 174-202)
        if update == "O":
            O, P_heat = _psup_O(pb, exits, P, P_heat, alpha)
        elif update == "P":
            P, O_heat = _psup_P(pb, exits, O, O_heat, alpha)
        elif i % every == 0:
            O, P, P_heat, O_heat = _op_round(pb, exits, O, P, rounds, alpha)
            if probe_centering:                                 # dm.py:65-82 / 183-200
                cm = _probe_shift(P)
                P, O = _roll2(P, (-cm[0], -cm[1])), _roll2(O, (-cm[0], -cm[1]))
                P_heat = O_heat = None
                for s, e in pb.chunks():
                    exits[s:e] = _roll2(exits[s:e], (-cm[0], -cm[1]))
        else:
            O, P_heat = _psup_O(pb, exits, P, P_heat, alpha)
        if i < npm:                                             # dm.py:88-89
            P = _pmod_P(pb, P, alpha)
        # difference-map update (dm.py:91-97 / 203-224), frame chunk by chunk:
        # exits -= ex0; ex0 -= exits (= 2 ex0 - psi); the background likewise
        # against its frame mean; then the modulus projection of the
        # reflected pair and exits += its result
        if use_bg:
            b0 = _mean_frames(pb, bg)
        for s, e in pb.chunks():
            ex0 = pb.make_exits(O, P, s, e)
            ps = exits[s:e] - ex0
            ex0 = ex0 - ps
            if use_bg:
                bgs = bg[s:e] - b0
                bx = b0 - bgs
                ex0, bx, _ = _pmod_7(pb, ex0, bx, pb.amp(s, e), alpha)
                exits[s:e] = ps + ex0
                bg[s:e] = bgs + bx
            else:
                ex0, _ = _pmod_1(pb, ex0, pb.amp(s, e), alpha)
                exits[s:e] = ps + ex0
        # metric projection (dm.py:104-137 / 231-271): from copies of O, P;
        # an object-only step projects with P itself and shares the main
        # branch's heatmap cache, an OP round keeps its heatmaps to itself
        Os, Ps = O.clone(), P.clone()
        if update == "O":
            Os, P_heat = _psup_O(pb, exits, Ps, P_heat, alpha)
        elif update == "P":
            Ps, O_heat = _psup_P(pb, exits, Os, O_heat, alpha)
        elif i % every == 0:
            Os, Ps, _, _ = _op_round(pb, exits, Os, Ps, rounds, alpha)
            if probe_centering:                                 # dm.py:115-127 / 242-254
                cm = _probe_shift(Ps)
                Ps, Os = _roll2(Ps, (-cm[0], -cm[1])), _roll2(Os, (-cm[0], -cm[1]))
        else:
            Os, P_heat = _psup_O(pb, exits, P, P_heat, alpha)
        if i < npm:                                             # dm.py:136-137
            Ps = _pmod_P(pb, Ps, alpha)
        if use_bg:
            b0 = _mean_frames(pb, bg)
        emod = 0.0
        for s, e in pb.chunks():
            ex0 = pb.make_exits(Os, Ps, s, e)
            emod += _model_error(pb, ex0, b0 if use_bg else 0.0, pb.amp(s, e))
        cur = _snap(update, Os, Ps)
        eCons.append(_econ(bak, cur))                           # dm.py:142-149
        eMods.append(float(np.sqrt(emod / pb.I_norm)))
        bak = cur                                               # dm.py:158-160
    info = {"eMod": eMods, "eCon": eCons, "heatmap": P_heat}
    if use_bg:
        info["background"] = torch.fft.fftshift(b0) ** 2
    return O, P, info
