"""Drop-in ``ERA`` (ptychography/era.py:13-332) running on the GPU.

Same signature, positional order, return tuple and ``info`` keys as the
reference.  ``hardware`` is accepted and ignored, as in the reference; the
computation always runs in libptycho_gb300 (complex64 bulk, float-float
accumulated denominators and error sums).
"""
from . import _engine


def ERA(I, R, P, O, iters, OP_iters=1, mask=1, background=None, method=None, Pmod_probe=False,
        probe_centering=False, hardware='cpu', alpha=1.0e-10, dtype=None, full_output=True):
    """Error-reduction ptychography (era.py:13).

    Returns ``(O, info)``, ``(P, info)`` or ``(O, P, info)`` for methods updating
    the object, the probe, or both; without ``full_output`` only the arrays.
    ``R`` is shifted in place so that its maximum is 0 (era.py:504-505).
    """
    return _engine.run("era", I, R, P, O, iters, OP_iters, mask, background, method, Pmod_probe,
                       probe_centering, alpha, dtype, full_output)
