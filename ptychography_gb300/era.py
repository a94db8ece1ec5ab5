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


def ERA_batch(problems, iters, OP_iters=1, mask=1, background=None, method=None, Pmod_probe=False,
              probe_centering=False, hardware='cpu', alpha=1.0e-10, dtype=None, full_output=True):
    """Many independent ERA reconstructions launched together (no reference counterpart).

    ``problems`` is a sequence of ``(I, R, P, O)`` tuples or of dicts holding
    ``I``, ``R``, ``P``, ``O`` and any per-problem overrides of the keyword
    arguments (``mask``, ``background``, ``method``, ``OP_iters``,
    ``Pmod_probe``, ``probe_centering``, ``alpha``, ``dtype``).  All
    reconstructions run ``iters`` iterations inside one CUDA graph, one branch
    each, so small problems fill the GPU together.  Returns the list of what
    ``ERA`` returns for each problem; the results equal those of separate ERA
    calls made in the same order (NumPy's global RNG is drawn in that order).
    """
    defaults = dict(OP_iters=OP_iters, mask=mask, background=background, method=method,
                    Pmod_probe=Pmod_probe, probe_centering=probe_centering, alpha=alpha,
                    dtype=dtype, full_output=full_output)
    return _engine.run_batch("era", problems, iters, defaults)
