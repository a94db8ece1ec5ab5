"""Drop-in ``DM`` (ptychography/dm.py:13-333) running on the GPU.

Note the reference's positional order after ``background`` differs from ERA's:
``Pmod_probe, probe_centering, method``.  Returns the main-branch object /
probe; ``eMod``, ``eCon`` and ``info['I']`` describe the metric projection, as in
the reference (dm.py:104-160, 296-318).
"""
from . import _engine


def DM(I, R, P, O, iters, OP_iters=1, mask=1, background=None, Pmod_probe=False,
       probe_centering=False, method=None, hardware='cpu', alpha=1.0e-10, dtype=None,
       full_output=True):
    """Difference-map ptychography (dm.py:13)."""
    return _engine.run("dm", I, R, P, O, iters, OP_iters, mask, background, method, Pmod_probe,
                       probe_centering, alpha, dtype, full_output)


def DM_batch(problems, iters, OP_iters=1, mask=1, background=None, Pmod_probe=False,
             probe_centering=False, method=None, hardware='cpu', alpha=1.0e-10, dtype=None,
             full_output=True):
    """Many independent DM reconstructions launched together (no reference counterpart).

    Same problem format and result list as ``ERA_batch``; each result equals
    that of a separate ``DM`` call made in the same order.
    """
    defaults = dict(OP_iters=OP_iters, mask=mask, background=background, method=method,
                    Pmod_probe=Pmod_probe, probe_centering=probe_centering, alpha=alpha,
                    dtype=dtype, full_output=full_output)
    return _engine.run_batch("dm", problems, iters, defaults)
