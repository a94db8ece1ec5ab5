"""GB300-native ptychographic reconstruction, a drop-in for the ERA / DM /
forward_sim API of andyofmelbourne/Ptychography.

    import ptychography_gb300 as pty
    I, R, M, P, O, B = pty.forward_sim(...)
    O, info = pty.ERA(I, R, P, None, 100, mask=M, method=1)

The reconstruction loops run in libptycho_gb300.so (hand-written sm_103a CUDA,
C ABI in include/ptycho_gb300.h); Python prepares inputs and returns outputs.
"""
from . import back_projection, cxi, dm, era, forward_models, warmstart  # noqa: F401
from ._engine import release_plan_cache
from .back_projection import Back_projection
from .dm import DM, DM_batch
from .era import ERA, ERA_batch
from .cxi import read_cxi, write_cxi
from .forward_models import forward_sim
from .warmstart import WarmStartNet

__all__ = ["ERA", "DM", "ERA_batch", "DM_batch", "write_cxi", "read_cxi", "forward_sim", "Back_projection",
           "WarmStartNet", "release_plan_cache", "era", "dm", "forward_models", "back_projection", "warmstart"]
__version__ = "0.1.0"
