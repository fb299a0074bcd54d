"""GB300-native (sm_103a) se_e2_a descriptor hot path.

``libgbdp.so`` (hand-written CUDA behind the C ABI of include/gbdp.h) does the
work; this package binds it with ctypes and registers the reference's
``torch.ops.deepmd`` operators on top of it.
"""

from . import _lib  # noqa: F401
from . import ops  # noqa: F401
from .ops import NeighborPlan, env_mat_packed, register  # noqa: F401


def load_library():
    """Load libgbdp.so and register the torch.ops.deepmd operators."""
    lib = _lib.load()
    ops.register()
    return lib
