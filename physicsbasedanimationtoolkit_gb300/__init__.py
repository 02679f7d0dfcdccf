"""GB300-native Vertex Block Descent (VBD) for tetrahedral Stable Neo-Hookean meshes.

A drop-in for PhysicsBasedAnimationToolkit's VBD time step (``pbat.sim.vbd`` / ``pbat.gpu.vbd``):
hand-written sm_103a CUDA kernels behind the C ABI of ``include/pbat_gb300.h``, reached from Python
through ``ctypes``.  ``from physicsbasedanimationtoolkit_gb300 import pbat`` gives the reference's
module shape.
"""

from . import meshgen  # noqa: F401
from . import pbat  # noqa: F401
from ._build import build  # noqa: F401
from ._capi import PbgbError, lib  # noqa: F401

__version__ = "0.1.0"
