"""rebound_gb300: GB300-native (sm_103a) force-and-step hot path for REBOUND.

Importing the package loads librebound_gb300.so (built in-tree with nvcc); it
raises if the CUDA library is missing or cannot be built.  There is no CPU
fallback on the product path.
"""
from ._lib import PARTICLE_DTYPE, COLLISION_DTYPE, RGPUError, load  # noqa: F401
from .simulation import Collision, Simulation, Simulationarchive, accelerations  # noqa: F401
from . import ics  # noqa: F401

__version__ = "0.1.0"
