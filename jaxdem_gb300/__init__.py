"""jaxdem_gb300: GB300-native engine for JaxDEM's per-step hot path.

Drop-in host API mirroring ``jaxdem`` (``State``, ``System``, the component
factories and their registry keys) over a CUDA engine for sm_103a exposed
through a C ABI (``include/jdem_gb300.h``).  Every step, force, energy and
neighbour-list evaluation runs on the GPU; there is no CPU fallback.
"""

from . import utils
from ._lib import Engine, JdemError
from .colliders import Collider, DynamicCellList, NaiveSimulator
from .domains import Domain, FreeDomain, PeriodicDomain, ReflectDomain
from .factory import Factory
from .forces import ForceManager, ForceModel, SpringForce
from .integrators import Integrator, LinearIntegrator, RotationIntegrator
from .materials import Material, MaterialMatchmaker, MaterialTable
from .state import Quaternion, State
from .system import System

__version__ = "0.1.0"

__all__ = [
    "Collider", "DynamicCellList", "NaiveSimulator", "Domain", "FreeDomain", "PeriodicDomain", "ReflectDomain",
    "Engine", "Factory", "ForceManager", "ForceModel", "Integrator", "JdemError", "LinearIntegrator",
    "Material", "MaterialMatchmaker", "MaterialTable", "Quaternion", "RotationIntegrator", "SpringForce",
    "State", "System", "utils",
]
