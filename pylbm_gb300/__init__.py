"""GB300 stream+collide backend for pylbm (``generator='cuda'``).

``Simulation`` runs pylbm's per-time-step hot path -- the fused pull
streaming, moment relaxation and boundary-node updates -- as sm_103a kernels
behind pylbm's ``Simulation(dico)`` / ``one_time_step()`` / ``m[...]`` API.
The C ABI of the kernels is declared in include/lbm_gb300.h.
"""
from . import boundary as bc
from .boundary import (AntiBounceBack, BounceBack, BouzidiAntiBounceBack, BouzidiBounceBack, Neumann, NeumannX,
                       NeumannY, NeumannZ)
from .domain import Domain
from .geometry import (Circle, CylinderCircle, CylinderEllipse, CylinderTriangle, Ellipse, Ellipsoid, Parallelepiped,
                       Parallelogram, Sphere, Triangle)
from .output import H5File
from .runtime import pinned_empty
from .scheme import Scheme, SchemeError
from .simulation import Simulation
from .stencil import Stencil

__version__ = "0.1.0"

__all__ = ["Simulation", "Scheme", "SchemeError", "Domain", "Stencil", "Circle", "Ellipse", "Parallelogram", "Triangle",
           "Sphere", "Ellipsoid", "CylinderCircle", "CylinderEllipse", "CylinderTriangle", "Parallelepiped",
           "H5File", "pinned_empty", "bc", "BounceBack", "AntiBounceBack", "BouzidiBounceBack", "BouzidiAntiBounceBack", "Neumann",
           "NeumannX", "NeumannY", "NeumannZ"]
