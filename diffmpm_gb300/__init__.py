"""diffmpm_gb300 -- the explicit MPM time step of geoelements/diffmpm on GB300.

The classes mirror the reference's object model (Mesh2D, Particles,
Quadrilateral4Node, MPMExplicit, ...).  Every step runs in the CUDA library
``libdiffmpm_gb300.so`` (C ABI: include/diffmpm_gb300.h); there is no CPU path.
"""
from .constraint import Constraint, ParticleVelocityConstraint
from .element import Linear1D, Quadrilateral4Node
from .engine import Batch, Simulation
from .forces import NodalForce, ParticleTraction
from .functions import Linear, Unit
from .material import LinearElastic, Newtonian, SimpleMaterial
from .mesh import Mesh1D, Mesh2D
from .mpm import MPM
from .node import Nodes
from .particle import Particles
from .solver import MPMExplicit
from ._lib import MpmError, OutOfMeshError

__all__ = [
    "Batch", "Constraint", "Linear1D", "Quadrilateral4Node", "Simulation", "NodalForce",
    "ParticleTraction", "ParticleVelocityConstraint", "Linear", "Unit", "LinearElastic", "Newtonian", "SimpleMaterial",
    "Mesh1D", "Mesh2D", "MPM", "Nodes", "Particles", "MPMExplicit", "MpmError", "OutOfMeshError",
]
__version__ = "0.1.0"
