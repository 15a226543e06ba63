"""gpb — GB300-native batched rigid-body step (the drop-in for gorilla-physics'
per-mechanism `step` / `simulate` over tens of thousands of mechanisms).

All arithmetic runs in the CUDA kernels of libgpb.so (sm_103a); this package
only describes mechanisms and calls the C ABI of include/gpb.h.
"""

from ._abi import (ALGO_ABA, ALGO_CRBA, FIXED, FLOATING, FP64, HUNT_CROSSLEY, LINEAR_SPRING_DAMPER, MIXED, MIXED_REFINED, PRISMATIC,
                   REVOLUTE, RUNGE_KUTTA_2, RUNGE_KUTTA_4, SEMI_IMPLICIT_EULER, VELOCITY_STEPPING, GpbError, lib)
from .batch import Batch, Context, Integrator, Precision, simulate, simulate_steps
from .collision import collide_cuboids
from .serve import Server, SlotClass
from .model import (WORLD_FRAME, ContactPoint, Cuboid, FixedJoint, FloatingJoint, HalfSpace,
                    MechanismState, Model, PrismaticJoint, RevoluteJoint, RigidBody,
                    SpatialInertia, Transform3D)

__all__ = [
    "Batch", "Context", "Integrator", "Precision", "simulate", "simulate_steps", "Model",
    "MechanismState", "Transform3D", "SpatialInertia", "RigidBody", "ContactPoint", "HalfSpace",
    "RevoluteJoint", "PrismaticJoint", "FloatingJoint", "FixedJoint", "WORLD_FRAME", "GpbError",
    "lib", "FIXED", "REVOLUTE", "PRISMATIC", "FLOATING", "SEMI_IMPLICIT_EULER", "RUNGE_KUTTA_2",
    "RUNGE_KUTTA_4", "VELOCITY_STEPPING", "FP64", "MIXED", "MIXED_REFINED", "HUNT_CROSSLEY", "LINEAR_SPRING_DAMPER",
    "Server", "SlotClass", "ALGO_CRBA", "ALGO_ABA", "Cuboid", "collide_cuboids",
]
