"""GB300-native (sm_103a) stable-fluids frame step with the reference's API.

The compute path is ``libeqfluid.so`` (CUDA kernels + the C ABI declared in
``include/eqfluid.h``); ``simulation`` mirrors the reference's Rust
``src/simulation`` API on top of it.
"""
from ._lib import EqError, load  # noqa: F401
from .simulation import (  # noqa: F401
    ContainerWall,
    CurrentSimulation,
    Fluid,
    FluidConfigs,
    FluidStep,
    InvalidRectangle,
    ObstaclesType,
    Rectangle,
    SimulationConfigs,
)
