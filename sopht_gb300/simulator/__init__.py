"""Flow simulators and immersed-body coupling (sopht.simulator counterparts)."""

from .adjoint import BodyForceObjective2D, time_integrated_body_force
from .batch import BatchedFlowSimulator2D
from .flow import (
    FlowSimulator,
    PassiveTransportFlowSimulator,
    UnboundedNavierStokesFlowSimulator2D,
    UnboundedNavierStokesFlowSimulator3D,
    create_unbounded_flow_simulator_2d,
    create_unbounded_flow_simulator_3d,
)
from .immersed_body import (
    CircularCylinderForcingGrid,
    CosseratRodElementCentricForcingGrid,
    CosseratRodFlowInteraction,
    CosseratRodNodalForcingGrid,
    Cylinder,
    FlowForces,
    ImmersedBodyFlowInteraction,
    ImmersedBodyForcingGrid,
    RigidBodyFlowInteraction,
    TwoDimensionalCylinderForcingGrid,
)

__all__ = [
    "BatchedFlowSimulator2D",
    "BodyForceObjective2D",
    "CircularCylinderForcingGrid",
    "CosseratRodElementCentricForcingGrid",
    "CosseratRodFlowInteraction",
    "CosseratRodNodalForcingGrid",
    "Cylinder",
    "FlowForces",
    "FlowSimulator",
    "ImmersedBodyFlowInteraction",
    "ImmersedBodyForcingGrid",
    "PassiveTransportFlowSimulator",
    "RigidBodyFlowInteraction",
    "TwoDimensionalCylinderForcingGrid",
    "UnboundedNavierStokesFlowSimulator2D",
    "UnboundedNavierStokesFlowSimulator3D",
    "create_unbounded_flow_simulator_2d",
    "create_unbounded_flow_simulator_3d",
    "time_integrated_body_force",
]
