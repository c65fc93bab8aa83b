"""Flow simulators and immersed-body coupling (sopht.simulator counterparts)."""

from .adjoint import BodyForceObjective2D, time_integrated_body_force
from .batch import BatchedFlowSimulator2D
from .rods import CosseratRodBatch
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
    CosseratRodEdgeForcingGrid,
    CosseratRodElementCentricForcingGrid,
    CosseratRodFlowInteraction,
    CosseratRodNodalForcingGrid,
    CosseratRodSurfaceForcingGrid,
    Cylinder,
    FlowForces,
    ImmersedBodyFlowInteraction,
    ImmersedBodyForcingGrid,
    OpenEndCircularCylinderForcingGrid,
    RectangularPlane,
    RectangularPlaneForcingGrid,
    RigidBodyFlowInteraction,
    Sphere,
    SphereForcingGrid,
    ThreeDimensionalRigidBodyForcingGrid,
    TwoDimensionalCylinderForcingGrid,
)

__all__ = [
    "BatchedFlowSimulator2D",
    "BodyForceObjective2D",
    "CircularCylinderForcingGrid",
    "CosseratRodEdgeForcingGrid",
    "CosseratRodBatch",
    "CosseratRodElementCentricForcingGrid",
    "CosseratRodFlowInteraction",
    "CosseratRodNodalForcingGrid",
    "CosseratRodSurfaceForcingGrid",
    "Cylinder",
    "FlowForces",
    "FlowSimulator",
    "ImmersedBodyFlowInteraction",
    "ImmersedBodyForcingGrid",
    "OpenEndCircularCylinderForcingGrid",
    "PassiveTransportFlowSimulator",
    "RectangularPlane",
    "RectangularPlaneForcingGrid",
    "RigidBodyFlowInteraction",
    "Sphere",
    "SphereForcingGrid",
    "ThreeDimensionalRigidBodyForcingGrid",
    "TwoDimensionalCylinderForcingGrid",
    "UnboundedNavierStokesFlowSimulator2D",
    "UnboundedNavierStokesFlowSimulator3D",
    "create_unbounded_flow_simulator_2d",
    "create_unbounded_flow_simulator_3d",
    "time_integrated_body_force",
]
