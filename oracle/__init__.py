"""CPU oracle for the SophT flow-step hot path (TEST INFRASTRUCTURE ONLY).

This package is a numpy/scipy restatement of the reference implementation's
algorithm for the flow step: the 2D/3D Eulerian stencil operators, the unbounded
domain-doubled FFT Poisson solve, the immersed-boundary interpolation/spreading
with virtual-boundary forcing, and the simulator step drivers.  Each function
cites the reference file and lines it follows.

It exists to check the CUDA path, and only three callers may use it: the tests
under ``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py``.  The product package ``sopht_gb300``
never imports it and has no CPU fallback.

Parity pinning: the oracle is checked against golden fixtures produced by
running the reference package itself (``tests/golden/make_golden.py``) and
against the known-answer cases of the reference's own tests.  ``rod`` (the
discrete Cosserat rod model pyelastica implements, for a future batched rod
integrator) is the exception: pyelastica is not installed, so its parity is
unpinned and it is pinned to analytic solutions and conservation laws instead.

Precision: every routine takes ``real_t`` (``np.float32`` or ``np.float64``) and
follows the reference's numpy type promotion (weak Python scalars, float64
marker positions), so the FP32 mode reproduces the reference FP32 path and the
FP64 mode is the accuracy yardstick.
"""

from .flow import (
    CircularCylinderOracle,
    ImmersedBodyInteractionOracle,
    NavierStokes2DOracle,
    NavierStokes3DOracle,
    RodElementCentricGridOracle,
    RodNodalGridOracle,
    stable_timestep,
)
from .ib import VirtualBoundaryForcingOracle
from .poisson import UnboundedPoisson2D, UnboundedPoisson3D

__all__ = [
    "CircularCylinderOracle",
    "ImmersedBodyInteractionOracle",
    "NavierStokes2DOracle",
    "NavierStokes3DOracle",
    "RodElementCentricGridOracle",
    "RodNodalGridOracle",
    "UnboundedPoisson2D",
    "UnboundedPoisson3D",
    "VirtualBoundaryForcingOracle",
    "stable_timestep",
]
