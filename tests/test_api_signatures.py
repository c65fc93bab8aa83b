"""The drop-in API: every public callable of the reference's API modules exists here with the same
parameter names, order and defaults, except the ones outside the flow-step path.

``tests/golden/reference_signatures.json`` is written by ``make_golden.py`` from the reference's
``__all__`` of ``sopht.simulator``, ``sopht.numeric.eulerian_grid_ops``,
``sopht.numeric.immersed_boundary_ops`` and ``sopht.utils`` (classes: their constructors).
"""

from __future__ import annotations

import importlib
import inspect
import json

import pytest
from conftest import GOLDEN

SIGNATURES = json.loads((GOLDEN / "reference_signatures.json").read_text())

# outside the flow-step path (no configuration calls them), each named with its reason
NOT_PROVIDED = {
    # FFTW plumbing and the scipy round-trip check, replaced by the library's own FFT inside the solve
    "sopht.numeric.eulerian_grid_ops.FFTPyFFTW2D", "sopht.numeric.eulerian_grid_ops.FFTPyFFTW3D",
    "sopht.numeric.eulerian_grid_ops.fft_ifft_via_scipy_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.fft_ifft_via_scipy_kernel_3d",
    # bounded Neumann solver, used by no configuration
    "sopht.numeric.eulerian_grid_ops.FastDiagPoissonSolver2D",
    "sopht.numeric.eulerian_grid_ops.FastDiagPoissonSolver3D",
    # Brinkmann penalisation, level sets, in-plane curl, penalised-velocity update, stretching kernels
    "sopht.numeric.eulerian_grid_ops.gen_brinkmann_penalise_pyst_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.gen_brinkmann_penalise_pyst_kernel_3d",
    "sopht.numeric.eulerian_grid_ops.gen_brinkmann_penalise_vs_fixed_val_pyst_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.gen_char_func_from_level_set_via_sine_heaviside_pyst_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.gen_char_func_from_level_set_via_sine_heaviside_pyst_kernel_3d",
    "sopht.numeric.eulerian_grid_ops.gen_inplane_field_curl_pyst_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.gen_update_vorticity_from_penalised_velocity_pyst_kernel_2d",
    "sopht.numeric.eulerian_grid_ops.gen_update_vorticity_from_penalised_velocity_pyst_kernel_3d",
    "sopht.numeric.eulerian_grid_ops.gen_vorticity_stretching_flux_pyst_kernel_3d",
    "sopht.numeric.eulerian_grid_ops.gen_vorticity_stretching_timestep_euler_forward_pyst_kernel_3d",
    "sopht.numeric.eulerian_grid_ops.gen_vorticity_stretching_timestep_ssprk3_pyst_kernel_3d",
    # experimental Brinkmann IB; the grid communicators are restated inside the IB kernels
    "sopht.numeric.immersed_boundary_ops.BrinkmannBoundaryForcing",
    "sopht.numeric.immersed_boundary_ops.EulerianLagrangianGridCommunicator2D",
    "sopht.numeric.immersed_boundary_ops.EulerianLagrangianGridCommunicator3D",
    # plotting and video (matplotlib, ffmpeg), and pystencils configuration
    "sopht.utils.create_figure_and_axes", "sopht.utils.get_lab_cmap", "sopht.utils.save_and_clear_fig",
    "sopht.utils.make_dir_and_transfer_h5_data", "sopht.utils.make_video_from_image_series",
    "sopht.utils.plot_video_of_rod_surface", "sopht.utils.get_pyst_dtype", "sopht.utils.get_pyst_kernel_config",
}


MODULES = ("sopht.numeric.immersed_boundary_ops", "sopht.numeric.eulerian_grid_ops", "sopht.simulator", "sopht.utils")


def _split(qualified):
    module = next(m for m in MODULES if qualified.startswith(m + "."))
    return module, qualified[len(module) + 1:].split(".")


def _listed(qualified):
    module, path = _split(qualified)
    return f"{module}.{path[0]}" in NOT_PROVIDED


def _ours(qualified):
    module, path = _split(qualified)
    obj = importlib.import_module(module.replace("sopht.", "sopht_gb300.", 1))
    for part in path:
        obj = getattr(obj, part, None)
        if obj is None:
            return None
    return obj


PROVIDED = sorted(q for q in SIGNATURES if not _listed(q))


def test_every_reference_callable_is_provided_or_listed():
    missing = [q for q in PROVIDED if _ours(q) is None]
    assert not missing, missing
    assert all(q in SIGNATURES for q in NOT_PROVIDED)


@pytest.mark.parametrize("qualified", PROVIDED)
def test_same_parameters_and_defaults(qualified):
    obj = _ours(qualified)
    sig = inspect.signature(obj.__init__ if inspect.isclass(obj) else obj)
    ours = {p.name: p for p in sig.parameters.values() if p.name != "self"}
    takes_kwargs = any(p.kind == p.VAR_KEYWORD for p in ours.values())
    positional = [p.name for p in sig.parameters.values()
                  if p.name != "self" and p.kind in (p.POSITIONAL_ONLY, p.POSITIONAL_OR_KEYWORD)]
    ref_names = [name for name, _ in SIGNATURES[qualified]]
    for i, (name, default) in enumerate(SIGNATURES[qualified]):
        if name not in ours:
            assert takes_kwargs, f"{qualified}: no parameter {name!r}"
            continue
        if default is not None:
            assert ours[name].default is not inspect.Parameter.empty, f"{qualified}({name}): no default"
            assert repr(ours[name].default) == default, f"{qualified}({name}): {ours[name].default!r} != {default}"
    # the reference's positional order is kept for the parameters both have
    shared = [n for n in ref_names if n in positional]
    assert shared == [n for n in positional if n in shared], qualified


def test_factory_functions_reject_unknown_flow_types_before_any_device_work():
    """flow_simulators_{2,3}d.py: an unknown flow_type is a ValueError."""
    import sopht_gb300.simulator as sps
    with pytest.raises(ValueError, match="Invalid flow type given"):
        sps.create_unbounded_flow_simulator_2d(grid_size=(8, 8), x_range=1.0, kinematic_viscosity=1e-3,
                                               flow_type="passive_scalar")
    with pytest.raises(ValueError, match="Invalid flow type given"):
        sps.create_unbounded_flow_simulator_3d(grid_size=(8, 8, 8), x_range=1.0, kinematic_viscosity=1e-3,
                                               flow_type="stokes")


@pytest.mark.parametrize("cls,kwargs,message", [
    ("PassiveTransportFlowSimulator", dict(grid_dim=3, grid_size=(8, 8, 8), field_type="tensor"),
     "Invalid field type. Supported values include 'scalar' and 'vector'"),
    ("PassiveTransportFlowSimulator", dict(grid_dim=2, grid_size=(8, 8), field_type="vector"),
     "Passive transport of vector 2D fields not supported yet."),
    ("PassiveTransportFlowSimulator", dict(grid_dim=4, grid_size=(8, 8)),
     "Invalid grid dimensions. Supported values include 2 and 3."),
    ("UnboundedNavierStokesFlowSimulator3D", dict(grid_size=(8, 8, 8), poisson_solver_type="fft"),
     "Invalid Poisson solver type given"),
    ("UnboundedNavierStokesFlowSimulator3D",
     dict(grid_size=(8, 8, 8), filter_vorticity=True, filter_setting_dict={"order": 2, "type": "bogus"}),
     "Invalid filter type"),
])
def test_constructor_errors_like_the_reference(cls, kwargs, message):
    """The reference's argument errors (same type and message), raised before any device work."""
    import sopht_gb300.simulator as sps
    kw = dict(kinematic_viscosity=1e-3, x_range=1.0, **kwargs)
    with pytest.raises(ValueError) as err:
        getattr(sps, cls)(**kw)
    assert str(err.value) == message


@pytest.mark.parametrize("kwargs,message", [
    (dict(grid_dim=4), "Invalid grid dimensions, must be either 2 or 3"),
    (dict(grid_dim=2, interp_kernel_width=3), "Interpolation kernel inconsistent with interpolation kernel width!"),
])
def test_virtual_boundary_forcing_errors_like_the_reference(kwargs, message):
    from sopht_gb300.numeric.immersed_boundary_ops import VirtualBoundaryForcing
    import numpy as np
    base = dict(virtual_boundary_stiffness_coeff=1.0, virtual_boundary_damping_coeff=1.0, dx=0.1, num_lag_nodes=3,
                real_t=np.float32, **kwargs)
    with pytest.raises(ValueError) as err:
        VirtualBoundaryForcing(**base)
    assert str(err.value) == message
