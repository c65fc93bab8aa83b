"""ctypes binding of the C ABI in ``include/sopht_gb300.h``.

The library is built in-tree (``sopht_gb300/libsopht_gb300.so``) by
``sopht_gb300.build``.  There is no fallback: if the library cannot be loaded
every operator raises, so a missing build can never silently run elsewhere.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_char_p, c_double, c_int, c_int32, c_int64, c_void_p
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libsopht_gb300.so"

SG_OK = 0
SG_ERR_INVALID_ARG = 1
SG_ERR_SHAPE = 2
SG_ERR_CUDA = 3
SG_ERR_UNSUPPORTED = 4
SG_ERR_OUT_OF_DOMAIN = 5
SG_F32 = 0
SG_F64 = 1


class StepScalars(ctypes.Structure):
    """Mirror of ``sg_step_scalars``."""

    _fields_ = [
        ("dt", c_double),
        ("forcing_prefac", c_double),
        ("advection_prefac", c_double),
        ("diffusion_prefac", c_double),
        ("free_stream", c_double * 3),
    ]


class Batch2DMember(ctypes.Structure):
    """Mirror of ``sg_batch2d_member``."""

    _fields_ = [
        ("plan", c_void_p), ("vorticity", c_void_p), ("velocity", c_void_p), ("forcing", c_void_p),
        ("stream_func", c_void_p), ("cfl", c_double), ("nu", c_double), ("flow_density", c_double),
        ("dt_prefac", c_double), ("free_stream", c_double * 2), ("n_lag", c_int), ("kernel_type", c_int),
        ("dx", c_double), ("shift", c_double), ("position", c_void_p), ("body_velocity", c_void_p),
        ("nearest", c_void_p), ("weights", c_void_p), ("flow_velocity", c_void_p),
        ("velocity_mismatch", c_void_p), ("position_mismatch", c_void_p), ("lag_forcing", c_void_p),
        ("stiffness", c_double), ("damping", c_double), ("status", c_void_p),
    ]


class RodBatch(ctypes.Structure):
    """Mirror of ``sg_rod_batch`` (device array pointers; read on the host)."""

    _fields_ = [("n_rods", c_int), ("n_elems", c_int)] + [(name, c_void_p) for name in (
        "position", "velocity", "directors", "omega", "mass", "rest_lengths", "rest_voronoi_lengths",
        "shear_matrix", "bend_matrix", "mass_second_moment", "inv_mass_second_moment", "rest_sigma", "rest_kappa",
        "external_forces", "external_torques", "clamped", "clamp_position", "clamp_directors")]


class RodCoupling(ctypes.Structure):
    """Mirror of ``sg_rod_coupling`` (read on the host)."""

    _fields_ = [("dtype", c_int), ("nz", c_int), ("ny", c_int), ("nx", c_int), ("dx", c_double), ("shift", c_double),
                ("kernel_type", c_int)] + [(name, c_void_p) for name in (
                    "flow_velocity", "marker_position", "marker_velocity", "nearest", "weights", "flow_velocity_lag",
                    "velocity_mismatch", "position_mismatch", "lag_forcing")] + [
                ("stiffness", c_double), ("damping", c_double), ("flow_dt", c_double), ("flow_time", c_double),
                ("dev_scalars", c_void_p), ("dev_time_end", c_void_p), ("max_rod_dt", c_double),
                ("damping_rate", c_double), ("drive_phase", c_void_p), ("drive_amplitude", c_double),
                ("drive_frequency", c_double), ("drive_axis", c_double * 3), ("status", c_void_p)]


_SIGNATURES = {
    "sg_last_error": (c_char_p, []),
    "sg_version": (c_int, []),
    "sg_poisson_plan_create": (c_int, [c_int, c_int, c_int, c_int, c_double, c_int, c_int, POINTER(c_void_p)]),
    "sg_poisson_plan_destroy": (c_int, [c_void_p]),
    "sg_poisson_plan_bytes": (c_int64, [c_void_p]),
    "sg_poisson_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int64, c_void_p]),
    "sg_poisson2d_solve_noalloc": (c_int, [c_int, c_int, c_double, c_void_p, c_void_p, c_void_p]),
    "sg_flow_plan_create": (c_int, [c_int, c_int, c_int, c_int, c_double, c_int, c_int, c_void_p, c_void_p,
                                    c_void_p, c_int, c_int, POINTER(c_void_p)]),
    "sg_flow_plan_destroy": (c_int, [c_void_p]),
    "sg_flow_plan_bytes": (c_int64, [c_void_p]),
    "sg_flow_set_timing_events": (c_int, [c_void_p, c_int, POINTER(c_void_p)]),
    "sg_flow_read_device_time": (c_int, [c_void_p, POINTER(c_double)]),
    "sg_flow_prime_max": (c_int, [c_void_p, c_void_p, c_void_p]),
    "sg_flow_step": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, POINTER(StepScalars), c_void_p,
                             c_void_p]),
    "sg_max_abs_sum": (c_int, [c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_flow_host_max": (c_int, [c_void_p, c_void_p, POINTER(c_double), c_void_p]),
    "sg_flow_device_dt": (c_int, [c_void_p, c_void_p, c_double, c_double, c_double, c_double, POINTER(c_double),
                                  POINTER(c_void_p), c_void_p]),
    "sg_advection_eno3_step_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_diffusion_step_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_forcing_curl_update_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_outplane_curl_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_penalise_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "sg_curl_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_forcing_curl_update_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double,
                                          c_void_p]),
    "sg_cross_3d": (c_int, [c_int, c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_diffusion_step_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_divergence_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_penalise_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p,
                               c_void_p]),
    "sg_laplacian_filter_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_int, c_int, c_void_p, c_void_p,
                                       c_void_p]),
    "sg_elementwise": (c_int, [c_int, c_int, c_int64, c_void_p, c_void_p, c_void_p, c_double, c_double, c_void_p]),
    "sg_set_boundary_zone": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_double, c_void_p]),
    "sg_diffusion_flux": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_int, c_void_p]),
    "sg_advection_eno3_flux_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_advection_eno3_step_3d": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double,
                                          c_void_p]),
    "sg_advection_eno3_flux_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double,
                                          c_void_p]),
    "sg_passive_transport_step": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                          c_double, c_double, c_void_p]),
    "sg_ib_interaction": (c_int, [c_int, c_int, c_int, c_int, c_int, c_double, c_double, c_int, c_int, c_void_p,
                                  c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                  c_double, c_double, c_int, c_double, c_void_p, c_void_p, c_void_p]),
    "sg_ib_spread": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_int, c_void_p]),
    "sg_ib_mismatch_step": (c_int, [c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_ib_bind": (c_int, [c_int, c_int, c_int, c_int, c_int, c_double, c_double, c_int, c_int, c_void_p, c_void_p,
                           c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_void_p)]),
    "sg_ib_binding_buffers": (c_int, [c_void_p, POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p)]),
    "sg_ib_binding_wait": (c_int, [c_void_p, c_int]),
    "sg_ib_bound_step": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_double, c_double, c_int, c_double,
                                 c_int, c_void_p]),
    "sg_ib_unbind": (c_int, [c_void_p]),
    "sg_rod_element_kinematics": (c_int, [c_int, c_int, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_void_p,
                                          c_void_p, c_void_p]),
    # adjoints
    "sg_adj_partials_count_2d": (c_int64, [c_int, c_int]),
    "sg_sum_partials": (c_int, [c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_outplane_curl_adj_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_penalise_adj_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "sg_diffusion_adj_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                    c_void_p]),
    "sg_advection_eno3_adj_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                         c_void_p, c_void_p]),
    "sg_forcing_curl_adj_2d": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p]),
    "sg_poisson_solve_adj": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_int64, c_void_p]),
    "sg_flow_poisson_plan": (c_void_p, [c_void_p]),
    "sg_flow_set_tape": (c_int, [c_void_p, c_void_p, c_void_p]),
    "sg_ns2d_reverse_sweep": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_ib_interaction_adj": (c_int, [c_int, c_int, c_int, c_int, c_int, c_double, c_int, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_double, c_double, c_double, c_void_p, c_void_p,
                                      c_void_p, c_void_p, c_void_p]),
    "sg_ib_interp_adj": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_void_p]),
    "sg_lag_weighted_sum": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_rod_batch_step": (c_int, [POINTER(RodBatch), c_int, c_double, c_double, c_void_p]),
    "sg_rod_batch_element_markers": (c_int, [POINTER(RodBatch), c_int, c_void_p, c_void_p, c_void_p]),
    "sg_rod_batch_element_loads": (c_int, [POINTER(RodBatch), c_int, c_int, c_void_p, c_void_p]),
    "sg_rod_batch_coupled_substeps": (c_int, [POINTER(RodBatch), POINTER(RodCoupling), c_void_p]),
    "sg_flow_device_time_slot": (c_int, [c_void_p, POINTER(c_void_p)]),
    "sg_event_record": (c_int, [c_void_p, c_void_p]),
    "sg_rotational_update_3d": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_int,
                                        c_void_p, c_void_p]),
    "sg_flow_kernel_status": (c_int, [c_void_p, POINTER(ctypes.c_int32)]),
    "sg_diffusion_3d_staged": (c_int, [c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_int,
                                       c_void_p, c_void_p]),
    "sg_ops_kernel_status": (c_int, [POINTER(ctypes.c_int32)]),
    "sg_forcing_curl_3d_staged": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_int,
                                          c_void_p, c_void_p]),
    "sg_curl_3d_staged": (c_int, [c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_double, c_void_p, c_void_p, c_int,
                                  c_void_p, c_void_p]),
    "sg_ib_spread_sorted_scratch_bytes": (c_int64, [c_int, c_int, c_int, c_int, c_int]),
    "sg_ib_spread_sorted": (c_int, [c_int, c_int, c_int, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_int, c_void_p, c_int64, c_void_p]),
    "sg_batch2d_create": (c_int, [c_int, POINTER(Batch2DMember), POINTER(c_void_p)]),
    "sg_batch2d_set_tuning": (c_int, [c_void_p, c_int, c_int, c_int]),
    "sg_batch2d_step": (c_int, [c_void_p, c_void_p]),
    "sg_batch2d_destroy": (c_int, [c_void_p]),
}

_lib = None


class SophtGB300Error(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, name: str, status: int, message: str) -> None:
        super().__init__(f"{name} failed with status {status}: {message}")
        self.status = status


def load(path: Path | str | None = None) -> ctypes.CDLL:
    """Load the library (once) and attach the argument types of every entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -m sopht_gb300.build` (needs nvcc for sm_103a). "
            "sopht_gb300 has no CPU fallback.")
    lib = ctypes.CDLL(str(p))
    for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
    if path is None:
        _lib = lib
    return lib


def call(name: str, *args) -> None:
    """Call entry point ``name``; raise ValueError/RuntimeError on failure."""
    lib = load()
    status = getattr(lib, name)(*args)
    if status != SG_OK:
        msg = (lib.sg_last_error() or b"").decode(errors="replace")
        if status in (SG_ERR_INVALID_ARG, SG_ERR_SHAPE, SG_ERR_UNSUPPORTED):
            raise ValueError(f"{name}: {msg}")
        raise SophtGB300Error(name, status, msg)


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)
