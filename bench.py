"""Benchmark: coupled flow steps/s of the SophT flow-step hot path on GB300.

Workloads (``--workload``, one GPU each; the default is the headline one):

  carpet256  (default) 3D 256^3, fp32, a 4 x 4 carpet of 16 Cosserat rods (100
             elements, length 0.2, radius 0.005, E = 1e5, density 1) clamped on the
             plane z0 = 6 dx whose bases turn by 0.2 sin(2 pi t + phase) rad about y
             (seeded phases), element-centric cosine-delta forcing (K = -2e4, C = -1e2),
             U = 1 along x, Re = 500 on the rod length.
  rod128     3D unbounded vorticity Navier-Stokes on 128^3, fp32, cubic domain of
             side 1 (Poisson by domain doubling, 256^3 FFT), one clamped Cosserat rod of
             64 elements (length 0.3, radius 0.01, E = 1e5, density 1) at the domain
             centre with an element-centric forcing grid and cosine-delta
             virtual-boundary coupling (K = -2e4, C = -1e2), inflow U = 1, Re = 100 on
             the rod length.
  cylinder2d 2D 256(y) x 512(x), fp32, x-domain 1, cylinder of diameter 0.1 at
             (0.25, 0.25) with 96 markers, K = -5e4, C = -20, U = 1,
             Re = 200 on the diameter, CFL 0.1.
  batch64    64 2D cylinder flows of uneven sizes (128x256 to 512x1024) and
             Reynolds numbers advanced by the batched persistent launches, against
             the same 64 instances run one after another.
  adjoint2d  the cylinder flow's drag integrated over 200 frozen-dt steps and its
             gradient with respect to the marker wall velocities and the viscosity
             (adjoint step time against the forward step, finite differences, the
             oracle's FP64 adjoint).
  pointsource256  passive transport (ENO3 advection + diffusion) of a vector point
             source at 256^3, with the reference example's 128^3 run for accuracy.

One step of a rod workload is the reference examples' loop
(flow_past_rod_case.py:231-250): the stable dt with dt_prefac 0.25, the rods
advanced through it in int(dt / rod_dt) position-Verlet sub-steps with the flow
forces at each half step (one launch for every rod), the interaction and
spreading of the final configuration, then the flow time step.  rod_dt is half
the explicit stability limit of the rods' axial and shear waves, dl sqrt(rho / E).
The cylinder is held in place.

Arms
  default            this repository's GPU path.
      value  : device-resident steps/s: a CUDA graph of K whole coupled steps
               (device dt + rod sub-steps + IB interaction + spread + flow step),
               replayed until about a second has passed; the median replay.
      e2e    : the same steps through the public Python API (host dt each step,
               the Lagrangian forcing read back each step).
  --impl reference   the reference algorithm's CPU implementation (the numpy/
               scipy oracle of this repository, since the reference's own JIT
               dependencies are not installable), all host cores, bounded sample.

Prints one JSON line on rank 0.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import time
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "flow steps/s & Gcell-updates/s vs plain GPU path at stated FP64-oracle L2 error"

# bytes per cell moved by each pass of this fp32 step (read + write), for the per-pass GB/s
PASSES_3D = {"stencils": 96, "poisson_load": 60, "y_fft": 72, "z_conv": 108, "y_ifft": 72, "x_c2r": 36, "curl": 24}
PASSES_2D = {"sweep": 24, "poisson_load": 32, "y_conv": 20, "x_c2r": 12, "curl": 12}
# compulsory bytes per cell-step of the fused design (fp32): 408 in 3D, 88 in 2D -- the step roofline
STEP_BYTES = {3: 408, 2: 88}
ROD_MATERIAL = {"E": 1e5, "density": 1.0, "G": 1e5 / 1.5}  # G = E / (1 + Poisson 0.5), the examples' rule


@dataclass
class Workload:
    name: str
    description: str
    grid: tuple
    nu: float
    u_inf: np.ndarray
    kind: str                      # "rods" or "cylinder"
    bodies: list = field(default_factory=list)
    K: float = 0.0
    C: float = 0.0
    x_range: float = 1.0
    cfl: float = 0.1
    n_markers: int = 96
    actuation: dict = None         # rods: {"amplitude", "frequency", "phases"} of a sinusoidal base rotation
    accuracy_checkpoints: tuple = (1, 10, 100)
    dt_prefac: float = 1.0

    @property
    def rod_dt(self):
        """Half the explicit stability limit of the rods' axial and shear waves: 0.5 dl sqrt(rho / E)."""
        b = self.bodies[0]
        return 0.5 * (b["length"] / b["n_elem"]) * np.sqrt(ROD_MATERIAL["density"] / ROD_MATERIAL["E"])

    @property
    def dim(self):
        return len(self.grid)

    @property
    def passes(self):
        return PASSES_3D if self.dim == 3 else PASSES_2D

    @property
    def cells(self):
        return int(np.prod(self.grid))

    def initial_vorticity(self, real_t):
        rng = np.random.default_rng(42)
        shape = self.grid if self.dim == 2 else (3, *self.grid)
        return (1e-3 * rng.standard_normal(shape)).astype(real_t)


def batch_members_spec(n=64, seed=42):
    """64 uneven 2D cylinder flows: size class, Reynolds number and centre jitter per instance."""
    rng = np.random.default_rng(seed)
    classes = [(128, 256), (256, 512), (384, 768), (512, 1024)]
    out = []
    for _ in range(n):
        ny, nx = classes[int(rng.integers(0, 4))]
        re = float(rng.uniform(50, 400))
        jit = rng.uniform(-0.02, 0.02, 2)
        out.append(dict(grid=(ny, nx), nu=1.0 * 0.1 / re,
                        centre=(0.25 + jit[0], 0.5 * ny / nx + jit[1], 0.0)))
    return out


def make_workload(name: str) -> Workload:
    if name == "rod128":
        length = 0.3
        return Workload(
            name, "3D unbounded vorticity NS 128^3 fp32 (256^3 doubled FFT), one clamped Cosserat rod (64 "
                  "elements, E 1e5, density 1) integrated on the GPU, element-centric cosine-delta forcing, U=1 "
                  "inflow, Re=100 on rod length, CFL 0.1 with dt_prefac 0.25",
            (128, 128, 128), 1.0 * length / 100.0, np.array([1.0, 0.0, 0.0]), "rods",
            bodies=[dict(base=(0.5, 0.5, 0.5 - length / 2), length=length, radius=0.01, n_elem=64)],
            K=-2e4, C=-1e2, accuracy_checkpoints=(1, 10, 100, 500), dt_prefac=0.25)
    if name == "cylinder2d":
        return Workload(
            name, "2D unbounded vorticity NS 256x512 fp32, cylinder D=0.1 at (0.25, 0.25), 96 markers, "
                  "U=1, Re=200 on the diameter, CFL 0.1",
            (256, 512), 1.0 * 0.1 / 200.0, np.array([1.0, 0.0]), "cylinder",
            bodies=[dict(centre=(0.25, 0.25, 0.0), radius=0.05)], K=-5e4, C=-20.0, n_markers=96,
            accuracy_checkpoints=(1, 10, 100, 1000))
    if name == "carpet256":
        n = 256
        dx = 1.0 / n
        length = 0.2
        bodies = []
        for i in range(4):
            for j in range(4):
                bodies.append(dict(base=(0.3 + 0.13 * i, 0.3 + 0.13 * j, 6 * dx), length=length,
                                   radius=0.005, n_elem=100))
        phases = np.random.default_rng(42).uniform(0.0, 2 * np.pi, len(bodies))
        return Workload(
            name, "3D unbounded vorticity NS 256^3 fp32 (512^3 doubled FFT), 4x4 carpet of 16 Cosserat rods (100 "
                  "elements each, E 1e5, density 1) integrated on the GPU, clamped at z0 = 6 dx with bases turning "
                  "0.2 sin(2 pi t + phase) rad about y (seeded phases), U=1 along x, Re=500 on rod length, CFL 0.1 "
                  "with dt_prefac 0.25",
            (n, n, n), 1.0 * length / 500.0, np.array([1.0, 0.0, 0.0]), "rods", bodies=bodies, K=-2e4, C=-1e2,
            actuation={"amplitude": 0.2, "frequency": 1.0, "phases": phases},
            accuracy_checkpoints=tuple(range(20, 201, 20)), dt_prefac=0.25)
    raise ValueError(f"unknown workload {name}")


# ------------------------------------------------------------------ clocks


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 20 ms around a timed region.

    ``start`` returns once the first sample has been written, so the region that follows is
    sampled from its beginning; ``stop`` keeps the samples whose timestamps fall between the
    two calls (all of them if none do or the timestamps cannot be read)."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"sg_clocks_{os.getpid()}.csv"
        self.t0 = self.t1 = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        deadline = time.time() + 5.0
        while time.time() < deadline and self.proc.poll() is None:
            if self.path.exists() and self.path.stat().st_size > 0:
                break
            time.sleep(0.01)
        self.t0 = time.time()

    @staticmethod
    def parse(lines, t0=None, t1=None):
        """Median SM clock, max clock and throttle reasons of the sample lines (CSV of FIELDS)."""
        import datetime
        rows = []
        for line in lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 10:
                continue
            try:
                sm, smax = float(parts[2]), float(parts[3])
            except ValueError:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                ts = None
            rows.append((ts, sm, smax, parts[6:10]))
        inside = [r for r in rows if t0 is not None and r[0] is not None and t0 <= r[0] <= t1]
        use = inside if inside else rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in use for n, flag in zip(names, r[3], strict=False) if flag.lower() == "active"})
        return {"sm_mhz": float(np.median([r[1] for r in use])) if use else None,
                "sm_max_mhz": max(r[2] for r in use) if use else None,
                "samples": len(use), "samples_in_timed_region": len(inside), "reasons": reasons}

    def stop(self):
        self.t1 = time.time()
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        out = self.parse(self.path.read_text().splitlines(), self.t0, self.t1)
        self.path.unlink(missing_ok=True)
        return out


# ---------------------------------------------------------------- GPU arm


def make_gpu_case(wl: Workload, real_t, device):
    import torch

    import sopht_gb300.simulator as sps

    Sim = sps.UnboundedNavierStokesFlowSimulator2D if wl.dim == 2 else sps.UnboundedNavierStokesFlowSimulator3D
    sim = Sim(grid_size=wl.grid, x_range=wl.x_range, kinematic_viscosity=wl.nu, cfl=wl.cfl, real_t=real_t,
              with_forcing=True, with_free_stream_flow=True, device=device)
    sim.vorticity_field.copy_(torch.from_numpy(wl.initial_vorticity(real_t)).to(device))
    if wl.kind == "cylinder":
        inters = []
        for b in wl.bodies:
            cyl = sps.Cylinder(b["centre"], base_radius=b["radius"])
            inters.append(sps.RigidBodyFlowInteraction(
                rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field,
                eul_grid_velocity_field=sim.velocity_field, virtual_boundary_stiffness_coeff=wl.K,
                virtual_boundary_damping_coeff=wl.C, dx=sim.dx, grid_dim=2, real_t=real_t,
                forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=wl.n_markers))
        return sim, inters
    m = ROD_MATERIAL
    rods = [sps.StraightRod(b["n_elem"], b["base"], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0], b["length"], b["radius"],
                            m["density"], m["E"], shear_modulus=m["G"]) for b in wl.bodies]
    batch = sps.CosseratRodBatch(rods, clamped=[True] * len(rods), device=device)
    inter = sps.CosseratRodBatchFlowInteraction(batch, sim.eul_grid_forcing_field, sim.velocity_field, wl.K, wl.C,
                                                dx=sim.dx, real_t=real_t)
    if wl.actuation:
        a = wl.actuation
        inter.set_base_drive(a["amplitude"], a["frequency"], a["phases"], axis=(0.0, 1.0, 0.0))
    return sim, [inter]


def public_api_step(wl, sim, inters):
    """One coupled step through the drop-in API (the reference example loops' order)."""
    dt = sim.compute_stable_timestep(dt_prefac=wl.dt_prefac)
    for inter in inters:
        if wl.kind == "rods":
            inter.advance_rods(dt, wl.rod_dt, flow_time=sim.time)
        else:
            inter.time_step(dt=dt)
        inter()
    sim.time_step(dt=dt, free_stream_velocity=wl.u_inf)
    if wl.kind == "rods":
        return [inter.lag_grid_forcing_field.cpu() for inter in inters]
    return [inter.lag_grid_forcing_host() for inter in inters]


def device_step(wl, sim, inters, events=None, rod_event=None, stream=None):
    """The same step with dt on the device (capturable)."""
    from sopht_gb300 import _lib
    dsc = sim.device_stable_timestep(dt_prefac=wl.dt_prefac, free_stream_velocity=wl.u_inf, recompute_max=False)
    if rod_event is not None:
        _lib.call("sg_event_record", rod_event.cuda_event, stream.cuda_stream)
    for inter in inters:
        if wl.kind == "rods":
            inter.device_call(dsc, sim.device_time_slot(), wl.rod_dt)
        else:
            inter.device_call(dsc)
    if events is not None:
        arr = (ctypes.c_void_p * len(events))(*[e.cuda_event for e in events])
        _lib.call("sg_flow_set_timing_events", sim._plan, len(events), arr)
    sim.time_step_device(dsc)


def run_gpu(args, wl: Workload, rank, world):
    import torch

    from sopht_gb300.build import build

    build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    rt = np.float32
    sim, inters = make_gpu_case(wl, rt, device)
    if wl.kind == "cylinder":
        for inter in inters:
            inter.upload_kinematics()
    sim.prime_velocity_max()
    stream = torch.cuda.Stream(device)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            device_step(wl, sim, inters)
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    pass_names = list(wl.passes)
    n_ev = len(pass_names) + 1
    seg = min(steps, 25)
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ev)] for _ in range(seg)]
    rod_events = [torch.cuda.Event(enable_timing=True) for _ in range(seg)]
    with torch.cuda.stream(stream):
        for ev_list in events + [rod_events]:  # torch creates the CUDA events lazily, on first record
            for e in ev_list:
                e.record(stream)
    torch.cuda.synchronize()
    # the timed graph holds exactly K = --steps coupled steps and no timing nodes; a second,
    # instrumented graph of the same steps gives the per-pass breakdown
    graph = torch.cuda.CUDAGraph()
    graph_inst = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(graph, stream=stream):
            for _ in range(steps):
                device_step(wl, sim, inters)
        with torch.cuda.graph(graph_inst, stream=stream):
            for k in range(seg):
                device_step(wl, sim, inters, events[k], rod_events[k], stream)
    torch.cuda.synchronize()
    t_probe = time.perf_counter()
    with torch.cuda.stream(stream):
        graph.replay()  # one untimed replay after capture, also sizing the number of timed replays
    torch.cuda.synchronize()
    probe_s = time.perf_counter() - t_probe
    replays = int(min(200, max(7, np.ceil(1.5 / max(probe_s, 1e-4)))))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(replays)]
    stops = [torch.cuda.Event(enable_timing=True) for _ in range(replays)]
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        for r in range(replays):
            starts[r].record(stream)
            graph.replay()
            stops[r].record(stream)
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t_wall) * 1e3
    clock_info = clocks.stop()
    replay_ms = np.array([a.elapsed_time(b) for a, b in zip(starts, stops, strict=True)])
    if replay_ms.sum() < 0.5 * wall_ms:
        raise RuntimeError(f"event time {replay_ms.sum():.3f} ms disagrees with wall time {wall_ms:.3f} ms")
    elapsed_ms = float(np.median(replay_ms))
    if world > 1:
        elapsed_ms = max_over_ranks(elapsed_ms, device)
        torch.distributed.barrier()
    with torch.cuda.stream(stream):
        graph_inst.replay()
    torch.cuda.synchronize()
    cells = wl.cells
    kernels = {}
    if wl.kind == "rods":
        vals = [rod_events[k].elapsed_time(events[k][0]) for k in range(seg)]
        kernels["rods_and_ib"] = {"ms": round(float(np.mean(vals)), 5), "launches_timed": len(vals),
                                  "what": "rod sub-steps (one launch), element markers, interaction, spreading"}
    for i, name in enumerate(pass_names):
        vals = [events[k][i].elapsed_time(events[k][i + 1]) for k in range(seg)]
        ms = float(np.mean(vals))
        kernels[name] = {"ms": round(ms, 5), "GB_s": round(wl.passes[name] * cells / (ms * 1e-3) / 1e9, 1),
                         "launches_timed": len(vals)}
    graph_inst.reset()
    del graph_inst
    value = world * steps / (elapsed_ms * 1e-3)
    graph.reset()
    del graph
    n_sub = None
    if wl.kind == "rods":
        dt_now = float(sim.compute_stable_timestep(dt_prefac=wl.dt_prefac))
        n_sub = int(dt_now / min(dt_now, wl.rod_dt))
        inters[0].check_markers_in_domain()
    del sim, inters

    # end to end through the public API: host dt, the rod loop, interaction, flow step, forcing read back
    sim_e, inters_e = make_gpu_case(wl, rt, device)
    for _ in range(args.warmup):
        public_api_step(wl, sim_e, inters_e)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    for _ in range(steps):
        public_api_step(wl, sim_e, inters_e)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        e2e_s = max_over_ranks(e2e_s, device)
    n_lag = sum(inter.num_lag_nodes for inter in inters_e)
    if wl.kind == "rods":
        h2d = 56  # the step's host scalars (dt and prefactors)
        d2h = 8 + wl.dim * n_lag * 4  # the velocity max for the host dt, the Lagrangian forcing
    else:
        h2d = 2 * wl.dim * n_lag * 8 + 56  # marker kinematics, host scalars
        d2h = 8 + wl.dim * n_lag * 4
    del sim_e, inters_e

    accuracy = None
    if rank == 0 and not args.skip_accuracy:
        accuracy = accuracy_checkpoints(wl, device, [c for c in wl.accuracy_checkpoints if c <= args.accuracy_steps],
                                        cpu_oracle=(wl.dim == 2 and not args.skip_cpu))
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = run_cpu_sample(wl, args.cpu_seconds)
    others = None
    if rank == 0 and world == 1 and not args.no_others:
        others = run_other_configs(args, exclude=wl.name)
    if rank != 0:
        return
    top = max(pass_names, key=lambda k: kernels[k]["ms"])
    hbm = load_peaks().get("hbm_gbs")
    peak = hbm or 6800.0
    algo = wl.passes[top] * cells
    achieved = algo / (kernels[top]["ms"] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 3),
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else "fallback 6800 GB/s",
                "traffic": traffic_from_profiles(wl.name, top), "algorithmic_bytes_per_launch": algo}
    step_ms = elapsed_ms / steps
    step_bytes = STEP_BYTES[wl.dim] * cells
    # this library's kernels per step: the device dt; for rods the coupled sub-step kernel, the element
    # markers, the interaction and the spreading (the sorted form from SORTED_SPREAD_MIN_MARKERS markers
    # on: its pair and group kernels, plus the radix sort's own); per cylinder an interaction and a spread;
    # then the flow step (3D: forcing curl, rotational update, diffusion, load, y FFT, z convolution,
    # y inverse, x C2R, curl; 2D: sweep, load, column convolution, x C2R, curl)
    if wl.kind == "rods":
        from sopht_gb300.numeric import VirtualBoundaryForcing
        n_markers = len(wl.bodies) * wl.bodies[0]["n_elem"] if wl.bodies else 0
        body_launches = 3 + (2 if n_markers >= VirtualBoundaryForcing.SORTED_SPREAD_MIN_MARKERS else 1)
    else:
        body_launches = 2 * len(wl.bodies)
    launches_per_step = 1 + body_launches + (9 if wl.dim == 3 else 5)
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "flow steps/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "gcell_updates_per_s": round(world * cells * steps / (elapsed_ms * 1e-3) / 1e9, 3),
        "config": {"workload": wl.description, "name": wl.name, "grid": list(wl.grid),
                   "dt_rule": f"compute_stable_timestep, CFL 0.1, dt_prefac {wl.dt_prefac}",
                   "bodies": len(wl.bodies),
                   "body_kinematics": (f"Cosserat rods integrated on the GPU inside the timed step: {n_sub} rod "
                                       f"sub-steps of at most {wl.rod_dt:.3e} per flow step, flow forces at each "
                                       "half step" + ("; clamped bases driven by a sinusoidal rotation"
                                                      if wl.actuation else "; clamped base")
                                       if wl.kind == "rods" else "cylinder held in place"),
                   "parallelism": "replicas only" if world > 1 else "single GPU",
                   "l2": "no flush: the step working set exceeds the 126 MB L2" if cells * 4 * 20 > 126e6 else
                         "working set fits in L2 (launch-latency-bound size)",
                   "timing": f"a graph of the {steps} steps replayed {replays} times; the median replay"},
        "roofline": roofline,
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "bytes_per_cell_step": STEP_BYTES[wl.dim],
                          "achieved_GB_s": round(step_bytes / (step_ms * 1e-3) / 1e9, 1),
                          "frac": round(step_bytes / (step_ms * 1e-3) / 1e9 / peak, 3)},
        "replay_ms": {"min": round(float(replay_ms.min()), 4), "median": round(float(np.median(replay_ms)), 4),
                      "max": round(float(replay_ms.max()), 4), "replays": replays},
        "kernels": kernels,
        "e2e": {"value": round(world * steps / e2e_s, 2), "unit": "flow steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": ("public API per step: host dt (sync), the rod loop and interaction, the flow step, the "
                         "Lagrangian forcing read back" if wl.kind == "rods" else
                         "public API per step: host dt (sync), marker kinematics up from pinned memory, the "
                         "interaction, the flow step, the Lagrangian forcing read back")},
        "gpu_launches": launches_per_step * steps,
        "clocks": clock_info,
        "accuracy": accuracy,
        "cpu_baseline": cpu,
        "other_configs": others,
    }
    print(json.dumps(out), flush=True)


def run_other_configs(args, exclude):
    """The other configurations' own bench lines (device-timed numbers), run as separate processes
    after the headline measurement, when the run time allows."""
    out = {}
    for name in ("rod128", "cylinder2d", "batch64", "adjoint2d"):
        if name == exclude:
            continue
        cmd = [sys.executable, str(Path(__file__).resolve()), "--workload", name, "--steps", "20", "--warmup", "3",
               "--skip-cpu", "--skip-accuracy", "--no-others", "--adjoint-steps", "200", "--adjoint-cpu-steps", "0"]
        try:
            res = subprocess.run(cmd, capture_output=True, text=True, timeout=240)
            line = [ln for ln in res.stdout.splitlines() if ln.startswith("{")][-1]
            d = json.loads(line)
        except Exception as exc:  # noqa: BLE001 - report, do not fail the headline line
            out[name] = {"error": f"{type(exc).__name__}: {exc}"[:200]}
            continue
        keep = {k: d.get(k) for k in ("metric", "value", "unit", "ms_per_step", "gcell_updates_per_s",
                                      "speedup_vs_sequential", "sequential_plain_gpu", "adjoint_over_forward",
                                      "step_roofline", "e2e")}
        keep["config"] = (d.get("config") or {}).get("workload")
        out[name] = {k: v for k, v in keep.items() if v is not None}
    return out


def _batch_instances(spec, device):
    import torch

    import sopht_gb300.simulator as sps
    sims, inters = [], []
    for k, m in enumerate(spec):
        sim = sps.UnboundedNavierStokesFlowSimulator2D(
            grid_size=m["grid"], x_range=1.0, kinematic_viscosity=m["nu"], cfl=0.1, real_t=np.float32,
            with_forcing=True, with_free_stream_flow=True, device=device)
        rng = np.random.default_rng(1000 + k)
        sim.vorticity_field.copy_(torch.from_numpy((1e-3 * rng.standard_normal(m["grid"])).astype(np.float32))
                                  .to(device))
        cyl = sps.Cylinder(m["centre"], base_radius=0.05)
        inters.append(sps.RigidBodyFlowInteraction(
            rigid_body=cyl, eul_grid_forcing_field=sim.eul_grid_forcing_field,
            eul_grid_velocity_field=sim.velocity_field, virtual_boundary_stiffness_coeff=-5e4,
            virtual_boundary_damping_coeff=-20.0, dx=sim.dx, grid_dim=2, real_t=np.float32,
            forcing_grid_cls=sps.CircularCylinderForcingGrid, num_forcing_points=96))
        sims.append(sim)
    return sims, inters


def run_batch(args, rank, world):
    """64 uneven 2D instances: batched persistent launches vs 64 sequential plain-GPU runs."""
    import torch

    from sopht_gb300.build import build
    from sopht_gb300.simulator import BatchedFlowSimulator2D

    build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    spec = batch_members_spec()
    fs = np.array([1.0, 0.0])
    sims, inters = _batch_instances(spec, device)
    batch = BatchedFlowSimulator2D(sims, inters, free_stream_velocities=[fs] * len(sims))
    batch.prime()
    best = batch.autotune(steps=3)
    stream = torch.cuda.Stream(device)
    seg = min(args.steps, 25)
    n_seg = max(1, args.steps // seg)
    steps = seg * n_seg
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        stream.wait_stream(torch.cuda.current_stream())
        for _ in range(args.warmup):
            batch.step()
        with torch.cuda.graph(graph, stream=stream):
            for _ in range(seg):
                batch.step()
    with torch.cuda.stream(stream):
        graph.replay()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(n_seg):
            graph.replay()
        stop.record(stream)
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t_wall) * 1e3
    clock_info = clocks.stop()
    batch_ms = start.elapsed_time(stop)
    if batch_ms < 0.5 * wall_ms:
        raise RuntimeError(f"event time {batch_ms:.3f} ms disagrees with wall time {wall_ms:.3f} ms")
    n = len(sims)
    cells = sum(int(np.prod(m["grid"])) for m in spec)
    batched_rate = n * steps / (batch_ms * 1e-3)
    graph.reset()
    del graph, batch

    # 64 sequential plain-GPU runs: each instance alone, its device-dt coupled step in its own graph
    seq_steps = max(5, min(steps, 25))
    seq_ms = 0.0
    sims2, inters2 = _batch_instances(spec, device)
    for sim, inter in zip(sims2, inters2, strict=True):
        inter.upload_kinematics()
        sim.prime_velocity_max()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            stream.wait_stream(torch.cuda.current_stream())
            for _ in range(2):
                dsc = sim.device_stable_timestep(free_stream_velocity=fs, recompute_max=False)
                inter.device_call(dsc)
                sim.time_step_device(dsc)
            with torch.cuda.graph(g, stream=stream):
                for _ in range(seq_steps):
                    dsc = sim.device_stable_timestep(free_stream_velocity=fs, recompute_max=False)
                    inter.device_call(dsc)
                    sim.time_step_device(dsc)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            g.replay()
            stop.record(stream)
        torch.cuda.synchronize()
        seq_ms += start.elapsed_time(stop)
        g.reset()
    sequential_rate = n * seq_steps / (seq_ms * 1e-3)
    # the plain drop-in loop (host dt, per-call launches) for the same 64 instances
    host_steps = 3
    t0 = time.perf_counter()
    for sim, inter in zip(sims2, inters2, strict=True):
        for _ in range(host_steps):
            dt = sim.compute_stable_timestep()
            inter.time_step(dt=dt)
            inter()
            sim.time_step(dt=dt, free_stream_velocity=fs)
    torch.cuda.synchronize()
    host_rate = n * host_steps / (time.perf_counter() - t0)
    if rank != 0:
        return
    out = {
        "metric": "instance-steps/s (64 uneven 2D instances, batched vs 64 sequential plain-GPU runs)",
        "value": round(world * batched_rate, 1), "unit": "instance-steps/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(batch_ms / steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "gcell_updates_per_s": round(world * cells * steps / (batch_ms * 1e-3) / 1e9, 3),
        "config": {"workload": "batch of 64 2D cylinder flows, grids drawn from {128x256, 256x512, 384x768, "
                               "512x1024}, Re ~ U[50, 400], centre jitter U[-0.02, 0.02]^2, seed 42",
                   "instances": n, "total_cells": cells, "autotuned": {"sweep_tile_y": best[0], "fft_threads": best[2],
                                                                        "blocks_per_sm": best[1]}},
        "sequential_plain_gpu": {"value": round(sequential_rate, 1), "unit": "instance-steps/s",
                                 "note": f"each instance alone, device-dt coupled step in a CUDA graph of "
                                         f"{seq_steps} steps, instances one after another"},
        "speedup_vs_sequential": round(batched_rate / sequential_rate, 2),
        "plain_dropin_host_loop": {"value": round(host_rate, 1), "unit": "instance-steps/s",
                                   "note": "public API per step (host dt), instances one after another"},
        "clocks": clock_info,
    }
    print(json.dumps(out), flush=True)


def _adjoint_case(wl, real_t, device, dts, checkpoint_every, use_graphs):
    """The cylinder2d flow with a prescribed wall velocity, as a differentiable objective."""
    from sopht_gb300.simulator import BodyForceObjective2D
    sim, inters = make_gpu_case(wl, real_t, device)
    obj = BodyForceObjective2D(sim, inters[0], dts, free_stream_velocity=wl.u_inf[:2], direction=(1.0, 0.0),
                               checkpoint_every=checkpoint_every, use_graphs=use_graphs)
    return sim, inters[0], obj


def wall_velocity(wl, inter, seed=42):
    """Tangential marker velocity with amplitude U[0, 0.2] per marker (seeded)."""
    pos = inter.forcing_grid.position_field
    c = np.asarray(wl.bodies[0]["centre"][:2]).reshape(2, 1)
    rel = pos - c
    tangent = np.stack([-rel[1], rel[0]]) / np.linalg.norm(rel, axis=0)
    amp = np.random.default_rng(seed).uniform(0.0, 0.2, pos.shape[1])
    return tangent * amp


def frozen_dt_sequence(wl, device, V, n_steps):
    """dt of each step of the forward run with the wall velocity (compute_stable_timestep, CFL 0.1)."""
    import torch
    sim, inters = make_gpu_case(wl, np.float32, device)
    inter = inters[0]
    inter.upload_kinematics()
    Vd = torch.as_tensor(V, dtype=torch.float64, device=device)
    dts = []
    for _ in range(n_steps):
        dt = float(sim.compute_stable_timestep())
        inter._interaction(sim.velocity_field, inter._pos_stage.dev, Vd, xi_step=True, xi_dt=dt)
        inter._spread(sim.eul_grid_forcing_field, reset=True)
        sim.time_step(dt=dt, free_stream_velocity=wl.u_inf)
        dts.append(dt)
    return dts


def run_adjoint(args, rank, world):
    """Drag gradient through 200 steps of the 2D cylinder flow (wall velocity + viscosity)."""
    import torch

    from sopht_gb300.build import build
    from sopht_gb300.simulator import time_integrated_body_force

    build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    wl = make_workload("cylinder2d")
    n_steps, ck = args.adjoint_steps, 20
    _, inter0, _ = _adjoint_case(wl, np.float32, device, [1e-4], ck, False)
    V = wall_velocity(wl, inter0)
    dts = frozen_dt_sequence(wl, device, V, n_steps)
    Vt = torch.as_tensor(V, dtype=torch.float64, device=device)
    nu = wl.nu
    # fp32 objective, both passes captured in CUDA graphs
    sim, inter, obj = _adjoint_case(wl, np.float32, device, dts, ck, True)
    for _ in range(max(1, args.warmup)):
        obj.value_and_grad(Vt, nu)
    torch.cuda.synchronize()
    reps = max(1, args.steps // n_steps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    clocks = ClockSampler(local)
    clocks.start()
    fwd_ms = bwd_ms = 0.0
    for _ in range(reps):
        ev[0].record()
        obj.forward(Vt, nu)
        ev[1].record()
        obj._run("backward", obj._backward_pass)
        ev[2].record()
        torch.cuda.synchronize()
        fwd_ms += ev[0].elapsed_time(ev[1])
        bwd_ms += ev[1].elapsed_time(ev[2])
    clock_info = clocks.stop()
    fwd_step = fwd_ms / (reps * n_steps)
    bwd_step = bwd_ms / (reps * n_steps)
    # the plain drop-in forward step (device dt, graph) of the same flow, for reference
    psim, pinters = make_gpu_case(wl, np.float32, device)
    for pi in pinters:
        pi.upload_kinematics()
    psim.prime_velocity_max()
    stream = torch.cuda.Stream(device)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        stream.wait_stream(torch.cuda.current_stream())
        for _ in range(3):
            device_step(wl, psim, pinters)
        with torch.cuda.graph(g, stream=stream):
            for _ in range(25):
                device_step(wl, psim, pinters)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        g.replay()
        ev[0].record(stream)
        for _ in range(8):
            g.replay()
        ev[1].record(stream)
    torch.cuda.synchronize()
    plain_step = ev[0].elapsed_time(ev[1]) / (8 * 25)
    # end to end through the autograd API: V from pinned host memory, gradient read back
    Vh = torch.as_tensor(V, dtype=torch.float64).pin_memory()
    gh = torch.empty_like(Vh).pin_memory()

    def autograd_gradient():
        Vd = Vh.to(device, non_blocking=True).requires_grad_(True)
        nut = torch.tensor(nu, dtype=torch.float64, device=device, requires_grad=True)
        loss = time_integrated_body_force(obj, Vd, nut)
        loss.backward()
        gh.copy_(Vd.grad)
        return float(nut.grad.item())

    # the first backward() of a process starts autograd's per-device worker thread: timed apart
    t0 = time.perf_counter()
    autograd_gradient()
    first_call_s = time.perf_counter() - t0
    for _ in range(max(0, args.warmup - 1)):
        autograd_gradient()
    e2e_reps = 5
    t0 = time.perf_counter()
    for _ in range(e2e_reps):
        autograd_gradient()
    e2e_s = (time.perf_counter() - t0) / e2e_reps
    # gradients: fp32 and fp64 adjoints, FP64 central differences, FP64 CPU oracle
    L32, g32, n32 = obj.value_and_grad(Vt, nu)
    _, _, obj64 = _adjoint_case(wl, np.float64, device, dts, ck, True)
    L64, g64, n64 = obj64.value_and_grad(Vt, nu)
    g32n, g64n = g32.cpu().numpy(), g64.cpu().numpy()
    rel = lambda a, b: float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))  # noqa
    rng = np.random.default_rng(7)
    comps = [tuple(int(c) for c in rng.integers(0, (2, V.shape[1]))) for _ in range(6)]
    # central differences in FP64 over a range of steps: large steps cross ENO3 upwind-branch switches
    # (the flux is discontinuous where u_j = -u_{j+1}), small ones measure the derivative itself
    fd = {"components": [list(c) for c in comps], "adjoint_fp64": [float(g64n[d, k]) for d, k in comps],
          "adjoint_fp32": [float(g32n[d, k]) for d, k in comps], "nu_adjoint_fp64": n64, "nu_adjoint_fp32": n32,
          "steps": {}}
    for h in (1e-3, 1e-4, 1e-5, 1e-6):
        rows = []
        for (d, k) in comps:
            E = torch.zeros_like(Vt)
            E[d, k] = 1.0
            rows.append((obj64.forward(Vt + h * E, nu).item() - obj64.forward(Vt - h * E, nu).item()) / (2 * h))
        fnu = (obj64.forward(Vt, nu + h * nu).item() - obj64.forward(Vt, nu - h * nu).item()) / (2 * h * nu)
        fdv = np.array(rows)
        fd["steps"][f"{h:g}"] = {
            "fd": [float(x) for x in fdv],
            "rel_err_fp64_adjoint": rel([g64n[d, k] for d, k in comps], fdv),
            "rel_err_fp32_adjoint": rel([g32n[d, k] for d, k in comps], fdv),
            "nu_fd": float(fnu), "nu_rel_err_fp64": abs(n64 - fnu) / abs(fnu),
            "nu_rel_err_fp32": abs(n32 - fnu) / abs(fnu)}
    fd["note"] = "h is absolute for V and relative for nu"
    cpu_ref = None
    if not args.skip_cpu:
        from oracle.adjoint import DragProblem2D
        from oracle.flow import CircularCylinderOracle, NavierStokes2DOracle
        w0 = wl.initial_vorticity(np.float64)
        b = wl.bodies[0]

        def make_flow():
            f = NavierStokes2DOracle(wl.grid, wl.x_range, nu, cfl=wl.cfl, real_t=np.float64, with_forcing=True,
                                     with_free_stream_flow=True)
            f.vorticity_field[...] = w0
            return f

        cyl = CircularCylinderOracle(b["centre"], b["radius"], wl.n_markers)
        hsp = cyl.get_maximum_lagrangian_grid_spacing()
        n_cpu = min(n_steps, args.adjoint_cpu_steps)
        prob = DragProblem2D(make_flow, cyl.position_field, wl.K * hsp, wl.C * hsp, dts[:n_cpu], wl.u_inf[:2])
        t0 = time.perf_counter()
        Lc, gc, nc = prob.gradient(V, nu)
        cpu_s = time.perf_counter() - t0
        if n_cpu == n_steps:
            gpu64, gpu32, Lg, ng64, ng32 = g64n, g32n, L64, n64, n32
        else:
            _, _, o64s = _adjoint_case(wl, np.float64, device, dts[:n_cpu], ck, False)
            _, _, o32s = _adjoint_case(wl, np.float32, device, dts[:n_cpu], ck, False)
            Lg, g_a, ng64 = o64s.value_and_grad(Vt, nu)
            _, g_b, ng32 = o32s.value_and_grad(Vt, nu)
            gpu64, gpu32 = g_a.cpu().numpy(), g_b.cpu().numpy()
        cpu_ref = {"steps": n_cpu, "seconds": round(cpu_s, 2),
                   "loss_rel_err_fp64_gpu": abs(Lg - Lc) / abs(Lc),
                   "grad_rel_l2_fp64_gpu": rel(gpu64, gc), "grad_rel_l2_fp32_gpu": rel(gpu32, gc),
                   "nu_rel_err_fp64_gpu": abs(ng64 - nc) / abs(nc), "nu_rel_err_fp32_gpu": abs(ng32 - nc) / abs(nc),
                   "kind": "the oracle's FP64 hand-written adjoint (numpy), itself pinned to oracle FD in tests"}
    if rank != 0:
        return
    # forward step: interaction, spread (zero + spread), loss sum, flow step (sweep, load, column
    # convolution, C2R, curl); reverse step adds curl^T, the 3-pass solve, the reverse sweep, the
    # partial sum, the IB transpose and interpolation^T after the 8-kernel recompute
    launches_fwd = 9 * n_steps
    launches_bwd = (8 + 8) * n_steps
    out = {
        "metric": "adjoint steps/s (drag gradient through the 2D cylinder step; adjoint step / forward step)",
        "value": round(1e3 / bwd_step, 1), "unit": "adjoint steps/s", "n_gpus": world,
        "steps": reps * n_steps, "warmup": args.warmup, "ms_per_step": round(bwd_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "2D 256x512 fp32 cylinder flow (D=0.1 at (0.25,0.25), 96 markers, K=-5e4, C=-20, "
                               "U=1, Re=200 on D), tangential wall velocity U[0,0.2] per marker (seed 42); "
                               "loss = drag integrated over the steps with the dt sequence frozen",
                   "steps_per_gradient": n_steps, "checkpoint_every": ck, "params": int(V.size) + 1,
                   "l2": "no flush: every step reads and writes the whole working set"},
        "forward_ms_per_step": round(fwd_step, 5),
        "adjoint_ms_per_step": round(bwd_step, 5),
        "adjoint_over_forward": round(bwd_step / fwd_step, 3),
        "plain_dropin_forward_ms_per_step": round(plain_step, 5),
        "adjoint_over_plain_forward": round(bwd_step / plain_step, 3),
        "e2e": {"value": round(n_steps / e2e_s, 1), "unit": "forward+adjoint steps/s",
                "h2d_bytes_per_step": round(V.size * 8 / n_steps, 3),
                "d2h_bytes_per_step": round((V.size + 1) * 8 / n_steps, 3),
                "note": "loss.backward() through time_integrated_body_force, V from pinned host memory, "
                        "dL/dV and dL/dnu read back; graphs already captured, autograd warmed up",
                "reps": e2e_reps, "first_call_ms": round(first_call_s * 1e3, 2)},
        "gpu_launches": reps * (launches_fwd + launches_bwd),
        "loss": {"fp32": L32, "fp64": L64},
        "grad_fp32_vs_fp64_rel_l2": rel(g32n, g64n),
        "nu_grad": {"fp32": n32, "fp64": n64},
        "finite_differences_fp64_gpu": fd,
        "cpu_reference_gradient": cpu_ref,
        "clocks": clock_info,
    }
    print(json.dumps(out), flush=True)


def point_source(position, centre, nu, mag, t, real_t):
    """Diffused point source (heat-kernel Gaussian) of the passive-transport example
    (examples/3d_examples/PointSourceAdvectAndDiffuseCase/point_source_helpers.py)."""
    r2 = sum((position[d] - centre[d]) ** 2 for d in range(3))
    return (mag / (4 * real_t(np.pi) * nu * t) ** 1.5 * np.exp(-r2 / (4 * nu * t))).astype(real_t)


def _passive_case(grid, real_t, device, nu=1e-3, t0=5.0, centre=(0.3, 0.3, 0.3)):
    import torch

    from sopht_gb300.simulator import PassiveTransportFlowSimulator
    sim = PassiveTransportFlowSimulator(kinematic_viscosity=nu, grid_dim=3, grid_size=grid, x_range=1.0,
                                        real_t=real_t, time=t0, field_type="vector", device=device)
    mag = 4.0 * np.pi * nu * t0**1.5
    f0 = point_source(sim.position_field, centre, nu, mag, t0, real_t)
    for c in range(3):
        sim.primary_field[c].copy_(torch.from_numpy(f0).to(device))
    sim.velocity_field.fill_(1.0)
    return sim, f0, mag


def run_passive(args, rank, world):
    """Passive transport of a vector point source (point_source_advection_diffusion.py): timed at 256^3,
    where the working set (field, velocity, scratch: 470 MB) exceeds the L2; the example's own 128^3 run
    from t = 5.0 to 5.4 gives the accuracy figures."""
    import torch

    from sopht_gb300 import _lib
    from sopht_gb300.build import build
    from sopht_gb300.utils import ptr, sg_dtype, stream_ptr

    build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    grid = (256, 256, 256)
    cells = int(np.prod(grid))
    sim, _, _ = _passive_case(grid, np.float32, device)
    dt = sim.compute_stable_timestep()  # the velocity field is uniform and constant: dt is the same every step
    stream = torch.cuda.Stream(device)
    seg = min(args.steps, 25)
    n_seg = max(1, args.steps // seg)
    steps = seg * n_seg
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        stream.wait_stream(torch.cuda.current_stream())
        for _ in range(args.warmup):
            sim.time_step(dt=dt)
        with torch.cuda.graph(graph, stream=stream):
            for _ in range(seg):
                sim.time_step(dt=dt)
    with torch.cuda.stream(stream):
        graph.replay()
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    clocks.start()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        start.record(stream)
        for _ in range(n_seg):
            graph.replay()
        stop.record(stream)
    torch.cuda.synchronize()
    wall_ms = (time.perf_counter() - t_wall) * 1e3
    clock_info = clocks.stop()
    elapsed_ms = start.elapsed_time(stop)
    if elapsed_ms < 0.5 * wall_ms:
        raise RuntimeError(f"event time {elapsed_ms:.3f} ms disagrees with wall time {wall_ms:.3f} ms")
    graph.reset()
    del graph
    # the two kernels of one component, timed alone on the launching stream
    n = cells
    dt_by_dx = float(np.float32(dt / sim.dx))
    k = float(np.float32(sim.kinematic_viscosity * dt / sim.dx / sim.dx))
    reps = 20
    kern_ms = {}
    tmp = torch.empty_like(sim.primary_field)
    with torch.cuda.stream(stream):
        s = stream_ptr(device)
        for name in ("eno3_3d", "diffusion3d_3comp"):
            for r in range(reps + 3):
                if r == 3:
                    start.record(stream)
                if name == "eno3_3d":
                    _lib.call("sg_advection_eno3_step_3d", sg_dtype(np.float32), *grid, 3, ptr(sim.primary_field),
                              ptr(tmp), ptr(sim.velocity_field), dt_by_dx, s)
                else:
                    _lib.call("sg_diffusion_step_3d", sg_dtype(np.float32), *grid, ptr(sim.primary_field),
                              ptr(tmp), k, s)
            stop.record(stream)
            torch.cuda.synchronize()
            kern_ms[name] = start.elapsed_time(stop) / reps
    del tmp
    # end to end through the public API: host stable dt (one D2H read of the max) and the step call
    sim_e, _, _ = _passive_case(grid, np.float32, device)
    for _ in range(args.warmup):
        sim_e.time_step(dt=sim_e.compute_stable_timestep())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sim_e.time_step(dt=sim_e.compute_stable_timestep())
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    del sim_e
    # accuracy: the example's 128^3 run to t = 5.4 in FP32 and FP64 on the GPU, errors against the translated
    # point source as the example prints them; FP64 GPU steps against the FP64 oracle from the same state
    acc = {}
    small = (128, 128, 128)
    finals = {}
    for real_t in (() if args.skip_accuracy else (np.float32, np.float64)):
        s_sim, _, mag = _passive_case(small, real_t, device)
        n_steps = 0
        while s_sim.time < 5.4:
            s_sim.time_step(dt=s_sim.compute_stable_timestep())
            n_steps += 1
        t_end = float(s_sim.time)
        shift = 1.0 * (t_end - 5.0)
        exact = point_source(s_sim.position_field, (0.3 + shift,) * 3, 1e-3, mag, 5.0, real_t)
        w = s_sim.primary_field.cpu().numpy()
        err = np.fabs(w - exact[None])
        finals[real_t] = w.astype(np.float64)
        acc["fp32" if real_t == np.float32 else "fp64"] = {
            "steps": n_steps, "t_end": t_end, "l2_error": float(np.linalg.norm(err) * float(s_sim.dx) ** 1.5),
            "linf_error": float(err.max())}
    if finals:
        acc["fp32_vs_fp64_rel_l2"] = float(np.linalg.norm(finals[np.float32] - finals[np.float64])
                                           / np.linalg.norm(finals[np.float64]))
    cpu = None
    if not args.skip_cpu:
        from oracle.flow import PassiveTransportOracle
        g_sim, f0, _ = _passive_case(small, np.float64, device)
        ora = PassiveTransportOracle(1e-3, 3, small, 1.0, real_t=np.float64, time=5.0, field_type="vector")
        ora.primary_field[...] = f0[None]
        ora.velocity_field[...] = 1.0
        for _ in range(3):
            d = ora.compute_stable_timestep()
            assert g_sim.compute_stable_timestep() == d
            ora.time_step(d)
            g_sim.time_step(dt=d)
        gw = g_sim.primary_field.cpu().numpy()
        acc["fp64_gpu_vs_fp64_oracle_rel_l2_3_steps_128cube"] = float(np.linalg.norm(gw - ora.primary_field)
                                                                     / np.linalg.norm(ora.primary_field))
        # CPU baseline: the oracle (fp32, sweeps on z-slabs across the cores) on the same 256^3 workload,
        # a bounded sample
        from oracle.threaded import ThreadedPassiveTransportOracle
        c_ora = ThreadedPassiveTransportOracle(1e-3, 3, grid, 1.0, real_t=np.float32, time=5.0,
                                               field_type="vector")
        c_ora.velocity_field[...] = 1.0
        c_ora.primary_field[...] = point_source(c_ora.position_field, (0.3,) * 3, 1e-3,
                                                4.0 * np.pi * 1e-3 * 5.0**1.5, 5.0, np.float32)[None]
        c_ora.time_step(c_ora.compute_stable_timestep())
        nc, tc = 0, time.perf_counter()
        while True:
            c_ora.time_step(c_ora.compute_stable_timestep())
            nc += 1
            el = time.perf_counter() - tc
            if el >= args.cpu_seconds:
                break
        cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
        cpu = {"value": round(nc / el, 4), "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": f"{nc} steps of the same 256^3 vector workload after 1 warm-up step ({el:.1f} s), "
                         "numpy sweeps on z-slabs across all cores, fp32"}
    if rank != 0:
        return
    peaks = load_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    eno3_bytes = 36 * cells  # three components: field 12 + velocity 12 read, 12 written per cell
    out = {
        "metric": "passive-transport steps/s (vector point source, ENO3 advection + diffusion)",
        "value": round(world * steps / (elapsed_ms * 1e-3), 2), "unit": "steps/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(elapsed_ms / steps, 5), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "gcell_updates_per_s": round(world * cells * steps / (elapsed_ms * 1e-3) / 1e9, 3),
        "config": {"workload": "3D 256^3 fp32 passive transport of a vector point source (nu 1e-3, uniform "
                               "velocity 1 on every axis, x_range 1), the example's 128^3 case for accuracy",
                   "grid": list(grid), "field_type": "vector", "dt_rule": "compute_stable_timestep, CFL 0.1",
                   "l2": "no flush: the working set (470 MB) exceeds the 126 MB L2"},
        "step_bytes_per_cell": {"design": 60, "compulsory": 36,
                                "note": "ENO3 reads the 3 components and the velocity and writes a 3-component "
                                        "scratch (36 B), diffusion reads it and writes the field (24 B)"},
        "step_roofline": {"achieved_GB_s": round(60 * cells * steps / (elapsed_ms * 1e-3) / 1e9, 1),
                          "frac": round(60 * cells * steps / (elapsed_ms * 1e-3) / 1e9 / peak, 3)},
        "roofline": {"bound": "hbm", "kernel": "eno3_3d", "achieved": round(eno3_bytes / (kern_ms["eno3_3d"] * 1e-3)
                                                                             / 1e9, 1),
                     "peak": peak, "unit": "GB/s",
                     "frac": round(eno3_bytes / (kern_ms["eno3_3d"] * 1e-3) / 1e9 / peak, 3),
                     "traffic": traffic_from_profiles("pointsource256", "eno3_3d"),
                     "algorithmic_bytes_per_launch": eno3_bytes,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks else "fallback"},
        "kernels_ms": {k: round(v, 5) for k, v in kern_ms.items()},
        "kernels_note": "eno3_3d: the 3-component launch of the step (36 B/cell); diffusion3d_3comp: the "
                        "3-component diffusion of the step (24 B/cell)",
        "e2e": {"value": round(world * steps / e2e_s, 2), "unit": "steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 8,
                "note": "public API per step: compute_stable_timestep (max reduction, 8-byte read) and time_step"},
        "gpu_launches": steps * 2,
        "cpu_baseline": cpu,
        "accuracy": acc,
        "clocks": clock_info,
    }
    print(json.dumps(out), flush=True)


def run_passive_reference(args, rank, world):
    """The reference's passive-transport algorithm on the host cores (the numpy oracle), same 256^3 workload."""
    if rank != 0:
        return
    from oracle.threaded import ThreadedPassiveTransportOracle
    grid = (256, 256, 256)
    ora = ThreadedPassiveTransportOracle(1e-3, 3, grid, 1.0, real_t=np.float32, time=5.0, field_type="vector")
    ora.velocity_field[...] = 1.0
    ora.primary_field[...] = point_source(ora.position_field, (0.3,) * 3, 1e-3, 4.0 * np.pi * 1e-3 * 5.0**1.5, 5.0,
                                          np.float32)[None]
    ora.time_step(ora.compute_stable_timestep())
    budget = max(10.0, min(180.0, float(args.cpu_seconds) * 4))
    n, t0 = 0, time.perf_counter()
    while True:
        ora.time_step(ora.compute_stable_timestep())
        n += 1
        el = time.perf_counter() - t0
        if el >= budget or n >= args.steps:
            break
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    v = round(n / el, 4)
    out = {"impl": "reference", "metric": "passive-transport steps/s (vector point source, ENO3 advection + "
                                          "diffusion)",
           "value": v, "unit": "steps/s", "n_gpus": world, "steps": n, "warmup": 1, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "ms_per_step": round(1e3 / v, 2),
           "config": {"workload": "3D 256^3 fp32 passive transport of a vector point source", "grid": list(grid)},
           "cpu_baseline": {"value": v, "unit": "steps/s", "cores": cores, "kind": "port",
                            "sample": f"{n} steps after 1 warm-up step ({el:.1f} s), numpy sweeps on "
                                      "z-slabs across all cores, fp32"},
           "e2e": {"value": v, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def accuracy_checkpoints(wl, device, checkpoints, cpu_oracle=False):
    """Relative L2 of the fp32 GPU path against the same path in FP64 on the GPU (and, in 2D, the FP64
    CPU oracle) at the checkpoint steps.  All runs take the FP64 GPU run's dt sequence, so the errors
    measure arithmetic precision only."""
    import torch
    if not checkpoints:
        return None
    runs = {rt: make_gpu_case(wl, rt, device) for rt in (np.float32, np.float64)}
    orc = make_cpu_case(wl, np.float64) if cpu_oracle else None
    out = {"checkpoints": [], "fp64_reference": "this path in FP64 on the GPU (validated against the CPU oracle "
                                                "in tests)" + ("; plus the FP64 CPU oracle" if orc else "")}
    t = 0.0
    for step in range(1, max(checkpoints) + 1):
        dt = float(runs[np.float64][0].compute_stable_timestep(dt_prefac=wl.dt_prefac))
        for rt, (sim, inters) in runs.items():
            for inter in inters:
                if wl.kind == "rods":
                    inter.advance_rods(dt, wl.rod_dt, flow_time=t)
                else:
                    inter.time_step(dt=dt)
                inter()
            sim.time_step(dt=dt, free_stream_velocity=wl.u_inf)
        if orc:
            cpu_step(wl, orc[0], orc[1], dt=dt, t=t)
        t += dt
        if step in checkpoints:
            torch.cuda.synchronize()
            f = {rt: (sim.vorticity_field.double().cpu().numpy(), sim.velocity_field.double().cpu().numpy())
                 for rt, (sim, _) in runs.items()}
            row = {"step": step}
            for i, name in enumerate(("vorticity", "velocity")):
                a, b = f[np.float32][i], f[np.float64][i]
                row[f"{name}_rel_l2_fp32_vs_fp64_gpu"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
                if orc:
                    ref = (orc[0].vorticity_field, orc[0].velocity_field)[i]
                    row[f"{name}_rel_l2_fp32_vs_fp64_oracle"] = float(np.linalg.norm(a - ref) / np.linalg.norm(ref))
                    row[f"{name}_rel_l2_fp64_gpu_vs_fp64_oracle"] = float(np.linalg.norm(b - ref) /
                                                                          np.linalg.norm(ref))
            out["checkpoints"].append(row)
    del runs
    return out


def max_over_ranks(value, device=None):
    """The largest of every rank's ``value`` (a replica's time: the job ends with the slowest); the
    value itself when no process group is running."""
    import torch
    if not (torch.distributed.is_available() and torch.distributed.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


def traffic_from_profiles(workload, kernel):
    """DRAM bytes per launch recorded by the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(workload, {}).get(kernel)
        except Exception:
            return None
    return None


# ------------------------------------------------------------ CPU (oracle)


def make_cpu_case(wl: Workload, real_t=np.float32):
    from oracle.flow import (
        CircularCylinderOracle,
        ImmersedBodyInteractionOracle,
        NavierStokes2DOracle,
        RodElementCentricGridOracle,
    )
    from oracle.rod import CosseratRod, element_centric_view
    from oracle.threaded import ThreadedNavierStokes3DOracle
    rt = real_t
    # 3D: every sweep on z-slabs across the host cores, bitwise the serial oracle
    Sim = NavierStokes2DOracle if wl.dim == 2 else ThreadedNavierStokes3DOracle
    sim = Sim(wl.grid, wl.x_range, wl.nu, cfl=wl.cfl, real_t=rt, with_forcing=True, with_free_stream_flow=True)
    sim.vorticity_field[...] = wl.initial_vorticity(rt)
    inters, rods = [], []
    for k, b in enumerate(wl.bodies):
        if wl.kind == "cylinder":
            grid = CircularCylinderOracle(b["centre"], b["radius"], wl.n_markers)
            forces, torques = np.zeros((3, 1)), np.zeros((3, 1))
        else:
            m = ROD_MATERIAL
            rod = CosseratRod(b["n_elem"], b["base"], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0], b["length"], b["radius"],
                              m["density"], m["E"], shear_modulus=m["G"])
            rod.clamp_start()
            if wl.actuation:
                a = wl.actuation
                rod.drive = (a["amplitude"], a["frequency"], float(a["phases"][k]), np.array([0.0, 1.0, 0.0]))
            rods.append(rod)
            grid = RodElementCentricGridOracle(element_centric_view(rod))
            forces, torques = np.zeros((3, rod.n + 1)), np.zeros((3, rod.n))
        inters.append(ImmersedBodyInteractionOracle(sim.eul_grid_forcing_field, sim.velocity_field, forces,
                                                    torques, grid, wl.K, wl.C, sim.dx, wl.dim, real_t=rt))
    sim.rods = rods
    return sim, inters


def cpu_step(wl, sim, inters, dt=None, t=None):
    """One coupled step of the reference loop on the oracle (the rod loop of flow_past_rod_case.py:
    231-250 for rod workloads)."""
    from oracle.rod import coupled_rod_loop
    if dt is None:
        dt = sim.compute_stable_timestep(dt_prefac=wl.dt_prefac)
    if wl.kind == "rods":
        t0 = sim.time if t is None else t
        for rod in sim.rods:
            rod.time = t0
        coupled_rod_loop(sim.rods, inters, dt, wl.rod_dt)
        for inter in inters:
            inter()
    else:
        for inter in inters:
            inter.time_step(dt)
            inter()
    sim.time_step(dt, wl.u_inf)


def run_cpu_sample(wl, seconds, max_steps=None):
    sim, inters = make_cpu_case(wl)
    cpu_step(wl, sim, inters)  # warm-up (plans, caches)
    n = 0
    t0 = time.perf_counter()
    while True:
        cpu_step(wl, sim, inters)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_steps and n >= max_steps):
            break
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"value": round(n / el, 4), "unit": "flow steps/s", "cores": cores, "kind": "port",
            "sample": f"{n} coupled steps of the same workload ({wl.name}) after 1 warm-up step ({el:.1f} s), "
                      + ("numpy sweeps on z-slabs across all cores, " if wl.dim == 3 else "numpy sweeps, ")
                      + "scipy.fft with workers = all cores, fp32"
                      + ("; the rods' sub-steps on the numpy rod model" if wl.kind == "rods" else "")}


def run_reference(args, wl, rank, world):
    if rank != 0:
        return
    budget = max(10.0, min(180.0, float(args.cpu_seconds) * 4))
    cpu = run_cpu_sample(wl, budget, max_steps=args.steps)
    out = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": "flow steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "ms_per_step": round(1e3 / cpu["value"], 2),
           "config": {"workload": wl.description, "name": wl.name, "grid": list(wl.grid),
                      "dt_rule": f"compute_stable_timestep, CFL 0.1, dt_prefac {wl.dt_prefac}"},
           "cpu_baseline": cpu,
           "e2e": {"value": cpu["value"], "unit": "flow steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference's pystencils/pyfftw/numba stack is not installable offline; its algorithm runs "
                   "as the numpy/scipy oracle of this repository (pinned to fixtures produced by the reference)"}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="carpet256",
                    choices=["rod128", "cylinder2d", "carpet256", "batch64", "adjoint2d", "pointsource256"])
    ap.add_argument("--adjoint-steps", type=int, default=200)
    ap.add_argument("--adjoint-cpu-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--accuracy-steps", type=int, default=1000)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    ap.add_argument("--no-others", action="store_true", help="skip the other configurations' lines")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.workload == "batch64":
        run_batch(args, int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")))
        return
    if args.workload == "adjoint2d":
        run_adjoint(args, int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")))
        return
    if args.workload == "pointsource256":
        if args.impl == "reference":
            run_passive_reference(args, int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")))
        else:
            run_passive(args, int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")))
        return
    wl = make_workload(args.workload)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    try:
        if args.impl == "reference":
            run_reference(args, wl, rank, world)
        else:
            run_gpu(args, wl, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
