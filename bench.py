"""Benchmark: the coupled 3D rod-in-flow step on GB300 (flow steps/s).

Workload (one GPU): unbounded vorticity Navier-Stokes on a 128^3 grid, fp32,
cubic domain of side 1 (Poisson by domain doubling to a 256^3 FFT), one
clamped rod of 64 elements (length 0.3, radius 0.01) at the domain centre with
an element-centric forcing grid and cosine-delta virtual-boundary coupling
(K = -2e4, C = -1e2), uniform inflow U = 1, Re = 100 on the rod length
(nu = 3e-3), dt from the stable-timestep rule at CFL 0.1.  One step is: stable
dt, interactor time_step + interaction + spreading, flow time step.

The rod stays on the host (pyelastica's role); here it is held rigid and
clamped (its markers do not move), which is the configuration's initial
state; the rod dynamics integrator is not part of the timed path in either arm.

Arms
  default            this repository's GPU path.
      value  : device-resident steps/s: a CUDA graph of the whole coupled step
               (device dt + IB interaction + spread + flow step) replayed K times.
      e2e    : the same steps through the public Python API, per step uploading
               the marker kinematics from pinned host memory and reading the
               Lagrangian forcing back (what a host rod integrator needs).
  --impl reference   the reference algorithm's CPU implementation (the numpy/
               scipy oracle of this repository, since the reference's own JIT
               dependencies are not installable), all host cores, bounded sample.

Prints one JSON line on rank 0.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

GRID = (128, 128, 128)
X_RANGE = 1.0
U_INF = np.array([1.0, 0.0, 0.0])
ROD_LENGTH, ROD_RADIUS, N_ELEM = 0.3, 0.01, 64
NU = 1.0 * ROD_LENGTH / 100.0
K_STIFF, C_DAMP = -2e4, -1e2
CFL = 0.1
METRIC = "flow steps/s & Gcell-updates/s vs plain GPU path at stated FP64-oracle L2 error"
WORKLOAD = ("3D unbounded vorticity NS 128^3 fp32 (256^3 doubled FFT), one clamped rod (64 elements, "
            "element-centric cosine-delta forcing), U=1 inflow, Re=100 on rod length, CFL 0.1")

# algorithmic bytes per cell per pass of the fused fp32 3D step (3 components)
PASS_NAMES = ["forcing_curl", "uxw_update", "diffusion", "poisson_load", "y_fft", "z_conv", "y_ifft",
              "x_c2r", "curl"]
PASS_BYTES = {  # per cell, fp32, read + write
    "forcing_curl": 36, "uxw_update": 36, "diffusion": 24, "poisson_load": 60, "y_fft": 72, "z_conv": 108,
    "y_ifft": 72, "x_c2r": 36, "curl": 24}


class RodState:
    """A straight clamped rod with the attributes the forcing grids read."""

    def __init__(self):
        n = N_ELEM
        base = np.array([0.5, 0.5, 0.5 - ROD_LENGTH / 2])
        s = np.linspace(0.0, ROD_LENGTH, n + 1)
        self.n_elems = n
        self.position_collection = base[:, None] + np.outer([0.0, 0.0, 1.0], s)
        self.velocity_collection = np.zeros((3, n + 1))
        area = np.pi * ROD_RADIUS**2
        self.mass = np.full(n + 1, area * ROD_LENGTH / n)
        self.mass[[0, -1]] *= 0.5
        self.lengths = np.full(n, ROD_LENGTH / n)
        self.director_collection = np.repeat(np.eye(3)[:, :, None], n, axis=2)


def initial_vorticity(real_t):
    rng = np.random.default_rng(42)
    return (1e-3 * rng.standard_normal((3, *GRID))).astype(real_t)


# ------------------------------------------------------------------ clocks


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"sg_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9], strict=False):
                if flag.lower() == "active":
                    reasons.add(name)
        self.path.unlink(missing_ok=True)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------- GPU arm


def make_gpu_case(real_t, device):
    import torch

    import sopht_gb300.simulator as sps

    sim = sps.UnboundedNavierStokesFlowSimulator3D(
        grid_size=GRID, x_range=X_RANGE, kinematic_viscosity=NU, cfl=CFL, real_t=real_t, with_forcing=True,
        with_free_stream_flow=True, device=device)
    sim.vorticity_field.copy_(torch.from_numpy(initial_vorticity(real_t)).to(device))
    rod = RodState()
    inter = sps.CosseratRodFlowInteraction(
        cosserat_rod=rod, eul_grid_forcing_field=sim.eul_grid_forcing_field,
        eul_grid_velocity_field=sim.velocity_field, virtual_boundary_stiffness_coeff=K_STIFF,
        virtual_boundary_damping_coeff=C_DAMP, dx=sim.dx, grid_dim=3, real_t=real_t,
        forcing_grid_cls=sps.CosseratRodElementCentricForcingGrid)
    return sim, inter


def public_api_step(sim, inter):
    """One coupled step through the drop-in API (flow_past_rod_case.py:231-250 order)."""
    dt = sim.compute_stable_timestep()
    inter.time_step(dt=dt)
    inter()
    sim.time_step(dt=dt, free_stream_velocity=U_INF)
    return inter.lag_grid_forcing_host()


def device_step(sim, inter, events=None):
    """The same step with dt on the device (capturable)."""
    from sopht_gb300 import _lib
    dsc = sim.device_stable_timestep(free_stream_velocity=U_INF, recompute_max=False)
    inter.device_call(dsc)
    if events is not None:
        arr = (__import__("ctypes").c_void_p * len(events))(*[e.cuda_event for e in events])
        _lib.call("sg_flow_set_timing_events", sim._plan, len(events), arr)
    sim.time_step_device(dsc)


def run_gpu(args, rank, world):
    import torch

    from sopht_gb300.build import build

    build()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    rt = np.float32
    sim, inter = make_gpu_case(rt, device)
    inter.upload_kinematics()
    # initial max |u| for the first device dt
    sim.device_stable_timestep(free_stream_velocity=U_INF, recompute_max=True)
    stream = torch.cuda.Stream(device)
    torch.cuda.synchronize()
    # warm-up (also compiles nothing: kernels are AOT) and graph capture of S steps
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            device_step(sim, inter)
    torch.cuda.synchronize()
    seg = min(args.steps, 25)
    n_seg = max(1, args.steps // seg)
    steps = seg * n_seg
    n_ev = len(PASS_NAMES) + 1
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ev)] for _ in range(seg)]
    with torch.cuda.stream(stream):
        for ev_list in events:  # torch creates the CUDA events lazily, on first record
            for e in ev_list:
                e.record(stream)
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(stream):
        stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(graph, stream=stream):
            for k in range(seg):
                device_step(sim, inter, events[k])
    torch.cuda.synchronize()
    graph.replay()  # one untimed replay after capture
    torch.cuda.synchronize()
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    start.record(stream)
    for _ in range(n_seg):
        graph.replay()
    stop.record(stream)
    torch.cuda.synchronize()
    clock_info = clocks.stop()
    elapsed_ms = start.elapsed_time(stop)
    if world > 1:
        t = torch.tensor([elapsed_ms], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        torch.distributed.barrier()
    # per-pass durations from the last replay
    per_pass = {name: [] for name in PASS_NAMES}
    for k in range(seg):
        for i, name in enumerate(PASS_NAMES):
            per_pass[name].append(events[k][i].elapsed_time(events[k][i + 1]))
    cells = int(np.prod(GRID))
    kernels = {}
    for name, vals in per_pass.items():
        ms = float(np.mean(vals))
        kernels[name] = {"ms": round(ms, 5), "GB_s": round(PASS_BYTES[name] * cells / (ms * 1e-3) / 1e9, 1),
                         "launches_timed": len(vals)}
    value = world * steps / (elapsed_ms * 1e-3)

    # end to end through the public API: host dt, H2D marker kinematics, D2H forcing
    sim_e, inter_e = make_gpu_case(rt, device)
    for _ in range(args.warmup):
        public_api_step(sim_e, inter_e)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e2e_steps = steps
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        public_api_step(sim_e, inter_e)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if world > 1:
        t = torch.tensor([e2e_s], device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    n_lag = inter_e.num_lag_nodes
    h2d = 2 * 3 * n_lag * 8
    d2h = 3 * n_lag * 4 + 8

    accuracy = None
    if rank == 0 and not args.skip_accuracy:
        accuracy = accuracy_vs_fp64(args, device, min(steps, args.accuracy_steps))
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        cpu = run_cpu_sample(args.cpu_seconds)
    if rank != 0:
        return
    top = max(kernels, key=lambda k: kernels[k]["ms"])
    peaks = load_peaks()
    hbm = peaks.get("hbm_gbs")
    algo = PASS_BYTES[top] * cells
    achieved = algo / (kernels[top]["ms"] * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 3) if hbm else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if hbm else "fallback 6800 GB/s",
                "traffic": traffic_from_profiles(top), "algorithmic_bytes_per_launch": algo}
    if not hbm:
        roofline["peak"] = 6800.0
        roofline["frac"] = round(achieved / 6800.0, 3)
    step_ms = elapsed_ms / steps
    step_bytes = sum(PASS_BYTES.values()) * cells
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "flow steps/s", "n_gpus": world, "steps": steps,
        "warmup": args.warmup, "ms_per_step": round(step_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "gcell_updates_per_s": round(world * cells * steps / (elapsed_ms * 1e-3) / 1e9, 3),
        "config": {"workload": WORKLOAD, "grid": list(GRID), "dt_rule": "compute_stable_timestep, CFL 0.1",
                   "rod": "rigid clamped stand-in, host-side; rod integrator not timed", "parallelism":
                   "replicas only" if world > 1 else "single GPU",
                   "l2": "no flush: step working set ~250 MB > 126 MB L2"},
        "roofline": roofline,
        "step_roofline": {"algorithmic_bytes_per_step": step_bytes,
                          "achieved_GB_s": round(step_bytes / (step_ms * 1e-3) / 1e9, 1),
                          "frac": round(step_bytes / (step_ms * 1e-3) / 1e9 / (hbm or 6800.0), 3)},
        "kernels": kernels,
        "e2e": {"value": round(world * e2e_steps / e2e_s, 2), "unit": "flow steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "note": "public API per step: host dt (sync), H2D marker positions+velocities, D2H lag forcing"},
        "gpu_launches": 12 * steps,
        "clocks": clock_info,
        "accuracy": accuracy,
        "cpu_baseline": cpu,
    }
    print(json.dumps(out), flush=True)


def accuracy_vs_fp64(args, device, steps):
    """Relative L2 of the fp32 GPU path against the same path in fp64 after `steps` steps."""
    import torch
    res = {}
    fields = {}
    for rt in (np.float32, np.float64):
        sim, inter = make_gpu_case(rt, device)
        for _ in range(steps):
            dt = sim.compute_stable_timestep()
            inter.time_step(dt=dt)
            inter()
            sim.time_step(dt=dt, free_stream_velocity=U_INF)
        torch.cuda.synchronize()
        fields[rt] = (sim.vorticity_field.double().cpu().numpy(), sim.velocity_field.double().cpu().numpy())
        del sim, inter
    for i, name in enumerate(("vorticity", "velocity")):
        a, b = fields[np.float32][i], fields[np.float64][i]
        res[f"{name}_rel_l2_vs_fp64"] = float(np.linalg.norm(a - b) / np.linalg.norm(b))
    res["steps"] = steps
    res["fp64_reference"] = "this path in FP64 on the GPU (validated against the CPU oracle in tests)"
    return res


def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


def traffic_from_profiles(kernel):
    """DRAM bytes per launch recorded by the committed ncu summary, if any."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text()).get(kernel)
        except Exception:
            return None
    return None


# ------------------------------------------------------------ CPU (oracle)


def make_cpu_case():
    from oracle.flow import ImmersedBodyInteractionOracle, NavierStokes3DOracle, RodElementCentricGridOracle
    rt = np.float32
    sim = NavierStokes3DOracle(GRID, X_RANGE, NU, cfl=CFL, real_t=rt, with_forcing=True,
                               with_free_stream_flow=True)
    sim.vorticity_field[...] = initial_vorticity(rt)
    rod = RodState()
    grid = RodElementCentricGridOracle(rod)
    inter = ImmersedBodyInteractionOracle(sim.eul_grid_forcing_field, sim.velocity_field,
                                          np.zeros((3, N_ELEM + 1)), np.zeros((3, N_ELEM)), grid, K_STIFF,
                                          C_DAMP, sim.dx, 3, real_t=rt)
    return sim, inter


def cpu_step(sim, inter):
    dt = sim.compute_stable_timestep()
    inter.time_step(dt)
    inter()
    sim.time_step(dt, U_INF)


def run_cpu_sample(seconds, max_steps=None):
    sim, inter = make_cpu_case()
    cpu_step(sim, inter)  # warm-up (plans, caches)
    n = 0
    t0 = time.perf_counter()
    while True:
        cpu_step(sim, inter)
        n += 1
        el = time.perf_counter() - t0
        if el >= seconds or (max_steps and n >= max_steps):
            break
    cores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
    return {"value": round(n / el, 4), "unit": "flow steps/s", "cores": cores, "kind": "port",
            "sample": f"{n} coupled steps of the same 128^3 workload after 1 warm-up step ({el:.1f} s), "
                      "numpy + scipy.fft with workers = all cores, fp32"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    budget = max(10.0, min(180.0, float(args.cpu_seconds) * 4))
    cpu = run_cpu_sample(budget, max_steps=args.steps)
    out = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": "flow steps/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "ms_per_step": round(1e3 / cpu["value"], 2),
           "config": {"workload": WORKLOAD, "grid": list(GRID), "dt_rule": "compute_stable_timestep, CFL 0.1"},
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
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-accuracy", action="store_true")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        torch.distributed.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    try:
        if args.impl == "reference":
            run_reference(args, rank, world)
        else:
            run_gpu(args, rank, world)
    finally:
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
