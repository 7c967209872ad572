"""Benchmark of the fused heat + phase-field step on GB300.

Workload (default): single-track laser scan, 400 x 200 x 100 cells (8M) at
h = 1 um, Voronoi polycrystal of 2000 grains with 20 orientations, cubic
anisotropy 0.15, explicit FD heat equation with a Gaussian surface source
(200 W, r = 50 um, absorptivity 0.4, 0.8 m/s along x, T0 = 300 K),
Arrhenius mobility, float32.  A "step" is one fused heat + phase-field update
of the whole grid; the default K = 2000 steps is the workload's full run.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Rank 0 prints one JSON line.  Under torchrun each rank runs its own replica
(the path does not shard on one box: "replicas only"), value sums over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

WORKLOAD = dict(name="laser_track_8M", Nx=400, Ny=200, Nz=100, h=1e-6, num_grains=2000,
                num_oris=20, anisotropy=0.15, power=200.0, radius=5e-5, absorptivity=0.4,
                speed=0.8, T0=300.0, T_liquidus=1623.0, seed=2)
PF_KEYS = dict(T_liquidus=1623.0, gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6, m_g=2.4e5,
               ad_hoc=1.0)
METRIC = "cell_orientation_updates_per_s"
UNIT = "cell*ori/s"
KERNEL = ("pf_lane_kernel<NV=5, ANISO=true, TSRC=heat, TX=16, S=4, COMP=true> (fused "
          "compensated heat + anisotropic phase field, one cell per thread, 16x16 tiles, "
          "4-slot TMA ring)")


def gamma_args(w):
    g = dict(eta=w["absorptivity"], r=w["radius"], rho=8440.0, h=10.0, eps=0.4, SB=5.67e-8,
             T0=w["T0"], Ts=1563.0, Tl=1623.0)
    g["L"] = 290e3 / (g["Tl"] - g["Ts"])
    return g


def algorithmic_bytes_per_step(w):
    """Read eta + write eta + read T + write T, float32 (padding and halo
    re-reads excluded): N (2 n 4 + 2 4)."""
    N = w["Nx"] * w["Ny"] * w["Nz"]
    return N * (2 * w["num_oris"] * 4 + 8)


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def reduce_over_ranks(ms, units):
    """Replicas: the slowest rank's timed region (max) and the units all
    ranks processed (sum), over the default process group (NCCL on GPUs,
    gloo on CPU)."""
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes per launch of the top kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "pf_lane_laser_track_8M.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def build_case(w, device_run=True):
    """The laser-track workload (``jax_am_gb300.workloads.laser_track_case``)
    at the grid of ``w``."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import single_track
    pf_args = dict(PF_KEYS, Nx=w["Nx"], Ny=w["Ny"], Nz=w["Nz"], h=w["h"],
                   num_grains=w["num_grains"], num_oris=w["num_oris"], anisotropy=w["anisotropy"],
                   T_liquidus=w["T_liquidus"])
    poly = Field(pf_args, seed=w["seed"])
    solver = PFSolver(pf_args, poly)
    g = gamma_args(w)
    path = single_track(50e-6, 0.5 * w["Ny"] * w["h"], w["speed"], w["power"], 1.0)
    return solver, g, path, poly


def time_serving(num_jobs=256, rate=50.0):
    """The serving stream (256 directional-solidification jobs, Poisson
    arrivals at 50 jobs/s, HBM budget 120 GB), all against the wall clock
    with real-time arrivals: continuous batching, against two sequential
    plain baselines (one job at a time): ``PFSolver.stepper`` per step from
    Python (the reference driver's loop) and a resident graph-replayed run
    per job (``QuenchRun``, the best plain path).  Then the batched kernel
    alone: the whole stream admitted at once (no arrival gaps), timed with
    CUDA events, as algorithmic bandwidth (eta read and written once per
    cell, orientation and step) against the measured HBM peak."""
    from jax_am_gb300.serving import BatchServer, run_sequential, run_sequential_resident
    from jax_am_gb300.workloads import serving_stream
    t0 = time.perf_counter()
    jobs = serving_stream(num_jobs, rate)
    setup = time.perf_counter() - t0
    seq_jobs = [j.fresh() for j in jobs]
    res_jobs = [j.fresh() for j in jobs]
    kern_jobs = [j.fresh() for j in jobs]
    srv = BatchServer(hbm_budget=120e9, max_jobs=256, graph_steps=16)
    for j in jobs:
        srv.submit(j)
    batched = srv.run(realtime=True)
    batched_results = [j.result for j in jobs]
    sequential = run_sequential(seq_jobs, realtime=True)
    resident = run_sequential_resident(res_jobs, realtime=True)
    worst = max(float((a - b.result).abs().max().item()) for a, b in zip(batched_results, seq_jobs))
    worst_r = max(float((a - b.result).abs().max().item())
                  for a, b in zip(batched_results, res_jobs))
    del seq_jobs, res_jobs
    # the batched kernel alone over the whole stream
    srv2 = BatchServer(hbm_budget=120e9, max_jobs=256, graph_steps=16)
    for j in kern_jobs:
        j.arrival = 0.0
        srv2.submit(j)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    srv2.run(realtime=False)
    e1.record()
    torch.cuda.synchronize()
    kern_s = e0.elapsed_time(e1) / 1e3
    units = sum(j.cells * j.num_oris * j.steps for j in kern_jobs)
    gbs = units * 8 / kern_s / 1e9
    keys = ("jobs_per_s", "p50_s", "p99_s", "mean_s", "wall_s")
    return {
        "workload": f"{num_jobs} directional-solidification jobs, Poisson {rate:g} jobs/s, "
                    "Nx,Ny~U[32,160], Nz~U[16,64], n~U[10,30], steps~U[100,2000], "
                    "G~U[5e5,2e6] K/m, budget 120 GB",
        "batched": {k: batched[k] for k in keys},
        "sequential": {k: sequential[k] for k in keys},
        "sequential_resident": {k: resident[k] for k in keys},
        "jobs_per_s_ratio": batched["jobs_per_s"] / sequential["jobs_per_s"],
        "jobs_per_s_ratio_vs_resident": batched["jobs_per_s"] / resident["jobs_per_s"],
        "peak_hbm_gb": srv.peak_bytes / 1e9,
        "max_abs_diff_batched_vs_sequential": worst,
        "max_abs_diff_batched_vs_resident": worst_r,
        "setup_s": setup,
        "gpu_launches_batched": srv.launches,
        "batch_kernel": {"seconds": kern_s, "cell_ori_updates": units,
                         "achieved_GBps": gbs, "roofline_frac": gbs / measured_peak()[0],
                         "note": "all 256 jobs admitted at once; eta read + written once "
                                 "per cell, orientation and step (unpadded n)"},
    }


def time_adjoint():
    """The differentiable run (128 x 128 x 64, n = 10, 500 steps, checkpoint
    every 25): forward, then dJ/d(P, v, eta0) by the hand-written adjoint."""
    from jax_am_gb300.workloads import differentiable_run
    prob, P, v = differentiable_run()
    eta0 = prob.solver.ini_cond()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    J = prob.forward(P, v, eta0)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    dP, dv, de = prob.gradient()
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    return {"workload": "128x128x64 cells, 300 grains, n=10, laser 200 W 0.8 m/s, 500 steps, "
                        "checkpoint every 25",
            "J": J, "dJ_dP": dP, "dJ_dv": dv, "dJ_deta0_norm": float(de.norm().item()),
            "forward_s": t1 - t0, "gradient_s": t2 - t1}


def time_heat_step(steps=200, warmup=10, grid=(800, 400, 200)):
    """The standalone explicit heat step (``pfg_heat_step``, the drop-in for
    ``gamma.update_T``) on an 800 x 400 x 200 grid (64M interior cells,
    ghosted float32: 257 MB per buffer, so the two ping-pong buffers exceed
    L2), both axis orders, CUDA events: microseconds per step and algorithmic
    bandwidth (read + write 4 bytes per interior cell) against the measured
    HBM peak.  ``warmup`` ping-pong pairs (two launches each) precede the
    timed ``steps`` launches of each axis order."""
    import ctypes
    from jax_am_gb300 import _lib
    from jax_am_gb300.cfd.gamma import make_heat_params
    lib = _lib.load()
    w = WORKLOAD
    nx, ny, nz = grid
    peak = measured_peak()[0]
    out = {"workload": f"{nx}x{ny}x{nz} interior cells, 200 W Gaussian, float32",
           "l2": "inputs larger than L2 (two ghosted buffers of "
                 f"{(nx + 2) * (ny + 2) * (nz + 2) * 4 / 1e6:.0f} MB)"}
    for name, layout in (("xyz_reference_order", _lib.LAYOUT_XYZ), ("zyx", _lib.LAYOUT_ZYX)):
        shape = (nx + 2, ny + 2, nz + 2) if layout == _lib.LAYOUT_XYZ else (nz + 2, ny + 2, nx + 2)
        a = torch.full(shape, w["T0"], device="cuda")
        b = a.clone()
        h = make_heat_params(gamma_args(w), nx, ny, nz, w["h"], w["h"], w["h"], layout=layout)
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def step(src, dst):
            _lib.check(lib.pfg_heat_step(ctypes.byref(h), _lib.ptr(src), _lib.ptr(dst), 50e-6,
                                         100e-6, w["power"], 2e-9, s), "pfg_heat_step")
        for _ in range(warmup):
            step(a, b)
            step(b, a)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for k in range(steps):
            if k % 2 == 0:
                step(a, b)
            else:
                step(b, a)
        e1.record()
        torch.cuda.synchronize()
        us = e0.elapsed_time(e1) / steps * 1e3
        gbs = nx * ny * nz * 8 / (us * 1e-6) / 1e9
        out[name] = {"us_per_step": us, "achieved_GBps": gbs, "roofline_frac": gbs / peak}
        del a, b
    return out


def time_inspect(solver, run, reps=50):
    """The reference's inspect_sol metrics on the laser-track state
    (``PFSolver.inspect``'s kernels: argmax changes, liquid cells, max T,
    non-finite values, one pass over eta and T) and the full diagnostics
    (energy and per-orientation mass as well), CUDA events over ``reps``
    back-to-back launches: microseconds per record and the bandwidth of the
    inspect pass (eta + ghosted T read once) against the measured HBM peak."""
    eta, T = run.state, run.T_ghosted

    def timed(entry):
        for _ in range(3):
            solver._diag_launch(eta, T, None, None, True, entry)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            solver._diag_launch(eta, T, None, None, True, entry)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps * 1e3
    us = timed("pfg_pf_inspect")
    gbs = (eta.numel() + T.numel()) * 4 / (us * 1e-6) / 1e9
    return {"workload": "laser_track_8M state (400x200x100 cells, n=20), ghosted T",
            "inspect_us": us, "achieved_GBps": gbs, "roofline_frac": gbs / measured_peak()[0],
            "full_diag_us": timed("pfg_pf_diag")}


def time_cfd(steps=20, warmup=3, cpu=False):
    """The implicit CFD solver (``AM_3d``, float64) on the reference's
    standalone CFD driver configuration (``workloads.cfd_simple_case``):
    ``warmup`` steps (the melt pool forms and the flow starts), then
    ``steps`` timed steps with CUDA events around ``time_integration`` (which
    reads only convergence flags on the host).  ``cpu``: also time one step
    of the float64 CPU oracle from the same state (tens of seconds)."""
    from jax_am_gb300.cfd import cfd_am as G
    from jax_am_gb300.workloads import cfd_simple_case
    s = G.AM_3d(cfd_simple_case())
    for _ in range(warmup):
        s.time_integration()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    its = []
    e0.record()
    for _ in range(steps):
        s.time_integration()
        its.append(s.iterations())
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    mean = lambda xs: sum(xs) / len(xs)  # noqa: E731
    out = {"workload": "cfd_simple_2M: 464x93x46 cells, 348x46x18 flow box, 100 W at 0.5 m/s "
                       "(applications/cfd/simple), float64",
           "warmup_steps": warmup, "steps": steps, "ms_per_step": ms,
           "cells_per_s": 464 * 93 * 46 / (ms / 1e3),
           "newton_per_step": mean([i["newton"] for i in its]),
           "energy_krylov_per_step": mean([i["energy_krylov"] for i in its]),
           "momentum_krylov_per_step": mean([sum(i["momentum_krylov"]) for i in its]),
           "pressure_krylov_per_step": mean([i["pressure_krylov"] for i in its]),
           "T_max": float(s.T.max()), "vel_max": float(s.vel.abs().max())}
    if cpu:
        import numpy as np
        from oracle import cfd_oracle as C
        a = cfd_simple_case()
        mesh, ml = a["mesh"], a["mesh_local"]
        o = C.AM3d(dict(a, cp=C.LinClip(*G.linear_clip_params(a["cp"])),
                        k=C.LinClip(*G.linear_clip_params(a["k"]))),
                   C.Mesh(mesh.domain, mesh.shape), C.Mesh(ml.domain, ml.shape))
        for name in ("T", "vel", "conv", "grad_p0"):
            setattr(o, name, getattr(s, name).cpu().numpy().reshape(getattr(o, name).shape))
        o.conv_T = s.conv_T.cpu().numpy()[..., 0]
        o.solidID = s.solidID.cpu().numpy()[..., 0]
        o.t = s.t
        t0 = time.perf_counter()
        o.time_integration()
        cpu_s = time.perf_counter() - t0
        out["cpu_oracle"] = {"s_per_step": cpu_s, "kind": "port", "cores": 1,
                             "sample": "one step of the float64 NumPy oracle from the GPU "
                                       "run's state", "iterations": o.last_iters}
    return out


def _time_run(run, steps):
    run.prepare()  # graph capture (one eager step) outside the timed region
    run.run(run.graph_steps)  # warm-up: one replay
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run.run(steps)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def time_other_configs(peak):
    """The other single-solve configurations on the device (graph replay,
    CUDA events): directional solidification at full size (64 x 64 x 32,
    40 grains, n = 20, periodic x/y, moving gradient, liquid forcing, its 200
    steps) and the large multi-track scan (800 x 400 x 200, 20000 grains,
    n = 30, A = 0.15, fused heat, three 250 W tracks at 1 m/s scanned in turn;
    200 of its 5000 steps, the per-step cost being the same)."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, Quench
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import HeatPFRun, QuenchRun, raster
    from jax_am_gb300.workloads import PF_KEYS as WK, gamma_args as wg
    from jax_am_gb300 import _lib
    out = {}
    a1 = dict(WK, Nx=64, Ny=64, Nz=32, h=1e-6, num_grains=40, num_oris=20, T_liquidus=1700.0,
              anisotropy=0.0, force_liquid_zero=True, liquid_shift=1.0,
              bc=("periodic", "periodic", "neumann"))
    s1 = PFSolver(a1, Field(a1, seed=1))
    run1 = QuenchRun(s1, Quench(1700.0, 1e6, 0.1, z0=16e-6), float(np.float32(s1.stable_dt())))
    ms = _time_run(run1, 200)
    N1 = 64 * 64 * 32
    out["directional_solidification_128K"] = {
        "steps": 200, "ms_per_step": ms, "cell_ori_updates_per_s": N1 * 20 / (ms / 1e3),
        "achieved_GBps": N1 * 20 * 8 / (ms / 1e3) / 1e9, "plan": _lib.describe_plan(s1.params)}
    del run1, s1
    a5 = dict(WK, Nx=800, Ny=400, Nz=200, h=1e-6, num_grains=20000, num_oris=30,
              anisotropy=0.15, T_liquidus=1623.0)
    s5 = PFSolver(a5, Field(a5, seed=5))
    run5 = HeatPFRun(s5, wg(), raster([100e-6, 200e-6, 300e-6], 1.0, 250.0, 50e-6, 750e-6))
    ms = _time_run(run5, 200)
    N5 = 800 * 400 * 200
    ach = N5 * (2 * 30 * 4 + 8) / (ms / 1e3) / 1e9
    out["large_multi_track_64M"] = {
        "steps": 200, "ms_per_step": ms, "cell_ori_updates_per_s": N5 * 30 / (ms / 1e3),
        "achieved_GBps": ach, "roofline_frac": ach / peak, "plan": _lib.describe_plan(s5.params),
        "l2": "inputs larger than L2 (eta 7.7 GB per buffer)"}
    del run5, s5
    torch.cuda.empty_cache()
    return out


def time_cpu_baseline(w, budget_s=15.0, threads=None, sample=(100, 50, 25), steps_max=50):
    """The float32 PyTorch restatement of the same fused step on the host
    cores, on a reduced grid (bounded sample), in cell*ori updates/s."""
    from oracle import pf_torch as PT
    from jax_am_gb300.phase_field.utils import grain_directions, random_quaternions
    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    nx, ny, nz = sample
    n = w["num_oris"]
    rng = np.random.default_rng(0)
    a = dict(PF_KEYS, anisotropy=w["anisotropy"], h=(w["h"],) * 3)
    dirs = torch.tensor(grain_directions(random_quaternions(n, rng)), dtype=torch.float32)
    inds = rng.integers(0, n, nx * ny * nz)
    eta = torch.zeros((nz * ny * nx, n))
    eta[torch.arange(nz * ny * nx), torch.tensor(inds)] = 1.0
    eta = eta.reshape(nz, ny, nx, n)
    Tg = torch.full((nz + 2, ny + 2, nx + 2), w["T0"])
    g = gamma_args(w)
    dt = 3e-8

    def laser(t):
        return 20e-6 + w["speed"] * t, 0.5 * ny * w["h"], w["power"]

    with torch.no_grad():
        PT.coupled_step(eta, Tg, 0.0, dt, a, g, laser, dirs)  # warm-up
        t0 = time.perf_counter()
        steps = 0
        while steps < steps_max and (time.perf_counter() - t0) < budget_s:
            eta, Tg = PT.coupled_step(eta, Tg, steps * dt, dt, a, g, laser, dirs)
            steps += 1
        el = time.perf_counter() - t0
    value = nx * ny * nz * n * steps / el
    return {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{steps} fused steps of the float32 PyTorch-CPU restatement "
                      f"(oracle/pf_torch.py) on {nx}x{ny}x{nz} cells, n={n}, A={w['anisotropy']}, "
                      f"{el:.1f} s"}


def time_cpu_full(w, warmup, steps, budget_s=60.0, warmup_budget_s=10.0, threads=None):
    """The float32 PyTorch restatement of the fused step (``oracle/pf_torch.py``)
    on the full benchmarked grid: the same Voronoi polycrystal (seed), laser
    path and time step as the GPU arm, all host threads.  ``warmup`` untimed
    steps (at most ``warmup_budget_s`` of them), then timed steps until
    ``steps`` are done or ``budget_s`` has passed (at least one): the bounded
    sample of the workload."""
    from oracle import pf_torch as PT
    from jax_am_gb300.cfd.gamma import stable_dt as heat_dt
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.utils import Field
    threads = threads or os.cpu_count()
    torch.set_num_threads(threads)
    nx, ny, nz, n = w["Nx"], w["Ny"], w["Nz"], w["num_oris"]
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=w["h"], num_grains=w["num_grains"],
                   num_oris=n, anisotropy=w["anisotropy"], T_liquidus=w["T_liquidus"])
    poly = Field(pf_args, seed=w["seed"])
    N = nx * ny * nz
    eta = torch.zeros((N, n))
    eta[torch.arange(N), torch.as_tensor(np.asarray(poly.cell_ori_inds))] = 1.0
    eta = eta.reshape(nz, ny, nx, n)
    dirs = torch.tensor(np.asarray(poly.unique_grain_directions), dtype=torch.float32)
    a = dict(PF_KEYS, T_liquidus=w["T_liquidus"], anisotropy=w["anisotropy"], h=(w["h"],) * 3)
    g = gamma_args(w)
    dt = float(np.float32(min(PFSolver.stable_dt_for(pf_args), heat_dt(g, w["h"], w["h"], w["h"]))))
    Tg = torch.full((nz + 2, ny + 2, nx + 2), w["T0"])
    x_start, y = 50e-6, 0.5 * ny * w["h"]

    def laser(t):
        return x_start + w["speed"] * t, y, w["power"]

    k = 0
    with torch.no_grad():
        t0 = time.perf_counter()
        while k < warmup and (k == 0 or time.perf_counter() - t0 < warmup_budget_s):
            eta, Tg = PT.coupled_step(eta, Tg, k * dt, dt, a, g, laser, dirs)
            k += 1
        w_done = k
        t0 = time.perf_counter()
        done = 0
        while done < steps and (done == 0 or time.perf_counter() - t0 < budget_s):
            eta, Tg = PT.coupled_step(eta, Tg, k * dt, dt, a, g, laser, dirs)
            k += 1
            done += 1
        el = time.perf_counter() - t0
    return {"value": N * n * done / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{done} timed fused steps (after {w_done} warm-up steps) of the float32 "
                      f"PyTorch-CPU restatement (oracle/pf_torch.py) on the full "
                      f"{nx}x{ny}x{nz} grid, n={n}, A={w['anisotropy']}, the GPU arm's "
                      f"polycrystal, laser path and dt, {el:.1f} s",
            "steps_timed": done, "seconds": el}


def time_cpu_numpy(w, budget_s=8.0, sample=(50, 25, 13), steps_max=10):
    """The float64 NumPy oracle (``oracle/pf_oracle.py``, the restatement the
    parity tests check against) on the same physics, a smaller bounded sample:
    the second CPU reference point beside the float32 PyTorch port."""
    from oracle import pf_oracle as O
    from jax_am_gb300.phase_field.utils import grain_directions, random_quaternions
    nx, ny, nz = sample
    n = w["num_oris"]
    rng = np.random.default_rng(0)
    args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, anisotropy=w["anisotropy"], h=(w["h"],) * 3,
                num_oris=n)
    dirs = grain_directions(random_quaternions(n, rng)).astype(np.float64)
    eta = np.zeros((nx * ny * nz, n))
    eta[np.arange(nx * ny * nz), rng.integers(0, n, nx * ny * nz)] = 1.0
    Tg = np.full((nx + 2, ny + 2, nz + 2), w["T0"])
    g = gamma_args(w)
    dt = 3e-8

    def laser(t):
        return 20e-6 + w["speed"] * t, 0.5 * ny * w["h"], w["power"]

    t0 = time.perf_counter()
    steps = 0
    while steps < steps_max and (steps == 0 or time.perf_counter() - t0 < budget_s):
        eta, Tg = O.coupled_step(eta, Tg, steps * dt, dt, args, g, laser, dirs)
        steps += 1
    el = time.perf_counter() - t0
    return {"value": nx * ny * nz * n * steps / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{steps} fused steps of the float64 NumPy oracle (oracle/pf_oracle.py) on "
                      f"{nx}x{ny}x{nz} cells, n={n}, A={w['anisotropy']}, {el:.1f} s"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    cb = time_cpu_full(WORKLOAD, args.warmup, args.steps)
    cb["small_sample"] = time_cpu_baseline(WORKLOAD, budget_s=10.0, steps_max=10 ** 6)
    line = {
        "impl": "reference", "metric": METRIC, "value": cb["value"], "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": WORKLOAD["name"],
                   "grid": [WORKLOAD["Nx"], WORKLOAD["Ny"], WORKLOAD["Nz"]],
                   "num_oris": WORKLOAD["num_oris"], "num_grains": WORKLOAD["num_grains"],
                   "anisotropy": WORKLOAD["anisotropy"],
                   "heat": "fused explicit FD + Gaussian 200 W"},
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "JAX (the reference's runtime) is not installable here; the reference arm times "
                "the PyTorch-CPU restatement of the reference algorithm on all host threads, on "
                "the full benchmarked grid (a bounded number of steps)",
    }
    print(json.dumps(line), flush=True)


def profile_run(args):
    """Eager steps of the laser-track workload, one kernel launch per step:
    ``ncu -k regex:pf_ -s <warmup> -c 1 python bench.py --profile`` captures
    the first timed launch.  ``--profile-oris N`` runs the same grid with N
    orientations (N = 30: the 8-byte-vector path of the TMA kernel)."""
    import __graft_entry__
    __graft_entry__.build()
    from jax_am_gb300.runner import HeatPFRun
    from jax_am_gb300 import _lib
    solver, g, path, poly = build_case(dict(WORKLOAD, num_oris=args.profile_oris))
    run = HeatPFRun(solver, g, path)
    if args.state_in:  # a state saved by an earlier --state-out run
        st = torch.load(args.state_in)
        run.eta[run.cur].copy_(st["eta"])
        run.Tg[run.cur].copy_(st["Tg"])
        if run.compensated:
            run.Tl[run.cur].copy_(st["Tl"])
        run.clk[run.cur].copy_(st["clk"])
    run.run(args.warmup, graph=False)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run.run(args.steps, graph=False)
    e1.record()
    torch.cuda.synchronize()
    if args.state_out:
        torch.save({"eta": run.eta[run.cur].cpu(), "Tg": run.Tg[run.cur].cpu(),
                    "Tl": run.Tl[run.cur].cpu() if run.compensated else None,
                    "clk": run.clk[run.cur].cpu()}, args.state_out)
    print(json.dumps({"profile": True, "ms_per_step": e0.elapsed_time(e1) / args.steps,
                      "plan": _lib.describe_plan(solver.params)}), flush=True)


def profile_batch(args):
    """Eager launches of the batched serving kernel: the first 64 jobs of the
    serving stream admitted at once (about 2 GB resident), ``--warmup``
    launches, then ``--steps`` timed ones (each advances every job by a
    step): ``ncu -k regex:pf_batch_kernel -s <warmup> -c 1 python bench.py
    --profile-batch`` captures the first timed launch."""
    import __graft_entry__
    __graft_entry__.build()
    import ctypes
    from jax_am_gb300 import _lib
    from jax_am_gb300.serving import BatchServer
    from jax_am_gb300.workloads import serving_stream
    jobs = serving_stream(256, 50.0)[:64]
    srv = BatchServer(hbm_budget=120e9, max_jobs=64, graph_steps=16)
    for j in jobs:
        j.arrival = 0.0
        srv.submit(j)
    srv._admit(float("inf"))
    srv._encode()
    lib = _lib.load()
    tab = ctypes.c_void_p(srv.table_dev.data_ptr())
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for k in range(args.warmup):
        _lib.check(lib.pfg_batch_step(tab, k, s), "pfg_batch_step")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for k in range(args.warmup, args.warmup + args.steps):
        _lib.check(lib.pfg_batch_step(tab, k, s), "pfg_batch_step")
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # eta read and written once per cell and stored orientation (padded)
    nbytes = sum(j.cells * j._n_store * 8 for j in jobs)
    print(json.dumps({"profile_batch": True, "jobs": len(jobs), "ms_per_launch": ms,
                      "bytes_per_launch": nbytes,
                      "achieved_GBps": nbytes / (ms / 1e3) / 1e9}), flush=True)


def profile_cfd(args):
    """``--steps`` eager steps of the CFD driver case (``time_cfd``'s
    workload), each phase in an NVTX range (``AM_3d.energy``,
    ``AM_3d.flow``): ``ncu --nvtx --nvtx-include "AM_3d.flow/" ...
    python bench.py --profile-cfd --steps 3`` captures the third step's flow
    solve (the first two have no flow yet)."""
    import __graft_entry__
    __graft_entry__.build()
    from jax_am_gb300.cfd import cfd_am as G
    from jax_am_gb300.workloads import cfd_simple_case
    s = G.AM_3d(cfd_simple_case())
    for _ in range(args.steps):
        s.time_integration()
    torch.cuda.synchronize()
    print(json.dumps({"profile_cfd": True, "steps": args.steps, **s.iterations()}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-cfd", action="store_true", help="skip the implicit CFD solver leg")
    ap.add_argument("--profile-cfd", action="store_true",
                    help="eager steps of the CFD driver case for ncu (see profile_cfd)")
    ap.add_argument("--cfd-cpu", action="store_true",
                    help="also time one step of the float64 CPU oracle of the CFD solver")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the directional-solidification and 64M multi-track legs")
    ap.add_argument("--profile", action="store_true",
                    help="eager launches only (warmup then steps), for ncu captures")
    ap.add_argument("--profile-oris", type=int, default=WORKLOAD["num_oris"],
                    help="orientation count of the --profile workload")
    ap.add_argument("--state-out", default=None,
                    help="--profile: save the state after the run (eta, T, clock) to this file")
    ap.add_argument("--state-in", default=None,
                    help="--profile: start from a state saved by --state-out (a late state "
                         "with few launches before an ncu capture)")
    ap.add_argument("--profile-batch", action="store_true",
                    help="eager launches of the batched serving kernel on 64 jobs, for ncu")
    ap.add_argument("--profile-inspect", action="store_true",
                    help="the inspect_sol metrics kernels only, on the laser-track state "
                         "after --warmup steps (50 timed records each), for ncu captures")
    ap.add_argument("--profile-heat", action="store_true",
                    help="the standalone heat step only (warmup pairs, then steps launches "
                         "per axis order), for ncu captures")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.profile_inspect:
        import __graft_entry__
        __graft_entry__.build()
        from jax_am_gb300.runner import HeatPFRun
        solver, g, path, _ = build_case(WORKLOAD)
        run = HeatPFRun(solver, g, path)
        run.run(args.warmup, graph=False)
        print(json.dumps({"profile_inspect": True, **time_inspect(solver, run)}), flush=True)
        return
    if args.profile_heat:
        import __graft_entry__
        __graft_entry__.build()
        print(json.dumps({"profile_heat": True,
                          **time_heat_step(steps=args.steps, warmup=args.warmup)}), flush=True)
        return
    if args.profile_cfd:
        profile_cfd(args)
        return
    if args.profile_batch:
        profile_batch(args)
        return
    if args.profile:
        profile_run(args)
        return
    if args.impl == "reference":
        run_reference(args)
        return

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__
    __graft_entry__.build()
    from jax_am_gb300.runner import HeatPFRun
    from jax_am_gb300 import _lib

    w = WORKLOAD
    solver, g, path, poly = build_case(w)
    N = w["Nx"] * w["Ny"] * w["Nz"]
    n = w["num_oris"]
    run = HeatPFRun(solver, g, path)
    run_dt = run.dt
    # W warm-up steps: W - 1 eager steps, then the graph capture, which takes
    # one more eager step; the timed region below only replays the graph
    run.run(args.warmup - 1, graph=False)
    run.prepare()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    stream = torch.cuda.current_stream()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    launches0 = run.launches
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    run.run(args.steps, graph=True)
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    gpu_launches = run.launches - launches0
    units = N * n * args.steps
    if world > 1:
        ms, units = reduce_over_ranks(ms, units)
    ms_per_step = ms / args.steps
    value = units / (ms / 1e3)

    # roofline of the fused kernel: one launch per step
    bytes_step = algorithmic_bytes_per_step(w)
    peak, peak_kind = measured_peak()
    achieved = bytes_step / (ms_per_step / 1e3) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic_per_launch(),
                "peak_source": f"{peak_kind} hbm_gbs (MEASURED_PEAKS.json)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s", "kernel": KERNEL,
                "algorithmic_bytes_per_launch": bytes_step}

    # the inspect_sol metrics on the state just reached (the pass e2e runs every 20 steps)
    inspect = time_inspect(solver, run) if rank == 0 else None

    # the same step with a float32 temperature, for comparison: not the
    # product path (it misses the 1e-3 K parity bound over 2000 steps)
    fp32_T = None
    if rank == 0 and not args.no_configs:
        del run
        torch.cuda.empty_cache()
        run32 = HeatPFRun(solver, g, path, compensated=False)
        run32.run(args.warmup - 1, graph=False)
        ms32 = _time_run(run32, 200)
        fp32_T = {"steps": 200, "ms_per_step": ms32,
                  "roofline_frac": bytes_step / (ms32 / 1e3) / 1e9 / peak,
                  "note": "the bench step with a float32 temperature (pfg_heat_pf_step), "
                          "200 graph-replayed steps after the first W + 20: not the product "
                          "path (the compensated step is); over the 2000-step "
                          "run it differs from float64 by up to 0.42 K (latent-heat and "
                          "zeta switches taken the other way), outside the 1e-3 K bound"}
        del run32
        torch.cuda.empty_cache()

    # end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = time_e2e(solver, g, path, w, args.steps)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = time_cpu_full(w, warmup=1, steps=12, budget_s=15.0)
        cpu["small_sample"] = time_cpu_baseline(w, budget_s=5.0)
        cpu["numpy_f64"] = time_cpu_numpy(w)
    serving = None
    if rank == 0 and not args.no_serving:
        serving = time_serving()
    adjoint = None
    if rank == 0 and not args.no_adjoint:
        adjoint = time_adjoint()
    others = None
    if rank == 0 and not args.no_configs:
        others = time_other_configs(peak)
    cfd = None
    if rank == 0 and not args.no_cfd:
        cfd = time_cfd(cpu=args.cfd_cpu)
    heat = None
    if rank == 0 and not args.no_configs:
        heat = time_heat_step()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": w["name"], "grid": [w["Nx"], w["Ny"], w["Nz"]],
                       "num_oris": n, "num_grains": w["num_grains"],
                       "anisotropy": w["anisotropy"], "dt": run_dt,
                       "heat": "fused explicit FD + Gaussian 200 W", "parallelism": "replicas",
                       "l2": "inputs larger than L2 (eta 640 MB per buffer)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": gpu_launches, "clocks": clocks,
            "plan": _lib.describe_plan(solver.params),
            "serving": serving, "adjoint": adjoint, "other_configs": others,
            "cfd_am3d": cfd, "heat_step": heat, "inspect": inspect,
            "float32_temperature_step": fp32_T,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def time_e2e(solver, g, path, w, steps):
    """The same K-step solve through the public API starting from host
    memory: the initial eta and T are copied from pinned host buffers, the
    run steps on the device with the reference's inspect_sol cadence (every
    20 steps a metrics record is read back to the host), and the final eta
    and T are copied back.  Bytes per step are the totals divided by K."""
    from jax_am_gb300.runner import HeatPFRun
    N = w["Nx"] * w["Ny"] * w["Nz"]
    n = w["num_oris"]
    eta_h = solver.ini_cond().cpu().pin_memory()
    T_h = torch.full((w["Nz"] + 2, w["Ny"] + 2, w["Nx"] + 2), w["T0"]).pin_memory()
    eta_out = torch.empty_like(eta_h).pin_memory()
    T_out = torch.empty_like(T_h).pin_memory()
    Tlo_out = torch.empty_like(T_h).pin_memory()  # low part of the compensated temperature
    check_every = 20
    # the solver's resident buffers and its captured graph are set up before
    # the timed region (as a driver builds its solver before the solve)
    run = HeatPFRun(solver, g, path)
    run.prepare()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run.load(eta_h, T_h, t0=0.0)  # host -> device copies of the initial state
    d2h_diag = 0
    done = 0
    pending = None
    while done < steps:
        k = min(check_every, steps - done)
        run.run(k, graph=True)
        done += k
        # the metrics of these k steps are enqueued behind them; the previous
        # interval's are read while these steps run (no idle GPU in between)
        nxt = solver.inspect_async(run.state, run.T_ghosted, T_ghosted=True)
        d2h_diag += 8 * (6 + 64)
        if pending is not None and pending.result()["n_nonfinite"]:
            raise ValueError("non-finite eta")
        pending = nxt
    if pending.result()["n_nonfinite"]:
        raise ValueError("non-finite eta")
    eta_out.copy_(run.state, non_blocking=True)
    T_out.copy_(run.T_ghosted, non_blocking=True)
    if run.compensated:
        Tlo_out.copy_(run.Tl[run.cur], non_blocking=True)
    torch.cuda.synchronize()
    el = time.perf_counter() - t0
    h2d = eta_h.numel() * 4 + T_h.numel() * 4
    d2h = eta_out.numel() * 4 + T_out.numel() * 4 * (2 if run.compensated else 1) + d2h_diag
    return {"value": N * n * steps / el, "unit": UNIT, "h2d_bytes_per_step": h2d / steps,
            "d2h_bytes_per_step": d2h / steps, "seconds": el,
            "path": "HeatPFRun (public API) + the inspect_sol metrics (PFSolver.inspect_async) "
                    "every 20 steps, the reference drivers' check_sol_interval, each interval's "
                    "metrics read and checked while the next interval runs; state uploaded from "
                    "and returned to pinned host memory"}


if __name__ == "__main__":
    main()
