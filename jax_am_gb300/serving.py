"""Continuous-batching serving of many directional-solidification solves.

The reference solves one polycrystal per Python driver process, one kernel
dispatch per step (``applications/phase_field/solidification/example.py:
63-90``).  ``BatchServer`` keeps many jobs resident in HBM at once and
advances all of them together:

* **Admission.**  Submitted jobs wait in a FIFO queue until their arrival
  time has passed, a table slot is free and their memory (the eta double
  buffer) fits under the HBM budget; then they are admitted, mid-flight of
  the others.
* **Packed job table.**  Every active job has a record in a device table
  (``pfg_batch_encode``): its grid, parameters, buffers and step counters.
  One ``pfg_batch_step`` launch advances every active job by one step (a
  fixed grid of persistent CTAs walks the tiles of all jobs).
* **Graph replay.**  A CUDA graph of ``graph_steps`` launches plus one
  ``pfg_batch_advance`` (which moves every job's step counter on the device)
  is captured once and replayed; the table is rewritten only when jobs are
  admitted or retired.
* **Retirement.**  A job that has taken its steps leaves the table; its final
  state is ``eta[steps % 2]``; its memory returns to the budget.

Latency of a job = completion time - arrival time (queueing included).
"""
import ctypes
import time
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch

from . import _lib
from .phase_field.allen_cahn import PFSolver, Quench, make_pf_params


@dataclass
class Job:
    """One directional-solidification solve: ``steps`` explicit steps of
    ``dt`` under the moving gradient ``quench``, from one-hot eta (or
    ``eta0``) on ``polycrystal``."""
    pf_args: dict
    polycrystal: object
    quench: Quench
    steps: int
    dt: float
    arrival: float = 0.0
    eta0: Optional[torch.Tensor] = None
    t0: float = 0.0
    # filled in by the server
    id: int = -1
    admitted: float = float("nan")
    finished: float = float("nan")
    result: Optional[torch.Tensor] = None
    _params: object = field(default=None, repr=False)
    _eta: Optional[list] = field(default=None, repr=False)  # the two eta buffers
    _base: int = 0
    _n_store: int = 0  # orientations per cell as stored on the device (padded)

    @property
    def cells(self):
        return int(self.pf_args["Nx"]) * int(self.pf_args["Ny"]) * int(self.pf_args["Nz"])

    @property
    def num_oris(self):
        return int(self.pf_args["num_oris"])

    @property
    def nbytes(self):
        """HBM held while active: the float32 eta double buffer."""
        return 2 * self.cells * (self._n_store or self.num_oris) * 4

    @property
    def latency(self):
        return self.finished - self.arrival

    def fresh(self):
        """The same job (inputs shared) with no run state."""
        return Job(self.pf_args, self.polycrystal, self.quench, self.steps, self.dt,
                   arrival=self.arrival, eta0=self.eta0, t0=self.t0)


class _PaddedDirections:
    """A polycrystal view whose orientation list is padded with zero
    directions to ``n_store`` entries."""

    def __init__(self, polycrystal, n_store):
        self.mesh_h_xyz = polycrystal.mesh_h_xyz
        d = np.asarray(polycrystal.unique_grain_directions, dtype=np.float64)
        pad = np.zeros((3, n_store, 3))
        pad[:, : d.shape[1]] = d
        self.unique_grain_directions = pad


def one_hot(polycrystal, N, n):
    inds = torch.as_tensor(np.asarray(polycrystal.cell_ori_inds), dtype=torch.int64, device="cuda")
    eta = torch.zeros((N, n), dtype=torch.float32, device="cuda")
    eta.scatter_(1, inds.view(-1, 1), 1.0)
    return eta


class BatchServer:
    """Continuously batched solver for many independent jobs on one GPU."""

    def __init__(self, hbm_budget=120e9, max_jobs=256, graph_steps=16, pad_oris=True):
        self.lib = _lib.load()
        # Store every job with its orientation count rounded up to a multiple
        # of 4 (extra orientations are zero and stay exactly zero: their
        # Laplacian and bulk terms vanish), so that every cell is a whole
        # number of 16-byte vectors and the batch kernel's vector path runs.
        self.pad_oris = bool(pad_oris)
        self.hbm_budget = float(hbm_budget)
        self.max_jobs = int(max_jobs)
        self.graph_steps = int(graph_steps)
        self.table_bytes = int(self.lib.pfg_batch_table_bytes(self.max_jobs))
        self.table_dev = torch.zeros(self.table_bytes, dtype=torch.uint8, device="cuda")
        self.table_host = torch.zeros(self.table_bytes, dtype=torch.uint8).pin_memory()
        self.queue = []
        self.active = []
        self.done = []
        self.used_bytes = 0
        self.peak_bytes = 0
        self.launches = 0
        self._graph = None
        self._next_id = 0
        self._inflight = []  # events of replays the host has queued ahead of the GPU
        self.max_ahead = 2

    # ---- submission and admission -------------------------------------------
    def submit(self, job: Job):
        n = job.num_oris
        n_store = 4 * ((n + 3) // 4) if self.pad_oris else n
        if n_store > _lib.MAX_ORIS:
            n_store = n
        job._n_store = n_store
        if job.nbytes > self.hbm_budget:
            raise ValueError(f"job needs {job.nbytes} bytes, more than the HBM budget")
        job.id = self._next_id
        self._next_id += 1
        if n_store == n:
            job._params = make_pf_params(job.pf_args, job.polycrystal)
        else:
            job._params = make_pf_params(dict(job.pf_args, num_oris=n_store),
                                         _PaddedDirections(job.polycrystal, n_store))
        self.queue.append(job)
        return job.id

    def _admit(self, now):
        admitted = False
        while (self.queue and self.queue[0].arrival <= now and len(self.active) < self.max_jobs
               and self.used_bytes + self.queue[0].nbytes <= self.hbm_budget):
            job = self.queue.pop(0)
            N, n, ns = job.cells, job.num_oris, job._n_store
            # two allocations: a (2, N, n) tensor would put the second buffer
            # at N*n*4 bytes, not 16-byte aligned for odd N*n
            job._eta = [torch.empty((N, ns), dtype=torch.float32, device="cuda") for _ in range(2)]
            src = job.eta0 if job.eta0 is not None else one_hot(job.polycrystal, N, n)
            src = torch.as_tensor(src, dtype=torch.float32, device="cuda").reshape(N, n)
            if ns == n:
                job._eta[0].copy_(src)
            else:
                job._eta[0].zero_()
                job._eta[0][:, :n].copy_(src)
            job._base = 0
            job.admitted = now
            self.used_bytes += job.nbytes
            self.peak_bytes = max(self.peak_bytes, self.used_bytes)
            self.active.append(job)
            admitted = True
        return admitted

    # ---- device table and graph ---------------------------------------------
    def _encode(self):
        jobs = (_lib.BatchJob * max(1, len(self.active)))()
        for i, job in enumerate(self.active):
            b = jobs[i]
            b.params = job._params
            b.quench = job.quench.struct(job._params.h_z)
            b.eta[0] = job._eta[0].data_ptr()
            b.eta[1] = job._eta[1].data_ptr()
            b.t0 = job.t0
            b.dt = job.dt
            b.base_step = job._base
            b.target_steps = job.steps
        total = ctypes.c_int64(0)
        torch.cuda.current_stream().synchronize()  # the host buffer may still be in flight
        st = self.lib.pfg_batch_encode(jobs, len(self.active),
                                       ctypes.c_void_p(self.table_host.data_ptr()),
                                       self.table_bytes, ctypes.byref(total))
        _lib.check(st, "pfg_batch_encode")
        self.table_dev.copy_(self.table_host, non_blocking=True)
        return int(total.value)

    def _launch_all(self):
        s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        tab = ctypes.c_void_p(self.table_dev.data_ptr())
        for k in range(self.graph_steps):
            _lib.check(self.lib.pfg_batch_step(tab, k, s), "pfg_batch_step")
        _lib.check(self.lib.pfg_batch_advance(tab, self.graph_steps, s), "pfg_batch_advance")

    def _replay(self, use_graph=True):
        if not use_graph:
            self._launch_all()
        else:
            if self._graph is None:
                # configure the kernels (shared-memory attribute) outside the capture
                self.lib.pfg_batch_step(ctypes.c_void_p(self.table_dev.data_ptr()), 1 << 30,
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._launch_all()
                self._graph = g
            self._graph.replay()
        self.launches += self.graph_steps + 1
        for job in self.active:
            job._base += self.graph_steps

    # ---- serving loop -----------------------------------------------------------
    def run(self, use_graph=True, clock=time.perf_counter, realtime=True):
        """Serve until every submitted job is done.  With ``realtime`` the
        jobs' ``arrival`` times are honoured against the wall clock;
        otherwise every job is available at once.  Returns a summary dict."""
        self.queue.sort(key=lambda j: j.arrival)
        start = clock()
        dirty = True
        while self.queue or self.active:
            now = clock() - start if realtime else float("inf")
            if self._admit(now):
                dirty = True
            if not self.active:
                if self.queue and realtime:
                    wait = self.queue[0].arrival - (clock() - start)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                continue
            if dirty:
                self._encode()
                dirty = False
            # bound how far the host runs ahead, so that new arrivals are
            # admitted within a couple of replays of their arrival
            while len(self._inflight) >= self.max_ahead:
                self._inflight.pop(0).synchronize()
            self._replay(use_graph)
            ev = torch.cuda.Event()
            ev.record()
            self._inflight.append(ev)
            finished = [j for j in self.active if j._base >= j.steps]
            if finished:
                torch.cuda.current_stream().synchronize()
                t_done = clock() - start
                self._inflight.clear()
                for job in finished:
                    job.finished = t_done
                    job.result = job._eta[job.steps & 1][:, : job.num_oris].clone(
                        memory_format=torch.contiguous_format)
                    job._eta = None
                    self.active.remove(job)
                    self.used_bytes -= job.nbytes
                    self.done.append(job)
                dirty = True
        torch.cuda.synchronize()
        return summarize(self.done, clock() - start)


def summarize(jobs, wall):
    if not jobs:
        return {"jobs": 0}
    lat = np.array([j.latency for j in jobs])
    first = min(j.arrival for j in jobs)
    last = max(j.finished for j in jobs)
    return {
        "jobs": len(jobs),
        "jobs_per_s": len(jobs) / max(last - first, 1e-9),
        "p50_s": float(np.percentile(lat, 50)),
        "p99_s": float(np.percentile(lat, 99)),
        "mean_s": float(lat.mean()),
        "wall_s": wall,
        "cell_ori_updates": float(sum(j.cells * j.num_oris * j.steps for j in jobs)),
    }


def run_sequential(jobs, clock=time.perf_counter, realtime=True):
    """The plain baseline: jobs in arrival order, one at a time, each stepped
    from Python through ``PFSolver.stepper`` as the reference's driver loop
    does (one dispatch per step).  Returns the same summary as the server."""
    jobs = sorted(jobs, key=lambda j: j.arrival)
    start = clock()
    for job in jobs:
        if realtime:
            while clock() - start < job.arrival:
                time.sleep(min(job.arrival - (clock() - start), 0.01))
        solver = PFSolver(job.pf_args, job.polycrystal)
        eta = job.eta0 if job.eta0 is not None else solver.ini_cond()
        state = (eta, job.t0)
        t = job.t0
        job.admitted = clock() - start
        for _ in range(job.steps):
            t_next = t + job.dt
            state, _ = solver.stepper(state, t_next, [job.quench])
            t = t_next
        torch.cuda.current_stream().synchronize()
        job.finished = clock() - start
        job.result = state[0]
    return summarize(jobs, clock() - start)


def run_sequential_resident(jobs, clock=time.perf_counter, realtime=True):
    """The best plain baseline: jobs in arrival order, one at a time, each as
    a resident run (``runner.QuenchRun``: state in HBM, the moving gradient
    evaluated in the step kernel, a captured CUDA graph of 20 steps
    replayed), so that a job costs its kernel launches and one graph capture
    rather than one Python dispatch per step.  Returns the same summary as
    the server."""
    from .runner import QuenchRun
    jobs = sorted(jobs, key=lambda j: j.arrival)
    start = clock()
    for job in jobs:
        if realtime:
            while clock() - start < job.arrival:
                time.sleep(min(job.arrival - (clock() - start), 0.01))
        solver = PFSolver(job.pf_args, job.polycrystal)
        job.admitted = clock() - start
        run = QuenchRun(solver, job.quench, job.dt, eta0=job.eta0, t0=job.t0)
        run.run(job.steps)
        torch.cuda.current_stream().synchronize()
        job.finished = clock() - start
        job.result = run.state
    return summarize(jobs, clock() - start)

