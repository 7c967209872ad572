"""Resident, graph-replayed time stepping on one GPU.

The reference drives every step from a Python loop with one host-to-device
dispatch per step (``applications/phase_field/solidification/example.py:83``,
``applications/cfd/gamma/example.py:111-113``).  Here the state stays in HBM
in double buffers, the simulation clock lives on the device (each step reads
one clock and writes the other), and a CUDA graph of an even number of steps
is captured once and replayed, so a run of K steps costs K kernel launches
from one graph launch per replay and no host round trip.

* ``QuenchRun``: phase field under the moving linear gradient of the
  directional-solidification driver, T evaluated inside the kernel.
* ``HeatPFRun``: the fused heat + phase-field step with a tool-path laser.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .cfd.gamma import make_heat_params, stable_dt as heat_stable_dt
from .phase_field.allen_cahn import PFSolver, Quench


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class _GraphRun:
    graph_steps = 20  # steps per captured graph (even: buffers return to their start)

    def __init__(self):
        self.cur = 0
        self.clk = torch.zeros((2, 2), dtype=torch.int64, device="cuda")
        self._graph = None
        self._graph_src = 0
        self.launches = 0

    def _launch(self, src):
        raise NotImplementedError

    def step(self):
        """One eager step."""
        self._launch(self.cur)
        self.cur ^= 1

    def _capture(self):
        # one eager step first: kernel attributes are configured outside the capture
        self.step()
        g = torch.cuda.CUDAGraph()
        start, counted = self.cur, self.launches
        with torch.cuda.graph(g):
            src = start
            for _ in range(self.graph_steps):
                self._launch(src)
                src ^= 1
        self.launches = counted  # captured launches run at replay, counted there
        self._graph = g
        self._graph_src = start  # the buffer the graph reads first (and ends in)
        return 1

    def prepare(self):
        """Capture the replayed graph now, so that a later ``run`` only
        replays it.  The capture takes one eager step (kernel attributes are
        set outside the capture); returns the number of steps taken (1, or 0
        when the graph exists already)."""
        if self._graph is not None:
            return 0
        return self._capture()

    def run(self, steps, graph=True):
        """Advance ``steps`` steps (graph replay when ``graph``).  The graph
        reads the buffer it was captured from, so after an odd number of
        eager steps one more eager step comes first."""
        done = 0
        if graph and steps >= self.graph_steps:
            if self._graph is None:
                done += self._capture()
            if self.cur != self._graph_src and steps - done > self.graph_steps:
                self.step()
                done += 1
            while self.cur == self._graph_src and steps - done >= self.graph_steps:
                self._graph.replay()
                self.launches += self.graph_steps
                done += self.graph_steps
        while done < steps:
            self.step()
            done += 1
        return self

    def set_time(self, t, step=0):
        c = self.clk[self.cur]
        c[1] = int(step)
        c[0:1].view(torch.float64)[0] = float(t)

    @property
    def t(self):
        return float(self.clk[self.cur][0:1].view(torch.float64).item())

    @property
    def steps_taken(self):
        return int(self.clk[self.cur][1].item())


class QuenchRun(_GraphRun):
    """Phase field under a ``Quench`` gradient, state resident on the GPU."""

    def __init__(self, solver: PFSolver, quench: Quench, dt, eta0=None, t0=0.0):
        super().__init__()
        self.solver = solver
        self.quench = quench
        self.q = quench.struct(solver.params.h_z)
        self.dt = float(dt)
        e0 = solver.ini_cond() if eta0 is None else eta0
        self.eta = [e0.contiguous().clone(), torch.empty_like(e0)]
        self.set_time(t0)

    def _launch(self, src):
        s = self.solver
        st = s.lib.pfg_pf_step_quench(ctypes.byref(s.params), ctypes.byref(self.q),
                                       _lib.ptr(self.eta[src]), _lib.ptr(self.eta[src ^ 1]),
                                       _lib.ptr(self.clk[src]), _lib.ptr(self.clk[src ^ 1]),
                                       self.dt, _stream())
        _lib.check(st, "pfg_pf_step_quench")
        self.launches += 1

    @property
    def state(self):
        return self.eta[self.cur]


class PointSourceRun(_GraphRun):
    """Phase field under a moving point source (``PointSource``), state
    resident on the GPU; the device step count selects the source record, so
    a replayed graph follows the tool path with no host work per step."""

    def __init__(self, solver: PFSolver, source, dt, eta0=None, t0=0.0, step0=0):
        super().__init__()
        self.solver = solver
        self.source = source
        self.src = source.struct(solver.params)
        self.dt = float(dt)
        e0 = solver.ini_cond() if eta0 is None else eta0
        self.eta = [e0.contiguous().clone(), torch.empty_like(e0)]
        self.set_time(t0, step0)

    def _launch(self, src):
        s = self.solver
        st = s.lib.pfg_pf_step_point_source(ctypes.byref(s.params), ctypes.byref(self.src),
                                             _lib.ptr(self.eta[src]), _lib.ptr(self.eta[src ^ 1]),
                                             _lib.ptr(self.clk[src]), _lib.ptr(self.clk[src ^ 1]),
                                             self.dt, _stream())
        _lib.check(st, "pfg_pf_step_point_source")
        self.launches += 1

    @property
    def state(self):
        return self.eta[self.cur]

    def T(self):
        """(N, 1) T of the next step (for inspect_sol / write_sols)."""
        return self.source.T(self.solver, step=self.steps_taken)


def single_track(x_start, y, speed, power, t_end, t_start=0.0):
    """Tool path of one straight track along +x."""
    return [(t_start, t_end, x_start, y, x_start + speed * (t_end - t_start), y, power)]


def raster(tracks, speed, power, x_start, x_end, t_start=0.0):
    """Sequential tracks along +x at the given y positions, one after the
    other, as the reference's multi-track raster (``applications/phase_field/
    multi_scan/pf_params.yaml:84-88``) scans them."""
    segs, t = [], t_start
    for y in tracks:
        dur = (x_end - x_start) / speed
        segs.append((t, t + dur, x_start, y, x_end, y, power))
        t += dur
    return segs


class HeatPFRun(_GraphRun):
    """Fused explicit heat + phase-field run with a tool-path laser.

    ``compensated`` (default: wherever the step kernels support it: the
    cell-per-lane kernel (num_oris = 20) and the TMA-fed kernel) keeps the
    temperature as two float32 fields whose sum is T
    (``pfg_heat_pf_step_comp``): a 2000-step laser run then tracks a
    float64 run to ~1e-6 K instead of ~1e-2 K (plus O(1 K) where a cell near
    the latent-heat or liquidus switch takes the other branch).
    ``T_ghosted`` is the float32 temperature (the high part);
    ``T_ghosted_f64`` the full value."""

    def __init__(self, solver: PFSolver, gamma_args, path, dt=None, eta0=None, T_init=None,
                 t0=0.0, compensated=None):
        super().__init__()
        self.solver = solver
        p = solver.params
        self.heat = make_heat_params(gamma_args, p.nx, p.ny, p.nz, p.h_x, p.h_y, p.h_z,
                                     layout=_lib.LAYOUT_ZYX, path=path)
        if dt is None:
            dt = min(solver.stable_dt(), heat_stable_dt(gamma_args, p.h_x, p.h_y, p.h_z))
        self.dt = float(dt)
        e0 = solver.ini_cond() if eta0 is None else eta0
        self.eta = [e0.contiguous().clone(), torch.empty_like(e0)]
        shape = (p.nz + 2, p.ny + 2, p.nx + 2)
        if T_init is None:
            Tg = torch.full(shape, float(gamma_args["T0"]), dtype=torch.float32, device="cuda")
        else:
            Tg = T_init.to("cuda", torch.float32).reshape(shape).contiguous()
        self.Tg = [Tg.clone(), Tg.clone()]  # edge ghosts stay equal in both buffers
        supported = solver.lib.pfg_heat_pf_step_comp_supported(ctypes.byref(p)) == 1
        if compensated is None:
            compensated = supported
        elif compensated and not supported:
            raise ValueError("the compensated fused step needs the cell-per-lane or the "
                             "TMA-fed step kernel (num_oris = 20, or a multiple of 4, or even "
                             "with even Nx and Neumann x faces)")
        self.compensated = bool(compensated)
        self.Tl = [torch.zeros_like(Tg), torch.zeros_like(Tg)] if self.compensated else None
        self.set_time(t0)

    def _launch(self, src):
        s = self.solver
        if self.compensated:
            st = s.lib.pfg_heat_pf_step_comp(
                ctypes.byref(s.params), ctypes.byref(self.heat), _lib.ptr(self.eta[src]),
                _lib.ptr(self.eta[src ^ 1]), _lib.ptr(self.Tg[src]), _lib.ptr(self.Tl[src]),
                _lib.ptr(self.Tg[src ^ 1]), _lib.ptr(self.Tl[src ^ 1]), _lib.ptr(self.clk[src]),
                _lib.ptr(self.clk[src ^ 1]), self.dt, _stream())
            _lib.check(st, "pfg_heat_pf_step_comp")
        else:
            st = s.lib.pfg_heat_pf_step(ctypes.byref(s.params), ctypes.byref(self.heat),
                                         _lib.ptr(self.eta[src]), _lib.ptr(self.eta[src ^ 1]),
                                         _lib.ptr(self.Tg[src]), _lib.ptr(self.Tg[src ^ 1]),
                                         _lib.ptr(self.clk[src]), _lib.ptr(self.clk[src ^ 1]),
                                         self.dt, _stream())
            _lib.check(st, "pfg_heat_pf_step")
        self.launches += 1

    @property
    def state(self):
        return self.eta[self.cur]

    def load(self, eta, T_init=None, t0=0.0):
        """Copy a new state into the resident buffers (asynchronously on the
        current stream; host tensors should be pinned): eta into the buffer
        the next step reads, the ghosted T into both T buffers, the clock to
        ``t0``.  A captured graph keeps its buffers, so it replays the new
        state."""
        p = self.solver.params
        self.eta[self.cur].copy_(eta.reshape(self.eta[self.cur].shape), non_blocking=True)
        if T_init is not None:
            shape = (p.nz + 2, p.ny + 2, p.nx + 2)
            self.Tg[self.cur].copy_(T_init.reshape(shape), non_blocking=True)
            self.Tg[self.cur ^ 1].copy_(self.Tg[self.cur], non_blocking=True)
            if self.compensated:
                self.Tl[0].zero_()
                self.Tl[1].zero_()
        self.set_time(t0)
        return self

    @property
    def T_ghosted(self):
        return self.Tg[self.cur]

    @property
    def T_ghosted_f64(self):
        """The ghosted temperature in float64 (high + low part when compensated)."""
        T = self.Tg[self.cur].double()
        return T + self.Tl[self.cur].double() if self.compensated else T

    @property
    def T_cells(self):
        """(N, 1) interior temperature in the phase-field cell order."""
        return self.Tg[self.cur][1:-1, 1:-1, 1:-1].reshape(-1, 1)
