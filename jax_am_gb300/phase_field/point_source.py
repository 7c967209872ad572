"""Moving point-source temperature (Rosenthal solution) evaluated inside the
phase-field step.

The reference's laser drivers compute an analytic temperature on the host
side of every step and hand it to ``PFSolver.stepper``:

* ``applications/phase_field/simple/example.py:21-37``: a source moving
  along x at constant power and speed from 0.2 domain_x, on the top face at
  mid-width;
* ``applications/phase_field/simple/example_grf.py:21-46``: the same with the
  power and speed ramped linearly over t_OFF (Q 35 -> 15 W, speed 0.5 -> 1.5
  times the average) and the position advanced by the mean speed;
* ``applications/phase_field/multi_scan/example.py:33-84``: a source following
  a raster tool path sampled at dt (``read_path``), with the exponent's
  projection along the moving direction and T clipped at 2000 K.

Here the source's state for every step is one record of a device table
(``pfg_point_source``); the step kernel evaluates T per cell from the record
of the step it is taking (``pfg_pf_step_point_source``), so no temperature
array is ever written.  ``PointSource.T`` produces the same T as an array
when a driver wants it (``inspect_sol``, ``write_sols``).
"""
import ctypes

import numpy as np
import torch

from .. import _lib

# material constants of the reference drivers (simple/example.py:26-28)
Q_DEFAULT = 25.0
ALPHA = 5.2e-6
KAPPA = 27.0


def read_path(pf_args):
    """The raster tool path sampled at dt (``multi_scan/example.py:52-84``):
    times, positions, power switch and unit moving direction per step."""
    x_c = pf_args["laser_path"]["x_pos"]
    y_c = pf_args["laser_path"]["y_pos"]
    z_c = pf_args["laser_path"]["z_pos"]
    power = pf_args["laser_path"]["switch"][:-1]
    ts, xs, ys, zs, ps, dirs = [], [], [], [], [], []
    t_pre = 0.0
    for i in range(len(x_c) - 1):
        d = np.array([x_c[i + 1] - x_c[i], y_c[i + 1] - y_c[i], z_c[i + 1] - z_c[i]])
        dist = np.linalg.norm(d)
        unit = d / dist
        travel = dist / pf_args["vel"]
        t_seg = np.arange(t_pre, t_pre + travel, pf_args["dt"])
        m = len(t_seg)
        ts.append(t_seg)
        xs.append(np.linspace(x_c[i], x_c[i + 1], m))
        ys.append(np.linspace(y_c[i], y_c[i + 1], m))
        zs.append(np.linspace(z_c[i], z_c[i + 1], m))
        ps.append(np.linspace(power[i], power[i], m))
        dirs.append(np.repeat(unit[None, :], m, axis=0))
        t_pre = t_pre + travel
    return (np.hstack(ts), np.hstack(xs), np.hstack(ys), np.hstack(zs), np.hstack(ps),
            np.vstack(dirs))


class PointSource:
    """A moving point source: one record (time, position, direction, power,
    speed) per step, resident on the GPU.

    Pass it in place of the T array in ``PFSolver.stepper``'s ``ode_params``
    (the record for the step is the one whose time is nearest to ``t_prev``),
    or run it with ``runner.PointSourceRun`` (the step count on the device
    selects the record)."""

    def __init__(self, ts, xs, ys, zs, dirs, Q, vel, T_ambient, alpha=ALPHA, kappa=KAPPA,
                 T_clip=np.inf, cell_size=None, first_centre=None):
        ts = np.atleast_1d(np.asarray(ts, dtype=np.float64))
        K = len(ts)
        rec = np.zeros(K, dtype=[("t", "<f8"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4"),
                                 ("ux", "<f4"), ("uy", "<f4"), ("uz", "<f4"), ("Q", "<f4"),
                                 ("vel", "<f4")])
        assert rec.dtype.itemsize == ctypes.sizeof(_lib.PointSourceRecord)
        dirs = np.broadcast_to(np.asarray(dirs, dtype=np.float64), (K, 3))
        rec["t"] = ts
        rec["x"] = np.broadcast_to(xs, (K,))
        rec["y"] = np.broadcast_to(ys, (K,))
        rec["z"] = np.broadcast_to(zs, (K,))
        rec["ux"], rec["uy"], rec["uz"] = dirs[:, 0], dirs[:, 1], dirs[:, 2]
        rec["Q"] = np.broadcast_to(Q, (K,))
        rec["vel"] = np.broadcast_to(vel, (K,))
        self.records = rec
        self.ts = ts
        self.table = torch.from_numpy(rec.view(np.uint8).copy()).to("cuda")
        self.T_ambient, self.alpha, self.kappa, self.T_clip = T_ambient, alpha, kappa, T_clip
        self.cell_size = cell_size
        self.first_centre = first_centre

    # ---- the reference drivers' sources ---------------------------------------
    @classmethod
    def simple(cls, pf_args, ts):
        """``simple/example.py:21-37`` at the step times ``ts``."""
        ts = np.asarray(ts, dtype=np.float64)
        x0 = 0.2 * pf_args["domain_x"]
        vel = 0.6 * pf_args["domain_x"] / pf_args["t_OFF"]
        return cls(ts, x0 + vel * ts, 0.5 * pf_args["domain_y"], pf_args["domain_z"], (1, 0, 0),
                   Q_DEFAULT, vel, pf_args["T_ambient"])

    @classmethod
    def ramped(cls, pf_args, ts):
        """``simple/example_grf.py:21-46``: power and speed ramped over t_OFF."""
        ts = np.asarray(ts, dtype=np.float64)
        x0 = 0.2 * pf_args["domain_x"]
        vel_avg = 0.6 * pf_args["domain_x"] / pf_args["t_OFF"]
        Q = ts / pf_args["t_OFF"] * (15.0 - 35.0) + 35.0
        vel_min, vel_max = 0.5 * vel_avg, 1.5 * vel_avg
        vel = ts / pf_args["t_OFF"] * (vel_max - vel_min) + vel_min
        return cls(ts, x0 + (vel + vel_min) / 2.0 * ts, 0.5 * pf_args["domain_y"],
                   pf_args["domain_z"], (1, 0, 0), Q, vel, pf_args["T_ambient"])

    @classmethod
    def raster(cls, pf_args):
        """``multi_scan/example.py:33-84``: the sampled tool path, constant
        speed ``vel``, T clipped at 2000 K (the power switch does not enter T
        in the reference)."""
        ts, xs, ys, zs, ps, dirs = read_path(pf_args)
        return cls(ts, xs, ys, zs, dirs, Q_DEFAULT, pf_args["vel"], pf_args["T_ambient"],
                   T_clip=2000.0)

    # ---- device side --------------------------------------------------------
    def struct(self, params):
        """The ``pfg_point_sources`` struct for a grid with ``params``."""
        hx, hy, hz = (float(v) for v in (self.cell_size or (params.h_x, params.h_y, params.h_z)))
        x0, y0, z0 = self.first_centre or (0.5 * hx, 0.5 * hy, 0.5 * hz)
        return _lib.PointSources(float(self.T_ambient), float(self.alpha), float(self.kappa),
                                 float(self.T_clip), float(x0), float(y0), float(z0), 0,
                                 self.table.data_ptr(), len(self.ts))

    def index_at(self, t):
        """Record whose time is nearest to ``t``."""
        return int(np.argmin(np.abs(self.ts - float(t))))

    def T(self, solver, step=None, t=None):
        """(N, 1) float32 CUDA T of the step starting at record ``step`` (or
        at the record nearest ``t``), as the step kernel evaluates it."""
        k = self.index_at(t) if step is None else int(step)
        clk = torch.zeros(2, dtype=torch.int64, device="cuda")
        clk[1] = k
        out = torch.empty((solver.N, 1), dtype=torch.float32, device="cuda")
        src = self.struct(solver.params)
        st = solver.lib.pfg_point_source_T(ctypes.byref(solver.params), ctypes.byref(src),
                                           _lib.ptr(clk), _lib.ptr(out),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        _lib.check(st, "pfg_point_source_T")
        return out
