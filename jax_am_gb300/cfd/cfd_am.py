"""Drop-in for JAX-AM's implicit CFD / energy solver (``jax_am/cfd/cfd_am.py``).

``mesh3d(domain, N)`` and ``AM_3d(args)`` keep the reference's names, the
``args`` keys of its drivers (``applications/cfd/simple/cfd_params.json``,
``applications/phase_field/coupled/cfd_params.json``) and its state:
``T`` (Nx, Ny, Nz, 1), ``vel``, ``conv`` and ``grad_p0`` (Nx, Ny, Nz, 3),
``conv_T`` and ``solidID`` (Nx, Ny, Nz, 1), ``t``.  Arrays are float64 CUDA
tensors (the reference enables ``jax_enable_x64``, ``cfd_am.py:10``).

``time_integration()`` (``cfd_am.py:167-194``) runs three calls of
``libpfgb300.so``: the implicit energy solve (Newton with BiCGSTAB,
``pfg_cfd_energy_solve``), the solid-fraction update
(``pfg_cfd_solid_update``), and the flow step in the local box that follows
the beam (``pfg_cfd_flow_step``: momentum, pressure, projection and the
convective terms of the next step).  Each call returns when its iterative
solves have converged; the host reads only convergence flags.

``args['cp']`` and ``args['k']`` are ``a * clip(T, lo, hi) + b`` in every
driver of the reference; pass a ``LinearClip`` or any callable of that form
(it is probed once on NumPy arrays and rejected with ``ValueError`` if it is
not of that form).

``T`` is a new tensor after every step (so that a caller holding the
previous ``T``, as the coupled driver does with ``T_past``, keeps it); the
other fields are updated in place.
"""
import ctypes
import glob
import os
import time

import numpy as np
import torch

from .. import _lib


class LinearClip:
    """``a * clip(T, lo, hi) + b``; callable on NumPy arrays and tensors."""

    def __init__(self, a, b, lo, hi):
        self.a, self.b, self.lo, self.hi = float(a), float(b), float(lo), float(hi)

    def __call__(self, T):
        if torch.is_tensor(T):
            return self.a * torch.clamp(T, self.lo, self.hi) + self.b
        return self.a * np.clip(T, self.lo, self.hi) + self.b

    def __repr__(self):
        return f"LinearClip(a={self.a}, b={self.b}, lo={self.lo}, hi={self.hi})"


def linear_clip_params(fn, name="function"):
    """(a, b, lo, hi) of ``fn`` = a clip(T, lo, hi) + b, read from a
    ``LinearClip`` or probed on 0..20000 K; ``ValueError`` otherwise."""
    if all(hasattr(fn, k) for k in ("a", "b", "lo", "hi")):
        return float(fn.a), float(fn.b), float(fn.lo), float(fn.hi)
    T = np.arange(0.0, 20000.0, 0.25)
    y = np.asarray(fn(T), dtype=np.float64)
    if y.shape != T.shape or not np.all(np.isfinite(y)):
        raise ValueError(f"{name} must map a float64 array of temperatures to one of the same shape")
    ymin, ymax = float(y.min()), float(y.max())
    if ymax == ymin:
        return 0.0, ymin, 0.0, 1.0
    mid = np.flatnonzero((y > ymin) & (y < ymax))
    if mid.size == 0:
        raise ValueError(f"{name} is not of the form a * clip(T, lo, hi) + b")
    Tm = float(T[mid[mid.size // 2]])
    a = (float(fn(np.array([Tm + 0.125]))[0]) - float(fn(np.array([Tm - 0.125]))[0])) / 0.25
    b = float(fn(np.array([Tm]))[0]) - a * Tm
    lo, hi = sorted(((ymin - b) / a, (ymax - b) / a))
    fit = a * np.clip(T, lo, hi) + b
    if np.abs(fit - y).max() > 1e-9 * max(abs(ymin), abs(ymax)):
        raise ValueError(f"{name} is not of the form a * clip(T, lo, hi) + b")
    return a, b, lo, hi


class mesh3d:
    """``mesh3d`` (``cfd_am.py:668-745``): the box mesh of N cells over
    ``domain``.  Cell centres (``Xc``) and the neighbour list
    (``cell_conn``) are built on first use only (the solver never needs
    them: the kernels index the structured grid directly)."""

    def __init__(self, domain, N):
        self.shape = [int(n) for n in N]
        self.dim = 3
        self.domain = [float(d) for d in domain]
        self.cell_num = int(np.prod(self.shape))
        self.dX = np.array([d / n for d, n in zip(self.domain, self.shape)])
        dx, dy, dz = self.dX
        self.dV = dx * dy * dz
        self.D = np.array([-dx, dx, -dy, dy, -dz, dz])
        self.dS = np.array([-dy * dz, dy * dz, -dz * dx, dz * dx, -dx * dy, dx * dy])
        self.surf_set_num = [self.shape[1] * self.shape[2]] * 2 + \
                            [self.shape[0] * self.shape[2]] * 2 + [self.shape[0] * self.shape[1]] * 2
        self._Xc = None
        self._cell_conn = None

    @property
    def Xc(self):
        if self._Xc is None:
            c = [(n[1:] + n[:-1]) / 2 for n in
                 (np.linspace(0.0, L, k + 1) for L, k in zip(self.domain, self.shape))]
            X, Y, Z = np.meshgrid(*c, indexing="ij")
            self._Xc = np.stack((X, Y, Z), axis=3).reshape(-1, 3)
        return self._Xc

    @property
    def cell_conn(self):
        if self._cell_conn is None:
            idx = np.pad(np.arange(self.cell_num).reshape(self.shape), 1, mode="edge")
            c = idx[1:-1, 1:-1, 1:-1]
            self._cell_conn = np.stack((c, idx[:-2, 1:-1, 1:-1], idx[2:, 1:-1, 1:-1],
                                        idx[1:-1, :-2, 1:-1], idx[1:-1, 2:, 1:-1],
                                        idx[1:-1, 1:-1, :-2], idx[1:-1, 1:-1, 2:]),
                                       axis=3).reshape(-1, 7)
        return self._cell_conn

    def grid(self):
        g = _lib.CfdGrid()
        g.nx, g.ny, g.nz = self.shape
        g.dx, g.dy, g.dz = (float(v) for v in self.dX)
        g.lx, g.ly, g.lz = self.domain
        return g


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class AM_3d:
    """``AM_3d`` (``cfd_am.py:142-385``) on the GPU."""

    def __init__(self, args, device="cuda"):
        self.args = args
        self.default_args()
        self.msh = args["mesh"]
        self.msh_local = args["mesh_local"]
        self.meshio_mesh = args.get("meshio_mesh")
        self.t = 0.0
        self.device = torch.device(device)
        self._cp = linear_clip_params(args["cp"], "cp")
        self._k = linear_clip_params(args["k"], "k")
        shape = list(self.msh.shape)
        f64 = dict(dtype=torch.float64, device=self.device)
        self.T = torch.zeros(shape + [1], **f64) + float(args["T_ref"])
        self.solidID = torch.zeros(shape + [1], **f64)
        self.conv_T = torch.zeros(shape + [1], **f64)
        self.Q = torch.zeros(shape + [1], **f64)
        self.vel = torch.zeros(shape + [3], **f64)
        self.conv = torch.zeros(shape + [3], **f64)
        self.grad_p0 = torch.zeros(shape + [3], **f64)
        self._grid = self.msh.grid()
        self._grid_l = self.msh_local.grid()
        lib = _lib.load()
        nbytes = lib.pfg_cfd_workspace_bytes(ctypes.byref(self._grid), ctypes.byref(self._grid_l))
        if nbytes < 0:
            raise ValueError("bad CFD grid")
        self._ws = torch.empty(int(nbytes), dtype=torch.uint8, device=self.device)
        self.stats = _lib.CfdStats()
        if "data_dir" in args:
            self.clean_sols()

    def default_args(self):
        """``cfd_am.py:154-165``."""
        a = self.args
        a.setdefault("h", 0.0)
        a.setdefault("stefan_boltzmann", 5.67e-8)
        a.setdefault("emissivity", 0.0)
        if a["heat_source"] == 1:
            assert "phi" in a, "Body heat source is used but necessary parameter 'phi' is not set!"

    def toolpath(self, t):
        """``cfd_am.py:280-285``."""
        a = self.args
        return (a["X0"][0] + t * a["speed"], a["X0"][1], a["X0"][2],
                a["P"] * (t < a["t_OFF"]))

    def get_moving_box_boundary(self, t):
        """``cfd_am.py:237-252``: Python's round, clipped to the grid; the box
        is top-aligned along z."""
        xl, yl, zl, _ = self.toolpath(t)
        N, NL, dX = self.msh.shape, self.msh_local.shape, self.msh.dX
        x0 = round(xl / dX[0]) - round(NL[0] / 2)
        x0 = int(np.clip(x0, 0, N[0] - NL[0]))
        y0 = round(yl / dX[1]) - round(NL[1] / 2)
        y0 = int(np.clip(y0, 0, N[1] - NL[1]))
        z0 = N[2] - NL[2]
        return x0, x0 + NL[0], y0, y0 + NL[1], z0, N[2]

    def fluid_frac(self, T):
        """``cfd_am.py:360-363``."""
        Tl, Ts = self.args["Tl"], self.args["Ts"]
        return (torch.clamp(T, Ts, Tl) - Ts) / (Tl - Ts)

    def _energy_struct(self):
        a = self.args
        e = _lib.CfdEnergy()
        e.cp = _lib.LinClipC(*self._cp)
        e.k = _lib.LinClipC(*self._k)
        e.rho, e.latent_heat, e.Ts, e.Tl, e.dt = (float(a[k]) for k in
                                                 ("rho", "latent_heat", "Ts", "Tl", "dt"))
        e.T_ref, e.h_conv = float(a["T_ref"]), float(a["h"])
        e.emissivity, e.sigma = float(a["emissivity"]), float(a["stefan_boltzmann"])
        e.heat_source = int(a["heat_source"])
        e.max_newton = 50
        xl, yl, zl, P = self.toolpath(self.t)
        e.P, e.eta, e.rb = float(P), float(a["eta"]), float(a["rb"])
        e.phi = float(a.get("phi", 0.0))
        e.speed = float(a["speed"])
        e.xl, e.yl, e.zl = float(xl), float(yl), float(zl)
        e.newton_tol = 1e-5
        return e

    def time_integration(self):
        """One step (``cfd_am.py:167-194``)."""
        lib = _lib.load()
        a = self.args
        s = _stream()
        e = self._energy_struct()
        T_new = torch.empty_like(self.T)
        # NVTX ranges name the two phases for profilers (ncu --nvtx-include)
        torch.cuda.nvtx.range_push("AM_3d.energy")
        st = lib.pfg_cfd_energy_solve(ctypes.byref(self._grid), ctypes.byref(e),
                                      _lib.ptr(self.T), _lib.ptr(self.conv_T), _lib.ptr(T_new),
                                      _lib.ptr(self._ws), self._ws.numel(),
                                      ctypes.byref(self.stats), s)
        _lib.check(st, "pfg_cfd_energy_solve")
        self.T = T_new
        st = lib.pfg_cfd_solid_update(ctypes.byref(self._grid), float(a["Ts"]), float(a["Tl"]),
                                      _lib.ptr(self.T), _lib.ptr(self.solidID), s)
        _lib.check(st, "pfg_cfd_solid_update")
        torch.cuda.nvtx.range_pop()
        torch.cuda.nvtx.range_push("AM_3d.flow")
        x0, _, y0, _, z0, _ = self.get_moving_box_boundary(self.t)
        f = _lib.CfdFlow()
        f.rho, f.visco, f.dt = float(a["rho"]), float(a["visco"]), float(a["dt"])
        f.marangoni, f.Ts, f.Tl = float(a["Marangoni"]), float(a["Ts"]), float(a["Tl"])
        f.x0, f.y0, f.z0 = x0, y0, z0
        st = lib.pfg_cfd_flow_step(ctypes.byref(self._grid), ctypes.byref(self._grid_l),
                                   ctypes.byref(f), _lib.ptr(self.T), _lib.ptr(self.vel),
                                   _lib.ptr(self.conv), _lib.ptr(self.grad_p0),
                                   _lib.ptr(self.conv_T), _lib.ptr(self._ws), self._ws.numel(),
                                   ctypes.byref(self.stats), s)
        torch.cuda.nvtx.range_pop()
        _lib.check(st, "pfg_cfd_flow_step")
        self.t += a["dt"]

    def iterations(self):
        """Iteration counts of the last step: Newton steps, BiCGSTAB
        iterations of the energy solve (summed), of the three momentum
        solves and of the pressure solve."""
        s = self.stats
        return dict(newton=s.newton_iters, energy_krylov=s.energy_krylov,
                    momentum_krylov=list(s.momentum_krylov), pressure_krylov=s.pressure_krylov)

    def clean_sols(self):
        """``cfd_am.py:366-371``."""
        folder = os.path.join(self.args["data_dir"], "vtk/cfd/sols")
        os.makedirs(folder, exist_ok=True)
        for f in glob.glob(folder + "/*"):
            os.remove(f)

    def inspect_sol(self, step, num_steps):
        """``cfd_am.py:373-377``."""
        print(f"\nstep {step} of {num_steps}, unix timestamp = {time.time()}")
        vmax = float(torch.linalg.norm(self.vel, dim=3).max())
        print(f"T_max:{float(self.T.max())}, vmax:{vmax}\n")
        if not bool(torch.isfinite(self.T).all()):
            raise ValueError("Found np.inf or np.nan in T0 - stop the program")

    def write_sols(self, step):
        """``cfd_am.py:379-385``: T, vel and solidID as float32 cell data of a
        VTU file (written by ``phase_field.vtu``; the reference uses meshio)."""
        from ..phase_field.vtu import write_vtu
        print("\nWrite CFD sols to file...\n")
        step = step // self.args["write_sol_interval"]
        path = os.path.join(self.args["data_dir"], f"vtk/cfd/sols/u{step:03d}.vtu")
        # VTU cells are x-fastest; the solver's arrays are z-fastest
        def xfast(a):
            return a.permute(2, 1, 0, 3).reshape(-1, a.shape[3]).float()
        write_vtu(path, tuple(self.msh.shape), tuple(float(v) for v in self.msh.dX),
                  {"T": xfast(self.T), "vel": xfast(self.vel), "solidID": xfast(self.solidID)})
        return path
