"""Drop-in for JAX-AM's phase-field solver (``jax_am/phase_field/allen_cahn.py``).

``PFSolver(pf_args, polycrystal)`` keeps the reference's constructor,
``ini_cond``, ``stepper``, ``inspect_sol``, ``write_sols`` and ``clean_sols``.
Arrays are PyTorch CUDA tensors (float32); NumPy inputs are copied to the
GPU.  Every step runs in ``libpfgb300.so`` (hand-written sm_103a kernels);
there is no CPU path.

Extensions, all off by default so the defaults reproduce the reference:
``pf_args['bc']`` ("neumann" or "periodic", per axis or for all),
``pf_args['force_liquid_zero']`` with ``pf_args['liquid_shift']`` (the
reference's ``get_force_eta_fn``, whose call is commented out of its
``stepper``), and a ``Quench`` temperature source evaluated inside the kernel.
"""
import ctypes
import glob
import os
import time

import numpy as np
import torch

from .. import _lib
from .coupling import InterpolatedT
from .point_source import PointSource

_BC = {"neumann": _lib.BC_NEUMANN, "periodic": _lib.BC_PERIODIC}


def _bc_codes(bc):
    if bc is None:
        bc = "neumann"
    if isinstance(bc, str):
        bc = (bc,) * 3
    if len(bc) != 3 or any(b not in _BC for b in bc):
        raise ValueError(f"bc must be 'neumann'/'periodic' or a tuple of three, got {bc!r}")
    return tuple(_BC[b] for b in bc)


def make_pf_params(pf_args, polycrystal):
    """Fill the C ``pfg_pf_params`` struct from the reference ``pf_args`` dict
    (``pf_params.yaml`` keys) and a polycrystal (``mesh_h_xyz``,
    ``unique_grain_directions``)."""
    p = _lib.PfParams()
    n = int(pf_args["num_oris"])
    if not 1 <= n <= _lib.MAX_ORIS:
        raise ValueError(f"num_oris = {n} is outside [1, {_lib.MAX_ORIS}]")
    p.nx, p.ny, p.nz = int(pf_args["Nx"]), int(pf_args["Ny"]), int(pf_args["Nz"])
    p.num_oris = n
    p.h_x, p.h_y, p.h_z = (float(v) for v in polycrystal.mesh_h_xyz)
    for key in ("T_liquidus", "gas_const", "Qg", "L0", "kappa_g", "m_g", "anisotropy", "ad_hoc"):
        setattr(p, key, float(pf_args[key]))
    p.bc_x, p.bc_y, p.bc_z = _bc_codes(pf_args.get("bc"))
    p.force_liquid_zero = int(bool(pf_args.get("force_liquid_zero", False)))
    p.liquid_shift = float(pf_args.get("liquid_shift", 1.0))
    dirs = np.asarray(polycrystal.unique_grain_directions, dtype=np.float64)
    if dirs.shape != (3, n, 3):
        raise ValueError(f"unique_grain_directions must be (3, {n}, 3), got {dirs.shape}")
    flat = dirs.astype(np.float32).ravel()
    ctypes.memmove(p.grain_dirs, flat.ctypes.data, flat.nbytes)
    return p


class Quench:
    """Moving linear gradient T = T_base + grad (z - z0) - grad vel t
    (``applications/phase_field/solidification/example.py:21-34``; the
    reference uses T_base = T_liquidus and z0 = 0).  Passed in place of the T
    array in ``ode_params``, it is evaluated inside the step kernel, one value
    per z plane, at the start-of-step time."""

    def __init__(self, T_base, grad, vel, z0=0.0):
        self.T_base, self.grad, self.vel, self.z0 = float(T_base), float(grad), float(vel), float(z0)

    def struct(self, h_z):
        return _lib.Quench(self.T_base, self.grad, self.vel, self.z0, 0.5 * float(h_z))

    def __call__(self, centroids, t):
        """T at the cell centres (N, 1) as a NumPy array (host convenience)."""
        z = np.asarray(centroids)[:, 2]
        return (self.T_base + self.grad * (z - self.z0) - self.grad * self.vel * t)[:, None]


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def as_device_f32(x, shape=None, name="array"):
    """A contiguous float32 CUDA tensor view/copy of ``x``."""
    if not torch.is_tensor(x):
        x = torch.as_tensor(np.asarray(x))
    if not x.is_cuda:
        x = x.to("cuda", non_blocking=False)
    if x.dtype != torch.float32:
        x = x.float()
    x = x.contiguous()
    if shape is not None and x.numel() != int(np.prod(shape)):
        raise ValueError(f"{name} has {x.numel()} entries, expected {int(np.prod(shape))}")
    return x


class PendingMetrics:
    """The metrics record of ``PFSolver.inspect_async``, read on demand."""

    def __init__(self, solver, host, event):
        self._solver, self._host, self._event = solver, host, event

    def done(self):
        return self._event.query()

    def result(self):
        self._event.synchronize()
        return self._solver._metrics(_lib.Diag.from_buffer_copy(self._host.numpy().tobytes()))


class PFSolver:
    """Explicit-Euler Allen-Cahn grain growth on one GPU
    (reference: ``allen_cahn.py:131-210``)."""

    def __init__(self, pf_args, polycrystal):
        self.pf_args = pf_args
        self.polycrystal = polycrystal
        self.lib = _lib.load()
        self.params = make_pf_params(pf_args, polycrystal)
        self.N = self.params.nx * self.params.ny * self.params.nz
        self.n = self.params.num_oris
        self._clock = None
        self._diag_scratch = None
        self._diag_out = None
        self._argmax0 = None
        self._argmax0_src = None
        self.clean_sols()

    # ---- reference API --------------------------------------------------
    def stepper(self, state_pre, t_crt, ode_params, out=None):
        """One explicit Euler step (``allen_cahn.py:139-143``).

        ``state_pre = (eta, t_prev)`` with eta (N, num_oris); ``ode_params =
        [T]`` with T (N, 1) at the start of the step, or ``[Quench(...)]``, or
        ``[PointSource(...)]`` (evaluated in the kernel from the record
        nearest ``t_prev``), or ``[InterpolatedT(...)]`` (interpolated in
        time at ``t_crt`` in the kernel).
        Returns ``((eta_new, t_crt), eta_new)``.  ``out`` optionally receives
        the result (it must not alias eta)."""
        eta, t_prev = state_pre
        (T,) = ode_params
        eta = as_device_f32(eta, (self.N, self.n), "eta")
        if out is None:
            out = torch.empty_like(eta)
        elif out.data_ptr() == eta.data_ptr():
            raise ValueError("out must not alias eta")
        dt = float(t_crt) - float(t_prev)
        if isinstance(T, Quench):
            clk = self._clocks()
            clk[0].fill_(0)
            clk[0].view(torch.float64)[0] = float(t_prev)
            q = T.struct(self.params.h_z)
            st = self.lib.pfg_pf_step_quench(ctypes.byref(self.params), ctypes.byref(q),
                                              _lib.ptr(eta), _lib.ptr(out), _lib.ptr(clk[0]),
                                              _lib.ptr(clk[1]), dt, _stream())
        elif isinstance(T, InterpolatedT):
            if T.T_past.numel() != self.N:
                raise ValueError(f"InterpolatedT holds {T.T_past.numel()} cells, expected {self.N}")
            clk = self._clocks()
            clk[0].fill_(0)
            clk[0].view(torch.float64)[0] = float(t_prev)
            w = T.struct()
            st = self.lib.pfg_pf_step_interp(ctypes.byref(self.params), ctypes.byref(w),
                                              _lib.ptr(T.T_past), _lib.ptr(T.T_future),
                                              _lib.ptr(eta), _lib.ptr(out), _lib.ptr(clk[0]),
                                              _lib.ptr(clk[1]), dt, _stream())
        elif isinstance(T, PointSource):
            clk = self._clocks()
            clk[0].fill_(0)
            clk[0].view(torch.float64)[0] = float(t_prev)
            clk[0][1] = T.index_at(t_prev)
            src = T.struct(self.params)
            st = self.lib.pfg_pf_step_point_source(ctypes.byref(self.params), ctypes.byref(src),
                                                    _lib.ptr(eta), _lib.ptr(out),
                                                    _lib.ptr(clk[0]), _lib.ptr(clk[1]), dt,
                                                    _stream())
        else:
            T = as_device_f32(T, (self.N,), "T")
            st = self.lib.pfg_pf_step(ctypes.byref(self.params), _lib.ptr(eta), _lib.ptr(out),
                                      _lib.ptr(T), dt, _stream())
        _lib.check(st, "pfg_pf_step")
        return (out, t_crt), out

    def ini_cond(self):
        """One-hot eta from ``polycrystal.cell_ori_inds`` (``allen_cahn.py:145-153``)."""
        inds = torch.as_tensor(np.asarray(self.polycrystal.cell_ori_inds), dtype=torch.int64,
                               device="cuda")
        eta = torch.zeros((self.N, self.n), dtype=torch.float32, device="cuda")
        eta.scatter_(1, inds.view(-1, 1), 1.0)
        return eta

    def clean_sols(self):
        """Empty ``<data_dir>/vtk/pf/sols`` (``allen_cahn.py:155-163``), if a
        ``data_dir`` is configured."""
        if "data_dir" not in self.pf_args:
            return
        folder = os.path.join(self.pf_args["data_dir"], "vtk/pf/sols")
        os.makedirs(folder, exist_ok=True)
        for f in glob.glob(folder + "/*"):
            os.remove(f)

    def inspect_sol(self, pf_sol, pf_sol0, T, ts, step):
        """Print the reference's run-time metrics (``allen_cahn.py:165-180``)
        from one on-device reduction; raises ValueError on NaN/Inf."""
        d = self.inspect(pf_sol, T, pf_sol0)
        print(f"\nstep {step} of {len(ts[1:])}, unix timestamp = {time.time()}")
        print(f"percent of change of orientations = {d['pct_ori_changed']}%")
        print(f"percet of T >= T_liquidus = {d['pct_liquid']}%")
        print(f"max T = {d['max_T']}\n")
        if d["n_nonfinite"] > 0:
            raise ValueError("Found np.inf or np.nan in pf_sol - stop the program")
        return d

    def write_sols(self, pf_sol, T, step):
        """Write T and the argmax orientation map for step ``step //
        write_sol_interval`` (``allen_cahn.py:182-210``): a VTU file
        ``<data_dir>/vtk/pf/sols/u<k>.vtu`` with cell data ``T``, ``ori_inds``
        and, when the polycrystal carries the IPF colours of its orientations
        (``unique_oris_rgb``, (3, num_oris, 3): the x, y and z keys, as the
        reference's ``Field.get_unique_ori_colors`` gives them), ``ipf_x``,
        ``ipf_y``, ``ipf_z``: each cell's colour gathered by its argmax
        orientation, black (0) where T > T_liquidus (``allen_cahn.py:186-
        196``).  Also a NumPy ``.npz`` of T, ori_inds and the liquid mask
        under ``<data_dir>/numpy/pf/sols`` (what ``grains.process_eta``
        reads).  Returns the ``.npz`` path."""
        folder = os.path.join(self.pf_args.get("data_dir", "."), "numpy/pf/sols")
        os.makedirs(folder, exist_ok=True)
        k = step // int(self.pf_args.get("write_sol_interval", 1))
        T = as_device_f32(T, (self.N,), "T").view(-1)
        argmax = self.argmax(pf_sol)
        liquid = T > float(self.pf_args["T_liquidus"])
        path = os.path.join(folder, f"u{k:03d}.npz")
        np.savez_compressed(path, T=T.cpu().numpy(), ori_inds=argmax.cpu().numpy(),
                            liquid=liquid.cpu().numpy())
        cell_data = {"T": T}
        rgb = getattr(self.polycrystal, "unique_oris_rgb", None)
        if rgb is not None:
            rgb = torch.as_tensor(np.asarray(rgb), device="cuda")
            if rgb.shape[:2] != (3, self.n):
                raise ValueError(f"unique_oris_rgb has shape {tuple(rgb.shape)}, expected "
                                 f"(3, {self.n}, k)")
            inds = argmax.long()
            for axis, name in enumerate(("ipf_x", "ipf_y", "ipf_z")):
                c = rgb[axis].index_select(0, inds)
                c[liquid] = 0
                cell_data[name] = c
        cell_data["ori_inds"] = argmax
        from .vtu import write_vtu
        p = self.params
        write_vtu(os.path.join(self.pf_args.get("data_dir", "."), f"vtk/pf/sols/u{k:03d}.vtu"),
                  (p.nx, p.ny, p.nz), (p.h_x, p.h_y, p.h_z), cell_data)
        return path

    # ---- extensions ---------------------------------------------------------
    def _clocks(self):
        if self._clock is None:
            self._clock = torch.zeros((2, 2), dtype=torch.int64, device="cuda")
        return self._clock

    def argmax(self, eta):
        """First-maximum orientation index per cell (int32), from the diagnostics kernel."""
        out = torch.empty(self.N, dtype=torch.int32, device="cuda")
        self._diag(eta, torch.zeros(self.N, device="cuda"), None, out, ghosted=False,
                   entry="pfg_pf_inspect")
        return out

    def _diag_launch(self, eta, T, argmax0, argmax_out, ghosted, entry):
        if self._diag_scratch is None:
            nbytes = self.lib.pfg_pf_diag_scratch_bytes(ctypes.byref(self.params))
            self._diag_scratch = torch.empty(max(int(nbytes), 16), dtype=torch.uint8,
                                             device="cuda")
            self._diag_out = torch.empty(ctypes.sizeof(_lib.Diag), dtype=torch.uint8,
                                         device="cuda")
        st = getattr(self.lib, entry)(ctypes.byref(self.params), _lib.ptr(eta), _lib.ptr(T),
                                  int(ghosted), _lib.ptr(argmax0), _lib.ptr(argmax_out),
                                  _lib.ptr(self._diag_scratch), self._diag_scratch.numel(),
                                  _lib.ptr(self._diag_out), _stream())
        _lib.check(st, entry)

    def _diag(self, eta, T, argmax0, argmax_out, ghosted, entry="pfg_pf_diag"):
        self._diag_launch(eta, T, argmax0, argmax_out, ghosted, entry)
        host = self._diag_out.cpu().numpy()
        return _lib.Diag.from_buffer_copy(host.tobytes())

    def _diag_inputs(self, eta, T, eta0):
        eta = as_device_f32(eta, (self.N, self.n), "eta")
        T = as_device_f32(T, None, "T")
        a0 = None
        if eta0 is not None:
            if self._argmax0_src is not eta0:
                self._argmax0 = self.argmax(as_device_f32(eta0, (self.N, self.n), "eta0"))
                self._argmax0_src = eta0
            a0 = self._argmax0
        return eta, T, a0

    def inspect(self, eta, T, eta0=None, T_ghosted=False):
        """The reference's inspect_sol metrics only (argmax changes, liquid
        fraction, max T, NaN count), one pass over eta on the GPU."""
        return self.diagnostics(eta, T, eta0, T_ghosted, _entry="pfg_pf_inspect")

    def inspect_async(self, eta, T, eta0=None, T_ghosted=False):
        """``inspect`` without waiting for it: the metrics kernel and a copy of
        its record to pinned host memory are enqueued on the current stream,
        and ``result()`` of the returned ``PendingMetrics`` waits for them and
        gives ``inspect``'s dict.  Work enqueued later on the same stream runs
        after the kernel has read ``eta`` and ``T``, so a driver can launch
        its next steps first and read these metrics while they run (the
        reference's ``inspect_sol`` is synchronous: ``inspect``)."""
        eta, T, a0 = self._diag_inputs(eta, T, eta0)
        self._diag_launch(eta, T, a0, None, T_ghosted, "pfg_pf_inspect")
        host = torch.empty(self._diag_out.numel(), dtype=torch.uint8, pin_memory=True)
        host.copy_(self._diag_out, non_blocking=True)
        event = torch.cuda.Event()
        event.record()
        return PendingMetrics(self, host, event)

    def diagnostics(self, eta, T, eta0=None, T_ghosted=False, _entry="pfg_pf_diag"):
        """Energy, mass, liquid fraction, argmax changes and NaN count of a
        state, reduced on the GPU (compensated accumulation)."""
        eta, T, a0 = self._diag_inputs(eta, T, eta0)
        return self._metrics(self._diag(eta, T, a0, None, T_ghosted, _entry))

    def _metrics(self, d):
        N = max(int(d.n_cells), 1)
        return {
            "energy": d.energy, "max_T": d.max_T, "n_cells": d.n_cells,
            "n_ori_changed": d.n_ori_changed, "n_liquid": d.n_liquid,
            "n_nonfinite": d.n_nonfinite, "mass": np.array(d.mass[: self.n]),
            "pct_ori_changed": d.n_ori_changed / N * 100.0,
            "pct_liquid": d.n_liquid / N * 100.0,
        }

    def stable_dt(self, T_max=2000.0, safety=0.9):
        """Largest stable explicit dt at temperatures up to ``T_max`` (see
        ``stable_dt_for``) for this solver's grid."""
        p = self.params
        return PFSolver.stable_dt_for(self.pf_args, T_max, safety, (p.h_x, p.h_y, p.h_z))

    @staticmethod
    def stable_dt_for(pf_args, T_max=2000.0, safety=0.9, h=None):
        """The diffusive limit 1 / (2 sum_d 1/h_d^2 Lg kappa_g ad_hoc (1 + A))
        with Lg = L0 exp(-Qg / (R min(T_max, 2000))), times ``safety``.
        ``h`` defaults to ``pf_args['h']`` or domain / N."""
        a = pf_args
        if h is None:
            if "h" in a:
                h = (a["h"],) * 3 if np.isscalar(a["h"]) else tuple(a["h"])
            else:
                h = (a["domain_x"] / a["Nx"], a["domain_y"] / a["Ny"], a["domain_z"] / a["Nz"])
        T = min(float(T_max), 2000.0)
        Lg = a["L0"] * np.exp(-a["Qg"] / (a["gas_const"] * T))
        s = sum(1.0 / float(v) ** 2 for v in h)
        lim = 1.0 / (2.0 * s * Lg * a["kappa_g"] * a["ad_hoc"] * (1.0 + a["anisotropy"]))
        return safety * lim


def explicit_euler(state_pre, t_crt, solver, ode_params):
    """``explicit_euler(state_pre, t_crt, f, ode_params)`` of the reference
    (``allen_cahn.py:106-114``) with the solver in place of ``f``."""
    return solver.stepper(state_pre, t_crt, ode_params)


def rk4(state_pre, t_crt, solver, ode_params):
    """``rk4(state_pre, t_crt, f, ode_params)`` of the reference
    (``allen_cahn.py:91-104``, unused by its drivers) with the solver in place
    of ``f``.  Each stage increment k = h f(y_s) is read off one explicit
    step from y_s (k = euler(y_s, h) - y_s); the temperature in
    ``ode_params`` is held over the step as the reference's state_rhs does."""
    y, t_prev = state_pre
    y = as_device_f32(y, (solver.N, solver.n), "eta")
    h = float(t_crt) - float(t_prev)

    def k_of(ys, ts):
        (e, _), _ = solver.stepper((ys, ts), ts + h, ode_params)
        return e - ys

    k1 = k_of(y, t_prev)
    k2 = k_of(y + 0.5 * k1, t_prev + 0.5 * h)
    k3 = k_of(y + 0.5 * k2, t_prev + 0.5 * h)
    k4 = k_of(y + k3, t_prev + h)
    y_crt = y + (k1 + 2.0 * k2 + 2.0 * k3 + k4) / 6.0
    return (y_crt, t_crt), y_crt
