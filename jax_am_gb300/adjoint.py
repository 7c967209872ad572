"""Gradients of a laser-scan objective through the fused heat + phase-field run.

The forward problem is the coupled run of ``runner.HeatPFRun`` with one
straight laser track: power ``P``, speed ``v``, starting at ``x_start`` on the
line ``y`` at time 0.  The objective is the volume average
J = mean over cells of sum_i w_i eta_i^2 at the final step.  The gradient
with respect to (P, v, eta0) is computed by the hand-written discrete adjoint
(``pfg_adjoint_step``) with step checkpointing: the forward run stores the
state every ``checkpoint_every`` steps; the backward sweep recomputes each
segment from its checkpoint, keeps that segment's states, and runs the
adjoint steps over it in reverse.  ``HeatPFObjective`` exposes this as a
``torch.autograd.Function``.

The reference has no adjoint of this path; its gradients would come from
``jax.grad`` of the whole run.  This module is checked against float64
autograd of the oracle's restatement and against central finite differences.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .cfd.gamma import make_heat_params
from .phase_field.allen_cahn import PFSolver


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class LaserTrackProblem:
    """Forward run and adjoint of J(P, v, eta0) for one straight track along +x."""

    def __init__(self, pf_args, polycrystal, gamma_args, weights, dt, steps, x_start, y,
                 checkpoint_every=25, T_init=None):
        self.solver = PFSolver(pf_args, polycrystal)
        self.lib = self.solver.lib
        self.p = self.solver.params
        self.gamma_args = dict(gamma_args)
        self.dt = float(np.float32(dt))
        self.steps = int(steps)
        self.C = max(1, int(checkpoint_every))
        self.x_start, self.y = float(x_start), float(y)
        self.t_end = self.steps * self.dt * 2.0 + 1.0  # the track outlasts the run
        p = self.p
        self.N = p.nx * p.ny * p.nz
        self.n = p.num_oris
        self.gshape = (p.nz + 2, p.ny + 2, p.nx + 2)
        self.w = torch.as_tensor(np.asarray(weights, dtype=np.float32), device="cuda")
        if T_init is None:
            T_init = torch.full(self.gshape, float(gamma_args["T0"]), dtype=torch.float32)
        self.T_init = T_init.to("cuda", torch.float32).reshape(self.gshape).contiguous()
        self._ckpt = None

    def heat_params(self, P, v):
        x1 = self.x_start + v * self.t_end
        path = [(0.0, self.t_end, self.x_start, self.y, x1, self.y, P)]
        return make_heat_params(self.gamma_args, self.p.nx, self.p.ny, self.p.nz, self.p.h_x,
                                self.p.h_y, self.p.h_z, path=path)

    def _step(self, h, eta_in, eta_out, T_in, T_out, clk_in, clk_out):
        st = self.lib.pfg_heat_pf_step(ctypes.byref(self.p), ctypes.byref(h), _lib.ptr(eta_in),
                                       _lib.ptr(eta_out), _lib.ptr(T_in), _lib.ptr(T_out),
                                       _lib.ptr(clk_in), _lib.ptr(clk_out), self.dt, _stream())
        _lib.check(st, "pfg_heat_pf_step")

    def _run(self, h, eta, T, clk, steps, keep=None):
        """Advance (eta, T, clk) by `steps` steps in double buffers; keep(k, eta, T)
        is called with the state before each step."""
        e = [eta.clone(), torch.empty_like(eta)]
        t = [T.clone(), T.clone()]
        c = [clk.clone(), torch.zeros_like(clk)]
        cur = 0
        for k in range(steps):
            if keep is not None:
                keep(k, e[cur], t[cur], c[cur])
            self._step(h, e[cur], e[cur ^ 1], t[cur], t[cur ^ 1], c[cur], c[cur ^ 1])
            cur ^= 1
        return e[cur], t[cur], c[cur]

    def objective(self, eta, lam_seed=None):
        J = torch.zeros(1, dtype=torch.float64, device="cuda")
        st = self.lib.pfg_objective(ctypes.byref(self.p), _lib.ptr(eta), _lib.ptr(self.w),
                                    _lib.ptr(J), _lib.ptr(lam_seed), _stream())
        _lib.check(st, "pfg_objective")
        return J

    def forward(self, P, v, eta0):
        """J(P, v, eta0); stores the checkpoints for ``gradient``."""
        self.P, self.v = float(P), float(v)
        h = self.heat_params(self.P, self.v)
        eta = eta0.to("cuda", torch.float32).reshape(self.N, self.n).contiguous()
        clk = torch.zeros(2, dtype=torch.int64, device="cuda")
        ckpt = []

        def keep(k, e, T, c):
            if k % self.C == 0:
                ckpt.append((e.clone(), T.clone(), c.clone()))

        eta_f, T_f, _ = self._run(h, eta, self.T_init, clk, self.steps, keep)
        self._ckpt = ckpt
        self._eta_final = eta_f
        return float(self.objective(eta_f).item())

    def gradient(self):
        """(dJ/dP, dJ/dv, dJ/deta0) of the last ``forward`` call."""
        assert self._ckpt is not None, "call forward() first"
        h = self.heat_params(self.P, self.v)
        lam = torch.empty(self.N, self.n, dtype=torch.float32, device="cuda")
        self.objective(self._eta_final, lam)
        lam2 = torch.empty_like(lam)
        Tb = torch.zeros(self.gshape, dtype=torch.float32, device="cuda")
        Tb2 = torch.zeros_like(Tb)
        grads = torch.zeros(2, dtype=torch.float64, device="cuda")
        nbytes = int(self.lib.pfg_adjoint_scratch_bytes(ctypes.byref(self.p)))
        scratch = torch.empty(nbytes // 4 + 1, dtype=torch.float32, device="cuda")
        dt = self.dt
        # the device clock at each step: float32 dt summed in float64, in order
        times = [0.0]
        for _ in range(self.steps):
            times.append(times[-1] + dt)
        for seg in reversed(range(len(self._ckpt))):
            k0 = seg * self.C
            nseg = min(self.C, self.steps - k0)
            states = []
            e0, T0, c0 = self._ckpt[seg]
            self._run(h, e0, T0, c0, nseg,
                      keep=lambda k, e, T, c: states.append((e.clone(), T.clone())))
            for j in reversed(range(nseg)):
                k = k0 + j
                t = times[k]
                e_k, T_k = states[j]
                st = self.lib.pfg_adjoint_step(
                    ctypes.byref(self.p), ctypes.byref(h), _lib.ptr(e_k), _lib.ptr(T_k), t, dt,
                    _lib.ptr(lam), _lib.ptr(Tb), _lib.ptr(lam2), _lib.ptr(Tb2), _lib.ptr(scratch),
                    scratch.numel() * 4, _lib.ptr(grads), float(t + 0.5 * dt), _stream())
                _lib.check(st, "pfg_adjoint_step")
                lam, lam2 = lam2, lam
                Tb, Tb2 = Tb2, Tb
        g = grads.cpu().numpy()
        return float(g[0]), float(g[1]), lam.clone()


class HeatPFObjective(torch.autograd.Function):
    """J(P, v, eta0) as an autograd node; ``problem`` is a LaserTrackProblem."""

    @staticmethod
    def forward(ctx, P, v, eta0, problem):
        J = problem.forward(float(P), float(v), eta0.detach())
        ctx.problem = problem
        ctx.dtype = eta0.dtype
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gJ):
        dP, dv, deta = ctx.problem.gradient()
        g = float(gJ)
        return (torch.tensor(g * dP, dtype=torch.float64), torch.tensor(g * dv, dtype=torch.float64),
                (g * deta).to(ctx.dtype), None)
