"""One-way coupling of a coarser temperature solver to the phase field.

The reference's coupled driver (``applications/phase_field/coupled/
example.py:23-111``) advances a CFD solver with a time step ``dt_cfd`` larger
than the phase field's, keeps its last two temperature fields ``T_past`` and
``T_future`` (cells ordered (Nx, Ny, Nz)), and feeds every phase-field step
the temperature linearly interpolated in time at the step's end time,
transposed into the phase-field cell order (``convert_temperature`` and
``interpolate_T``, ``example.py:31-42``).

Here ``convert_temperature`` runs on the GPU (``pfg_transpose_xyz``), and the
interpolation happens per cell inside the step kernel: pass an
``InterpolatedT`` in place of the T array in ``PFSolver.stepper``'s
``ode_params`` (``pfg_pf_step_interp``), so no interpolated array is written.
"""
import ctypes

import torch

from .. import _lib


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def convert_temperature(T_cfd):
    """(Nx, Ny, Nz) temperature of the coarse solver -> (N, 1) float32 CUDA
    tensor in the phase-field cell order (``example.py:31-36``)."""
    T = torch.as_tensor(T_cfd).to("cuda", torch.float32).contiguous()
    if T.dim() != 3:
        raise ValueError(f"T_cfd must be (Nx, Ny, Nz), got {tuple(T.shape)}")
    nx, ny, nz = T.shape
    out = torch.empty((nx * ny * nz, 1), dtype=torch.float32, device="cuda")
    st = _lib.load().pfg_transpose_xyz(nx, ny, nz, _lib.ptr(T), _lib.ptr(out), _stream())
    _lib.check(st, "pfg_transpose_xyz")
    return out


def interpolate_T(T_past, T_future, t_pf, t_cfd, dt_cfd):
    """``interpolate_T`` of the reference (``example.py:38-42``) on arrays:
    r T_past + (1 - r) T_future with r = (t_cfd - t_pf) / dt_cfd."""
    r = (float(t_cfd) - float(t_pf)) / float(dt_cfd)
    return r * T_past + (1.0 - r) * T_future


class InterpolatedT:
    """T_past and T_future (each (N,) or (N, 1), the phase-field cell order,
    e.g. from ``convert_temperature``) at times t_future - dt_coarse and
    t_future; a step ending at t uses r T_past + (1 - r) T_future,
    r = (t_future - t) / dt_coarse, evaluated per cell in the kernel."""

    def __init__(self, T_past, T_future, t_future, dt_coarse):
        self.T_past = torch.as_tensor(T_past).to("cuda", torch.float32).reshape(-1).contiguous()
        self.T_future = torch.as_tensor(T_future).to("cuda", torch.float32).reshape(-1).contiguous()
        if self.T_past.numel() != self.T_future.numel():
            raise ValueError("T_past and T_future differ in size")
        self.t_future = float(t_future)
        self.dt_coarse = float(dt_coarse)

    def struct(self):
        return _lib.Interp(self.t_future, self.dt_coarse)
