"""Drop-in for JAX-AM's explicit heat step (``jax_am/cfd/gamma.py``).

``update_T(T, xl, yl, x, y, P, dx, dy, dz, dt, gamma_args)`` keeps the
reference signature: ``T`` is the ghosted (nx+2, ny+2, nz+2) field in the
reference's axis order and ``x``/``y`` the (nx, ny, nz) cell-centre
coordinates (only the first centre and the spacing are used; the grid must be
uniform).  The step runs in ``libpfgb300.so``; the kernel reads the reference
layout directly through its strides, so no transpose is made.
"""
import ctypes

import numpy as np
import torch

from .. import _lib

GAMMA_KEYS = ("rho", "h", "eps", "SB", "T0", "Ts", "Tl", "L", "eta", "r")


def make_heat_params(gamma_args, nx, ny, nz, dx, dy, dz, x_first=None, y_first=None,
                     layout=_lib.LAYOUT_ZYX, path=None):
    """Fill the C ``pfg_heat_params`` struct from the reference ``gamma_args``
    dict (``applications/cfd/gamma/example.py:67-79``).  ``path`` is a list of
    (t0, t1, x0, y0, x1, y1, power) tool-path segments for the fused step."""
    missing = [k for k in GAMMA_KEYS if k not in gamma_args]
    if missing:
        raise ValueError(f"gamma_args is missing {missing}")
    h = _lib.HeatParams()
    h.nx, h.ny, h.nz = int(nx), int(ny), int(nz)
    h.dx, h.dy, h.dz = float(dx), float(dy), float(dz)
    g = gamma_args
    h.rho, h.h_conv, h.emissivity, h.sigma_sb = g["rho"], g["h"], g["eps"], g["SB"]
    h.T0, h.Ts, h.Tl, h.latent = g["T0"], g["Ts"], g["Tl"], g["L"]
    h.absorptivity, h.beam_radius = g["eta"], g["r"]
    h.x_first = float(dx) / 2.0 if x_first is None else float(x_first)
    h.y_first = float(dy) / 2.0 if y_first is None else float(y_first)
    h.layout = int(layout)
    path = list(path or [])
    if len(path) > _lib.MAX_SEGMENTS:
        raise ValueError(f"at most {_lib.MAX_SEGMENTS} tool-path segments")
    h.num_segments = len(path)
    for i, seg in enumerate(path):
        h.path[i] = _lib.Segment(*[float(v) for v in seg], 0.0)
    return h


_coord_cache = {}


def update_T(T, xl, yl, x, y, P, dx, dy, dz, dt, gamma_args, out=None):
    """One explicit heat step (``gamma.py:55-61``); returns the new ghosted T
    (a new tensor unless ``out`` is given)."""
    lib = _lib.load()
    if not torch.is_tensor(T):
        T = torch.as_tensor(np.asarray(T))
    T = T.to("cuda").float().contiguous()
    if T.dim() != 3:
        raise ValueError("T must be the ghosted (nx+2, ny+2, nz+2) field")
    nx, ny, nz = (s - 2 for s in T.shape)
    key = (id(x), id(y), float(dx), float(dy))
    if key not in _coord_cache:
        xa = x.detach().cpu().numpy() if torch.is_tensor(x) else np.asarray(x)
        ya = y.detach().cpu().numpy() if torch.is_tensor(y) else np.asarray(y)
        xt, yt = xa[:, :, -1], ya[:, :, -1]
        ex = xt[0, 0] + float(dx) * np.arange(nx)[:, None]
        ey = yt[0, 0] + float(dy) * np.arange(ny)[None, :]
        if not (np.allclose(xt, ex, rtol=1e-6, atol=1e-12) and np.allclose(yt, ey, rtol=1e-6,
                                                                          atol=1e-12)):
            raise ValueError("x and y must be uniform cell-centre grids with spacing dx, dy")
        _coord_cache.clear()
        _coord_cache[key] = (float(xt[0, 0]), float(yt[0, 0]))
    x_first, y_first = _coord_cache[key]
    h = make_heat_params(gamma_args, nx, ny, nz, dx, dy, dz, x_first, y_first,
                         layout=_lib.LAYOUT_XYZ)
    if out is None:
        out = T.clone()  # edge/corner ghosts are carried over unchanged
    st = lib.pfg_heat_step(ctypes.byref(h), _lib.ptr(T), _lib.ptr(out), float(xl), float(yl),
                           float(P), float(dt),
                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check(st, "pfg_heat_step")
    return out


def stable_dt(gamma_args, dx, dy, dz, safety=0.9):
    """Explicit stability limit of the heat step, 1 / (2 alpha_max sum 1/d^2)
    with alpha_max = max k/(rho cp) over T (k and cp are clipped at Tl)."""
    T = np.linspace(300.0, gamma_args["Tl"], 2048)
    k = 0.0163 * T + 4.5847
    cp = 0.2441 * T + 338.39
    alpha = np.max(k / cp) / gamma_args["rho"]
    return safety / (2.0 * alpha * (1 / dx ** 2 + 1 / dy ** 2 + 1 / dz ** 2))
