"""PyTorch restatement of the fused heat + phase-field step (any device).

TEST INFRASTRUCTURE ONLY, like ``pf_oracle.py``: used by the tests (float64
autograd as the stand-in for the reference's ``jax.grad``) and by the CPU
baseline leg of ``bench.py`` (float32, all host threads).  Never imported by
``jax_am_gb300``.

Same algorithm as ``pf_oracle`` (``allen_cahn.py:42-85,106-114``,
``gamma.py:9-61``), written with torch tensors.  The anisotropy uses the
arccos-free closed form cos^2 t = max_k (d_k.e)^2 / |e|^2 (equal to the
reference's ``update_anisotropy_helper``, ``allen_cahn.py:28-39``, which the
float64 tests check), so that autograd has no arccos singularities.  The
heat field is held in the z-major ghosted order (nz+2, ny+2, nx+2).
"""
import math

import torch


def _shift(e, axis, step, periodic):
    """Neighbour along ``axis`` of the (Nz, Ny, Nx, n) grid: +1 or -1
    (periodic wrap, or the edge cell repeated: ``allen_cahn.py:61-66``)."""
    if periodic:
        return torch.roll(e, -step, dims=axis)
    n = e.shape[axis]
    if n == 1:
        return e
    if step > 0:
        return torch.cat((e.narrow(axis, 1, n - 1), e.narrow(axis, n - 1, 1)), dim=axis)
    return torch.cat((e.narrow(axis, 0, 1), e.narrow(axis, 0, n - 1)), dim=axis)


def pf_increment(eta4, T3, a, dirs, bc=(False, False, False)):
    """dt-free rhs of the Allen-Cahn step on the (Nz, Ny, Nx, n) grid.
    ``a``: dict with T_liquidus, gas_const, Qg, L0, kappa_g, m_g, anisotropy,
    ad_hoc and h = (hx, hy, hz); ``bc``: periodic flag per (x, y, z)."""
    hx, hy, hz = a["h"]
    Tc = torch.where(T3 > 2000.0, torch.full_like(T3, 2000.0), T3)
    zeta = 0.5 * (1.0 - torch.tanh(1e10 * (Tc / a["T_liquidus"] - 1.0)))
    S = torch.sum(eta4 ** 2, dim=-1, keepdim=True)
    z = zeta[..., None]
    grad = a["m_g"] * (eta4 ** 3 - eta4 + 4.0 * eta4 * (S - eta4 ** 2)
                       + 2.0 * (1.0 - z) ** 2 * eta4) / a["ad_hoc"]
    xm, xp = _shift(eta4, 2, -1, bc[0]), _shift(eta4, 2, 1, bc[0])
    ym, yp = _shift(eta4, 1, -1, bc[1]), _shift(eta4, 1, 1, bc[1])
    zm, zp = _shift(eta4, 0, -1, bc[2]), _shift(eta4, 0, 1, bc[2])
    lap = (((xp - eta4) + (xm - eta4)) / hx ** 2 + ((yp - eta4) + (ym - eta4)) / hy ** 2
           + ((zp - eta4) + (zm - eta4)) / hz ** 2)
    if a["anisotropy"] > 0.0:
        gx, gy, gz = xp - xm, yp - ym, zp - zm  # central differences, (..., n)
        ee = gx * gx + gy * gy + gz * gz
        m = None
        for k in range(3):  # (d_k . e)^2 for the three rotated cube axes
            d = dirs[k]  # (n, 3)
            p = gx * d[:, 0] + gy * d[:, 1] + gz * d[:, 2]
            m = p * p if m is None else torch.maximum(m, p * p)
        safe = torch.where(ee > 0, ee, torch.ones_like(ee))
        c2 = torch.where(ee > 0, torch.clamp(m / safe, max=1.0), torch.ones_like(ee))
        aniso = 1.0 + a["anisotropy"] * (c2 ** 2 + (1.0 - c2) ** 2)
    else:
        aniso = 1.0
    lap_term = -aniso * a["kappa_g"] * a["ad_hoc"] * lap
    Lg = a["L0"] * torch.exp(-a["Qg"] / (Tc * a["gas_const"]))
    return -Lg[..., None] * (grad + lap_term)


def heat_step(Tg, xl, yl, P, dt, g, h):
    """One explicit heat step on the ghosted (nz+2, ny+2, nx+2) field
    (``gamma.py:55-61``).  ``g`` holds the gamma_args keys, ``h`` = (dx, dy, dz)."""
    dx, dy, dz = h
    nz, ny, nx = (s - 2 for s in Tg.shape)
    clipk = torch.clamp(Tg, 300.0, g["Tl"])
    fl = (torch.clamp(Tg, g["Ts"], g["Tl"]) - g["Ts"]) / (g["Tl"] - g["Ts"])
    k = 0.0163 * clipk + 4.5847
    cp = 0.2441 * clipk + 338.39 + ((fl > 0) & (fl < 1)).to(Tg.dtype) * g["L"]

    def robin(Tf):
        return g["h"] * (Tf - g["T0"]) + g["SB"] * g["eps"] * (Tf ** 4 - g["T0"] ** 4)

    I = slice(1, -1)
    T = Tg.clone()
    x = dx / 2.0 + dx * torch.arange(nx, dtype=Tg.dtype, device=Tg.device)
    y = dy / 2.0 + dy * torch.arange(ny, dtype=Tg.dtype, device=Tg.device)
    beam = (2.0 * P * g["eta"] / math.pi / g["r"] ** 2
            * torch.exp(-2.0 * ((x[None, :] - xl) ** 2 + (y[:, None] - yl) ** 2) / g["r"] ** 2))
    T[I, I, 0] = Tg[I, I, 1] - robin((Tg[I, I, 1] + Tg[I, I, 0]) / 2) / k[I, I, 1] * dx
    T[I, I, -1] = Tg[I, I, -2] - robin((Tg[I, I, -2] + Tg[I, I, -1]) / 2) / k[I, I, -2] * dx
    T[I, 0, I] = Tg[I, 1, I] - robin((Tg[I, 1, I] + Tg[I, 0, I]) / 2) / k[I, 1, I] * dy
    T[I, -1, I] = Tg[I, -2, I] - robin((Tg[I, -2, I] + Tg[I, -1, I]) / 2) / k[I, -2, I] * dy
    T[0, I, I] = Tg[1, I, I] - robin((Tg[1, I, I] + Tg[0, I, I]) / 2) / k[1, I, I] * dz
    T[-1, I, I] = Tg[-2, I, I] - (robin((Tg[-2, I, I] + Tg[-1, I, I]) / 2) - beam) / k[-2, I, I] * dz
    lap = ((T[I, I, :-2] - 2 * T[I, I, 1:-1] + T[I, I, 2:]) / dx ** 2
           + (T[I, :-2, I] - 2 * T[I, 1:-1, I] + T[I, 2:, I]) / dy ** 2
           + (T[:-2, I, I] - 2 * T[1:-1, I, I] + T[2:, I, I]) / dz ** 2)
    out = T.clone()
    out[I, I, I] = T[I, I, I] + dt * (k[I, I, I] / g["rho"] / cp[I, I, I] * lap)
    return out


def pf_increment_chunked(eta4, T3, a, dirs, chunk):
    """``pf_increment`` with Neumann faces, evaluated ``chunk`` z planes at a
    time (each chunk with its neighbour planes), so that the float64
    temporaries of a large grid stay a few planes deep.  Equal to
    ``pf_increment`` of the whole grid: a chunk's edge planes see their true
    neighbours, and the edge replication at a chunk's halo only affects the
    halo planes, whose values are dropped."""
    nz = eta4.shape[0]
    out = torch.empty_like(eta4)
    for z0 in range(0, nz, chunk):
        z1 = min(z0 + chunk, nz)
        lo, hi = max(z0 - 1, 0), min(z1 + 1, nz)
        inc = pf_increment(eta4[lo:hi], T3[lo:hi], a, dirs)
        out[z0:z1] = inc[z0 - lo:z1 - lo]
    return out


def coupled_step(eta4, Tg, t, dt, a, g, laser, dirs, force_liquid=False, shift=1.0, chunk=None):
    """Fused step: phase field at the start-of-step T, heat with the beam at
    the mid-step time (same convention as ``pf_oracle.coupled_step``).
    ``chunk``: evaluate the phase field ``chunk`` z planes at a time
    (``pf_increment_chunked``; Neumann faces, as the heat coupling has)."""
    T3 = Tg[1:-1, 1:-1, 1:-1]
    if chunk:
        eta_new = eta4 + dt * pf_increment_chunked(eta4, T3, a, dirs, chunk)
    else:
        eta_new = eta4 + dt * pf_increment(eta4, T3, a, dirs)
    if force_liquid:
        eta_new = torch.where((T3 > a["T_liquidus"] + shift)[..., None],
                              torch.zeros_like(eta_new), eta_new)
    xl, yl, P = laser(t + 0.5 * dt)
    return eta_new, heat_step(Tg, xl, yl, P, dt, g, a["h"])
