"""Shared pieces of the float32-vs-float64 configuration tests: the
comparison (max |d eta|, max |dT|, argmax maps with mismatches allowed only at
float64 near-ties) and the fused laser run against the float64 PyTorch
restatement of the oracle on the GPU."""
import numpy as np
import torch

from oracle import pf_torch as PT

ETA_TOL = 1e-4
T_TOL = 1e-3
T_LIQ = 1623.0  # T_liquidus of the laser configurations
PF_KEYS = dict(gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6, m_g=2.4e5, ad_hoc=1.0)


def _f32(v):
    return float(np.float32(v))


def _oracle_args(pf_args, poly):
    """The phase-field parameters as the GPU receives them (float32 values,
    widened): the float64 run then evaluates exactly the model the float32
    run approximates."""
    a = {k: _f32(pf_args[k]) for k in ("T_liquidus", "gas_const", "Qg", "L0", "kappa_g", "m_g",
                                        "anisotropy", "ad_hoc")}
    a["h"] = tuple(_f32(v) for v in poly.mesh_h_xyz)
    return a


def _oracle_gamma(g):
    """gamma_args as the GPU receives them (float32 values, widened)."""
    return {k: _f32(v) for k, v in g.items()}


def _dirs(poly):
    d = np.asarray(poly.unique_grain_directions, dtype=np.float32).astype(np.float64)
    return torch.tensor(d, device="cuda")


def _compare(name, e_gpu, e_ref, T_gpu=None, T_ref=None):
    n = e_ref.shape[-1]
    e_ref = e_ref.reshape(-1, n)
    e_gpu = e_gpu.double().reshape(-1, n)
    err = float((e_gpu - e_ref).abs().max())
    am_g = torch.argmax(e_gpu, dim=1)
    am_r = torch.argmax(e_ref, dim=1)
    bad = am_g != am_r
    mism = int(bad.sum())
    if mism:
        top2 = torch.topk(e_ref[bad], 2, dim=1).values
        gap = float((top2[:, 0] - top2[:, 1]).max())
        assert gap <= 2 * err, f"{name}: argmax mismatch away from a tie (gap {gap})"
    t_err = None
    if T_gpu is not None:
        t_err = float((T_gpu.double() - T_ref).abs().max())
    print(f"{name}: max |d eta| float32 GPU vs float64 = {err:.3e}, "
          f"argmax mismatches = {mism} of {e_ref.shape[0]}"
          + (f", max |dT| = {t_err:.3e} K" if t_err is not None else ""))
    assert err <= ETA_TOL
    if t_err is not None:
        assert t_err <= T_TOL


def _laser_case(shape, n, grains, aniso, path, steps, seed, name, chunk=None, graph=True,
                compensated=None):
    """Fused laser run of ``steps`` steps on the GPU against the float64
    PyTorch restatement; returns the highest interior temperature the float64
    run reached in any step (so that callers can require the melt branch:
    T >= T_liquidus switches zeta and the liquid front).  ``chunk``: evaluate
    the float64 phase field that many z planes at a time (large grids).
    ``compensated``: True / False to require that temperature state (None:
    the run's default)."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import HeatPFRun
    from jax_am_gb300.workloads import gamma_args
    nx, ny, nz = shape
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_grains=grains, num_oris=n,
                   T_liquidus=1623.0, anisotropy=aniso)
    poly = Field(pf_args, seed=seed)
    s = PFSolver(pf_args, poly)
    g = gamma_args()
    run = HeatPFRun(s, g, path, compensated=compensated)
    if compensated is not None:
        assert run.compensated == compensated
    dt = float(np.float32(run.dt))
    run.run(steps, graph=graph)
    a = _oracle_args(pf_args, poly)
    dirs = _dirs(poly)
    e = s.ini_cond().double().reshape(nz, ny, nx, -1)
    Tg = torch.full((nz + 2, ny + 2, nx + 2), float(g["T0"]), dtype=torch.float64, device="cuda")
    path32 = [tuple(float(np.float32(v)) for v in seg) for seg in path]

    def laser(tm):
        for (t0, t1, x0, y0, x1, y1, P) in path32:
            if t0 <= tm < t1:
                f = (tm - t0) / (t1 - t0)
                return x0 + f * (x1 - x0), y0 + f * (y1 - y0), P
        return 0.0, 0.0, 0.0

    t = 0.0
    g64 = _oracle_gamma(g)
    Tmax = torch.zeros((), dtype=torch.float64, device="cuda")
    for _ in range(steps):
        e, Tg = PT.coupled_step(e, Tg, t, dt, a, g64, laser, dirs, chunk=chunk)
        Tmax = torch.maximum(Tmax, Tg[1:-1, 1:-1, 1:-1].max())
        t += dt
    _compare(name, run.state, e, run.T_ghosted_f64[1:-1, 1:-1, 1:-1], Tg[1:-1, 1:-1, 1:-1])
    return float(Tmax)
