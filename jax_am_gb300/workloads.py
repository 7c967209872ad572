"""Seeded synthetic workloads with the sizes and distributions of the
benchmark configurations (the reference's own Neper inputs are not shipped,
so every polycrystal here is generated; see ``phase_field.utils.Field``).

* ``directional_solidification``: 64 x 64 x 32 cells, 40 grains, 20
  orientations, isotropic, moving gradient 1e6 K/m at 0.1 m/s with the
  liquid above T_melt = 1700 K forced to eta = 0.
* ``laser_track``: 400 x 200 x 100 cells, 2000 grains, 20 orientations,
  anisotropy 0.15, fused heat with a 200 W / 50 um / 0.4 Gaussian at 0.8 m/s.
* ``differentiable_run``: 128 x 128 x 64 cells, 300 grains, 10 orientations,
  the laser of ``laser_track``, 500 steps, checkpoint every 25, objective
  mean sum_i w_i eta_i^2 with w_i ~ U(0, 1).
* ``serving_stream``: 256 directional-solidification jobs with Poisson
  arrivals at 50 jobs/s, Nx, Ny ~ U[32, 160], Nz ~ U[16, 64],
  num_oris ~ U[10, 30], grains = cells / 2000, steps ~ U[100, 2000],
  gradient ~ U[5e5, 2e6] K/m.
* ``cfd_simple_case``: the implicit CFD solver on the reference's standalone
  CFD driver (``applications/cfd/simple/example.py:22-41`` and its
  ``cfd_params.json``): 464 x 93 x 46 cells over 1 x 0.2 x 0.1 mm, a
  348 x 46 x 18 local flow box, a 100 W surface Gaussian at 0.5 m/s.
"""
import numpy as np

PF_KEYS = dict(gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6, m_g=2.4e5, ad_hoc=1.0)


def gamma_args(absorptivity=0.4, radius=5e-5, T0=300.0):
    g = dict(eta=absorptivity, r=radius, rho=8440.0, h=10.0, eps=0.4, SB=5.67e-8, T0=T0,
             Ts=1563.0, Tl=1623.0)
    g["L"] = 290e3 / (g["Tl"] - g["Ts"])
    return g


def solidification_job(shape, num_oris, steps, grad, seed, arrival=0.0, num_grains=None,
                       T_melt=1700.0, vel=0.1):
    """One directional-solidification job (serving unit)."""
    from .phase_field.allen_cahn import PFSolver, Quench
    from .phase_field.utils import Field
    from .serving import Job
    nx, ny, nz = shape
    cells = nx * ny * nz
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_oris=num_oris,
                   num_grains=num_grains or max(1, cells // 2000), T_liquidus=T_melt,
                   anisotropy=0.0, force_liquid_zero=True, liquid_shift=1.0)
    poly = Field(pf_args, seed=seed)
    dt = float(np.float32(PFSolver.stable_dt_for(pf_args)))
    quench = Quench(T_melt, grad, vel, z0=0.5 * nz * 1e-6)
    return Job(pf_args, poly, quench, int(steps), dt, arrival=float(arrival))


def serving_stream(num_jobs=256, rate=50.0, seed=4):
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, num_jobs)
    arrivals = np.cumsum(gaps) - gaps[0]
    jobs = []
    for j in range(num_jobs):
        nx, ny = int(rng.integers(32, 161)), int(rng.integers(32, 161))
        nz = int(rng.integers(16, 65))
        n = int(rng.integers(10, 31))
        steps = int(rng.integers(100, 2001))
        grad = float(rng.uniform(5e5, 2e6))
        jobs.append(solidification_job((nx, ny, nz), n, steps, grad, seed=1000 + j,
                                       arrival=arrivals[j]))
    return jobs


def laser_track_case(seed=2):
    from .phase_field.allen_cahn import PFSolver
    from .phase_field.utils import Field
    from .runner import single_track
    pf_args = dict(PF_KEYS, Nx=400, Ny=200, Nz=100, h=1e-6, num_grains=2000, num_oris=20,
                   anisotropy=0.15, T_liquidus=1623.0)
    poly = Field(pf_args, seed=seed)
    solver = PFSolver(pf_args, poly)
    path = single_track(50e-6, 100e-6, 0.8, 200.0, 1.0)
    return solver, gamma_args(), path, poly


def differentiable_run(steps=500, checkpoint_every=25, seed=3):
    from .adjoint import LaserTrackProblem
    from .cfd.gamma import stable_dt as heat_dt
    from .phase_field.allen_cahn import PFSolver
    from .phase_field.utils import Field
    pf_args = dict(PF_KEYS, Nx=128, Ny=128, Nz=64, h=1e-6, num_grains=300, num_oris=10,
                   anisotropy=0.0, T_liquidus=1623.0)
    poly = Field(pf_args, seed=seed)
    g = gamma_args()
    dt = min(PFSolver.stable_dt_for(pf_args), heat_dt(g, 1e-6, 1e-6, 1e-6))
    w = np.random.default_rng(seed).random(10).astype(np.float32)
    prob = LaserTrackProblem(pf_args, poly, g, w, dt, steps, x_start=20e-6, y=64e-6,
                             checkpoint_every=checkpoint_every)
    return prob, 200.0, 0.8


def cfd_simple_case():
    """``args`` for ``jax_am_gb300.cfd.cfd_am.AM_3d`` (meshes included)."""
    from .cfd import cfd_am as G
    dom, N = [1e-3, 2e-4, 1e-4], [464, 93, 46]
    NL = [round(0.75 * N[0]), round(0.5 * N[1]), round(0.4 * N[2])]
    args = dict(rho=8440.0, visco=7e-3, Marangoni=-2e-5, dt=1e-6, t_OFF=0.0012, speed=0.5,
                X0=[2e-4, 1e-4, 1e-4], rb=5e-5, eta=0.43, P=100.0, T_ref=300.0, Ts=1563.0,
                Tl=1623.0, latent_heat=270000.0, heat_source=0,
                cp=G.LinearClip(0.2441, 338.39, 300.0, 1563.0),
                k=G.LinearClip(0.0163105, 4.5847, 300.0, 1563.0))
    args["mesh"] = G.mesh3d(dom, N)
    args["mesh_local"] = G.mesh3d([0.75 * dom[0], 0.5 * dom[1], 0.4 * dom[2]], NL)
    return args
