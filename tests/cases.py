"""Seeded test inputs shared by the CPU and GPU test files.

Every value handed to the GPU is float32; the oracle gets the same values
widened to float64, so the comparison measures the kernels' float32
arithmetic and not input rounding."""
import numpy as np

from jax_am_gb300.phase_field.utils import grain_directions, random_quaternions

PF_DEFAULTS = dict(dim=3, T_liquidus=1623.0, gas_const=8.3, Qg=1.4e5, L0=3.5e3,
                   kappa_g=2.77e-6, m_g=2.4e5, ad_hoc=1.0)

GAMMA_DEFAULTS = dict(eta=0.4, r=5e-5, rho=8440.0, h=10.0, eps=0.4, SB=5.67e-8, T0=300.0,
                      Ts=1563.0, Tl=1623.0)
GAMMA_DEFAULTS["L"] = 290e3 / (GAMMA_DEFAULTS["Tl"] - GAMMA_DEFAULTS["Ts"])


class Poly:
    """Duck-typed polycrystal: what ``PFSolver`` reads from ``Field``."""

    def __init__(self, shape_xyz, h, n, rng):
        Nx, Ny, Nz = shape_xyz
        self.mesh_h_xyz = tuple(float(np.float32(v)) for v in h)
        self.quaternions = random_quaternions(n, rng)
        d = grain_directions(self.quaternions)
        self.unique_grain_directions = d.astype(np.float32).astype(np.float64)
        self.cell_ori_inds = rng.integers(0, n, Nx * Ny * Nz)
        zs, ys, xs = np.meshgrid((np.arange(Nz) + 0.5) * h[2], (np.arange(Ny) + 0.5) * h[1],
                                 (np.arange(Nx) + 0.5) * h[0], indexing="ij")
        self.centroids = np.stack((xs.ravel(), ys.ravel(), zs.ravel()), axis=1)


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def pf_case(shape_xyz, n, anisotropy=0.0, seed=0, h=(1e-6, 1.1e-6, 0.9e-6), bc=None,
            force=False, noise=0.5, T_range=(1400.0, 2100.0)):
    """A polycrystal, a perturbed one-hot eta, a temperature field, the
    pf_args dict for PFSolver and the args dict for the oracle."""
    rng = np.random.default_rng(seed)
    Nx, Ny, Nz = shape_xyz
    N = Nx * Ny * Nz
    poly = Poly(shape_xyz, h, n, rng)
    eta = np.zeros((N, n))
    eta[np.arange(N), poly.cell_ori_inds] = 1.0
    mask = rng.random(N) < noise
    eta[mask] = rng.random((int(mask.sum()), n))
    eta = f32(eta)
    T = rng.uniform(*T_range, (N, 1))
    T[rng.random(N) < 0.05] = PF_DEFAULTS["T_liquidus"]
    T = f32(T)
    pf_args = dict(PF_DEFAULTS, num_oris=n, Nx=Nx, Ny=Ny, Nz=Nz, anisotropy=anisotropy)
    if bc is not None:
        pf_args["bc"] = bc
    if force:
        pf_args["force_liquid_zero"] = True
        pf_args["liquid_shift"] = 1.0
    oargs = dict(pf_args, h=poly.mesh_h_xyz)
    obc = ("neumann",) * 3 if bc is None else ((bc,) * 3 if isinstance(bc, str) else tuple(bc))
    return poly, eta, T, pf_args, oargs, obc
