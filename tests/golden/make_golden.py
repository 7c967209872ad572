"""Generate the golden vectors in ``tests/golden/*.npz`` by running the
reference's OWN source files (JAX-AM, from the tree given by --ref or JAX_AM_REF) in this
container.

JAX is not installed and cannot be, so ``jax_standin.py`` supplies ``jax`` /
``jax.numpy`` (NumPy arithmetic, PyTorch autograd for ``jax.grad``).  Modules
the reference imports only for meshing, plotting or file output (``meshio``,
``orix``, ``matplotlib``, ``pyfiglet``, the CFD solver, ``common``) are
replaced by empty stubs; none of them is on the computed path.

What is exercised, unmodified:

* ``jax_am/phase_field/allen_cahn.py``: ``PFSolver.__init__``, ``ini_cond``,
  ``stepper`` (-> ``explicit_euler`` -> ``state_rhs`` incl. ``jax.grad`` of
  ``local_energy_fn`` and the anisotropy helper), ``get_force_eta_fn`` and
  ``inspect_sol`` (stdout parsed).
* ``jax_am/cfd/gamma.py``: ``update_T`` in float64 and float32.
* ``applications/phase_field/{solidification,simple,multi_scan}/example.py``:
  ``get_T_fn`` and ``read_path``.

Run from the repository root:
``python tests/golden/make_golden.py --ref <reference tree>``
"""
import contextlib
import importlib.util
import io
import os
import re
import sys
import tempfile
import types
from unittest import mock

import numpy as onp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from ref_path import reference_root  # noqa: E402

REF = reference_root()
import jax_standin  # noqa: E402

jax_standin.install()


def _stub(name):
    mod = types.ModuleType(name)
    mod.__getattr__ = lambda attr: mock.MagicMock(name=f"{name}.{attr}")
    sys.modules[name] = mod
    return mod


class _Figlet:
    def __init__(self, **_k):
        pass

    def renderText(self, _s):
        return ""


_stub("pyfiglet").Figlet = _Figlet
for _name in ("meshio", "orix", "orix.quaternion", "orix.plot", "orix.vector", "matplotlib",
              "matplotlib.pyplot", "jax_am.cfd.cfd_am", "jax_am.phase_field.utils",
              "jax_am.common", "yaml", "pandas"):
    _stub(_name)

sys.path.insert(0, REF)
from jax_am.phase_field import allen_cahn as ref_ac  # noqa: E402
from jax_am.cfd import gamma as ref_gamma  # noqa: E402
from scipy.spatial.transform import Rotation  # noqa: E402

A = jax_standin.asarray
PF_KEYS = dict(dim=3, T_liquidus=1623.0, gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6,
               m_g=2.4e5, ad_hoc=1.0)


def _load_example(rel):
    path = os.path.join(REF, rel)
    spec = importlib.util.spec_from_file_location("ref_" + rel.replace("/", "_")[:-3], path)
    mod = importlib.util.module_from_spec(spec)
    with contextlib.redirect_stdout(io.StringIO()):
        spec.loader.exec_module(mod)
    return mod


class _Poly:
    pass


def grain_directions(quats_scalar_first):
    """(3, n, 3) rotated cube axes, as ``utils.py:104-109`` builds them."""
    scipy_quat = onp.concatenate((quats_scalar_first[:, 1:], quats_scalar_first[:, :1]), axis=1)
    r = Rotation.from_quat(scipy_quat)
    return onp.stack((r.apply([1.0, 0, 0]), r.apply([0, 1.0, 0]), r.apply([0, 0, 1.0])))


def _blocky_polycrystal(rng, Nz, Ny, Nx, n):
    """Cells in 2x2x2 blocks share an orientation, so some edges are exactly
    zero (exercises the reference's NaN-to-zero branch)."""
    zz, yy, xx = onp.meshgrid(onp.arange(Nz) // 2, onp.arange(Ny) // 2, onp.arange(Nx) // 2,
                              indexing="ij")
    block = (zz * 97 + yy * 31 + xx * 7).reshape(-1)
    return (block * 13 + rng.integers(0, n)) % n


def make_pf_case(name, rng, Nz, Ny, Nx, n, anisotropy, h, dt, steps, noise_frac):
    quats = Rotation.random(n, random_state=int(rng.integers(1 << 30))).as_quat()
    quats = onp.concatenate((quats[:, 3:], quats[:, :3]), axis=1)  # scalar-first, as orix
    dirs = grain_directions(quats)
    poly = _Poly()
    poly.mesh_h_xyz = h
    poly.unique_grain_directions = dirs
    N = Nz * Ny * Nx
    poly.centroids = onp.zeros((N, 3))
    poly.cell_ori_inds = _blocky_polycrystal(rng, Nz, Ny, Nx, n)
    args = dict(PF_KEYS, num_oris=n, Nx=Nx, Ny=Ny, Nz=Nz, anisotropy=anisotropy,
                data_dir=tempfile.mkdtemp())
    with contextlib.redirect_stdout(io.StringIO()):
        solver = ref_ac.PFSolver(args, poly)
        eta0 = onp.asarray(solver.ini_cond())
    # perturb a fraction of cells so that gradients and S are non-trivial
    mask = rng.random(N) < noise_frac
    eta_in = eta0.copy()
    eta_in[mask] = rng.random((mask.sum(), n))
    T = rng.uniform(1450.0, 2100.0, (N, 1))
    T[rng.random(N) < 0.1] = 1623.0  # exactly at the liquidus: zeta = 1/2
    state = (A(eta_in), 0.0)
    outs = []
    t = 0.0
    with contextlib.redirect_stdout(io.StringIO()):
        for _ in range(steps):
            t = t + dt
            state, _ = solver.stepper(state, t, [A(T)])
            outs.append(onp.asarray(state[0]))
    onp.savez_compressed(os.path.join(HERE, name), Nz=Nz, Ny=Ny, Nx=Nx, n=n,
                         anisotropy=anisotropy, h=onp.array(h), dt=dt, steps=steps,
                         grain_dirs=dirs, quats=quats, cell_ori_inds=poly.cell_ori_inds,
                         eta_ini=eta0, eta_in=eta_in, T=T, eta_out=onp.stack(outs),
                         pf_keys=onp.array(list(PF_KEYS.values())))
    return solver, eta_in, T, outs


def make_force_and_inspect(solver, eta_in, T, eta_out):
    force = ref_ac.get_force_eta_fn(solver.pf_args)
    eta_f, _ = force((A(eta_out), 0.0), A(T))
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        solver.inspect_sol(A(eta_out), A(eta_in), A(T), onp.arange(11), 10)
    text = buf.getvalue()
    vals = [float(v) for v in re.findall(r"= ([-0-9.eE+]+)%?", text)]
    onp.savez_compressed(os.path.join(HERE, "pf_force_inspect.npz"), eta=eta_out, T=T,
                         eta0=eta_in, eta_forced=onp.asarray(eta_f),
                         inspect=onp.array(vals[1:4]))


def make_heat_case(name, dtype, rng, nx, ny, nz, steps):
    g = dict(eta=0.4, r=5e-5, rho=8440.0, h=10.0, eps=0.4, SB=5.67e-8, T0=300.0, Ts=1563.0,
             Tl=1623.0)
    g["L"] = 290e3 / (g["Tl"] - g["Ts"])
    dx, dy, dz, dt = 5e-6, 6e-6, 4e-6, 1e-7
    x_ = onp.linspace(dx / 2.0, dx / 2.0 + dx * (nx - 1), nx)
    y_ = onp.linspace(dy / 2.0, dy / 2.0 + dy * (ny - 1), ny)
    z_ = onp.linspace(dz / 2.0, dz / 2.0 + dz * (nz - 1), nz)
    x, y, _ = onp.meshgrid(x_, y_, z_, indexing="ij")
    T0 = rng.uniform(300.0, 2200.0, (nx + 2, ny + 2, nz + 2))
    T0[..., :] = onp.where(rng.random(T0.shape) < 0.15, rng.uniform(1563.0, 1623.0, T0.shape), T0)
    T0 = T0.astype(dtype)
    xl0, yl, vel, P = 1.0e-5, 0.5 * ny * dy, 0.8, 200.0
    T = A(T0)
    outs, lasers = [], []
    for i in range(steps):
        xl = xl0 + vel * (i + 0.5) * dt
        gc = {k: dtype(v) for k, v in g.items()} if dtype == onp.float32 else g
        T = ref_gamma.update_T(T, dtype(xl), dtype(yl), A(x, dtype), A(y, dtype), dtype(P),
                               dtype(dx), dtype(dy), dtype(dz), dtype(dt), gc)
        outs.append(onp.asarray(T))
        lasers.append((xl, yl, P))
    onp.savez_compressed(os.path.join(HERE, name), T_in=T0, T_out=onp.stack(outs),
                         lasers=onp.array(lasers), dxyzt=onp.array([dx, dy, dz, dt]),
                         gamma=onp.array([g[k] for k in ("eta", "r", "rho", "h", "eps", "SB", "T0",
                                                        "Ts", "Tl", "L")]))


def make_tsources(rng):
    sol = _load_example("applications/phase_field/solidification/example.py")
    simple = _load_example("applications/phase_field/simple/example.py")
    multi = _load_example("applications/phase_field/multi_scan/example.py")
    poly = _Poly()
    poly.centroids = rng.uniform(0.0, 1e-4, (64, 3))
    args = dict(T_liquidus=1623.0, domain_x=1e-3, domain_y=2.4e-4, domain_z=1e-4, t_OFF=2.4e-3,
                T_ambient=300.0, vel=0.25, dt=2e-7,
                laser_path=dict(x_pos=[0.1e-3, 0.9e-3, 0.9e-3, 0.1e-3],
                                y_pos=[0.17e-3, 0.17e-3, 0.07e-3, 0.07e-3],
                                z_pos=[0.1e-3, 0.1e-3, 0.1e-3, 0.1e-3], switch=[1, 1, 1, 0]))
    t = 3.7e-4
    T_q = onp.asarray(sol.get_T_fn(poly, args)(t))
    T_r = onp.asarray(simple.get_T_fn(poly, args)(t))
    with contextlib.redirect_stdout(io.StringIO()):
        ts, xs, ys, zs, ps, mov = multi.read_path(args)
    i = 1234
    T_m = onp.asarray(multi.get_T_fn(poly, args)(ts[i], xs[i], ys[i], zs[i], ps[i], mov[i]))
    onp.savez_compressed(os.path.join(HERE, "tsources.npz"), centroids=poly.centroids, t=t,
                         T_quench=T_q, T_rosenthal=T_r, path_ts=ts, path_xs=xs, path_ys=ys,
                         path_zs=zs, path_ps=ps, path_dirs=mov, path_i=i, T_path=T_m)


def main():
    rng = onp.random.default_rng(20261203)
    make_pf_case("pf_iso.npz", rng, 4, 5, 6, 5, 0.0, (1e-6, 1.1e-6, 0.9e-6), 2e-8, 3, 0.5)
    s, e_in, T, outs = make_pf_case("pf_aniso.npz", rng, 6, 4, 8, 6, 0.15, (1e-6, 1e-6, 1.2e-6),
                                    2e-8, 3, 0.4)
    make_force_and_inspect(s, e_in, T, outs[-1])
    make_pf_case("pf_aniso_n20.npz", rng, 3, 4, 5, 20, 0.15, (1e-6, 1e-6, 1e-6), 1e-8, 2, 0.6)
    make_heat_case("heat_f64.npz", onp.float64, rng, 6, 5, 4, 3)
    make_heat_case("heat_f32.npz", onp.float32, rng, 7, 4, 5, 3)
    make_tsources(rng)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
