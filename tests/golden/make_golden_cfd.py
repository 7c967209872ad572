"""Generate ``tests/golden/cfd_am3d.npz`` by running the reference's OWN
``jax_am/cfd/cfd_am.py`` (from the tree given by --ref or JAX_AM_REF) in this container.

JAX is not installed and cannot be, so ``jax_standin.py`` supplies ``jax``
(NumPy arithmetic, PyTorch autograd for ``jax.jacrev``, a restatement of
``jax.scipy.sparse.linalg.bicgstab``).  ``meshio`` output is not used: the
meshio mesh argument is a placeholder and ``write_sols`` is not called.

What is exercised, unmodified: ``mesh3d``, ``AM_3d.__init__`` and
``time_integration`` -> ``energy_eqn.update`` (``poisson`` residual, ``jacrev``
Jacobian, ``solver_nonlinear``), ``velocity_eqn.update`` (``solver_linear``
for the three momentum components and the pressure, the Marangoni boundary
condition), ``update_convective_terms`` (``get_face_vels``, ``div``),
``gradient``, the tool path and the moving local box, for a surface-flux case
and a body-source case.

Run from the repository root:
``python tests/golden/make_golden_cfd.py --ref <reference tree>``
"""
import contextlib
import importlib.util
import io
import os
import sys
import tempfile

import numpy as onp

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from ref_path import reference_root  # noqa: E402

REF = reference_root()
import jax_standin  # noqa: E402

jax_standin.install()
import jax.numpy as jnp  # noqa: E402  (the stand-in)

H = 5e-6
GRID = (12, 8, 5)
LOCAL = (8, 4, 3)
STEPS = 5
BASE = dict(rho=8440.0, visco=7e-3, Marangoni=-2e-5, dt=1e-6, t_OFF=1.0, speed=5.0,
            X0=[2e-5, 2e-5, 2.5e-5], rb=2e-5, eta=0.43, P=30.0, T_ref=300.0, Ts=1563.0,
            Tl=1623.0, latent_heat=270000.0, h=10.0, emissivity=0.3)
# cp and k of the reference drivers: a * clip(T, lo, hi) + b
CP = (0.2441, 338.39, 300.0, 1563.0)
K = (0.0163105, 4.5847, 300.0, 1563.0)
CASES = {
    "surface": dict(BASE, heat_source=0),
    "body": dict(BASE, heat_source=1, phi=4e-16, h=0.0, emissivity=0.0),
}


def load_cfd_am():
    path = os.path.join(REF, "jax_am", "cfd", "cfd_am.py")
    spec = importlib.util.spec_from_file_location("ref_cfd_am", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def run_case(cfd, args, tmp):
    mesh = cfd.mesh3d([GRID[0] * H, GRID[1] * H, GRID[2] * H], list(GRID))
    mesh_local = cfd.mesh3d([LOCAL[0] * H, LOCAL[1] * H, LOCAL[2] * H], list(LOCAL))
    a = dict(args)
    a["mesh"], a["mesh_local"], a["meshio_mesh"] = mesh, mesh_local, None
    a["cp"] = lambda T: CP[0] * jnp.clip(T, CP[2], CP[3]) + CP[1]
    a["k"] = lambda T: K[0] * jnp.clip(T, K[2], K[3]) + K[1]
    a["data_dir"] = tmp
    with contextlib.redirect_stdout(io.StringIO()):
        solver = cfd.AM_3d(a)
    out = {k: [] for k in ("T", "vel", "conv_T", "conv", "grad_p0", "solidID")}
    for _ in range(STEPS):
        solver.time_integration()
        for k in out:
            out[k].append(onp.asarray(getattr(solver, k), dtype=onp.float64).copy())
    return {k: onp.stack(v) for k, v in out.items()}


def main():
    cfd = load_cfd_am()
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, args in CASES.items():
            res = run_case(cfd, args, tmp)
            for k, v in res.items():
                arrays[f"{name}_{k}"] = v
            print(name, "T max per step", [float(t.max()) for t in res["T"]],
                  "|vel| max", float(onp.abs(res["vel"]).max()))
    arrays["grid"] = onp.array(GRID)
    arrays["local"] = onp.array(LOCAL)
    arrays["h"] = onp.array(H)
    arrays["steps"] = onp.array(STEPS)
    arrays["cp"] = onp.array(CP)
    arrays["k"] = onp.array(K)
    onp.savez_compressed(os.path.join(HERE, "cfd_am3d.npz"), **arrays)


if __name__ == "__main__":
    main()
