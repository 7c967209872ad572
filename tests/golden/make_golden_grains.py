"""Generate ``tests/golden/grains.npz`` by running the reference's OWN grain
post-processing (``jax_am/phase_field/utils.py``: ``compute_edges_in_order``,
``BFS``, ``get_aspect_ratio_inputs``, ``compute_aspect_ratios_and_vols``,
the body of ``process_eta`` at utils.py:181-310) in this container.

``jax`` is the stand-in of ``jax_standin.py``; ``orix``, ``meshio`` and
``matplotlib`` (imported by utils.py for orientation sampling, file input and
plotting, none of them on this path) are empty stubs.  scikit-learn's ``PCA``
(imported by utils.py) is the real one.  ``process_eta`` itself reads a VTU
file; its computation is reproduced here from in-memory arrays exactly as it
builds them: ``nonliquid = T < T_liquidus``, uniform cell volumes
``domain_vol / N`` and the cell centres as centroids.

Cases: Voronoi-like orientation maps with a liquid pool (T above the
liquidus), isolated single cells, 2- to 4-cell grains (aspect ratio 1 by the
reference's small-grain rule), straight rods and thin plates.

Run from the repository root:
``python tests/golden/make_golden_grains.py --ref <reference tree>``
"""
import contextlib
import importlib.util
import io
import os
import sys
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


for _name in ("orix", "orix.quaternion", "orix.plot", "orix.vector", "meshio", "matplotlib",
              "matplotlib.pyplot"):
    _stub(_name)


def _load_utils():
    path = os.path.join(REF, "jax_am", "phase_field", "utils.py")
    spec = importlib.util.spec_from_file_location("ref_pf_utils", path)
    mod = importlib.util.module_from_spec(spec)
    with contextlib.redirect_stdout(io.StringIO()):
        spec.loader.exec_module(mod)
    return mod


U = _load_utils()


def reference_grains(ori, T, T_liq, Nx, Ny, Nz, h):
    """process_eta's computation (utils.py:181-214) on in-memory arrays."""
    pf_args = dict(Nx=Nx, Ny=Ny, Nz=Nz, num_oris=int(ori.max()) + 1, T_liquidus=T_liq,
                   domain_x=Nx * h, domain_y=Ny * h, domain_z=Nz * h)
    N = Nx * Ny * Nz
    nonliquid = T.reshape(-1) < pf_args["T_liquidus"]
    zz, yy, xx = onp.meshgrid(onp.arange(Nz), onp.arange(Ny), onp.arange(Nx), indexing="ij")
    centroids = onp.stack(((xx.ravel() + 0.5) * h, (yy.ravel() + 0.5) * h, (zz.ravel() + 0.5) * h),
                          axis=1)
    domain_vol = pf_args["domain_x"] * pf_args["domain_y"] * pf_args["domain_z"]
    volumes = domain_vol / N * onp.ones(N)
    with contextlib.redirect_stdout(io.StringIO()):
        edges_in_order = U.compute_edges_in_order(pf_args)
        grains = U.BFS(edges_in_order, nonliquid, ori, pf_args)
        vols, cents = U.get_aspect_ratio_inputs(grains, volumes, centroids)
        res = U.compute_aspect_ratios_and_vols(vols, cents)
    labels = -onp.ones(N, dtype=onp.int64)
    for k, g in enumerate(grains):
        labels[onp.array(g)] = k
    return labels, onp.array(res[0]), onp.array(res[1])


def make_case(rng, Nx, Ny, Nz, n, seeds, liquid_frac, h=1e-6):
    N = Nx * Ny * Nz
    zz, yy, xx = onp.meshgrid(onp.arange(Nz), onp.arange(Ny), onp.arange(Nx), indexing="ij")
    pts = onp.stack((xx.ravel(), yy.ravel(), zz.ravel()), axis=1).astype(float)
    sp = rng.uniform(0, 1, (seeds, 3)) * onp.array([Nx, Ny, Nz])
    d2 = ((pts[:, None, :] - sp[None, :, :]) ** 2).sum(-1)
    grain = onp.argmin(d2, axis=1)
    ori = rng.integers(0, n, seeds)[grain]
    # speckle: isolated cells and small clusters of other orientations
    flip = rng.random(N) < 0.03
    ori[flip] = rng.integers(0, n, int(flip.sum()))
    T = rng.uniform(1400.0, 1600.0, N).astype(onp.float32)
    # a liquid pool around a random centre, and cells exactly at the liquidus
    c = rng.uniform(0, 1, 3) * onp.array([Nx, Ny, Nz])
    r = (liquid_frac * N * 3 / (4 * onp.pi)) ** (1 / 3)
    T[((pts - c) ** 2).sum(-1) < r * r] = 1700.0
    T[rng.random(N) < 0.02] = 1623.0
    return ori.astype(onp.int64), T


def make_shapes(Nx, Ny, Nz):
    """Rods along each axis, a plate, an L-shape, tiny grains in a 0 matrix."""
    ori = onp.zeros((Nz, Ny, Nx), dtype=onp.int64)
    ori[1, 1, 1:Nx - 1] = 1          # rod along x
    ori[1:Nz - 1, 3, 3] = 2          # rod along z
    ori[2, 1:Ny - 1, Nx - 2] = 3     # rod along y
    ori[Nz - 2, 4:7, 4:9] = 4        # plate
    ori[3, 6, 6] = 5                 # single cell
    ori[3, 8, 6:8] = 5               # two cells (same orientation, separate grain)
    ori[4, 8:10, 8:10] = 6           # four cells
    T = onp.full(ori.size, 1500.0, dtype=onp.float32)
    return ori.ravel(), T


def main():
    rng = onp.random.default_rng(11)
    cases = {}
    for name, (Nx, Ny, Nz, n, seeds, lf) in {
        "voronoi_a": (14, 11, 9, 5, 30, 0.1),
        "voronoi_b": (21, 8, 13, 9, 60, 0.2),
        "voronoi_c": (10, 10, 10, 3, 12, 0.0),
    }.items():
        ori, T = make_case(rng, Nx, Ny, Nz, n, seeds, lf)
        cases[name] = (Nx, Ny, Nz, ori, T)
    ori, T = make_shapes(12, 11, 7)
    cases["shapes"] = (12, 11, 7, ori, T)
    out = {}
    for name, (Nx, Ny, Nz, ori, T) in cases.items():
        labels, vols, ars = reference_grains(ori, T, 1623.0, Nx, Ny, Nz, 1e-6)
        out[f"{name}_shape"] = onp.array([Nx, Ny, Nz])
        out[f"{name}_ori"] = ori
        out[f"{name}_T"] = T
        out[f"{name}_labels"] = labels
        out[f"{name}_vols"] = vols
        out[f"{name}_ars"] = ars
        print(f"{name}: {len(vols)} grains, {int((labels < 0).sum())} liquid cells, "
              f"aspect ratios {onp.nanmin(ars):.3f} .. {onp.nanmax(ars):.3f}")
    out["T_liquidus"] = onp.array(1623.0)
    out["h"] = onp.array(1e-6)
    onp.savez_compressed(os.path.join(HERE, "grains.npz"), **out)


if __name__ == "__main__":
    main()
