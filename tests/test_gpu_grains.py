"""Grain segmentation on the GPU (pfg_grains + segment_grains) against the
reference's own BFS / PCA output (golden vectors from
tests/golden/make_golden_grains.py), against the oracle's restatement on
random maps, and against scipy.ndimage's connected-component labelling at a
larger size.  Tolerances: labels and cell counts exact; volumes 1e-12
relative; aspect ratios 1e-9 relative, collinear grains (inf, or a huge
finite value where the reference's PCA rounds) compared as a class."""
import os

import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.test_oracle_golden import _check_aspect_ratios

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def _args(Nx, Ny, Nz, h=1e-6, n=None):
    a = dict(Nx=Nx, Ny=Ny, Nz=Nz, h=h, T_liquidus=1623.0)
    if n is not None:
        a["num_oris"] = n
    return a


@pytest.mark.parametrize("case", ["voronoi_a", "voronoi_b", "voronoi_c", "shapes"])
def test_grains_match_reference_golden(case):
    from jax_am_gb300.phase_field.grains import segment_grains
    d = np.load(os.path.join(G, "grains.npz"))
    Nx, Ny, Nz = (int(v) for v in d[f"{case}_shape"])
    res = segment_grains(_args(Nx, Ny, Nz), d[f"{case}_ori"], d[f"{case}_T"])
    np.testing.assert_array_equal(res["labels"].cpu().numpy(), d[f"{case}_labels"])
    np.testing.assert_allclose(res["volumes"], d[f"{case}_vols"], rtol=1e-12)
    _check_aspect_ratios(res["aspect_ratios"], d[f"{case}_ars"])


def _random_map(rng, Nx, Ny, Nz, n, seeds, liquid):
    zz, yy, xx = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    pts = np.stack((xx.ravel(), yy.ravel(), zz.ravel()), axis=1).astype(float)
    sp = rng.uniform(0, 1, (seeds, 3)) * np.array([Nx, Ny, Nz])
    from scipy.spatial import cKDTree
    grain = cKDTree(sp).query(pts)[1]
    ori = rng.integers(0, n, seeds)[grain]
    flip = rng.random(len(ori)) < 0.02
    ori[flip] = rng.integers(0, n, int(flip.sum()))
    T = rng.uniform(1400.0, 1600.0, len(ori)).astype(np.float32)
    T[rng.random(len(ori)) < liquid] = 1700.0
    return ori.astype(np.int32), T


@pytest.mark.parametrize("shape,n,seeds,liquid", [((33, 17, 9), 6, 40, 0.05),
                                                  ((1, 1, 1), 1, 1, 0.0),
                                                  ((64, 1, 1), 2, 5, 0.3),
                                                  ((5, 40, 3), 3, 9, 0.0)])
def test_grains_match_oracle(shape, n, seeds, liquid):
    from jax_am_gb300.phase_field.grains import segment_grains
    rng = np.random.default_rng(sum(shape) + n)
    Nx, Ny, Nz = shape
    ori, T = _random_map(rng, Nx, Ny, Nz, n, seeds, liquid)
    res = segment_grains(_args(Nx, Ny, Nz), ori, T)
    labels, K = O.grain_components(ori, T, 1623.0, Nx, Ny, Nz)
    vols, ars = O.grain_volumes_and_aspect_ratios(labels, K, Nx, Ny, Nz, 1e-6)
    np.testing.assert_array_equal(res["labels"].cpu().numpy(), labels)
    np.testing.assert_allclose(res["volumes"], vols, rtol=1e-12)
    _check_aspect_ratios(res["aspect_ratios"], ars)


def test_ghosted_temperature_and_small_capacity():
    """The ghosted heat state gives the same grains as the per-cell T, and a
    grain array too small for the first call is regrown."""
    from jax_am_gb300.phase_field.grains import segment_grains
    rng = np.random.default_rng(3)
    Nx, Ny, Nz = 20, 14, 11
    ori, T = _random_map(rng, Nx, Ny, Nz, 4, 30, 0.1)
    Tg = np.full((Nz + 2, Ny + 2, Nx + 2), 5000.0, dtype=np.float32)  # ghosts never read
    Tg[1:-1, 1:-1, 1:-1] = T.reshape(Nz, Ny, Nx)
    a = segment_grains(_args(Nx, Ny, Nz), ori, T)
    b = segment_grains(_args(Nx, Ny, Nz), ori, Tg, T_ghosted=True, max_grains=3)
    assert len(a["cells"]) > 3
    assert torch.equal(a["labels"], b["labels"])
    np.testing.assert_array_equal(a["cells"], b["cells"])
    np.testing.assert_array_equal(a["aspect_ratios"], b["aspect_ratios"])


def test_grains_match_scipy_labelling_at_scale():
    """160 x 120 x 60 cells, 3000 Voronoi grains with 20 orientations, a liquid
    pool: the components equal scipy.ndimage.label's per orientation (same
    partition of the cells), and the cell counts add up."""
    from scipy import ndimage
    from jax_am_gb300.phase_field.grains import segment_grains
    rng = np.random.default_rng(7)
    Nx, Ny, Nz = 160, 120, 60
    ori, T = _random_map(rng, Nx, Ny, Nz, 20, 3000, 0.0)
    zz, yy, xx = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    pool = ((xx - 80) ** 2 + (yy - 60) ** 2 + (zz - 60) ** 2 < 30 ** 2).ravel()
    T[pool] = 1700.0
    res = segment_grains(_args(Nx, Ny, Nz), ori, T)
    lab = res["labels"].cpu().numpy().reshape(Nz, Ny, Nx)
    solid = (T < 1623.0).reshape(Nz, Ny, Nx)
    o3 = ori.reshape(Nz, Ny, Nx)
    total = 0
    for k in range(20):
        ref, nk = ndimage.label(solid & (o3 == k))
        total += nk
        mine = lab[solid & (o3 == k)]
        theirs = ref[solid & (o3 == k)]
        # same partition: the map ours -> scipy's is a bijection
        pairs = np.unique(np.stack((mine, theirs), axis=1), axis=0)
        assert len(pairs) == nk == len(np.unique(mine))
    assert len(res["cells"]) == total
    assert int(res["cells"].sum()) == int(solid.sum())
    assert (lab[~solid] == -1).all()
    # grains are listed by orientation, then by their smallest cell
    keys = np.stack((res["ori"], res["first_cell"]), axis=1)
    assert (np.lexsort((keys[:, 1], keys[:, 0])) == np.arange(len(keys))).all()


def test_process_eta_from_written_solution(tmp_path):
    """PFSolver.write_sols then process_eta (the reference's post-processing
    entry) on a short run, against the oracle on the same written arrays."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.grains import process_eta
    from jax_am_gb300.phase_field.utils import Field
    Nx, Ny, Nz = 30, 24, 12
    pf_args = dict(Nx=Nx, Ny=Ny, Nz=Nz, h=1e-6, num_grains=25, num_oris=8, T_liquidus=1623.0,
                   gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6, m_g=2.4e5,
                   anisotropy=0.0, ad_hoc=1.0, data_dir=str(tmp_path), write_sol_interval=1,
                   domain_x=Nx * 1e-6, domain_y=Ny * 1e-6, domain_z=Nz * 1e-6)
    poly = Field(pf_args, seed=4)
    s = PFSolver(pf_args, poly)
    rng = np.random.default_rng(5)
    T = torch.tensor(rng.uniform(1500.0, 1700.0, (s.N, 1)), dtype=torch.float32, device="cuda")
    state = (s.ini_cond(), 0.0)
    for k in range(20):
        state, _ = s.stepper(state, (k + 1) * 1e-8, [T])
    s.write_sols(state[0], T, 13)
    vols, ars = process_eta(pf_args, step=13)
    d = np.load(tmp_path / "numpy/pf/sols/u013.npz")
    from jax_am_gb300.phase_field.vtu import read_vtu
    v = read_vtu(str(tmp_path / "vtk/pf/sols/u013.vtu"))
    np.testing.assert_array_equal(v["ori_inds"], d["ori_inds"])
    np.testing.assert_array_equal(v["T"], d["T"])
    labels, K = O.grain_components(d["ori_inds"], d["T"], 1623.0, Nx, Ny, Nz)
    ov, oa = O.grain_volumes_and_aspect_ratios(labels, K, Nx, Ny, Nz, 1e-6)
    assert len(vols) == K
    np.testing.assert_allclose(vols, ov, rtol=1e-12)
    _check_aspect_ratios(np.array(ars), oa)
