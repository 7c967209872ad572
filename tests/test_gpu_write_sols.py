"""``PFSolver.write_sols`` (``allen_cahn.py:182-210``): the VTU file read
back holds T, the argmax orientation map (first maximum, as ``np.argmax``)
and the IPF colours gathered by that map, with liquid cells (T >
T_liquidus) black, exactly as the reference computes them with NumPy."""
import numpy as np
import pytest
import torch

from tests.cases import pf_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


@pytest.mark.parametrize("with_rgb", [True, False])
def test_write_sols_round_trip(tmp_path, with_rgb):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.vtu import read_vtu
    poly, eta, T, pf_args, _, _ = pf_case((9, 7, 5), 6, 0.15, seed=11)
    rng = np.random.default_rng(12)
    rgb = rng.random((3, 6, 3))
    if with_rgb:
        poly.unique_oris_rgb = rgb
    T = T.copy()
    T[::7] = pf_args["T_liquidus"]          # exactly at T_liquidus: not liquid (strict >)
    T[3::11] = pf_args["T_liquidus"] + 5.0  # liquid
    eta = eta.copy()
    eta[::13, 0] = eta[::13, 1] = 2.0       # ties: the first maximum wins
    pf_args = dict(pf_args, data_dir=str(tmp_path), write_sol_interval=5)
    s = PFSolver(pf_args, poly)
    s.write_sols(torch.tensor(eta, dtype=torch.float32, device="cuda"),
                 torch.tensor(T, dtype=torch.float32, device="cuda"), 10)
    d = read_vtu(str(tmp_path / "vtk/pf/sols/u002.vtu"))
    e32 = eta.astype(np.float32)
    T32 = T.reshape(-1).astype(np.float32)
    inds = np.argmax(e32, axis=1)
    np.testing.assert_array_equal(d["ori_inds"], inds.astype(np.int32))
    np.testing.assert_array_equal(d["T"], T32)
    liquid = T32 > np.float32(pf_args["T_liquidus"])
    assert liquid.any() and (~liquid).any()
    for k, name in enumerate(("ipf_x", "ipf_y", "ipf_z")):
        if not with_rgb:
            assert name not in d
            continue
        want = np.take(rgb[k], inds, axis=0)
        want[liquid] = 0.0
        np.testing.assert_array_equal(d[name], want)
