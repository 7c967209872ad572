"""The on-device diagnostics (PFSolver.inspect_sol's metrics, energy and
mass, argmax map) against the oracle.  Tolerances: counts, max T and the
argmax map exact; mass 1e-12 relative (compensated sums); energy 1e-6
relative (float32 per-cell energy densities, compensated accumulation)."""
import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.cases import f32, pf_case

pytestmark = pytest.mark.gpu
ENERGY_RTOL = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


@pytest.mark.parametrize("shape,n,bc", [((9, 7, 5), 5, None), ((17, 13, 6), 20, "periodic"),
                                        ((4, 4, 4), 33, None), ((31, 2, 3), 64, None),
                                        ((64, 48, 40), 20, None), ((50, 40, 30), 7, "periodic"),
                                        ((2, 1, 1), 1, None), ((3, 1, 2), 12, None),
                                        ((10, 9, 8), 4, ("periodic", "neumann", "periodic")),
                                        ((33, 5, 7), 8, None), ((40, 17, 3), 16, "periodic"),
                                        ((1, 1, 37), 20, None), ((90, 70, 20), 20, "periodic")])
def test_diag_vs_oracle(shape, n, bc):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    poly, eta, T, pf_args, oargs, obc = pf_case(shape, n, 0.0, seed=12, bc=bc)
    s = PFSolver(pf_args, poly)
    eta0 = np.roll(eta, 1, axis=1)
    ties = np.zeros(n)
    ties[[0, n - 1]] = np.float32(0.7)  # a tie: first maximum wins
    eta[0] = ties
    eta[1] = 0.0  # all zero: index 0
    d = s.diagnostics(eta, T, eta0)
    m = O.inspect(eta, eta0, T, oargs["T_liquidus"])
    assert d["n_ori_changed"] == round(m["pct_ori_changed"] * len(eta) / 100)
    assert d["pct_liquid"] == pytest.approx(m["pct_liquid"], abs=1e-12)
    assert d["max_T"] == m["max_T"]
    assert d["n_nonfinite"] == 0
    np.testing.assert_allclose(d["mass"], eta.sum(axis=0), rtol=1e-12)
    e_ref = O.free_energy(eta, T, oargs, None, obc)
    assert d["energy"] == pytest.approx(e_ref, rel=ENERGY_RTOL)
    am = s.argmax(torch.tensor(eta, dtype=torch.float32, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(am, np.argmax(eta.astype(np.float32), axis=1))


def test_inspect_sol_raises_on_nan(capsys):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    poly, eta, T, pf_args, oargs, obc = pf_case((5, 5, 5), 4, 0.0, seed=13)
    s = PFSolver(pf_args, poly)
    eta[17, 2] = np.nan
    eta[33, 0] = np.inf
    d = s.diagnostics(eta, T)
    assert d["n_nonfinite"] == 2
    with pytest.raises(ValueError):
        s.inspect_sol(eta, eta, T, np.arange(11), 10)
    assert "percent of change of orientations" in capsys.readouterr().out


@pytest.mark.parametrize("shape,n,bc", [((17, 13, 6), 20, "periodic"), ((9, 7, 5), 5, None),
                                        ((64, 48, 40), 12, None), ((4, 4, 4), 33, None),
                                        ((31, 2, 3), 64, None), ((50, 40, 30), 7, "periodic"),
                                        ((2, 1, 1), 1, None), ((100, 50, 25), 20, None)])
def test_inspect_matches_full_diagnostics(shape, n, bc):
    """pfg_pf_inspect (the inspect_sol metrics only) gives the same counts,
    max T and argmax map as the full reduction, and zero energy and mass:
    with first-maximum ties, an all-zero cell, NaN and Inf values, partial
    last chunks of 32 cells and n from 1 to 64."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    poly, eta, T, pf_args, oargs, obc = pf_case(shape, n, 0.0, seed=5, bc=bc)
    s = PFSolver(pf_args, poly)
    eta0 = np.roll(eta, 1, axis=1)
    N = len(eta)
    ties = np.zeros(n, dtype=eta.dtype)
    ties[[0, n - 1]] = 0.7
    eta[0] = ties
    if N > 1:
        eta[1] = 0.0
    if N > 2:
        eta[N - 1, n // 2] = np.nan  # NaN wins the argmax
        eta[N // 2, 0] = np.inf
    full = s.diagnostics(eta, T, eta0)
    light = s.inspect(eta, T, eta0)
    for key in ("n_ori_changed", "n_liquid", "n_nonfinite", "max_T", "n_cells"):
        assert light[key] == full[key], key
    assert light["n_nonfinite"] == (2 if N > 2 else 0)
    assert light["energy"] == 0.0 and not np.any(light["mass"])
    m = O.inspect(eta, eta0, T, oargs["T_liquidus"])
    assert light["pct_liquid"] == pytest.approx(m["pct_liquid"], abs=1e-12)
    # argmax maps of both kernels, and numpy's (NaN first, then first maximum)
    ed = torch.tensor(eta, dtype=torch.float32, device="cuda")
    Td = torch.tensor(np.asarray(T, dtype=np.float32).reshape(-1), device="cuda")
    maps = []
    for entry in ("pfg_pf_diag", "pfg_pf_inspect"):
        am = torch.empty(N, dtype=torch.int32, device="cuda")
        s._diag(ed, Td, None, am, False, entry)
        maps.append(am.cpu().numpy())
    np.testing.assert_array_equal(maps[0], maps[1])
    np.testing.assert_array_equal(maps[1], np.argmax(eta.astype(np.float32), axis=1))


def test_inspect_async_is_ordered_before_later_steps():
    """inspect_async's record is the state it was given even when further
    steps are enqueued before result() is read; it equals inspect's."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.runner import HeatPFRun, single_track
    from tests.cases import GAMMA_DEFAULTS
    poly, eta, _, pf_args, _, _ = pf_case((48, 32, 16), 20, 0.15, seed=3, h=(1e-6,) * 3)
    s = PFSolver(pf_args, poly)
    run = HeatPFRun(s, dict(GAMMA_DEFAULTS), single_track(5e-6, 16e-6, 0.8, 200.0, 1e-3),
                    dt=2e-9, eta0=torch.tensor(eta, dtype=torch.float32, device="cuda"))
    run.run(20)
    ref = s.inspect(run.state, run.T_ghosted, eta0=eta, T_ghosted=True)
    pend = s.inspect_async(run.state, run.T_ghosted, eta0=eta, T_ghosted=True)
    run.run(40)  # overwrites both state buffers before the record is read
    got = pend.result()
    later = s.inspect(run.state, run.T_ghosted, eta0=eta, T_ghosted=True)
    for k in ("max_T", "n_cells", "n_ori_changed", "n_liquid", "n_nonfinite"):
        assert got[k] == ref[k], k
    assert later["max_T"] != ref["max_T"]  # the later state differs
    assert pend.done()


@pytest.mark.parametrize("n", [20, 12])
def test_diag_non_finite_values(n):
    """The full record with NaN and infinity in eta (lane-per-cell path for
    n <= 20): the count of non-finite values and np.argmax's rules (the first
    NaN wins; infinity is a maximum)."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    poly, eta, T, pf_args, oargs, obc = pf_case((21, 11, 5), n, 0.0, seed=14)
    s = PFSolver(pf_args, poly)
    eta = eta.copy()
    eta[3, 5] = np.nan
    eta[3, 2] = np.nan
    eta[40, 1] = np.inf
    eta[77, n - 1] = -np.inf
    # eta0 = eta: the record's own argmax must equal the reference argmax of
    # eta0 in every cell, NaN and infinity cells included
    d = s.diagnostics(eta, T, eta)
    assert d["n_nonfinite"] == 4
    assert d["n_ori_changed"] == 0
    got = s.argmax(torch.tensor(eta, dtype=torch.float32, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(got, np.argmax(eta.astype(np.float32), axis=1))
    m = O.inspect(np.nan_to_num(eta), eta, T, oargs["T_liquidus"])
    assert d["max_T"] == m["max_T"]

