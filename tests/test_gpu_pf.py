"""Parity of the CUDA phase-field step with the FP64 oracle and with golden
vectors produced by the reference's own source.

Tolerance: max |d eta| <= 1e-4 after the listed steps (float32 kernel vs
float64 reference); argmax orientation maps are compared exactly and any
mismatched cells are counted."""
import os

import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.cases import f32, pf_case

pytestmark = pytest.mark.gpu

ETA_TOL = 1e-4
G = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


@pytest.fixture(params=[0, 1, 2, 3, 512],
                ids=["auto", "generic", "warp_cpasync", "tma256", "tma512"])
def variant(request):
    """Run a test on the warp-per-cells kernel and on the generic kernel."""
    from jax_am_gb300 import _lib
    lib = _lib.load()
    if request.param == 512:  # the TMA-fed kernel with one 512-thread CTA per SM
        assert lib.pfg_set_kernel_variant(3) == 0 and lib.pfg_tune(5, 512) == 0
    else:
        assert lib.pfg_set_kernel_variant(request.param) == 0
    yield request.param
    lib.pfg_set_kernel_variant(0)
    lib.pfg_tune(5, 0)
    assert _lib.device_error() == 0, "a bounded device-side wait ran out"


def _solver(pf_args, poly):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    return PFSolver(pf_args, poly)


def _run_gpu(solver, eta, T, dt, steps):
    state = (torch.tensor(eta, dtype=torch.float32, device="cuda"), 0.0)
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    t = 0.0
    for _ in range(steps):
        t += dt
        state, _ = solver.stepper(state, t, [Td])
    return state[0].double().cpu().numpy()


def _run_oracle(eta, T, oargs, dirs, bc, dt, steps, force=False):
    t = 0.0
    dt = float(np.float32(dt))
    for _ in range(steps):
        eta = O.explicit_euler(eta, t, t + dt, T, oargs, dirs, bc)
        if force:
            eta = O.force_liquid_zero(eta, T, oargs["T_liquidus"], oargs.get("liquid_shift", 1.0))
        t += dt
    return eta


def _argmax_mismatch(a, b):
    return int(np.sum(np.argmax(a, axis=1) != np.argmax(b, axis=1)))


@pytest.mark.parametrize("name", ["pf_iso.npz", "pf_aniso.npz", "pf_aniso_n20.npz"])
def test_matches_reference_golden(name, variant):
    d = np.load(os.path.join(G, name))
    keys = ("dim", "T_liquidus", "gas_const", "Qg", "L0", "kappa_g", "m_g", "ad_hoc")

    class P:
        mesh_h_xyz = tuple(d["h"].tolist())
        unique_grain_directions = d["grain_dirs"]
        cell_ori_inds = d["cell_ori_inds"]

    pf_args = dict(zip(keys, d["pf_keys"].tolist()), num_oris=int(d["n"]), Nx=int(d["Nx"]),
                   Ny=int(d["Ny"]), Nz=int(d["Nz"]), anisotropy=float(d["anisotropy"]))
    s = _solver(pf_args, P())
    steps = int(d["steps"])
    got = _run_gpu(s, d["eta_in"], d["T"], float(d["dt"]), steps)
    err = np.abs(got - d["eta_out"][-1]).max()
    print(f"{name}: max |d eta| vs reference = {err:.3e}")
    assert err <= ETA_TOL
    assert _argmax_mismatch(got, d["eta_out"][-1]) == 0


CASES = [
    # shape (x, y, z), n, anisotropy, bc, force
    ((1, 1, 1), 1, 0.0, None, False),
    ((1, 1, 1), 3, 0.15, None, False),
    ((7, 5, 3), 2, 0.0, None, False),
    ((7, 5, 3), 5, 0.15, None, False),
    ((13, 11, 7), 20, 0.15, None, False),
    ((13, 11, 7), 20, 0.0, "periodic", False),
    ((9, 17, 5), 10, 0.15, ("periodic", "neumann", "periodic"), False),
    ((31, 3, 4), 30, 0.15, None, True),
    ((6, 6, 19), 31, 0.15, ("neumann", "periodic", "neumann"), False),
    ((5, 4, 3), 32, 0.0, None, True),
    ((5, 4, 3), 33, 0.15, None, False),
    ((4, 3, 5), 64, 0.15, "periodic", False),
    ((53, 23, 9), 12, 0.15, None, False),
    ((60, 41, 11), 20, 0.15, None, False),
    # even nx with num_oris % 4 == 2: the TMA kernel's 8-byte-vector rows
    ((8, 5, 4), 2, 0.15, None, False),
    ((34, 9, 6), 6, 0.15, None, False),
    ((40, 7, 5), 10, 0.0, None, True),
    ((2, 3, 4), 14, 0.15, None, False),
    ((66, 13, 5), 18, 0.15, None, False),
    ((100, 11, 4), 22, 0.15, None, False),
    ((4, 17, 9), 26, 0.15, None, False),
    ((64, 9, 7), 30, 0.15, ("neumann", "periodic", "periodic"), False),
]


@pytest.mark.parametrize("shape,n,aniso,bc,force", CASES)
def test_random_vs_oracle(shape, n, aniso, bc, force, variant):
    poly, eta, T, pf_args, oargs, obc = pf_case(shape, n, aniso, seed=hash((shape, n)) & 0xffff,
                                                bc=bc, force=force)
    s = _solver(pf_args, poly)
    dt = 1e-8
    steps = 3
    got = _run_gpu(s, eta, T, dt, steps)
    ref = _run_oracle(eta, T, oargs, poly.unique_grain_directions, obc, dt, steps, force)
    err = np.abs(got - ref).max()
    mism = _argmax_mismatch(got, ref)
    print(f"[{variant}] {shape} n={n} A={aniso} bc={bc}: max |d eta| = {err:.3e}, "
          f"argmax mismatches = {mism}")
    assert err <= ETA_TOL
    assert mism == 0


def test_many_steps_directional_solidification(variant):
    """Config-1 physics on a reduced grid: Voronoi polycrystal, moving
    gradient 1e6 K/m at 0.1 m/s with the front mid-height, liquid forcing,
    200 steps at the stable dt; state compared after every 50 steps."""
    from jax_am_gb300.phase_field.allen_cahn import Quench
    from jax_am_gb300.phase_field.utils import Field
    pf_args = dict(Nx=24, Ny=20, Nz=16, h=1e-6, num_grains=12, num_oris=20, T_liquidus=1700.0,
                   gas_const=8.3, Qg=1.4e5, L0=3.5e3, kappa_g=2.77e-6, m_g=2.4e5,
                   anisotropy=0.0, ad_hoc=1.0, force_liquid_zero=True, liquid_shift=1.0)
    poly = Field(pf_args, seed=7)
    s = _solver(pf_args, poly)
    q = Quench(1700.0, 1e6, 0.1, z0=8e-6)
    dt = s.stable_dt()
    eta_gpu = s.ini_cond()
    eta_ref = eta_gpu.double().cpu().numpy()
    oargs = dict(pf_args, h=poly.mesh_h_xyz)
    # the kernel evaluates the gradient per plane at z = h/2 + iz h in float64
    h_z = poly.mesh_h_xyz[2]
    iz = np.repeat(np.arange(16), 24 * 20)
    cent = np.zeros((len(iz), 3))
    cent[:, 2] = 0.5 * h_z + iz * h_z
    state = (eta_gpu, 0.0)
    t = 0.0
    dt32 = float(np.float32(dt))
    worst = 0.0
    for k in range(200):
        Tk = np.float32(O.T_quench(cent, t, 1700.0, 1e6, 0.1, z0=8e-6))
        state, _ = s.stepper(state, t + dt32, [q])
        eta_ref = O.explicit_euler(eta_ref, t, t + dt32, Tk.astype(np.float64), oargs,
                                   poly.unique_grain_directions)
        eta_ref = O.force_liquid_zero(eta_ref, Tk, 1700.0, 1.0)
        t += dt32
        if (k + 1) % 50 == 0:
            got = state[0].double().cpu().numpy()
            err = np.abs(got - eta_ref).max()
            worst = max(worst, err)
            assert err <= ETA_TOL, f"step {k + 1}: {err}"
            assert _argmax_mismatch(got, eta_ref) == 0
    print(f"200-step directional solidification: max |d eta| = {worst:.3e}")


def test_stepper_contract():
    poly, eta, T, pf_args, oargs, obc = pf_case((6, 5, 4), 5, 0.15, seed=3)
    s = _solver(pf_args, poly)
    e = torch.tensor(eta, dtype=torch.float32, device="cuda")
    (e1, t1), y = s.stepper((e, 0.0), 1e-8, [T])  # NumPy T is accepted
    assert t1 == 1e-8 and y.data_ptr() == e1.data_ptr() and e1.data_ptr() != e.data_ptr()
    assert torch.equal(e, torch.tensor(eta, dtype=torch.float32, device="cuda"))  # input kept
    with pytest.raises(ValueError):
        s.stepper((e[:-1], 0.0), 1e-8, [T])
    with pytest.raises(ValueError):
        s.stepper((e, 0.0), 1e-8, [T[:-1]])
    with pytest.raises(ValueError):
        s.stepper((e, 0.0), 1e-8, [T], out=e)


def test_ini_cond_one_hot():
    poly, eta, T, pf_args, oargs, obc = pf_case((7, 6, 5), 9, seed=4)
    s = _solver(pf_args, poly)
    np.testing.assert_array_equal(s.ini_cond().cpu().numpy(),
                                  O.ini_cond(poly.cell_ori_inds, 9))


def test_uniform_grain_is_stationary(variant):
    """One-hot eta in a uniform solid grain: rhs = m_g (1 - 1) = 0 and a zero
    Laplacian, so the step leaves it unchanged exactly."""
    poly, eta, T, pf_args, oargs, obc = pf_case((8, 8, 8), 6, 0.15, seed=5, noise=0.0)
    poly.cell_ori_inds[:] = 2
    eta = np.zeros_like(eta)
    eta[:, 2] = 1.0
    s = _solver(pf_args, poly)
    got = _run_gpu(s, eta, np.full_like(T, 1500.0), 1e-8, 5)
    np.testing.assert_array_equal(got, eta)


def test_liquid_decay_rate():
    """Uniform eta in a liquid (zeta = 0): d eta/dt = -Lg m_g (eta^3 - eta +
    4 eta (S - eta^2) + 2 eta)."""
    poly, eta, T, pf_args, oargs, obc = pf_case((4, 4, 4), 3, 0.0, seed=6, noise=0.0)
    eta = np.tile(f32([0.3, 0.5, 0.2]), (64, 1))
    Tl = np.full((64, 1), 1900.0)
    s = _solver(pf_args, poly)
    dt = 1e-8
    got = _run_gpu(s, eta, Tl, dt, 1)
    Lg = 3.5e3 * np.exp(-1.4e5 / (1900.0 * 8.3))
    S = np.sum(eta[0] ** 2)
    e = eta[0]
    expect = e - dt * Lg * 2.4e5 * (e ** 3 - e + 4 * e * (S - e ** 2) + 2 * e)
    np.testing.assert_allclose(got[0], expect, atol=1e-6)
    np.testing.assert_allclose(got, np.tile(got[0], (64, 1)), atol=0)


@pytest.mark.parametrize("n,aniso", [(20, 0.15), (10, 0.15), (30, 0.0), (7, 0.15), (8, 0.15),
                                     (64, 0.0)])
def test_warp_and_generic_kernels_agree(n, aniso):
    """Both kernels compute the same update; they differ only in float32
    rounding (packed FMAs, approximate reciprocal in the anisotropy)."""
    from jax_am_gb300 import _lib
    lib = _lib.load()
    poly, eta, T, pf_args, oargs, obc = pf_case((41, 29, 13), n, aniso, seed=n)
    outs = []
    for v in (0, 1, 2, 3):
        lib.pfg_set_kernel_variant(v)
        s = _solver(pf_args, poly)
        outs.append(_run_gpu(s, eta, T, 1e-8, 4))
    lib.pfg_set_kernel_variant(0)
    for o in (outs[0], outs[2], outs[3]):
        assert np.abs(o - outs[1]).max() <= 1e-5
    assert _lib.device_error() == 0


def test_plans_report_the_kernel_used():
    from jax_am_gb300 import _lib
    from jax_am_gb300.phase_field.allen_cahn import make_pf_params
    lib = _lib.load()
    for shape, n, bc, kernel, vec in (((30, 20, 10), 20, None, 4, 4),
                                      ((30, 20, 10), 20, "periodic", 4, 4),
                                      ((30, 20, 10), 12, None, 3, 4),
                                      ((30, 20, 10), 10, None, 3, 2), ((30, 20, 10), 30, None, 3, 2),
                                      ((31, 20, 10), 30, None, 2, 2),
                                      ((30, 20, 10), 30, "periodic", 2, 2),
                                      ((30, 20, 10), 7, None, 2, 1), ((30, 20, 10), 33, None, 1, 1)):
        poly, eta, T, pf_args, _, _ = pf_case(shape, n, 0.15, seed=n, bc=bc)
        plan = _lib.describe_plan(make_pf_params(pf_args, poly))
        assert plan["kernel"] == kernel and plan["vec"] == vec, (shape, n, bc, plan)
        if kernel == 4:  # cell per lane: 16 x 16 tiles, a warp owns 8 x 4 cells
            assert (plan["tile_x"], plan["tile_y"], plan["warps_x"], plan["rows_per_warp"],
                    plan["lanes_per_cell"]) == (16, 16, 2, 4, 1), plan
    lib.pfg_set_kernel_variant(1)
    assert _lib.describe_plan(make_pf_params(pf_args, poly))["kernel"] == 1
    poly, eta, T, pf_args, _, _ = pf_case((30, 20, 10), 20, 0.15, seed=20)
    lib.pfg_set_kernel_variant(3)  # the TMA-fed kernel ahead of the cell-per-lane kernel
    assert _lib.describe_plan(make_pf_params(pf_args, poly))["kernel"] == 3
    lib.pfg_set_kernel_variant(0)


@pytest.mark.parametrize("aniso", [0.0, 0.15])
def test_rk4_vs_oracle(aniso):
    """The reference's rk4 (allen_cahn.py:91-104) through the GPU step, three
    steps, against the float64 oracle's RK4."""
    from jax_am_gb300.phase_field.allen_cahn import rk4
    poly, eta, T, pf_args, oargs, obc = pf_case((21, 13, 7), 10, aniso, seed=77)
    s = _solver(pf_args, poly)
    Td = torch.tensor(T, dtype=torch.float32, device="cuda")
    state = (torch.tensor(eta, dtype=torch.float32, device="cuda"), 0.0)
    ref = eta.copy()
    dt = 1e-8
    for k in range(3):
        state, _ = rk4(state, (k + 1) * dt, s, [Td])
        ref = O.rk4(ref, k * dt, (k + 1) * dt, T, oargs, poly.unique_grain_directions, obc)
    got = state[0].double().cpu().numpy()
    err = np.abs(got - ref).max()
    print(f"rk4 A={aniso}: max |d eta| = {err:.3e}")
    assert err <= ETA_TOL
    assert _argmax_mismatch(got, ref) == 0


def test_liquidus_not_a_float32_value():
    """T_liquidus = 1623.1 K has no float32 value.  The C ABI holds it as a
    float32 (``pfg_pf_params.T_liquidus``), so the step compares T with
    float32(1623.1) exactly as the reference does on float32 arrays (NumPy
    and jax.numpy round the Python float to the array's float32): a cell at
    T = float32(1623.1) has T / T_liquidus = 1 and zeta = 1/2.  Checked
    against the oracle given the float32-rounded T_liquidus, on cells placed
    exactly there and one float32 step either side, and the inspect metrics
    count T >= float32(1623.1) as liquid."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    poly, eta, T, pf_args, oargs, obc = pf_case((12, 9, 7), 20, 0.15, seed=31)
    tl32 = np.float32(1623.1)
    T = T.copy()
    T[0::5] = float(tl32)
    T[1::5] = float(np.nextafter(tl32, np.float32(np.inf)))
    T[2::5] = float(np.nextafter(tl32, np.float32(-np.inf)))
    pf_args = dict(pf_args, T_liquidus=1623.1)
    oargs = dict(oargs, T_liquidus=float(tl32))
    s = PFSolver(pf_args, poly)
    got = _run_gpu(s, eta, T, 1e-8, 3)
    ref = _run_oracle(eta, T, oargs, poly.unique_grain_directions, obc, 1e-8, 3)
    err = np.abs(got - ref).max()
    print(f"T_liquidus 1623.1 (float32 {float(tl32)!r}): max |d eta| = {err:.3e}")
    assert err <= ETA_TOL
    assert _argmax_mismatch(got, ref) == 0
    d = s.inspect_sol(torch.tensor(eta, dtype=torch.float32, device="cuda"),
                      torch.tensor(eta, dtype=torch.float32, device="cuda"),
                      torch.tensor(T, dtype=torch.float32, device="cuda"), [0.0, 1e-8], 1)
    want = 100.0 * np.mean(T.astype(np.float32).reshape(-1) >= tl32)
    assert abs(d["pct_liquid"] - want) <= 1e-9
