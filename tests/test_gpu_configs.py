"""The float32 GPU path against a float64 run of the oracle's PyTorch
restatement (on the GPU, in float64) for the benchmark configurations:
directional solidification at full size (64 x 64 x 32, n = 20, 200 steps),
the single-track laser scan and the multi-track scan on reduced grids with
the configurations' physics.  The error after the run is printed per
configuration; tolerances: max |d eta| <= 1e-4, max |dT| <= 1e-3 K; argmax
orientation maps compared exactly, and every mismatched cell must be a near
tie in the float64 run (top-two gap within twice the eta error)."""
import numpy as np
import pytest
import torch

from oracle import pf_torch as PT
from tests.laser_parity import PF_KEYS, T_LIQ, _compare, _dirs, _laser_case, _oracle_args

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def test_directional_solidification_full_size():
    """64 x 64 x 32 cells, 40 grains, n = 20, isotropic, periodic x/y and
    Neumann z, T = 1700 K + 1e6 K/m (z - 16 um) - 1e6 * 0.1 t, liquid above
    T_melt + 1 K set to eta = 0, 200 steps at the stable dt."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, Quench
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import QuenchRun
    nx, ny, nz = 64, 64, 32
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_grains=40, num_oris=20,
                   T_liquidus=1700.0, anisotropy=0.0, force_liquid_zero=True, liquid_shift=1.0,
                   bc=("periodic", "periodic", "neumann"))
    poly = Field(pf_args, seed=1)
    s = PFSolver(pf_args, poly)
    q = Quench(1700.0, 1e6, 0.1, z0=16e-6)
    dt = float(np.float32(s.stable_dt()))
    run = QuenchRun(s, q, dt)
    run.run(200)
    a = _oracle_args(pf_args, poly)
    dirs = _dirs(poly)
    e = s.ini_cond().double().reshape(nz, ny, nx, -1)
    zc = 0.5e-6 + 1e-6 * np.arange(nz)
    t = 0.0
    for _ in range(200):
        Tz = np.float32(1700.0 + 1e6 * (zc - 16e-6) - 1e6 * 0.1 * t).astype(np.float64)
        T3 = torch.tensor(Tz, device="cuda")[:, None, None].expand(nz, ny, nx)
        e = e + dt * PT.pf_increment(e, T3, a, dirs, bc=(True, True, False))
        e = torch.where((T3 > 1701.0)[..., None], torch.zeros_like(e), e)
        t += dt
    _compare("directional solidification 64x64x32 n=20, 200 steps", run.state, e)


def test_single_track_laser_reduced():
    """Single-track physics (n = 20, A = 0.15, 200 W, r = 50 um, absorptivity
    0.4, 0.8 m/s, T0 = 300 K) on 100 x 50 x 25 cells, 200 fused steps."""
    from jax_am_gb300.runner import single_track
    path = single_track(20e-6, 25e-6, 0.8, 200.0, 1.0)
    Tmax = _laser_case((100, 50, 25), 20, 60, 0.15, path, 200, 2,
                       "single track 100x50x25 n=20 A=0.15, 200 steps")
    assert Tmax >= T_LIQ, f"the laser never melted the surface (T max {Tmax:.1f} K)"


def test_multi_track_laser_reduced():
    """Multi-track physics (n = 30, A = 0.15, three tracks 100 um apart at
    250 W and 1.0 m/s, scanned one after the other) on 80 x 40 x 20 cells
    with 1 um long tracks 10 um apart, so that all three are scanned in the
    150 fused steps."""
    from jax_am_gb300.runner import raster
    path = raster([10e-6, 20e-6, 30e-6], 1.0, 250.0, 20e-6, 21e-6)
    Tmax = _laser_case((80, 40, 20), 30, 40, 0.15, path, 150, 5,
                       "multi track 80x40x20 n=30 A=0.15, 150 steps")
    assert Tmax >= T_LIQ, f"the laser never melted the surface (T max {Tmax:.1f} K)"


@pytest.fixture(params=[0, 3], ids=["lane", "tma_fixed"])
def n20_kernel(request):
    """The two step kernels of the n = 20 workloads: the cell-per-lane kernel
    (variant 0, the default) and the TMA-fed kernel's compile-time 24 x 10
    plan (variant 3)."""
    from jax_am_gb300 import _lib
    lib = _lib.load()
    assert lib.pfg_set_kernel_variant(request.param) == 0
    yield request.param
    lib.pfg_set_kernel_variant(0)
    assert _lib.device_error() == 0, "a bounded device-side wait ran out"


def _assert_n20_plan(pf_args, poly, variant):
    """Variant 0 runs the cell-per-lane kernel (16 x 16 tiles, 4 slots);
    variant 3 the TMA-fed kernel's compile-time 24 x 10 plan (FixedPlan<1> in
    pf_tma.cu), taken exactly when the planner picks this plan."""
    from jax_am_gb300 import _lib
    from jax_am_gb300.phase_field.allen_cahn import make_pf_params
    p = _lib.describe_plan(make_pf_params(pf_args, poly))
    if variant == 0:
        assert (p["kernel"], p["vec"], p["tile_x"], p["tile_y"], p["slots"], p["fixed"]) == \
            (4, 4, 16, 16, 4, 0), p
        return
    got = (p["kernel"], p["vec"], p["tile_x"], p["tile_y"], p["rows_per_warp"], p["warps_x"],
           p["slots"], p["fixed"])
    assert got == (3, 4, 24, 10, 5, 4, 4, 1), p


def test_fixed_plan_fused_laser_vs_oracle(n20_kernel):
    """200 x 100 x 50 cells with n = 20 (partial tiles along x and y for the
    24 x 10 plan, as on the bench grid): 40 fused heat + anisotropic steps
    against the float64 oracle."""
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import single_track
    pf_args = dict(PF_KEYS, Nx=200, Ny=100, Nz=50, h=1e-6, num_grains=300, num_oris=20,
                   T_liquidus=1623.0, anisotropy=0.15)
    _assert_n20_plan(pf_args, Field(pf_args, seed=5), n20_kernel)
    path = single_track(20e-6, 50e-6, 0.8, 200.0, 1.0)
    Tmax = _laser_case((200, 100, 50), 20, 300, 0.15, path, 40, 5,
                       f"n=20 kernel {n20_kernel}, 200x100x50 A=0.15, 40 fused steps")
    assert Tmax >= T_LIQ, f"the laser never melted the surface (T max {Tmax:.1f} K)"


@pytest.mark.parametrize("aniso", [0.0, 0.15])
def test_fixed_plan_T_array_vs_oracle(aniso, n20_kernel):
    """120 x 100 x 40 cells, n = 20, a temperature array (the drivers'
    stepper form): the n = 20 kernels against float64, three steps."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.utils import Field
    nx, ny, nz = 120, 100, 40
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_grains=200, num_oris=20,
                   T_liquidus=1623.0, anisotropy=aniso)
    poly = Field(pf_args, seed=6)
    _assert_n20_plan(pf_args, poly, n20_kernel)
    s = PFSolver(pf_args, poly)
    g = torch.Generator(device="cuda").manual_seed(7)
    e0 = s.ini_cond()
    e0 = torch.clamp(e0 + 0.3 * torch.rand(e0.shape, generator=g, device="cuda"), 0.0, 1.0)
    T = 1450.0 + 300.0 * torch.rand((s.N, 1), generator=g, device="cuda")
    dt = float(np.float32(1e-8))
    state = (e0.clone(), 0.0)
    for k in range(3):
        state, _ = s.stepper(state, (k + 1) * dt, [T])
    a = _oracle_args(pf_args, poly)
    e = e0.double().reshape(nz, ny, nx, -1)
    T3 = T.double().reshape(nz, ny, nx)
    for _ in range(3):
        e = e + dt * PT.pf_increment(e, T3, a, _dirs(poly))
    _compare(f"n=20 kernel {n20_kernel}, T array, A={aniso}", state[0], e)


def test_fixed_plan30_vs_oracle():
    """320 x 160 x 80 cells with n = 30 (8-byte vectors): the compile-time
    16 x 9 plan (FixedPlan<2>) of the multi-track configuration; three
    temperature-array steps and 40 fused heat + anisotropic steps against the
    float64 oracle."""
    from jax_am_gb300 import _lib
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, make_pf_params
    from jax_am_gb300.phase_field.utils import Field
    from jax_am_gb300.runner import single_track
    nx, ny, nz = 320, 160, 80
    pf_args = dict(PF_KEYS, Nx=nx, Ny=ny, Nz=nz, h=1e-6, num_grains=400, num_oris=30,
                   T_liquidus=1623.0, anisotropy=0.15)
    poly = Field(pf_args, seed=8)
    p = _lib.describe_plan(make_pf_params(pf_args, poly))
    assert (p["kernel"], p["vec"], p["tile_x"], p["tile_y"], p["rows_per_warp"], p["warps_x"],
            p["fixed"]) == (3, 2, 16, 9, 9, 8, 2), p
    s = PFSolver(pf_args, poly)
    g = torch.Generator(device="cuda").manual_seed(9)
    e0 = s.ini_cond()
    e0 = torch.clamp(e0 + 0.3 * torch.rand(e0.shape, generator=g, device="cuda"), 0.0, 1.0)
    T = 1450.0 + 300.0 * torch.rand((s.N, 1), generator=g, device="cuda")
    dt = float(np.float32(1e-8))
    state = (e0.clone(), 0.0)
    for k in range(3):
        state, _ = s.stepper(state, (k + 1) * dt, [T])
    a = _oracle_args(pf_args, poly)
    e = e0.double().reshape(nz, ny, nx, -1)
    T3 = T.double().reshape(nz, ny, nx)
    for _ in range(3):
        e = e + dt * PT.pf_increment(e, T3, a, _dirs(poly))
    _compare("fixed 16x9 plan, T array, n=30", state[0], e)
    del state, e, e0, T, T3, s
    torch.cuda.empty_cache()
    path = single_track(20e-6, 80e-6, 0.8, 200.0, 1.0)
    Tmax = _laser_case((nx, ny, nz), 30, 400, 0.15, path, 40, 8,
                       "fixed 16x9 plan, 320x160x80 n=30 A=0.15, 40 fused steps")
    assert Tmax >= T_LIQ, f"the laser never melted the surface (T max {Tmax:.1f} K)"
