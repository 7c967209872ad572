"""The moving point-source step (pfg_pf_step_point_source) and its T
(pfg_point_source_T) against the reference drivers' own temperatures
(golden vectors from tests/golden/make_golden_point_sources.py), against the
T-array step given the same T, and against the float64 oracle over many
steps.  Tolerances: T 3e-6 relative (float32 evaluation of the float64
formula); eta 1e-6 against the T-array step, 1e-4 against the oracle;
argmax maps exact."""
import os

import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.cases import PF_DEFAULTS, Poly, f32

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def _golden():
    d = np.load(os.path.join(G, "point_sources.npz"))
    Nx, Ny, Nz = (int(v) for v in d["shape"])
    dom = [float(v) for v in d["domain"]]
    args = dict(domain_x=dom[0], domain_y=dom[1], domain_z=dom[2], t_OFF=float(d["t_OFF"]),
                T_ambient=float(d["T_ambient"]), vel=float(d["vel"]), dt=float(d["dt"]),
                laser_path=dict(x_pos=list(d["x_pos"]), y_pos=list(d["y_pos"]),
                                z_pos=list(d["z_pos"]), switch=list(d["switch"])))
    return d, (Nx, Ny, Nz), dom, args


def _solver(shape, dom, n=8, aniso=0.15, seed=0):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    Nx, Ny, Nz = shape
    h = (dom[0] / Nx, dom[1] / Ny, dom[2] / Nz)
    poly = Poly(shape, h, n, np.random.default_rng(seed))
    pf_args = dict(PF_DEFAULTS, num_oris=n, Nx=Nx, Ny=Ny, Nz=Nz, anisotropy=aniso)
    return PFSolver(pf_args, poly), poly, pf_args


@pytest.mark.parametrize("kind", ["simple", "ramped", "raster"])
def test_T_matches_reference_drivers(kind):
    from jax_am_gb300.phase_field.point_source import PointSource
    d, shape, dom, args = _golden()
    s, _, _ = _solver(shape, dom)
    if kind == "raster":
        src = PointSource.raster(args)
        steps, ref = d["path_steps"], d["T_path"]
    else:
        src = (PointSource.simple if kind == "simple" else PointSource.ramped)(args, d["times"])
        steps, ref = range(len(d["times"])), d["T_" + ("simple" if kind == "simple" else "grf")]
    worst = 0.0
    for j, k in enumerate(steps):
        got = src.T(s, step=int(k)).double().cpu().numpy()
        worst = max(worst, float(np.max(np.abs(got - ref[j]) / ref[j])))
        np.testing.assert_allclose(got, ref[j], rtol=3e-6)
    print(f"{kind}: max relative |dT| vs reference = {worst:.2e}")


@pytest.fixture(params=[0, 1, 2, 3], ids=["auto", "generic", "warp_cpasync", "tma256"])
def variant(request):
    from jax_am_gb300 import _lib
    lib = _lib.load()
    lib.pfg_set_kernel_variant(request.param)
    yield request.param
    lib.pfg_set_kernel_variant(0)
    assert _lib.device_error() == 0


@pytest.mark.parametrize("n", [8, 6])
def test_step_equals_T_array_step(variant, n):
    """One step with the source evaluated in the kernel equals the step fed
    with the source's T array (same float32 T)."""
    from jax_am_gb300.phase_field.point_source import PointSource
    d, shape, dom, args = _golden()
    s, _, _ = _solver(shape, dom, n=n)
    src = PointSource.raster(args)
    rng = np.random.default_rng(n)
    eta = torch.tensor(rng.random((s.N, n)), dtype=torch.float32, device="cuda")
    for k in (0, 71, 300):
        t = float(src.ts[k])
        (a, _), _ = s.stepper((eta, t), t + 1e-8, [src])
        (b, _), _ = s.stepper((eta, t), t + 1e-8, [src.T(s, step=k)])
        err = float((a - b).abs().max())
        assert err <= 1e-6, (k, err)


def test_many_steps_vs_float64_oracle():
    """60 raster steps at 5e-9 s, n = 8, A = 0.15, the hot source near cells
    above the liquidus: eta against the float64 oracle fed the kernel's T."""
    from jax_am_gb300.phase_field.point_source import PointSource
    from jax_am_gb300.runner import PointSourceRun
    d, shape, dom, args = _golden()
    s, poly, pf_args = _solver(shape, dom, n=8, aniso=0.15, seed=3)
    src = PointSource.raster(args)
    dt = float(np.float32(5e-9))
    rng = np.random.default_rng(4)
    eta0 = f32(np.clip(s.ini_cond().cpu().numpy() + 0.3 * rng.random((s.N, 8)), 0, 1))
    run = PointSourceRun(s, src, dt, eta0=torch.tensor(eta0, dtype=torch.float32, device="cuda"),
                         step0=100)
    oargs = dict(pf_args, h=poly.mesh_h_xyz)
    e = eta0.copy()
    hot = 0
    for k in range(60):
        T = src.T(s, step=100 + k).double().cpu().numpy()
        hot = max(hot, int((T > 1623.0).sum()))
        e = O.explicit_euler(e, k * dt, (k + 1) * dt, T, oargs, poly.unique_grain_directions)
    run.run(60)
    got = run.state.double().cpu().numpy()
    err = float(np.abs(got - e).max())
    mism = int(np.sum(np.argmax(got, axis=1) != np.argmax(e, axis=1)))
    print(f"raster 60 steps: max |d eta| = {err:.3e}, argmax mismatches = {mism}, "
          f"cells above the liquidus = {hot}")
    assert hot > 0
    assert err <= 1e-4 and mism == 0
    assert run.steps_taken == 160


def test_graph_run_equals_stepper_loop():
    """PointSourceRun (graph replay, record from the device step count) equals
    PFSolver.stepper called per step with the source (record from t_prev)."""
    from jax_am_gb300.phase_field.point_source import PointSource
    from jax_am_gb300.runner import PointSourceRun
    d, shape, dom, args = _golden()
    s, _, _ = _solver(shape, dom, n=8, seed=5)
    src = PointSource.raster(args)
    dt = float(src.ts[1] - src.ts[0])
    run = PointSourceRun(s, src, dt)
    run.run(45)
    state = (s.ini_cond(), float(src.ts[0]))
    for k in range(45):
        state, _ = s.stepper(state, float(src.ts[k + 1]), [src])
    assert torch.equal(run.state, state[0])
