"""Parity of the CUDA heat step and the fused heat + phase-field step with the
FP64 oracle and the reference's golden vectors.  Tolerances: |d T| <= 1e-3 K,
max |d eta| <= 1e-4."""
import os

import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.cases import GAMMA_DEFAULTS, f32, pf_case

pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(__file__), "golden")
T_TOL = 1e-3
ETA_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def _gamma_from(d):
    keys = ("eta", "r", "rho", "h", "eps", "SB", "T0", "Ts", "Tl", "L")
    return dict(zip(keys, d["gamma"].tolist()))


@pytest.mark.parametrize("name", ["heat_f32.npz", "heat_f64.npz"])
def test_update_T_matches_reference_golden(name):
    from jax_am_gb300.cfd.gamma import update_T
    d = np.load(os.path.join(G, name))
    g = _gamma_from(d)
    dx, dy, dz, dt = d["dxyzt"].tolist()
    T = torch.tensor(d["T_in"], dtype=torch.float32, device="cuda")
    nx, ny, nz = (s - 2 for s in T.shape)
    x_ = dx / 2 + dx * np.arange(nx)
    y_ = dy / 2 + dy * np.arange(ny)
    z_ = dz / 2 + dz * np.arange(nz)
    x, y, _ = np.meshgrid(x_, y_, z_, indexing="ij")
    worst = 0.0
    for k, (xl, yl, P) in enumerate(d["lasers"]):
        T = update_T(T, xl, yl, x, y, P, dx, dy, dz, dt, g)
        err = np.abs(T.double().cpu().numpy() - d["T_out"][k]).max()
        worst = max(worst, err)
    print(f"{name}: max |d T| vs reference = {worst:.3e} K")
    assert worst <= T_TOL


@pytest.mark.parametrize("shape", [(19, 13, 7), (50, 20, 50), (400, 200, 100)])
def test_heat_layouts_agree_and_match_oracle(shape):
    """The kernel on the reference (x-major) layout and on the z-major layout
    gives identical results, equal to the oracle within tolerance; edge and
    corner ghosts are left untouched.  At 50 x 20 x 50 whole warps of a
    chunk touch no domain face (50 cells per row, chunks 8..40 of 50 along the
    slowest axis), so the face-free path runs beside the face path; 400 x 200
    x 100 is the laser-track grid (8M cells, 61-74 % face-free warps)."""
    from jax_am_gb300 import _lib
    from jax_am_gb300.cfd.gamma import make_heat_params
    import ctypes
    rng = np.random.default_rng(11)
    nx, ny, nz = shape
    dx, dy, dz, dt = 2e-6, 2.5e-6, 1.5e-6, 5e-9
    g = dict(GAMMA_DEFAULTS)
    Tx = f32(rng.uniform(300, 2500, (nx + 2, ny + 2, nz + 2)))
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = []
    for layout, arr in ((_lib.LAYOUT_XYZ, Tx), (_lib.LAYOUT_ZYX, Tx.transpose(2, 1, 0))):
        h = make_heat_params(g, nx, ny, nz, dx, dy, dz, layout=layout)
        tin = torch.tensor(np.ascontiguousarray(arr), dtype=torch.float32, device="cuda")
        tout = tin.clone()
        st = lib.pfg_heat_step(ctypes.byref(h), _lib.ptr(tin), _lib.ptr(tout), 1.3e-5, 1.1e-5,
                               180.0, dt, stream)
        _lib.check(st, "pfg_heat_step")
        o = tout.double().cpu().numpy()
        outs.append(o if layout == _lib.LAYOUT_XYZ else o.transpose(2, 1, 0))
    np.testing.assert_array_equal(outs[0], outs[1])
    xt, yt = O.cell_centres_top(nx, ny, dx, dy)
    ref = O.heat_update_T(Tx, 1.3e-5, 1.1e-5, xt, yt, 180.0, dx, dy, dz, dt, g)
    assert np.abs(outs[0] - ref).max() <= T_TOL
    # edges and corners of the ghost layer are never written
    for sl in ((0, 0), (0, -1), (-1, 0), (-1, -1)):
        np.testing.assert_array_equal(outs[0][sl[0], sl[1], :], Tx[sl[0], sl[1], :])


def test_mushy_zone_edges_match_reference_division():
    """Latent heat enters cp exactly where the reference's float32 liquid
    fraction (clip(T, Ts, Tl) - Ts) / (Tl - Ts) lies strictly inside (0, 1):
    cells at Ts, one ulp above Ts, one ulp below Tl and at Tl, each with six
    neighbours 60 K hotter (a Laplacian large enough that a wrong cp moves
    the cell by far more than the tolerance), in the face-free interior and
    next to faces, both axis orders."""
    from jax_am_gb300 import _lib
    from jax_am_gb300.cfd.gamma import make_heat_params
    import ctypes
    g = dict(GAMMA_DEFAULTS)
    Ts, Tl = np.float32(g["Ts"]), np.float32(g["Tl"])
    edges = [Ts, np.nextafter(Ts, np.float32(np.inf)), np.nextafter(Tl, np.float32(0)), Tl]
    fl = [(np.clip(e, Ts, Tl) - Ts) / (Tl - Ts) for e in edges]  # float32, as the reference
    assert fl[0] == 0 and 0 < fl[1] and fl[2] < 1 and fl[3] == 1
    nx, ny, nz = 50, 20, 50
    dx = dy = dz = 1e-6
    dt = 2e-9
    rng = np.random.default_rng(3)
    Tx = f32(rng.uniform(1540.0, 1650.0, (nx + 2, ny + 2, nz + 2)))
    cells = [(i, j, k) for i in (1, 25, 50) for j in (1, 10, 20) for k in (1, 25, 50)]
    for c, (i, j, k) in enumerate(cells):
        v = edges[c % 4]
        Tx[i, j, k] = v
        Tx[i - 1, j, k] = Tx[i, j - 1, k] = Tx[i, j, k - 1] = v + 60.0
        Tx[i + 1, j, k] = Tx[i, j + 1, k] = Tx[i, j, k + 1] = v + 60.0
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    xt, yt = O.cell_centres_top(nx, ny, dx, dy)
    ref = O.heat_update_T(Tx.astype(np.float64), 1.3e-5, 1.1e-5, xt, yt, 180.0, dx, dy, dz, dt, g)
    for layout, arr in ((_lib.LAYOUT_XYZ, Tx), (_lib.LAYOUT_ZYX, Tx.transpose(2, 1, 0))):
        h = make_heat_params(g, nx, ny, nz, dx, dy, dz, layout=layout)
        tin = torch.tensor(np.ascontiguousarray(arr), dtype=torch.float32, device="cuda")
        tout = tin.clone()
        _lib.check(lib.pfg_heat_step(ctypes.byref(h), _lib.ptr(tin), _lib.ptr(tout), 1.3e-5,
                                     1.1e-5, 180.0, dt, stream), "pfg_heat_step")
        o = tout.double().cpu().numpy()
        o = o if layout == _lib.LAYOUT_XYZ else o.transpose(2, 1, 0)
        for (i, j, k) in cells:
            assert abs(o[i, j, k] - ref[i, j, k]) <= T_TOL, ((i, j, k), o[i, j, k], ref[i, j, k])
        assert np.abs(o - ref)[1:-1, 1:-1, 1:-1].max() <= T_TOL


def test_uniform_ambient_stays_uniform():
    """With T = T0 everywhere and no beam, the Robin faces give zero flux and
    the field stays exactly at T0."""
    from jax_am_gb300.cfd.gamma import update_T
    g = dict(GAMMA_DEFAULTS)
    T = torch.full((8, 7, 6), 300.0, device="cuda")
    x = np.zeros((6, 5, 4)) + 0.5e-6 + 1e-6 * np.arange(6)[:, None, None]
    y = np.zeros((6, 5, 4)) + 0.5e-6 + 1e-6 * np.arange(5)[None, :, None]
    for _ in range(10):
        T = update_T(T, 0.0, 0.0, x, y, 0.0, 1e-6, 1e-6, 1e-6, 1e-8, g)
    assert torch.all(T == 300.0)


def _laser_fn(path):
    def laser(t):
        for (t0, t1, x0, y0, x1, y1, P) in path:
            t0, t1, x0, y0, x1, y1, P = (float(np.float32(v)) for v in (t0, t1, x0, y0, x1, y1, P))
            if t0 <= t < t1:
                f = (t - t0) / (t1 - t0)
                return x0 + f * (x1 - x0), y0 + f * (y1 - y0), P
        return 0.0, 0.0, 0.0
    return laser


@pytest.fixture(params=[0, 1, 2, 3, 512],
                ids=["auto", "generic", "warp_cpasync", "tma256", "tma512"])
def variant(request):
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


@pytest.mark.parametrize("shape,n,aniso,steps", [((12, 10, 8), 5, 0.15, 6),
                                                 ((33, 17, 9), 20, 0.15, 4),
                                                 ((7, 9, 5), 10, 0.0, 5),
                                                 ((50, 26, 12), 30, 0.15, 3)])
def test_fused_heat_pf_vs_oracle(shape, n, aniso, steps, variant):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.runner import HeatPFRun, single_track
    poly, eta, _, pf_args, oargs, obc = pf_case(shape, n, aniso, seed=21, h=(1e-6, 1e-6, 1e-6))
    nx, ny, nz = shape
    g = dict(GAMMA_DEFAULTS)
    rng = np.random.default_rng(5)
    Tx = f32(rng.uniform(1400.0, 2100.0, (nx + 2, ny + 2, nz + 2)))  # reference layout
    path = single_track(2e-6, 0.5 * ny * 1e-6, 0.8, 200.0, 1e-3)
    s = PFSolver(pf_args, poly)
    run = HeatPFRun(s, g, path, dt=2e-9, eta0=torch.tensor(eta, dtype=torch.float32,
                                                            device="cuda"),
                    T_init=torch.tensor(Tx.transpose(2, 1, 0).copy()))
    run.run(steps, graph=False)
    laser = _laser_fn(path)
    e_ref, T_ref = eta, Tx
    t = 0.0
    dt = float(np.float32(2e-9))
    for _ in range(steps):
        e_ref, T_ref = O.coupled_step(e_ref, T_ref, t, dt, oargs, g, laser,
                                      poly.unique_grain_directions)
        t += dt
    T_gpu = run.T_ghosted_f64.cpu().numpy().transpose(2, 1, 0)
    e_gpu = run.state.double().cpu().numpy()
    I = (slice(1, -1),) * 3
    t_err = np.abs(T_gpu[I] - T_ref[I]).max()
    # ghost faces too (edges/corners excluded)
    faces = [np.abs(T_gpu[0, 1:-1, 1:-1] - T_ref[0, 1:-1, 1:-1]).max(),
             np.abs(T_gpu[:, 1:-1, -1][1:-1] - T_ref[:, 1:-1, -1][1:-1]).max()]
    e_err = np.abs(e_gpu - e_ref).max()
    print(f"fused {shape} n={n}: |dT| = {t_err:.3e} K, faces {max(faces):.3e}, |d eta| = {e_err:.3e}")
    assert t_err <= T_TOL and max(faces) <= T_TOL
    assert e_err <= ETA_TOL
    assert abs(run.t - steps * dt) < 1e-15 and run.steps_taken == steps


def test_graph_replay_equals_eager():
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.runner import HeatPFRun, single_track
    poly, eta, _, pf_args, oargs, obc = pf_case((20, 12, 10), 8, 0.15, seed=9,
                                                h=(1e-6, 1e-6, 1e-6))
    g = dict(GAMMA_DEFAULTS)
    path = single_track(3e-6, 6e-6, 0.8, 200.0, 1e-3)
    e0 = torch.tensor(eta, dtype=torch.float32, device="cuda")
    runs = []
    for graph in (False, True):
        s = PFSolver(pf_args, poly)
        r = HeatPFRun(s, g, path, dt=3e-9, eta0=e0)
        r.run(47, graph=graph)
        torch.cuda.synchronize()
        runs.append(r)
    assert torch.equal(runs[0].state, runs[1].state)
    assert torch.equal(runs[0].T_ghosted, runs[1].T_ghosted)
    assert runs[0].steps_taken == runs[1].steps_taken == 47
