"""The coupled driver's glue on the GPU: convert_temperature (pfg_transpose_xyz)
exactly, the in-kernel time interpolation (pfg_pf_step_interp) against the
T-array step fed the interpolated field, and a multi-rate run (coarse fields
every 4 phase-field steps, as coupled/example.py:92-111 steps) against the
float64 oracle.  Tolerances: transpose exact; eta 1e-6 against the T-array
step and 1e-4 against the oracle; argmax maps exact."""
import numpy as np
import pytest
import torch

from oracle import pf_oracle as O
from tests.cases import f32, pf_case

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


@pytest.mark.parametrize("shape", [(37, 5, 66), (1, 1, 1), (64, 3, 32), (33, 65, 2)])
def test_convert_temperature_is_the_transpose(shape):
    from jax_am_gb300.phase_field.coupling import convert_temperature
    T = np.random.default_rng(sum(shape)).random(shape).astype(np.float32)
    got = convert_temperature(T).cpu().numpy()
    np.testing.assert_array_equal(got, np.transpose(T, (2, 1, 0)).reshape(-1, 1))


@pytest.fixture(params=[0, 1, 2, 3], ids=["auto", "generic", "warp_cpasync", "tma256"])
def variant(request):
    from jax_am_gb300 import _lib
    lib = _lib.load()
    lib.pfg_set_kernel_variant(request.param)
    yield request.param
    lib.pfg_set_kernel_variant(0)
    assert _lib.device_error() == 0


@pytest.mark.parametrize("n", [8, 6])
def test_interpolated_step_equals_T_array_step(variant, n):
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.coupling import InterpolatedT
    poly, eta, T, pf_args, oargs, _ = pf_case((23, 17, 9), n, 0.15, seed=n)
    s = PFSolver(pf_args, poly)
    rng = np.random.default_rng(1)
    Tp = torch.tensor(rng.uniform(1400, 2000, s.N), dtype=torch.float32, device="cuda")
    Tf = torch.tensor(rng.uniform(1400, 2000, s.N), dtype=torch.float32, device="cuda")
    e = torch.tensor(eta, dtype=torch.float32, device="cuda")
    # steps of 2e-8 s (inside the explicit stability limit of this grid)
    src = InterpolatedT(Tp, Tf, t_future=8e-8, dt_coarse=8e-8)
    for t_prev in (0.0, 2e-8, 6e-8):
        t_crt = t_prev + 2e-8
        (a, _), _ = s.stepper((e, t_prev), t_crt, [src])
        r = np.float32((8e-8 - t_crt) / 8e-8)
        Tmix = r * Tp + (np.float32(1.0) - r) * Tf
        (b, _), _ = s.stepper((e, t_prev), t_crt, [Tmix])
        err = float((a - b).abs().max())
        assert err <= 1e-6, (t_prev, err)


def test_multi_rate_run_vs_float64_oracle():
    """A coarse field every 4e-8 s (a moving hot spot, given in the coarse
    solver's (Nx, Ny, Nz) order), 24 phase-field steps of 1e-8 s, T at each
    step's end time interpolated between the two coarse fields around it."""
    from jax_am_gb300.phase_field.allen_cahn import PFSolver
    from jax_am_gb300.phase_field.coupling import InterpolatedT, convert_temperature
    shape = (20, 14, 10)
    Nx, Ny, Nz = shape
    poly, eta, _, pf_args, oargs, _ = pf_case(shape, 8, 0.15, seed=7, noise=0.4)
    s = PFSolver(pf_args, poly)
    xs, ys, zs = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")

    def coarse(t):  # (Nx, Ny, Nz) float32 field of the coarse solver at time t
        xc = 4 + t / 4e-8 * 2.0
        d2 = (xs - xc) ** 2 + (ys - 7) ** 2 + (zs - 9) ** 2
        return np.float32(1400.0 + 500.0 * np.exp(-d2 / 20.0))

    dt_pf, dt_cfd = 1e-8, 4e-8
    state = (torch.tensor(eta, dtype=torch.float32, device="cuda"), 0.0)
    e_ref = eta.copy()
    t_cfd = dt_cfd
    T_past, T_future = coarse(0.0), coarse(dt_cfd)
    hot = 0
    for i in range(1, 25):
        t_pf = i * dt_pf
        if t_pf > t_cfd + dt_cfd * (1 - 1e-9):  # the driver's advance, on exact step multiples
            T_past, T_future = T_future, coarse(t_cfd + dt_cfd)
            t_cfd += dt_cfd
        src = InterpolatedT(convert_temperature(T_past), convert_temperature(T_future), t_cfd,
                            dt_cfd)
        state, _ = s.stepper(state, t_pf, [src])
        r = (t_cfd - t_pf) / dt_cfd
        Tmix = (np.float32(r) * T_past + (np.float32(1.0) - np.float32(r)) * T_future)
        T_cells = f32(np.transpose(Tmix, (2, 1, 0)).reshape(-1, 1))
        hot = max(hot, int((T_cells > 1623.0).sum()))
        e_ref = O.explicit_euler(e_ref, t_pf - dt_pf, t_pf, T_cells, oargs,
                                 poly.unique_grain_directions)
    got = state[0].double().cpu().numpy()
    err = float(np.abs(got - e_ref).max())
    mism = int(np.sum(np.argmax(got, axis=1) != np.argmax(e_ref, axis=1)))
    print(f"multi-rate coupling, 24 steps: max |d eta| = {err:.3e}, argmax mismatches = {mism}, "
          f"cells above the liquidus = {hot}")
    assert hot > 0 and err <= 1e-4 and mism == 0
