"""The PyTorch restatement (CPU baseline and float64 autograd stand-in) agrees
with the NumPy oracle, which is pinned to the reference's golden vectors."""
import numpy as np
import torch

from oracle import pf_oracle as O
from oracle import pf_torch as PT
from tests.cases import GAMMA_DEFAULTS, f32, pf_case


def test_torch_coupled_step_matches_numpy_oracle():
    shape = (11, 7, 5)
    nx, ny, nz = shape
    poly, eta, _, pf_args, oargs, _ = pf_case(shape, 6, 0.15, seed=31, h=(1e-6, 1.2e-6, 0.8e-6))
    rng = np.random.default_rng(3)
    Tx = f32(rng.uniform(1400.0, 2300.0, (nx + 2, ny + 2, nz + 2)))
    g = dict(GAMMA_DEFAULTS)

    def laser(t):
        return 3e-6 + 0.8 * t, 4e-6, 200.0

    dt = 2e-9
    e_np, T_np = eta, Tx
    e_t = torch.tensor(eta.reshape(nz, ny, nx, 6))
    T_t = torch.tensor(Tx.transpose(2, 1, 0).copy())
    dirs = torch.tensor(poly.unique_grain_directions)
    for k in range(3):
        e_np, T_np = O.coupled_step(e_np, T_np, k * dt, dt, oargs, g, laser,
                                    poly.unique_grain_directions, force_liquid=True)
        e_t, T_t = PT.coupled_step(e_t, T_t, k * dt, dt, oargs, g, laser, dirs, force_liquid=True)
    np.testing.assert_allclose(e_t.numpy().reshape(-1, 6), e_np, rtol=1e-11, atol=1e-13)
    Tt = T_t.numpy().transpose(2, 1, 0)
    I = (slice(1, -1),) * 3
    np.testing.assert_allclose(Tt[I], T_np[I], rtol=1e-12)
    np.testing.assert_allclose(Tt[0, 1:-1, 1:-1], T_np[0, 1:-1, 1:-1], rtol=1e-12)
    np.testing.assert_allclose(Tt[1:-1, 1:-1, -1], T_np[1:-1, 1:-1, -1], rtol=1e-12)
