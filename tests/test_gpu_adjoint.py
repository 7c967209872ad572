"""The hand-written adjoint of the fused heat + phase-field run against float64
autograd of the oracle's PyTorch restatement (the stand-in for the
reference's jax.grad) and against central finite differences at 1e-3
relative.  Tolerance: 2e-2 relative on dJ/dP and dJ/dv, 2e-2 relative
(l2) on dJ/d eta0 (the GPU forward and adjoint are float32)."""
import numpy as np
import pytest
import torch

from oracle import pf_torch as PT
from tests.cases import GAMMA_DEFAULTS, f32, pf_case

pytestmark = pytest.mark.gpu
GRAD_RTOL = 2e-2


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def _setup(aniso, steps, ckpt, shape=(10, 8, 6), n=4, seed=3):
    poly, eta, _, pf_args, oargs, _ = pf_case(shape, n, aniso, seed=seed, h=(1e-6,) * 3,
                                              noise=0.6)
    nx, ny, nz = shape
    rng = np.random.default_rng(seed + 1)
    Tg = f32(rng.uniform(1000.0, 1400.0, (nz + 2, ny + 2, nx + 2)))
    g = dict(GAMMA_DEFAULTS, r=8e-6)
    w = f32(rng.random(n))
    return poly, eta, Tg, pf_args, oargs, g, w


def _torch_J(P, v, eta0, Tg, oargs, g, w, dirs, steps, dt, x_start, y, shape):
    nx, ny, nz = shape
    e = eta0.reshape(nz, ny, nx, -1)
    T = Tg
    t = 0.0
    for _ in range(steps):
        def laser(tm, P=P, v=v):
            return x_start + v * tm, y, P
        e, T = PT.coupled_step(e, T, t, dt, oargs, g, laser, dirs)
        t += dt
    return torch.mean(torch.sum(w * e.reshape(-1, e.shape[-1]) ** 2, dim=1))


@pytest.mark.parametrize("aniso,steps,ckpt", [(0.0, 12, 5), (0.15, 10, 4)])
def test_adjoint_matches_float64_autograd_and_fd(aniso, steps, ckpt):
    from jax_am_gb300.adjoint import HeatPFObjective, LaserTrackProblem
    shape = (10, 8, 6)
    poly, eta, Tg, pf_args, oargs, g, w = _setup(aniso, steps, ckpt, shape)
    dt = float(np.float32(3e-8))
    x_start, y = 2e-6, 4e-6
    P0, v0 = 2.0, 0.8
    prob = LaserTrackProblem(pf_args, poly, g, w, dt, steps, x_start, y, checkpoint_every=ckpt,
                             T_init=torch.tensor(Tg))
    # the GPU run through the autograd node
    P = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
    v = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    e0 = torch.tensor(eta, dtype=torch.float32, device="cuda", requires_grad=True)
    J = HeatPFObjective.apply(P, v, e0, prob)
    J.backward()
    gP, gv, ge = P.grad.item(), v.grad.item(), e0.grad.double().cpu().numpy()

    # float64 autograd of the oracle restatement
    dirs = torch.tensor(poly.unique_grain_directions)
    Pt = torch.tensor(P0, dtype=torch.float64, requires_grad=True)
    vt = torch.tensor(v0, dtype=torch.float64, requires_grad=True)
    et = torch.tensor(eta, dtype=torch.float64, requires_grad=True)
    wt = torch.tensor(w)
    Tt = torch.tensor(Tg)
    Jt = _torch_J(Pt, vt, et, Tt, oargs, g, wt, dirs, steps, dt, x_start, y, shape)
    Jt.backward()
    rP = abs(gP - Pt.grad.item()) / abs(Pt.grad.item())
    rv = abs(gv - vt.grad.item()) / abs(vt.grad.item())
    ref_e = et.grad.numpy()
    re = np.linalg.norm(ge - ref_e) / np.linalg.norm(ref_e)
    print(f"A={aniso}: J gpu {J.item():.8e} vs f64 {Jt.item():.8e}; "
          f"dJ/dP {gP:.6e} vs {Pt.grad.item():.6e} (rel {rP:.2e}); "
          f"dJ/dv {gv:.6e} vs {vt.grad.item():.6e} (rel {rv:.2e}); dJ/deta0 rel {re:.2e}")
    assert abs(J.item() - Jt.item()) <= 1e-5 * abs(Jt.item())
    assert rP <= GRAD_RTOL and rv <= GRAD_RTOL and re <= GRAD_RTOL

    # central finite differences at 1e-3 relative on the float64 forward
    with torch.no_grad():
        def Jf(Pv, vv, ev):
            return _torch_J(torch.tensor(Pv), torch.tensor(vv), ev, Tt, oargs, g, wt, dirs, steps,
                            dt, x_start, y, shape).item()
        eps = 1e-3
        fdP = (Jf(P0 * (1 + eps), v0, torch.tensor(eta)) -
               Jf(P0 * (1 - eps), v0, torch.tensor(eta))) / (2 * eps * P0)
        fdv = (Jf(P0, v0 * (1 + eps), torch.tensor(eta)) -
               Jf(P0, v0 * (1 - eps), torch.tensor(eta))) / (2 * eps * v0)
        rng = np.random.default_rng(9)
        dirn = rng.standard_normal(eta.shape)
        he = 1e-3
        fde = (Jf(P0, v0, torch.tensor(eta + he * dirn)) -
               Jf(P0, v0, torch.tensor(eta - he * dirn))) / (2 * he)
    rfP = abs(gP - fdP) / abs(fdP)
    rfv = abs(gv - fdv) / abs(fdv)
    rfe = abs(np.sum(ge * dirn) - fde) / abs(fde)
    print(f"   FD: dJ/dP {fdP:.6e} (rel {rfP:.2e}), dJ/dv {fdv:.6e} (rel {rfv:.2e}), "
          f"directional dJ/deta0 {fde:.6e} (rel {rfe:.2e})")
    assert rfP <= GRAD_RTOL and rfv <= GRAD_RTOL and rfe <= GRAD_RTOL
    from jax_am_gb300 import _lib
    assert _lib.device_error() == 0
