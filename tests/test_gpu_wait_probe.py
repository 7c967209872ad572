"""The bounded-wait path of the TMA-fed step kernels, made to run out on
purpose without faulting or hanging anything: the wait probe (``pfg_tune``
key 8) makes every thread of every CTA wait, for the given number of clock
cycles, on a shared-memory barrier that nothing ever arrives on.  The wait
runs out, the kernel sets the device error flag (PFG_ERR_TIMEOUT), waits for
its bulk copies in flight with the full bound and returns early.  The host
reads the flag; the context stays usable, and the next step without the
probe gives exactly the clean result."""
import numpy as np
import pytest
import torch

from tests.cases import pf_case

pytestmark = pytest.mark.gpu

PFG_ERR_TIMEOUT = 6


@pytest.fixture(scope="module", autouse=True)
def _built():
    from jax_am_gb300 import _build
    _build.build()


def _step(solver, eta, T, fused=None):
    if fused is not None:
        fused.run(1, graph=False)
        torch.cuda.synchronize()
        return fused.state.clone(), fused.T_ghosted.clone()
    state, _ = solver.stepper((eta, 0.0), 1e-8, [T])
    torch.cuda.synchronize()
    return state[0], None


@pytest.mark.parametrize("variant,kernel", [(0, 4), (3, 3)], ids=["lane", "tma"])
@pytest.mark.parametrize("fused", [False, True], ids=["T_array", "fused_heat"])
def test_wait_probe_times_out_and_recovers(variant, kernel, fused):
    from jax_am_gb300 import _lib
    from jax_am_gb300.phase_field.allen_cahn import PFSolver, make_pf_params
    from jax_am_gb300.runner import HeatPFRun, single_track
    from jax_am_gb300.workloads import gamma_args
    lib = _lib.load()
    assert lib.pfg_set_kernel_variant(variant) == 0
    try:
        poly, eta, T, pf_args, _, _ = pf_case((40, 24, 12), 20, 0.15, seed=3)
        s = PFSolver(pf_args, poly)
        assert _lib.describe_plan(make_pf_params(pf_args, poly))["kernel"] == kernel
        eta_d = torch.tensor(eta, dtype=torch.float32, device="cuda")
        T_d = torch.tensor(T, dtype=torch.float32, device="cuda")

        def fresh():
            if not fused:
                return None
            return HeatPFRun(s, gamma_args(), single_track(5e-6, 12e-6, 0.8, 200.0, 1.0),
                             eta0=eta_d)
        assert _lib.device_error(clear=True) == 0
        clean = _step(s, eta_d, T_d, fresh())
        assert _lib.device_error(clear=True) == 0
        assert lib.pfg_tune(8, 20000) == 0  # probe: about 10 us on a barrier nobody completes
        try:
            _step(s, eta_d, T_d, fresh())
            err = _lib.device_error(clear=True)
        finally:
            assert lib.pfg_tune(8, 0) == 0
        assert err == PFG_ERR_TIMEOUT
        again = _step(s, eta_d, T_d, fresh())
        assert _lib.device_error(clear=True) == 0
        assert torch.equal(again[0], clean[0])
        if fused:
            assert torch.equal(again[1], clean[1])
    finally:
        lib.pfg_set_kernel_variant(0)
