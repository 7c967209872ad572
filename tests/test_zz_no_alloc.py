"""The allocation-free diagnostics entry point, called through the C ABI.

pfg_pf_diag_noalloc exists for callers that may not allocate device memory
or pass a scratch buffer (a host framework that owns all device memory and
hands a plugin only pre-planned buffers, or a fixed-budget real-time loop).
It keeps its partial sums in a static device array instead.  This test calls
it twice in a row -- a large grid, then a smaller one, so leftovers of the
first call sit in the shared array during the second -- and checks each
result against the allocating pfg_pf_diag.  The file sorts last so a run that
stops at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest
import torch

from tests.cases import pf_case

pytestmark = pytest.mark.gpu


def _diag_dict(raw):
    from jax_am_gb300 import _lib
    d = _lib.Diag.from_buffer_copy(raw.cpu().numpy().tobytes())
    return d


def test_noalloc_diag_matches_allocating_entry_point():
    from jax_am_gb300 import _build, _lib
    from jax_am_gb300.phase_field.allen_cahn import make_pf_params
    _build.build()
    lib = _lib.load()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for shape, n, seed in (((61, 37, 23), 20, 41), ((9, 7, 5), 7, 42)):
        poly, eta, T, pf_args, _, _ = pf_case(shape, n, 0.0, seed=seed)
        params = make_pf_params(pf_args, poly)
        N = int(np.prod(shape))
        eta_d = torch.tensor(eta, dtype=torch.float32, device="cuda")
        T_d = torch.tensor(T, dtype=torch.float32, device="cuda")
        a0 = torch.tensor(np.argmax(np.roll(eta, 1, axis=1), axis=1), dtype=torch.int32,
                          device="cuda")
        nbytes = lib.pfg_pf_diag_scratch_bytes(ctypes.byref(params))
        scratch = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        size = ctypes.sizeof(_lib.Diag)
        out_ref = torch.zeros(size, dtype=torch.uint8, device="cuda")
        out_new = torch.zeros(size, dtype=torch.uint8, device="cuda")
        am_ref = torch.empty(N, dtype=torch.int32, device="cuda")
        am_new = torch.empty(N, dtype=torch.int32, device="cuda")
        st = lib.pfg_pf_diag(ctypes.byref(params), _lib.ptr(eta_d), _lib.ptr(T_d), 0,
                             _lib.ptr(a0), _lib.ptr(am_ref), _lib.ptr(scratch), nbytes,
                             _lib.ptr(out_ref), stream)
        _lib.check(st, "pfg_pf_diag")
        st = lib.pfg_pf_diag_noalloc(ctypes.byref(params), _lib.ptr(eta_d), _lib.ptr(T_d), 0,
                                     _lib.ptr(a0), _lib.ptr(am_new), _lib.ptr(out_new), stream)
        _lib.check(st, "pfg_pf_diag_noalloc")
        torch.cuda.synchronize()
        ref, new = _diag_dict(out_ref), _diag_dict(out_new)
        assert new.n_cells == ref.n_cells == N
        assert new.n_ori_changed == ref.n_ori_changed
        assert new.n_liquid == ref.n_liquid
        assert new.n_nonfinite == ref.n_nonfinite == 0
        assert new.max_T == pytest.approx(ref.max_T, rel=1e-12)
        assert new.energy == pytest.approx(ref.energy, rel=1e-12)
        np.testing.assert_allclose(np.array(new.mass[:n]), np.array(ref.mass[:n]), rtol=1e-12)
        assert torch.equal(am_new, am_ref)
