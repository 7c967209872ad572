"""The C-ABI library on a machine without a GPU: it builds, loads, exports
every entry point the header declares, its structs match the Python mirrors,
and argument validation answers without touching a device."""
import ctypes
import os
import re

import pytest

from jax_am_gb300 import _build, _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "pf_gb300.h")


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pfg_\w+)\s*\(", text)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 8
    for name in names:
        assert hasattr(lib, name), f"{name} declared in pf_gb300.h but not exported"


def test_struct_sizes_match(lib):
    for which, cls in _lib._STRUCTS:
        assert lib.pfg_struct_size(which) == ctypes.sizeof(cls)
    assert lib.pfg_abi_version() == 1


def _params(**kw):
    p = _lib.PfParams()
    p.nx, p.ny, p.nz, p.num_oris = 4, 4, 4, 3
    p.h_x = p.h_y = p.h_z = 1e-6
    p.T_liquidus, p.gas_const, p.Qg, p.L0 = 1623.0, 8.3, 1.4e5, 3.5e3
    p.kappa_g, p.m_g, p.anisotropy, p.ad_hoc = 2.77e-6, 2.4e5, 0.0, 1.0
    for k, v in kw.items():
        setattr(p, k, v)
    return p


@pytest.mark.parametrize("kw,status", [
    (dict(nx=0), 1), (dict(num_oris=0), 1), (dict(num_oris=65), 1), (dict(h_y=0.0), 4),
    (dict(bc_z=7), 4), (dict(ad_hoc=0.0), 4),
])
def test_validation_without_device(lib, kw, status):
    p = _params(**kw)
    buf = ctypes.c_void_p(16)
    assert lib.pfg_pf_step(ctypes.byref(p), buf, buf, buf, 1e-8, None) == status
    assert lib.pfg_status_string(status).decode()


def test_null_and_alignment(lib):
    p = _params()
    a = ctypes.c_void_p(16)
    assert lib.pfg_pf_step(ctypes.byref(p), None, a, a, 1e-8, None) == 2
    assert lib.pfg_pf_step(ctypes.byref(p), ctypes.c_void_p(20), a, a, 1e-8, None) == 3
    assert lib.pfg_pf_step(None, a, a, a, 1e-8, None) == 2


def test_no_device_is_reported(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = _params()
    a = ctypes.c_void_p(16)
    assert lib.pfg_pf_step(ctypes.byref(p), a, a, a, 1e-8, None) == 8
    with pytest.raises(_lib.PFGError):
        _lib.check(8, "pfg_pf_step")
    with pytest.raises(ValueError):
        _lib.check(1, "pfg_pf_step")
