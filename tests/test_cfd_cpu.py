"""Host logic of the CFD drop-in (``jax_am_gb300.cfd.cfd_am``) without a GPU:
the cp/k form probe, the mesh quantities and the moving box against the
oracle, and the C ABI's argument checks (which return before any CUDA call).
"""
import ctypes

import numpy as np
import pytest

from jax_am_gb300 import _lib
from jax_am_gb300.cfd import cfd_am as G
from oracle import cfd_oracle as C


def test_linear_clip_probe():
    # the drivers' forms (applications/cfd/ambench/example.py:44-45)
    a, b, lo, hi = G.linear_clip_params(lambda T: 0.2174 * np.clip(T, 300, 1609) + 370.0)
    assert np.allclose([a, b, lo, hi], [0.2174, 370.0, 300.0, 1609.0], rtol=1e-9)
    a, b, lo, hi = G.linear_clip_params(lambda T: 0.01674 * np.clip(T, 300.3, 1563) + 3.9)
    assert np.allclose([a, b, lo, hi], [0.01674, 3.9, 300.3, 1563.0], rtol=1e-9)
    assert G.linear_clip_params(G.LinearClip(1, 2, 3, 4)) == (1.0, 2.0, 3.0, 4.0)
    with pytest.raises(ValueError):
        G.linear_clip_params(lambda T: T ** 2)
    with pytest.raises(ValueError):
        G.linear_clip_params(lambda T: np.sin(T))


def test_mesh_matches_oracle():
    dom, N = [1e-3, 2e-4, 1e-4], [46, 9, 5]
    m, o = G.mesh3d(dom, N), C.Mesh(dom, N)
    assert np.array_equal(m.dX, o.dX) and m.dV == o.dV
    assert np.array_equal(m.D, o.D) and np.array_equal(m.dS, o.dS)
    assert np.array_equal(m.Xc, o.Xc)
    conn = m.cell_conn
    assert conn.shape == (m.cell_num, 7)
    # the cell itself first, then mirrored neighbours (x-, x+, y-, y+, z-, z+)
    assert conn[0, 0] == 0 and conn[0, 1] == 0 and conn[0, 2] == 9 * 5
    assert conn[0, 5] == 0 and conn[0, 6] == 1


def test_moving_box_matches_oracle():
    h = 5e-6
    args = dict(X0=[2e-5, 2e-5, 2.5e-5], speed=5.0, P=30.0, t_OFF=1.0)
    mesh, local = G.mesh3d([12 * h, 8 * h, 5 * h], [12, 8, 5]), G.mesh3d([8 * h, 4 * h, 3 * h],
                                                                          [8, 4, 3])
    o = C.AM3d(dict(args, T_ref=300.0), C.Mesh(mesh.domain, mesh.shape),
               C.Mesh(local.domain, local.shape))
    solver = G.AM_3d.__new__(G.AM_3d)  # the box logic needs no device state
    solver.args, solver.msh, solver.msh_local = args, mesh, local
    for step in range(12):
        t = step * 1e-6
        assert solver.get_moving_box_boundary(t) == o.box(t)
        assert solver.toolpath(t) == o.toolpath(t)


def _grid(n=(4, 3, 2), h=1e-6):
    g = _lib.CfdGrid()
    g.nx, g.ny, g.nz = n
    g.dx = g.dy = g.dz = h
    g.lx, g.ly, g.lz = (v * h for v in n)
    return g


def test_abi_checks_without_device():
    lib = _lib.load()
    g, gl = _grid(), _grid((2, 2, 1))
    need = lib.pfg_cfd_workspace_bytes(ctypes.byref(g), ctypes.byref(gl))
    assert need > 0
    fake = ctypes.c_void_p(1 << 20)  # never dereferenced: the checks return first
    e = _lib.CfdEnergy()
    e.dt, e.Ts, e.Tl, e.max_newton = 1e-6, 1563.0, 1623.0, 50
    # scratch too small -> capacity (the energy solve alone needs no local box)
    need_e = lib.pfg_cfd_workspace_bytes(ctypes.byref(g), None)
    assert 0 < need_e < need
    st = lib.pfg_cfd_energy_solve(ctypes.byref(g), ctypes.byref(e), fake, fake, fake, fake,
                                  need_e - 8, None, None)
    assert st == 7
    # bad heat-source code -> parameter error
    e.heat_source = 2
    st = lib.pfg_cfd_energy_solve(ctypes.byref(g), ctypes.byref(e), fake, fake, fake, fake, need,
                                  None, None)
    assert st == 4
    # a box that leaves the grid -> shape error
    f = _lib.CfdFlow()
    f.rho, f.visco, f.dt, f.Ts, f.Tl = 8440.0, 7e-3, 1e-6, 1563.0, 1623.0
    f.x0 = 3
    st = lib.pfg_cfd_flow_step(ctypes.byref(g), ctypes.byref(gl), ctypes.byref(f), fake, fake,
                               fake, fake, fake, fake, need, None, None)
    assert st == 1
    # NULL field -> null error
    f.x0 = 0
    st = lib.pfg_cfd_flow_step(ctypes.byref(g), ctypes.byref(gl), ctypes.byref(f), None, fake,
                               fake, fake, fake, fake, need, None, None)
    assert st == 2
    bad = _grid((0, 3, 2))
    assert lib.pfg_cfd_solid_update(ctypes.byref(bad), 1563.0, 1623.0, fake, fake, None) == 1
