"""The FP64 oracle against golden vectors produced by the reference's own
source files (``tests/golden/make_golden.py``)."""
import os

import numpy as np
import pytest

from oracle import pf_oracle as O

G = os.path.join(os.path.dirname(__file__), "golden")


def _load(name):
    return np.load(os.path.join(G, name))


def _args(d):
    keys = ("dim", "T_liquidus", "gas_const", "Qg", "L0", "kappa_g", "m_g", "ad_hoc")
    a = dict(zip(keys, d["pf_keys"].tolist()))
    a.update(Nx=int(d["Nx"]), Ny=int(d["Ny"]), Nz=int(d["Nz"]), num_oris=int(d["n"]),
             anisotropy=float(d["anisotropy"]), h=tuple(d["h"].tolist()))
    return a


@pytest.mark.parametrize("name", ["pf_iso.npz", "pf_aniso.npz", "pf_aniso_n20.npz"])
def test_pf_steps_match_reference(name):
    d = _load(name)
    a = _args(d)
    eta = d["eta_in"]
    dt = float(d["dt"])
    t = 0.0
    for k in range(int(d["steps"])):
        eta = O.explicit_euler(eta, t, t + dt, d["T"], a, d["grain_dirs"])
        t += dt
        np.testing.assert_allclose(eta, d["eta_out"][k], rtol=1e-12, atol=1e-14)


def test_ini_cond_matches_reference():
    d = _load("pf_aniso.npz")
    np.testing.assert_array_equal(O.ini_cond(d["cell_ori_inds"], int(d["n"])), d["eta_ini"])


def test_force_and_inspect_match_reference():
    d = _load("pf_force_inspect.npz")
    np.testing.assert_array_equal(O.force_liquid_zero(d["eta"], d["T"], 1623.0, 1.0),
                                  d["eta_forced"])
    m = O.inspect(d["eta"], d["eta0"], d["T"], 1623.0)
    np.testing.assert_allclose([m["pct_ori_changed"], m["pct_liquid"], m["max_T"]],
                               d["inspect"], rtol=1e-12)


def _gamma(d):
    keys = ("eta", "r", "rho", "h", "eps", "SB", "T0", "Ts", "Tl", "L")
    return dict(zip(keys, d["gamma"].tolist()))


@pytest.mark.parametrize("name,dtype,rtol", [("heat_f64.npz", np.float64, 1e-13),
                                             ("heat_f32.npz", np.float32, 2e-6)])
def test_heat_matches_reference(name, dtype, rtol):
    d = _load(name)
    g = _gamma(d)
    dx, dy, dz, dt = d["dxyzt"].tolist()
    T = d["T_in"].astype(np.float64)
    nx, ny = T.shape[0] - 2, T.shape[1] - 2
    xt, yt = O.cell_centres_top(nx, ny, dx, dy)
    for k, (xl, yl, P) in enumerate(d["lasers"]):
        T = O.heat_update_T(T, xl, yl, xt, yt, P, dx, dy, dz, dt, g)
        np.testing.assert_allclose(T, d["T_out"][k], rtol=rtol)


def test_tsources_match_reference():
    d = _load("tsources.npz")
    c, t = d["centroids"], float(d["t"])
    np.testing.assert_allclose(O.T_quench(c, t, 1623.0), d["T_quench"], rtol=1e-13)
    np.testing.assert_allclose(
        O.T_rosenthal(c, t, 300.0, x0=0.2e-3, vel=0.6e-3 / 2.4e-3, y_c=1.2e-4, z_top=1e-4),
        d["T_rosenthal"], rtol=1e-12)
    ts, xs, ys, zs, ps, dirs = O.read_path([0.1e-3, 0.9e-3, 0.9e-3, 0.1e-3],
                                           [0.17e-3, 0.17e-3, 0.07e-3, 0.07e-3],
                                           [0.1e-3] * 4, [1, 1, 1, 0], 0.25, 2e-7)
    for a, b in ((ts, "path_ts"), (xs, "path_xs"), (ys, "path_ys"), (zs, "path_zs"),
                 (ps, "path_ps"), (dirs, "path_dirs")):
        np.testing.assert_allclose(a, d[b], rtol=1e-13)
    i = int(d["path_i"])
    np.testing.assert_allclose(
        O.T_rosenthal_path(c, 300.0, 0.25, xs[i], ys[i], zs[i], dirs[i]), d["T_path"], rtol=1e-12)


@pytest.mark.parametrize("case", ["voronoi_a", "voronoi_b", "voronoi_c", "shapes"])
def test_grains_match_reference(case):
    """Grain components, volumes and aspect ratios against the reference's
    own BFS / PCA code (tests/golden/make_golden_grains.py)."""
    d = np.load(os.path.join(G, "grains.npz"))
    Nx, Ny, Nz = (int(v) for v in d[f"{case}_shape"])
    labels, K = O.grain_components(d[f"{case}_ori"], d[f"{case}_T"], float(d["T_liquidus"]),
                                   Nx, Ny, Nz)
    np.testing.assert_array_equal(labels, d[f"{case}_labels"])
    vols, ars = O.grain_volumes_and_aspect_ratios(labels, K, Nx, Ny, Nz, float(d["h"]))
    np.testing.assert_allclose(vols, d[f"{case}_vols"], rtol=1e-12)
    _check_aspect_ratios(ars, d[f"{case}_ars"])


def _check_aspect_ratios(ars, ref):
    """Collinear grains have two zero PCA variances: the ratio is inf, or a
    huge finite number where rounding left the variances at ~1e-32 of the
    largest; both count as degenerate (> 1e8).  Others agree to 1e-9."""
    deg_ref = ~np.isfinite(ref) | (ref > 1e8)
    deg = ~np.isfinite(ars) | (ars > 1e8)
    assert np.array_equal(deg, deg_ref)
    np.testing.assert_allclose(ars[~deg_ref], ref[~deg_ref], rtol=1e-9)


def test_product_read_path_matches_reference():
    """The tool-path sampler of jax_am_gb300 (host side of the point-source
    step) against the reference's own read_path output."""
    from jax_am_gb300.phase_field.point_source import read_path
    d = np.load(os.path.join(G, "point_sources.npz"))
    args = dict(vel=float(d["vel"]), dt=float(d["dt"]),
                laser_path=dict(x_pos=list(d["x_pos"]), y_pos=list(d["y_pos"]),
                                z_pos=list(d["z_pos"]), switch=list(d["switch"])))
    out = read_path(args)
    for a, key in zip(out, ("path_ts", "path_xs", "path_ys", "path_zs", "path_ps", "path_dirs")):
        np.testing.assert_allclose(a, d[key], rtol=1e-13, atol=1e-18)
