"""FP64 CPU oracle for the phase-field grain-growth step and the explicit heat step.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the
checker or as the timed CPU baseline.  The product path (``jax_am_gb300``)
never calls it.

It restates, in plain NumPy float64, the reference JAX-AM algorithm for:

* the multi-order-parameter Allen-Cahn right-hand side
  (``jax_am/phase_field/allen_cahn.py:42-85``), including the cubic
  anisotropy helper written with ``arccos`` exactly as the reference does
  (``allen_cahn.py:28-39``);
* the explicit Euler update (``allen_cahn.py:106-114``);
* the liquid forcing (``allen_cahn.py:117-128``);
* the one-hot initial condition (``allen_cahn.py:145-153``);
* the run-time inspection metrics (``allen_cahn.py:165-180``);
* the explicit finite-difference heat step with Robin/radiation faces and a
  Gaussian surface flux (``jax_am/cfd/gamma.py:9-61``), on the reference's
  ghosted ``(nx+2, ny+2, nz+2)`` x-major layout;
* the analytic temperature sources of the phase-field drivers
  (``applications/phase_field/solidification/example.py:21-34``,
  ``applications/phase_field/simple/example.py:21-37``,
  ``applications/phase_field/multi_scan/example.py:33-84``);
* the grain post-processing of ``process_eta``: breadth-first search for
  same-orientation solid components and their volumes and PCA aspect ratios
  (``jax_am/phase_field/utils.py:181-310``).

Parity pin: the functions here are checked against golden vectors that the
reference's own source files produced when run in this container with a
NumPy/PyTorch stand-in for the absent ``jax`` package
(``tests/golden/make_golden.py``).  JAX itself could not be run, so the pin
is "reference source under a stand-in", not "reference under JAX".

Extensions beyond the reference (checked only against this oracle's own
consistency): periodic boundaries per axis (``bc``) and liquid forcing as a
flag.
"""
import numpy as np

NEUMANN = "neumann"
PERIODIC = "periodic"


# ---------------------------------------------------------------------------
# Phase field
# ---------------------------------------------------------------------------

def zeta_of_T(T, T_liquidus):
    """Liquid indicator after the 2000 K clip (``allen_cahn.py:55-57``).

    Returns (T_clipped, zeta)."""
    T = np.where(T > 2000.0, 2000.0, T)
    zeta = 0.5 * (1.0 - np.tanh(1e10 * (T / T_liquidus - 1.0)))
    return T, zeta


def local_energy_grad(eta, zeta, m_g, ad_hoc, gamma=1.0):
    """d/d(eta) of the local free energy, divided by ``ad_hoc``.

    The reference builds f = m_g [sum(eta^4/4 - eta^2/2)
    + gamma (sum_{jk} (eta_j eta_k)^2 - sum eta^4)
    + (1 - zeta)^2 sum eta^2] and differentiates it with ``jax.grad``
    (``allen_cahn.py:42-51,58``).  Differentiating by hand, with
    S = sum_j eta_j^2 per cell:
    df/deta_i = m_g [eta_i^3 - eta_i + 4 gamma eta_i (S - eta_i^2)
    + 2 (1 - zeta)^2 eta_i].
    """
    S = np.sum(eta ** 2, axis=1, keepdims=True)
    z = zeta.reshape(-1, 1)
    g = eta ** 3 - eta + 4.0 * gamma * eta * (S - eta ** 2) + 2.0 * (1.0 - z) ** 2 * eta
    return m_g * g / ad_hoc


def neighbours(eta4, bc=(NEUMANN, NEUMANN, NEUMANN)):
    """The six shifted copies of eta on the ``(Nz, Ny, Nx, n)`` grid.

    Neumann = replicate the edge cell, as the reference's concatenations do
    (``allen_cahn.py:60-66``); periodic wraps around (extension).
    ``bc`` is given per axis in (x, y, z) order.
    Returns (neg_x, pos_x, neg_y, pos_y, neg_z, pos_z)."""
    out = []
    for axis_xyz, grid_axis in ((0, 2), (1, 1), (2, 0)):
        if bc[axis_xyz] == PERIODIC:
            neg = np.roll(eta4, 1, axis=grid_axis)
            pos = np.roll(eta4, -1, axis=grid_axis)
        else:
            n_ax = eta4.shape[grid_axis]
            idx_neg = np.concatenate(([0], np.arange(n_ax - 1)))
            idx_pos = np.concatenate((np.arange(1, n_ax), [n_ax - 1]))
            neg = np.take(eta4, idx_neg, axis=grid_axis)
            pos = np.take(eta4, idx_pos, axis=grid_axis)
        out += [neg, pos]
    return tuple(out)


def anisotropy_term(edges, grain_dirs, anisotropy):
    """Cubic anisotropy factor per (cell, orientation) (``allen_cahn.py:28-39``).

    ``edges`` is ``(Nz, Ny, Nx, n, 3)``: the central differences
    (eta_+ - eta_-) along x, y, z.  ``grain_dirs`` is ``(3, n, 3)``: the three
    rotated cube axes of every orientation.  Written with ``arccos`` and the
    NaN-to-zero rule exactly as the reference does."""
    n = grain_dirs.shape[1]
    e = edges.reshape(-1, n, 3)
    norm = np.linalg.norm(e, axis=-1)
    with np.errstate(invalid="ignore", divide="ignore"):
        cosines = np.sum(grain_dirs[None, :, :, :] * e[:, None, :, :], axis=-1) / norm[:, None, :]
        angles = np.arccos(cosines)
    angles = np.where(np.isfinite(angles), angles, 0.0)
    angles = np.where(angles < np.pi / 2.0, angles, np.pi - angles)
    angles = np.min(angles, axis=1)
    a = 1.0 + anisotropy * (np.cos(angles) ** 4 + np.sin(angles) ** 4)
    return a.reshape(edges.shape[:4])


def pf_rhs(eta, T, args, grain_dirs=None, bc=(NEUMANN, NEUMANN, NEUMANN)):
    """Right-hand side d(eta)/dt (``allen_cahn.py:53-85``).

    eta: ``(N, n)`` cells in z-major order (x fastest), orientation innermost.
    T: ``(N, 1)`` or ``(N,)``.  ``args`` holds the reference ``pf_args`` keys
    (Nx, Ny, Nz, num_oris, T_liquidus, gas_const, Qg, L0, kappa_g, m_g,
    anisotropy, ad_hoc) plus ``h`` = (h_x, h_y, h_z)."""
    Nx, Ny, Nz, n = args["Nx"], args["Ny"], args["Nz"], args["num_oris"]
    hx, hy, hz = args["h"]
    T = np.asarray(T, dtype=np.float64).reshape(-1, 1)
    T, zeta = zeta_of_T(T, args["T_liquidus"])
    grad = local_energy_grad(eta, zeta, args["m_g"], args["ad_hoc"])
    e4 = eta.reshape(Nz, Ny, Nx, n)
    nx_, px_, ny_, py_, nz_, pz_ = neighbours(e4, bc)
    if args["anisotropy"] > 0.0:
        edges = np.stack((px_ - nx_, py_ - ny_, pz_ - nz_), axis=-1)
        aniso = anisotropy_term(edges, grain_dirs, args["anisotropy"])[..., None]
    else:
        aniso = 1.0
    lap_xyz = -(np.stack((((px_ - e4) + (nx_ - e4)) / hx ** 2,
                          ((py_ - e4) + (ny_ - e4)) / hy ** 2,
                          ((pz_ - e4) + (nz_ - e4)) / hz ** 2), axis=-1)
                * aniso * args["kappa_g"] * args["ad_hoc"])
    lap = np.sum(lap_xyz.reshape(-1, n, 3), axis=-1)
    Lg = args["L0"] * np.exp(-args["Qg"] / (T * args["gas_const"]))
    return -Lg * (grad + lap)


def explicit_euler(eta, t_prev, t_crt, T, args, grain_dirs=None, bc=(NEUMANN,) * 3):
    """y <- y + (t_crt - t_prev) f(y, t_prev, [T]) (``allen_cahn.py:106-114``)."""
    return eta + (t_crt - t_prev) * pf_rhs(eta, T, args, grain_dirs, bc)


def force_liquid_zero(eta, T, T_liquidus, shift=1.0):
    """eta = 0 where T > T_liquidus + shift (``allen_cahn.py:117-128``)."""
    liquid = np.asarray(T).reshape(-1, 1) > T_liquidus + shift
    return np.where(liquid, 0.0, eta)


def ini_cond(cell_ori_inds, num_oris):
    """One-hot eta from the per-cell orientation index (``allen_cahn.py:145-153``)."""
    N = len(cell_ori_inds)
    eta = np.zeros((N, num_oris))
    eta[np.arange(N), cell_ori_inds] = 1.0
    return eta


def inspect(eta, eta0, T, T_liquidus):
    """The metrics ``PFSolver.inspect_sol`` prints (``allen_cahn.py:165-180``).

    Returns a dict with the percentage of cells whose argmax orientation
    changed, the percentage of cells with T >= T_liquidus, max T and whether
    every eta is finite."""
    a0 = np.argmax(eta0, axis=1)
    a1 = np.argmax(eta, axis=1)
    T = np.asarray(T).reshape(-1)
    return {
        "pct_ori_changed": float(np.sum(a0 != a1) / len(a1) * 100.0),
        "pct_liquid": float(np.sum(T >= T_liquidus) / len(T) * 100.0),
        "max_T": float(np.max(T)),
        "all_finite": bool(np.all(np.isfinite(eta))),
    }


def free_energy(eta, T, args, grain_dirs=None, bc=(NEUMANN,) * 3):
    """Total free energy F = sum over cells of [local + gradient] energy times
    the cell volume, in float64.  The local part is the reference's
    ``local_energy_fn`` (``allen_cahn.py:42-49``) per cell; the gradient part
    is kappa_g/2 sum_i a_i |grad eta_i|^2 with one-sided forward differences
    (zero across Neumann faces).  Used as a diagnostic, not by the step."""
    Nx, Ny, Nz, n = args["Nx"], args["Ny"], args["Nz"], args["num_oris"]
    hx, hy, hz = args["h"]
    T = np.asarray(T, dtype=np.float64).reshape(-1, 1)
    _, zeta = zeta_of_T(T, args["T_liquidus"])
    S = np.sum(eta ** 2, axis=1)
    f_loc = (np.sum(eta ** 4 / 4.0 - eta ** 2 / 2.0, axis=1)
             + (S ** 2 - np.sum(eta ** 4, axis=1))
             + (1.0 - zeta.reshape(-1)) ** 2 * S)
    f_loc = args["m_g"] * f_loc
    e4 = eta.reshape(Nz, Ny, Nx, n)
    _, px_, _, py_, _, pz_ = neighbours(e4, bc)
    g2 = ((px_ - e4) / hx) ** 2 + ((py_ - e4) / hy) ** 2 + ((pz_ - e4) / hz) ** 2
    f_grad = 0.5 * args["kappa_g"] * np.sum(g2.reshape(-1, n), axis=1)
    vol = hx * hy * hz
    return float(np.sum(f_loc + f_grad) * vol)


# ---------------------------------------------------------------------------
# Explicit finite-difference heat equation (jax_am/cfd/gamma.py)
# ---------------------------------------------------------------------------

def heat_update_mat(T, g):
    """Liquid fraction, conductivity and heat capacity (``gamma.py:9-15``)."""
    fl = (np.clip(T, g["Ts"], g["Tl"]) - g["Ts"]) / (g["Tl"] - g["Ts"])
    k = 0.0163 * np.clip(T, 300.0, g["Tl"]) + 4.5847
    cp = 0.2441 * np.clip(T, 300.0, g["Tl"]) + 338.39 + (fl > 0) * (fl < 1) * g["L"]
    return fl, k, cp


def _robin(Tf, g, sign):
    return sign * (g["h"] * (Tf - g["T0"]) + g["SB"] * g["eps"] * (Tf ** 4 - g["T0"] ** 4))


def heat_bc(T, k, xl, yl, x_top, y_top, P, dx, dy, dz, g):
    """Ghost faces from convection + radiation, plus the Gaussian surface flux
    on the top z face (``gamma.py:18-43``).  ``T`` is ``(nx+2, ny+2, nz+2)``;
    ``x_top``/``y_top`` are the ``(nx, ny)`` cell-centre coordinates of the
    top interior layer.  Every face flux is computed from the incoming T
    before any ghost is overwritten, as in the reference."""
    T = T.copy()
    I = slice(1, -1)
    q_xn = _robin((T[1, I, I] + T[0, I, I]) / 2.0, g, -1.0)
    q_xp = _robin((T[-2, I, I] + T[-1, I, I]) / 2.0, g, 1.0)
    q_yn = _robin((T[I, 1, I] + T[I, 0, I]) / 2.0, g, -1.0)
    q_yp = _robin((T[I, -2, I] + T[I, -1, I]) / 2.0, g, 1.0)
    q_zn = _robin((T[I, I, 1] + T[I, I, 0]) / 2.0, g, -1.0)
    q_zp = (_robin((T[I, I, -2] + T[I, I, -1]) / 2.0, g, 1.0)
            - 2.0 * P * g["eta"] / np.pi / g["r"] ** 2
            * np.exp(-2.0 * ((x_top - xl) ** 2 + (y_top - yl) ** 2) / g["r"] ** 2))
    T[0, I, I] = T[1, I, I] + q_xn / k[1, I, I] * dx
    T[-1, I, I] = T[-2, I, I] - q_xp / k[-2, I, I] * dx
    T[I, 0, I] = T[I, 1, I] + q_yn / k[I, 1, I] * dy
    T[I, -1, I] = T[I, -2, I] - q_yp / k[I, -2, I] * dy
    T[I, I, 0] = T[I, I, 1] + q_zn / k[I, I, 1] * dz
    T[I, I, -1] = T[I, I, -2] - q_zp / k[I, I, -2] * dz
    return T


def heat_laplace(f, dx, dy, dz):
    """Second differences on the interior (``gamma.py:46-52``)."""
    f_xx = (f[0:-2, :, :] - 2 * f[1:-1, :, :] + f[2:, :, :]) / dx ** 2
    f_yy = (f[:, 0:-2, :] - 2 * f[:, 1:-1, :] + f[:, 2:, :]) / dy ** 2
    f_zz = (f[:, :, 0:-2] - 2 * f[:, :, 1:-1] + f[:, :, 2:]) / dz ** 2
    return f_xx[:, 1:-1, 1:-1], f_yy[1:-1, :, 1:-1], f_zz[1:-1, 1:-1, :]


def heat_update_T(T, xl, yl, x_top, y_top, P, dx, dy, dz, dt, g):
    """One explicit heat step (``gamma.py:55-61``); ghosts are part of the state."""
    _, k, cp = heat_update_mat(T, g)
    T = heat_bc(T, k, xl, yl, x_top, y_top, P, dx, dy, dz, g)
    T_xx, T_yy, T_zz = heat_laplace(T, dx, dy, dz)
    T = T.copy()
    T[1:-1, 1:-1, 1:-1] += dt * (k[1:-1, 1:-1, 1:-1] / g["rho"] / cp[1:-1, 1:-1, 1:-1]
                                 * (T_xx + T_yy + T_zz))
    return T


def cell_centres_top(nx, ny, dx, dy):
    """(nx, ny) cell-centre x and y of the top layer, as the heat driver builds
    them (``applications/cfd/gamma/example.py:61-65``)."""
    x_ = dx / 2.0 + dx * np.arange(nx)
    y_ = dy / 2.0 + dy * np.arange(ny)
    return np.meshgrid(x_, y_, indexing="ij")


def coupled_step(eta, Tg, t, dt, args, g, laser, grain_dirs=None,
                 bc=(NEUMANN,) * 3, force_liquid=False, shift=1.0):
    """One fused heat + phase-field step.

    The phase-field update uses the temperature at the start of the step, as
    the reference drivers do (``applications/phase_field/solidification/
    example.py:83-86``: T is refreshed after ``stepper``).  The heat step is
    ``gamma.update_T`` with the laser at the mid-step time, as the heat driver
    samples it (``applications/cfd/gamma/example.py:88``).  ``laser(t)``
    returns (xl, yl, P).  ``Tg`` is the reference ghosted x-major layout."""
    Nx, Ny, Nz = args["Nx"], args["Ny"], args["Nz"]
    hx, hy, hz = args["h"]
    T_int = Tg[1:-1, 1:-1, 1:-1].transpose(2, 1, 0).reshape(-1, 1)
    eta_new = explicit_euler(eta, t, t + dt, T_int, args, grain_dirs, bc)
    if force_liquid:
        eta_new = force_liquid_zero(eta_new, T_int, args["T_liquidus"], shift)
    xl, yl, P = laser(t + 0.5 * dt)
    x_top, y_top = cell_centres_top(Nx, Ny, hx, hy)
    Tg_new = heat_update_T(Tg, xl, yl, x_top, y_top, P, hx, hy, hz, dt, g)
    return eta_new, Tg_new


# ---------------------------------------------------------------------------
# Analytic temperature sources of the phase-field drivers
# ---------------------------------------------------------------------------

def T_quench(centroids, t, T_liquidus, thermal_grad=5e5, vel=0.2, z0=0.0):
    """Moving linear gradient (``solidification/example.py:21-34``), with an
    optional front offset ``z0`` (zero in the reference)."""
    z = centroids[:, 2]
    return (T_liquidus + thermal_grad * (z - z0) - thermal_grad * vel * t)[:, None]


def T_rosenthal(centroids, t, T_ambient, x0, vel, y_c, z_top, Q=25.0, alpha=5.2e-6, kappa=27.0):
    """Moving point source (``simple/example.py:21-37``)."""
    X = centroids[:, 0] - x0 - vel * t
    Y = centroids[:, 1] - y_c
    Z = centroids[:, 2] - z_top
    R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    return (T_ambient + Q / (2 * np.pi * kappa) / R * np.exp(-vel / (2 * alpha) * (R + X)))[:, None]


def T_rosenthal_path(centroids, T_ambient, vel, xl, yl, zl, unit_dir,
                     Q=25.0, alpha=5.2e-6, kappa=27.0):
    """Point source along a tool path, clipped at 2000 K
    (``multi_scan/example.py:33-49``)."""
    X = centroids[:, 0] - xl
    Y = centroids[:, 1] - yl
    Z = centroids[:, 2] - zl
    R = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    proj = X * unit_dir[0] + Y * unit_dir[1] + Z * unit_dir[2]
    T = T_ambient + Q / (2 * np.pi * kappa) / R * np.exp(-vel / (2 * alpha) * (R + proj))
    return np.where(T > 2000.0, 2000.0, T)[:, None]


def read_path(x_corners, y_corners, z_corners, switch, vel, dt):
    """Raster tool path sampled at dt (``multi_scan/example.py:52-84``)."""
    power = switch[:-1]
    ts, xs, ys, zs, ps, dirs = [], [], [], [], [], []
    t_pre = 0.0
    for i in range(len(x_corners) - 1):
        d = np.array([x_corners[i + 1] - x_corners[i], y_corners[i + 1] - y_corners[i],
                      z_corners[i + 1] - z_corners[i]])
        dist = np.linalg.norm(d)
        travel = dist / vel
        t_seg = np.arange(t_pre, t_pre + travel, dt)
        m = len(t_seg)
        ts.append(t_seg)
        xs.append(np.linspace(x_corners[i], x_corners[i + 1], m))
        ys.append(np.linspace(y_corners[i], y_corners[i + 1], m))
        zs.append(np.linspace(z_corners[i], z_corners[i + 1], m))
        ps.append(np.linspace(power[i], power[i], m))
        dirs.append(np.repeat((d / dist)[None, :], m, axis=0))
        t_pre += travel
    return (np.hstack(ts), np.hstack(xs), np.hstack(ys), np.hstack(zs), np.hstack(ps),
            np.vstack(dirs))


# ---------------------------------------------------------------------------
# Grain post-processing (jax_am/phase_field/utils.py:181-310)
# ---------------------------------------------------------------------------

def grain_components(ori, T, T_liquidus, Nx, Ny, Nz):
    """Connected same-orientation solid components, numbered as the
    reference's ``BFS`` + ``combined`` list orders them (``utils.py:
    219-263``): by orientation, then by discovery in increasing cell index.
    Solid means ``T < T_liquidus`` (``utils.py:193``); the graph is the
    6-neighbourhood without wrap (``compute_edges_in_order``,
    ``utils.py:219-235``).  Returns (labels (N,), -1 in liquid; K)."""
    from collections import deque
    N = Nx * Ny * Nz
    ori = np.asarray(ori).reshape(-1)
    solid = np.asarray(T).reshape(-1) < T_liquidus
    comp = -np.ones(N, dtype=np.int64)
    found = []  # (orientation, first cell) of every component in discovery order
    for i in range(N):
        if comp[i] >= 0 or not solid[i]:
            continue
        k = len(found)
        found.append((int(ori[i]), i))
        comp[i] = k
        q = deque([i])
        while q:
            s = q.popleft()
            z, r = divmod(s, Nx * Ny)
            y, x = divmod(r, Nx)
            for dx, dy, dz in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
                xx, yy, zz = x + dx, y + dy, z + dz
                if 0 <= xx < Nx and 0 <= yy < Ny and 0 <= zz < Nz:
                    c = (zz * Ny + yy) * Nx + xx
                    if comp[c] < 0 and solid[c] and ori[c] == ori[i]:
                        comp[c] = k
                        q.append(c)
    order = sorted(range(len(found)), key=lambda k: found[k])
    rank = np.empty(len(found), dtype=np.int64)
    rank[order] = np.arange(len(found))
    labels = np.where(comp >= 0, rank[np.maximum(comp, 0)], -1)
    return labels, len(found)


def grain_volumes_and_aspect_ratios(labels, K, Nx, Ny, Nz, h):
    """``get_aspect_ratio_inputs`` + ``compute_aspect_ratios_and_vols``
    (``utils.py:266-310``): volume = cells x domain_vol / N (uniform cells,
    ``utils.py:204-205``); grains of fewer than 5 cells get aspect ratio 1;
    otherwise the PCA explained variances ev (covariance eigenvalues with
    ddof = 1, descending) of the volume-weighted cell centres give
    2 sqrt(ev0) / (sqrt(ev1) + sqrt(ev2))."""
    N = Nx * Ny * Nz
    vol = (Nx * h) * (Ny * h) * (Nz * h) / N
    zz, yy, xx = np.meshgrid(np.arange(Nz), np.arange(Ny), np.arange(Nx), indexing="ij")
    cent = np.stack(((xx.ravel() + 0.5) * h, (yy.ravel() + 0.5) * h, (zz.ravel() + 0.5) * h), axis=1)
    vols, ars = [], []
    for k in range(K):
        cells = np.nonzero(labels == k)[0]
        vols.append(len(cells) * vol)
        if len(cells) < 5:
            ars.append(1.0)
            continue
        p = cent[cells] * vol
        ev = np.sort(np.linalg.eigvalsh(np.cov(p.T, ddof=1)))[::-1]
        ln = np.sqrt(np.maximum(ev, 0.0))
        with np.errstate(divide="ignore", invalid="ignore"):
            ars.append(2.0 * ln[0] / (ln[1] + ln[2]))
    return np.array(vols), np.array(ars)



def rk4(eta, t_prev, t_crt, T, args, grain_dirs=None, bc=(NEUMANN,) * 3):
    """Fourth-order Runge-Kutta step (``allen_cahn.py:91-104``) with T held."""
    h = t_crt - t_prev
    k1 = h * pf_rhs(eta, T, args, grain_dirs, bc)
    k2 = h * pf_rhs(eta + k1 / 2.0, T, args, grain_dirs, bc)
    k3 = h * pf_rhs(eta + k2 / 2.0, T, args, grain_dirs, bc)
    k4 = h * pf_rhs(eta + k3, T, args, grain_dirs, bc)
    return eta + (k1 + 2 * k2 + 2 * k3 + k4) / 6.0
