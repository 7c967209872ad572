"""FP64 CPU oracle for the implicit CFD / energy solver ``AM_3d``.

TEST INFRASTRUCTURE ONLY.  Only ``tests/`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker or as the timed
CPU baseline.  The product path (``jax_am_gb300``) never calls it.

It restates, in plain NumPy float64, the finite-volume solver of
``jax_am/cfd/cfd_am.py`` on its structured (Nx, Ny, Nz) mesh (cell index
(i Ny + j) Nz + k, z fastest):

* the mesh quantities and the mirrored neighbour list of ``mesh3d``
  (``cfd_am.py:668-745``): a boundary cell's missing neighbour is the cell
  itself, so boundary faces carry no diffusive flux of their own;
* the "poisson" residual and its per-cell Jacobian (``cfd_am.py:388-493``):
  ``-sum_f (U_nb - U_p) / D_f * mu_f * dS_f - source * dV``, Dirichlet and
  Neumann faces applied to the residual (``:426-444``) and Dirichlet faces to
  the Jacobian diagonal (``:456-472``); the Jacobi preconditioner sums every
  stencil entry that points back at the cell (``:474-488``).  The Jacobian is
  written out analytically; the reference takes it with ``jax.jacrev``,
  whose derivative of ``clip`` at a tie (``x == lo`` or ``x == hi``) is 1/2
  (JAX's max/min share the gradient equally at a tie);
* the energy equation (``cfd_am.py:495-525``): conductivity ``k(T)`` through
  the harmonic face mean (``:414-417``), ``cp(T0)`` plus the latent-heat
  bump inside the mushy zone, implicit in T with explicit convection and
  source, solved by ``solver_nonlinear`` (``:780-812``: Newton, relative
  residual 1e-5, at most 50 iterations, Jacobi-preconditioned BiCGSTAB);
* BiCGSTAB with JAX's semantics (``jax.scipy.sparse.linalg.bicgstab``, the
  preconditioned algorithm of van der Vorst with JAX's stopping rule
  ``|r|^2 <= max(tol^2 |b|^2, atol^2)``, its early exit on ``|s|^2`` and its
  breakdown codes; x0 = 0, maxiter = 10 N unless given);
* the velocity equation (``cfd_am.py:528-590``): three momentum solves with
  the Darcy term ``1e7 rho (1 - fl)^2 / (fl^3 + 1e-5) u``, Dirichlet walls and
  the Marangoni shear on the top face (``:287-323``), then the pressure
  Poisson (no preconditioner, tol 1e-10) and the projection;
* face velocities, the theta-blended upwind divergence and the gradient
  (``cfd_am.py:14-139``);
* ``AM_3d.time_integration`` (``cfd_am.py:167-194``) with its tool path,
  body or surface heat source and moving local box (``:223-252``,
  ``:280-285``, ``:325-364``).

``cp`` and ``k`` are ``a clip(T, lo, hi) + b`` (``LinClip``), the form every
driver of the reference uses (``applications/cfd/simple/example.py:39-40``,
``applications/cfd/ambench/example.py:44-45``,
``applications/phase_field/coupled/example.py:73-74``).

Parity pin: checked against golden vectors that the reference's own
``cfd_am.py`` produced in this container under a NumPy/PyTorch stand-in for
the absent ``jax`` package (``tests/golden/make_golden_cfd.py``).
"""
import numpy as np


class LinClip:
    """``a * clip(T, lo, hi) + b`` with JAX's derivative (1/2 at a tie)."""

    def __init__(self, a, b, lo, hi):
        self.a, self.b, self.lo, self.hi = float(a), float(b), float(lo), float(hi)

    def __call__(self, T):
        return self.a * np.clip(T, self.lo, self.hi) + self.b

    def deriv(self, T):
        T = np.asarray(T, dtype=np.float64)
        inside = (T > self.lo) & (T < self.hi)
        tie = (T == self.lo) | (T == self.hi)
        return self.a * np.where(inside, 1.0, np.where(tie, 0.5, 0.0))


class Mesh:
    """``mesh3d`` (``cfd_am.py:668-694``): a box of N cells."""

    def __init__(self, domain, N):
        self.shape = tuple(int(n) for n in N)
        self.domain = tuple(float(d) for d in domain)
        self.dX = np.array([d / n for d, n in zip(self.domain, self.shape)])
        dx, dy, dz = self.dX
        self.dV = dx * dy * dz
        self.D = np.array([-dx, dx, -dy, dy, -dz, dz])
        self.dS = np.array([-dy * dz, dy * dz, -dz * dx, dz * dx, -dx * dy, dx * dy])
        self.cell_num = int(np.prod(self.shape))
        # cell centres: midpoints of numpy.linspace nodes (cfd_am.py:672-680)
        xs, ys, zs = ((n[1:] + n[:-1]) / 2 for n in
                      (np.linspace(0.0, L, k + 1) for L, k in zip(self.domain, self.shape)))
        X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
        self.Xc = np.stack((X, Y, Z), axis=3).reshape(-1, 3)


def neighbours(U):
    """The six mirrored neighbours of every cell of a 3-D array, in the
    reference's order (x-, x+, y-, y+, z-, z+)."""
    P = np.pad(U, 1, mode="edge")
    c = (slice(1, -1),) * 3
    out = []
    for ax in range(3):
        for d in (-1, 1):
            idx = list(c)
            idx[ax] = slice(1 + d, P.shape[ax] - 1 + d)
            out.append(P[tuple(idx)])
    return out


def mirrored(shape):
    """(6, Nx, Ny, Nz) booleans: neighbour f of the cell is the cell itself."""
    Nx, Ny, Nz = shape
    i, j, k = np.meshgrid(np.arange(Nx), np.arange(Ny), np.arange(Nz), indexing="ij")
    return np.stack([i == 0, i == Nx - 1, j == 0, j == Ny - 1, k == 0, k == Nz - 1])


def face_masks(shape):
    """The same as ``mirrored``: a cell lies on face f exactly when its
    neighbour across f is mirrored (``get_surface``, ``cfd_am.py:708-745``)."""
    return mirrored(shape)


# ---------------------------------------------------------------------------
# linear algebra
# ---------------------------------------------------------------------------

def apply_op(values, U):
    """``compute_linearized_residual`` (``cfd_am.py:483-484``): values (7,
    Nx, Ny, Nz) applied to the cell and its mirrored neighbours."""
    out = values[0] * U
    for f, Un in enumerate(neighbours(U)):
        out = out + values[1 + f] * Un
    return out


def jacobi_diag(values):
    """``precond_values`` (``cfd_am.py:480-481``): entries pointing at the
    cell itself, summed."""
    m = mirrored(values.shape[1:])
    d = values[0].copy()
    for f in range(6):
        d = d + np.where(m[f], values[1 + f], 0.0)
    return d


def bicgstab(A, b, M=None, tol=1e-5, atol=0.0, maxiter=None):
    """``jax.scipy.sparse.linalg.bicgstab`` semantics on flat float64
    vectors; returns (x, k): k iterations, or -10 (rho = 0) / -11 (alpha or
    omega = 0) after a breakdown.  Scalars are float64 with IEEE division
    (0/0 = NaN as in JAX: at an early exit omega is NaN and unused)."""
    if maxiter is None:
        maxiter = 10 * b.size
    if M is None:
        M = lambda v: v  # noqa: E731
    dot = lambda u, v: np.float64(np.dot(u, v))  # noqa: E731
    atol2 = max(np.float64(tol) ** 2 * dot(b, b), np.float64(atol) ** 2)
    x = np.zeros_like(b)
    r = b - A(x)
    rhat = r.copy()
    p = r.copy()
    q = r.copy()
    rho = alpha = omega = np.float64(1.0)
    k = 0
    with np.errstate(divide="ignore", invalid="ignore"):
        while dot(r, r) > atol2 and k < maxiter and k >= 0:
            rho_ = dot(rhat, r)
            beta = rho_ / rho * alpha / omega
            p = r + beta * (p - omega * q)
            phat = M(p)
            q = A(phat)
            alpha_ = rho_ / dot(rhat, q)
            s = r - alpha_ * q
            exit_early = dot(s, s) < atol2
            shat = M(s)
            t = A(shat)
            omega_ = dot(t, s) / dot(t, t)
            if exit_early:
                x = x + alpha_ * phat
                r = s
            else:
                x = x + (alpha_ * phat + omega_ * shat)
                r = s - omega_ * t
            k = -11 if (omega_ == 0 or alpha_ == 0) else k + 1
            if rho_ == 0:
                k = -10
            rho, alpha, omega = rho_, alpha_, omega_
    return x, k


# ---------------------------------------------------------------------------
# energy equation
# ---------------------------------------------------------------------------

def cp_eff(args, T0):
    """``cp_fn`` (``cfd_am.py:497-498``)."""
    bump = args["latent_heat"] / (args["Tl"] - args["Ts"])
    return args["cp"](T0) + bump * ((T0 > args["Ts"]) & (T0 < args["Tl"]))


def energy_residual(mesh, args, U, T0, conv, Q, q_top):
    """Residual of the energy equation at U (3-D arrays); q_top (Nx, Ny) is
    the top face's Neumann value (``cfd_am.py:334-358``)."""
    k = args["k"]
    kU = k(U)
    lap = np.zeros_like(U)
    for f, Un in enumerate(neighbours(U)):
        kn = k(Un)
        mu = 2.0 * kU * kn / (kn + kU)
        lap = lap + (Un - U) / mesh.D[f] * mu * mesh.dS[f]
    cp0 = cp_eff(args, T0)
    src = -args["rho"] * (U - T0) * cp0 / args["dt"] - args["rho"] * cp0 * conv + Q
    res = -lap - src * mesh.dV
    res[:, :, -1] -= q_top * abs(mesh.dS[5])
    return res


def energy_jacobian(mesh, args, U, T0):
    """(7, Nx, Ny, Nz) Jacobian rows of the energy residual (the values
    ``jax.jacrev`` gives, ``cfd_am.py:474-481``)."""
    k = args["k"]
    kU, dkU = k(U), k.deriv(U)
    vals = np.zeros((7,) + U.shape)
    for f, Un in enumerate(neighbours(U)):
        kn, dkn = k(Un), k.deriv(Un)
        den = kn + kU
        mu = 2.0 * kU * kn / den
        dmu_p = 2.0 * dkU * kn * kn / (den * den)
        dmu_n = 2.0 * dkn * kU * kU / (den * den)
        g = mesh.dS[f] / mesh.D[f]
        vals[0] += g * mu - (Un - U) * g * dmu_p
        vals[1 + f] = -(g * mu + (Un - U) * g * dmu_n)
    vals[0] += args["rho"] * cp_eff(args, T0) / args["dt"] * mesh.dV
    return vals


def solve_energy(mesh, args, T0, conv, Q, q_top, tol=1e-5, max_it=50):
    """``energy_eqn.update`` + ``solver_nonlinear`` (``cfd_am.py:516-525,
    780-812``); returns (T, Newton iterations, BiCGSTAB iterations)."""
    U = T0.copy()
    b = -energy_residual(mesh, args, U, T0, conv, Q, q_top)
    res_init = np.linalg.norm(b)
    it, lin = 0, []
    while np.linalg.norm(b) / res_init > tol and it < max_it:
        vals = energy_jacobian(mesh, args, U, T0)
        diag = jacobi_diag(vals)
        shape = U.shape
        A = lambda v: apply_op(vals, v.reshape(shape)).ravel()  # noqa: E731
        inv = 1.0 / diag.ravel()  # jacobiPreconditioner: 1./precond_values * U
        M = lambda v: inv * v  # noqa: E731
        inc, kk = bicgstab(A, b.ravel(), M)
        lin.append(kk)
        U = U + inc.reshape(shape)
        b = -energy_residual(mesh, args, U, T0, conv, Q, q_top)
        it += 1
    return U, it, lin


# ---------------------------------------------------------------------------
# velocity equation
# ---------------------------------------------------------------------------

def fluid_frac(args, T):
    """``AM_3d.fluid_frac`` (``cfd_am.py:360-363``)."""
    return (np.clip(T, args["Ts"], args["Tl"]) - args["Ts"]) / (args["Tl"] - args["Ts"])


def marangoni(mesh_l, args, T_top):
    """Top-face shear (``cfd_am.py:291-299``): (Nx, Ny, 3) for the local
    box's top temperatures T_top (Nx, Ny)."""
    fl = fluid_frac(args, T_top)
    P = np.pad(T_top, 1, mode="edge")
    c = args["Marangoni"] / args["visco"]
    gx = (P[2:, 1:-1] - P[:-2, 1:-1]) / 2.0 / mesh_l.dX[0] * c * fl
    gy = (P[1:-1, 2:] - P[1:-1, :-2]) / 2.0 / mesh_l.dX[1] * c * fl
    return np.stack((gx, gy, np.zeros_like(gx)), axis=2)


def momentum_system(mesh_l, args, u0, conv, grad_p, fl, comp, mg):
    """Right-hand side b = -residual(0) and Jacobian rows of momentum
    component ``comp`` (``cfd_am.py:528-575``, ``solver_linear``
    ``:748-778``): Dirichlet zero on every face except the top for u and v,
    which is Neumann with value visco * mg[..., comp]."""
    visco, rho, dt = args["visco"], args["rho"], args["dt"]
    shape = u0.shape
    fm = face_masks(shape)
    # residual at U = 0: -source(0) dV, then the boundary fluxes
    src0 = -rho * (0.0 - u0) / dt - rho * conv - grad_p
    res = -src0 * mesh_l.dV
    dirichlet = [0, 1, 2, 3, 4] + ([] if comp < 2 else [5])
    if comp < 2:
        res[:, :, -1] -= visco * mg[:, :, comp] * abs(mesh_l.dS[5])
    vals = np.zeros((7,) + shape)
    darcy = 1e7 * rho * (1.0 - fl) ** 2 / (fl ** 3 + 1e-5)
    for f in range(6):
        g = mesh_l.dS[f] / mesh_l.D[f]
        vals[0] += g * visco
        vals[1 + f] = -g * visco
    vals[0] += (rho / dt + darcy) * mesh_l.dV
    for f in dirichlet:
        vals[0] += np.where(fm[f], visco * 2.0 / mesh_l.D[f] * mesh_l.dS[f], 0.0)
    return -res, vals


def pressure_values(mesh_l):
    """Jacobian rows of the pressure Poisson (``cfd_am.py:538-547``)."""
    vals = np.zeros((7,) + mesh_l.shape)
    for f in range(6):
        g = mesh_l.dS[f] / mesh_l.D[f]
        vals[0] += g
        vals[1 + f] = -g
    return vals


def face_velocities(vel):
    """``get_face_vels`` with the velocity ghost cells (``cfd_am.py:94-112``):
    every boundary face velocity is zero (wall ghosts mirror with a sign
    change; the top's normal component too)."""
    u, v, w = vel[..., 0], vel[..., 1], vel[..., 2]
    Nx, Ny, Nz = u.shape
    uf = np.zeros((Nx + 1, Ny, Nz))
    uf[1:-1] = (u[1:] + u[:-1]) / 2.0
    uf[0] = (-u[0] + u[0]) / 2.0
    uf[-1] = (u[-1] - u[-1]) / 2.0
    vf = np.zeros((Nx, Ny + 1, Nz))
    vf[:, 1:-1] = (v[:, 1:] + v[:, :-1]) / 2.0
    vf[:, 0] = (-v[:, 0] + v[:, 0]) / 2.0
    vf[:, -1] = (v[:, -1] - v[:, -1]) / 2.0
    wf = np.zeros((Nx, Ny, Nz + 1))
    wf[:, :, 1:-1] = (w[:, :, 1:] + w[:, :, :-1]) / 2.0
    wf[:, :, 0] = (-w[:, :, 0] + w[:, :, 0]) / 2.0
    wf[:, :, -1] = (w[:, :, -1] - w[:, :, -1]) / 2.0
    return uf, vf, wf


def upwind_div(f, faces, dX, theta=0.125):
    """``div`` (``cfd_am.py:53-79``) of a scalar field f (Nx, Ny, Nz) with
    zero-gradient ghosts: face values blend the central average (theta) with
    the upwind linear extrapolation (1 - theta)."""
    out = np.zeros_like(f)
    for ax in range(3):
        n = f.shape[ax]
        pad = [(0, 0)] * 3
        pad[ax] = (2, 2)
        fx = np.pad(f, pad, mode="edge")

        def sl(a, b):
            idx = [slice(None)] * 3
            idx[ax] = slice(a, b)
            return fx[tuple(idx)]

        fl1, fr1 = sl(1, n + 2), sl(2, n + 3)   # cells left / right of each face
        fl2, fr2 = sl(0, n + 1), sl(3, n + 4)
        uf = faces[ax]
        face = (theta * (fl1 / 2 + fr1 / 2)
                + (1 - theta) * (3 * fl1 / 2 - fl2 / 2) * (uf >= 0)
                + (1 - theta) * (3 * fr1 / 2 - fr2 / 2) * (uf < 0))
        flux = face * uf
        idx_hi = [slice(None)] * 3
        idx_lo = [slice(None)] * 3
        idx_hi[ax] = slice(1, None)
        idx_lo[ax] = slice(None, -1)
        out = out + (flux[tuple(idx_hi)] - flux[tuple(idx_lo)]) / dX[ax]
    return out


def gradient(p, dX):
    """``gradient`` (``cfd_am.py:82-91``): (Nx, Ny, Nz, 3) central
    differences, one-sided halves at the boundary (zero-gradient ghosts)."""
    out = []
    for ax in range(3):
        P = np.pad(p, [(1, 1) if a == ax else (0, 0) for a in range(3)], mode="edge")
        idx_p = [slice(None)] * 3
        idx_m = [slice(None)] * 3
        idx_p[ax] = slice(2, None)
        idx_m[ax] = slice(None, -2)
        out.append((P[tuple(idx_p)] - P[tuple(idx_m)]) / dX[ax] / 2.0)
    return np.stack(out, axis=3)


def solve_velocity(mesh_l, args, vel0, conv0, grad_p0, fl, T):
    """``velocity_eqn.update`` (``cfd_am.py:557-590``) on the local box;
    returns (vel, grad_p0 + grad p, marangoni shear, iterations)."""
    mg = marangoni(mesh_l, args, T[:, :, -1])
    shape = fl.shape
    vel = np.zeros(shape + (3,))
    iters = []
    for comp in range(3):
        b, vals = momentum_system(mesh_l, args, vel0[..., comp], conv0[..., comp],
                                  grad_p0[..., comp], fl, comp, mg)
        diag = jacobi_diag(vals)
        A = lambda v, vals=vals: apply_op(vals, v.reshape(shape)).ravel()  # noqa: E731
        M = lambda v, inv=1.0 / diag.ravel(): inv * v  # noqa: E731
        x, kk = bicgstab(A, b.ravel(), M, tol=1e-10, maxiter=10000)
        iters.append(kk)
        vel[..., comp] = x.reshape(shape)
    uf, vf, wf = face_velocities(vel)
    dX = mesh_l.dX
    div_vel = ((uf[1:] - uf[:-1]) / dX[0] + (vf[:, 1:] - vf[:, :-1]) / dX[1]
               + (wf[:, :, 1:] - wf[:, :, :-1]) / dX[2]) / args["dt"] * args["rho"]
    pv = pressure_values(mesh_l)
    A = lambda v: apply_op(pv, v.reshape(shape)).ravel()  # noqa: E731
    b = -(div_vel * mesh_l.dV).ravel()
    p, kk = bicgstab(A, b, None, tol=1e-10, maxiter=10000)
    iters.append(kk)
    gp = gradient(p.reshape(shape), dX)
    vel = vel - args["dt"] * gp / args["rho"]
    return vel, grad_p0 + gp, mg, iters


# ---------------------------------------------------------------------------
# AM_3d
# ---------------------------------------------------------------------------

class AM3d:
    """``AM_3d`` (``cfd_am.py:142-385``) state and ``time_integration``."""

    def __init__(self, args, mesh, mesh_local):
        self.args = dict(args)
        self.args.setdefault("h", 0.0)
        self.args.setdefault("stefan_boltzmann", 5.67e-8)
        self.args.setdefault("emissivity", 0.0)
        self.msh, self.msh_local = mesh, mesh_local
        self.t = 0.0
        shape = mesh.shape
        self.T = np.zeros(shape) + args["T_ref"]
        self.solidID = np.zeros(shape)
        self.conv_T = np.zeros(shape)
        self.vel = np.zeros(shape + (3,))
        self.conv = np.zeros(shape + (3,))
        self.grad_p0 = np.zeros(shape + (3,))
        self.last_iters = None

    def toolpath(self, t):
        a = self.args
        return (a["X0"][0] + t * a["speed"], a["X0"][1], a["X0"][2],
                a["P"] * (t < a["t_OFF"]))

    def body_source(self, t):
        """``get_body_heat_source`` (``cfd_am.py:223-235``)."""
        a = self.args
        xl, yl, zl, P = self.toolpath(t)
        r = a["rb"]
        d = a["phi"] * P / a["speed"] / r ** 2
        Xc = self.msh.Xc
        q = 2 * P * a["eta"] / d / np.pi / r ** 2 * np.exp(
            -2 * ((Xc[:, 0] - xl) ** 2 + (Xc[:, 1] - yl) ** 2) / r ** 2)
        q = q * ((zl - Xc[:, 2]) <= d)
        return q.reshape(self.msh.shape)

    def top_flux(self, t, T_top):
        """Top-face Neumann value (``cfd_am.py:334-358``)."""
        a = self.args
        q = -a["h"] * (T_top - a["T_ref"]) - a["stefan_boltzmann"] * a["emissivity"] * (
            T_top ** 4 - a["T_ref"] ** 4)
        if a["heat_source"] == 0:
            xl, yl, _, P = self.toolpath(t)
            r = a["rb"]
            Xc = self.msh.Xc.reshape(self.msh.shape + (3,))[:, :, -1]
            q = q + 2 * P * a["eta"] / np.pi / r ** 2 * np.exp(
                -2 * ((Xc[..., 0] - xl) ** 2 + (Xc[..., 1] - yl) ** 2) / r ** 2)
        return q

    def box(self, t):
        """``get_moving_box_boundary`` (``cfd_am.py:237-252``): Python's
        round (half to even) of the beam position in cells."""
        xl, yl, zl, _ = self.toolpath(t)
        N, NL, dX = self.msh.shape, self.msh_local.shape, self.msh.dX
        x0 = round(float(xl / dX[0])) - round(NL[0] / 2)
        x0 = int(np.clip(x0, 0, N[0] - NL[0]))
        y0 = round(float(yl / dX[1])) - round(NL[1] / 2)
        y0 = int(np.clip(y0, 0, N[1] - NL[1]))
        z0 = N[2] - NL[2]
        return x0, x0 + NL[0], y0, y0 + NL[1], z0, N[2]

    def time_integration(self):
        a, t = self.args, self.t
        Q = self.body_source(t) if a["heat_source"] == 1 else np.zeros(self.msh.shape)
        q_top = self.top_flux(t, self.T[:, :, -1])
        T, n_it, lin = solve_energy(self.msh, a, self.T, self.conv_T, Q, q_top)
        self.T = T
        fl0 = fluid_frac(a, T)
        self.solidID = np.maximum(self.solidID, fl0)
        x0, x1, y0, y1, z0, z1 = self.box(t)
        b = (slice(x0, x1), slice(y0, y1), slice(z0, z1))
        vel, gp, mg, v_it = solve_velocity(self.msh_local, a, self.vel[b], self.conv[b],
                                           self.grad_p0[b], fl0[b], T[b])
        # convective terms on the box with the global spacing (cfd_am.py:254-259)
        faces = face_velocities(vel)
        conv_T = upwind_div(T[b], faces, self.msh.dX)
        conv = np.stack([upwind_div(vel[..., c], faces, self.msh.dX) for c in range(3)], axis=3)
        self.vel[b] = vel
        self.grad_p0[b] = gp
        self.conv[b] = conv
        self.conv_T[b] = conv_T
        self.t += a["dt"]
        self.last_iters = dict(newton=n_it, energy_lin=lin, velocity=v_it, box=(x0, y0, z0))
