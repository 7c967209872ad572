"""A minimal stand-in for the ``jax`` package, used ONLY to run the reference's
own phase-field, heat and CFD source files in this container to produce
golden vectors (``make_golden.py``, ``make_golden_cfd.py``).  JAX itself is not installed and there is no
network, so the reference cannot be imported as shipped.

Test infrastructure, not product code: nothing in ``jax_am_gb300`` imports it.

What it provides, and the JAX semantics it restates:

* ``jax.numpy``: every attribute forwards to NumPy.  Arrays that come back are
  a thin ``ndarray`` subclass with JAX's functional ``.at[idx].set/add``
  update (a copy, as in JAX).
* ``jax.jit`` (with or without ``static_argnums``): identity.  Tracing and
  compilation do not change values beyond operation order.
* ``jax.vmap(f, in_axes=(0, 0))``: ``f`` mapped over the leading axis and the
  results stacked.
* ``jax.grad(f, argnums=0)``: reverse-mode derivative taken with PyTorch
  autograd in float64.  While the gradient is being traced the ``jax.numpy``
  functions used by the reference (``sum``, ``outer``, ``stack``) dispatch to
  their ``torch`` equivalents when handed a tensor.
* ``jax.config.update``: records the x64 switch; arrays keep the dtype they
  are created with (the fixtures pick float64 or float32 explicitly).
* ``jax.jacrev(f)``: the Jacobian of a scalar per-cell kernel with respect
  to its first (vector) argument, PyTorch autograd in float64; ``jnp.clip``
  on a traced tensor has JAX's derivative (half of the gradient on each side
  of a tie, as JAX's max and min give).
* ``jax.lax.while_loop``: a Python loop.
* ``jax.scipy.sparse.linalg.bicgstab``: the preconditioned BiCGSTAB of van
  der Vorst as JAX implements it (x0 = 0, maxiter = 10 size, stop when
  |r|^2 <= max(tol^2 |b|^2, atol^2), early exit on |s|^2, breakdown codes
  -10 / -11), float64.
* ``jax.experimental.sparse.BCOO``: a placeholder (imported, never used on
  the solver path of ``cfd_am.py``).
"""
import sys
import types

import numpy as onp
import torch


class JArray(onp.ndarray):
    """``ndarray`` with JAX's out-of-place ``.at[...]`` updates.  Compared with
    ``None`` it is unequal (a JAX array defers that comparison to Python's
    identity test), and mixed with a ``torch.Tensor`` inside a traced
    derivative it takes part as a tensor."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)

    def __eq__(self, other):
        if other is None:
            return False
        return super().__eq__(other)

    def __ne__(self, other):
        if other is None:
            return True
        return super().__ne__(other)

    __hash__ = None

    @classmethod
    def __torch_function__(cls, func, types, args=(), kwargs=None):
        def conv(a):
            if isinstance(a, JArray):
                return torch.from_numpy(onp.ascontiguousarray(a.view(onp.ndarray)))
            if isinstance(a, (list, tuple)):
                return type(a)(conv(b) for b in a)
            return a
        return func(*conv(tuple(args)), **{k: conv(v) for k, v in (kwargs or {}).items()})


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtIdx(self._arr, idx)


class _AtIdx:
    def __init__(self, arr, idx):
        self._arr, self._idx = arr, idx

    def set(self, value):
        out = onp.array(self._arr, copy=True)
        out[self._idx] = onp.asarray(value)
        return out.view(JArray)

    def add(self, value):
        out = onp.array(self._arr, copy=True)
        onp.add.at(out, self._idx, onp.asarray(value))
        return out.view(JArray)


def _wrap(x):
    if isinstance(x, onp.ndarray) and not isinstance(x, JArray):
        return x.view(JArray)
    return x


def _has_tensor(args, kwargs):
    for a in list(args) + list(kwargs.values()):
        if isinstance(a, torch.Tensor):
            return True
        if isinstance(a, (list, tuple)) and any(isinstance(b, torch.Tensor) for b in a):
            return True
    return False


class _JaxClip(torch.autograd.Function):
    """``jnp.clip(x, lo, hi)`` = min(max(x, lo), hi) with JAX's derivative:
    max and min pass half of the gradient to each side of a tie."""

    @staticmethod
    def forward(ctx, x, lo, hi):
        ctx.save_for_backward(x)
        ctx.lo, ctx.hi = float(lo), float(hi)
        return torch.clamp(x, ctx.lo, ctx.hi)

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        inside = (x > ctx.lo) & (x < ctx.hi)
        tie = (x == ctx.lo) | (x == ctx.hi)
        w = torch.where(inside, torch.ones_like(x), torch.where(tie, torch.full_like(x, 0.5),
                                                                  torch.zeros_like(x)))
        return g * w, None, None


def _torch_call(name, *args, **kwargs):
    if "axis" in kwargs:
        kwargs["dim"] = kwargs.pop("axis")
    if name == "sum":
        return torch.sum(*args, **kwargs)
    if name == "outer":
        return torch.outer(*args)
    if name == "stack":
        return torch.stack(*args, **kwargs)
    if name == "clip":
        x, lo, hi = args
        return _JaxClip.apply(x, lo, hi)
    if name == "exp":
        return torch.exp(*args)
    raise NotImplementedError(f"jax.numpy.{name} on a traced tensor")


def _make_numpy_module():
    mod = types.ModuleType("jax.numpy")

    def __getattr__(name):
        target = getattr(onp, name)
        if not callable(target) or isinstance(target, type):
            return target

        def fn(*args, **kwargs):
            if _has_tensor(args, kwargs):
                return _torch_call(name, *args, **kwargs)
            return _wrap(target(*args, **kwargs))

        fn.__name__ = name
        return fn

    mod.__getattr__ = __getattr__
    mod.pi = onp.pi
    linalg = types.ModuleType("jax.numpy.linalg")
    linalg.norm = lambda *a, **k: _wrap(onp.linalg.norm(*a, **k))
    mod.linalg = linalg
    return mod


def _jit(fun=None, **_kw):
    if fun is None:
        return lambda f: f
    return fun


def _vmap(fun, in_axes=0):
    def mapped(*args):
        n = args[0].shape[0]
        outs = [fun(*[a[i] for a in args]) for i in range(n)]
        if isinstance(outs[0], torch.Tensor):
            return torch.stack(outs)
        return _wrap(onp.stack(outs))
    return mapped


def _grad(fun, argnums=0):
    def g(*args):
        targs = list(args)
        x = torch.tensor(onp.asarray(args[argnums], dtype=onp.float64), requires_grad=True)
        targs[argnums] = x
        for i, a in enumerate(targs):
            if i != argnums and isinstance(a, onp.ndarray):
                targs[i] = torch.from_numpy(onp.asarray(a, dtype=onp.float64))
        y = fun(*targs)
        y.backward()
        return _wrap(x.grad.numpy().astype(onp.asarray(args[argnums]).dtype))
    return g


def _jacrev(fun, argnums=0):
    """Reverse-mode Jacobian of a scalar function of one vector argument
    (the per-cell residual kernels of ``cfd_am.py``), float64 autograd."""
    def j(*args):
        targs = list(args)
        x = torch.tensor(onp.asarray(args[argnums], dtype=onp.float64), requires_grad=True)
        targs[argnums] = x
        y = fun(*targs)
        (g,) = torch.autograd.grad(y, x, allow_unused=True)
        if g is None:
            g = torch.zeros_like(x)
        return _wrap(g.detach().numpy().copy())
    return j


def _while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def _vdot(a, b):
    return onp.float64(onp.dot(onp.ravel(a), onp.ravel(b)))


def _bicgstab(A, b, x0=None, *, tol=1e-5, atol=0.0, maxiter=None, M=None):
    """``jax.scipy.sparse.linalg.bicgstab``: preconditioned BiCGSTAB (van der
    Vorst) with JAX's stopping rule |r|^2 <= max(tol^2 |b|^2, atol^2), its
    early exit on |s|^2 and its breakdown codes; returns (x, None)."""
    b = onp.asarray(b, dtype=onp.float64)
    if x0 is None:
        x0 = onp.zeros_like(b)
    if maxiter is None:
        maxiter = 10 * b.size
    if M is None:
        M = lambda v: v  # noqa: E731
    matvec = lambda v: onp.asarray(A(_wrap(v)), dtype=onp.float64)  # noqa: E731
    prec = lambda v: onp.asarray(M(_wrap(v)), dtype=onp.float64)  # noqa: E731
    atol2 = max(onp.float64(tol) ** 2 * _vdot(b, b), onp.float64(atol) ** 2)

    def cond_fun(value):
        x, r, *_, k = value
        return (_vdot(r, r) > atol2) and (k < maxiter) and (k >= 0)

    def body_fun(value):
        x, r, rhat, alpha, omega, rho, p, q, k = value
        rho_ = _vdot(rhat, r)
        beta = rho_ / rho * alpha / omega
        p_ = r + beta * (p - omega * q)
        phat = prec(p_)
        q_ = matvec(phat)
        alpha_ = rho_ / _vdot(rhat, q_)
        s = r - alpha_ * q_
        exit_early = _vdot(s, s) < atol2
        shat = prec(s)
        t = matvec(shat)
        omega_ = _vdot(t, s) / _vdot(t, t)
        if exit_early:
            x_ = x + alpha_ * phat
            r_ = s
        else:
            x_ = x + (alpha_ * phat + omega_ * shat)
            r_ = s - omega_ * t
        k_ = -11 if (omega_ == 0 or alpha_ == 0) else k + 1
        k_ = -10 if rho_ == 0 else k_
        return x_, r_, rhat, alpha_, omega_, rho_, p_, q_, k_

    r0 = b - matvec(onp.asarray(x0, dtype=onp.float64))
    one = onp.float64(1.0)
    init = (onp.asarray(x0, dtype=onp.float64), r0, r0, one, one, one, r0, r0, 0)
    with onp.errstate(divide="ignore", invalid="ignore"):  # 0/0 = NaN as in JAX
        x_final, *_ = _while_loop(cond_fun, body_fun, init)
    return _wrap(x_final), None


class _Config:
    def __init__(self):
        self.values = {}

    def update(self, k, v):
        self.values[k] = v


def install():
    """Register the stand-in as ``jax`` / ``jax.numpy`` in ``sys.modules``."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_is_standin", False):
        return sys.modules["jax"]
    jax = types.ModuleType("jax")
    jax._is_standin = True
    jax.numpy = _make_numpy_module()
    jax.jit = _jit
    jax.vmap = _vmap
    jax.grad = _grad
    jax.jacrev = _jacrev
    jax.config = _Config()
    lax = types.ModuleType("jax.lax")
    lax.while_loop = _while_loop
    jax.lax = lax
    scipy_mod = types.ModuleType("jax.scipy")
    sparse_mod = types.ModuleType("jax.scipy.sparse")
    linalg_mod = types.ModuleType("jax.scipy.sparse.linalg")
    linalg_mod.bicgstab = _bicgstab
    sparse_mod.linalg = linalg_mod
    scipy_mod.sparse = sparse_mod
    jax.scipy = scipy_mod
    experimental = types.ModuleType("jax.experimental")
    exp_sparse = types.ModuleType("jax.experimental.sparse")
    exp_sparse.BCOO = None  # imported by cfd_am.py, never used on its solver path
    experimental.sparse = exp_sparse
    jax.experimental = experimental
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jax.numpy
    sys.modules["jax.lax"] = lax
    sys.modules["jax.scipy"] = scipy_mod
    sys.modules["jax.scipy.sparse"] = sparse_mod
    sys.modules["jax.scipy.sparse.linalg"] = linalg_mod
    sys.modules["jax.experimental"] = experimental
    sys.modules["jax.experimental.sparse"] = exp_sparse
    return jax


def asarray(x, dtype=None):
    """A JArray copy of ``x`` (the stand-in's ``jnp.asarray``)."""
    return onp.array(x, dtype=dtype).view(JArray)
