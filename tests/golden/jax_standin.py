"""A minimal stand-in for the ``jax`` package, used ONLY to run the reference's
own phase-field and heat source files in this container to produce golden
vectors (``make_golden.py``).  JAX itself is not installed and there is no
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
"""
import sys
import types

import numpy as onp
import torch


class JArray(onp.ndarray):
    """``ndarray`` with JAX's out-of-place ``.at[...]`` updates."""

    def __array_finalize__(self, obj):
        pass

    @property
    def at(self):
        return _At(self)


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


def _torch_call(name, *args, **kwargs):
    if "axis" in kwargs:
        kwargs["dim"] = kwargs.pop("axis")
    if name == "sum":
        return torch.sum(*args, **kwargs)
    if name == "outer":
        return torch.outer(*args)
    if name == "stack":
        return torch.stack(*args, **kwargs)
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
    jax.config = _Config()
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jax.numpy
    return jax


def asarray(x, dtype=None):
    """A JArray copy of ``x`` (the stand-in's ``jnp.asarray``)."""
    return onp.array(x, dtype=dtype).view(JArray)
