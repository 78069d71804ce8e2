"""Test-only numpy stand-in for ``jax``/``jax.numpy``/``jax.lax``/``flax.core``.

The reference's JAX stencils (``src/ice3/jax/**`` of maurinl26/dwarf-p-ice3)
only use a small, purely elementwise subset of JAX.  Installing these fake
modules lets the golden-vector generator execute that reference code
*unmodified* in float64 on the CPU, without jax being installed:

* ``jax.numpy``: numpy re-exported, with results viewed as an ndarray
  subclass that provides the functional ``x.at[idx].set(v)`` update;
* ``jax.lax.while_loop``: a plain Python loop;
* ``jax.jit``: identity (static arguments ignored);
* ``flax.core.FrozenDict``: a hashable ``dict``.

This file is test infrastructure: nothing in the product imports it.
"""
from __future__ import annotations

import sys
import types

import numpy as np


class _AtIndex:
    def __init__(self, arr, idx):
        self._arr = arr
        self._idx = idx

    def set(self, value):
        out = np.array(self._arr, copy=True).view(ShimArray)
        out[self._idx] = value
        return out

    def add(self, value):
        out = np.array(self._arr, copy=True).view(ShimArray)
        out[self._idx] += value
        return out


class _At:
    def __init__(self, arr):
        self._arr = arr

    def __getitem__(self, idx):
        return _AtIndex(self._arr, idx)


class ShimArray(np.ndarray):
    """ndarray with JAX's ``.at[...]`` functional-update syntax."""

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self


def _wrap_result(x):
    if isinstance(x, np.ndarray) and not isinstance(x, ShimArray):
        return x.view(ShimArray)
    if isinstance(x, tuple):
        return tuple(_wrap_result(v) for v in x)
    if isinstance(x, list):
        return [_wrap_result(v) for v in x]
    return x


def _wrap_callable(fn):
    def wrapped(*args, **kwargs):
        return _wrap_result(fn(*args, **kwargs))

    wrapped.__name__ = getattr(fn, "__name__", "wrapped")
    wrapped.__wrapped__ = fn
    return wrapped


class _JnpModule(types.ModuleType):
    """``jax.numpy``: every numpy attribute, callables wrapped to return ShimArray."""

    _passthrough = {"ndarray", "float32", "float64", "int32", "int64", "bool_",
                    "newaxis", "pi", "inf", "nan", "e", "dtype", "uint32"}

    def __getattr__(self, name):
        obj = getattr(np, name)
        if name in self._passthrough or isinstance(obj, type):
            return obj
        if callable(obj):
            return _wrap_callable(obj)
        return obj

    def array(self, x, dtype=None, **kw):
        return np.array(x, dtype=dtype).view(ShimArray)

    def asarray(self, x, dtype=None, **kw):
        return np.asarray(x, dtype=dtype).view(ShimArray)


def _while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def _fori_loop(lower, upper, body_fun, init_val):
    val = init_val
    for i in range(lower, upper):
        val = body_fun(i, val)
    return val


def _jit(fn=None, **_kw):
    if fn is None:
        return lambda f: f
    return fn


class FrozenDict(dict):
    def __hash__(self):
        return hash(tuple(sorted(self.keys())))


def install() -> None:
    """Register the fake modules in ``sys.modules`` (idempotent)."""
    if "jax" in sys.modules and getattr(sys.modules["jax"], "_ice3_refshim", False):
        return
    jax = types.ModuleType("jax")
    jax._ice3_refshim = True
    jnp = _JnpModule("jax.numpy")
    lax = types.ModuleType("jax.lax")
    lax.while_loop = _while_loop
    lax.fori_loop = _fori_loop
    lax.select = _wrap_callable(np.where)
    lax.cond = lambda p, t, f, *a: t(*a) if p else f(*a)
    jax.numpy = jnp
    jax.lax = lax
    jax.jit = _jit
    jax.Array = np.ndarray
    jax.vmap = lambda f, *a, **k: f
    config = types.SimpleNamespace(update=lambda *a, **k: None)
    jax.config = config
    flax = types.ModuleType("flax")
    flax_core = types.ModuleType("flax.core")
    flax_core.FrozenDict = FrozenDict
    flax.core = flax_core
    sys.modules["jax"] = jax
    sys.modules["jax.numpy"] = jnp
    sys.modules["jax.lax"] = lax
    sys.modules["flax"] = flax
    sys.modules["flax.core"] = flax_core
