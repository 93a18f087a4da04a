"""A NumPy stand-in for the few `jax` names the reference's hot-path modules use.

Test infrastructure only: tests/golden/make_ref_golden.py puts this directory
first on sys.path so that the reference package (a JAX program; JAX is not
installable here) can be imported and executed unmodified on NumPy arrays.
Everything runs eagerly in float64 / complex128, which is what the reference
computes with x64 enabled (config.py:24-25).

Mapping:
  jax.numpy        -> numpy (module attribute lookups fall through to numpy)
  jax.vmap         -> a Python loop over axis 0 of every leaf, results stacked
  jax.lax.scan     -> a Python loop
  jax.random.*     -> draws taken from a queue the caller fills (`feed`), so
                      the reference consumes exactly the fields and comb
                      uniforms that the oracle and the engine are given
  jax.scipy.linalg -> scipy.linalg
  jax.tree_util    -> tuple/list-aware map; the pytree decorator is a no-op
"""
from __future__ import annotations

import numpy as _np

from . import lax, random, tree_util  # noqa: F401
from . import numpy  # noqa: F401
from . import scipy  # noqa: F401

Array = _np.ndarray
__version__ = "0.0-numpy-standin"


def _leaves(x):
    if isinstance(x, (tuple, list)):
        out = []
        for e in x:
            out.extend(_leaves(e))
        return out
    return [x]


def _take(x, i, axis):
    if axis is None:
        return x
    if isinstance(x, tuple):
        return tuple(_take(e, i, axis) for e in x)
    if isinstance(x, list):
        return [_take(e, i, axis) for e in x]
    return _np.asarray(x)[i]


def _stack(results):
    first = results[0]
    if isinstance(first, tuple):
        return tuple(_stack([r[k] for r in results]) for k in range(len(first)))
    if isinstance(first, list):
        return [_stack([r[k] for r in results]) for k in range(len(first))]
    return _np.stack([_np.asarray(r) for r in results], axis=0)


def vmap(fn, in_axes=0):
    """Map fn over axis 0 of its arguments (in_axes 0 / None per argument)."""

    def mapped(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)
        n = None
        for a, ax in zip(args, axes):
            if ax is not None:
                n = len(_leaves(a)[0])
                break
        if n is None:
            raise ValueError("vmap stand-in: no mapped argument")
        return _stack([fn(*(_take(a, i, ax) for a, ax in zip(args, axes))) for i in range(n)])

    return mapped


def jit(fn=None, **_kw):
    if fn is None:
        return lambda f: f
    return fn


class _Config:
    def update(self, *_a, **_k):
        pass


config = _Config()
