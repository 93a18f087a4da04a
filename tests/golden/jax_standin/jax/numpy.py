"""jax.numpy stand-in: NumPy itself (see the package docstring).

JAX functions always return arrays, never Python or NumPy scalars; the
wrapped names below return 0-d arrays where NumPy would return a scalar, so
that expressions such as (1.0j * sqrt(dt)).astype(...) behave as in JAX.
"""
import numpy as _np
from numpy import *  # noqa: F401,F403
from numpy import linalg  # noqa: F401


def _as_array(f):
    def g(*a, **k):
        return _np.asarray(f(*a, **k))

    g.__name__ = f.__name__
    return g


for _name in ("sqrt", "exp", "log", "sum", "mean", "real", "imag", "abs", "clip", "where", "prod", "trace",
              "angle", "cos", "sin", "asarray", "array", "conj", "einsum", "cumsum", "searchsorted", "diag", "full"):
    globals()[_name] = _as_array(getattr(_np, _name))


def __getattr__(name):
    return getattr(_np, name)
