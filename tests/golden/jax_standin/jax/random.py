"""jax.random stand-in: keys are placeholders, draws come from a queue.

The generator script calls feed(normals=[...], uniforms=[...]); every
jax.random.normal(key, shape) pops the next normal array (its shape must
match) and every jax.random.uniform(key) the next uniform.  The reference
then consumes exactly the injected fields and comb uniforms.
"""
import numpy as _np

_normals = []
_uniforms = []


def feed(normals=(), uniforms=()):
    _normals[:] = [_np.asarray(a, dtype=_np.float64) for a in normals]
    _uniforms[:] = [float(u) for u in uniforms]


def remaining():
    return len(_normals), len(_uniforms)


def PRNGKey(seed):  # noqa: N802 - the jax name
    return _np.array([0, int(seed)], dtype=_np.uint32)


def split(key, num=2):
    return tuple(_np.array(key) for _ in range(num))


def normal(key, shape=(), dtype=None):
    if not _normals:
        raise RuntimeError("jax stand-in: no injected normals left")
    a = _normals.pop(0)
    if tuple(a.shape) != tuple(shape):
        raise ValueError(f"jax stand-in: injected normals {a.shape} != requested {tuple(shape)}")
    return a


def uniform(key, shape=(), dtype=None, minval=0.0, maxval=1.0):
    if not _uniforms:
        raise RuntimeError("jax stand-in: no injected uniforms left")
    if tuple(shape) != ():
        raise ValueError("jax stand-in: only scalar uniforms are injected")
    return _np.float64(_uniforms.pop(0))
