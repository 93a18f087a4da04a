"""jax.lax stand-in: scan as a loop, complex from two real arrays."""
import numpy as _np


def scan(f, init, xs=None, length=None):
    carry = init
    ys = []
    if xs is None:
        for _ in range(int(length)):
            carry, y = f(carry, None)
            ys.append(y)
    else:
        n = len(xs[0]) if isinstance(xs, tuple) else len(xs)
        for i in range(n):
            x = tuple(e[i] for e in xs) if isinstance(xs, tuple) else xs[i]
            carry, y = f(carry, x)
            ys.append(y)
    if not ys or ys[0] is None:
        return carry, None
    if isinstance(ys[0], tuple):
        return carry, tuple(_np.stack([y[k] for y in ys]) for k in range(len(ys[0])))
    return carry, _np.stack(ys)


def complex(re, im):  # noqa: A001 - the jax.lax name
    return _np.asarray(re) + 1j * _np.asarray(im)
