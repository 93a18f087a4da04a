"""jax.scipy.linalg stand-in: scipy.linalg (expm: Pade scaling and squaring, as JAX's)."""
from scipy.linalg import *  # noqa: F401,F403
from scipy.linalg import expm  # noqa: F401
