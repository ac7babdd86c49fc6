"""jax.scipy of the numpy stand-in."""

from . import special  # noqa: F401
