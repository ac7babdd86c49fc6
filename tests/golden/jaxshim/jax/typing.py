"""jax.typing of the numpy stand-in."""

from typing import Any

ArrayLike = Any
DTypeLike = Any
