"""jax.numpy.linalg of the numpy stand-in."""

from __future__ import annotations

import numpy as _np

from .._core import _unwrap, wrap


def __getattr__(name):
    fn = getattr(_np.linalg, name)

    def f(*a, **k):
        return wrap(fn(*[_unwrap(x) for x in a], **k))

    return f
