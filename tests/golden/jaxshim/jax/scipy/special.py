"""jax.scipy.special of the numpy stand-in (scipy.special)."""

import scipy.special as _sp

from .._core import _unwrap, wrap


def __getattr__(name):
    fn = getattr(_sp, name)

    def f(*a, **k):
        return wrap(fn(*[_unwrap(x) for x in a], **k))

    return f
