"""jax.random of the numpy stand-in: keys are (2,) uint32 arrays driving numpy generators.

The streams are not JAX's threefry streams; the golden vectors pass every random input
explicitly, so nothing they record depends on these draws."""

from __future__ import annotations

import numpy as _np

from ._core import _unwrap, canon_dtype, wrap


def PRNGKey(seed):
    return wrap(_np.array([0, int(seed) & 0xFFFFFFFF], _np.uint32))


key = PRNGKey


def _gen(k):
    a = _np.asarray(_unwrap(k)).astype(_np.uint64)
    return _np.random.Generator(_np.random.PCG64(int(a[0]) << 32 | int(a[1])))


def split(k, num=2):
    g = _gen(k)
    return wrap(g.integers(0, 2**32, size=(int(num), 2), dtype=_np.uint64).astype(_np.uint32))


def fold_in(k, data):
    g = _np.random.Generator(_np.random.PCG64([int(x) for x in _np.asarray(_unwrap(k))] + [int(data)]))
    return wrap(g.integers(0, 2**32, size=2, dtype=_np.uint64).astype(_np.uint32))


def uniform(k, shape=(), dtype=float, minval=0.0, maxval=1.0):
    return wrap(_gen(k).uniform(_unwrap(minval), _unwrap(maxval), size=shape).astype(canon_dtype(dtype)))


def normal(k, shape=(), dtype=float):
    return wrap(_gen(k).normal(size=shape).astype(canon_dtype(dtype)))


def permutation(k, x):
    return wrap(_gen(k).permutation(_unwrap(x)))
