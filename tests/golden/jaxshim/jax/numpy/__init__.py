"""jax.numpy of the numpy stand-in: numpy functions with JAX's dtype defaults, returning Arrays."""

from __future__ import annotations

import numpy as _np

from .._core import Array as ndarray  # noqa: F401
from .._core import Array, _unwrap, asarray, canon_dtype, wrap
from . import linalg  # noqa: F401

float16, float32, float64 = _np.float16, _np.float32, _np.float64
int8, int16, int32, int64 = _np.int8, _np.int16, _np.int32, _np.int64
uint8, uint16, uint32, uint64 = _np.uint8, _np.uint16, _np.uint32, _np.uint64
bool_ = _np.bool_
complex64, complex128 = _np.complex64, _np.complex128
integer, floating, number, inexact, signedinteger = _np.integer, _np.floating, _np.number, _np.inexact, _np.signedinteger
dtype = _np.dtype
pi, e, inf, nan, newaxis = _np.pi, _np.e, _np.inf, _np.nan, None
iinfo, finfo, issubdtype = _np.iinfo, _np.finfo, _np.issubdtype


def _w(fn):
    def f(*args, **kw):
        return wrap(fn(*_unwrap(list(args)), **{k: _unwrap(v) for k, v in kw.items()}))

    f.__name__ = getattr(fn, "__name__", "f")
    return f


def array(x, dtype=None, copy=True, **k):
    if isinstance(x, (list, tuple)) and any(isinstance(v, Array) for v in x):
        x = [_np.asarray(v) if isinstance(v, Array) else v for v in x]
    if dtype is None:
        a = _np.array(_unwrap(x))
        if isinstance(x, float) or (a.dtype == _np.float64):
            return wrap(a)
        return wrap(a)
    return wrap(_np.array(_unwrap(x), dtype=canon_dtype(dtype)))


def _dt(dtype, default):
    return canon_dtype(default if dtype is None else dtype)


def zeros(shape, dtype=None, **k):
    return wrap(_np.zeros(shape, _dt(dtype, float)))


def ones(shape, dtype=None, **k):
    return wrap(_np.ones(shape, _dt(dtype, float)))


def empty(shape, dtype=None, **k):
    return wrap(_np.zeros(shape, _dt(dtype, float)))


def full(shape, fill_value, dtype=None, **k):
    if dtype is None:
        fv = _np.asarray(_unwrap(fill_value))
        dtype = fv.dtype if not isinstance(fill_value, (int, float, bool)) else type(fill_value)
    return wrap(_np.full(shape, _unwrap(fill_value), _dt(dtype, float)))


def zeros_like(a, dtype=None, **k):
    return wrap(_np.zeros_like(_np.asarray(_unwrap(a)), dtype=canon_dtype(dtype)))


def ones_like(a, dtype=None, **k):
    return wrap(_np.ones_like(_np.asarray(_unwrap(a)), dtype=canon_dtype(dtype)))


def full_like(a, fill_value, dtype=None, **k):
    return wrap(_np.full_like(_np.asarray(_unwrap(a)), _unwrap(fill_value), dtype=canon_dtype(dtype)))


def empty_like(a, dtype=None, **k):
    return zeros_like(a, dtype)


def arange(*args, dtype=None, **k):
    args = [_unwrap(a) for a in args]
    if dtype is None:
        dtype = float if any(isinstance(a, float) or (hasattr(a, "dtype") and a.dtype.kind == "f") for a in args) else int
    return wrap(_np.arange(*args, dtype=canon_dtype(dtype)))


def eye(N, M=None, k=0, dtype=None):
    return wrap(_np.eye(N, M, k, dtype=_dt(dtype, float)))


def linspace(start, stop, num=50, endpoint=True, dtype=None, **k):
    return wrap(_np.linspace(_unwrap(start), _unwrap(stop), num, endpoint=endpoint, dtype=canon_dtype(dtype)))


def searchsorted(a, v, side="left", sorter=None, method=None):
    return wrap(_np.searchsorted(_np.asarray(_unwrap(a)), _unwrap(v), side=side, sorter=sorter).astype(canon_dtype(int)))


def bincount(x, weights=None, minlength=0, length=None):
    x = _np.asarray(_unwrap(x))
    w = None if weights is None else _np.asarray(_unwrap(weights))
    n = length if length is not None else max(int(minlength), int(x.max()) + 1 if x.size else 0)
    keep = (x >= 0) & (x < n)
    out = _np.bincount(x[keep], None if w is None else w[keep], minlength=n)[:n]
    if w is None:
        out = out.astype(canon_dtype(int))
    return wrap(out)


def unique(ar, return_index=False, return_inverse=False, return_counts=False, axis=None, size=None,
           fill_value=None):
    res = _np.unique(_np.asarray(_unwrap(ar)), return_index=return_index, return_inverse=return_inverse,
                     return_counts=return_counts, axis=axis)
    if size is not None:
        def pad(a, fv):
            a = _np.asarray(a)
            if a.shape[0] >= size:
                return a[:size]
            fill = a[0] if fv is None and a.size else (0 if fv is None else fv)
            return _np.concatenate([a, _np.full((size - a.shape[0],) + a.shape[1:], fill, a.dtype)])

        if isinstance(res, tuple):
            res = (pad(res[0], fill_value),) + tuple(res[1:])
        else:
            res = pad(res, fill_value)
    return wrap(res)


def where(cond, x=None, y=None, **k):
    if x is None:
        return wrap(_np.where(_np.asarray(_unwrap(cond))))
    return wrap(_np.where(_np.asarray(_unwrap(cond)), _unwrap(x), _unwrap(y)))


def round(a, decimals=0):  # noqa: A001
    return wrap(_np.round(_np.asarray(_unwrap(a)), decimals))


def vecdot(a, b, axis=-1):
    return wrap(_np.sum(_np.asarray(_unwrap(a)) * _np.asarray(_unwrap(b)), axis=axis))


def isin(element, test_elements, **k):
    return wrap(_np.isin(_unwrap(element), _unwrap(test_elements)))


def copy(a, **k):
    return wrap(_np.array(_unwrap(a), copy=True))


def shape(a):
    return _np.shape(_unwrap(a))


def ndim(a):
    return _np.ndim(_unwrap(a))


def size(a, axis=None):
    return _np.size(_unwrap(a), axis)


def result_type(*a):
    return canon_dtype(_np.result_type(*[_unwrap(x) for x in a]))


_WRAPPED = {}


def __getattr__(name):
    # cached outside the module namespace: names such as ``any`` or ``max`` must not
    # shadow the builtins this module's own functions use
    if name in _WRAPPED:
        return _WRAPPED[name]
    fn = getattr(_np, name)
    if callable(fn) and not isinstance(fn, type):
        w = _WRAPPED[name] = _w(fn)
        return w
    return fn
