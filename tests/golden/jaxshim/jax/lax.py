"""jax.lax of the numpy stand-in: control flow as Python, sort stable."""

from __future__ import annotations

import numpy as _np

from ._core import Array, _unwrap, asarray, canon_dtype, wrap
from .tree_util import tree_flatten, tree_map, tree_unflatten


def while_loop(cond_fun, body_fun, init_val):
    val = init_val
    while bool(cond_fun(val)):
        val = body_fun(val)
    return val


def fori_loop(lower, upper, body_fun, init_val, unroll=None):
    val = init_val
    for i in range(int(lower), int(upper)):
        val = body_fun(asarray(i), val)
    return val


def scan(f, init, xs=None, length=None, reverse=False, unroll=1, **k):
    if xs is None:
        n = int(length)
        items = [None] * n
    else:
        leaves, td = tree_flatten(xs)
        n = int(_np.shape(leaves[0])[0]) if leaves else int(length)
        items = [tree_unflatten(td, [l[i] for l in leaves]) for i in range(n)]
    order = range(n - 1, -1, -1) if reverse else range(n)
    carry, ys = init, [None] * n
    for i in order:
        carry, y = f(carry, items[i])
        ys[i] = y
    if n == 0 or ys[0] is None:
        return carry, None
    return carry, tree_map(lambda *v: wrap(_np.stack([_np.asarray(_unwrap(x)) for x in v])), *ys)


def cond(pred, true_fun, false_fun, *operands, **k):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def switch(index, branches, *operands):
    i = int(_np.clip(int(index), 0, len(branches) - 1))
    return branches[i](*operands)


def select(pred, on_true, on_false):
    return wrap(_np.where(_unwrap(pred), _unwrap(on_true), _unwrap(on_false)))


def iota(dtype, size, dimension=0, **k):
    return wrap(_np.arange(int(size), dtype=canon_dtype(dtype)))


def sort(operand, dimension=-1, is_stable=True, num_keys=1):
    if isinstance(operand, (list, tuple)):
        ops = [_np.asarray(_unwrap(o)) for o in operand]
        keys = ops[:num_keys]
        order = _np.lexsort(tuple(reversed([_np.moveaxis(kk, dimension, -1) for kk in keys])), axis=-1)
        out = [_np.take_along_axis(_np.moveaxis(o, dimension, -1), order, axis=-1) for o in ops]
        return type(operand)(wrap(_np.moveaxis(o, -1, dimension)) for o in out)
    return wrap(_np.sort(_np.asarray(_unwrap(operand)), axis=dimension, kind="stable"))


def rsqrt(x):
    x = _np.asarray(_unwrap(x))
    return wrap(_np.asarray(1.0, x.dtype) / _np.sqrt(x))


def stop_gradient(x):
    return x


def top_k(operand, k):
    a = _np.asarray(_unwrap(operand))
    idx = _np.argsort(-a, axis=-1, kind="stable")[..., :k]
    return wrap(_np.take_along_axis(a, idx, -1)), wrap(idx.astype(_np.int32))


def map(f, xs, **k):  # noqa: A001
    leaves, td = tree_flatten(xs)
    n = int(_np.shape(leaves[0])[0])
    ys = [f(tree_unflatten(td, [l[i] for l in leaves])) for i in range(n)]
    return tree_map(lambda *v: wrap(_np.stack([_np.asarray(_unwrap(x)) for x in v])), *ys)


def clamp(lo, x, hi):
    return wrap(_np.clip(_unwrap(x), _unwrap(lo), _unwrap(hi)))


def dynamic_slice(operand, start_indices, slice_sizes):
    a = _np.asarray(_unwrap(operand))
    idx = tuple(slice(int(s), int(s) + int(n)) for s, n in zip(start_indices, slice_sizes))
    return wrap(a[idx])


def pow(x, y):  # noqa: A001
    return wrap(_np.power(_unwrap(x), _unwrap(y)))


def __getattr__(name):
    fn = getattr(_np, name)

    def f(*a, **k):
        return wrap(fn(*[_unwrap(x) for x in a], **k))

    return f
