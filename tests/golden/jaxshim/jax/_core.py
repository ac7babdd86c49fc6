"""Array type and dtype rules of the numpy stand-in for JAX (golden-vector generation only)."""

from __future__ import annotations

import numpy as np

X64 = {"on": False}


def canon_dtype(dt):
    """JAX's canonical dtype: 64-bit types become 32-bit while x64 is off."""
    if dt is None:
        return None
    if dt is int:
        return np.dtype(np.int64 if X64["on"] else np.int32)
    if dt is float:
        return np.dtype(np.float64 if X64["on"] else np.float32)
    if dt is bool:
        return np.dtype(bool)
    if dt is complex:
        return np.dtype(np.complex128 if X64["on"] else np.complex64)
    dt = np.dtype(dt)
    if not X64["on"]:
        if dt == np.float64:
            return np.dtype(np.float32)
        if dt == np.int64:
            return np.dtype(np.int32)
        if dt == np.uint64:
            return np.dtype(np.uint32)
        if dt == np.complex128:
            return np.dtype(np.complex64)
    return dt


class Array(np.ndarray):
    """numpy array with JAX's functional ``.at[...]`` updates and 32-bit dtype rules."""

    __array_priority__ = 100

    def __array_finalize__(self, obj):
        pass

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        args = [np.asarray(x) if isinstance(x, Array) else x for x in inputs]
        if "out" in kwargs:
            kwargs["out"] = tuple(np.asarray(o) if isinstance(o, Array) else o for o in kwargs["out"])
        res = getattr(ufunc, method)(*args, **kwargs)
        return wrap(res)

    def __getitem__(self, idx):
        base = np.asarray(self)
        if isinstance(idx, tuple):
            out, ax = [], 0
            for i in idx:
                if i is None:
                    out.append(i)
                    continue
                if i is Ellipsis:
                    out.append(i)
                    ax = base.ndim - (len([x for x in idx if x is not None and x is not Ellipsis]) - ax - 1)
                    continue
                out.append(_clamp_index(i, base.shape[ax]) if ax < base.ndim else i)
                ax += 1
            idx = tuple(out)
        else:
            idx = _clamp_index(idx, base.shape[0]) if base.ndim else idx
        r = np.ndarray.__getitem__(base, idx)
        return wrap(r)

    # JAX arrays are immutable: augmented assignment rebinds to a new array
    def __iadd__(self, o):
        return self + o

    def __isub__(self, o):
        return self - o

    def __imul__(self, o):
        return self * o

    def __itruediv__(self, o):
        return self / o

    def __ifloordiv__(self, o):
        return self // o

    def __imod__(self, o):
        return self % o

    def __ipow__(self, o):
        return self**o

    def __iand__(self, o):
        return self & o

    def __ior__(self, o):
        return self | o

    def __ixor__(self, o):
        return self ^ o

    def __setitem__(self, idx, v):
        raise TypeError("JAX arrays are immutable; use x.at[idx].set(v)")

    def astype(self, dtype, *a, **k):
        return wrap(np.asarray(self).astype(canon_dtype(dtype)))

    @property
    def at(self):
        return _At(self)

    def block_until_ready(self):
        return self

    def item(self, *a):
        return np.asarray(self).item(*a)

    def __bool__(self):
        return bool(np.asarray(self))

    def __index__(self):
        return int(np.asarray(self))

    def __hash__(self):
        raise TypeError("unhashable type: jax Array")


def _clamp_index(i, n):
    """JAX gathers clamp out-of-range integer indices (after one negative wrap)."""
    if isinstance(i, Array):
        i = np.asarray(i)
    if isinstance(i, (int, np.integer)) and not isinstance(i, bool):
        i = int(i)
        if i < 0:
            i += n
        return min(max(i, 0), n - 1)
    if isinstance(i, np.ndarray) and i.dtype.kind in "iu":
        j = np.where(i < 0, i + n, i)
        return np.clip(j, 0, n - 1)
    return i


def wrap(x):
    """numpy result -> Array with canonical dtype (tuples and lists element-wise)."""
    if isinstance(x, (tuple, list)):
        return type(x)(wrap(v) for v in x)
    if isinstance(x, Array):
        dt = canon_dtype(x.dtype)
        return x if dt == x.dtype else np.asarray(x).astype(dt).view(Array)
    if isinstance(x, (np.ndarray, np.generic)):
        a = np.asarray(x)
        dt = canon_dtype(a.dtype)
        if dt != a.dtype:
            a = a.astype(dt)
        elif not a.flags.writeable or a.base is not None:
            pass
        return a.view(Array)
    return x


def asarray(x, dtype=None):
    if isinstance(x, Array) and dtype is None:
        return x
    if dtype is not None:
        return wrap(np.asarray(_unwrap(x), dtype=canon_dtype(dtype)))
    if isinstance(x, bool):
        return wrap(np.asarray(x))
    if isinstance(x, int):
        return wrap(np.asarray(x, dtype=canon_dtype(int)))
    if isinstance(x, float):
        return wrap(np.asarray(x, dtype=canon_dtype(float)))
    return wrap(np.array(_unwrap(x), copy=True))


def _unwrap(x):
    if isinstance(x, Array):
        return np.asarray(x)
    if isinstance(x, (list, tuple)):
        return type(x)(_unwrap(v) for v in x)
    return x


def _norm_index(idx):
    if isinstance(idx, Array):
        return np.asarray(idx)
    if isinstance(idx, tuple):
        return tuple(_norm_index(i) for i in idx)
    return idx


def _drop_mask(base, idx):
    """For a single integer-array index along axis 0: the entries inside [-n, n)."""
    if isinstance(idx, np.ndarray) and idx.dtype.kind in "iu":
        n = base.shape[0]
        return (idx >= -n) & (idx < n)
    return None


class _AtOp:
    def __init__(self, arr, idx):
        self.arr = arr
        self.idx = _norm_index(idx)

    def _apply(self, fn, values, mode=None):
        base = np.array(np.asarray(self.arr), copy=True)
        vals = np.asarray(_unwrap(values))
        if vals.dtype != base.dtype:
            vals = vals.astype(base.dtype)
        idx = self.idx
        comps = idx if isinstance(idx, tuple) else (idx,)
        if comps and all(isinstance(c, np.ndarray) and c.dtype.kind in "iu" for c in comps):
            # advanced integer indexing: scatter indices outside the array are dropped
            bc = np.broadcast_arrays(*comps)
            keep = np.ones(bc[0].shape, bool)
            for ax, c in enumerate(bc):
                n = base.shape[ax]
                keep &= (c >= -n) & (c < n)
            sub_shape = bc[0].shape + base.shape[len(bc):]
            v = np.broadcast_to(vals, sub_shape)
            fn(base, tuple(c[keep] for c in bc), v[keep])
            return wrap(base)
        fn(base, idx, vals)
        return wrap(base)

    def set(self, values, mode=None, **k):
        def f(b, i, v):
            b[i] = v

        return self._apply(f, values, mode)

    def add(self, values, mode=None, **k):
        return self._apply(lambda b, i, v: np.add.at(b, i, v), values, mode)

    def subtract(self, values, mode=None, **k):
        return self._apply(lambda b, i, v: np.subtract.at(b, i, v), values, mode)

    def multiply(self, values, mode=None, **k):
        return self._apply(lambda b, i, v: np.multiply.at(b, i, v), values, mode)

    def min(self, values, mode=None, **k):
        return self._apply(lambda b, i, v: np.minimum.at(b, i, v), values, mode)

    def max(self, values, mode=None, **k):
        return self._apply(lambda b, i, v: np.maximum.at(b, i, v), values, mode)

    def get(self, mode=None, fill_value=None, **k):
        base = np.asarray(self.arr)
        idx = self.idx
        keep = _drop_mask(base, idx)
        if keep is not None and not keep.all():
            safe = np.where(keep, idx, 0)
            out = np.array(base[safe], copy=True)
            fv = fill_value if fill_value is not None else (np.nan if base.dtype.kind == "f" else 0)
            out[~keep] = fv
            return wrap(out)
        return wrap(base[idx])


class _At:
    def __init__(self, arr):
        self.arr = arr

    def __getitem__(self, idx):
        return _AtOp(self.arr, idx)
