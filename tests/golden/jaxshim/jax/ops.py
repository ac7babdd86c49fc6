"""jax.ops segment reductions of the numpy stand-in (out-of-range ids dropped)."""

from __future__ import annotations

import numpy as _np

from ._core import _unwrap, wrap


def _seg(data, segment_ids, num_segments, ufunc, init):
    d = _np.asarray(_unwrap(data))
    ids = _np.asarray(_unwrap(segment_ids))
    n = int(num_segments) if num_segments is not None else int(ids.max()) + 1
    out = _np.full((n,) + d.shape[1:], init, d.dtype)
    keep = (ids >= 0) & (ids < n)
    ufunc.at(out, ids[keep], d[keep])
    return wrap(out)


def segment_sum(data, segment_ids, num_segments=None, **k):
    return _seg(data, segment_ids, num_segments, _np.add, 0)


def segment_max(data, segment_ids, num_segments=None, **k):
    d = _np.asarray(_unwrap(data))
    init = -_np.inf if d.dtype.kind == "f" else _np.iinfo(d.dtype).min
    return _seg(data, segment_ids, num_segments, _np.maximum, init)


def segment_min(data, segment_ids, num_segments=None, **k):
    d = _np.asarray(_unwrap(data))
    init = _np.inf if d.dtype.kind == "f" else _np.iinfo(d.dtype).max
    return _seg(data, segment_ids, num_segments, _np.minimum, init)


def segment_prod(data, segment_ids, num_segments=None, **k):
    return _seg(data, segment_ids, num_segments, _np.multiply, 1)
