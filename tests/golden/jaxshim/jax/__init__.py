"""A numpy stand-in for the JAX API subset JaxDEM's hot path uses (golden-vector generation).

jit and named_call are identity wrappers, vmap loops over the mapped axis and stacks the
results, and lax control flow runs as Python.  See tests/golden/jaxshim/README.txt.
"""

from __future__ import annotations

import dataclasses as _dc
import types as _types

import numpy as _np

from . import debug, lax, nn, ops, random, scipy, tree_util  # noqa: F401
from . import numpy  # noqa: F401
from . import typing  # noqa: F401
from ._core import X64 as _X64
from ._core import Array, _unwrap, wrap

__version__ = "0.8.1"


class _Config:
    def update(self, name, value):
        if name == "jax_enable_x64":
            _X64["on"] = bool(value)

    @property
    def jax_enable_x64(self):
        return _X64["on"]

    def __getattr__(self, name):
        return False


config = _Config()


def _fresh(x):
    """The same pytree in new containers: a traced function sees copies of the caller's
    dataclasses, so rebinding their fields (``state.vel += ...``) never reaches the caller."""
    leaves, td = tree_util.tree_flatten(x)
    return td.unflatten(leaves)


def jit(fun=None, **kw):
    if fun is None:
        return lambda f: jit(f, **kw)

    def traced(*a, **k):
        return fun(*[_fresh(x) for x in a], **{key: _fresh(v) for key, v in k.items()})

    traced.__name__ = getattr(fun, "__name__", "jitted")
    traced.__wrapped__ = fun
    return traced


def named_call(fun, name=None):
    return fun


def _axis_leaves(args, in_axes):
    """Per argument: (leaves, treedef, axis or None per leaf)."""
    if not isinstance(in_axes, (tuple, list)):
        in_axes = (in_axes,) * len(args)
    out = []
    for a, ax in zip(args, in_axes):
        leaves, td = tree_util.tree_flatten(a)
        if isinstance(ax, int) or ax is None:
            axes = [ax] * len(leaves)
        else:
            axes, _ = tree_util.tree_flatten(ax, is_leaf=lambda x: x is None)
            if len(axes) != len(leaves):
                axes = [axes[0]] * len(leaves)
        out.append((leaves, td, axes))
    return out


def vmap(fun, in_axes=0, out_axes=0, axis_size=None, **kw):
    def wrapped(*args):
        spec = _axis_leaves(args, in_axes)
        n = axis_size
        for leaves, _, axes in spec:
            for l, ax in zip(leaves, axes):
                if ax is not None:
                    n = _np.shape(_unwrap(l))[ax]
                    break
            if n is not None:
                break
        outs = []
        for i in range(int(n)):
            call = []
            for leaves, td, axes in spec:
                sl = [l if ax is None else wrap(_np.take(_np.asarray(_unwrap(l)), i, axis=ax)) for l, ax in zip(leaves, axes)]
                call.append(td.unflatten(sl))
            outs.append(fun(*call))
        if n == 0:
            raise NotImplementedError("vmap over an empty axis")
        return tree_util.tree_map(
            lambda *v: wrap(_np.stack([_np.asarray(_unwrap(x)) for x in v], axis=out_axes if isinstance(out_axes, int) else 0)),
            *outs)

    return wrapped


def pure_callback(callback, result_shape_dtypes, *args, **kw):
    return callback(*args)


def device_get(x):
    return x


def block_until_ready(x):
    return x


def grad(*a, **k):
    raise NotImplementedError("jax.grad is outside the numpy stand-in")


hessian = grad
jacfwd = grad
jacrev = grad


@_dc.dataclass
class ShapeDtypeStruct:
    shape: tuple
    dtype: object


def devices(*a):
    return ["cpu"]


def _static(*args, **kwargs):
    metadata = dict(kwargs.pop("metadata", {}) or {})
    metadata["static"] = True
    return _dc.field(*args, metadata=metadata, **kwargs)


tree = _types.SimpleNamespace(
    map=tree_util.tree_map,
    leaves=tree_util.tree_leaves,
    flatten=tree_util.tree_flatten,
    unflatten=tree_util.tree_unflatten,
    structure=tree_util.tree_structure,
    static=_static,
)


class custom_vjp:  # noqa: N801
    """Differentiation rules are irrelevant without autodiff: calls go to the function."""

    def __init__(self, fun, nondiff_argnums=()):
        self.fun = fun

    def defvjp(self, fwd, bwd, **k):
        return None

    def __call__(self, *a, **k):
        return self.fun(*a, **k)


class custom_jvp(custom_vjp):  # noqa: N801
    def defjvp(self, jvp, **k):
        return jvp

    def defjvps(self, *a):
        return None


def checkpoint(fun=None, **k):
    return (lambda f: f) if fun is None else fun


remat = checkpoint


class ensure_compile_time_eval:  # noqa: N801
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
