"""Pytrees of the numpy stand-in for JAX: tuples, lists, dicts, None and registered dataclasses."""

from __future__ import annotations

import dataclasses

_REG = {}  # cls -> (data_fields, meta_fields) or (flatten, unflatten) for generic nodes


def register_dataclass(cls=None, data_fields=None, meta_fields=None, drop_fields=()):
    def reg(c):
        if data_fields is None:
            fs = [f for f in dataclasses.fields(c) if f.init or True]
            df = [f.name for f in fs if not f.metadata.get("static", False)]
            mf = [f.name for f in fs if f.metadata.get("static", False)]
        else:
            df, mf = list(data_fields), list(meta_fields or [])
        _REG[c] = ("dataclass", df, mf)
        return c

    return reg(cls) if cls is not None else reg


def register_pytree_node(cls, flatten, unflatten):
    _REG[cls] = ("generic", flatten, unflatten)
    return cls


def register_pytree_node_class(cls):
    _REG[cls] = ("generic", lambda x: x.tree_flatten(), lambda aux, ch: cls.tree_unflatten(aux, ch))
    return cls


class _Node:
    __slots__ = ("kind", "aux", "children")

    def __init__(self, kind, aux, children):
        self.kind, self.aux, self.children = kind, aux, children


LEAF = _Node("leaf", None, ())


def _is_node(x):
    return x is None or type(x) in (tuple, list, dict) or type(x) in _REG or (
        isinstance(x, tuple) and hasattr(x, "_fields"))


def _flatten(x, leaves, is_leaf):
    if is_leaf is not None and is_leaf(x):
        leaves.append(x)
        return LEAF
    if x is None:
        return _Node("none", None, ())
    t = type(x)
    if t is tuple or t is list:
        return _Node(t.__name__, None, tuple(_flatten(v, leaves, is_leaf) for v in x))
    if isinstance(x, tuple) and hasattr(x, "_fields"):
        return _Node("namedtuple", t, tuple(_flatten(v, leaves, is_leaf) for v in x))
    if t is dict:
        keys = sorted(x.keys())
        return _Node("dict", tuple(keys), tuple(_flatten(x[k], leaves, is_leaf) for k in keys))
    if t in _REG:
        r = _REG[t]
        if r[0] == "dataclass":
            _, df, mf = r
            meta = tuple((k, getattr(x, k)) for k in mf)
            return _Node("dataclass", (t, tuple(df), meta), tuple(_flatten(getattr(x, k), leaves, is_leaf) for k in df))
        _, fl, _unfl = r
        ch, aux = fl(x)
        return _Node("generic", (t, aux), tuple(_flatten(v, leaves, is_leaf) for v in ch))
    leaves.append(x)
    return LEAF


def _unflatten(node, it):
    k = node.kind
    if k == "leaf":
        return next(it)
    if k == "none":
        return None
    ch = [_unflatten(c, it) for c in node.children]
    if k == "tuple":
        return tuple(ch)
    if k == "list":
        return list(ch)
    if k == "namedtuple":
        return node.aux(*ch)
    if k == "dict":
        return dict(zip(node.aux, ch))
    if k == "dataclass":
        t, df, meta = node.aux
        kw = dict(zip(df, ch))
        kw.update(dict(meta))
        try:
            return t(**kw)
        except TypeError:
            obj = object.__new__(t)
            for name, v in kw.items():
                object.__setattr__(obj, name, v)
            return obj
    t, aux = node.aux
    return _REG[t][2](aux, ch)


class PyTreeDef:
    def __init__(self, node, n):
        self.node, self.num_leaves = node, n

    def unflatten(self, leaves):
        return _unflatten(self.node, iter(leaves))


def tree_flatten(x, is_leaf=None):
    leaves = []
    node = _flatten(x, leaves, is_leaf)
    return leaves, PyTreeDef(node, len(leaves))


def tree_unflatten(treedef, leaves):
    return treedef.unflatten(list(leaves))


def tree_leaves(x, is_leaf=None):
    return tree_flatten(x, is_leaf)[0]


def tree_structure(x, is_leaf=None):
    return tree_flatten(x, is_leaf)[1]


def tree_map(f, tree, *rest, is_leaf=None):
    leaves, td = tree_flatten(tree, is_leaf)
    others = [td_leaves_like(r, td, is_leaf) for r in rest]
    return td.unflatten([f(*xs) for xs in zip(leaves, *others)])


def td_leaves_like(tree, td, is_leaf):
    leaves, _ = tree_flatten(tree, is_leaf)
    if len(leaves) != td.num_leaves:
        raise ValueError("pytree structures differ")
    return leaves


class Partial:
    def __init__(self, func, *args, **kw):
        self.func, self.args, self.kw = func, args, kw

    def __call__(self, *a, **k):
        return self.func(*self.args, *a, **{**self.kw, **k})
