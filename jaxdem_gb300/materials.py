"""Materials, matchmakers and the material table (host side).

Mirrors ``jaxdem/materials`` and ``jaxdem/material_matchmakers``: the kernel
only receives ``young_eff`` (M, M) and the per-material ``density`` used for
masses.  Harmonic matcher: ``harmonic.py:32-40``; linear: ``linear.py:31-33``;
table construction: ``material_table.py:77-128``.
"""

from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Sequence

import numpy as np

from .factory import Factory


class Material(Factory):
    """Base of material property records."""


@Material.register("elastic")
@dataclass
class Elastic(Material):
    young: float
    poisson: float
    density: float = 1.0


@Material.register("elasticfrict")
@dataclass
class ElasticFriction(Material):
    young: float
    poisson: float
    mu: float
    e: float = 1.0
    density: float = 1.0
    mu_r: float = 0.0  # rolling friction (materials/elastic_mats.py:45)


class MaterialMatchmaker(Factory):
    """Rule combining two materials' scalar property into a pair property."""

    @staticmethod
    def get_effective_property(a, b):  # pragma: no cover - abstract
        raise NotImplementedError


@MaterialMatchmaker.register("harmonic")
@dataclass
class HarmonicMaterialMatchmaker(MaterialMatchmaker):
    @staticmethod
    def get_effective_property(a, b):
        """``2 a b / (a + b)``, 0 when either is 0 (``harmonic.py:32-40``)."""
        a = np.asarray(a, np.float32)
        b = np.asarray(b, np.float32)
        zero = (a == 0) | (b == 0)
        sa = np.where(zero, np.float32(1), a)
        sb = np.where(zero, np.float32(1), b)
        return np.where(zero, np.float32(0), np.float32(2.0) * sa * sb / (sa + sb)).astype(np.float32)


@MaterialMatchmaker.register("linear")
@dataclass
class LinearMaterialMatchmaker(MaterialMatchmaker):
    @staticmethod
    def get_effective_property(a, b):
        """Arithmetic mean (``linear.py:31-33``)."""
        return ((np.asarray(a, np.float32) + np.asarray(b, np.float32)) / np.float32(2)).astype(np.float32)


@dataclass(frozen=True)
class MaterialTable:
    """Scalar properties (M,) and effective pair properties (M, M)."""

    props: dict
    pair: dict
    matcher: MaterialMatchmaker

    @staticmethod
    def from_materials(mats: Sequence[Material], *, matcher: MaterialMatchmaker | None = None,
                       fill: float = 0.0) -> "MaterialTable":
        if not mats or not all(isinstance(m, Material) for m in mats):
            raise TypeError("from_materials expects a non-empty sequence of Material instances")
        keys = sorted({f.name for m in mats for f in fields(m)})
        scal = {k: np.asarray([getattr(m, k, fill) for m in mats], np.float32) for k in keys}
        if matcher is None:
            matcher = MaterialMatchmaker.create("harmonic")
        pair = {f"{k}_eff": matcher.get_effective_property(v[:, None], v[None, :]) for k, v in scal.items()}
        return MaterialTable(props=scal, pair=pair, matcher=matcher)

    def __getattr__(self, name):
        props = object.__getattribute__(self, "props")
        pair = object.__getattribute__(self, "pair")
        if name in props:
            return props[name]
        if name in pair:
            return pair[name]
        raise AttributeError(name)

    @property
    def M(self) -> int:
        return int(next(iter(self.props.values())).shape[0])
