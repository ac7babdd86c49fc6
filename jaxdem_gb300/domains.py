"""Domains (``jaxdem/domains``): box, anchor and boundary rule of a system.

The device kernels implement the three domains the hot path uses: periodic
minimum image (``periodic.py:74-79``), reflecting walls with the Verlet
time-of-collision correction (``reflect.py:99-299``, ``_toc.py:11-94``) and
the free bounding box (``free.py:40-63``).  These classes carry the
parameters and the host-side ``displacement``/``shift`` helpers.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Any

import numpy as np

from .factory import Factory

F32 = np.float32


@dataclass
class Domain(Factory):
    box_size: np.ndarray
    inv_box_size: np.ndarray
    anchor: np.ndarray

    @property
    def periodic(self) -> bool:
        return False

    @classmethod
    def Create(cls, dim: int, box_size=None, anchor=None, **kw: Any):
        """``Domain.Create`` (``domains/__init__.py:62-121``)."""
        box = np.ones(dim, F32) if box_size is None else np.asarray(box_size, F32)
        if box.shape != (dim,):
            raise ValueError(f"box_size must have shape ({dim},), got shape {box.shape}.")
        anc = np.zeros_like(box) if anchor is None else np.asarray(anchor, F32)
        if anc.shape != (dim,):
            raise ValueError(f"anchor must have shape ({dim},), got shape {anc.shape}.")
        return cls(box_size=box, inv_box_size=(F32(1.0) / box).astype(F32), anchor=anc, **kw)

    @staticmethod
    def displacement(ri, rj, system):
        return np.asarray(ri, F32) - np.asarray(rj, F32)

    @staticmethod
    def shift(state, system):
        return state, system

    @staticmethod
    def apply(state, system):
        """``Domain.apply`` (``domains/__init__.py:123-189``): the base domain leaves
        state and system unchanged."""
        return state, system


@Domain.register("free")
@dataclass
class FreeDomain(Domain):
    @staticmethod
    def apply(state, system):
        """``FreeDomain.apply`` (``free.py:40-63``): box and anchor follow the
        particles' bounding box, reduced on the GPU."""
        from . import session

        return session.domain_apply(state, system)


@Domain.register("periodic")
@dataclass
class PeriodicDomain(Domain):
    @property
    def periodic(self) -> bool:
        return True

    @staticmethod
    def displacement(ri, rj, system):
        """Minimum image with true division (``periodic.py:37-71``)."""
        rij = np.asarray(ri, F32) - np.asarray(rj, F32)
        b = system.domain.box_size
        return (rij - b * np.round(rij / b)).astype(F32)

    @staticmethod
    def shift(state, system):
        """Wrap ``pos_c`` into the box (``periodic.py:82-116``)."""
        st = state.copy()
        b, a = system.domain.box_size, system.domain.anchor
        st.pos_c = (st.pos_c - b * np.floor((st.pos_c - a) / b)).astype(F32)
        return st, system


@Domain.register("reflect")
@dataclass
class ReflectDomain(Domain):
    restitution_coefficient: Any = 1.0

    @classmethod
    def Create(cls, dim: int, box_size=None, anchor=None, restitution_coefficient: float = 1.0, **kw: Any):
        """``ReflectDomain.Create`` (``reflect.py:42-97``)."""
        if not (0.0 < float(restitution_coefficient) <= 1.0):
            raise ValueError(f"restitution_coefficient must be in (0, 1], got {restitution_coefficient}.")
        return super().Create(dim, box_size=box_size, anchor=anchor,
                              restitution_coefficient=F32(restitution_coefficient), **kw)

    @staticmethod
    def apply(state, system):
        """``ReflectDomain.apply`` (``reflect.py:99-299``) for spheres on the GPU: wall
        impulses with the Verlet time-of-collision correction."""
        from . import session

        return session.domain_apply(state, system)
