"""Colliders (``jaxdem/colliders``): contact detection + pair forces on the GPU.

``DynamicCellList`` keeps the reference's construction rule
(``cell_list.py:374-432``) for ``cell_size`` and ``neighbor_mask`` (used by
``create_neighbor_list``) and adds one GB300 knob, ``skin``: the engine bins
particles into cells of edge ``2 max(rad) + skin`` and re-sorts only when the
accumulated displacement exceeds ``skin / 2``.  The contact set, and hence
the force on every particle, does not depend on the binning; only the
floating-point summation order does.

``naive`` (``colliders/naive.py``) is accepted as a key and runs the same
device path: the all-pairs sum and the cell-list sum contain the same nonzero
terms.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Optional

import numpy as np

from .factory import Factory

F32 = np.float32


@dataclass
class Collider(Factory):
    overflow: bool = field(default=False, kw_only=True)

    @staticmethod
    def compute_force(state, system):
        """No-op collider (``colliders/__init__.py:218-222``): zero force and torque."""
        st = state.copy()
        st.force = np.zeros_like(st.force)
        st.torque = np.zeros_like(st.torque)
        return st, system

    @staticmethod
    def compute_potential_energy(state, system):
        return state, system, F32(0.0)

    @staticmethod
    def create_neighbor_list(state, system, cutoff: float, max_neighbors: int):
        n = state.N
        return state, system, np.full((n, max_neighbors), -1, np.int64), False


Collider.register("")(Collider)


def _default_cell(rad: np.ndarray) -> F32:
    rmin, rmax = F32(np.min(rad)), F32(np.max(rad))
    alpha = rmax / rmin
    return F32(2.0) * rmax if alpha < 2.5 else F32(0.5) * rmax


@Collider.register("CellList")
@dataclass
class DynamicCellList(Collider):
    neighbor_mask: np.ndarray = None
    cell_size: Any = None
    skin: Any = None

    @classmethod
    def Create(cls, state, cell_size=None, search_range=None, box_size=None, skin: Optional[float] = None):
        """``DynamicCellList.Create`` (``cell_list.py:374-432``) plus the binning ``skin``."""
        rad = np.asarray(state._rad, F32)
        max_rad = F32(np.max(rad)) if rad.size else F32(1.0)
        if cell_size is None:
            cell_size = _default_cell(rad) if rad.size else F32(2.0)
        cell_size = F32(cell_size)
        if box_size is not None:
            box = np.asarray(box_size, F32)
            for _ in range(2):
                sr = max(1, int(np.ceil(F32(2) * max_rad / cell_size))) if search_range is None else int(search_range)
                g = np.maximum(np.floor(box / cell_size).astype(np.int64), 2 * sr + 1)
                cell_size = F32(np.min(box / g.astype(F32)))
        if search_range is None:
            search_range = max(1, int(np.ceil(F32(2) * max_rad / cell_size)))
        r = np.arange(-int(search_range), int(search_range) + 1)
        mesh = np.meshgrid(*([r] * state.dim), indexing="ij")
        mask = np.stack([m.ravel() for m in mesh], axis=1).astype(np.int32)
        if skin is None:
            from .autotune import default_skin

            skin = default_skin(float(max_rad))
        return cls(neighbor_mask=mask, cell_size=F32(cell_size), skin=F32(skin))

    @property
    def search_range(self) -> int:
        return max(int(np.max(self.neighbor_mask)), 1)

    @staticmethod
    def compute_force(state, system):
        """``DynamicCellList.compute_force`` (``cell_list.py:434-464``) on the GPU."""
        from . import session

        return session.compute_force(state, system)

    @staticmethod
    def compute_potential_energy(state, system):
        """``cell_list.py:466-496`` on the GPU; returns ``(state, system, energy)``."""
        from . import session

        e = session.energies(state, system)
        pe = e[..., 0]
        return state, system, (F32(pe) if np.ndim(pe) == 0 else pe.astype(F32))

    @staticmethod
    def create_neighbor_list(state, system, cutoff: float, max_neighbors: int):
        """``cell_list.py:498-595`` on the GPU: ``(state, system, nl, overflow)``."""
        from . import session

        nl, ovf = session.neighbor_list(state, system, cutoff, max_neighbors)
        return state, system, nl, ovf


Collider.register("CellListGB300")(DynamicCellList)


@Collider.register("naive")
@dataclass
class NaiveSimulator(Collider):
    skin: Any = None

    @classmethod
    def Create(cls, skin: Optional[float] = None):
        return cls(skin=skin)

    @staticmethod
    def compute_force(state, system):
        from . import session

        return session.compute_force(state, system)

    @staticmethod
    def compute_potential_energy(state, system):
        from . import session

        e = session.energies(state, system)
        pe = e[..., 0]
        return state, system, (F32(pe) if np.ndim(pe) == 0 else pe.astype(F32))
