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


@Collider.register("NeighborList")
@dataclass
class NeighborList(Collider):
    """Verlet neighbour-list collider (``colliders/neighbor_list.py:134-``).

    Candidates within ``cutoff + skin`` are cached and rebuilt once the
    largest displacement since the last build exceeds ``skin / 2``
    (``neighbor_list.py:58-131``).  The device engine runs exactly this scheme
    for every collider, with a per-pair list cutoff ``r_i + r_j + skin``, so
    this type selects the same device path with the caller's skin and initial
    list capacity.  The list lives on the device; ``create_neighbor_list``
    returns the reference's padded ``(N, max_neighbors)`` form.

    Spheres interact within ``r_i + r_j``, so the reference misses contacts
    when ``cutoff`` is below ``2 max(rad)``; the device list never misses a
    contact and such a cutoff is rejected rather than silently changing the
    force.
    """

    cutoff: Any = None
    skin: Any = None
    max_neighbors: Any = None
    secondary_collider_type: str = "CellList"

    @classmethod
    def Create(cls, state, cutoff: float, skin: Optional[float] = None, skin_fraction: Optional[float] = None,
               max_neighbors: Optional[int] = None, number_density: float = 1.0, safety_factor: float = 1.2,
               secondary_collider_type: str = "CellList", secondary_collider_kw: Optional[dict] = None):
        """``NeighborList.Create`` (``neighbor_list.py:287-440``): absolute ``skin`` or
        ``skin_fraction`` of the cutoff (default 0.05), and the neighbour-count estimate
        ``ceil(safety_factor * V(cutoff + skin) * density)`` when ``max_neighbors`` is
        not given."""
        if skin is not None and skin_fraction is not None:
            raise ValueError("Pass either `skin` (absolute distance) or `skin_fraction` "
                             "(fraction of the cutoff), not both.")
        cutoff = float(cutoff)
        skin_val = float(skin) if skin is not None else float(0.05 if skin_fraction is None else skin_fraction) * cutoff
        rad = np.asarray(state._rad, F32)
        rmax = float(rad.max()) if rad.size else 0.0
        if F32(cutoff) < F32(2.0) * F32(rmax):  # float32, as the state's radii
            raise NotImplementedError(
                f"NeighborList cutoff {cutoff:g} is below the largest contact distance {2 * rmax:g}: the "
                "reference would miss those contacts, the GB300 list does not")
        if max_neighbors is None:
            list_cutoff = cutoff + skin_val
            pos = np.asarray(state.pos, np.float64).reshape(-1, state.dim)
            if pos.size:
                ext = np.maximum(pos.max(axis=0) - pos.min(axis=0) + 2.0 * rmax, 1.0)
                density = max(float(number_density), pos.shape[0] / float(np.prod(ext)))
            else:
                density = float(number_density)
            vol = np.pi * list_cutoff ** state.dim * (1.0 if state.dim == 2 else 4.0 / 3.0)
            max_neighbors = max(1, int(np.ceil(safety_factor * vol * density)))
        return cls(cutoff=F32(cutoff), skin=F32(skin_val), max_neighbors=int(max_neighbors),
                   secondary_collider_type=str(secondary_collider_type))

    @staticmethod
    def compute_force(state, system):
        """``neighbor_list.py:594-672`` on the GPU (rebuild when due, then the list sum)."""
        from . import session

        return session.compute_force(state, system)

    @staticmethod
    def compute_potential_energy(state, system):
        """``neighbor_list.py:674-734`` on the GPU; returns ``(state, system, energy)``."""
        from . import session

        e = session.energies(state, system)
        pe = e[..., 0]
        return state, system, (F32(pe) if np.ndim(pe) == 0 else pe.astype(F32))

    @staticmethod
    def create_neighbor_list(state, system, cutoff: float, max_neighbors: int):
        """``neighbor_list.py:485-543`` on the GPU: ``(state, system, nl, overflow)``."""
        from . import session

        nl, ovf = session.neighbor_list(state, system, cutoff, max_neighbors)
        return state, system, nl, ovf
