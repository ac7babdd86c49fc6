"""Force model and force manager (``jaxdem/forces``).

``SpringForce`` (``forces/spring.py:69-147``), ``HertzianForce``
(``forces/hertz.py:22-170``) and ``CundallStrackForce``
(``forces/cundall_strack.py:22-242``) are evaluated on the device by the
collider kernels; these classes carry their identity and material
requirements.  ``ForceManager`` (``forces/force_manager.py``) carries gravity
and the per-step external buffers; the device applies gravity
(``force_manager.py:393-397``) inside the fused step kernel.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Sequence

import numpy as np

from .factory import Factory

F32 = np.float32


class ForceModel(Factory):
    @property
    def required_material_properties(self) -> tuple:
        return ()

    @property
    def requires_history(self) -> bool:
        return False


@ForceModel.register("spring")
@dataclass
class SpringForce(ForceModel):
    """Linear normal spring: F = k max(0, Ri + Rj - r) r_hat, E = k delta^2 / 2."""

    @property
    def required_material_properties(self) -> tuple:
        return ("young_eff",)


@ForceModel.register("hertz")
@dataclass
class HertzianForce(ForceModel):
    """Hertz normal contact (``forces/hertz.py:22-170``): F = k delta^(3/2) n,
    E = 0.4 k delta^(5/2), k = (4/3) E* sqrt(R*), R* = Ri Rj / (Ri + Rj), with E*
    from the per-material ``young`` and ``poisson`` (no matchmaker)."""

    @property
    def required_material_properties(self) -> tuple:
        return ("young", "poisson")


def hertz_pair_constant(young, poisson) -> np.ndarray:
    """(M, M) float32 table of (4/3) E*, in the reference's float32 order
    (``hertz.py:99-105``): E* = 1 / ((1 - nu_i**2) / E_i + (1 - nu_j**2) / E_j),
    then (4/3) * E*.  The device multiplies it by sqrt(R*) per pair."""
    E = np.asarray(young, F32).reshape(-1)
    nu = np.asarray(poisson, F32).reshape(-1)
    a = (F32(1.0) - nu * nu) / E
    with np.errstate(divide="ignore"):
        e_star = (F32(1.0) / (a[:, None] + a[None, :])).astype(F32)
    return (F32(4.0 / 3.0) * e_star).astype(F32)


@ForceModel.register("cundallstrack")
@dataclass
class CundallStrackForce(ForceModel):
    """Stateless Cundall-Strack spring-dashpot (``forces/cundall_strack.py:22-242``):
    normal spring kn delta with viscous damping (strictly repulsive), tangential
    dashpot capped by Coulomb friction, rolling-friction torque; per-material
    ``young``, ``poisson``, ``e``, ``mu`` and ``mu_r``."""

    @property
    def required_material_properties(self) -> tuple:
        return ("young", "poisson", "e", "mu", "mu_r")


def cundall_strack_tables(young, poisson, e, mu, mu_r) -> tuple:
    """Per-material-pair damping ratio beta (M, M) and per-material
    (young, shear modulus, mu, mu_r) (M, 4), float32 in the reference's order
    (``cundall_strack.py:128-150``): G = E / (2 (1 + nu)); e_eff = min(e_i, e_j);
    beta = -ln(e_eff) / sqrt(pi**2 + ln(e_eff)**2), 1 where e_eff = 0."""
    E = np.asarray(young, F32).reshape(-1)
    nu = np.asarray(poisson, F32).reshape(-1)
    G = (E / (F32(2.0) * (F32(1.0) + nu))).astype(F32)
    ee = np.asarray(e, F32).reshape(-1)
    e_eff = np.minimum(ee[:, None], ee[None, :])
    e_safe = np.where(e_eff > 0, e_eff, F32(1.0)).astype(F32)
    ln_e = np.log(e_safe).astype(F32)
    beta = np.where(e_eff > 0, -ln_e / np.sqrt(F32(np.pi ** 2) + ln_e * ln_e), F32(1.0)).astype(F32)
    props = np.stack([E, G, np.asarray(mu, F32).reshape(-1), np.asarray(mu_r, F32).reshape(-1)], 1)
    return beta, np.ascontiguousarray(props, F32)


@dataclass
class ForceManager:
    gravity: np.ndarray
    external_force: np.ndarray
    external_force_com: np.ndarray
    external_torque: np.ndarray
    force_functions: tuple = ()
    energy_functions: tuple = ()
    is_com_force: tuple = ()

    @staticmethod
    def create(state_shape: Sequence[int], *, gravity=None, force_functions: Sequence[Any] = ()) -> "ForceManager":
        """``ForceManager.create`` (``force_manager.py:80-190``)."""
        dim = state_shape[-1]
        g = np.zeros(dim, F32) if gravity is None else np.asarray(gravity, F32)
        ad = 1 if dim == 2 else 3
        funcs = tuple(f if isinstance(f, (tuple, list)) else (f,) for f in force_functions)
        return ForceManager(gravity=g, external_force=np.zeros(tuple(state_shape), F32),
                            external_force_com=np.zeros(tuple(state_shape), F32),
                            external_torque=np.zeros((*tuple(state_shape)[:-1], ad), F32),
                            force_functions=tuple(f[0] for f in funcs),
                            energy_functions=tuple(f[1] if len(f) > 1 and callable(f[1]) else None for f in funcs),
                            is_com_force=tuple(bool(f[-1]) if isinstance(f[-1], bool) else False for f in funcs))

    @staticmethod
    def apply(state, system):
        """``ForceManager.apply`` (``force_manager.py:338-425``) for spheres on the GPU:
        external forces and gravity join the contact force; the returned system's external
        buffers are cleared."""
        from . import session

        return session.force_manager_apply(state, system)

    @staticmethod
    def add_force(state, system, force, *, is_com: bool = False):
        """Accumulate a one-step external force (``force_manager.py:192-``)."""
        fm = system.force_manager
        if is_com:
            fm.external_force_com = (fm.external_force_com + np.asarray(force, F32)).astype(F32)
        else:
            fm.external_force = (fm.external_force + np.asarray(force, F32)).astype(F32)
        return system
