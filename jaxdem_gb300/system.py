"""``System``: configuration of a simulation and the stepping entry points.

Mirrors ``jaxdem/system.py``: ``System.create`` (``:228-604``) assembles the
components from registry keys or instances, ``System.step`` (``:701-748``)
advances ``n`` steps and ``System.trajectory_rollout`` (``:606-699``)
collects one ``save_fn`` output per frame after its steps.  Stepping runs the
fused GB300 engine through the C ABI; an unsupported configuration raises
``NotImplementedError`` (there is no CPU fallback).
"""

from __future__ import annotations

import dataclasses
import inspect
from dataclasses import dataclass, field
from typing import Any, Callable, Optional, Sequence

import numpy as np

from .colliders import Collider
from .domains import Domain
from .factory import _normalize_key
from .forces import ForceManager, ForceModel
from .integrators import LinearIntegrator, RotationIntegrator
from .materials import Material, MaterialTable

F32 = np.float32


def _save_state_system(state, system):
    return state, system


def _check_material_table(mat_table: MaterialTable, required: Sequence[str]) -> None:
    """``_check_material_table`` (``system.py:27-52``)."""
    missing = [k for k in required if k not in mat_table.props and k not in mat_table.pair]
    if missing:
        raise KeyError(f"MaterialTable lacks fields {missing}, required by the selected force model.")


@dataclass
class System:
    linear_integrator: LinearIntegrator
    rotation_integrator: RotationIntegrator
    collider: Collider
    domain: Domain
    force_manager: ForceManager
    bonded_force_model: Any
    force_model: ForceModel
    mat_table: MaterialTable
    dt: Any
    time: Any
    dim: Any
    step_count: Any
    key: Any
    interact_same_bond_id: Any
    user_pre_step_actions: Callable = field(default=_save_state_system)
    user_post_step_actions: Callable = field(default=_save_state_system)

    @staticmethod
    def create(state_shape: Optional[Sequence[int]] = None, *, state=None, dt: float = 0.005, time: float = 0.0,
               linear_integrator_type: Optional[str] = "verlet", rotation_integrator_type: Optional[str] = "verletspiral",
               collider_type: str = "naive", domain_type: str = "free", bonded_force_model_type: Optional[str] = None,
               bonded_force_model_kw: Optional[dict] = None, bonded_force_model: Any = None,
               force_model_type: str = "spring", force_manager_kw: Optional[dict] = None,
               mat_table: Optional[MaterialTable] = None, linear_integrator=None, rotation_integrator=None,
               collider=None, domain=None, force_model=None, force_manager=None,
               linear_integrator_kw: Optional[dict] = None, rotation_integrator_kw: Optional[dict] = None,
               collider_kw: Optional[dict] = None, domain_kw: Optional[dict] = None,
               force_model_kw: Optional[dict] = None, seed: int = 0, key: Any = None,
               interact_same_bond_id: bool = False, user_pre_step_actions: Optional[Callable] = None,
               user_post_step_actions: Optional[Callable] = None, **unused: Any) -> "System":
        """``System.create`` (``system.py:228-604``)."""
        if state is not None:
            if state_shape is not None and tuple(state_shape) != tuple(state.shape):
                raise ValueError(f"state_shape {tuple(state_shape)} does not match the shape "
                                 f"of the provided state {tuple(state.shape)}.")
            state_shape = tuple(state.shape)
        if state_shape is None:
            raise TypeError("System.create requires either `state_shape` or `state`.")
        dim = int(state_shape[-1])
        linear_integrator_type = "" if linear_integrator_type is None else linear_integrator_type
        rotation_integrator_type = "" if rotation_integrator_type is None else rotation_integrator_type
        collider_kw = {} if collider_kw is None else dict(collider_kw)
        domain_kw = {} if domain_kw is None else dict(domain_kw)
        force_manager_kw = {"gravity": None, "force_functions": ()} if force_manager_kw is None \
            else dict(force_manager_kw)
        if mat_table is None:
            mat_table = MaterialTable.from_materials(
                [Material.create("elastic", density=0.27, young=1.0e4, poisson=0.3)])
        if force_model is None:
            force_model = ForceModel.create(force_model_type, **(force_model_kw or {}))
        _check_material_table(mat_table, force_model.required_material_properties)
        if bonded_force_model is None and bonded_force_model_type is not None:
            raise NotImplementedError("bonded force models are outside the GB300 hot path")
        if force_manager is None:
            force_manager = ForceManager.create(tuple(state_shape), **force_manager_kw)
        if collider is None:
            if state is not None and "state" not in collider_kw:
                sub = Collider._registry.get(_normalize_key(collider_type))
                create_fn = getattr(sub, "Create", None)
                if create_fn is not None and "state" in inspect.signature(create_fn).parameters:
                    collider_kw["state"] = state
            collider = Collider.create(collider_type, **collider_kw)
        if linear_integrator is None:
            linear_integrator = LinearIntegrator.create(linear_integrator_type, **(linear_integrator_kw or {}))
        if rotation_integrator is None:
            rotation_integrator = RotationIntegrator.create(rotation_integrator_type, **(rotation_integrator_kw or {}))
        if domain is None:
            domain = Domain.create(domain_type, dim=dim, **domain_kw)
        return System(
            linear_integrator=linear_integrator, rotation_integrator=rotation_integrator, collider=collider,
            domain=domain, force_manager=force_manager, bonded_force_model=bonded_force_model,
            force_model=force_model, mat_table=mat_table, dim=np.int32(dim), dt=F32(dt), time=F32(time),
            step_count=np.int32(0), key=key if key is not None else np.array([0, seed], np.uint32),
            interact_same_bond_id=bool(interact_same_bond_id),
            user_pre_step_actions=user_pre_step_actions or _save_state_system,
            user_post_step_actions=user_post_step_actions or _save_state_system)

    # ---------------------------------------------------------------- step
    @staticmethod
    def step(state, system: "System", *, n: int = 1):
        """Advance ``n`` steps (``system.py:701-748``) on the GB300 engine."""
        from . import session

        return session.step(state, system, int(n))

    @staticmethod
    def trajectory_rollout(state, system: "System", *, n: Optional[int] = None, stride: int = 1,
                           strides=None, save_fn: Callable = _save_state_system, unroll: int = 2):
        """Frames saved after their steps (``system.py:606-699``); a stride of 0 saves the current state."""
        from . import session

        stride = int(stride)
        if strides is not None:
            strides = np.asarray(strides, np.int64)
            if strides.ndim != 1:
                raise ValueError("`strides` must be a 1D array.")
        elif n is None:
            raise ValueError("`n` must be provided when `strides` is None.")
        else:
            strides = np.full(int(n), stride, np.int64)
        return session.rollout(state, system, strides, save_fn)

    @staticmethod
    def stack(systems: Sequence["System"]) -> "System":
        """Stack along a new leading axis (``system.py:750-``)."""
        return _tree_stack(systems)


def _tree_stack(items):
    first = items[0]
    if isinstance(first, np.ndarray) or np.isscalar(first) or isinstance(first, (np.generic, float, int, bool)):
        return np.stack([np.asarray(x) for x in items])
    if dataclasses.is_dataclass(first):
        kw = {}
        for f in dataclasses.fields(first):
            vals = [getattr(x, f.name) for x in items]
            v0 = vals[0]
            if callable(v0) and not dataclasses.is_dataclass(v0):
                kw[f.name] = v0
            elif v0 is None or isinstance(v0, (str, tuple, dict)):
                kw[f.name] = v0
            else:
                kw[f.name] = _tree_stack(vals)
        return dataclasses.replace(first, **kw)
    return first
