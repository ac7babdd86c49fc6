"""Integrators (``jaxdem/integrators``) with the reference's stage interface.

Each registered type keeps its registry key and the static
``step_before_force(state, system)`` / ``step_after_force(state, system)``
methods of ``Integrator`` (``integrators/__init__.py:51-91``), so code that
runs the reference's stage order through the split factory types finds them.
The stages run on the GPU through ``jdem_integrate`` with the fused step
kernel's arithmetic: VelocityVerlet (``velocity_verlet.py:29-95``),
DirectEuler (``direct_euler.py:30-66``; its before-force stage is the base
no-op), VelocityVerletSpiral (``velocity_verlet_spiral.py:36-180``) and Spiral
(``spiral.py:56-144``; after-force only).  ``System.step`` does not go through
these methods: its fused kernels apply the same stages inside one step.  The
empty key is the no-op integrator (``integrators/__init__.py:148-149``).
"""

from __future__ import annotations

from dataclasses import dataclass

from .factory import Factory


class Integrator(Factory):
    """Base integrator: both stages leave the state unchanged."""

    KEY_LINEAR = ""
    KEY_ROTATION = ""

    @classmethod
    def _stage(cls, state, system, stage: int):
        if not cls.KEY_LINEAR and not cls.KEY_ROTATION:
            return state, system
        from . import session

        return session.integrate_stage(state, system, cls.KEY_LINEAR, cls.KEY_ROTATION, stage)

    @classmethod
    def step_before_force(cls, state, system):
        """Advance the state before the force evaluation (stage 0 of ``jdem_integrate``)."""
        return cls._stage(state, system, 0)

    @classmethod
    def step_after_force(cls, state, system):
        """Advance the state after the force evaluation (stage 1 of ``jdem_integrate``)."""
        return cls._stage(state, system, 1)

    @classmethod
    def initialize(cls, state, system):
        """``Integrator.initialize``: nothing to prepare for these methods."""
        return state, system


class LinearIntegrator(Integrator):
    pass


class RotationIntegrator(Integrator):
    pass


@dataclass
class _NoLinear(LinearIntegrator):
    pass


@dataclass
class _NoRotation(RotationIntegrator):
    pass


LinearIntegrator.register("")(_NoLinear)
RotationIntegrator.register("")(_NoRotation)


@LinearIntegrator.register("verlet")
@dataclass
class VelocityVerlet(LinearIntegrator):
    KEY_LINEAR = "verlet"


@LinearIntegrator.register("euler")
@dataclass
class DirectEuler(LinearIntegrator):
    KEY_LINEAR = "euler"


@RotationIntegrator.register("verletspiral")
@dataclass
class VelocityVerletSpiral(RotationIntegrator):
    KEY_ROTATION = "verletspiral"


@RotationIntegrator.register("spiral")
@dataclass
class Spiral(RotationIntegrator):
    KEY_ROTATION = "spiral"
