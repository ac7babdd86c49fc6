"""Integrators (``jaxdem/integrators``): identities of the update rules.

The device kernels apply them: VelocityVerlet (``velocity_verlet.py:29-95``),
DirectEuler (``direct_euler.py:30-66``), VelocityVerletSpiral
(``velocity_verlet_spiral.py:36-180``), Spiral (``spiral.py``); the empty key
is the no-op integrator (``integrators/__init__.py:148-149``).
"""

from __future__ import annotations

from dataclasses import dataclass

from .factory import Factory


class Integrator(Factory):
    pass


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
    pass


@LinearIntegrator.register("euler")
@dataclass
class DirectEuler(LinearIntegrator):
    pass


@RotationIntegrator.register("verletspiral")
@dataclass
class VelocityVerletSpiral(RotationIntegrator):
    pass


@RotationIntegrator.register("spiral")
@dataclass
class Spiral(RotationIntegrator):
    pass
