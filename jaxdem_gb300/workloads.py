"""Seeded synthetic inputs with the shapes and distributions of the five
benchmark configurations (the reference publishes no dataset; these stand in).

All arrays are float32 and generated with ``numpy.random.Generator(PCG64(seed))``.
Masses are ``density * volume`` with density 1 (``State.create`` with a
``MaterialTable``, ``state.py:807-809``); the spring stiffness is k = 1e3
(harmonic matcher of a single material gives ``young_eff = young``).

=====  ===================================================================
name   recipe
=====  ===================================================================
c1     3D, N = 4096, r = 0.5, periodic cube at packing fraction 0.40,
       uniform positions, v ~ N(0, 0.1^2), dt = 1e-3, 1000 steps
c2     3D, N = 2^20, r in {0.5, 0.7} 50/50, periodic cube at 0.55,
       uniform positions + jitter, v ~ N(0, 0.05^2), dt = 5e-4, 200 steps
c3     2D, N = 2^22, r ~ U[0.4, 0.6], reflecting square at area fraction
       0.70, gravity (0, -1), v = 0, dt = 5e-4, 500 steps
c4     4096 independent 3D periodic systems, N ~ logU[64, 16384],
       packing fraction ~ U[0.30, 0.60], r in {0.5, 0.7}, v ~ N(0, 0.1^2),
       dt = 1e-3, 1000 steps in 50-step chunks
c5     20000 rollout requests, Poisson arrivals at 200/s, N ~ logU[256,
       262144], dim 2 or 3, fraction ~ U[0.3, 0.6], r ~ U[0.4, 0.6],
       steps ~ U{100..10000}, periodic
=====  ===================================================================
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

F32 = np.float32
K_SPRING = 1.0e3
DENSITY = 1.0


def volume(rad: np.ndarray, dim: int) -> np.ndarray:
    rad = np.asarray(rad, F32)
    if dim == 2:
        return (F32(np.pi) * rad * rad).astype(F32)
    return (F32(4.0 / 3.0) * F32(np.pi) * rad * rad * rad).astype(F32)


@dataclass
class Workload:
    """One system: arrays in the reference layout plus its System parameters."""

    name: str
    dim: int
    pos: np.ndarray
    vel: np.ndarray
    rad: np.ndarray
    mass: np.ndarray
    domain: str
    box_size: np.ndarray
    anchor: np.ndarray
    dt: float
    steps: int
    gravity: np.ndarray
    restitution: float = 1.0
    young: float = K_SPRING

    @property
    def N(self) -> int:
        return int(self.pos.shape[0])

    def desc(self, cell_size: Optional[float] = None, search_range: int = 1) -> dict:
        rmax = float(self.rad.max()) if self.N else 0.5
        return dict(n=self.N, domain=self.domain, linear="verlet", rotation="", dt=self.dt,
                    box_size=self.box_size, anchor=self.anchor, restitution=self.restitution,
                    gravity=self.gravity, cell_size=2.0 * rmax if cell_size is None else cell_size,
                    search_range=search_range)


def _periodic_box(rad: np.ndarray, dim: int, phi: float) -> float:
    return float((volume(rad, dim).astype(np.float64).sum() / phi) ** (1.0 / dim))


def periodic_system(name: str, rng: np.random.Generator, N: int, dim: int, rad: np.ndarray, phi: float,
                    vel_sigma: float, dt: float, steps: int, jitter: float = 0.0) -> Workload:
    L = _periodic_box(rad, dim, phi)
    pos = rng.uniform(0.0, L, size=(N, dim))
    if jitter > 0:
        pos = pos + rng.uniform(-jitter, jitter, size=(N, dim))
        pos = np.mod(pos, L)
    vel = rng.normal(0.0, vel_sigma, size=(N, dim)) if vel_sigma > 0 else np.zeros((N, dim))
    rad = rad.astype(F32)
    return Workload(name=name, dim=dim, pos=pos.astype(F32), vel=vel.astype(F32), rad=rad,
                    mass=(F32(DENSITY) * volume(rad, dim)).astype(F32), domain="periodic",
                    box_size=np.full(dim, L, F32), anchor=np.zeros(dim, F32), dt=dt, steps=steps,
                    gravity=np.zeros(dim, F32))


def c1(N: int = 4096, seed: int = 1) -> Workload:
    rng = np.random.Generator(np.random.PCG64(seed))
    rad = np.full(N, 0.5)
    return periodic_system("c1", rng, N, 3, rad, 0.40, 0.1, 1e-3, 1000)


def _bidisperse(rng, N):
    rad = np.where(np.arange(N) < N // 2, 0.5, 0.7)
    rng.shuffle(rad)
    return rad


def c2(N: int = 1 << 20, seed: int = 2) -> Workload:
    rng = np.random.Generator(np.random.PCG64(seed))
    rad = _bidisperse(rng, N)
    # jitter of 1e-3 of the reference cell edge 2 * 0.7
    return periodic_system("c2", rng, N, 3, rad, 0.55, 0.05, 5e-4, 200, jitter=1e-3 * 1.4)


def c3(N: int = 1 << 22, seed: int = 3) -> Workload:
    rng = np.random.Generator(np.random.PCG64(seed))
    rad = rng.uniform(0.4, 0.6, size=N).astype(F32)
    L = _periodic_box(rad, 2, 0.70)
    pos = rng.uniform(0.0, 1.0, size=(N, 2)) * (L - 2 * rad[:, None]) + rad[:, None]
    return Workload(name="c3", dim=2, pos=pos.astype(F32), vel=np.zeros((N, 2), F32), rad=rad,
                    mass=(F32(DENSITY) * volume(rad, 2)).astype(F32), domain="reflect",
                    box_size=np.full(2, L, F32), anchor=np.zeros(2, F32), dt=5e-4, steps=500,
                    gravity=np.array([0.0, -1.0], F32), restitution=1.0)


def c4(n_systems: int = 4096, seed: int = 4, n_min: int = 64, n_max: int = 16384) -> list:
    rng = np.random.Generator(np.random.PCG64(seed))
    ns = np.round(np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=n_systems))).astype(np.int64)
    phis = rng.uniform(0.30, 0.60, size=n_systems)
    out = []
    for s in range(n_systems):
        rad = _bidisperse(rng, int(ns[s]))
        out.append(periodic_system(f"c4_{s}", rng, int(ns[s]), 3, rad, float(phis[s]), 0.1, 1e-3, 1000))
    return out


@dataclass
class Request:
    rid: int
    arrival: float
    N: int
    dim: int
    phi: float
    steps: int
    seed: int

    def workload(self) -> Workload:
        rng = np.random.Generator(np.random.PCG64(self.seed))
        rad = rng.uniform(0.4, 0.6, size=self.N)
        return periodic_system(f"req{self.rid}", rng, self.N, self.dim, rad, self.phi, 0.1, 1e-3, self.steps)


def c5(n_requests: int = 20000, rate: float = 200.0, seed: int = 5, n_min: int = 256, n_max: int = 262144,
       steps_min: int = 100, steps_max: int = 10000) -> list:
    rng = np.random.Generator(np.random.PCG64(seed))
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    arr = np.cumsum(gaps) - gaps[0]
    Ns = np.round(np.exp(rng.uniform(np.log(n_min), np.log(n_max), size=n_requests))).astype(np.int64)
    dims = rng.integers(2, 4, size=n_requests)
    phis = rng.uniform(0.3, 0.6, size=n_requests)
    steps = rng.integers(steps_min, steps_max + 1, size=n_requests)
    seeds = rng.integers(0, 2**31 - 1, size=n_requests)
    return [Request(rid=i, arrival=float(arr[i]), N=int(Ns[i]), dim=int(dims[i]), phi=float(phis[i]),
                    steps=int(steps[i]), seed=int(seeds[i])) for i in range(n_requests)]
