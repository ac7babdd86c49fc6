"""Shared helpers for the parity tests: oracle systems and error metrics."""

from __future__ import annotations

import numpy as np

from oracle import dem_ref as R

F32 = np.float32


def force_err(gpu, ref):
    """max_i |F_gpu - F_ref| / max(|F_ref|, 1e-3 rms|F_ref|) with float64 norms."""
    ref = np.asarray(ref, np.float64)
    gpu = np.asarray(gpu, np.float64)
    na = np.linalg.norm(ref, axis=-1)
    rms = np.sqrt(np.mean(na ** 2)) if na.size else 0.0
    floor = max(1e-3 * rms, 1e-30)
    return float((np.linalg.norm(gpu - ref, axis=-1) / np.maximum(na, floor)).max()) if na.size else 0.0


def global_force_err(gpu, ref):
    """||F_gpu - F_ref||_2 / ||F_ref||_2 over all particles, float64 norms (0 without forces).
    The per-particle floored bar of force_err implies the same bar here."""
    ref = np.asarray(ref, np.float64)
    gpu = np.asarray(gpu, np.float64)
    nr = np.linalg.norm(ref)
    return float(np.linalg.norm(gpu - ref) / nr) if nr > 0 else 0.0


def min_image_diff(a, b, box=None):
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    if box is not None:
        box = np.asarray(box, np.float64)
        d = d - box * np.round(d / box)
    return np.abs(d).max() if d.size else 0.0


def osystem(w, domain=None, cell_size=None, search_range=None, young=None, linear="verlet", rotation="",
            gravity=None):
    dim = w.dim
    cell, mask = R.cell_list_create(w.rad, dim, cell_size=cell_size, search_range=search_range)
    return R.OSystem(dim=dim, domain=domain or w.domain, box_size=np.asarray(w.box_size, F32).copy(),
                     anchor=np.asarray(w.anchor, F32).copy(),
                     young_eff=np.array([[1e3]], F32) if young is None else np.asarray(young, F32),
                     dt=F32(w.dt), cell_size=cell, neighbor_mask=mask,
                     gravity=np.asarray(w.gravity if gravity is None else gravity, F32),
                     restitution=F32(w.restitution), linear=linear, rotation=rotation)


def ostate(w, **kw):
    return R.make_state(w.pos, vel=w.vel, rad=w.rad, mass=w.mass, **kw)
