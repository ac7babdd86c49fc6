"""Stream-ordered use of the C ABI (jdem_set_stream), as an XLA FFI handler drives it.

The reference's System.step (system.py:701-748) is a functional XLA computation: its
inputs are produced and its outputs consumed by other work on XLA's compute stream,
with no host synchronisation in between.  Here torch plays that role: a kernel on a
side stream is still busy (a long sleep) when the positions are written and the engine
is called on the same stream; the engine's output is consumed by another torch kernel
on that stream, and only then does the host wait.  The results must equal, bit for bit,
the same upload / steps / download done with host synchronisation in between.
"""

from __future__ import annotations

import numpy as np
import pytest

from jaxdem_gb300 import workloads as W
from jaxdem_gb300._lib import Engine

pytestmark = pytest.mark.gpu

K = np.array([[W.K_SPRING]], np.float32)


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _synchronised(w, steps):
    eng = Engine(w.dim, [w.desc()], K, skin=0.3)
    try:
        eng.upload(pos=w.pos, rad=w.rad, mass=w.mass, vel=w.vel)
        eng.step(steps)
        return eng.download()
    finally:
        eng.close()


@pytest.mark.parametrize("dim", [3, 2])
def test_caller_stream_ordering_matches_synchronised_path(dim):
    torch = pytest.importorskip("torch")
    w = W.c1(N=6000, seed=21) if dim == 3 else W.c3(N=6000, seed=22)
    steps = 37
    want = _synchronised(w, steps)

    dev = torch.device("cuda:0")
    side = torch.cuda.Stream(device=dev)
    pos_src = torch.from_numpy(w.pos).pin_memory()
    eng = Engine(w.dim, [w.desc()], K, skin=0.3)
    try:
        with torch.cuda.stream(side):
            pos = torch.zeros((w.N, w.dim), dtype=torch.float32, device=dev)
            vel = torch.from_numpy(w.vel).to(dev, non_blocking=True)
            rad = torch.from_numpy(w.rad).to(dev, non_blocking=True)
            mass = torch.from_numpy(w.mass).to(dev, non_blocking=True)
            out_pos = torch.full_like(pos, float("nan"))
            out_vel = torch.full_like(pos, float("nan"))
            out_frc = torch.full_like(pos, float("nan"))
            torch.cuda._sleep(200_000_000)  # ~0.1 s of GPU time ahead of the positions' producer
            pos.copy_(pos_src, non_blocking=True)  # the producer: still queued when the engine is called
            eng.set_stream(side.cuda_stream)
            assert eng.stream() == side.cuda_stream
            eng.upload_device(pos_c=pos, vel=vel, rad=rad, mass=mass)
            eng.step_async(steps)
            eng.download_device(wait=False, pos_c=out_pos, vel=out_vel, force=out_frc)
            # the consumer, queued on the same stream without any host wait
            got_pos = out_pos.clone()
            got_vel = out_vel.clone()
            got_frc = out_frc.clone()
        side.synchronize()
        eng.sync()
        eng.set_stream(0)
        assert eng.stream() != side.cuda_stream
        # the handle keeps working on its own stream afterwards
        eng.step(3)
    finally:
        eng.close()
    assert np.array_equal(got_pos.cpu().numpy(), want["pos_c"])
    assert np.array_equal(got_vel.cpu().numpy(), want["vel"])
    assert np.array_equal(got_frc.cpu().numpy(), want["force"])
