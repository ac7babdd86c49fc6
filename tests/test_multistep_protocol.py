"""The grid-barrier protocol of the many-step kernel (jaxdem_gb300/csrc/jdem_multi.cu,
grid_barrier_max and k_multi), checked as a model on the CPU.

Each block, at step s: folds its largest squared drift into slot mx[s % 3]
(atomic max), arrives with one add on a never-reset count, waits until the
count reaches its target (the launch's base plus one grid per barrier), reads
slot s % 3; block 0 then zeroes slot (s + 2) % 3.  A launch starts from the
base and step index the previous launch's block 0 stored, and launches do not
overlap.  Random interleavings of the blocks' memory operations must give
every block the true maximum of every step, across launches of random
lengths.  A protocol that zeroes slot (s + 1) % 3 instead is caught, which
shows the interleavings reach the races that matter.
"""

from __future__ import annotations

import numpy as np


def run_model(n_blocks, launches, rng, zero_ahead=2):
    """Interleave the blocks of each launch at random; return the number of steps at
    which some block read a maximum other than the true one."""
    mem = {"count": 0, "base": 0, "mstep": 0, "mx": [0, 0, 0]}
    bad = 0
    step0 = 0
    for n_steps in launches:
        drift = rng.integers(1, 1 << 20, size=(n_steps, n_blocks))  # float bits stand-ins

        def block(b):
            nonlocal bad
            target = mem["base"]
            s = mem["mstep"]
            k = 0
            while True:
                slot = s % 3
                mem["mx"][slot] = max(mem["mx"][slot], int(drift[k, b]))
                yield
                mem["count"] += 1
                yield
                target += n_blocks
                while mem["count"] < target:
                    yield
                m2 = mem["mx"][slot]
                yield
                if m2 != int(drift[k].max()):
                    bad += 1
                if b == 0:
                    mem["mx"][(s + zero_ahead) % 3] = 0
                    yield
                s += 1
                k += 1
                if k == n_steps:
                    break
            if b == 0:
                mem["base"] = target
                mem["mstep"] = s

        live = {b: block(b) for b in range(n_blocks)}
        while live:
            b = list(live)[rng.integers(len(live))]
            try:
                next(live[b])
            except StopIteration:
                del live[b]
        step0 += n_steps
    assert mem["count"] == n_blocks * step0
    return bad


def test_every_block_reads_each_steps_maximum():
    rng = np.random.default_rng(2024)
    for _ in range(200):
        n_blocks = int(rng.integers(1, 6))
        launches = [int(x) for x in rng.integers(1, 6, size=int(rng.integers(1, 5)))]
        assert run_model(n_blocks, launches, rng) == 0


def test_zeroing_the_next_slot_is_caught():
    rng = np.random.default_rng(7)
    caught = sum(run_model(3, [4, 3, 5], rng, zero_ahead=1) for _ in range(200))
    assert caught > 0
