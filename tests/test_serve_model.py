"""The one-at-a-time latency model of the serving benchmark (host logic, no GPU)."""

from __future__ import annotations

import numpy as np

from jaxdem_gb300.serve import fifo_model
from jaxdem_gb300.workloads import Request


def _r(i, t, N, steps, dim=3):
    return Request(rid=i, arrival=t, N=N, dim=dim, phi=0.4, steps=steps, seed=i)


def test_fifo_model_recovers_a_linear_service_time_and_queues():
    # timed requests follow t = 0.01 + 1e-9 * N * steps exactly
    timed = [_r(i, 0.0, N, 100, d) for i, (N, d) in enumerate([(1000, 3), (50000, 3), (200000, 3),
                                                                 (2000, 2), (80000, 2)])]
    service = [0.01 + 1e-9 * r.N * r.steps for r in timed]
    window = [_r(0, 0.0, 100000, 1000), _r(1, 0.05, 100000, 1000), _r(2, 10.0, 1000, 100, dim=2)]
    m = fifo_model(window, timed, service)
    a, b = m["coef"]["3"]
    assert np.isclose(a, 0.01) and np.isclose(b, 1e-9)
    s0 = 0.01 + 1e-9 * 1e8  # 0.11 s each
    # the second arrives at 0.05 while the first runs until 0.11: it waits
    lat = [s0, 2 * s0 - 0.05, 0.01 + 1e-9 * 1e5]
    assert np.isclose(m["latency_s"]["mean"], np.mean(lat))
    assert np.isclose(m["latency_s"]["p50"], np.percentile(lat, 50))
