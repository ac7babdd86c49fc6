"""The bounds-checked build of the engine over its main paths.

``build.build(checked=True)`` compiles the kernels with ``-DJDEM_BOUNDS_CHECK``: every
list entry, list row length, cell key, sort permutation index, staged candidate index
and stencil range the kernels index with is range-checked, and a failed check sets
device status bit 32 and skips the access (the regular build compiles each check to
true).  ``bounds_cases.py`` runs the engine's main paths in a child process, once
through the regular library and once through the checked one: no case may set the bit,
and each case's positions, velocities, forces, contacts, neighbour list and frames must
equal the regular library's bit for bit.
"""

from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

from jaxdem_gb300 import build as engine_build

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
ST_INDEX_RANGE = 32


@pytest.fixture(scope="module", autouse=True)
def _build(built):
    return built


def _drive(lib: Path) -> dict:
    env = dict(os.environ, JDEM_LIBRARY=str(lib))
    r = subprocess.run([sys.executable, str(ROOT / "tests" / "bounds_cases.py")], env=env, capture_output=True,
                       text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-4000:]
    recs = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    return {rec["case"]: rec for rec in recs}


def test_checked_build_finds_no_index_out_of_range_and_changes_nothing():
    checked = engine_build.build(checked=True)
    plain = _drive(engine_build.LIB)
    got = _drive(checked)
    assert len(plain) == 13 and set(got) == set(plain)
    for case, rec in got.items():
        assert rec["status"] & ST_INDEX_RANGE == 0, (case, rec)
        assert rec == plain[case], case
