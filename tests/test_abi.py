"""The C ABI library loads and exports every entry point include/jdem_gb300.h declares.

No compute calls: this runs where there is no GPU.
"""

from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "jdem_gb300.h"


def declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(jdem_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib(built):
    from jaxdem_gb300._lib import load

    return load()


def test_header_declares_the_expected_entry_points():
    names = declared()
    for must in ("jdem_create", "jdem_upload", "jdem_step", "jdem_download", "jdem_compute_force",
                 "jdem_energy", "jdem_contacts", "jdem_neighbor_list", "jdem_last_error", "jdem_destroy"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_binding_covers_the_header(lib):
    from jaxdem_gb300 import serve
    from jaxdem_gb300._lib import EXPORTED

    bound = set(EXPORTED) | {p[0] for p in serve._PROTOS}
    extra = {"jdem_compute_force_noalloc"}  # bound in its own test file
    assert set(declared()) - extra <= bound


def test_abi_version_and_status_strings(lib):
    version = int(re.search(r"#define JDEM_ABI_VERSION (\d+)", HEADER.read_text()).group(1))
    assert lib.jdem_abi_version() == version
    assert lib.jdem_status_string(0) == b"ok"
    assert lib.jdem_status_string(7) == b"unsupported configuration"
    assert lib.jdem_status_string(99) == b"unknown status"


def test_null_arguments_are_rejected_without_device_work(lib):
    assert lib.jdem_destroy(None) == 1
    assert lib.jdem_step(None, 1) == 1
    assert lib.jdem_create(None, None) == 1
    assert lib.jdem_last_error(None) == b"null handle"
    # integrator stages: argument checks come before any device work
    args = [None] * 10
    assert lib.jdem_integrate(4, 8, 1, 0, 0, 1e-3, *args) == 1  # dim
    assert lib.jdem_integrate(3, 8, 1, 0, 2, 1e-3, *args) == 1  # stage
    assert lib.jdem_integrate(3, 8, 3, 0, 0, 1e-3, *args) == 1  # linear kind
    assert lib.jdem_integrate(3, 8, 1, 0, 0, 1e-3, *args) == 1  # missing arrays
    assert lib.jdem_integrate(3, 0, 1, 1, 0, 1e-3, *args) == 0  # nothing to do


def test_config_struct_layout_matches_header(lib):
    """ctypes mirrors of JdemSystemDesc / JdemConfig have the C sizes."""
    from jaxdem_gb300._lib import Config, HostState, SystemDesc

    assert C.sizeof(SystemDesc) == 8 + 4 * 4 + 12 + 12 + 4 + 12 + 4 + 4
    assert C.sizeof(HostState) == 14 * C.sizeof(C.c_void_p)
    assert C.sizeof(Config) >= 4 * 2 + C.sizeof(C.c_void_p)


def test_struct_sizes_match_the_c_header(tmp_path):
    """Compile a probe against include/jdem_gb300.h and compare with the ctypes mirrors."""
    import shutil
    import subprocess

    if not shutil.which("gcc"):
        pytest.skip("gcc not available")
    from jaxdem_gb300 import serve
    from jaxdem_gb300._lib import Config, HostState, Stats, SystemDesc

    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "jdem_gb300.h"\nint main(){printf("%zu %zu %zu %zu %zu %zu %zu %zu\\n",'
                   "sizeof(JdemSystemDesc),sizeof(JdemConfig),sizeof(JdemHostState),sizeof(JdemStats),"
                   "sizeof(JdemServeConfig),sizeof(JdemRequest),sizeof(JdemRequestInfo),sizeof(JdemServeStats));}")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [C.sizeof(t) for t in (SystemDesc, Config, HostState, Stats, serve.ServeConfig, serve.RequestStruct,
                                  serve.RequestInfo, serve.ServeStats)]
    assert got == want
