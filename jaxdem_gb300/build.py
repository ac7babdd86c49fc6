"""Build recipe of the engine library (nvcc, sm_103a only).

``build()`` compiles every ``csrc/*.cu`` translation unit in parallel and
links ``_lib/libjdem_gb300.so``.  Flags: ``-fmad=false`` keeps each float
product and sum rounding as written in the translation units whose kernels
restate the reference's float32 arithmetic (contact forces and their pair
predicate, integrators, domains, energies, the neighbour-list API); the list
build (``jdem_tiles.cu``, tests against a widened cutoff and fuses its own
multiply-adds) and the host-only units compile with contraction allowed.
``-lineinfo`` for profiler source correlation.

The XLA FFI handlers (``csrc/ffi/jdem_xla_ffi.cc``) are built into
``_lib/libjdem_xla_ffi.so`` only where jaxlib's FFI headers exist: the
directory named by ``JDEM_JAX_INCLUDE``, else ``jax.ffi.include_dir()``.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "libjdem_gb300.so"
# the bounds-checked build (-DJDEM_BOUNDS_CHECK: every range check of the kernels
# compiled in, a failed one reported as a device status bit); for tests only
CHECKED_LIB = OUT_DIR / "libjdem_gb300_checked.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# translation units free of reference arithmetic: multiply-add contraction allowed
CONTRACT_OK = {"jdem_tiles.cu", "jdem_engine.cu", "jdem_serve.cu", "jdem_rollout.cu"}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jaxdem_gb300")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def _stale(lib: Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + list((PKG.parent / "include").glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, checked: bool = False) -> Path:
    """Compile the CUDA sources and link the shared library; returns its path.
    ``checked`` builds the bounds-checked library (``CHECKED_LIB``) instead."""
    lib = CHECKED_LIB if checked else LIB
    if not force and not _stale(lib):
        return lib
    OUT_DIR.mkdir(exist_ok=True)
    obj_dir = OUT_DIR / ("obj_checked" if checked else "obj")
    obj_dir.mkdir(exist_ok=True)
    cc = nvcc()
    inc = ["-I", str(PKG.parent / "include"), "-I", str(CSRC)]
    defs = ["-DJDEM_BOUNDS_CHECK"] if checked else []

    def compile_one(src: Path) -> Path:
        obj = obj_dir / (src.stem + ".o")
        fmad = [] if src.name in CONTRACT_OK else ["-fmad=false"]
        cmd = [cc, *ARCH, *NVCC_FLAGS, *fmad, *defs, *inc, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = lib.with_suffix(".so.tmp")
    cmd = [cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    if not checked:
        build_xla_ffi(LIB)
    return lib


def jax_ffi_include() -> Path | None:
    """Directory holding ``xla/ffi/api/ffi.h`` (jaxlib), or None when jaxlib is absent."""
    env = os.environ.get("JDEM_JAX_INCLUDE")
    cands = [Path(env)] if env else []
    if not env:
        try:
            import jax.ffi  # noqa: PLC0415

            cands.append(Path(jax.ffi.include_dir()))
        except Exception:
            pass
    for c in cands:
        if (c / "xla" / "ffi" / "api" / "ffi.h").exists():
            return c
    return None


FFI_SRC = CSRC / "ffi" / "jdem_xla_ffi.cc"
FFI_LIB = OUT_DIR / "libjdem_xla_ffi.so"


def build_xla_ffi(lib: Path = LIB) -> Path | None:
    """Build the XLA FFI handler library against ``lib`` when jaxlib's headers are
    found; returns its path, or None (nothing to build against)."""
    inc_jax = jax_ffi_include()
    if inc_jax is None:
        return None
    if FFI_LIB.exists() and FFI_LIB.stat().st_mtime >= max(FFI_SRC.stat().st_mtime, lib.stat().st_mtime):
        return FFI_LIB
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", "-x", "cu",
           "-I", str(PKG.parent / "include"), "-I", str(inc_jax), str(FFI_SRC), "-o", str(FFI_LIB),
           "-L", str(OUT_DIR), "-ljdem_gb300", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"XLA FFI handler build failed:\n{r.stdout}\n{r.stderr}")
    return FFI_LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
