"""Import JaxDEM's reference source through the numpy stand-in for JAX (fixture generation only).

Modules JaxDEM imports at package import time but that the hot path never calls
(orbax checkpointing, h5py, vtk, flax/optax/distrax for the RL package) are replaced by
inert stubs: calling one yields another stub (a decorator stub returns the function), so
only code that never runs on the hot path can touch them."""

from __future__ import annotations

import importlib
import sys
import types
from pathlib import Path

HERE = Path(__file__).resolve().parent
SHIM = HERE / "jaxshim"


class _Stub(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        sub = _Stub(f"{self.__name__}.{name}")
        setattr(self, name, sub)
        return sub

    def __call__(self, *a, **k):
        # import-time calls (dtype constructors, decorators) get another inert stub
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return _Stub(f"{self.__name__}()")

    def __mro_entries__(self, bases):
        return (object,)


def _stub(name):
    parts = name.split(".")
    for i in range(1, len(parts) + 1):
        n = ".".join(parts[:i])
        if n not in sys.modules:
            m = _Stub(n)
            m.__path__ = []
            sys.modules[n] = m
            if i > 1:
                setattr(sys.modules[".".join(parts[: i - 1])], parts[i - 1], m)


class _StubFinder:
    """Last on sys.meta_path: any jax.* submodule the stand-in lacks becomes an inert stub."""

    def find_spec(self, name, path=None, target=None):
        if not name.startswith("jax."):
            return None
        import importlib.machinery

        return importlib.machinery.ModuleSpec(name, self, is_package=True)

    def create_module(self, spec):
        m = _Stub(spec.name)
        m.__path__ = []
        return m

    def exec_module(self, module):
        pass


def import_reference(reference_root: str = "/root/reference", x64: bool = False):
    """The reference's ``jaxdem`` package, running on the numpy stand-in."""
    if str(SHIM) not in sys.path:
        sys.path.insert(0, str(SHIM))
    for n in ("orbax.checkpoint.checkpoint_managers", "h5py", "vtk.util.numpy_support", "flax.nnx.nn.recurrent",
              "distrax._src.bijectors.bijector", "tqdm.auto"):
        _stub(n)
    if "optax" not in sys.modules:
        # System.create builds its default minimizer object (an optax transformation, a
        # NamedTuple of init/update functions) even when nothing minimizes
        from typing import Any, NamedTuple

        optax = types.ModuleType("optax")

        class GradientTransformation(NamedTuple):
            init: Any
            update: Any

        class GradientTransformationExtraArgs(NamedTuple):
            init: Any
            update: Any

        optax.GradientTransformation = GradientTransformation
        optax.GradientTransformationExtraArgs = GradientTransformationExtraArgs
        sys.modules["optax"] = optax
    if not any(isinstance(f, _StubFinder) for f in sys.meta_path):
        sys.meta_path.append(_StubFinder())
    import jax

    jax.config.update("jax_enable_x64", x64)
    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
    return importlib.import_module("jaxdem")
