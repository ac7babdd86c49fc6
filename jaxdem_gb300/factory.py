"""String-keyed plugin registry, mirroring JaxDEM's ``Factory`` (``jaxdem/factory.py``).

Same behaviour on the path the hot loop uses: keys are normalised by
``_normalize_key`` (``factory.py:28-35``), each registry root keeps its own
registry (``factory.py:79-89``), ``register`` refuses a key taken by another
class (``factory.py:240-320``) and ``create`` prefers a ``Create``
classmethod, drops unknown keyword arguments with a warning and checks the
rest against the signature (``factory.py:371-503``).
"""

from __future__ import annotations

import warnings
from inspect import signature
from typing import Any, Callable, ClassVar


def _normalize_key(key: str) -> str:
    """Lowercase, without spaces, underscores and hyphens (``factory.py:28-35``)."""
    return key.replace(" ", "").replace("_", "").replace("-", "").lower()


class Factory:
    """Base of every pluggable component (collider, domain, integrator, ...)."""

    _registry: ClassVar[dict[str, type]] = {}
    __registry_name__: ClassVar[str | None] = None

    def __init_subclass__(cls, **kw: Any) -> None:
        super().__init_subclass__(**kw)
        cls._registry = {}
        cls.__registry_name__ = None
        if "create" in cls.__dict__:
            raise TypeError(
                f"{cls.__name__} is not allowed to override the `create` method. "
                "Use `Create` instead for custom instantiation logic."
            )

    @classmethod
    def registry_name(cls) -> str:
        name = getattr(cls, "__registry_name__", None)
        if name is None:
            raise KeyError(f"{cls.__name__} is not registered in the Factory.")
        return str(name)

    @property
    def type_name(self) -> str:
        return type(self).registry_name()

    @classmethod
    def register(cls, key: str | None = None) -> Callable[[type], type]:
        def decorator(sub_cls: type) -> type:
            k = _normalize_key(sub_cls.__name__ if key is None else key)
            existing = cls._registry.get(k)
            if existing is not None and not (
                existing.__qualname__ == sub_cls.__qualname__ and existing.__module__ == sub_cls.__module__
            ):
                raise ValueError(f"{cls.__name__}: key '{k}' already registered for {existing.__name__}")
            cls._registry[k] = sub_cls
            own = sub_cls.__dict__.get("__registry_name__", None)
            if own is not None and own != k and sub_cls is not cls:
                # a class registered under several keys keeps its first name
                return sub_cls
            sub_cls.__registry_name__ = k
            return sub_cls

        return decorator

    @classmethod
    def create(cls, key: str, /, **kw: Any):
        try:
            sub_cls = cls._registry[_normalize_key(key)]
        except KeyError as err:
            raise KeyError(f"Unknown {cls.__name__} '{key}'. Available: {list(cls._registry)}") from err
        fn = getattr(sub_cls, "Create", None) or sub_cls
        sig = signature(fn)
        params = [p for p in sig.parameters if p != "self"]
        has_var_kw = any(p.kind == p.VAR_KEYWORD for p in sig.parameters.values())
        kw = dict(kw)
        if not has_var_kw:
            dropped = [p for p in kw if p not in params]
            for p in dropped:
                kw.pop(p)
            if dropped:
                warnings.warn(
                    f"{cls.__name__}.create('{key}'): ignoring unknown keyword(s) {dropped}. "
                    f"Expected signature: {sub_cls.__name__}{sig}",
                    stacklevel=2,
                )
        try:
            sig.bind_partial(**kw)
        except TypeError as err:
            raise TypeError(f"Invalid keyword(s) for {sub_cls.__name__}: {err}. Expected signature: {sig}") from None
        return fn(**kw)
