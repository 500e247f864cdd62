"""Name -> step-function registry with the reference's contract.

Same public surface and error behaviour as ``braincell/quad/_registry.py``:
``IntegratorEntry`` (:62), ``IntegratorRegistry`` (:104) with ``register`` (:128,
collisions raise ``ValueError`` unless ``override=True`` which warns with
``RuntimeWarning``; bad names / non-callables raise ``TypeError``), ``unregister``,
``entry`` (deprecated entries warn once with ``DeprecationWarning``), ``names``,
``by_category``, ``as_dict``, ``suggest`` (difflib close matches), plus the module
singleton ``get_registry`` (:350) and the ``register_integrator`` decorator (:355),
which returns the function unchanged.  Not thread-safe, like the reference.
"""

from __future__ import annotations

import difflib
import warnings
from dataclasses import dataclass
from typing import Callable, Iterable, Iterator

__all__ = ["IntegratorEntry", "IntegratorRegistry", "get_registry", "register_integrator"]


@dataclass(frozen=True)
class IntegratorEntry:
    name: str
    func: Callable
    aliases: tuple[str, ...] = ()
    category: str = "general"
    order: int | None = None
    description: str = ""
    deprecated: bool = False
    module: str = ""


class IntegratorRegistry:
    def __init__(self) -> None:
        self._entries: dict[str, IntegratorEntry] = {}
        self._aliases: dict[str, str] = {}
        self._warned: set[str] = set()

    def register(
        self,
        name: str,
        func: Callable,
        *,
        aliases: Iterable[str] = (),
        category: str = "general",
        order: int | None = None,
        description: str = "",
        deprecated: bool = False,
        override: bool = False,
    ) -> IntegratorEntry:
        if not isinstance(name, str) or not name:
            raise TypeError(f"Integrator name must be a non-empty string, got {name!r}.")
        if not callable(func):
            raise TypeError(f"Integrator {name!r} must be a callable, got {type(func).__name__}.")
        alias_tuple = tuple(aliases)
        for a in alias_tuple:
            if not isinstance(a, str) or not a:
                raise TypeError(f"Aliases for integrator {name!r} must be non-empty strings, got {a!r}.")
        if name in self._entries and not override:
            raise ValueError(
                f"Integrator {name!r} is already registered by {self._entries[name].module!r}. "
                "Pass override=True to replace it."
            )
        if name in self._aliases and self._aliases[name] != name:
            raise ValueError(
                f"Cannot register integrator {name!r}: the name is already an alias for {self._aliases[name]!r}."
            )
        for a in alias_tuple:
            if a in self._entries and a != name:
                raise ValueError(
                    f"Cannot register alias {a!r} for {name!r}: a canonical integrator with that name already exists."
                )
            owner = self._aliases.get(a)
            if owner is not None and owner != name:
                raise ValueError(f"Cannot register alias {a!r} for {name!r}: it is already an alias for {owner!r}.")
        if override and name in self._entries:
            warnings.warn(
                f"Overriding integrator {name!r} previously registered by {self._entries[name].module!r}.",
                RuntimeWarning,
                stacklevel=3,
            )
            for a, target in list(self._aliases.items()):
                if target == name:
                    del self._aliases[a]
        entry = IntegratorEntry(
            name=name,
            func=func,
            aliases=alias_tuple,
            category=category,
            order=order,
            description=description,
            deprecated=deprecated,
            module=getattr(func, "__module__", "") or "",
        )
        self._entries[name] = entry
        for a in alias_tuple:
            self._aliases[a] = name
        self._warned.discard(name)
        return entry

    def unregister(self, name: str) -> None:
        if name not in self._entries:
            raise KeyError(f"No integrator registered as {name!r}.")
        del self._entries[name]
        for a, target in list(self._aliases.items()):
            if target == name:
                del self._aliases[a]
        self._warned.discard(name)

    def __contains__(self, name: object) -> bool:
        return isinstance(name, str) and (name in self._entries or name in self._aliases)

    def __iter__(self) -> Iterator[str]:
        return iter(self._entries)

    def __len__(self) -> int:
        return len(self._entries)

    def __getitem__(self, name: str) -> Callable:
        return self.entry(name).func

    def get(self, name: str, default: Callable | None = None) -> Callable | None:
        try:
            return self[name]
        except KeyError:
            return default

    def entry(self, name: str) -> IntegratorEntry:
        canonical = self._aliases.get(name, name)
        try:
            e = self._entries[canonical]
        except KeyError as exc:
            raise KeyError(name) from exc
        if e.deprecated and name not in self._warned:
            self._warned.add(name)
            warnings.warn(f"Integrator {name!r} is deprecated.", DeprecationWarning, stacklevel=3)
        return e

    def resolve(self, name: str) -> str:
        return self.entry(name).name

    def names(self, *, include_aliases: bool = False) -> list[str]:
        out = sorted(self._entries)
        if include_aliases:
            out = sorted(set(out) | set(self._aliases))
        return out

    def by_category(self, category: str) -> list[IntegratorEntry]:
        return sorted((e for e in self._entries.values() if e.category == category), key=lambda e: e.name)

    def items(self) -> Iterator[tuple[str, Callable]]:
        for n, e in self._entries.items():
            yield n, e.func

    def entries(self) -> Iterator[IntegratorEntry]:
        return iter(self._entries.values())

    def as_dict(self, *, include_aliases: bool = True) -> dict[str, Callable]:
        out = {n: e.func for n, e in self._entries.items()}
        if include_aliases:
            for a, target in self._aliases.items():
                out[a] = self._entries[target].func
        return out

    def suggest(self, name: str, *, n: int = 1, cutoff: float = 0.6) -> list[str]:
        return difflib.get_close_matches(name, self.names(include_aliases=True), n=n, cutoff=cutoff)


_REGISTRY = IntegratorRegistry()


def get_registry() -> IntegratorRegistry:
    return _REGISTRY


def register_integrator(
    name: str,
    *,
    aliases: Iterable[str] = (),
    category: str = "general",
    order: int | None = None,
    description: str = "",
    deprecated: bool = False,
    override: bool = False,
) -> Callable[[Callable], Callable]:
    def _wrap(func: Callable) -> Callable:
        _REGISTRY.register(
            name,
            func,
            aliases=aliases,
            category=category,
            order=order,
            description=description,
            deprecated=deprecated,
            override=override,
        )
        return func

    return _wrap
