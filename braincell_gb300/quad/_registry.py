"""A name -> step-function table that honours the reference registry's public contract.

What a plugin and its callers rely on (``braincell/quad/_registry.py``: the
``register_integrator`` decorator at :355-406, the registry methods at :104-300)
is kept: ``register_integrator(name, *, aliases, category, order, description,
deprecated, override)`` returns the decorated function unchanged; a name or alias
already taken raises ``ValueError`` unless ``override=True`` replaces the owner's
entry (with a ``RuntimeWarning``); a bad name, alias or non-callable raises
``TypeError``; a deprecated entry warns (``DeprecationWarning``) the first time it
is looked up under each name; lookups of unknown names raise ``KeyError``; and
``suggest`` offers close matches for "Did you mean" hints.  Not thread-safe.

The table itself is this module's own: one dict from every known key (canonical
name or alias) to its canonical name, and one dict of entries.
"""

from __future__ import annotations

import difflib
import warnings
from dataclasses import dataclass
from typing import Callable, Iterable, Iterator

__all__ = ["IntegratorEntry", "IntegratorRegistry", "get_registry", "register_integrator"]


@dataclass(frozen=True)
class IntegratorEntry:
    """One registered step function and its metadata."""

    name: str
    func: Callable
    aliases: tuple[str, ...] = ()
    category: str = "general"
    order: int | None = None
    description: str = ""
    deprecated: bool = False
    module: str = ""


def _key(kind: str, value) -> str:
    if isinstance(value, str) and value:
        return value
    raise TypeError(f"{kind} must be a non-empty str (got {value!r})")


class IntegratorRegistry:
    """Canonical names and aliases share one key space; each key has one owner."""

    def __init__(self) -> None:
        self._owner: dict[str, str] = {}            # key (name or alias) -> canonical name
        self._table: dict[str, IntegratorEntry] = {}  # canonical name -> entry
        self._warned: set[str] = set()                # keys a deprecation warning was given for

    # ------------------------------------------------------------------ writing
    def register(self, name: str, func: Callable, *, aliases: Iterable[str] = (), category: str = "general",
                 order: int | None = None, description: str = "", deprecated: bool = False,
                 override: bool = False) -> IntegratorEntry:
        name = _key("integrator name", name)
        if not callable(func):
            raise TypeError(f"integrator {name!r}: expected a callable step function, got {type(func).__name__}")
        keys = (name,) + tuple(_key(f"alias of {name!r}", a) for a in aliases)
        replaced = self._table.get(name)
        for k in keys:
            owner = self._owner.get(k)
            if owner is None:
                continue
            if owner != name:  # another integrator's name or alias: never taken over
                what = "name" if k == name else "alias"
                raise ValueError(f"cannot register {what} {k!r} for {name!r}: the key belongs to {owner!r}")
            if not override:
                raise ValueError(f"cannot register {name!r}: registered already (from "
                                 f"{replaced.module or 'an unknown module'}); use override=True to replace it")
        if replaced is not None:
            warnings.warn(f"integrator {name!r} replaced (was from {replaced.module or 'an unknown module'})",
                          RuntimeWarning, stacklevel=3)
            self._drop(name)
        entry = IntegratorEntry(name, func, keys[1:], category, order, description, deprecated,
                                getattr(func, "__module__", "") or "")
        self._table[name] = entry
        for k in keys:
            self._owner[k] = name
        return entry

    def _drop(self, name: str) -> None:
        entry = self._table.pop(name)
        for k in (name,) + entry.aliases:
            if self._owner.get(k) == name:
                del self._owner[k]
            self._warned.discard(k)

    def unregister(self, name: str) -> None:
        if name not in self._table:
            raise KeyError(f"{name!r} is not a registered integrator name")
        self._drop(name)

    # ------------------------------------------------------------------ reading
    def entry(self, name: str) -> IntegratorEntry:
        if name not in self._owner:
            raise KeyError(name)
        e = self._table[self._owner[name]]
        if e.deprecated and name not in self._warned:
            self._warned.add(name)
            warnings.warn(f"the integrator {name!r} is deprecated", DeprecationWarning, stacklevel=3)
        return e

    def __getitem__(self, name: str) -> Callable:
        return self.entry(name).func

    def get(self, name: str, default: Callable | None = None) -> Callable | None:
        return self[name] if name in self._owner else default

    def resolve(self, name: str) -> str:
        return self.entry(name).name

    def __contains__(self, name: object) -> bool:
        return isinstance(name, str) and name in self._owner

    def __iter__(self) -> Iterator[str]:
        return iter(self._table)

    def __len__(self) -> int:
        return len(self._table)

    def names(self, *, include_aliases: bool = False) -> list[str]:
        return sorted(self._owner if include_aliases else self._table)

    def by_category(self, category: str) -> list[IntegratorEntry]:
        return [self._table[n] for n in sorted(self._table) if self._table[n].category == category]

    def items(self) -> Iterator[tuple[str, Callable]]:
        return ((n, e.func) for n, e in self._table.items())

    def entries(self) -> Iterator[IntegratorEntry]:
        return iter(self._table.values())

    def as_dict(self, *, include_aliases: bool = True) -> dict[str, Callable]:
        keys = self._owner if include_aliases else self._table
        return {k: self._table[self._owner[k]].func for k in keys}

    def suggest(self, name: str, *, n: int = 1, cutoff: float = 0.6) -> list[str]:
        return difflib.get_close_matches(name, self.names(include_aliases=True), n=n, cutoff=cutoff)


_REGISTRY = IntegratorRegistry()


def get_registry() -> IntegratorRegistry:
    """The process-wide table ``get_integrator`` resolves names in."""
    return _REGISTRY


def register_integrator(name: str, *, aliases: Iterable[str] = (), category: str = "general", order: int | None = None,
                        description: str = "", deprecated: bool = False,
                        override: bool = False) -> Callable[[Callable], Callable]:
    """Decorator: register the function in the process-wide table and return it unchanged."""

    def deco(func: Callable) -> Callable:
        _REGISTRY.register(name, func, aliases=aliases, category=category, order=order, description=description,
                           deprecated=deprecated, override=override)
        return func

    return deco
