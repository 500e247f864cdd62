"""Integrator registry mirror (``braincell/quad/__init__.py``) with the GB300 step registered.

``get_integrator(method)`` resolves a registered name or alias, returns a callable
unchanged, raises ``ValueError`` with a "Did you mean ...?" hint for unknown names
and ``TypeError`` for anything else (``quad/__init__.py:167-214``).
"""

from __future__ import annotations

from collections.abc import Mapping
from typing import Callable

from ._registry import IntegratorEntry, IntegratorRegistry, get_registry, register_integrator
from ._gb300 import gb300_staggered_step

__all__ = [
    "IntegratorEntry",
    "IntegratorRegistry",
    "get_registry",
    "register_integrator",
    "get_integrator",
    "all_integrators",
    "gb300_staggered_step",
]


class _RegistryView(Mapping):
    def __init__(self, reg: IntegratorRegistry) -> None:
        self._reg = reg

    def __getitem__(self, key: str) -> Callable:
        return self._reg[key]

    def __iter__(self):
        return iter(self._reg.as_dict(include_aliases=True))

    def __len__(self) -> int:
        return len(self._reg.as_dict(include_aliases=True))


all_integrators: Mapping[str, Callable] = _RegistryView(get_registry())


def get_integrator(method) -> Callable:
    if callable(method):
        return method
    if isinstance(method, str):
        reg = get_registry()
        try:
            return reg[method]
        except KeyError:
            sug = reg.suggest(method, n=1)
            hint = f" Did you mean {sug[0]!r}?" if sug else ""
            raise ValueError(f"Unknown integrator {method!r}.{hint} Available: {', '.join(reg.names())}.") from None
    raise TypeError(f"Integrator method must be a string or callable, got {type(method).__name__}.")
