"""Minimal simulation environment: ``dt`` and ``t`` lookups for step functions.

Stands in for ``brainstate.environ`` as the reference's solvers use it
(``quad/_staggered.py:130-131``: ``t = environ.get('t', 0.0)``,
``dt = environ.get('dt')``).  Values are floats in ms.
"""

from __future__ import annotations

import contextlib
import threading

__all__ = ["context", "get", "get_dt", "set"]

_local = threading.local()
_MISSING = object()


def _stack() -> list[dict]:
    st = getattr(_local, "stack", None)
    if st is None:
        st = [{}]
        _local.stack = st
    return st


def get(key: str, default=_MISSING):
    for frame in reversed(_stack()):
        if key in frame:
            return frame[key]
    if default is _MISSING:
        raise KeyError(f"'{key}' is not set in the simulation environment.")
    return default


def get_dt() -> float:
    return get("dt")


def set(**kwargs) -> None:  # noqa: A001 - mirrors brainstate.environ.set
    _stack()[0].update(kwargs)


@contextlib.contextmanager
def context(**kwargs):
    st = _stack()
    st.append(dict(kwargs))
    try:
        yield
    finally:
        st.pop()
