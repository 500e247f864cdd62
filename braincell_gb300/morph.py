"""Morphology declarations: branches made of frustum segments, attached into a tree.

Mirrors the construction surface of the reference's ``braincell.morph``:

* ``Branch.from_lengths(lengths=, radii=| radii_proximal=/radii_distal=, type=)``
  follows ``morph/branch.py:195`` (per-segment lengths, shared boundary radii or
  per-segment proximal/distal radii).
* ``Morphology.from_root(branch, name="soma")`` follows ``morph/morphology.py:315``.
* ``Morphology.attach(parent=, child_branch=, child_name=, parent_x=1.0, child_x=0.0)``
  follows ``morph/morphology.py:1412``.

Units are plain floats: lengths and radii in micrometres.  Branch indices are
assigned in attachment order (root = 0), as in the reference, and that order is
the order in which CVs and node-tree points are numbered downstream.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Sequence

import numpy as np

__all__ = ["Branch", "Morphology", "MorphoBranch", "MorphoEdge"]

_TYPES = ("soma", "axon", "basal_dendrite", "apical_dendrite", "dendrite", "custom")


@dataclass(frozen=True)
class Branch:
    """One unbranched cable made of ``n_segments`` frusta.

    ``lengths[i]`` is the length of segment ``i``; ``radii_proximal[i]`` and
    ``radii_distal[i]`` its end radii (um).
    """

    lengths: np.ndarray
    radii_proximal: np.ndarray
    radii_distal: np.ndarray
    type: str = "custom"
    points: np.ndarray | None = None  # [n_segments + 1, 3] um, when built from points

    @classmethod
    def from_lengths(
        cls,
        *,
        lengths: Sequence[float],
        radii: Sequence[float] | None = None,
        radii_proximal: Sequence[float] | None = None,
        radii_distal: Sequence[float] | None = None,
        type: str = "custom",
    ) -> "Branch":
        lengths_a = np.atleast_1d(np.asarray(lengths, dtype=np.float64))
        if lengths_a.ndim != 1 or lengths_a.size == 0:
            raise ValueError("lengths must be a non-empty 1-D sequence.")
        if radii is not None and (radii_proximal is not None or radii_distal is not None):
            raise TypeError("Pass either radii or (radii_proximal, radii_distal), not both.")
        if radii is not None:
            r = np.atleast_1d(np.asarray(radii, dtype=np.float64))
            if r.shape != (lengths_a.size + 1,):
                raise ValueError(f"radii must have shape ({lengths_a.size + 1},), got {r.shape}.")
            rp, rd = r[:-1].copy(), r[1:].copy()
        else:
            if radii_proximal is None or radii_distal is None:
                raise TypeError("Branch.from_lengths requires radii or both radii_proximal and radii_distal.")
            rp = np.atleast_1d(np.asarray(radii_proximal, dtype=np.float64))
            rd = np.atleast_1d(np.asarray(radii_distal, dtype=np.float64))
            if rp.shape != lengths_a.shape or rd.shape != lengths_a.shape:
                raise ValueError("radii_proximal / radii_distal must match lengths in shape.")
        if np.any(lengths_a < 0.0):
            raise ValueError("Segment lengths must be >= 0.")
        if np.any(rp <= 0.0) or np.any(rd <= 0.0):
            raise ValueError("All branch radii must be > 0.")
        if float(lengths_a.sum()) <= 1e-6:
            raise ValueError("Branch total length must be > 1e-6 um.")
        if type not in _TYPES:
            raise ValueError(f"Unknown branch type {type!r}; expected one of {_TYPES}.")
        if radii is None and lengths_a.size > 1:
            # zero-length jump segments at radius discontinuities (morph/branch.py:440-500)
            disc = ~np.isclose(rd[:-1], rp[1:])
            if disc.any():
                L, P, D = [], [], []
                for i in range(lengths_a.size):
                    L.append(lengths_a[i])
                    P.append(rp[i])
                    D.append(rd[i])
                    if i < lengths_a.size - 1 and disc[i]:
                        L.append(0.0)
                        P.append(rd[i])
                        D.append(rp[i + 1])
                lengths_a, rp, rd = np.asarray(L), np.asarray(P), np.asarray(D)
        return cls(lengths=lengths_a, radii_proximal=rp, radii_distal=rd, type=type)

    @classmethod
    def from_points(cls, *, points: Sequence[Sequence[float]], radii: Sequence[float],
                    type: str = "custom") -> "Branch":
        """Branch through ordered 3-D points (um) with a radius at every point.

        Follows ``morph/branch.py:287`` (``Branch.from_points``): segment lengths
        are the distances between consecutive points; a repeated point with a
        different radius is a zero-length segment (a radius jump).
        """
        pts = np.asarray(points, dtype=np.float64)
        r = np.asarray(radii, dtype=np.float64)
        if pts.ndim != 2 or pts.shape[1] != 3 or pts.shape[0] < 2:
            raise ValueError("points must have shape (n_points >= 2, 3).")
        if r.shape != (pts.shape[0],):
            raise ValueError("radii must give one radius per point.")
        lengths = np.linalg.norm(np.diff(pts, axis=0), axis=1)
        b = cls.from_lengths(lengths=lengths, radii=r, type=type)
        return cls(lengths=b.lengths, radii_proximal=b.radii_proximal, radii_distal=b.radii_distal, type=type,
                   points=pts)

    @property
    def length(self) -> float:
        return float(self.lengths.sum())

    @property
    def n_segments(self) -> int:
        return int(self.lengths.size)


@dataclass(frozen=True)
class MorphoBranch:
    """Handle to a branch inside a :class:`Morphology` (name + index)."""

    name: str
    index: int
    branch: Branch


@dataclass(frozen=True)
class MorphoEdge:
    """Attachment of ``child`` to ``parent`` at ``parent_x`` / ``child_x``."""

    parent: MorphoBranch
    child: MorphoBranch
    parent_x: float
    child_x: float


class Morphology:
    """A tree of branches rooted at ``branches[0]``."""

    def __init__(self, *, root_name: str | None, root_branch: Branch) -> None:
        if not isinstance(root_branch, Branch):
            raise TypeError(f"root_branch must be a Branch, got {type(root_branch).__name__}.")
        name = root_name if root_name is not None else root_branch.type
        self._nodes: list[MorphoBranch] = [MorphoBranch(name=name, index=0, branch=root_branch)]
        self._by_name: dict[str, MorphoBranch] = {name: self._nodes[0]}
        self._edges: list[MorphoEdge] = []
        self._parent: list[int] = [-1]
        self._type_counts: dict[str, int] = {root_branch.type: 1}

    @classmethod
    def from_root(cls, branch: Branch, *, name: str | None = "soma") -> "Morphology":
        return cls(root_name=name, root_branch=branch)

    def attach(
        self,
        *,
        parent,
        child_branch: Branch,
        child_name: str | None = None,
        parent_x: float = 1.0,
        child_x: float = 0.0,
    ) -> MorphoBranch:
        if isinstance(parent, str):
            if parent not in self._by_name:
                raise KeyError(f"Unknown parent branch {parent!r}.")
            parent_ref = self._by_name[parent]
        elif isinstance(parent, MorphoBranch):
            parent_ref = self._nodes[parent.index]
        elif isinstance(parent, (int, np.integer)):
            parent_ref = self._nodes[int(parent)]
        else:
            raise TypeError(f"parent must be a name, index or MorphoBranch, got {type(parent).__name__}.")
        if not isinstance(child_branch, Branch):
            raise TypeError(f"child_branch must be a Branch, got {type(child_branch).__name__}.")
        px, cx = float(parent_x), float(child_x)
        if not (0.0 <= px <= 1.0):
            raise ValueError(f"parent_x must lie in [0, 1], got {px}.")
        if cx not in (0.0, 1.0):
            raise ValueError(f"child_x must be 0 or 1, got {cx}.")
        if child_name is None:
            k = self._type_counts.get(child_branch.type, 0)
            child_name = f"{child_branch.type}_{k}"
        if child_name in self._by_name:
            raise ValueError(f"Branch name {child_name!r} already used.")
        self._type_counts[child_branch.type] = self._type_counts.get(child_branch.type, 0) + 1
        node = MorphoBranch(name=child_name, index=len(self._nodes), branch=child_branch)
        self._nodes.append(node)
        self._by_name[child_name] = node
        self._edges.append(MorphoEdge(parent=parent_ref, child=node, parent_x=px, child_x=cx))
        self._parent.append(parent_ref.index)
        return node

    @property
    def branches(self) -> tuple[Branch, ...]:
        return tuple(n.branch for n in self._nodes)

    @property
    def branch_names(self) -> tuple[str, ...]:
        return tuple(n.name for n in self._nodes)

    @property
    def edges(self) -> tuple[MorphoEdge, ...]:
        return tuple(self._edges)

    @property
    def root(self) -> MorphoBranch:
        return self._nodes[0]

    @property
    def parent_index(self) -> np.ndarray:
        return np.asarray(self._parent, dtype=np.int32)

    def branch(self, name_or_index) -> MorphoBranch:
        if isinstance(name_or_index, str):
            return self._by_name[name_or_index]
        return self._nodes[int(name_or_index)]

    def __len__(self) -> int:
        return len(self._nodes)
