"""SWC morphology reader.

Turns an SWC point list into a :class:`~braincell_gb300.morph.Morphology` of
unbranched sections, following the branch-extraction rules of the reference's
reader in its default ``mode="neuron"`` (``io/swc/reader.py``):

* rows are ``id type x y z radius parent``; type codes map to ``soma``, ``axon``,
  ``basal_dendrite``, ``apical_dendrite``, everything else ``custom``
  (``io/swc/types.py:21-32``);
* a section is extended through nodes with exactly one child of the same type
  (``reader.py:178-186``);
* soma roots (``reader.py:198-238``):
  - a single-point soma becomes a synthetic three-point section along x, centre
    ± radius, and its children attach at the middle (``reader.py:467-489``);
  - a NeuroMorpho three-point soma (a centre row with two childless soma rows at
    one radius from it, all of one radius, ``io/swc/soma.py``) becomes the same
    synthetic section (``reader.py:491-521``);
  - a non-branching multi-point soma is one section, children attaching at 0, 1
    or 0.5 (``reader.py:523-545``, ``_section_attach_x`` :631-636);
  - a branched soma splits into soma sections (``reader.py:567-621``);
* a first section under the soma that immediately forks continues into its first
  same-type child, and the other children attach to it at 0 ("con2prox",
  ``reader.py:252-266``); a generic (non-soma) root does the same
  (``reader.py:155-176``);
* a child section starts with a copy of its attachment point (with the parent's
  radius there, or -- under the soma -- its own first radius) unless that point
  is already its first point with the same radius; under a soma midpoint it is
  copied only for single-point sections (``reader.py:380-434``);
* the attachment position on the parent is its explicit value or the attach
  node's fraction of the parent's path length (``reader.py:436-462``).

Validation is limited to what the extraction needs: unique ids, existing parents,
one root, positive radii, no cycles.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from os import PathLike
from pathlib import Path

import numpy as np

from .morph import Branch, Morphology

__all__ = ["SwcRow", "parse_swc", "read_swc", "SWC_TYPES"]

SWC_TYPES = {0: "custom", 1: "soma", 2: "axon", 3: "basal_dendrite", 4: "apical_dendrite"}
MIN_SYNTHETIC_LENGTH_UM = 1e-6
_REL_TOL = 1e-6
_THREE_POINT_TOL_SCALE = 0.02


def _type(code: int) -> str:
    return SWC_TYPES.get(int(code), "custom")


@dataclass(frozen=True)
class SwcRow:
    node_id: int
    type_code: int
    x: float
    y: float
    z: float
    radius: float
    parent_id: int

    @property
    def point(self) -> np.ndarray:
        return np.array([self.x, self.y, self.z], dtype=np.float64)

    @property
    def kind(self) -> str:
        return _type(self.type_code)


@dataclass
class _Attach:
    node_id: int | None = None
    point: tuple | None = None
    radius: float | None = None
    parent_x: float | None = None


@dataclass
class _Section:
    point_ids: tuple
    kind: str
    parent: int | None
    attach: _Attach | None = None
    override_points: tuple | None = None
    override_radii: tuple | None = None


def parse_swc(text: str) -> list[SwcRow]:
    """Rows of an SWC text (comments and blank lines skipped), in file order."""
    rows = []
    for ln, raw in enumerate(text.splitlines(), start=1):
        line = raw.strip()
        if not line or line.startswith("#"):
            continue
        f = line.split()
        if len(f) < 7:
            raise ValueError(f"SWC line {ln}: expected 7 fields, got {len(f)}.")
        try:
            rows.append(SwcRow(int(f[0]), int(f[1]), float(f[2]), float(f[3]), float(f[4]), float(f[5]), int(f[6])))
        except ValueError as e:
            raise ValueError(f"SWC line {ln}: {e}") from None
    return rows


class _Tree:
    def __init__(self, rows: list[SwcRow]):
        if not rows:
            raise ValueError("SWC has no rows.")
        self.rows = rows
        self.nodes: dict[int, SwcRow] = {}
        for r in rows:
            if r.node_id in self.nodes:
                raise ValueError(f"SWC node id {r.node_id} appears twice.")
            if not (r.radius > 0.0):
                raise ValueError(f"SWC node {r.node_id} has radius {r.radius}; radii must be > 0.")
            self.nodes[r.node_id] = r
        self.children: dict[int, list[int]] = {i: [] for i in self.nodes}
        roots = []
        for r in rows:
            if r.parent_id == -1:
                roots.append(r.node_id)
            elif r.parent_id not in self.nodes:
                raise ValueError(f"SWC node {r.node_id} has unknown parent {r.parent_id}.")
            else:
                self.children[r.parent_id].append(r.node_id)
        for c in self.children.values():
            c.sort()
        if len(roots) != 1:
            raise ValueError(f"SWC must have exactly one root, found {len(roots)}.")
        self.root = roots[0]
        seen, stack = set(), [self.root]
        while stack:
            i = stack.pop()
            if i in seen:
                raise ValueError("SWC parent links form a cycle.")
            seen.add(i)
            stack.extend(self.children[i])
        if len(seen) != len(self.nodes):
            raise ValueError("SWC parent links form a cycle or a detached component.")

    def kind(self, i: int) -> str:
        return self.nodes[i].kind

    def same_kind_children(self, i: int, kind: str) -> list[int]:
        return [c for c in self.children[i] if self.kind(c) == kind]


def _walk(t: _Tree, start: int, kind: str) -> tuple[list[int], int]:
    """Extend from `start` through nodes with exactly one child of the same kind."""
    ids, cur = [start], start
    while len(t.children[cur]) == 1 and t.kind(t.children[cur][0]) == kind:
        cur = t.children[cur][0]
        ids.append(cur)
    return ids, cur


def _generic_sections(t: _Tree) -> list[_Section]:
    root = t.root
    kind = t.kind(root)
    secs: list[_Section] = []
    ids, cur, side = [root], root, ()
    same = t.same_kind_children(root, kind)
    if len(t.children[root]) != 1 and same:
        cur = same[0]
        ids.append(cur)
        side = tuple(c for c in t.children[root] if c != cur)
    more, cur = _walk(t, cur, kind)
    ids.extend(more[1:])
    secs.append(_Section(tuple(ids), kind, None))

    def child(parent: int, attach: _Attach, start: int) -> None:
        k = t.kind(start)
        pids, end = _walk(t, start, k)
        idx = len(secs)
        secs.append(_Section(tuple(pids), k, parent, attach))
        for c in t.children[end]:
            child(idx, _Attach(node_id=end), c)

    for c in side:
        child(0, _Attach(node_id=root), c)
    for c in t.children[cur]:
        child(0, _Attach(node_id=cur), c)
    return secs


def _soma_component(t: _Tree) -> set[int]:
    out, stack = set(), [t.root]
    while stack:
        i = stack.pop()
        if i in out or t.kind(i) != "soma":
            continue
        out.add(i)
        p = t.nodes[i].parent_id
        if p in t.nodes and t.kind(p) == "soma":
            stack.append(p)
        stack.extend(c for c in t.children[i] if t.kind(c) == "soma")
    return out


def _special_three_point(t: _Tree, rows: list[SwcRow]) -> list[SwcRow] | None:
    if len(rows) != 3:
        return None
    for cand in rows:
        others = [r for r in rows if r is not cand]
        if all(r.parent_id == cand.node_id for r in others):
            a, b = others
            break
    else:
        return None
    if t.children[a.node_id] or t.children[b.node_id]:
        return None
    tol = max(_THREE_POINT_TOL_SCALE * cand.radius, _REL_TOL)
    da, db = float(np.linalg.norm(cand.point - a.point)), float(np.linalg.norm(cand.point - b.point))
    if min(da, db) <= 0.0:
        return None
    radii = np.array([r.radius for r in rows])
    if not np.allclose(radii, radii[0], rtol=_REL_TOL, atol=tol):
        return None
    if not (math.isclose(da, cand.radius, rel_tol=_REL_TOL, abs_tol=tol)
            and math.isclose(db, cand.radius, rel_tol=_REL_TOL, abs_tol=tol)):
        return None
    return [cand, a, b]


def _synthetic_soma(center: np.ndarray, radius: float, ids: tuple) -> _Section:
    off = np.array([radius, 0.0, 0.0])
    return _Section(ids, "soma", None, override_points=(tuple(center - off), tuple(center), tuple(center + off)),
                    override_radii=(radius, radius, radius))


def _section_attach_x(ids: tuple, node: int) -> float:
    if node == ids[0]:
        return 0.0
    if node == ids[-1]:
        return 1.0
    return 0.5


def _soma_sections(t: _Tree) -> list[_Section]:
    soma = _soma_component(t)
    ordered = [r for r in t.rows if r.node_id in soma]
    tasks: list[tuple[_Attach, int, int]] = []  # (attach, child node, parent section)
    secs: list[_Section] = []
    special = _special_three_point(t, ordered)
    if len(ordered) == 1 or special is not None:
        c = special[0] if special is not None else ordered[0]
        radius = max(c.radius, MIN_SYNTHETIC_LENGTH_UM)
        ids = tuple(r.node_id for r in (special or ordered))
        secs.append(_synthetic_soma(c.point, radius, ids))
        for ch in t.children[c.node_id]:
            if t.kind(ch) != "soma":
                node = c.node_id if special is not None else None
                tasks.append((_Attach(node_id=node, point=tuple(c.point), radius=radius, parent_x=0.5), ch, 0))
    elif all(len(t.same_kind_children(i, "soma")) <= 1 for i in soma):
        ids = tuple(r.node_id for r in ordered)
        secs.append(_Section(ids, "soma", None))
        for i in ids:
            for ch in t.children[i]:
                if t.kind(ch) != "soma":
                    tasks.append((_Attach(node_id=i, parent_x=_section_attach_x(ids, i)), ch, 0))
    else:
        def section(parent: int | None, start: int, attach: _Attach | None) -> None:
            ids, cur, side = [start], start, ()
            if parent is None:
                sc = t.same_kind_children(cur, "soma")
                if len(sc) > 1:
                    cur = sc[0]
                    ids.append(cur)
                    side = tuple(sc[1:])
            while len(t.same_kind_children(cur, "soma")) == 1:
                cur = t.same_kind_children(cur, "soma")[0]
                ids.append(cur)
            idx = len(secs)
            secs.append(_Section(tuple(ids), "soma", parent, attach))
            eff = tuple(ids)
            if attach is not None and attach.node_id is not None and not (attach.parent_x == 0.5 and len(ids) > 1) \
                    and attach.node_id != ids[0]:
                eff = (attach.node_id, *ids)
            for i in ids:
                px = _section_attach_x(eff, i)
                for ch in t.children[i]:
                    if t.kind(ch) != "soma":
                        tasks.append((_Attach(node_id=i, parent_x=px), ch, idx))
            for ch in side:
                section(idx, ch, _Attach(node_id=start, parent_x=0.0))
            for ch in t.same_kind_children(cur, "soma"):
                section(idx, ch, _Attach(node_id=cur, parent_x=1.0))

        section(None, t.root, None)

    def child(parent: int, attach: _Attach, start: int) -> None:
        k = t.kind(start)
        ids, cur, side = [start], start, ()
        if secs[parent].kind == "soma":
            same = t.same_kind_children(cur, k)
            if len(t.children[cur]) != 1 and same:
                cur = same[0]
                ids.append(cur)
                side = tuple(c for c in t.children[start] if c != cur)
        more, cur = _walk(t, cur, k)
        ids.extend(more[1:])
        idx = len(secs)
        secs.append(_Section(tuple(ids), k, parent, attach))
        for c in side:
            child(idx, _Attach(node_id=start), c)
        for c in t.children[cur]:
            child(idx, _Attach(node_id=cur), c)

    for attach, ch, parent in tasks:
        child(parent, attach, ch)
    return secs


def _attach_x(t: _Tree, parent: _Section, attach: _Attach | None) -> float:
    if attach is None:
        return 1.0
    if attach.parent_x is not None:
        return float(attach.parent_x)
    pts = [t.nodes[i].point for i in parent.point_ids]
    if len(pts) == 1:
        return 1.0
    k = parent.point_ids.index(attach.node_id)
    seg = [float(np.linalg.norm(pts[i + 1] - pts[i])) for i in range(len(pts) - 1)]
    total = sum(seg)
    return 1.0 if total <= 0.0 else float(sum(seg[:k]) / total)


def _branch(t: _Tree, sec: _Section, parent_kind: str | None) -> Branch:
    if sec.override_points is not None:
        return Branch.from_points(points=sec.override_points, radii=sec.override_radii, type=sec.kind)
    pts = [t.nodes[i].point for i in sec.point_ids]
    radii = [t.nodes[i].radius for i in sec.point_ids]
    a = sec.attach
    if a is not None:
        if a.point is not None and a.radius is not None:
            apt, arad = np.array(a.point, dtype=np.float64), float(a.radius)
        else:
            apt, arad = t.nodes[a.node_id].point, t.nodes[a.node_id].radius
        copy = parent_kind != "soma" or len(sec.point_ids) == 1 or a.parent_x != 0.5
        child_rad = float(radii[0]) if parent_kind == "soma" else arad
        if copy and not (np.allclose(pts[0], apt) and np.isclose(radii[0], child_rad)):
            pts.insert(0, apt)
            radii.insert(0, child_rad)
    if len(pts) == 1:
        raise ValueError(f"SWC section starting at node {sec.point_ids[0]} has a single point.")
    return Branch.from_points(points=pts, radii=radii, type=sec.kind)


def read_swc(source: str | PathLike, *, text: bool = False) -> Morphology:
    """Read an SWC file (or, with ``text=True``, SWC content) into a Morphology."""
    content = source if text else Path(source).read_text(encoding="utf-8", errors="replace")
    t = _Tree(parse_swc(str(content)))
    secs = _soma_sections(t) if t.kind(t.root) == "soma" else _generic_sections(t)
    root = _branch(t, secs[0], None)
    morpho = Morphology.from_root(root, name="soma" if secs[0].kind == "soma" else None)
    views = {0: morpho.root}
    for i, sec in enumerate(secs[1:], start=1):
        parent = secs[sec.parent]
        views[i] = morpho.attach(parent=views[sec.parent], child_branch=_branch(t, sec, parent.kind),
                                 parent_x=_attach_x(t, parent, sec.attach), child_x=0.0)
    return morpho
