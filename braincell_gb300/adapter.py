"""Lowering of a braincell (reference) ``Cell`` into a :class:`CellBatch`.

This is the ``_spec_from_cell`` of the braincell-side plugin: it reads only the
attributes the reference exposes after discretisation and needs no import of
braincell itself, so it is tested here against duck-typed stand-ins.

* ``cell.morpho.branches`` -- ``MorphoBranch`` nodes in branch order
  (``morph/morphology.py:614-626``): ``.branch`` (``lengths``, ``radii_proximal``,
  ``radii_distal`` per frustum segment, ``morph/branch.py:141-146``), and the
  attachment ``.parent_id`` / ``.node_id`` / ``.parent_x`` / ``.child_x``
  (``morph/morphology.py:1776-1810``).
* ``cell.cvs`` -- the frozen ``CV`` records (``_discretization/base.py:87-176``):
  ``branch_id``, ``prox`` / ``dist``, ``cm``, ``ra``, ``v``, ``density_mech``
  (``Channel`` / ``Ion`` declarations with ``class_name``, ``name`` and a
  ``params`` mapping) and ``point_mech_roles`` (``position`` in prox / mid / dist
  with the point ``mechanism``; ``CurrentClamp`` with ``delay``, ``durations``,
  ``amplitudes``, ``_point.py:86-160``; ``StateProbe``).
* ``cell.pop_size`` -- replicas (``cell.py:203-268``).

Quantities are converted with ``to_decimal(unit)`` when they carry units
(brainunit) and read as plain numbers in this package's units otherwise (um, mV,
ms, nA, mS/cm^2, uF/cm^2, ohm cm, kelvin, mM).  The batch spec carries one
region per branch, so every CV of a branch must carry the same cable values and
density declarations; a cell painted at a finer grain is rejected with
``NotImplementedError``.  CVs must tile each branch uniformly (the reference's
``CVPerBranch`` / ``CVPerBranchList`` / ``MaxCVLen`` policies do).
"""

from __future__ import annotations

import numpy as np

from . import _abi
from .batch import CellBatch, concat_batches
from .catalogue import region_record
from .mech import CableProperty, Channel, Ion

__all__ = ["batch_from_reference_cell"]

# parameter name -> unit of this package (None: dimensionless)
_PARAM_UNITS = {
    "g_max": "mS/cm2", "E": "mV", "V_sh": "mV", "temp": "K", "temp_ref": "K", "temp_ref_p": "K",
    "temp_ref_q": "K", "tau": "ms", "tau_max": "ms", "d": "um", "C_rest": "mM", "Co": "mM", "Ci_initializer": "mM",
}


def _unit(name: str):
    import brainunit as u  # only reached for values that carry units

    return {"um": u.um, "mV": u.mV, "ms": u.ms, "nA": u.nA, "mS/cm2": u.mS / u.cm ** 2, "uF/cm2": u.uF / u.cm ** 2,
            "ohm cm": u.ohm * u.cm, "K": u.kelvin, "mM": u.mM}[name]


def _num(x, unit: str | None):
    """A float array from a quantity (converted to ``unit``) or a plain number."""
    if unit is not None and hasattr(x, "to_decimal"):
        x = x.to_decimal(_unit(unit))
    return np.asarray(x, dtype=np.float64)


def _scalar(x, unit: str | None) -> float:
    a = _num(x, unit)
    if a.size != 1:
        a = a.reshape(-1)
        if not np.all(a == a[0]):
            raise NotImplementedError("per-replica parameter values are not supported by the GB300 batch spec")
    return float(a.reshape(-1)[0])


def _decl(d):
    """A reference Channel / Ion declaration as this package's declaration."""
    kind = Channel if type(d).__name__ == "Channel" or getattr(d, "category", "") == "channel" else Ion
    params = {k: _scalar(v, _PARAM_UNITS.get(k)) for k, v in dict(d.params).items()}
    return kind(d.class_name, name=getattr(d, "name", None), **params)


def _decl_key(d):
    return (type(d).__name__, d.class_name, getattr(d, "name", None),
            tuple(sorted((k, _scalar(v, _PARAM_UNITS.get(k))) for k, v in dict(d.params).items())))


def batch_from_reference_cell(cell) -> CellBatch:
    """The batch (``pop_size`` replicas) of a discretised braincell ``Cell``."""
    nodes = list(cell.morpho.branches)
    nb = len(nodes)
    index_of = {getattr(n, "node_id", k): k for k, n in enumerate(nodes)}
    parent = np.full(nb, -1, np.int32)
    parent_x = np.zeros(nb)
    child_x = np.zeros(nb)
    seg_len, seg_rp, seg_rd, seg_off = [], [], [], [0]
    for k, n in enumerate(nodes):
        if n.parent_id is not None:
            parent[k] = index_of[n.parent_id]
            parent_x[k] = float(n.parent_x)
            child_x[k] = float(n.child_x)
        br = n.branch
        L = _num(br.lengths, "um").reshape(-1)
        seg_len.append(L)
        seg_rp.append(_num(br.radii_proximal, "um").reshape(-1))
        seg_rd.append(_num(br.radii_distal, "um").reshape(-1))
        seg_off.append(seg_off[-1] + L.size)
    if parent[0] != -1 or np.any(parent[1:] < 0):
        raise ValueError("the morphology's first branch must be its root")
    # CVs per branch, checked to tile the branch uniformly in order
    cvs = list(cell.cvs)
    by_branch: list[list] = [[] for _ in range(nb)]
    for cv in cvs:
        by_branch[int(cv.branch_id)].append(cv)
    ncv = np.zeros(nb, np.int32)
    regions: dict = {}
    region_list: list[tuple[CableProperty, list]] = []
    branch_region = np.zeros(nb, np.int32)
    pulses, probes = [], []
    for b in range(nb):
        cl = sorted(by_branch[b], key=lambda c: float(c.prox))
        n = len(cl)
        if n == 0:
            raise ValueError(f"branch {b} has no CV")
        ncv[b] = n
        for k, cv in enumerate(cl):
            if abs(float(cv.prox) - k / n) > 1e-9 or abs(float(cv.dist) - (k + 1) / n) > 1e-9:
                raise NotImplementedError(f"branch {b}: CVs do not tile the branch uniformly")
        keys = {(round(_scalar(cv.cm, "uF/cm2"), 12), round(_scalar(cv.ra, "ohm cm"), 12),
                 round(_scalar(cv.v, "mV"), 12), tuple(sorted(_decl_key(d) for d in cv.density_mech))) for cv in cl}
        if len(keys) != 1:
            raise NotImplementedError(f"branch {b}: its CVs carry different cable values or mechanisms; the GB300 "
                                      "batch spec paints whole branches")
        key = keys.pop()
        if key not in regions:
            cv = cl[0]
            cable = CableProperty(resting_potential=_scalar(cv.v, "mV"), membrane_capacitance=_scalar(cv.cm, "uF/cm2"),
                                  axial_resistivity=_scalar(cv.ra, "ohm cm"))
            regions[key] = len(region_list)
            region_list.append((cable, [_decl(d) for d in cv.density_mech]))
        branch_region[b] = regions[key]
        for cv in cl:
            for role in getattr(cv, "point_mech_roles", ()):
                pos = role.position
                x = float(cv.prox) if pos == "prox" else float(cv.dist) if pos == "dist" else \
                    0.5 * (float(cv.prox) + float(cv.dist))
                m = role.mechanism
                kind = type(m).__name__
                if kind == "CurrentClamp":
                    t = _scalar(m.delay, "ms")
                    durs = _num(m.durations, "ms").reshape(-1)
                    amps = _num(m.amplitudes, "nA").reshape(-1)
                    for dur, amp in zip(durs, amps):
                        pulses.append((b, x, t, t + float(dur), float(amp)))
                        t += float(dur)
                elif kind == "StateProbe":
                    probes.append((b, x))
                else:
                    raise NotImplementedError(f"point mechanism {kind} is not lowered to the GB300 batch spec")
    R = len(region_list)
    cm, ra = np.zeros(R), np.zeros(R)
    bits = np.zeros(R, np.uint32)
    params = np.zeros((R, _abi.BC_NPARAM))
    for r, (cable, mechs) in enumerate(region_list):
        bits[r], params[r] = region_record(mechs, cable)
        cm[r], ra[r] = cable.membrane_capacitance, cable.axial_resistivity
    one = CellBatch(
        n_regions=R,
        cell_branch_offsets=np.asarray([0, nb], np.int64),
        branch_parent=parent,
        branch_parent_x=parent_x,
        branch_child_x=child_x,
        branch_ncv=ncv,
        branch_region=branch_region,
        branch_seg_offsets=np.asarray(seg_off, np.int64),
        seg_length=np.concatenate(seg_len),
        seg_r_prox=np.concatenate(seg_rp),
        seg_r_dist=np.concatenate(seg_rd),
        region_cm=cm,
        region_ra=ra,
        region_mech=bits,
        region_params=params,
        pulse_cell=np.zeros(len(pulses), np.int32),
        pulse_branch=np.asarray([p[0] for p in pulses], np.int32),
        pulse_x=np.asarray([p[1] for p in pulses]),
        pulse_t_on=np.asarray([p[2] for p in pulses]),
        pulse_t_off=np.asarray([p[3] for p in pulses]),
        pulse_amp=np.asarray([p[4] for p in pulses]),
        probe_cell=np.zeros(len(probes), np.int32),
        probe_branch=np.asarray([p[0] for p in probes], np.int32),
        probe_x=np.asarray([p[1] for p in probes]),
    )
    P = int(np.prod(getattr(cell, "pop_size", (1,))))
    return one if P == 1 else concat_batches([one] * P)
