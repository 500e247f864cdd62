"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No dataset is involved; every input is generated.  Each cell is first drawn as a
small description (branch tree, lengths, radii, CV counts, conductance factors,
stimuli) from its own generator ``default_rng([seed, cell_index])``, so a subset of
cells is identical to the same cells inside the full batch.  A description can
be turned into a declared :class:`~braincell_gb300.cell.Cell` (for checking) or
appended to a flat :class:`~braincell_gb300.batch.CellBatch` (fast path for
10,000 cells).

* ``small``   -- 16 identical cells: 20x20 um soma (1 CV) + binary dendritic tree of
  depth 3 (14 branches, lengths U(50, 200) um, 8 CVs each, radius tapering 1.0 ->
  0.25 um with path distance); Leak 0.3 mS/cm^2 (E -70) everywhere, Na_Ba2002 120 and
  KDR_Ba2002 36 mS/cm^2 on the soma, CaL_IS2008 2 mS/cm^2 on dendrites; 0.2 nA soma
  clamp 10-60 ms; 4000 steps of 0.025 ms.
* ``uneven``  -- 10,000 cells, random binary/ternary trees (branch probability 0.7,
  max depth 8), CV count log-uniform 50-2000 at ~10 CVs per 100 um; the small mix
  plus HCN_HM1992 0.01 mS/cm^2 (E -43 mV) and K_Leak everywhere; each conductance
  scaled per cell by lognormal(0, 0.2); soma clamp U(0.05, 0.4) nA from U(5, 20) ms
  to the end; 8000 steps of 0.025 ms.
* ``large``   -- 256 cells of 10,000-20,000 CVs on ~300 branches; the small mix plus
  CalciumDetailed (C_rest = Ci0 = 5e-5 mM, tau 10 ms, d 0.5 um), CaT_HM1992 2.1 and
  AHP_De1994 0.3 mS/cm^2 on dendrites; 500 Poisson pulses per cell (0.1 nA, 1 ms,
  20 Hz per site) at random dendritic CVs; 4000 steps of 0.025 ms.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .batch import CellBatch
from .catalogue import region_record
from .mech import (
    AllRegion,
    CableProperty,
    Channel,
    CurrentClamp,
    CVPerBranchList,
    Ion,
    RootLocation,
    StateProbe,
    at,
    branch_in,
)
from .morph import Branch, Morphology

__all__ = ["CellDesc", "small", "uneven", "large", "desc_to_cell", "descs_to_batch", "CONFIGS"]

DT = 0.025
SOMA_L = 20.0
SOMA_R = 10.0
R_ROOT = 1.0
R_TIP = 0.25


@dataclass
class CellDesc:
    parent: list            # branch parent (branch 0 = soma, parent -1)
    length: list            # um
    r_prox: list
    r_dist: list
    ncv: list
    types: list             # "soma" / "dendrite"
    channels_soma: list     # [(class_name, params)]
    channels_dend: list
    ions_dend: list = field(default_factory=list)
    pulses: list = field(default_factory=list)  # (branch, x, t_on, t_off, amp)
    probes: list = field(default_factory=lambda: [(0, 0.5)])
    v_rest: float = -65.0


def _taper(dist_prox: np.ndarray, dist_dist: np.ndarray, dmax: float):
    rp = R_ROOT + (R_TIP - R_ROOT) * dist_prox / dmax
    rd = R_ROOT + (R_TIP - R_ROOT) * dist_dist / dmax
    return rp, rd


def _finish_tree(parent, length, ncv):
    """Radii by path distance from the soma's distal end, tapering to the farthest tip."""
    nb = len(parent)
    start = np.zeros(nb)
    end = np.zeros(nb)
    for b in range(1, nb):
        start[b] = end[parent[b]] if parent[b] > 0 else 0.0
        end[b] = start[b] + length[b]
    dmax = float(end[1:].max()) if nb > 1 else 1.0
    rp, rd = _taper(start, end, dmax)
    rp[0] = rd[0] = SOMA_R
    return list(rp), list(rd)


# ----------------------------------------------------------------------------- small


def _small_desc(seed: int = 0) -> CellDesc:
    rng = np.random.default_rng(seed)
    parent = [-1]
    depth = [0]
    frontier = [0]
    for d in range(1, 4):
        nxt = []
        for p in frontier:
            for _ in range(2):
                parent.append(p)
                depth.append(d)
                nxt.append(len(parent) - 1)
        frontier = nxt
    nb = len(parent)
    length = [SOMA_L] + list(rng.uniform(50.0, 200.0, size=nb - 1))
    ncv = [1] + [8] * (nb - 1)
    rp, rd = _finish_tree(parent, length, ncv)
    return CellDesc(
        parent=parent,
        length=length,
        r_prox=rp,
        r_dist=rd,
        ncv=ncv,
        types=["soma"] + ["dendrite"] * (nb - 1),
        channels_soma=[("IL", {"g_max": 0.3, "E": -70.0}), ("Na_Ba2002", {"g_max": 120.0}),
                       ("KDR_Ba2002", {"g_max": 36.0})],
        channels_dend=[("IL", {"g_max": 0.3, "E": -70.0}), ("CaL_IS2008", {"g_max": 2.0})],
        pulses=[(0, 0.5, 10.0, 60.0, 0.2)],
    )


def small(n_cells: int = 16, seed: int = 0) -> list[CellDesc]:
    d = _small_desc(seed)
    return [d] * n_cells


# ----------------------------------------------------------------------------- uneven


def _random_tree(rng, n_dend_cv: int, p_branch: float, max_depth: int, max_branches: int):
    parent = [-1]
    depth = [0]
    queue = []
    n_primary = int(rng.integers(2, 4))
    for _ in range(n_primary):
        parent.append(0)
        depth.append(1)
        queue.append(len(parent) - 1)
    qi = 0
    while qi < len(queue):
        b = queue[qi]
        qi += 1
        if depth[b] >= max_depth or rng.random() >= p_branch:
            continue
        k = int(rng.integers(2, 4))
        if len(parent) - 1 + k > max_branches:
            continue
        for _ in range(k):
            parent.append(b)
            depth.append(depth[b] + 1)
            queue.append(len(parent) - 1)
    return parent


def _uneven_desc(seed: int, i: int, n_range=(50, 2000)) -> CellDesc:
    rng = np.random.default_rng([seed, i])
    n_total = int(round(math.exp(rng.uniform(math.log(float(n_range[0])), math.log(float(n_range[1]))))))
    n_dend = max(n_total - 1, 3)
    parent = _random_tree(rng, n_dend, 0.7, 8, max(3, n_dend // 4))
    nb = len(parent)
    w = rng.uniform(0.5, 1.5, size=nb - 1)
    L_total = 10.0 * n_dend
    lengths = w / w.sum() * L_total
    ncv_d = np.maximum(1, np.ceil(lengths / 10.0 - 1e-9)).astype(int)
    length = [SOMA_L] + list(lengths)
    ncv = [1] + list(ncv_d)
    rp, rd = _finish_tree(parent, length, ncv)
    f = np.exp(rng.normal(0.0, 0.2, size=6))  # IL, Na, KDR, CaL, HCN, K_Leak
    amp = float(rng.uniform(0.05, 0.4))
    onset = float(rng.uniform(5.0, 20.0))
    leak = ("IL", {"g_max": 0.3 * f[0], "E": -70.0})
    hcn = ("HCN_HM1992", {"g_max": 0.01 * f[4], "E": -43.0})
    kleak = ("K_Leak", {"g_max": 0.005 * f[5]})
    return CellDesc(
        parent=parent,
        length=length,
        r_prox=rp,
        r_dist=rd,
        ncv=ncv,
        types=["soma"] + ["dendrite"] * (nb - 1),
        channels_soma=[leak, ("Na_Ba2002", {"g_max": 120.0 * f[1]}), ("KDR_Ba2002", {"g_max": 36.0 * f[2]}), hcn,
                       kleak],
        channels_dend=[leak, ("CaL_IS2008", {"g_max": 2.0 * f[3]}), hcn, kleak],
        pulses=[(0, 0.5, onset, 1e9, amp)],
    )


def uneven(n_cells: int = 10000, seed: int = 1, indices=None, n_range=(50, 2000)) -> list[CellDesc]:
    """Cells with log-uniform compartment counts in ``n_range`` (default: the uneven
    population, 50 to 2,000); a smaller range gives a population of small cells."""
    idx = range(n_cells) if indices is None else indices
    return [_uneven_desc(seed, int(i), n_range) for i in idx]


# ----------------------------------------------------------------------------- large


def _large_desc(seed: int, i: int, n_range=(10000, 20000), n_branches: int = 300, duration: float = 100.0,
                n_pulses: int = 500) -> CellDesc:
    rng = np.random.default_rng([seed, i])
    n_total = int(rng.integers(n_range[0], n_range[1] + 1))
    # binary growth until ~n_branches dendritic branches
    parent = [-1, 0, 0]
    leaves = [1, 2]
    while len(parent) - 1 + 2 <= n_branches:
        j = int(rng.integers(0, len(leaves)))
        b = leaves.pop(j)
        for _ in range(2):
            parent.append(b)
            leaves.append(len(parent) - 1)
    nb = len(parent)
    n_dend = n_total - 1
    w = rng.uniform(0.5, 1.5, size=nb - 1)
    ncv_d = np.maximum(1, np.floor(w / w.sum() * n_dend)).astype(int)
    ncv_d[0] += n_dend - int(ncv_d.sum())
    lengths = 10.0 * ncv_d
    length = [SOMA_L] + list(lengths.astype(float))
    ncv = [1] + list(ncv_d)
    rp, rd = _finish_tree(parent, length, ncv)
    # 500 Poisson pulses: sites at random dendritic CVs, 20 Hz per site
    rate = 20.0 / 1000.0  # per ms
    pulses = []
    cum = np.cumsum(ncv_d)
    dend_cv_total = int(cum[-1])
    while len(pulses) < n_pulses:
        k = int(rng.integers(0, dend_cv_total))
        bi = int(np.searchsorted(cum, k, side="right"))
        kk = k - (int(cum[bi - 1]) if bi > 0 else 0)
        b = bi + 1
        x = (kk + 0.5) / int(ncv_d[bi])
        t = rng.exponential(1.0 / rate)
        while t < duration and len(pulses) < n_pulses:
            pulses.append((b, x, float(t), float(t) + 1.0, 0.1))
            t += rng.exponential(1.0 / rate)
    leak = ("IL", {"g_max": 0.3, "E": -70.0})
    return CellDesc(
        parent=parent,
        length=length,
        r_prox=rp,
        r_dist=rd,
        ncv=ncv,
        types=["soma"] + ["dendrite"] * (nb - 1),
        channels_soma=[leak, ("Na_Ba2002", {"g_max": 120.0}), ("KDR_Ba2002", {"g_max": 36.0})],
        channels_dend=[leak, ("CaL_IS2008", {"g_max": 2.0}), ("CaT_HM1992", {"g_max": 2.1}),
                       ("AHP_De1994", {"g_max": 0.3})],
        ions_dend=[("CalciumDetailed", {"C_rest": 5e-5, "tau": 10.0, "d": 0.5, "Ci_initializer": 5e-5})],
        pulses=pulses,
    )


def large(n_cells: int = 256, seed: int = 2, indices=None, **kw) -> list[CellDesc]:
    idx = range(n_cells) if indices is None else indices
    return [_large_desc(seed, int(i), **kw) for i in idx]


# ----------------------------------------------------------------------------- conversions


def desc_to_cell(d: CellDesc, *, pop_size: int = 1, **cell_kw):
    """Declared Cell (Morphology + paint/place) for one description."""
    from .cell import Cell

    soma = Branch.from_lengths(lengths=[d.length[0]], radii=[d.r_prox[0], d.r_dist[0]], type="soma")
    morpho = Morphology.from_root(soma, name="soma")
    for b in range(1, len(d.parent)):
        br = Branch.from_lengths(lengths=[d.length[b]], radii=[d.r_prox[b], d.r_dist[b]], type="dendrite")
        morpho.attach(parent=int(d.parent[b]), child_branch=br, child_name=f"dend_{b}", parent_x=1.0, child_x=0.0)
    cell = Cell(morpho, pop_size=pop_size, cv_policy=CVPerBranchList(tuple(int(n) for n in d.ncv)), **cell_kw)
    cell.paint(AllRegion(), CableProperty(resting_potential=d.v_rest))
    cell.paint(branch_in("type", "soma"), *[Channel(n, **p) for n, p in d.channels_soma])
    cell.paint(branch_in("type", "dendrite"), *[Channel(n, **p) for n, p in d.channels_dend])
    if d.ions_dend:
        cell.paint(branch_in("type", "dendrite"), *[Ion(n, **p) for n, p in d.ions_dend])
    for (b, x, t_on, t_off, amp) in d.pulses:
        loc = RootLocation(x) if b == 0 else at(int(b), x)
        cell.place(loc, CurrentClamp(delay=t_on, durations=t_off - t_on, amplitudes=amp))
    for (b, x) in d.probes:
        cell.place(RootLocation(x) if b == 0 else at(int(b), x), StateProbe())
    return cell


def descs_to_batch(descs: list[CellDesc]) -> CellBatch:
    """Flat batch of many descriptions (two regions per cell: soma, dendrites)."""
    n = len(descs)
    R = 2
    cache: dict[int, tuple] = {}
    nb_tot = sum(len(d.parent) for d in descs)
    br_parent = np.empty(nb_tot, np.int32)
    br_len = np.empty(nb_tot)
    br_rp = np.empty(nb_tot)
    br_rd = np.empty(nb_tot)
    br_ncv = np.empty(nb_tot, np.int32)
    br_region = np.empty(nb_tot, np.int32)
    offs = np.zeros(n + 1, np.int64)
    region_cm = np.ones(n * R)
    region_ra = np.full(n * R, 100.0)
    region_mech = np.zeros(n * R, np.uint32)
    region_params = np.zeros((n * R, _abi.BC_NPARAM))
    pc, pb, px, pon, poff, pamp = [], [], [], [], [], []
    qc, qb, qx = [], [], []
    k = 0
    cable = CableProperty()
    for c, d in enumerate(descs):
        nb = len(d.parent)
        sl = slice(k, k + nb)
        br_parent[sl] = d.parent
        br_len[sl] = d.length
        br_rp[sl] = d.r_prox
        br_rd[sl] = d.r_dist
        br_ncv[sl] = d.ncv
        br_region[sl] = [0 if t == "soma" else 1 for t in d.types]
        k += nb
        offs[c + 1] = k
        key = id(d)
        if key not in cache:
            cab = CableProperty(resting_potential=d.v_rest) if d.v_rest != cable.resting_potential else cable
            soma = region_record([Channel(nm, **p) for nm, p in d.channels_soma], cab)
            dend = region_record([Channel(nm, **p) for nm, p in d.channels_dend] +
                                 [Ion(nm, **p) for nm, p in d.ions_dend], cab)
            cache[key] = (soma, dend)
        (ms, ps), (md, pd) = cache[key]
        region_mech[c * R] = ms
        region_mech[c * R + 1] = md
        region_params[c * R] = ps
        region_params[c * R + 1] = pd
        for (b, x, t_on, t_off, amp) in d.pulses:
            pc.append(c)
            pb.append(b)
            px.append(x)
            pon.append(t_on)
            poff.append(t_off)
            pamp.append(amp)
        for (b, x) in d.probes:
            qc.append(c)
            qb.append(b)
            qx.append(x)
    return CellBatch(
        n_regions=R,
        cell_branch_offsets=offs,
        branch_parent=br_parent,
        branch_parent_x=np.where(br_parent >= 0, 1.0, 0.0),
        branch_child_x=np.zeros(nb_tot),
        branch_ncv=br_ncv,
        branch_region=br_region,
        branch_seg_offsets=np.arange(nb_tot + 1, dtype=np.int64),
        seg_length=br_len,
        seg_r_prox=br_rp,
        seg_r_dist=br_rd,
        region_cm=region_cm,
        region_ra=region_ra,
        region_mech=region_mech,
        region_params=region_params,
        pulse_cell=np.asarray(pc, np.int32),
        pulse_branch=np.asarray(pb, np.int32),
        pulse_x=np.asarray(px),
        pulse_t_on=np.asarray(pon),
        pulse_t_off=np.asarray(poff),
        pulse_amp=np.asarray(pamp),
        probe_cell=np.asarray(qc, np.int32),
        probe_branch=np.asarray(qb, np.int32),
        probe_x=np.asarray(qx),
    )


CONFIGS = {
    "small": dict(make=small, n_steps=4000, dt=DT),
    "uneven": dict(make=uneven, n_steps=8000, dt=DT),
    "large": dict(make=large, n_steps=4000, dt=DT),
}
