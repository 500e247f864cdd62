"""Learned stand-ins for distal dendritic subtrees (GRU ports).

Every subtree of branches at depth >= ``cut_depth`` (the soma is depth 0) is cut
off its parent branch and replaced by a *port* on that parent's distal end.
Each step the port injects ``I = g (e + y_scale * y - V_end)`` nA into the end
point's row: ``g`` is the removed subtree's passive input conductance (uS) and
``e`` its passive reversal potential, so the linear part of the load is exact at
DC and implicit in the solve; ``y`` is the output of a GRU (hidden 64, BF16
tensor-core weights) that is fed the attachment compartment's voltage, the
stimulus current the subtree received and two static features of the subtree
(log input conductance, log membrane time constant), and learns the rest of the
subtree's current.  The GRU runs inside the step kernel.

Training data are trajectories of the *plain* solver on full cells: the port
current a subtree really delivered is ``g_att (V_end - V_att)`` (``g_att``: the
axial conductance between the attachment CV and the end point, whose row is
algebraic), recorded every step with probes.  Training uses the library's own
forward / backward / Adam kernels (:mod:`braincell_gb300.gru`).

A port whose input leaves the training envelope flags its cell; after a run,
flagged cells are run again with their full morphology (per-cell fallback).
"""

from __future__ import annotations

import gc
import math
import os
import time
from dataclasses import dataclass, field, replace

import numpy as np

from . import _abi
from .workloads import CellDesc, descs_to_batch

__all__ = ["CUT_DEPTH", "PACKAGED_MODEL", "Port", "SurrogateModel", "branch_depths", "reduce_desc", "passive_subtree",
           "ports_to_batch", "make_training_descs", "collect_trajectories", "train_surrogate", "run_surrogate",
           "fallback_plan_options", "SurrogateRunner",
           "SurrogateRun", "save_model", "load_model"]

CUT_DEPTH = 4
PACKAGED_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_uneven.npz")
NPARAM = 3 * 64 * 64 + 3 * 64 * 4 + 2 * 3 * 64 + 64 + 1
V_SCALE = 10.0       # mV
# Default launch shape of reduced plans: a tile with ports also holds the GRU
# weight fragments (32 KB of shared memory), so two tiles per SM fit ~1,800
# nodes each; 384 threads is the port kernel's register budget at two per SM.
PORT_TILE_NODES = 1800
PORT_THREADS = 384
# Serial-walk length of the reduced tiles' warp slots: a GB300 sweep of the 10,000-cell
# reduced run (1,000-step launches) gave 76.4 / 74.4 / 75.4 ms per 1,000 steps at 4 / 6 / 10.
PORT_LANE_NODES = 6
# Reduced plans launch their longest tiles first (tile_order 1): 74.0-74.3 against
# 74.7-74.9 ms per 1,000 steps in build order on the same GB300.
PORT_TILE_ORDER = 1
# Fallback (full-morphology) plans run the kernel without ports in large tiles.
FALLBACK_TILE_NODES = 2500
S_SCALE = 0.1        # nA: stimulus input scale (the step kernel's constant)
G_REF = 0.005        # uS, feature reference
TAU_REF = 5.0        # ms, feature reference


# ----------------------------------------------------------------------------- structure
def branch_depths(parent) -> np.ndarray:
    d = np.zeros(len(parent), np.int64)
    for b in range(1, len(parent)):
        d[b] = d[parent[b]] + 1
    return d


@dataclass
class Port:
    branch: int                # attachment branch, reduced numbering
    branch_full: int           # the same branch, original numbering
    subtree: list              # removed branches (original numbering)
    g: float                   # uS: passive input conductance of the subtree
    e: float                   # mV: passive reversal potential
    c_pf: float                # pF: membrane capacitance of the subtree
    stim: list = field(default_factory=list)  # (t_on, t_off, amp_nA) received by the subtree
    n_cv: int = 0              # compartments the port stands in for

    @property
    def feat(self) -> tuple:
        tau = self.c_pf / self.g * 1e-3  # pF / uS = us -> ms
        return (math.log(self.g / G_REF), math.log(tau / TAU_REF))


def _membrane(d: CellDesc) -> tuple[float, float]:
    """Passive (g_m in mS/cm^2, E_m in mV) of the dendritic membrane at rest."""
    from .catalogue import region_record
    from .mech import CableProperty, Channel

    _, rec = region_record([Channel(n, **p) for n, p in d.channels_dend], CableProperty(resting_potential=d.v_rest))
    P = _abi
    gl, el = rec[P.BC_P_IL_G], rec[P.BC_P_IL_E]
    gk, ek = rec[P.BC_P_KLEAK_G], rec[P.BC_P_EK]
    pinf = 1.0 / (1.0 + math.exp((d.v_rest + 75.0) / 5.5))
    gh, eh = rec[P.BC_P_HCN_G] * pinf, rec[P.BC_P_HCN_E]
    g = gl + gk + gh
    return g, (gl * el + gk * ek + gh * eh) / g if g > 0 else d.v_rest


def _desc_geometry(d: CellDesc):
    """All CVs of a description at once: per branch (area, rpx, rdx) as Python lists."""
    n = np.asarray(d.ncv, np.int64)
    L = np.asarray(d.length, float)
    rp, rdist = np.asarray(d.r_prox, float), np.asarray(d.r_dist, float)
    m = 2 * n
    br = np.repeat(np.arange(n.size), m)
    k = np.arange(int(m.sum())) - np.repeat(np.concatenate([[0], np.cumsum(m)[:-1]]), m)
    x0, x1 = k / m[br], (k + 1) / m[br]
    r0 = rp[br] + (rdist[br] - rp[br]) * x0
    r1 = rp[br] + (rdist[br] - rp[br]) * x1
    seg = L[br] / m[br]
    area = np.pi * (r0 + r1) * np.sqrt(seg ** 2 + (r1 - r0) ** 2)
    res = 100.0 * seg / (np.pi * r0 * r1) * 1e-2  # MOhm at 100 ohm cm
    cv_area = (area[0::2] + area[1::2]).tolist()
    rpx, rdx = res[0::2].tolist(), res[1::2].tolist()
    off = np.concatenate([[0], np.cumsum(n)]).tolist()
    return [(cv_area[off[b]:off[b + 1]], rpx[off[b]:off[b + 1]], rdx[off[b]:off[b + 1]]) for b in range(n.size)]


def _branch_passive(d: CellDesc, g_m: float, need) -> tuple[dict, dict]:
    """Per branch in ``need`` (closed under children): the passive input conductance
    (uS) seen from its proximal end looking distally, and its subtree's capacitance (pF)."""
    kids = [[] for _ in d.parent]
    for b in range(1, len(d.parent)):
        kids[d.parent[b]].append(b)
    geo = _desc_geometry(d)
    gms = g_m * 1e-5  # mS/cm^2 * um^2 -> uS
    G, Cp = {}, {}
    for b in sorted(need, key=lambda q: -q):  # children have larger indices than their parent
        area, rpx, rdx = geo[b]
        g_end = sum(G[c] for c in kids[b])
        g = gms * area[-1] + (1.0 / (rdx[-1] + 1.0 / g_end) if g_end > 0 else 0.0)
        for k in range(len(area) - 2, -1, -1):
            g = gms * area[k] + 1.0 / (rdx[k] + rpx[k + 1] + 1.0 / g)
        G[b] = 1.0 / (rpx[0] + 1.0 / g)
        Cp[b] = sum(area) * 1e-2 + sum(Cp[c] for c in kids[b])  # 1 uF/cm^2 -> pF
    return G, Cp


def passive_subtree(d: CellDesc, roots, g_m: float) -> tuple[float, float]:
    """(input conductance in uS, capacitance in pF) of the subtrees rooted at `roots`."""
    need = set()
    stack = list(roots)
    while stack:
        b = stack.pop()
        need.add(b)
        stack.extend(c for c in range(1, len(d.parent)) if d.parent[c] == b)
    G, Cp = _branch_passive(d, g_m, need)
    return sum(G[b] for b in roots), sum(Cp[b] for b in roots)


_MEMBRANE_CACHE: dict = {}


def _membrane_cached(d: CellDesc) -> tuple[float, float]:
    key = (repr(d.channels_dend), d.v_rest)
    if key not in _MEMBRANE_CACHE:
        _MEMBRANE_CACHE[key] = _membrane(d)
    return _MEMBRANE_CACHE[key]


def reduce_desc(d: CellDesc, cut_depth: int = CUT_DEPTH) -> tuple[CellDesc, list[Port]]:
    """The cell without its subtrees at depth >= cut_depth, and one port per cut point."""
    depth = branch_depths(d.parent)
    keep = [b for b in range(len(d.parent)) if depth[b] < cut_depth]
    new = {b: i for i, b in enumerate(keep)}
    g_m, e_m = _membrane_cached(d)
    owner = {}   # removed branch -> port attachment branch (original numbering)
    for b in range(len(d.parent)):
        if depth[b] >= cut_depth:
            a = b
            while depth[a] > cut_depth:
                a = d.parent[a]
            owner[b] = d.parent[a]
    ports = []
    G, Cp = _branch_passive(d, g_m, owner.keys()) if owner else ({}, {})
    for p in sorted(set(owner.values())):
        roots = [b for b in range(1, len(d.parent)) if d.parent[b] == p and depth[b] == cut_depth]
        sub = [b for b, o in owner.items() if o == p]
        g, c = sum(G[b] for b in roots), sum(Cp[b] for b in roots)
        ports.append(Port(branch=new[p], branch_full=p, subtree=sorted(sub), g=g, e=e_m, c_pf=c,
                          n_cv=int(sum(d.ncv[b] for b in sub))))
    by_full = {pt.branch_full: pt for pt in ports}
    pulses = []
    for (b, x, t_on, t_off, amp) in d.pulses:
        if b in new:
            pulses.append((new[b], x, t_on, t_off, amp))
        else:
            by_full[owner[b]].stim.append((t_on, t_off, amp))
    probes = [(new[b], x) for (b, x) in d.probes if b in new]
    rd = replace(d, parent=[new[d.parent[b]] if d.parent[b] >= 0 else -1 for b in keep],
                 length=[d.length[b] for b in keep], r_prox=[d.r_prox[b] for b in keep],
                 r_dist=[d.r_dist[b] for b in keep], ncv=[d.ncv[b] for b in keep],
                 types=[d.types[b] for b in keep], pulses=pulses, probes=probes)
    return rd, ports


def ports_to_batch(descs, ports_per_cell, batch=None):
    """Batch of the (reduced) descriptions with the port arrays filled in."""
    b = descs_to_batch(descs) if batch is None else batch
    pc, pb, pg, pe, pf = [], [], [], [], []
    qp, qon, qoff, qamp = [], [], [], []
    for c, ports in enumerate(ports_per_cell):
        for pt in ports:
            k = len(pc)
            pc.append(c)
            pb.append(pt.branch)
            pg.append(pt.g)
            pe.append(pt.e)
            pf.append(pt.feat)
            for (t_on, t_off, amp) in pt.stim:
                qp.append(k)
                qon.append(t_on)
                qoff.append(t_off)
                qamp.append(amp)
    b.port_cell = np.asarray(pc, np.int32)
    b.port_branch = np.asarray(pb, np.int32)
    b.port_g = np.asarray(pg, float)
    b.port_e = np.asarray(pe, float)
    b.port_feat = np.asarray(pf, float).reshape(-1, 2)
    b.port_pulse_port = np.asarray(qp, np.int32)
    b.port_pulse_t_on = np.asarray(qon, float)
    b.port_pulse_t_off = np.asarray(qoff, float)
    b.port_pulse_amp = np.asarray(qamp, float)
    return b


# ----------------------------------------------------------------------------- model
@dataclass
class SurrogateModel:
    theta: np.ndarray             # flat FP32 GRU parameters
    v_scale: float = V_SCALE
    y_scale: float = 1.0
    env_v: tuple = (-1e4, 1e4)    # envelope of V_att - e (mV)
    env_dvdt: float = 1e9         # envelope of |dV_att / dt| (mV/ms)
    cut_depth: int = CUT_DEPTH
    info: dict = field(default_factory=dict)

    def norm(self) -> np.ndarray:
        return np.array([self.v_scale, self.y_scale, self.env_v[0], self.env_v[1], self.env_dvdt], np.float32)


def save_model(m: SurrogateModel, path: str) -> None:
    import json

    np.savez(path, theta=np.asarray(m.theta, np.float32), norm=m.norm(), cut_depth=m.cut_depth,
             info=json.dumps(m.info))


def load_model(path: str) -> SurrogateModel:
    import json

    z = np.load(path, allow_pickle=False)
    nm = z["norm"]
    return SurrogateModel(theta=z["theta"].astype(np.float32), v_scale=float(nm[0]), y_scale=float(nm[1]),
                          env_v=(float(nm[2]), float(nm[3])), env_dvdt=float(nm[4]), cut_depth=int(z["cut_depth"]),
                          info=json.loads(str(z["info"])))


# ----------------------------------------------------------------------------- training data
def make_training_descs(n_cells: int, seed: int = 3, cut_depth: int = CUT_DEPTH, duration: float = 200.0,
                        rate=(5.0, 50.0), amp=(0.02, 0.2), pulse_ms: float = 1.0, quiet: float = 0.5):
    """Cells of the uneven-morphology family driven by a random soma clamp plus
    Poisson current pulses (rate and amplitude per subtree drawn from the given
    ranges) at random compartments of the distal subtrees; a share ``quiet`` of
    the subtrees gets no pulses, so that the unstimulated regime is covered."""
    from .workloads import uneven

    out = []
    for k, d in enumerate(uneven(n_cells, seed=seed)):
        rng = np.random.default_rng([seed, 7, k])
        _, ports = reduce_desc(d, cut_depth)
        pulses = list(d.pulses)
        for pt in ports:
            if rng.random() < quiet:
                continue
            lam = rng.uniform(*rate) / 1000.0
            a = rng.uniform(*amp)
            cv = [(b, (i + 0.5) / d.ncv[b]) for b in pt.subtree for i in range(d.ncv[b])]
            t = rng.exponential(1.0 / lam)
            while t < duration:
                b, x = cv[int(rng.integers(len(cv)))]
                pulses.append((b, x, float(t), float(t) + pulse_ms, float(a)))
                t += rng.exponential(1.0 / lam)
        out.append(replace(d, pulses=pulses))
    return out


def _g_att(d: CellDesc, b: int) -> float:
    """Axial conductance (uS) between the last CV midpoint of branch b and its end."""
    return 1.0 / _desc_geometry(d)[b][2][-1]


def collect_trajectories(descs, n_steps: int = 8000, dt: float = 0.025, cut_depth: int = CUT_DEPTH,
                         precision: str = "f32", device: int = 0, y_scale: float | None = None):
    """Run the full cells on the GPU and return (x [n_port, T, 4], y_raw [n_port, T], meta).

    y_raw is the port output that reproduces the subtree current in mV:
    (I_sub + g (V_end - e)) / g with I_sub = g_att (V_end - V_att)."""
    from .runtime import Plan

    full, ports_all, probe_rows = [], [], []
    for d in descs:
        _, ports = reduce_desc(d, cut_depth)
        probes = list(d.probes)
        rows = []
        for pt in ports:
            b = pt.branch_full
            rows.append((len(probes), len(probes) + 1))
            probes += [(b, 1.0 - 0.5 / d.ncv[b]), (b, 1.0)]
        full.append(replace(d, probes=probes))
        ports_all.append(ports)
        probe_rows.append(rows)
    batch = descs_to_batch(full)
    plan = Plan(batch, precision=precision, record_every=1, device=device)
    plan.run(n_steps, dt)
    tr = plan.traces()        # [n_probes, T]
    plan.close()
    base = np.concatenate([[0], np.cumsum([len(f.probes) for f in full])])
    xs, ys, meta = [], [], []
    t_steps = np.arange(n_steps) * dt
    for c, (d, ports, rows) in enumerate(zip(full, ports_all, probe_rows)):
        for pt, (ia, ie) in zip(ports, rows):
            va = np.concatenate([[d.v_rest], tr[base[c] + ia]])   # V_att^0 .. V_att^T
            ve = np.concatenate([[d.v_rest], tr[base[c] + ie]])
            i_sub = _g_att(d, pt.branch_full) * (ve[1:] - va[1:])
            y = (i_sub + pt.g * (ve[1:] - pt.e)) / pt.g
            S = np.zeros(n_steps)
            for (t_on, t_off, amp) in pt.stim:
                S[(t_steps >= t_on) & (t_steps < t_off)] += amp
            x = np.empty((n_steps, 4))
            x[:, 0] = (va[:-1] - pt.e) / V_SCALE
            x[:, 1] = S / S_SCALE
            x[:, 2], x[:, 3] = pt.feat
            xs.append(x)
            ys.append(y)
            meta.append((c, pt))
    return np.asarray(xs, np.float32), np.asarray(ys), meta


def _envelope(x: np.ndarray, dt: float) -> tuple[tuple, float]:
    """Training envelope: the 0.1-99.9 percentile range of V_att - e widened by half
    its width on each side, and twice the 99.9th percentile of |dV_att/dt|."""
    v = x[:, :, 0].astype(np.float64) * V_SCALE
    lo, hi = np.percentile(v, [0.1, 99.9])
    w = hi - lo
    dv = np.abs(np.diff(v, axis=1)) / dt
    return (float(lo - 0.5 * w), float(hi + 0.5 * w)), float(2.0 * np.percentile(dv, 99.9))


def train_surrogate(n_cells: int = 460, *, seed: int = 3, n_steps: int = 8000, dt: float = 0.025, epochs: int = 60,
                    batch: int = 512, window: int = 400, lr: float = 1e-3, lr_final: float | None = 1e-4,
                    time_budget_s: float | None = None, val_frac: float = 0.1, device: int = 0,
                    cut_depth: int = CUT_DEPTH, quiet: float = 0.5, verbose: bool = False):
    """Generate trajectories with the plain solver, train the GRU on the GPU, return the model."""
    from .gru import GRUTrainer, init_params

    t0 = time.perf_counter()
    descs = make_training_descs(n_cells, seed=seed, cut_depth=cut_depth, duration=n_steps * dt, quiet=quiet)
    x, y_raw, meta = collect_trajectories(descs, n_steps, dt, cut_depth, device=device)
    t_data = time.perf_counter() - t0
    y_scale = float(np.std(y_raw)) or 1.0
    y = (y_raw / y_scale).astype(np.float32)
    rng = np.random.default_rng(seed)
    idx = rng.permutation(len(x))
    n_val = max(1, int(val_frac * len(x)))
    vi, ti = idx[:n_val], idx[n_val:]
    tr = GRUTrainer(x[ti], y[ti], init_params(seed), batch=batch, window=window, lr=lr, device=device, seed=seed)
    v0 = tr.evaluate(x[vi], y[vi])
    log = tr.train(epochs=epochs, time_budget_s=time_budget_s, lr_final=lr_final)
    v1 = tr.evaluate(x[vi], y[vi])
    env_v, env_dvdt = _envelope(x, dt)
    info = dict(n_cells=n_cells, seed=seed, n_traj=int(len(x)), n_train=int(len(ti)), n_val=int(n_val),
                n_steps=n_steps, dt=dt, epochs=log.epochs, updates=log.updates, train_s=round(log.seconds, 2),
                data_s=round(t_data, 2), val_mse_before=v0, val_mse_after=v1,
                train_loss_first=log.loss[0] if log.loss else None, train_loss_last=log.loss[-1] if log.loss else None,
                batch=batch, window=window, lr=lr, lr_final=lr_final, quiet=quiet)
    if verbose:
        print(info)
    return SurrogateModel(theta=tr.theta(), y_scale=y_scale, env_v=env_v, env_dvdt=env_dvdt, cut_depth=cut_depth,
                          info=info)


# ----------------------------------------------------------------------------- running
def fallback_plan_options(descs, base: dict | None = None, threads: int = 512, n_sm: int = 152) -> dict:
    """Plan options for the full solve of fallback cells.  The solve runs next to
    the reduced launches, and its time is bounded by the step latency of its
    tiles, not by throughput: cells are packed into few full-size tiles so that
    they hold as few of the SMs the reduced run needs as possible."""
    kw = dict(base or {})
    kw["tile_nodes"] = FALLBACK_TILE_NODES
    kw["threads_per_tile"] = threads
    kw["threads_big"] = max(threads, 512)
    kw["threads_global"] = 512
    kw.pop("lane_nodes", None)
    kw.pop("tile_order", None)
    return kw


@dataclass
class SurrogateRun:
    reduced_cv: int
    full_cv: int
    n_ports: int
    fallback_cells: np.ndarray
    wall_ms: float                # reset to the end of the last fallback run (host clock)
    launches: int                 # kernel launches: resets, reduced-plan launches, fallback launches
    spikes: list                  # per cell: soma spike times (ms), fallback cells from the full solve
    traces: np.ndarray | None = None  # [n_cells, T] soma voltage when record_every > 0
    full_cells: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))  # kept at full morphology
    # device clock from the reset: "reduced_ms" at the end of the last reduced launch,
    # "fallbacks" one (steps seen when the flags were read, cells, start ms, end ms) per batch
    timeline: dict = field(default_factory=dict)

    @property
    def fallback_rate(self) -> float:
        """Fallbacks over the cells that ran with ports."""
        return float(self.fallback_cells.size) / max(len(self.spikes) - self.full_cells.size, 1)


class SurrogateRunner:
    """Cells with their distal subtrees replaced by GRU ports, with per-cell fallback.

    The reduced plan runs launch by launch; after each launch the envelope flags
    are read, the next launch is queued first, and the cells that newly left the
    envelope start their full-morphology solve from t = 0 on a second stream, so
    the fallback runs alongside the remaining reduced launches.  ``model=None``
    runs the ports with y = 0 (only the passive linear load): the method without
    the network."""

    def __init__(self, descs, model: SurrogateModel | None, *, precision: str = "f32", record_every: int = 0,
                 device: int = 0, plan_kw: dict | None = None, fallback: bool = True, full_cells=None,
                 full_plan_kw: dict | None = None, fallback_kw: dict | None = None, fallback_priority: int = -1,
                 tail_split: bool = True):
        """``full_cells``: indices of cells that keep their full morphology for the
        whole run (a mixed population); they run from t = 0 in a plain plan of
        their own (``full_plan_kw``, default: the fallback's launch shape) on a
        stream beside the reduced launches.  ``fallback_kw`` overrides plan options
        of the fallback solves, and ``fallback_priority`` is their streams' priority
        (-1 high, 0 the reduced launches' own).  ``tail_split`` runs the last launch's
        worth of steps as launches of a half, a quarter and a quarter."""
        from .gru import NPARAM
        from .runtime import Plan

        self.descs = list(descs)
        self.model = model
        self.precision, self.record_every, self.device = precision, int(record_every), int(device)
        self.plan_kw = dict(plan_kw or {})
        self.plan_kw.setdefault("tile_nodes", PORT_TILE_NODES)
        self.plan_kw.setdefault("lane_nodes", PORT_LANE_NODES)
        self.plan_kw.setdefault("tile_order", PORT_TILE_ORDER)
        for k in ("threads_per_tile", "threads_big", "threads_global"):
            self.plan_kw.setdefault(k, PORT_THREADS)
        self.fallback = fallback and model is not None
        self.fallback_kw = dict(fallback_kw or {})
        self.fallback_priority = int(fallback_priority)
        self.tail_split = bool(tail_split)
        n = len(self.descs)
        full = np.zeros(n, bool)
        if full_cells is not None:
            full[np.asarray(full_cells, dtype=np.int64)] = True
        self.full_idx = np.nonzero(full)[0]
        self.red_idx = np.nonzero(~full)[0]
        red, ports = [], []
        for i in self.red_idx:
            r, pts = reduce_desc(self.descs[i], model.cut_depth if model else CUT_DEPTH)
            red.append(replace(r, probes=[(0, 0.5)]))
            ports.append(pts)
        self.batch = ports_to_batch(red, ports)
        self.plan = Plan(self.batch, precision=precision, record_every=record_every, max_spikes=256, device=device,
                         **self.plan_kw)
        self.n_ports = int(self.batch.port_cell.size)
        if self.n_ports:
            if model is None:
                self.plan.set_surrogate(np.zeros(NPARAM, np.float32), (V_SCALE, 1.0, -1e4, 1e4, 1e9))
            else:
                self.plan.set_surrogate(model.theta, model.norm())
        self.full_plan = None
        if self.full_idx.size:
            fd = [replace(self.descs[i], probes=[(0, 0.5)]) for i in self.full_idx]
            kw = dict(full_plan_kw) if full_plan_kw is not None else fallback_plan_options(fd, self.plan_kw)
            self.full_plan = Plan(descs_to_batch(fd), precision=precision, record_every=record_every, max_spikes=256,
                                  device=device, **kw)
        self.full_cv = int(sum(int(sum(d.ncv)) for d in self.descs))

    def _fallback_plan(self, cells, n_steps: int):
        from .runtime import Plan

        fd = [replace(self.descs[i], probes=[(0, 0.5)]) for i in cells]
        kw = fallback_plan_options(fd, self.plan_kw, threads=512)
        # the whole run in one launch: each fallback tile takes an SM slot once and keeps
        # it, instead of queueing for a free slot behind the reduced tiles every launch
        kw["steps_per_launch"] = max(1, int(n_steps))
        kw.update(self.fallback_kw)
        return Plan(descs_to_batch(fd), precision=self.precision, record_every=self.record_every, max_spikes=256,
                    device=self.device, **kw)

    def run(self, n_steps: int, dt: float = 0.025) -> SurrogateRun:
        import torch

        if not hasattr(self, "_main"):
            # a non-blocking stream: the legacy default stream would order the
            # fallback streams' work behind the reduced launches
            self._main = torch.cuda.Stream(self.device)
        torch.cuda.current_stream(self.device).synchronize()
        # The host loop below is on the critical path of the fallback (flag reads,
        # plan builds, launches): the cyclic garbage collector is paused for its
        # length, since a full collection of a large heap takes tens of ms.
        gc_on = gc.isenabled()
        gc.disable()
        try:
            return self._run(n_steps, dt)
        finally:
            if gc_on:
                gc.enable()

    def _run(self, n_steps: int, dt: float) -> SurrogateRun:
        import torch

        plan = self.plan
        main = self._main
        sid = int(main.cuda_stream)
        n_red = self.red_idx.size
        spl = int(plan.info["steps_per_launch"])
        watch = self.fallback and self.n_ports > 0
        t0 = time.perf_counter()
        plan.reset(stream=sid)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev0.record(main)
        if self.full_plan is not None:
            # the full-morphology cells of a mixed population: the whole run, enqueued
            # at once on their own stream, beside the reduced launches
            if not hasattr(self, "_full_stream"):
                self._full_stream = torch.cuda.Stream(self.device)
            fs = int(self._full_stream.cuda_stream)
            self.full_plan.reset(stream=fs)
            self.full_plan.run(n_steps, dt, stream=fs, check=False)
        flagged = np.zeros(n_red, bool)
        fallbacks = []
        if not hasattr(self, "_flag_stream"):
            self._flag_stream = torch.cuda.Stream(self.device)
        # two launches stay queued: the flags after launch i are read on a stream that
        # waits for launch i only, while launch i + 1 keeps the GPU busy
        queued = []
        done = 0

        # the first launches are short, so that the envelope exits of the first
        # stimulus onsets are seen (and their full solves started) early
        lead = [max(1, spl // 4), max(1, spl // 4), max(1, spl // 2)]

        def enqueue():
            nonlocal done
            k = min(lead.pop(0) if lead else spl, n_steps - done)
            # the last launch's worth of steps in halves down to a quarter launch, so
            # that an exit near the end is read (and its full solve started) sooner
            r = n_steps - done
            if self.tail_split and not lead and r <= spl:
                k = r if r <= max(1, spl // 4) else max(max(1, spl // 4), r // 2)
            plan.run(k, dt, stream=sid, check=False)
            done += k
            ev = torch.cuda.Event(enable_timing=True)
            ev.record(main)
            queued.append((ev, done))

        enqueue()
        if done < n_steps:
            enqueue()
        last_ev = None
        while queued:
            ev, seen = queued.pop(0)
            last_ev = ev
            flags = None
            if watch:
                self._flag_stream.wait_event(ev)
                flags = plan.surrogate_flags(stream=int(self._flag_stream.cuda_stream))
            else:
                ev.synchronize()
            if done < n_steps:
                enqueue()
            if flags is not None:
                new = np.nonzero((flags != 0) & ~flagged)[0]
                if new.size:
                    flagged[new] = True
                    # high priority: the block scheduler gives the fallback's tiles the
                    # next free SM slots ahead of the queued reduced launches, so the
                    # full solve runs at its own step latency
                    side = torch.cuda.Stream(self.device, priority=self.fallback_priority)
                    fp = self._fallback_plan(self.red_idx[new], n_steps)
                    fs, fe = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    fs.record(side)
                    fp.run(n_steps, dt, stream=int(side.cuda_stream), check=False)
                    fe.record(side)
                    fallbacks.append((new, fp, side, seen, (fs, fe)))
        plan.check(stream=sid)
        for _, fp, side, _, _ in fallbacks:
            fp.check(stream=int(side.cuda_stream))
        if self.full_plan is not None:
            self.full_plan.check(stream=int(self._full_stream.cuda_stream))
        torch.cuda.synchronize(self.device)
        wall = (time.perf_counter() - t0) * 1e3
        timeline = {"reduced_ms": ev0.elapsed_time(last_ev) if last_ev is not None else 0.0,
                    "fallbacks": [(int(seen), int(cells.size), ev0.elapsed_time(fe[0]), ev0.elapsed_time(fe[1]))
                                  for cells, _, _, seen, fe in fallbacks]}
        n = len(self.descs)
        spikes = [None] * n
        traces = None
        red_sp = plan.spikes(stream=sid)
        red_tr = plan.traces(stream=sid) if self.record_every else None
        if red_tr is not None or self.full_plan is not None and self.record_every:
            T = (red_tr if red_tr is not None else self.full_plan.traces()).shape[1]
            traces = np.zeros((n, T))
        for j, i in enumerate(self.red_idx):
            spikes[i] = red_sp[j]
            if traces is not None and red_tr is not None:
                traces[i] = red_tr[j]
        launches = 1 + -(-n_steps // spl) * int(plan.info["n_launch_classes"])
        if self.full_plan is not None:
            fp = self.full_plan
            launches += 1 + -(-n_steps // int(fp.info["steps_per_launch"])) * int(fp.info["n_launch_classes"])
            fsp = fp.spikes()
            ftr = fp.traces() if self.record_every else None
            for j, i in enumerate(self.full_idx):
                spikes[i] = fsp[j]
                if traces is not None:
                    traces[i] = ftr[j]
        for cells, fp, side, _, _ in fallbacks:
            launches += 1 + -(-n_steps // int(fp.info["steps_per_launch"])) * int(fp.info["n_launch_classes"])
            fsp = fp.spikes(stream=int(side.cuda_stream))
            ftr = fp.traces(stream=int(side.cuda_stream)) if self.record_every else None
            for j, i in enumerate(self.red_idx[cells]):
                spikes[i] = fsp[j]
                if traces is not None:
                    traces[i] = ftr[j]
            fp.close()
        return SurrogateRun(reduced_cv=int(plan.n_cv), full_cv=self.full_cv, n_ports=self.n_ports,
                            fallback_cells=self.red_idx[np.nonzero(flagged)[0]], wall_ms=wall, launches=launches,
                            spikes=list(spikes), traces=traces, full_cells=self.full_idx, timeline=timeline)

    def close(self) -> None:
        self.plan.close()
        if self.full_plan is not None:
            self.full_plan.close()


def run_surrogate(descs, model: SurrogateModel | None, n_steps: int, dt: float = 0.025, *, precision: str = "f32",
                  record_every: int = 0, fallback: bool = True, device: int = 0, plan_kw: dict | None = None,
                  full_cells=None):
    """One run of :class:`SurrogateRunner` (the plan is built and released here)."""
    r = SurrogateRunner(descs, model, precision=precision, record_every=record_every, device=device,
                        plan_kw=plan_kw, fallback=fallback, full_cells=full_cells)
    try:
        return r.run(n_steps, dt)
    finally:
        r.close()
