"""Benchmark: compartment-steps/s of the GB300 Cell step on the uneven-morphology workload.

Workload (the configuration the headline metric is quoted on): 10,000 cells with
random binary/ternary dendritic trees (branch probability 0.7, max depth 8, seed 1),
50-2,000 compartments each (log-uniform, ~10 per 100 um), Na/KDR soma, CaL
dendrites, HCN + K_Leak + leak everywhere with per-cell lognormal conductance
factors, soma clamp 0.05-0.4 nA from 5-20 ms; 200 ms at dt = 0.025 ms (8,000
staggered steps), FP32 with float-float voltage.  One benchmark "step" is one
full 200 ms simulation of all 10,000 cells from reset.  Inputs are generated
(seeded), there is no dataset.

``python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
[--workload uneven|large]`` prints one JSON line.  ``--workload large`` measures the
large-cell configuration instead (256 cells of 10,000-20,000 compartments with
dynamic calcium, 4,000 steps; one bench step is one 100 ms simulation).  Under torchrun (N > 1) every rank simulates its own copy of
the workload (replicas only: cells are independent, no data-path collective) and
rank 0 prints the aggregate.
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "compartment-steps/s on 1 GB300, plain vs surrogate at <=0.1 ms spike-time error"
UNIT = "compartment-steps/s"
DT = 0.025
# Per workload: generator, default size, simulated steps and the algorithmic bytes of
# one compartment-step (8 B per mutable FP32 word read and written, 4 B per static
# word read: uneven 5 mutable (V, V_lo, CaL p, q, HCN p) + 4 static (parent, alpha,
# beta, d0) = 56 B; large adds Ci, Ci_lo, CaT p, q, AHP p = 96 B).
WORKLOADS = {
    "uneven": dict(cells=10000, seed=1, sim_steps=8000, bytes=56,
                   text="uneven-morphology batch: 10,000 cells, 50-2000 compartments, 200 ms at dt 0.025 ms "
                        "(8,000 staggered steps), FP32 + float-float V"),
    "large": dict(cells=256, seed=2, sim_steps=4000, bytes=96,
                  text="large cells: 256 cells of 10,000-20,000 compartments on ~300 branches, CalciumDetailed + "
                       "CaT + AHP dendrites, 500 Poisson pulses per cell, 100 ms at dt 0.025 ms (4,000 steps), "
                       "FP32 + float-float V and Ci"),
}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="uneven")
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--sim-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tile-nodes", type=int, default=2500)
    ap.add_argument("--threads", type=int, default=512)
    ap.add_argument("--threads-big", type=int, default=512)
    ap.add_argument("--steps-per-launch", type=int, default=1000)
    ap.add_argument("--lane-nodes", type=int, default=10)
    ap.add_argument("--narrow-lane-nodes", type=int, default=1)
    ap.add_argument("--lane-cell-nodes", type=int, default=0)
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--surrogate-threads", type=int, default=384)
    ap.add_argument("--surrogate-tile-nodes", type=int, default=1800)
    ap.add_argument("--surrogate-lane-nodes", type=int, default=6)
    ap.add_argument("--accuracy-cells", type=int, default=1000)
    ap.add_argument("--mixed-cells", type=int, default=10000)
    ap.add_argument("--mixed-steps", type=int, default=20000)
    ap.add_argument("--no-mixed", action="store_true")
    a = ap.parse_args()
    wl = WORKLOADS[a.workload]
    a.cells = wl["cells"] if a.cells is None else a.cells
    a.sim_steps = wl["sim_steps"] if a.sim_steps is None else a.sim_steps
    if a.workload != "uneven":
        a.no_surrogate = True  # the surrogate is trained on the uneven family
    return a


def _descs(workload, n, seed=None, indices=None):
    from braincell_gb300 import workloads as W

    make = {"uneven": W.uneven, "large": W.large}[workload]
    seed = WORKLOADS[workload]["seed"] if seed is None else seed
    return make(n, seed=seed) if indices is None else make(seed=seed, indices=list(indices))


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _traffic_per_node_launch(workload):
    """Measured DRAM traffic model of the dominant kernel (ncu summary under profiles/).

    A launch moves a fixed part per tile node (the blob staged into shared memory
    once and V written back once) plus a part per node and fused step (the
    mechanism states streamed every step, and for global-memory tiles the blob and
    scratch).  The summary gives both, fitted from ncu captures of launches of two
    lengths on cases larger than L2."""
    name = {"uneven": "tile_step_uneven.json", "large": "tile_step_large.json"}[workload]
    try:
        with open(os.path.join(ROOT, "profiles", name)) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling while the timed region runs: one
    ``nvidia-smi -lms 200`` process for the whole region (one NVML session, no
    process started per sample), its lines read by a thread."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._p = None
        self._t = None

    def _read(self):
        for line in self._p.stdout:
            parts = [x.strip() for x in line.strip().split(",")]
            if len(parts) >= 3:
                self.samples.append(parts)

    def __enter__(self):
        cmd = ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
               "-lms", "200"]
        if shutil.which("stdbuf"):
            cmd = ["stdbuf", "-oL"] + cmd  # a line per sample through the pipe
        try:
            self._p = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self._p = None
            return self
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *exc):
        if self._p is None:
            return
        self._p.terminate()
        try:
            self._p.wait(timeout=10)
        except subprocess.TimeoutExpired:
            self._p.kill()
            self._p.wait(timeout=10)
        if self._t is not None:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if len(s) > 3 + k and s[3 + k] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _cpu_model() -> str:
    """Host CPU name and core count, for the baseline records."""
    import platform

    name = ""
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                k, _, v = line.partition(":")
                if k.strip() in ("model name", "Model", "CPU part") and v.strip():
                    name = v.strip()
                    break
    except OSError:
        pass
    return f"{name or platform.processor() or 'unknown'} ({platform.machine()}, {os.cpu_count()} logical cores)"


def _oracle_cells(indices, workload="uneven"):
    from braincell_gb300 import workloads as W
    from oracle.staggered import OracleCell

    return [OracleCell(W.desc_to_cell(d)) for d in _descs(workload, 0, indices=indices)]


def cpu_baseline(workload="uneven"):
    """The float64 oracle (one core) on a bounded sample of the same workload: the
    cells are built (lowering, assembly, scheduling) before the clock starts, and
    only their time steps are timed."""
    cells, steps = (8, 1000) if workload == "uneven" else (1, 500)
    t0 = time.perf_counter()
    oc = _oracle_cells(range(cells), workload)
    setup = time.perf_counter() - t0
    ncv = sum(c.n_cv for c in oc)
    t0 = time.perf_counter()
    for c in oc:
        for _ in range(steps):
            c.step(DT)
    el = time.perf_counter() - t0
    return {"value": ncv * steps / el, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {cells} cells of the workload ({ncv} compartments) x {steps} steps, float64 NumPy "
                      f"oracle on one core; time steps only",
            "setup_s_untimed": round(setup, 3), "timed_s": round(el, 3), "cpu": _cpu_model()}


def _reference_worker(conn, indices, workload):
    """One process of the reference arm: builds its cells once, then advances them
    by the requested number of steps per message and answers with the work done."""
    cells = _oracle_cells(indices, workload)
    conn.send(sum(c.n_cv for c in cells))
    while True:
        steps = conn.recv()
        if steps is None:
            break
        for c in cells:
            for _ in range(steps):
                c.step(DT)
        conn.send(sum(c.n_cv for c in cells) * steps)
    conn.close()


def run_reference(a):
    """Reference arm: the CPU restatement of the reference path on all host cores.

    One process per core owns a fixed share of the workload's first cells (balanced
    by compartment count), built before any timing; each bench step advances every
    cell by ``steps_per`` time steps, and only those steps are timed."""
    import multiprocessing as mp

    from braincell_gb300 import workloads as W

    rank, world, _ = _dist()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    steps_per = 200 if a.workload == "uneven" else 20
    n_cells = 4 * cores if a.workload == "uneven" else cores
    sizes = [sum(d.ncv) for d in _descs(a.workload, 0, indices=range(n_cells))]
    shares = [[] for _ in range(cores)]
    load = [0] * cores
    for i in sorted(range(n_cells), key=lambda i: -sizes[i]):
        k = load.index(min(load))
        shares[k].append(i)
        load[k] += sizes[i]
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    t0 = time.perf_counter()
    for k in range(cores):
        here, there = ctx.Pipe()
        pr = ctx.Process(target=_reference_worker, args=(there, shares[k], a.workload), daemon=True)
        pr.start()
        pipes.append(here)
        procs.append(pr)
    ncv = sum(p.recv() for p in pipes)
    setup = time.perf_counter() - t0

    def one_step():
        for p in pipes:
            p.send(steps_per)
        return sum(p.recv() for p in pipes)

    for _ in range(a.warmup):
        one_step()
    work = 0
    t_all = time.perf_counter()
    for _ in range(a.steps):
        work += one_step()
    el = time.perf_counter() - t_all
    for p in pipes:
        p.send(None)
    for pr in procs:
        pr.join(timeout=30)
    value = work / el
    sample = (f"{n_cells} cells ({ncv} compartments) x {steps_per} steps per bench step, one process per core, "
              f"cells built before timing ({setup:.1f} s, untimed)")
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * el / a.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOADS[a.workload]["text"], "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
                         "cpu": _cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference (JAX/brainstate) is not installable offline, so its JAX CPU path is unavailable on "
                "this box; its algorithm is timed through the float64 NumPy restatement",
    }
    print(json.dumps(line), flush=True)


def _spike_report(sp, ref, bar_ms=0.1):
    """Spike-time agreement of paired spikes (in order, within cells of equal count):
    median, p99 and max error, the share within ``bar_ms``, and the cells whose
    counts differ (with the spikes they hold in the reference)."""
    e, mis = _spike_errors(sp, ref)
    unpaired = sum(abs(len(x) - len(y)) for x, y in zip(sp, ref))
    return {"median_ms": float(np.median(e)) if e.size else None,
            "p99_ms": float(np.percentile(e, 99)) if e.size else None,
            "max_ms": float(e.max()) if e.size else None,
            "spikes_paired": int(e.size),
            f"share_within_{bar_ms}_ms": float((e <= bar_ms).mean()) if e.size else None,
            "cells_with_spike_count_mismatch": mis, "spikes_unpaired": int(unpaired),
            "spiking_cells_reference": int(sum(1 for y in ref if len(y)))}


def _spike_errors(sp, ref):
    """Spike-time errors (ms) of spikes paired in order within cells of equal count, and
    the number of cells whose counts differ."""
    errs, mis = [], 0
    for x, y in zip(sp, ref):
        if len(x) != len(y):
            mis += 1
        k = min(len(x), len(y))
        if k:
            errs.extend(np.abs(np.asarray(x[:k]) - np.asarray(y[:k])).tolist())
    return np.asarray(errs), mis


def _first_crossing(trace):
    """Index of the first step at which the voltage reaches 0 mV from below (trace
    length if it never does)."""
    hit = np.nonzero((trace[1:] >= 0.0) & (trace[:-1] < 0.0))[0]
    return int(hit[0]) + 1 if hit.size else trace.size


def _onset(trace, dvdt=10.0):
    """Index of the first step whose voltage rate exceeds dvdt mV/ms (trace length if none)."""
    hit = np.nonzero(np.diff(trace) / DT > dvdt)[0]
    return int(hit[0]) + 1 if hit.size else trace.size


def _upstroke(trace, dvdt=10.0):
    """Start of the first spike's upstroke: the last step before the first 0 mV
    crossing whose voltage rate was at most dvdt mV/ms (trace length if no spike)."""
    k = _first_crossing(trace)
    if k >= trace.size:
        return trace.size
    calm = np.nonzero(np.diff(trace[:k]) / DT <= dvdt)[0]
    return int(calm[-1]) + 1 if calm.size else 0


def plain_accuracy(a, descs, local, n_oracle=2):
    """Accuracy of the plain solve, judged by the target's own words.

    * FP32 against the FP64 build of the same kernels (the on-GPU oracle run) on the
      first ``a.accuracy_cells`` cells for the whole simulation: the largest soma
      |dV| before the first 0 mV crossing (and, for reference, before the dV/dt >
      10 mV/ms onset), spike-time differences of paired spikes and the cells whose
      spike counts differ.
    * FP64 against the float64 CPU oracle on ``n_oracle`` cells, whole simulation:
      the largest |dV| over the soma trace, spikes included.
    """
    from dataclasses import replace

    from braincell_gb300 import workloads as W
    from braincell_gb300.runtime import Plan

    n = min(a.accuracy_cells, len(descs))
    sub = [replace(d, probes=[(0, 0.5)]) for d in descs[:n]]
    out = {"cells": n, "steps": a.sim_steps}
    runs = {}
    for prec in ("f32", "f64"):
        p = Plan(W.descs_to_batch(sub), precision=prec, device=local, record_every=1, max_spikes=256)
        p.run(a.sim_steps, DT)
        runs[prec] = (p.traces(), p.spikes())
        p.close()
    (t32, s32), (t64, s64) = runs["f32"], runs["f64"]
    to_cross, to_onset, to_up, gap = [], [], [], []
    for c in range(n):
        k = _first_crossing(t64[c])
        j = _onset(t64[c])
        u = _upstroke(t64[c])
        to_cross.append(float(np.abs(t32[c, :k] - t64[c, :k]).max()) if k else 0.0)
        to_onset.append(float(np.abs(t32[c, :j] - t64[c, :j]).max()) if j else 0.0)
        to_up.append(float(np.abs(t32[c, :u] - t64[c, :u]).max()) if u else 0.0)
        if k < t64.shape[1]:
            gap.append(k - j)
    to_up = np.asarray(to_up)
    e, mis = _spike_errors(s32, s64)
    to_cross = np.asarray(to_cross)
    out["fp32_vs_fp64_gpu"] = {
        "max_abs_dv_before_first_crossing_mV": float(to_cross.max()),
        "median_abs_dv_before_first_crossing_mV": float(np.median(to_cross)),
        "cells_within_1e-3_mV_to_first_crossing": int((to_cross <= 1e-3).sum()),
        "max_abs_dv_before_first_upstroke_mV": float(to_up.max()),
        "cells_within_1e-3_mV_to_first_upstroke": int((to_up <= 1e-3).sum()),
        "max_abs_dv_before_onset_mV": float(max(to_onset)),
        "onset_to_crossing_steps": {"median": float(np.median(gap)) if gap else None,
                                    "max": int(max(gap)) if gap else None},
        "spike_time_diff_ms": {"max": float(e.max()) if e.size else None,
                               "median": float(np.median(e)) if e.size else None,
                               "spikes_paired": int(e.size),
                               "within_0.05_ms": int((e <= 0.05).sum()) if e.size else 0},
        "cells_with_spike_count_mismatch": mis,
        "spiking_cells": int(sum(1 for x in s64 if len(x))),
    }
    # the target's own window: spike times over the first 100 ms
    early = [(np.asarray(x)[np.asarray(x) < 100.0], np.asarray(y)[np.asarray(y) < 100.0]) for x, y in zip(s32, s64)]
    e100, mis100 = _spike_errors([x for x, _ in early], [y for _, y in early])
    out["fp32_vs_fp64_gpu"]["first_100_ms"] = {
        "spike_time_diff_max_ms": float(e100.max()) if e100.size else None, "spikes_paired": int(e100.size),
        "within_0.05_ms": int((e100 <= 0.05).sum()) if e100.size else 0, "cells_with_spike_count_mismatch": mis100}
    if n_oracle:
        from oracle.staggered import OracleCell

        worst, sp_worst = 0.0, 0.0
        for c in range(min(n_oracle, n)):
            oc = OracleCell(W.desc_to_cell(sub[c]))
            otr, osp = oc.run(DT, a.sim_steps)
            worst = max(worst, float(np.abs(otr[0, 0] - t64[c]).max()))
            ref = np.asarray(osp[0][0])
            if len(ref) != len(s64[c]):
                sp_worst = float("inf")
            elif len(ref):
                sp_worst = max(sp_worst, float(np.abs(ref - s64[c]).max()))
        out["fp64_gpu_vs_cpu_oracle"] = {"cells": min(n_oracle, n), "max_abs_dv_whole_run_mV": worst,
                                         "spike_time_diff_max_ms": sp_worst}
    return out


def surrogate_leg(a, descs, local, sid, stream, plain_ms):
    """The surrogate-assisted form on the same workload: distal subtrees replaced by
    GRU ports (the packaged model trained by the library's kernels), per-cell
    fallback of envelope exits to the full solve, timed like the plain form;
    accuracy against the FP64 plain solve on the first cells of the workload."""
    import torch
    from dataclasses import replace

    from braincell_gb300 import surrogate as S
    from braincell_gb300 import workloads as W
    from braincell_gb300.runtime import Plan

    model = S.load_model(os.path.join(ROOT, "braincell_gb300", "data", "surrogate_uneven.npz"))
    T = a.surrogate_threads
    kw = dict(tile_nodes=a.surrogate_tile_nodes, threads_per_tile=T, threads_big=T, threads_global=T,
              steps_per_launch=a.steps_per_launch, lane_nodes=a.surrogate_lane_nodes,
              narrow_lane_nodes=a.narrow_lane_nodes, tile_order=1)
    t0 = time.perf_counter()
    runner = S.SurrogateRunner(descs, model, precision="f32", device=local, plan_kw=kw)
    t_setup = time.perf_counter() - t0
    for _ in range(a.warmup):
        runner.run(a.sim_steps, DT)
    torch.cuda.synchronize()
    walls, res, lines = [], None, []
    with ClockSampler(local) as clocks:
        for _ in range(max(a.steps, 5)):
            res = runner.run(a.sim_steps, DT)
            walls.append(res.wall_ms)
            fb = res.timeline.get("fallbacks", [])
            lines.append({"reduced_ms": round(res.timeline.get("reduced_ms", 0.0), 1),
                          "fallback_end_ms": round(max((f[3] for f in fb), default=0.0), 1),
                          "batches": [[f[0], f[1], round(f[2], 1), round(f[3], 1)] for f in fb]})
    ms = float(np.median(walls))
    info = runner.plan.info
    out = {"value": runner.full_cv * a.sim_steps / (ms * 1e-3),
           "unit": UNIT + " (full-morphology compartments)", "ms_per_step": ms, "speedup_vs_plain": plain_ms / ms,
           "n_ports": runner.n_ports, "reduced_compartments": int(runner.plan.n_cv),
           "full_compartments": runner.full_cv, "fallback_cells": int(res.fallback_cells.size),
           "fallback_rate": res.fallback_rate, "cut_depth": model.cut_depth, "threads_per_tile": T,
           "tiles": info["n_tiles"], "gpu_launches_per_step": res.launches,
           "clocks": clocks.summary(), "setup_s": round(t_setup, 2),
           "runs": len(walls), "ms_all_runs": [round(w, 1) for w in walls],
           "timeline": {"runs": lines,
                        "what": "device clock from the reset: end of the last reduced launch, end of the last "
                                "fallback solve, and per fallback batch [steps done when its flags were read, "
                                "cells, start ms, end ms]"},
           "timed": "median over the runs, host clock: reset + the reduced cells with GRU ports launch by launch, "
                    "flags read after each launch, the full solve of newly flagged cells from t = 0 on "
                    "high-priority side streams (plans built inside the timed region), until every stream is done"}
    runner.close()
    # accuracy on the first cells against the FP64 plain solve (the on-GPU oracle run)
    n_acc = min(a.accuracy_cells, len(descs))
    if n_acc:
        sub = list(descs[:n_acc])
        full = [replace(d, probes=[(0, 0.5)]) for d in sub]
        ref = Plan(W.descs_to_batch(full), precision="f64", device=local, record_every=1, max_spikes=256)
        ref.run(a.sim_steps, DT)
        tr64, sp64 = ref.traces(), ref.spikes()
        ref.close()
        r = S.run_surrogate(sub, model, a.sim_steps, record_every=1, fallback=True, device=local)
        rms = np.sqrt(np.mean((r.traces - tr64) ** 2, axis=1))
        lin = S.run_surrogate(sub, None, a.sim_steps, record_every=1, fallback=False, device=local)
        rms_lin = np.sqrt(np.mean((lin.traces - tr64) ** 2, axis=1))
        out["accuracy"] = {
            "cells": n_acc, "against": "FP64 plain solve on the GPU",
            "held_out": "seed 1 cells; the model was trained on seed 3 cells only",
            "fallback_rate": r.fallback_rate,
            "spike_time_error": _spike_report(r.spikes, sp64),
            "soma_rms_mV": {"median": float(np.median(rms)), "mean": float(np.mean(rms)),
                            "p99": float(np.percentile(rms, 99))},
            "without_network_soma_rms_mV": {"median": float(np.median(rms_lin)), "mean": float(np.mean(rms_lin))},
        }
    out["model"] = {k: model.info.get(k) for k in ("n_traj", "epochs", "updates", "train_s", "val_mse_after")}
    return out


def mixed_leg(a, local, model, record_every=4):
    """The mixed production run: ``a.mixed_cells`` cells of the uneven family drawn
    with seed 4, 30 % of them (a seeded draw) kept at full morphology and 70 % with
    their distal subtrees as GRU ports and per-cell fallback, ``a.mixed_steps``
    steps of 0.025 ms (500 ms), FP32 state with BF16 GRU weights.

    Reports compartment-steps/s of the plain form (every cell at full morphology,
    the same launch shape as the headline) and of the mixed form (full-morphology
    compartments counted for every cell), both host-clocked from reset to the end of
    every stream, the fallback rate, and accuracy against the FP64 plain solve on
    the first ``a.accuracy_cells`` cells (spike times from every spike; somatic RMS
    from the soma voltage sampled every ``record_every`` steps)."""
    import torch

    from braincell_gb300 import surrogate as S
    from braincell_gb300 import workloads as W
    from braincell_gb300.runtime import Plan

    n, steps = a.mixed_cells, a.mixed_steps
    descs = W.uneven(n, seed=4)
    full = np.sort(np.random.default_rng(4).choice(n, size=int(round(0.3 * n)), replace=False))
    total_cv = int(sum(int(sum(d.ncv)) for d in descs))
    out = {"cells": n, "steps": steps, "full_morphology_cells": int(full.size), "compartments": total_cv,
           "selection": "uneven generator seed 4; full-morphology cells drawn with default_rng(4)"}
    # plain form
    plan = Plan(W.descs_to_batch(descs), precision="f32", device=local, tile_nodes=a.tile_nodes,
                threads_per_tile=a.threads, threads_big=a.threads_big, steps_per_launch=a.steps_per_launch,
                record_every=0, lane_nodes=a.lane_nodes, narrow_lane_nodes=a.narrow_lane_nodes)
    st = torch.cuda.Stream(local)
    sid = int(st.cuda_stream)
    plan.reset(stream=sid)
    plan.run(2 * a.steps_per_launch, DT, stream=sid)
    walls = []
    for _ in range(2):
        torch.cuda.synchronize(local)
        t0 = time.perf_counter()
        plan.reset(stream=sid)
        plan.run(steps, DT, stream=sid, check=False)
        st.synchronize()
        walls.append((time.perf_counter() - t0) * 1e3)
        plan.check(stream=sid)
    plan.close()
    ms_plain = float(np.median(walls))
    out["plain"] = {"value": total_cv * steps / (ms_plain * 1e-3), "unit": UNIT, "ms": ms_plain,
                    "ms_all_runs": [round(w, 1) for w in walls]}
    # mixed surrogate form
    T = a.surrogate_threads
    kw = dict(tile_nodes=a.surrogate_tile_nodes, threads_per_tile=T, threads_big=T, threads_global=T,
              steps_per_launch=a.steps_per_launch, lane_nodes=a.surrogate_lane_nodes,
              narrow_lane_nodes=a.narrow_lane_nodes, tile_order=1)
    runner = S.SurrogateRunner(descs, model, precision="f32", device=local, plan_kw=kw, full_cells=full)
    runner.run(2 * a.steps_per_launch, DT)
    runs = [runner.run(steps, DT) for _ in range(3)]
    runner.close()
    ms = float(np.median([r.wall_ms for r in runs]))
    res = runs[-1]
    out["surrogate"] = {"value": total_cv * steps / (ms * 1e-3), "unit": UNIT + " (full-morphology compartments)",
                        "ms": ms, "ms_all_runs": [round(r.wall_ms, 1) for r in runs],
                        "speedup_vs_plain": ms_plain / ms, "fallback_cells": int(res.fallback_cells.size),
                        "fallback_rate": res.fallback_rate, "n_ports": runner.n_ports,
                        "reduced_compartments": int(runner.plan.n_cv)}
    # accuracy on the first cells (same full / port split) against the FP64 plain solve
    m = min(a.accuracy_cells, n)
    if m:
        from dataclasses import replace

        sub = [replace(d, probes=[(0, 0.5)]) for d in descs[:m]]
        ref = Plan(W.descs_to_batch(sub), precision="f64", device=local, record_every=record_every, max_spikes=512)
        ref.run(steps, DT)
        tr64, sp64 = ref.traces(), ref.spikes()
        ref.close()
        sub_full = full[full < m]
        r = S.run_surrogate(descs[:m], model, steps, record_every=record_every, fallback=True, device=local,
                            plan_kw=kw, full_cells=sub_full)
        port_cells = np.setdiff1d(np.arange(m), sub_full)
        rms = np.sqrt(np.mean((r.traces - tr64) ** 2, axis=1))
        out["accuracy"] = {
            "cells": m, "port_cells": int(port_cells.size), "against": "FP64 plain solve on the GPU",
            "fallback_rate": r.fallback_rate,
            "spike_time_error_all_cells": _spike_report(r.spikes, sp64),
            "spike_time_error_port_cells": _spike_report([r.spikes[i] for i in port_cells],
                                                         [sp64[i] for i in port_cells]),
            "soma_rms_mV": {"median": float(np.median(rms)), "mean": float(np.mean(rms)),
                            "p99": float(np.percentile(rms, 99)),
                            "port_cells_median": float(np.median(rms[port_cells]))},
            "soma_sampled_every_steps": record_every,
        }
    return out


def run_ours(a):
    import torch

    from braincell_gb300 import workloads as W
    from braincell_gb300.build import build_native
    from braincell_gb300.runtime import Plan
    from braincell_gb300.shard import reduce_max

    rank, world, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    build_native()
    # replicas only: every rank runs its own copy of the workload (its own seed)
    descs = _descs(a.workload, a.cells, seed=WORKLOADS[a.workload]["seed"] + rank)
    nbytes = WORKLOADS[a.workload]["bytes"]
    batch = W.descs_to_batch(descs)
    plan = Plan(batch, precision="f32", device=local, tile_nodes=a.tile_nodes, threads_per_tile=a.threads,
                threads_big=a.threads_big, steps_per_launch=a.steps_per_launch, record_every=0,
                lane_nodes=a.lane_nodes, narrow_lane_nodes=a.narrow_lane_nodes, lane_cell_nodes=a.lane_cell_nodes)
    info = plan.info
    n_cv = plan.n_cv
    stream = torch.cuda.current_stream(local)
    sid = int(stream.cuda_stream)

    def one_step():
        plan.reset(stream=sid)
        plan.run(a.sim_steps, DT, stream=sid, check=False)

    for _ in range(a.warmup):
        one_step()
    plan.check(stream=sid)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clocks:
        t_wall = time.perf_counter()
        ev0.record(stream)
        for _ in range(a.steps):
            one_step()
        ev1.record(stream)
        ev1.synchronize()
        t_wall = time.perf_counter() - t_wall
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    plan.check(stream=sid)
    ms = ev0.elapsed_time(ev1)
    ms = reduce_max(ms)
    comp_steps = n_cv * a.sim_steps * a.steps
    value = comp_steps * world / (ms * 1e-3)

    # kernel-only time of one simulation (the dominant kernel's launches), same stream
    plan.reset(stream=sid)
    kernel_ms = plan.run_timed(a.sim_steps, DT, stream=sid)
    launches_per_sim = -(-a.sim_steps // info["steps_per_launch"]) * info["n_launch_classes"]

    # end to end through the C ABI with host buffers: upload the initial voltages,
    # run the simulation, download the final voltages and spike counts
    v_host = plan.state("V", stream=sid)
    plan.reset(stream=sid)
    torch.cuda.synchronize()
    e2e_t = []
    for _ in range(max(1, a.steps)):
        t0 = time.perf_counter()
        plan.set_state("V", v_host, stream=sid)
        plan.run(a.sim_steps, DT, stream=sid)
        v_out = plan.state("V", stream=sid)
        counts = plan.spike_counts(stream=sid)
        e2e_t.append(time.perf_counter() - t0)
        plan.reset(stream=sid)
    e2e_s = reduce_max(float(np.median(e2e_t)))
    e2e_value = n_cv * a.sim_steps * world / e2e_s
    # bytes the API moves: upload = values + hi/lo offset tables (24 B/CV); download = its
    # offset tables up (16 B/CV) and values down (8 B/CV); spike counts down (4 B/probe)
    h2d_total = 24 * n_cv + 16 * n_cv
    d2h = 8 * n_cv + 4 * int(counts.size)

    peak, peak_kind = _peaks()
    achieved_gbs = nbytes * n_cv * a.sim_steps / (kernel_ms * 1e-3) / 1e9
    units_per_launch = n_cv * info["steps_per_launch"]
    prof = _traffic_per_node_launch(a.workload)
    traffic = None
    if prof and "dram_bytes_per_node_step" in prof:
        traffic = info["n_nodes"] * (prof.get("dram_bytes_per_node_launch_fixed", 0.0)
                                     + prof["dram_bytes_per_node_step"] * info["steps_per_launch"])
    clk = clocks.summary()
    sm_bound = None
    if prof and "warp_inst_per_node_step" in prof and clk.get("sm_mhz"):
        # the issue limit of this design: 4 warp schedulers per SM issue one warp
        # instruction per cycle each; ncu's instruction count per node-step (the
        # 1,000-cell capture) sets the node-steps/s that rate allows
        n_sm = torch.cuda.get_device_properties(local).multi_processor_count
        issue = 4.0 * n_sm * clk["sm_mhz"] * 1e6
        bound = issue / prof["warp_inst_per_node_step"] * n_cv / info["n_nodes"] * world
        sm_bound = {"bound": "sm_issue", "value": bound, "unit": UNIT, "frac": value / bound,
                    "warp_inst_per_node_step": prof["warp_inst_per_node_step"], "sms": n_sm,
                    "sm_mhz": clk["sm_mhz"]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded generator; no dataset)",
        "config": {"workload": WORKLOADS[a.workload]["text"],
                   "cells_per_gpu": a.cells, "compartments_per_gpu": n_cv, "sim_steps": a.sim_steps,
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                   "l2": "inputs larger than L2 (tile blobs + state arrays > 129 MB)",
                   "tiles": info["n_tiles"], "threads_per_tile": info["threads_per_tile"],
                   "tile_nodes": info["tile_nodes"], "steps_per_launch": info["steps_per_launch"],
                   "lane_nodes": a.lane_nodes, "narrow_lane_nodes": a.narrow_lane_nodes,
                   "lane_cell_nodes": a.lane_cell_nodes},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d_total), "d2h_bytes_per_step": int(d2h),
                "path": f"bc_state_upload (V) -> bc_run ({a.sim_steps:,} steps) -> bc_state_download (V) + "
                        "bc_spike_download"},
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peak, "unit": "GB/s",
                     "frac": achieved_gbs / peak, "peak_kind": peak_kind,
                     "traffic": traffic, "bytes_per_compartment_step": nbytes,
                     "algorithmic_bytes_per_launch": nbytes * units_per_launch,
                     "kernel_ms_per_sim": kernel_ms, "launches_per_sim": launches_per_sim},
        "sm_bound": sm_bound,
        "gpu_launches": a.steps * (1 + launches_per_sim),
        "clocks": clk,
        "wall_s_timed": t_wall,
    }
    if a.accuracy_cells:
        # the float64 CPU oracle takes ~16 ms per step of one large cell: the large
        # workload's CPU-oracle parity is in the tests (1,000 steps of a full-size cell)
        line["plain_accuracy"] = plain_accuracy(a, descs, local, n_oracle=2 if a.workload == "uneven" else 0)
    if not a.no_surrogate:
        sur = surrogate_leg(a, descs, local, sid, stream, ms / a.steps)
        sur["value"] = sur["value"] * world  # every rank runs its own replica
        line["surrogate"] = sur
        line["gpu_launches"] += a.steps * sur["gpu_launches_per_step"]
        if not a.no_mixed and rank == 0:
            from braincell_gb300 import surrogate as S

            line["mixed_production"] = mixed_leg(a, local, S.load_model(S.PACKAGED_MODEL))
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(a.workload)
    if rank == 0:
        print(json.dumps(line), flush=True)
    plan.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    a = _args()
    if a.warmup < 3:
        a.warmup = 3
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
