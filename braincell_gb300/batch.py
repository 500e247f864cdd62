"""Flat, morphology-level description of a batch of cells (the ``bc_batch_spec`` payload).

A :class:`CellBatch` is what crosses the C ABI: branches with their frustum
segments and CV counts, per-cell region tables (cable + mechanism records),
current-clamp segments and voltage probes.  Everything downstream of it --
geometry, CVs, node tree, axial coefficients, scheduling -- is done natively by
``bc_plan_create``.

:func:`lower_cell` converts one declared :class:`~braincell_gb300.cell.Cell`
(paint / place rules on a :class:`~braincell_gb300.morph.Morphology`) into a
batch with ``pop_size`` identical replicas, mirroring how the reference lowers
paint rules onto CVs (``_discretization/mechanism.py:514``) and place rules onto
points (``_compute/layouts.py:171``).
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from . import catalogue
from .catalogue import region_record
from .mech import CableProperty, CurrentClamp, CurrentProbe, ExpSyn, MechanismProbe, StateProbe

__all__ = ["CellBatch", "lower_cell", "concat_batches", "native_lowering"]


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


@dataclass
class CellBatch:
    n_regions: int
    cell_branch_offsets: np.ndarray
    branch_parent: np.ndarray
    branch_parent_x: np.ndarray
    branch_child_x: np.ndarray
    branch_ncv: np.ndarray
    branch_region: np.ndarray
    branch_seg_offsets: np.ndarray
    seg_length: np.ndarray
    seg_r_prox: np.ndarray
    seg_r_dist: np.ndarray
    region_cm: np.ndarray
    region_ra: np.ndarray
    region_mech: np.ndarray
    region_params: np.ndarray
    pulse_cell: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    pulse_branch: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    pulse_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    pulse_t_on: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    pulse_t_off: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    pulse_amp: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    probe_cell: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    probe_branch: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    probe_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    probe_field: np.ndarray | None = None  # BC_STATE_* view per probe (None: all V)
    syn_cell: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    syn_branch: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    syn_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    syn_tau: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    syn_e: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    conn_pre: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    conn_post: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int64))
    conn_weight: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    conn_delay: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    port_cell: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    port_branch: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    port_g: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    port_e: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    port_feat: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float64))
    port_pulse_port: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    port_pulse_t_on: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    port_pulse_t_off: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))
    port_pulse_amp: np.ndarray = field(default_factory=lambda: np.zeros(0, np.float64))

    _DTYPES = {
        "cell_branch_offsets": np.int64,
        "branch_parent": np.int32,
        "branch_parent_x": np.float64,
        "branch_child_x": np.float64,
        "branch_ncv": np.int32,
        "branch_region": np.int32,
        "branch_seg_offsets": np.int64,
        "seg_length": np.float64,
        "seg_r_prox": np.float64,
        "seg_r_dist": np.float64,
        "region_cm": np.float64,
        "region_ra": np.float64,
        "region_mech": np.uint32,
        "region_params": np.float64,
        "pulse_cell": np.int32,
        "pulse_branch": np.int32,
        "pulse_x": np.float64,
        "pulse_t_on": np.float64,
        "pulse_t_off": np.float64,
        "pulse_amp": np.float64,
        "probe_cell": np.int32,
        "probe_branch": np.int32,
        "probe_x": np.float64,
        "syn_cell": np.int32,
        "syn_branch": np.int32,
        "syn_x": np.float64,
        "syn_tau": np.float64,
        "syn_e": np.float64,
        "conn_pre": np.int32,
        "conn_post": np.int64,
        "conn_weight": np.float64,
        "conn_delay": np.float64,
        "port_cell": np.int32,
        "port_branch": np.int32,
        "port_g": np.float64,
        "port_e": np.float64,
        "port_feat": np.float64,
        "port_pulse_port": np.int32,
        "port_pulse_t_on": np.float64,
        "port_pulse_t_off": np.float64,
        "port_pulse_amp": np.float64,
        "probe_field": np.int32,
    }

    def __post_init__(self) -> None:
        if self.probe_field is None or np.size(self.probe_field) == 0:
            self.probe_field = np.zeros(np.size(self.probe_cell), np.int32)
        for name, dt in self._DTYPES.items():
            setattr(self, name, np.ascontiguousarray(getattr(self, name), dtype=dt))
        self.region_params = self.region_params.reshape(-1, _abi.BC_NPARAM)
        self.port_feat = self.port_feat.reshape(-1, 2)
        self.n_regions = int(self.n_regions)

    # ------------------------------------------------------------------ sizes
    @property
    def n_cells(self) -> int:
        return int(self.cell_branch_offsets.size - 1)

    @property
    def n_branches(self) -> int:
        return int(self.branch_parent.size)

    @property
    def n_cv(self) -> int:
        return int(self.branch_ncv.sum())

    def cell_ncv(self) -> np.ndarray:
        cs = np.concatenate([[0], np.cumsum(self.branch_ncv, dtype=np.int64)])
        return cs[self.cell_branch_offsets[1:]] - cs[self.cell_branch_offsets[:-1]]

    def cell_nbranch(self) -> np.ndarray:
        return np.diff(self.cell_branch_offsets)

    def select(self, cells) -> "CellBatch":
        """The batch of the given cells (in the given order), with their clamps and probes."""
        cells = np.asarray(cells, dtype=np.int64)
        if cells.ndim != 1 or np.any(cells < 0) or np.any(cells >= self.n_cells):
            raise ValueError("cells must be a 1-D array of cell indices of this batch.")
        R = self.n_regions
        b0, b1 = self.cell_branch_offsets[cells], self.cell_branch_offsets[cells + 1]
        br = np.concatenate([np.arange(a, b) for a, b in zip(b0, b1)]) if cells.size else np.zeros(0, np.int64)
        s0, s1 = self.branch_seg_offsets[br], self.branch_seg_offsets[br + 1]
        seg = np.concatenate([np.arange(a, b) for a, b in zip(s0, s1)]) if br.size else np.zeros(0, np.int64)
        rg = (cells[:, None] * R + np.arange(R)[None, :]).reshape(-1)
        new_id = np.full(self.n_cells, -1, np.int64)
        new_id[cells] = np.arange(cells.size)
        pk = new_id[self.pulse_cell] >= 0 if self.pulse_cell.size else np.zeros(0, bool)
        qk = new_id[self.probe_cell] >= 0 if self.probe_cell.size else np.zeros(0, bool)
        pord = np.argsort(new_id[self.pulse_cell[pk]], kind="stable")
        qord = np.argsort(new_id[self.probe_cell[qk]], kind="stable")
        sk = new_id[self.syn_cell] >= 0 if self.syn_cell.size else np.zeros(0, bool)
        sord = np.argsort(new_id[self.syn_cell[sk]], kind="stable")
        syn_old = np.nonzero(sk)[0][sord]
        new_syn = np.full(self.syn_cell.size, -1, np.int64)
        new_syn[syn_old] = np.arange(syn_old.size)
        ck = (new_id[self.conn_pre] >= 0) & (new_syn[self.conn_post] >= 0) if self.conn_pre.size else np.zeros(0, bool)
        ok = new_id[self.port_cell] >= 0 if self.port_cell.size else np.zeros(0, bool)
        port_old = np.nonzero(ok)[0][np.argsort(new_id[self.port_cell[ok]], kind="stable")]
        new_port = np.full(self.port_cell.size, -1, np.int64)
        new_port[port_old] = np.arange(port_old.size)
        ppk = new_port[self.port_pulse_port] >= 0 if self.port_pulse_port.size else np.zeros(0, bool)
        pp_old = np.nonzero(ppk)[0][np.argsort(new_port[self.port_pulse_port[ppk]], kind="stable")]
        return CellBatch(
            n_regions=R,
            cell_branch_offsets=np.concatenate([[0], np.cumsum(b1 - b0)]),
            branch_parent=self.branch_parent[br], branch_parent_x=self.branch_parent_x[br],
            branch_child_x=self.branch_child_x[br], branch_ncv=self.branch_ncv[br],
            branch_region=self.branch_region[br],
            branch_seg_offsets=np.concatenate([[0], np.cumsum(s1 - s0)]),
            seg_length=self.seg_length[seg], seg_r_prox=self.seg_r_prox[seg], seg_r_dist=self.seg_r_dist[seg],
            region_cm=self.region_cm[rg], region_ra=self.region_ra[rg], region_mech=self.region_mech[rg],
            region_params=self.region_params[rg],
            pulse_cell=new_id[self.pulse_cell[pk]][pord], pulse_branch=self.pulse_branch[pk][pord],
            pulse_x=self.pulse_x[pk][pord], pulse_t_on=self.pulse_t_on[pk][pord],
            pulse_t_off=self.pulse_t_off[pk][pord], pulse_amp=self.pulse_amp[pk][pord],
            probe_cell=new_id[self.probe_cell[qk]][qord], probe_branch=self.probe_branch[qk][qord],
            probe_x=self.probe_x[qk][qord], probe_field=self.probe_field[qk][qord],
            syn_cell=new_id[self.syn_cell[syn_old]], syn_branch=self.syn_branch[syn_old], syn_x=self.syn_x[syn_old],
            syn_tau=self.syn_tau[syn_old], syn_e=self.syn_e[syn_old],
            conn_pre=new_id[self.conn_pre[ck]], conn_post=new_syn[self.conn_post[ck]],
            conn_weight=self.conn_weight[ck], conn_delay=self.conn_delay[ck],
            port_cell=new_id[self.port_cell[port_old]], port_branch=self.port_branch[port_old],
            port_g=self.port_g[port_old], port_e=self.port_e[port_old], port_feat=self.port_feat[port_old],
            port_pulse_port=new_port[self.port_pulse_port[pp_old]], port_pulse_t_on=self.port_pulse_t_on[pp_old],
            port_pulse_t_off=self.port_pulse_t_off[pp_old], port_pulse_amp=self.port_pulse_amp[pp_old],
        )

    def validate(self) -> None:
        nb = self.n_branches
        if self.cell_branch_offsets[0] != 0 or self.cell_branch_offsets[-1] != nb:
            raise ValueError("cell_branch_offsets must start at 0 and end at n_branches.")
        if np.any(np.diff(self.cell_branch_offsets) <= 0):
            raise ValueError("every cell needs at least one branch.")
        if np.any(self.branch_ncv < 1):
            raise ValueError("branch_ncv must be >= 1.")
        if self.region_params.shape != (self.n_cells * self.n_regions, _abi.BC_NPARAM):
            raise ValueError("region_params has the wrong shape.")
        ns = self.syn_cell.size
        if any(getattr(self, k).size != ns for k in ("syn_branch", "syn_x", "syn_tau", "syn_e")):
            raise ValueError("synapse arrays must all have n_synapses entries.")
        nc = self.conn_pre.size
        if any(getattr(self, k).size != nc for k in ("conn_post", "conn_weight", "conn_delay")):
            raise ValueError("connection arrays must all have n_connections entries.")
        if self.probe_field.size != self.probe_cell.size:
            raise ValueError("probe_field must have one entry per probe.")
        npt = self.port_cell.size
        if any(getattr(self, k).shape[0] != npt for k in ("port_branch", "port_g", "port_e", "port_feat")):
            raise ValueError("port arrays must all have n_ports entries.")
        npp = self.port_pulse_port.size
        if any(getattr(self, k).size != npp for k in ("port_pulse_t_on", "port_pulse_t_off", "port_pulse_amp")):
            raise ValueError("port pulse arrays must all have n_port_pulses entries.")

    # ------------------------------------------------------------------ ABI
    def to_spec(self) -> tuple[_abi.BatchSpec, tuple]:
        """Return the ctypes spec plus the arrays it points into (keep them alive)."""
        self.validate()
        s = _abi.BatchSpec()
        s.n_cells = self.n_cells
        s.n_branches = self.n_branches
        s.n_segments = int(self.seg_length.size)
        s.n_regions = self.n_regions
        keep = []
        ctypes_of = {np.int64: C.c_int64, np.int32: C.c_int32, np.float64: C.c_double, np.uint32: C.c_uint32}
        for name, dt in self._DTYPES.items():
            arr = getattr(self, name)
            keep.append(arr)
            setattr(s, name, _ptr(arr, ctypes_of[dt]))
        s.n_pulses = int(self.pulse_cell.size)
        s.n_probes = int(self.probe_cell.size)
        s.n_synapses = int(self.syn_cell.size)
        s.n_connections = int(self.conn_pre.size)
        s.n_ports = int(self.port_cell.size)
        s.n_port_pulses = int(self.port_pulse_port.size)
        return s, tuple(keep)


def native_lowering(batch: CellBatch, cell: int) -> dict:
    """The native library's lowering of one cell (point tree + axial coefficients)."""
    lib = _abi.lib()
    spec, keep = batch.to_spec()
    ncv, nn = C.c_int32(), C.c_int32()
    _abi.check(lib.bc_lower_cell(C.byref(spec), int(cell), C.byref(ncv), C.byref(nn), None, None, None, None, None,
                                 None, None))
    out = {
        "cv_area": np.zeros(ncv.value), "cv_node": np.zeros(ncv.value, np.int32), "parent": np.zeros(nn.value, np.int32),
        "alpha": np.zeros(nn.value), "beta": np.zeros(nn.value), "diag": np.zeros(nn.value),
        "region": np.zeros(nn.value, np.int32),
    }
    d, i32 = C.POINTER(C.c_double), C.POINTER(C.c_int32)
    _abi.check(lib.bc_lower_cell(
        C.byref(spec), int(cell), C.byref(ncv), C.byref(nn), out["cv_area"].ctypes.data_as(d),
        out["cv_node"].ctypes.data_as(i32), out["parent"].ctypes.data_as(i32), out["alpha"].ctypes.data_as(d),
        out["beta"].ctypes.data_as(d), out["diag"].ctypes.data_as(d), out["region"].ctypes.data_as(i32)))
    del keep
    return out


def concat_batches(batches: list[CellBatch]) -> CellBatch:
    """Concatenate batches cell-wise (region tables padded to the widest)."""
    if not batches:
        raise ValueError("concat_batches needs at least one batch.")
    R = max(b.n_regions for b in batches)
    parts: dict[str, list] = {k: [] for k in CellBatch._DTYPES}
    br_off = 0
    seg_off = 0
    cell_off = 0
    syn_off = 0
    port_off = 0
    for b in batches:
        parts["cell_branch_offsets"].append(b.cell_branch_offsets[(1 if br_off or cell_off else 0):] + br_off)
        parts["branch_seg_offsets"].append(b.branch_seg_offsets[(1 if seg_off or cell_off else 0):] + seg_off)
        for k in ("branch_parent", "branch_parent_x", "branch_child_x", "branch_ncv", "branch_region",
                  "seg_length", "seg_r_prox", "seg_r_dist"):
            parts[k].append(getattr(b, k))
        nc = b.n_cells
        pad = R - b.n_regions
        for k in ("region_cm", "region_ra", "region_mech"):
            a = getattr(b, k).reshape(nc, b.n_regions)
            if pad:
                a = np.concatenate([a, np.repeat(a[:, :1], pad, axis=1)], axis=1)
            parts[k].append(a.reshape(-1))
        a = b.region_params.reshape(nc, b.n_regions, _abi.BC_NPARAM)
        if pad:
            a = np.concatenate([a, np.repeat(a[:, :1], pad, axis=1)], axis=1)
        parts["region_params"].append(a.reshape(-1, _abi.BC_NPARAM))
        parts["pulse_cell"].append(b.pulse_cell + cell_off)
        parts["probe_cell"].append(b.probe_cell + cell_off)
        parts["syn_cell"].append(b.syn_cell + cell_off)
        parts["conn_pre"].append(b.conn_pre + cell_off)
        parts["conn_post"].append(b.conn_post + syn_off)
        parts["port_cell"].append(b.port_cell + cell_off)
        parts["port_pulse_port"].append(b.port_pulse_port + port_off)
        for k in ("pulse_branch", "pulse_x", "pulse_t_on", "pulse_t_off", "pulse_amp", "probe_branch", "probe_x",
                  "syn_branch", "syn_x", "syn_tau", "syn_e", "conn_weight", "conn_delay", "probe_field", "port_branch", "port_g",
                  "port_e", "port_feat", "port_pulse_t_on", "port_pulse_t_off", "port_pulse_amp"):
            parts[k].append(getattr(b, k))
        syn_off += int(b.syn_cell.size)
        port_off += int(b.port_cell.size)
        br_off += b.n_branches
        seg_off += int(b.seg_length.size)
        cell_off += nc
    kw = {k: np.concatenate(v) for k, v in parts.items()}
    return CellBatch(n_regions=R, **kw)


# (mechanism class, field) -> BC_STATE_* view recorded by a MechanismProbe
PROBE_STATES = {
    ("Na_Ba2002", "p"): _abi.BC_STATE_NA_P, ("Na_Ba2002", "q"): _abi.BC_STATE_NA_Q,
    ("KDR_Ba2002", "p"): _abi.BC_STATE_KDR_P,
    ("CaL_IS2008", "p"): _abi.BC_STATE_CAL_P, ("CaL_IS2008", "q"): _abi.BC_STATE_CAL_Q,
    ("CaT_HM1992", "p"): _abi.BC_STATE_CAT_P, ("CaT_HM1992", "q"): _abi.BC_STATE_CAT_Q,
    ("HCN_HM1992", "p"): _abi.BC_STATE_HCN_P,
    ("AHP_De1994", "p"): _abi.BC_STATE_AHP_P,
    ("CalciumDetailed", "Ci"): _abi.BC_STATE_CA_CI,
    ("Na_HH1952", "p"): _abi.BC_STATE_NAHH_P, ("Na_HH1952", "q"): _abi.BC_STATE_NAHH_Q,
    ("K_HH1952", "p"): _abi.BC_STATE_KHH_P,
    ("KM_RI2021_SC", "n"): _abi.BC_STATE_KM_N,
    ("KA1_HM1992", "p"): _abi.BC_STATE_KA1_P, ("KA1_HM1992", "q"): _abi.BC_STATE_KA1_Q,
    ("KA2_HM1992", "p"): _abi.BC_STATE_KA2_P, ("KA2_HM1992", "q"): _abi.BC_STATE_KA2_Q,
    ("KK2A_HM1992", "p"): _abi.BC_STATE_KK2A_P, ("KK2A_HM1992", "q"): _abi.BC_STATE_KK2A_Q,
    ("KK2B_HM1992", "p"): _abi.BC_STATE_KK2B_P, ("KK2B_HM1992", "q"): _abi.BC_STATE_KK2B_Q,
    ("KNI_Ya1989", "p"): _abi.BC_STATE_KNI_P,
}
PROBE_STATES.update({
    ("Kv3p4_MA2020_GoC", "m"): _abi.BC_STATE_KV34_M, ("Kv3p4_MA2020_GoC", "h"): _abi.BC_STATE_KV34_H,
    ("Kv4p3_MA2020_GoC", "a"): _abi.BC_STATE_KV43_A, ("Kv4p3_MA2020_GoC", "b"): _abi.BC_STATE_KV43_B,
    ("Kv1p1_MA2020_GoC", "n"): _abi.BC_STATE_KV11_N, ("Kir2p3_MA2020_GrC", "d"): _abi.BC_STATE_KIR23_D,
    ("HCN1_MA2020_GoC", "o_fast"): _abi.BC_STATE_HCN1F_FAST, ("HCN1_MA2020_GoC", "o_slow"): _abi.BC_STATE_HCN1F_SLOW,
    ("HCN1_MA2024_PC", "h"): _abi.BC_STATE_HCN1H_H,
    ("CaHVA_MA2020_GoC", "s"): _abi.BC_STATE_CAHVA_S, ("CaHVA_MA2020_GoC", "u"): _abi.BC_STATE_CAHVA_U,
    ("Cav2p3_MA2020_GoC", "m"): _abi.BC_STATE_CAV23_M, ("Cav2p3_MA2020_GoC", "h"): _abi.BC_STATE_CAV23_H,
    ("Cav3p2_RI2021_SC", "m"): _abi.BC_STATE_CAV32_M, ("Cav3p2_RI2021_SC", "h"): _abi.BC_STATE_CAV32_H,
    # extension channels
    ("HCN2_MA2020_GoC", "o_fast"): _abi.BC_STATE_HCN2_FAST, ("HCN2_MA2020_GoC", "o_slow"): _abi.BC_STATE_HCN2_SLOW,
    ("Kv3p3_MA2024_PC", "n"): _abi.BC_STATE_KV33_N,
    ("Kv2p2_0010_MA2020_GrC", "m"): _abi.BC_STATE_KV22_M, ("Kv2p2_0010_MA2020_GrC", "h"): _abi.BC_STATE_KV22_H,
    ("Kv1p5_MA2024_PC", "m"): _abi.BC_STATE_KV15_M, ("Kv1p5_MA2024_PC", "n"): _abi.BC_STATE_KV15_N,
    ("Kv1p5_MA2024_PC", "u"): _abi.BC_STATE_KV15_U,
    ("NaF_SU2015_DCN", "m"): _abi.BC_STATE_NAF_M, ("NaF_SU2015_DCN", "h"): _abi.BC_STATE_NAF_H,
    ("NaP_SU2015_DCN", "m"): _abi.BC_STATE_NAP_M, ("NaP_SU2015_DCN", "h"): _abi.BC_STATE_NAP_H,
    ("Na_ZH2019_IO", "m"): _abi.BC_STATE_NAIO_M, ("Na_ZH2019_IO", "h"): _abi.BC_STATE_NAIO_H,
    ("fKdr_SU2015_DCN", "m"): _abi.BC_STATE_FKDR_M, ("sKdr_SU2015_DCN", "m"): _abi.BC_STATE_SKDR_M,
    ("Kdr_ZH2019_IO", "n"): _abi.BC_STATE_KDRIO_N, ("HCN_SU2015_DCN", "m"): _abi.BC_STATE_HCNDCN_M,
    ("HCN_ZH2019_IO", "q"): _abi.BC_STATE_HCNIO_Q,
    ("CaT_HP1992", "p"): _abi.BC_STATE_CATHP_P, ("CaT_HP1992", "q"): _abi.BC_STATE_CATHP_Q,
    ("CaHT_Re1993", "p"): _abi.BC_STATE_CAHTRE_P, ("CaHT_Re1993", "q"): _abi.BC_STATE_CAHTRE_Q,
    ("CaL_SU2015_DCN", "m"): _abi.BC_STATE_CALDCN_M, ("CaL_SU2015_DCN", "h"): _abi.BC_STATE_CALDCN_H,
    ("Kca3p1_MA2020_GoC", "p"): _abi.BC_STATE_KCA31_P, ("SK_SU2015_DCN", "z"): _abi.BC_STATE_SKDCN_Z,
    ("K_Kv_test", "n"): _abi.BC_STATE_KKV_N, ("CaN_IS2008", "p"): _abi.BC_STATE_CAN_P,
    ("Ca_ZH2019_IO", "h"): _abi.BC_STATE_CAIO_H,
    ("Cav3p1_MA2020_GoC", "p"): _abi.BC_STATE_CAV31_P, ("Cav3p1_MA2020_GoC", "q"): _abi.BC_STATE_CAV31_Q,
    ("Cav3p3_RI2021_SC", "n"): _abi.BC_STATE_CAV33_N, ("Cav3p3_RI2021_SC", "l"): _abi.BC_STATE_CAV33_L,
    **{(c, g): base + k for c, base in (("Cav1p2_MA2020_GoC", _abi.BC_STATE_CAV12_M),
                                        ("Cav1p3_MA2020_GoC", _abi.BC_STATE_CAV13_M))
       for k, g in enumerate(("m", "h", "n"))},
    ("Cav2p1_RI2021_SC", "m"): _abi.BC_STATE_CAV21_M, ("CaHVA_SU2015_DCN", "m"): _abi.BC_STATE_CAHVADCN_M,
    ("CaLVA_SU2015_DCN", "m"): _abi.BC_STATE_CALVADCN_M, ("CaLVA_SU2015_DCN", "h"): _abi.BC_STATE_CALVADCN_H,
})
for _cls, (_base, _names) in _abi.MARKOV_STATES.items():
    for _k, _n in enumerate(_names):
        PROBE_STATES[(_cls, _n)] = _base + _k
        if _cls == "Nav1p6_MA2020_GoC":  # Nav1p1 runs the same scheme in the same states
            for _nav11 in ("Nav1p1_MA2025_BC", "Nav1p1_RI2021_SC"):
                PROBE_STATES[(_nav11, _n)] = _base + _k


# CurrentProbe: mechanism class -> BC_CUR_* code; ion name -> the ion's total
PROBE_CURRENTS = {
    "IL": _abi.BC_CUR_IL, "K_Leak": _abi.BC_CUR_KLEAK, "Na_Ba2002": _abi.BC_CUR_NA, "KDR_Ba2002": _abi.BC_CUR_KDR,
    "CaL_IS2008": _abi.BC_CUR_CAL, "CaT_HM1992": _abi.BC_CUR_CAT, "HCN_HM1992": _abi.BC_CUR_HCN,
    "AHP_De1994": _abi.BC_CUR_AHP, "Na_HH1952": _abi.BC_CUR_NAHH, "K_HH1952": _abi.BC_CUR_KHH,
    "KM_RI2021_SC": _abi.BC_CUR_KM, "KA1_HM1992": _abi.BC_CUR_KA1, "KA2_HM1992": _abi.BC_CUR_KA2,
    "KK2A_HM1992": _abi.BC_CUR_KK2A, "KK2B_HM1992": _abi.BC_CUR_KK2B, "KNI_Ya1989": _abi.BC_CUR_KNI,
    "Nav1p6_MA2020_GoC": _abi.BC_CUR_NAV16, "Kca2p2_MA2020_GoC": _abi.BC_CUR_KCA22,
    "Kca1p1_MA2020_GoC": _abi.BC_CUR_KCA11,
    "Nav1p1_MA2025_BC": _abi.BC_CUR_NAV16, "Nav1p1_RI2021_SC": _abi.BC_CUR_NAV16,
    "Kv3p4_MA2020_GoC": _abi.BC_CUR_KV34, "Kv4p3_MA2020_GoC": _abi.BC_CUR_KV43, "Kv1p1_MA2020_GoC": _abi.BC_CUR_KV11,
    "Kir2p3_MA2020_GrC": _abi.BC_CUR_KIR23, "HCN1_MA2020_GoC": _abi.BC_CUR_HCN1F, "HCN1_MA2024_PC": _abi.BC_CUR_HCN1H,
    "CaHVA_MA2020_GoC": _abi.BC_CUR_CAHVA, "Cav2p3_MA2020_GoC": _abi.BC_CUR_CAV23, "Cav3p2_RI2021_SC": _abi.BC_CUR_CAV32,
    "HCN2_MA2020_GoC": _abi.BC_CUR_HCN2, "Kv3p3_MA2024_PC": _abi.BC_CUR_KV33,
    "Kv2p2_0010_MA2020_GrC": _abi.BC_CUR_KV22, "Kv1p5_MA2024_PC": _abi.BC_CUR_KV15, "NaF_SU2015_DCN": _abi.BC_CUR_NAF,
    "NaP_SU2015_DCN": _abi.BC_CUR_NAP, "Na_ZH2019_IO": _abi.BC_CUR_NAIO, "fKdr_SU2015_DCN": _abi.BC_CUR_FKDR,
    "sKdr_SU2015_DCN": _abi.BC_CUR_SKDR, "Kdr_ZH2019_IO": _abi.BC_CUR_KDRIO, "HCN_SU2015_DCN": _abi.BC_CUR_HCNDCN,
    "HCN_ZH2019_IO": _abi.BC_CUR_HCNIO, "CaT_HP1992": _abi.BC_CUR_CATHP, "CaHT_Re1993": _abi.BC_CUR_CAHTRE,
    "CaL_SU2015_DCN": _abi.BC_CUR_CALDCN, "Kca3p1_MA2020_GoC": _abi.BC_CUR_KCA31, "SK_SU2015_DCN": _abi.BC_CUR_SKDCN,
    "K_Kv_test": _abi.BC_CUR_KKV, "CaN_IS2008": _abi.BC_CUR_CAN, "Ca_ZH2019_IO": _abi.BC_CUR_CAIO,
    "Nav_MA2020_GrC": _abi.BC_CUR_NAVGRC, "Cav3p1_MA2020_GoC": _abi.BC_CUR_CAV31,
    "Cav3p3_RI2021_SC": _abi.BC_CUR_CAV33, "Cav1p2_MA2020_GoC": _abi.BC_CUR_CAV12, "Cav1p3_MA2020_GoC": _abi.BC_CUR_CAV13,
    "Cav2p1_RI2021_SC": _abi.BC_CUR_CAV21, "CaHVA_SU2015_DCN": _abi.BC_CUR_CAHVADCN,
    "CaLVA_SU2015_DCN": _abi.BC_CUR_CALVADCN,
}
ION_CURRENTS = {"na": _abi.BC_CUR_ION_NA, "k": _abi.BC_CUR_ION_K, "ca": _abi.BC_CUR_ION_CA}


# same-form classes record through the views of the class whose kernel they use
for _cls, _kern in catalogue.SAME_FORM.items():
    for (_c, _f), _view in list(PROBE_STATES.items()):
        if _c == _kern:
            PROBE_STATES[(_cls, _f)] = _view
    PROBE_CURRENTS[_cls] = PROBE_CURRENTS[_kern]


def probe_field_of(decl, mechs) -> int:
    """The BC_STATE_* view a MechanismProbe records, resolved against the mechanisms
    painted where it sits: ``decl.mechanism`` is a painted mechanism's instance name or
    class name (``_multi_compartment/probes.py:136-181`` looks it up the same way)."""
    if isinstance(decl, CurrentProbe):
        if decl.mechanism is None:
            if decl.ion not in ION_CURRENTS:
                raise KeyError(f"Probe {decl.name!r}: unknown ion {decl.ion!r} (one of {sorted(ION_CURRENTS)}).")
            return int(_abi.BC_PROBE_CURRENT + ION_CURRENTS[decl.ion])
        hits = [m for m in mechs if getattr(m, "instance_name", None) == decl.mechanism]
        if len(hits) != 1:
            raise KeyError(f"Probe {decl.name!r} could not find one mechanism named {decl.mechanism!r} here.")
        cls = "IL" if hits[0].class_name == "leaky" else hits[0].class_name
        if cls not in PROBE_CURRENTS:
            raise KeyError(f"Probe {decl.name!r}: no current for mechanism class {cls!r}.")
        return int(_abi.BC_PROBE_CURRENT + PROBE_CURRENTS[cls])
    hits = [m for m in mechs if getattr(m, "instance_name", None) == decl.mechanism]
    if len(hits) > 1:
        raise ValueError(f"Probe {decl.name!r} matched multiple mechanisms named {decl.mechanism!r}.")
    if not hits:
        raise KeyError(f"Probe {decl.name!r} could not find a mechanism or ion named {decl.mechanism!r} here.")
    key = (hits[0].class_name, decl.field)
    if key not in PROBE_STATES:
        raise KeyError(f"Probe {decl.name!r} field {decl.field!r} was not found on {hits[0].class_name}.")
    return int(PROBE_STATES[key])


def _branch_regions(cell) -> tuple[np.ndarray, list[tuple[CableProperty, list]]]:
    """Resolve paint rules to one (cable, mechanisms) region per branch."""
    morpho = cell.morpho
    nb = len(morpho.branches)
    cables: list[CableProperty] = [CableProperty() for _ in range(nb)]
    mechs: list[list] = [[] for _ in range(nb)]
    for region, decls in cell.paint_rules:
        mask = region.branch_mask(morpho)
        for d in decls:
            for b in np.nonzero(mask)[0]:
                if isinstance(d, CableProperty):
                    cables[b] = d
                else:
                    mechs[b].append(d)
    keys: dict = {}
    regions: list[tuple[CableProperty, list]] = []
    branch_region = np.zeros(nb, dtype=np.int32)
    for b in range(nb):
        key = (cables[b], tuple((type(m).__name__, m.class_name, tuple(sorted(m.params.items()))) for m in mechs[b]))
        if key not in keys:
            keys[key] = len(regions)
            regions.append((cables[b], mechs[b]))
        branch_region[b] = keys[key]
    return branch_region, regions


def lower_cell(cell, replicas: int | None = None) -> CellBatch:
    """Lower a declared Cell into a batch of ``replicas`` (default ``pop_size``) copies."""
    morpho = cell.morpho
    P = int(np.prod(cell.pop_size)) if replicas is None else int(replicas)
    nb = len(morpho.branches)
    parent = morpho.parent_index
    parent_x = np.zeros(nb)
    child_x = np.zeros(nb)
    for e in morpho.edges:
        parent_x[e.child.index] = e.parent_x
        child_x[e.child.index] = e.child_x
    ncv = np.asarray(cell.cv_policy.cv_counts(morpho), dtype=np.int32)
    seg_len, seg_rp, seg_rd, seg_off = [], [], [], [0]
    for br in morpho.branches:
        seg_len.append(br.lengths)
        seg_rp.append(br.radii_proximal)
        seg_rd.append(br.radii_distal)
        seg_off.append(seg_off[-1] + br.n_segments)
    branch_region, regions = _branch_regions(cell)
    R = len(regions)
    cm = np.zeros(R)
    ra = np.zeros(R)
    bits = np.zeros(R, dtype=np.uint32)
    params = np.zeros((R, _abi.BC_NPARAM))
    for r, (cable, mechs) in enumerate(regions):
        bits[r], params[r] = region_record(mechs, cable)
        cm[r] = cable.membrane_capacitance
        ra[r] = cable.axial_resistivity
        if cell.V_init is not None:
            params[r, _abi.BC_P_VREST] = float(cell.V_init)
    pulses: list[tuple[int, float, float, float, float]] = []
    probes: list[tuple[int, float, int]] = []
    syns: list[tuple[int, float, float, float]] = []
    for locset, decls in cell.place_rules:
        for (b, x) in locset.points(morpho):
            for d in decls:
                if isinstance(d, CurrentClamp):
                    for (t_on, t_off, amp) in d.segments():
                        pulses.append((b, x, t_on, t_off, amp))
                elif isinstance(d, StateProbe):
                    probes.append((b, x, 0))
                elif isinstance(d, (MechanismProbe, CurrentProbe)):
                    probes.append((b, x, probe_field_of(d, regions[int(branch_region[b])][1])))
                elif isinstance(d, ExpSyn):
                    syns.append((b, x, d.tau, d.e))
                else:
                    raise TypeError(f"Unsupported point mechanism {type(d).__name__}.")
    one = CellBatch(
        n_regions=R,
        cell_branch_offsets=np.asarray([0, nb]),
        branch_parent=parent,
        branch_parent_x=parent_x,
        branch_child_x=child_x,
        branch_ncv=ncv,
        branch_region=branch_region,
        branch_seg_offsets=np.asarray(seg_off),
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
        probe_field=np.asarray([p[2] for p in probes], np.int32),
        syn_cell=np.zeros(len(syns), np.int32),
        syn_branch=np.asarray([q[0] for q in syns], np.int32),
        syn_x=np.asarray([q[1] for q in syns]),
        syn_tau=np.asarray([q[2] for q in syns]),
        syn_e=np.asarray([q[3] for q in syns]),
    )
    if P == 1:
        return one
    return concat_batches([one] * P)
