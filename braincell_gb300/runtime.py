"""Host-side handle on a native plan: a batch of cells resident on one GB300.

:class:`Plan` owns the ``bc_plan_t`` created from a :class:`~braincell_gb300.batch.CellBatch`
and exposes reset / run / state views / probes.  Device memory belongs to the
plan; CUDA work is ordered on the caller's stream (the current torch stream by
default, when torch is importable).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .batch import CellBatch

__all__ = ["Plan", "current_stream"]

_PREC = {"f32": _abi.BC_PREC_F32, "float32": _abi.BC_PREC_F32, "f64": _abi.BC_PREC_F64, "float64": _abi.BC_PREC_F64}


def current_stream(device: int = 0) -> int:
    """Raw ``cudaStream_t`` of torch's current stream on ``device`` (0 = legacy default)."""
    try:
        import torch

        if torch.cuda.is_available():
            return int(torch.cuda.current_stream(device).cuda_stream)
    except Exception:  # pragma: no cover - torch missing or not initialised
        pass
    return 0


class Plan:
    def __init__(
        self,
        batch: CellBatch,
        *,
        precision: str = "f32",
        threads_per_tile: int = 0,
        tile_nodes: int = 0,
        lane_nodes: int = 0,
        narrow_lane_nodes: int = 0,
        steps_per_launch: int = 0,
        record_every: int = 1,
        max_spikes: int = 64,
        use_graph: bool = False,
        device: int = 0,
        threads_big: int = 0,
        threads_global: int = 0,
        dry_run: bool = False,
        lane_cell_nodes: int = 0,
        tile_order: int = 0,
    ) -> None:
        if precision not in _PREC:
            raise ValueError(f"precision must be one of {sorted(_PREC)}, got {precision!r}.")
        lib = _abi.lib()
        self._lib = lib
        self.batch = batch
        self.device = int(device)
        opts = _abi.PlanOptions()
        lib.bc_default_options(C.byref(opts))
        opts.precision = _PREC[precision]
        opts.threads_per_tile = int(threads_per_tile)
        opts.tile_nodes = int(tile_nodes)
        opts.lane_nodes = int(lane_nodes)
        opts.narrow_lane_nodes = int(narrow_lane_nodes)
        opts.steps_per_launch = int(steps_per_launch)
        opts.record_every = int(record_every)
        opts.max_spikes = int(max_spikes)
        opts.use_graph = int(bool(use_graph))
        opts.device = self.device
        opts.threads_big = int(threads_big)
        opts.threads_global = int(threads_global)
        opts.dry_run = int(bool(dry_run))
        opts.lane_cell_nodes = int(lane_cell_nodes)
        opts.tile_order = int(tile_order)
        spec, keep = batch.to_spec()
        handle = C.c_void_p()
        _abi.check(lib.bc_plan_create(C.byref(spec), C.byref(opts), C.byref(handle)))
        del keep
        self._h = handle
        self.precision = precision
        self.max_spikes = int(max_spikes)
        info = _abi.PlanInfo()
        _abi.check(lib.bc_plan_info(self._h, C.byref(info)))
        self.info = info.as_dict()
        self.n_cv = int(info.n_cv)
        self.n_cells = int(info.n_cells)
        self.n_probes = int(info.n_probes)

    def tile_stats(self) -> np.ndarray:
        """``[n_tiles, 6]``: nodes, chain records, phases, critical path, class, shared bytes."""
        out = np.zeros((int(self.info["n_tiles"]), 6), dtype=np.int64)
        _abi.check(self._lib.bc_plan_tile_stats(self._h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    # ------------------------------------------------------------------ lifecycle
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.bc_plan_destroy(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    def _stream(self, stream) -> C.c_void_p:
        return C.c_void_p(current_stream(self.device) if stream is None else int(stream))

    # ------------------------------------------------------------------ stepping
    def reset(self, stream=None) -> None:
        _abi.check(self._lib.bc_reset(self._h, self._stream(stream)))

    def run(self, n_steps: int, dt: float, stream=None, check: bool = True) -> None:
        if check:
            _abi.check(self._lib.bc_run(self._h, int(n_steps), float(dt), self._stream(stream)))
        else:
            _abi.check(self._lib.bc_run_async(self._h, int(n_steps), float(dt), self._stream(stream)))

    def check(self, stream=None) -> None:
        _abi.check(self._lib.bc_check(self._h, self._stream(stream)))

    def run_timed(self, n_steps: int, dt: float, stream=None) -> float:
        ms = C.c_double()
        _abi.check(self._lib.bc_run_timed(self._h, int(n_steps), float(dt), self._stream(stream), C.byref(ms)))
        return float(ms.value)

    # ------------------------------------------------------------------ surrogate ports
    def set_surrogate(self, theta, norm, stream=None) -> None:
        """Give the plan's ports their GRU: flat FP32 parameters and the five norm
        values (v_scale, y_scale, env_v_lo, env_v_hi, env_dvdt)."""
        th = np.ascontiguousarray(theta, dtype=np.float32)
        nm = np.ascontiguousarray(norm, dtype=np.float32)
        if th.size != int(self._lib.bc_gru_nparam()) or nm.size != _abi.BC_SURROGATE_NORM:
            raise ValueError("GRU parameter vector or norm of the wrong size.")
        fp = C.POINTER(C.c_float)
        _abi.check(self._lib.bc_surrogate_set(self._h, th.ctypes.data_as(fp), nm.ctypes.data_as(fp),
                                              self._stream(stream)))

    def surrogate_flags(self, stream=None) -> np.ndarray:
        """Per cell: 1 when a port input left the envelope since the last reset."""
        out = np.zeros(self.n_cells, dtype=np.int32)
        _abi.check(self._lib.bc_surrogate_flags(self._h, out.ctypes.data_as(C.POINTER(C.c_int32)),
                                                self._stream(stream)))
        return out

    @property
    def step_count(self) -> int:
        n = C.c_int64()
        _abi.check(self._lib.bc_step_count(self._h, C.byref(n)))
        return int(n.value)

    # ------------------------------------------------------------------ views
    def cell_ncv(self) -> np.ndarray:
        out = np.zeros(self.n_cells, dtype=np.int64)
        _abi.check(self._lib.bc_plan_cell_ncv(self._h, out.ctypes.data_as(C.POINTER(C.c_int64))))
        return out

    def state(self, name: str = "V", stream=None) -> np.ndarray:
        """Per-CV float64 copy of a state (NaN where the mechanism is absent)."""
        which = _abi.STATE_NAMES[name]
        out = np.empty(self.n_cv, dtype=np.float64)
        _abi.check(
            self._lib.bc_state_download(self._h, which, out.ctypes.data_as(C.POINTER(C.c_double)), self._stream(stream))
        )
        return out

    def state_into(self, name: str, out: np.ndarray, stream=None) -> np.ndarray:
        """Like :meth:`state`, into a caller-held float64 array, with no device allocation.

        Goes through ``bc_state_download_noalloc``: fixed library scratch instead of
        per-call buffers, for plans of at most ``BC_NOALLOC_MAX_CV`` CVs.  Calls from
        several threads at once race on that scratch and must be serialised.
        """
        if out.dtype != np.float64 or out.shape != (self.n_cv,) or not out.flags.c_contiguous:
            raise ValueError(f"out must be a contiguous float64 array of shape ({self.n_cv},)")
        which = _abi.STATE_NAMES[name]
        _abi.check(
            self._lib.bc_state_download_noalloc(
                self._h, which, out.ctypes.data_as(C.POINTER(C.c_double)), self._stream(stream))
        )
        return out

    def spike_state(self, v_th: float = 0.0, stream=None) -> np.ndarray:
        """Per-CV spike indicator of the last step taken (1.0 where V_last < v_th <= V),
        the reference's ``Cell.spike`` after a step; all zero after a reset."""
        out = np.empty(self.n_cv, dtype=np.float64)
        _abi.check(self._lib.bc_spike_state_download(self._h, float(v_th), out.ctypes.data_as(C.POINTER(C.c_double)),
                                                     self._stream(stream)))
        return out

    def set_pulse_amps(self, amps_nA, stream=None) -> None:
        """New amplitudes (nA) for every clamp pulse of the batch, in batch order."""
        arr = np.ascontiguousarray(np.asarray(amps_nA, dtype=np.float64).reshape(-1))
        if arr.size != int(self.batch.pulse_cell.size):
            raise ValueError(f"expected {self.batch.pulse_cell.size} amplitudes, got {arr.size}")
        _abi.check(self._lib.bc_pulse_set_amp(self._h, arr.ctypes.data_as(C.POINTER(C.c_double)),
                                              self._stream(stream)))

    def set_state(self, name: str, values, stream=None) -> None:
        which = _abi.STATE_NAMES[name]
        arr = np.ascontiguousarray(np.broadcast_to(np.asarray(values, dtype=np.float64), (self.n_cv,)))
        _abi.check(
            self._lib.bc_state_upload(self._h, which, arr.ctypes.data_as(C.POINTER(C.c_double)), self._stream(stream))
        )

    def traces(self, stream=None) -> np.ndarray:
        """Probe voltages, shape ``[n_probes, n_records]``."""
        n = C.c_int64()
        _abi.check(self._lib.bc_probe_count(self._h, C.byref(n)))
        rec = int(n.value)
        out = np.empty((rec, self.n_probes), dtype=np.float64)
        if rec and self.n_probes:
            _abi.check(
                self._lib.bc_probe_download(
                    self._h, out.ctypes.data_as(C.POINTER(C.c_double)), rec, self._stream(stream)
                )
            )
        return out.T.copy()

    def spikes(self, stream=None) -> list[np.ndarray]:
        """Upward 0 mV crossing times (ms) per probe, at most ``max_spikes`` each."""
        counts = np.zeros(max(self.n_probes, 1), dtype=np.int32)
        times = np.zeros(max(self.n_probes, 1) * max(self.max_spikes, 1), dtype=np.float64)
        if self.n_probes:
            _abi.check(
                self._lib.bc_spike_download(
                    self._h,
                    counts.ctypes.data_as(C.POINTER(C.c_int32)),
                    times.ctypes.data_as(C.POINTER(C.c_double)),
                    self._stream(stream),
                )
            )
        times = times.reshape(max(self.n_probes, 1), max(self.max_spikes, 1))
        return [times[k, : min(int(counts[k]), self.max_spikes)].copy() for k in range(self.n_probes)]

    def spike_counts(self, stream=None) -> np.ndarray:
        counts = np.zeros(max(self.n_probes, 1), dtype=np.int32)
        if self.n_probes:
            _abi.check(
                self._lib.bc_spike_download(self._h, counts.ctypes.data_as(C.POINTER(C.c_int32)), None,
                                            self._stream(stream))
            )
        return counts[: self.n_probes]

    def clear_probes(self, stream=None) -> None:
        _abi.check(self._lib.bc_probe_clear(self._h, self._stream(stream)))
