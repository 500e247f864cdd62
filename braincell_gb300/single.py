"""``SingleCompartment``: the reference's point-neuron model on the GB300 step.

Mirrors ``braincell/_single_compartment/base.py:33-278``:
``SingleCompartment(size, length=10 um, radius=5 um, C=1 uF/cm^2, V_th=0 mV,
V_initializer, solver, name, **ion_channels)`` with the membrane area
``2 pi radius length`` (:144-147), ``init_state`` / ``reset_state`` (:149-184) and
``update(I_ext)`` (:252-278), which calls ``self.solver(self, I_ext)`` once per step
and returns the spike indicator ``get_spike(last_V, V)`` (``_base.py:421-431``:
1 where ``last_V < V_th <= V``).

``I_ext`` is a current density in nA/cm^2 (the reference's default unit): a scalar or
one value per neuron.  Channels and ions are keyword declarations, e.g.
``SingleCompartment(100, na=Channel("Na_HH1952"), k=Channel("K_HH1952"),
leak=Channel("IL", g_max=0.3, E=-54.4))``.  ``V_initializer`` is a voltage (mV), an
array of ``size`` voltages, or a callable ``shape -> array``; it is evaluated by
``init_state`` and again by every ``reset_state``, and the gates start at their
steady state at each neuron's own voltage, as the reference's channel
``reset_state(V)`` puts them.  (The reference's default draws U(-70, -60) mV; the
default here is -65 mV.)

On the GB300 step the population is one device plan of ``size`` one-CV cylinders,
run one neuron per GPU thread (lane tiles; ``solver_options=dict(lane_cell_nodes=0)``
packs them into CTA tiles instead).
The ``"gb300_staggered"`` solver advances it by the staggered scheme restricted to one
compartment: the ionic current linearised at V_n, one implicit voltage step, then
calcium from the step-start current and every gate by exp-Euler at the new voltage.
The external current of a step reaches the kernel as the amplitude of one clamp
pulse per neuron (``bc_pulse_set_amp``).
"""

from __future__ import annotations

import math

import numpy as np

from . import _abi, environ
from .batch import CellBatch
from .catalogue import region_record
from .mech import CableProperty, Channel, Ion

__all__ = ["SingleCompartment"]

_FOREVER_MS = 1e12  # the per-neuron input pulse never ends


def _shape(size) -> tuple[int, ...]:
    t = (int(size),) if isinstance(size, (int, np.integer)) else tuple(int(x) for x in size)
    if not t or any(x <= 0 for x in t):
        raise ValueError(f"size must be a positive int or tuple of positive ints, got {size!r}.")
    return t


class SingleCompartment:
    def __init__(self, size, length: float = 10.0, radius: float = 5.0, C: float = 1.0, V_th=0.0,
                 V_initializer=-65.0, solver="gb300_staggered", name: str | None = None, *,
                 solver_options: dict | None = None, **ion_channels) -> None:
        from .quad import get_integrator

        self.varshape = _shape(size)
        self.n = int(np.prod(self.varshape))
        if not (length > 0.0 and radius > 0.0 and C > 0.0):
            raise ValueError("length, radius and C must be > 0.")
        self.length, self.radius, self.C = float(length), float(radius), float(C)
        self.V_th = np.broadcast_to(np.asarray(V_th, dtype=np.float64), self.varshape).copy()
        self.V_initializer = V_initializer
        self.name = name
        self.solver = get_integrator(solver)
        self.solver_options = dict(solver_options or {})
        for key, d in ion_channels.items():
            if not isinstance(d, (Channel, Ion)):
                raise TypeError(f"{key}: expected a mech.Channel or mech.Ion declaration, got {type(d).__name__}.")
        self.ion_channels = dict(ion_channels)
        self._runtime = None
        self._v0 = None
        self.spike = None

    @property
    def n_compartment(self) -> int:
        return 1

    @property
    def pop_size(self) -> tuple[int, ...]:
        return self.varshape

    @property
    def area(self) -> float:
        """Membrane area (um^2) that turns an injected current into a density."""
        return 2.0 * math.pi * self.radius * self.length

    # ------------------------------------------------------------------ lowering
    def _initial_voltages(self) -> np.ndarray:
        v = self.V_initializer(self.varshape) if callable(self.V_initializer) else self.V_initializer
        v = np.broadcast_to(np.asarray(v, dtype=np.float64), self.varshape).reshape(-1).copy()
        if not np.all(np.isfinite(v)):
            raise ValueError("V_initializer gave a non-finite voltage.")
        return v

    def batch(self, v0: np.ndarray) -> CellBatch:
        """``n`` one-branch, one-CV cylinders; neuron k's region carries V_rest = v0[k] so
        that a reset puts its gates at their steady state there; one input pulse each."""
        n = self.n
        mechs = list(self.ion_channels.values())
        params = np.zeros((n, _abi.BC_NPARAM))
        bits = np.zeros(n, np.uint32)
        cache: dict[float, tuple] = {}
        for k in range(n):
            key = float(v0[k])
            if key not in cache:
                cache[key] = region_record(mechs, CableProperty(resting_potential=key, membrane_capacitance=self.C))
            bits[k], params[k] = cache[key]
        z = np.zeros(n)
        return CellBatch(
            n_regions=1,
            cell_branch_offsets=np.arange(n + 1, dtype=np.int64),
            branch_parent=np.full(n, -1, np.int32),
            branch_parent_x=z.copy(),
            branch_child_x=z.copy(),
            branch_ncv=np.ones(n, np.int32),
            branch_region=np.zeros(n, np.int32),
            branch_seg_offsets=np.arange(n + 1, dtype=np.int64),
            seg_length=np.full(n, self.length),
            seg_r_prox=np.full(n, self.radius),
            seg_r_dist=np.full(n, self.radius),
            region_cm=np.full(n, self.C),
            region_ra=np.full(n, 100.0),
            region_mech=bits,
            region_params=params,
            pulse_cell=np.arange(n, dtype=np.int32),
            pulse_branch=np.zeros(n, np.int32),
            pulse_x=np.full(n, 0.5),
            pulse_t_on=np.full(n, -1.0),
            pulse_t_off=np.full(n, _FOREVER_MS),
            pulse_amp=z.copy(),
        )

    # ------------------------------------------------------------------ lifecycle
    def init_state(self, batch_size=None) -> None:
        if self._runtime is not None:
            return
        init = getattr(self.solver, "init_target", None)
        if init is None:
            raise TypeError(f"Solver {self.solver!r} cannot initialise a SingleCompartment runtime.")
        self._v0 = self._initial_voltages()
        self._runtime = init(self)
        self._runtime.reset()
        self._amps = np.zeros(self.n)
        self.spike = np.zeros(self.varshape)

    def reset_state(self, batch_size=None) -> None:
        if self._runtime is None:
            raise RuntimeError("reset_state() requires init_state() first.")
        v0 = self._initial_voltages()
        if not np.array_equal(v0, self._v0):  # new starting voltages: new steady-state gates
            self._runtime.close()
            self._runtime = None
            self.init_state()
            self._v0 = v0
            return
        self._runtime.reset()
        self.spike = np.zeros(self.varshape)

    def close(self) -> None:
        if self._runtime is not None:
            self._runtime.close()
        self._runtime = None

    @property
    def V(self) -> np.ndarray:
        if self._runtime is None:
            raise RuntimeError("V requires init_state() first.")
        return self._runtime.state("V").reshape(self.varshape)

    def state(self, name: str) -> np.ndarray:
        return self._runtime.state(name).reshape(self.varshape)

    # ------------------------------------------------------------------ stepping
    def _set_input(self, I_ext) -> None:
        """External current density (nA/cm^2) of the coming step -> pulse amplitudes (nA)."""
        dens = np.broadcast_to(np.asarray(I_ext, dtype=np.float64), self.varshape).reshape(-1)
        amps = dens * (self.area * 1e-8)  # nA/cm^2 x cm^2
        if not np.array_equal(amps, self._amps):
            self._runtime.set_pulse_amps(amps)
            self._amps = amps.copy()

    def update(self, I_ext=0.0) -> np.ndarray:
        """One step through ``self.solver(self, I_ext)``; returns the spike indicator."""
        if self._runtime is None:
            self.init_state()
        if environ.get("dt", None) is None:
            raise ValueError("SingleCompartment.update(...) requires environ['dt'] to be set.")
        self.solver(self, I_ext)
        rt = self._runtime
        if np.all(self.V_th == self.V_th.flat[0]):
            spk = rt.spike_state(float(self.V_th.flat[0]))
        else:
            v, last = rt.state("V"), rt.state("V_last")
            th = self.V_th.reshape(-1)
            spk = ((last < th) & (v >= th)).astype(np.float64)
        self.spike = spk.reshape(self.varshape)
        return self.spike
