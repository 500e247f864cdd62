"""``Cell``: declaration front end whose step is resolved through the integrator registry.

Mirrors the reference's ``braincell.Cell`` surface used on this path
(``_multi_compartment/cell.py:203-268`` constructor, ``:383-401`` paint/place,
``:490-552`` init_state, ``:2529-2550`` reset_state, ``:2288-2387`` update /
_update_dynamics, ``:2699`` run): a Cell is built from a
:class:`~braincell_gb300.morph.Morphology`, mechanisms are painted on regions and
point mechanisms placed at locations, and each step calls ``self.solver(self)``.
The solver defaults to ``"gb300_staggered"``; ``Cell.run`` hands the whole time
loop to the solver's batch runner when it has one (the GPU path fuses steps).
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import environ
from .batch import lower_cell
from .mech import CurrentProbe, CVPerBranch, CVPolicy, MechanismProbe, StateProbe
from .morph import Morphology

__all__ = ["Cell", "RunResult"]


@dataclass(frozen=True)
class RunResult:
    """``time``: ``(n_steps,)`` ms; ``traces``: probe name -> ``(pop, n_steps)`` mV."""

    time: np.ndarray
    traces: dict


def _pop(pop_size) -> tuple[int, ...]:
    if isinstance(pop_size, (int, np.integer)):
        if pop_size <= 0:
            raise ValueError(f"pop_size must be > 0, got {pop_size}.")
        return (int(pop_size),)
    t = tuple(int(x) for x in pop_size)
    if any(x <= 0 for x in t):
        raise ValueError(f"pop_size entries must be > 0, got {pop_size}.")
    return t


class Cell:
    def __init__(
        self,
        morpho: Morphology,
        *,
        pop_size=1,
        cv_policy: CVPolicy | None = None,
        V_th: float = 0.0,
        V_init: float | None = None,
        solver="gb300_staggered",
        cache_ion_total_current: bool = True,
        ion_channel_update_order: str = "family",
        name: str | None = None,
        **solver_options,
    ) -> None:
        from .quad import get_integrator

        if not isinstance(morpho, Morphology):
            raise TypeError(f"Cell expects Morphology, got {type(morpho).__name__!s}.")
        self.morpho = morpho
        self.pop_size = _pop(pop_size)
        self.cv_policy = CVPerBranch() if cv_policy is None else cv_policy
        if not isinstance(self.cv_policy, CVPolicy):
            raise TypeError(f"cv_policy must be CVPolicy, got {type(self.cv_policy).__name__!s}.")
        self.V_th = float(V_th)
        self.V_init = None if V_init is None else float(V_init)
        if not cache_ion_total_current:
            raise ValueError("The GB300 step always uses the step-start ion-current cache (cache_ion_total_current=True).")
        if ion_channel_update_order != "family":
            raise ValueError("ion_channel_update_order must be 'family' on the GB300 step.")
        self.cache_ion_total_current = True
        self.ion_channel_update_order = "family"
        self.name = name
        self.solver = get_integrator(solver)
        self.solver_options = dict(solver_options)
        self.paint_rules: list = []
        self.place_rules: list = []
        self._initialized = False
        self._runtime = None  # the solver's device state lives here (e.g. a Plan)
        self.spike = None
        _ = self.cv_policy.cv_counts(morpho)  # eager policy validation

    # ------------------------------------------------------------------ declaration
    def _raise_if_initialized(self, what: str) -> None:
        if self._initialized:
            raise RuntimeError(f"Cell.{what} is not allowed after init_state(); call reset() first.")

    def paint(self, region, *mechanisms) -> "Cell":
        self._raise_if_initialized("paint()")
        if not mechanisms:
            raise ValueError("paint() needs at least one mechanism.")
        self.paint_rules.append((region, tuple(mechanisms)))
        return self

    def place(self, locset, *mechanisms) -> "Cell":
        self._raise_if_initialized("place()")
        if not mechanisms:
            raise ValueError("place() needs at least one mechanism.")
        self.place_rules.append((locset, tuple(mechanisms)))
        return self

    @property
    def n_cv(self) -> int:
        return int(np.sum(self.cv_policy.cv_counts(self.morpho)))

    @property
    def varshape(self) -> tuple[int, ...]:
        return self.pop_size + (self.n_cv,)

    def batch(self):
        """The :class:`CellBatch` of this cell's ``pop_size`` replicas."""
        return lower_cell(self)

    def probe_names(self) -> list[str]:
        names = []
        k = 0
        for locset, decls in self.place_rules:
            for _pt in locset.points(self.morpho):
                for d in decls:
                    if isinstance(d, (StateProbe, MechanismProbe, CurrentProbe)):
                        names.append(d.name if d.name is not None else f"probe_{k}")
                        k += 1
        return names

    # ------------------------------------------------------------------ lifecycle
    def init_state(self, batch_size=None) -> None:
        if self._initialized:
            return
        init = getattr(self.solver, "init_target", None)
        if init is None:
            raise TypeError(f"Solver {self.solver!r} cannot initialise a Cell runtime.")
        self._runtime = init(self)
        self._initialized = True
        self.reset_state()

    def reset_state(self, batch_size=None) -> None:
        if not self._initialized:
            raise RuntimeError("reset_state() requires init_state() first.")
        self._runtime.reset()
        self.spike = np.zeros(self.varshape)

    def reset(self) -> None:
        """Tear the runtime down and return to the declaration phase."""
        if self._runtime is not None:
            self._runtime.close()
        self._runtime = None
        self._initialized = False

    @property
    def V(self) -> np.ndarray:
        if not self._initialized:
            raise RuntimeError("V requires init_state() first.")
        return self._runtime.state("V").reshape(self.varshape)

    def state(self, name: str) -> np.ndarray:
        return self._runtime.state(name).reshape(self.varshape)

    @property
    def current_time(self) -> float:
        dt = environ.get("dt", None)
        return 0.0 if dt is None else self._runtime.step_count * dt

    # ------------------------------------------------------------------ stepping
    def update(self):
        """One step through ``self.solver(self)``; returns the spike indicator per CV."""
        if not self._initialized:
            self.init_state()
        if environ.get("dt", None) is None:
            raise ValueError("Cell.update(...) requires environ['dt'] to be set.")
        self.solver(self)
        # get_spike(last_V, V) per CV (_base.py:421-431), from the voltage the device
        # kept at the start of the step
        self.spike = self._runtime.spike_state(self.V_th).reshape(self.varshape)
        return self.spike

    def run(self, *, dt: float, duration: float) -> RunResult:
        """Advance ``duration`` ms at ``dt`` ms and return the probe traces."""
        if not (dt > 0.0) or not (duration > 0.0):
            raise ValueError("Cell.run(...) needs dt > 0 and duration > 0.")
        names = self.probe_names()
        if not names:
            raise ValueError("Cell.run(...) requires at least one placed probe.")
        if not self._initialized:
            self.init_state()
        n_steps = int(np.arange(0.0, duration, dt).shape[0])
        runner = getattr(self.solver, "run_target", None)
        if runner is None:
            raise TypeError("The selected solver provides no batch runner for Cell.run().")
        t0 = self.current_time if environ.get("dt", None) == dt else self._runtime.step_count * dt
        traces = runner(self, n_steps=n_steps, dt=dt)  # [n_probe_total, n_steps]
        # Cell.spike holds the last step's per-CV indicator, as after n calls of update()
        self.spike = self._runtime.spike_state(self.V_th).reshape(self.varshape)
        P = int(np.prod(self.pop_size))
        nprobe = len(names)
        tr = traces.reshape(P, nprobe, -1)
        out = {n: tr[:, k, :].reshape(self.pop_size + (tr.shape[-1],)) for k, n in enumerate(names)}
        time = t0 + dt * np.arange(n_steps)
        return RunResult(time=time, traces=out)
