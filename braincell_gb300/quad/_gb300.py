"""The ``"gb300_staggered"`` integrator: the reference's staggered step on a GB300.

Registered like the reference registers ``"staggered"`` (``quad/_staggered.py:47-52``):
``register_integrator("gb300_staggered", aliases=("gb300", "staggered_gb300"),
category="staggered")``.  ``gb300_staggered_step(target, *args)`` advances the
target by one ``dt`` read from the environment, mutating its state in place and
returning ``None``, like ``staggered_step`` (:54-154).  The step runs entirely in
the native library; there is no CPU fallback.

Two hooks let a Cell hand over more than one step at a time:
``init_target(cell)`` builds the device plan, ``run_target(cell, n_steps, dt)``
advances ``n_steps`` fused steps and returns the probe traces.
"""

from __future__ import annotations

from .. import environ
from ._registry import register_integrator

__all__ = ["gb300_staggered_step"]


@register_integrator(
    "gb300_staggered",
    aliases=("gb300", "staggered_gb300"),
    category="staggered",
    description="Staggered DHS voltage / exp-Euler channel step fused into sm_103a kernels.",
)
def gb300_staggered_step(target, *args):
    """Advance ``target`` by one staggered step of ``environ['dt']``.

    A node-tree ``Cell`` is called as ``solver(cell)`` (``cell.py:2379``); a
    ``SingleCompartment`` as ``solver(neuron, I_ext)`` (``_single_compartment/
    base.py:275``), ``I_ext`` being the step's external current density (nA/cm^2).
    """
    from ..single import SingleCompartment

    if isinstance(target, SingleCompartment):
        if len(args) > 1:
            raise TypeError("gb300_staggered_step takes at most one argument (I_ext) for a SingleCompartment.")
        dt = environ.get("dt")
        if target._runtime is None:
            target.init_state()
        target._set_input(args[0] if args else 0.0)
        target._runtime.run(1, float(dt))
        return
    if not (hasattr(target, "batch") and hasattr(target, "morpho")):
        raise TypeError(
            f"The gb300_staggered integrator needs a node-tree Cell or a SingleCompartment target, "
            f"got {type(target).__name__}."
        )
    if args:
        raise TypeError("gb300_staggered_step takes no extra arguments for a Cell target.")
    dt = environ.get("dt")
    if getattr(target, "_runtime", None) is None:
        target.init_state()
    target._runtime.run(1, float(dt))


def _init_target(cell):
    from ..runtime import Plan
    from ..single import SingleCompartment

    if isinstance(cell, SingleCompartment):
        # one neuron per thread (lane tiles) unless the options say otherwise: on a
        # GB300 a population of 1,000,000 runs 2.0e10 steps/s that way against
        # 1.0e10 in packed tiles
        return Plan(cell.batch(cell._v0), record_every=0, **{"lane_cell_nodes": 3, **cell.solver_options})
    return Plan(cell.batch(), **cell.solver_options)


def _run_target(cell, *, n_steps: int, dt: float):
    plan = cell._runtime
    plan.clear_probes()
    plan.run(int(n_steps), float(dt))
    return plan.traces()


gb300_staggered_step.init_target = _init_target
gb300_staggered_step.run_target = _run_target
