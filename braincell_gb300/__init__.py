"""braincell_gb300: the multi-compartment Cell time step of braincell, native on GB300 (sm_103a).

Public surface (mirrors the reference's names on this path):

* morphology -- :class:`Branch`, :class:`Morphology`
* declarations -- ``mech`` (CableProperty, Channel, Ion, CurrentClamp, StateProbe,
  regions / locsets, CV policies)
* :class:`Cell` -- paint / place / init_state / reset_state / update / run
* :class:`SingleCompartment` -- point neurons, ``update(I_ext)`` per step
* ``quad`` -- integrator registry with ``"gb300_staggered"`` registered
* :class:`CellBatch` / :class:`Plan` -- many heterogeneous cells in one device plan
"""

from . import environ, mech, quad
from .batch import CellBatch, concat_batches, lower_cell
from .cell import Cell, RunResult
from .morph import Branch, Morphology
from .runtime import Plan
from .single import SingleCompartment

__all__ = [
    "Branch",
    "Morphology",
    "Cell",
    "RunResult",
    "CellBatch",
    "Plan",
    "SingleCompartment",
    "concat_batches",
    "lower_cell",
    "environ",
    "mech",
    "quad",
]

__version__ = "0.1.0"
