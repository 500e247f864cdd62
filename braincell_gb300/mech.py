"""Mechanism, region/locset and CV-policy declarations consumed by :class:`Cell`.

Mirrors the declaration names of the reference:

* ``CableProperty`` -- ``mech/_cable.py:42`` (defaults -65 mV, 1 uF/cm^2,
  100 ohm*cm, 36 degC as in ``_discretization/mechanism.py:66``).
* ``Channel`` / ``Ion`` -- ``mech/_density.py:315`` / ``:428`` (class name plus
  keyword parameters).
* ``CurrentClamp`` -- ``mech/_point.py:86`` (delay, durations, amplitudes).
* ``AllRegion``, ``branch_in``, ``RootLocation``, ``at`` -- ``filter/region.py:85,228``,
  ``filter/locset.py:105,110``.
* ``CVPerBranch``, ``CVPerBranchList``, ``MaxCVLen``, ``CompositeByTypePolicy``,
  ``CVPolicyByTypeRule`` -- ``_discretization/policy.py:84,124,177,298,328``.

Parameters are plain floats in fixed units: mV, ms, um, nA, mS/cm^2 for
conductance densities, uF/cm^2, ohm*cm, kelvin, mM.
"""

from __future__ import annotations

import math
import warnings
from dataclasses import dataclass, field
from typing import Sequence

import numpy as np

__all__ = [
    "CableProperty",
    "Channel",
    "Ion",
    "CurrentClamp",
    "StateProbe",
    "MechanismProbe",
    "CurrentProbe",
    "AllRegion",
    "BranchInFilter",
    "branch_in",
    "RootLocation",
    "AtLocation",
    "at",
    "CVPolicy",
    "CVPerBranch",
    "CVPerBranchList",
    "MaxCVLen",
    "CVPolicyByTypeRule",
    "CompositeByTypePolicy",
    "celsius2kelvin",
]

EPS_PARAM = 1e-9
EPS_LEN_UM = 1e-6


def celsius2kelvin(t_c: float) -> float:
    return float(t_c) + 273.15


# ----------------------------------------------------------------------------
# Density / point mechanism declarations


@dataclass(frozen=True)
class CableProperty:
    resting_potential: float = -65.0
    membrane_capacitance: float = 1.0
    axial_resistivity: float = 100.0
    temperature: float = field(default_factory=lambda: celsius2kelvin(36.0))

    def __post_init__(self) -> None:
        if self.membrane_capacitance <= 0.0:
            raise ValueError("membrane_capacitance must be > 0.")
        if self.axial_resistivity <= 0.0:
            raise ValueError("axial_resistivity must be > 0.")


class _Density:
    category = "density"

    def __init__(self, class_name, *, name: str | None = None, **params) -> None:
        if isinstance(class_name, type):
            class_name = class_name.__name__
        if not isinstance(class_name, str) or not class_name:
            raise TypeError(f"class_name must be a non-empty str, got {class_name!r}.")
        self.class_name = class_name
        self.name = name
        self.params = dict(params)

    @property
    def instance_name(self) -> str:
        return self.name if self.name is not None else self.class_name

    def __repr__(self) -> str:
        return f"{type(self).__name__}({self.class_name!r}, {self.params})"


# The reference keeps the class names from before its rename (the new name with a
# leading ``I``) as deprecated aliases that warn and resolve to the new class
# (channel/__init__.py:49-86); a declaration under an old name resolves the same way.
DEPRECATED_CHANNEL_NAMES = {
    "INa_HH1952": "Na_HH1952", "INa_Ba2002": "Na_Ba2002", "INa_TM1991": "Na_TM1991", "IK_HH1952": "K_HH1952",
    "IK_TM1991": "K_TM1991", "IK_Leak": "K_Leak", "IKDR_Ba2002": "KDR_Ba2002", "IKNI_Ya1989": "KNI_Ya1989",
    "IKA1_HM1992": "KA1_HM1992", "IKA2_HM1992": "KA2_HM1992", "IKK2A_HM1992": "KK2A_HM1992",
    "IKK2B_HM1992": "KK2B_HM1992", "ICaN_IS2008": "CaN_IS2008", "ICaL_IS2008": "CaL_IS2008",
    "ICaT_HM1992": "CaT_HM1992", "ICaT_HP1992": "CaT_HP1992", "ICaHT_HM1992": "CaHT_HM1992",
    "ICaHT_Re1993": "CaHT_Re1993", "IAHP_De1994": "AHP_De1994",
}


class Channel(_Density):
    """Distributed ion-channel declaration: ``Channel("Na_Ba2002", g_max=120.0)``."""

    category = "channel"

    def __init__(self, class_name, *, name: str | None = None, **params) -> None:
        if isinstance(class_name, str) and class_name in DEPRECATED_CHANNEL_NAMES:
            new = DEPRECATED_CHANNEL_NAMES[class_name]
            warnings.warn(f"{class_name} is deprecated and will be removed; use {new} instead.", DeprecationWarning,
                          stacklevel=2)
            class_name = new
        super().__init__(class_name, name=name, **params)


class Ion(_Density):
    """Ion declaration: ``Ion("CalciumDetailed", C_rest=5e-5, tau=10.0, d=0.5)``."""

    category = "ion"


@dataclass(frozen=True)
class CurrentClamp:
    """Piecewise-constant clamp: segment ``k`` is active for
    ``starts[k] <= t - delay < ends[k]`` with ``ends = cumsum(durations)``."""

    delay: float = 0.0
    durations: Sequence[float] | float = 1.0
    amplitudes: Sequence[float] | float = 0.0

    def __post_init__(self) -> None:
        d = np.atleast_1d(np.asarray(self.durations, dtype=np.float64))
        a = np.atleast_1d(np.asarray(self.amplitudes, dtype=np.float64))
        if d.shape != a.shape:
            raise ValueError("durations and amplitudes must have the same length.")
        if np.any(d <= 0.0):
            raise ValueError("CurrentClamp durations must be > 0.")
        object.__setattr__(self, "durations", tuple(float(x) for x in d))
        object.__setattr__(self, "amplitudes", tuple(float(x) for x in a))

    def segments(self) -> list[tuple[float, float, float]]:
        """Absolute ``(t_on, t_off, amplitude_nA)`` per segment."""
        out = []
        start = 0.0
        for dur, amp in zip(self.durations, self.amplitudes):
            out.append((self.delay + start, self.delay + start + dur, amp))
            start += dur
        return out


@dataclass(frozen=True)
class ExpSyn:
    """Exponential synapse placed at a point (``synapse/markov.py:65``, NEURON
    ``expsyn.mod``): state ``g`` (uS) with ``g' = -g / tau``; an arriving event adds
    its weight to ``g`` at the start of a step; current ``i = g (V - e)`` (nA,
    outward positive).  ``weight`` is the default event weight of connections that
    give none.
    """

    tau: float = 0.1      # ms
    e: float = 0.0        # mV
    weight: float = 1.0   # uS
    name: str | None = None

    def __post_init__(self) -> None:
        if not (self.tau > 0.0):
            raise ValueError(f"ExpSyn tau must be > 0 ms, got {self.tau}.")


@dataclass(frozen=True)
class StateProbe:
    """Voltage probe at a placed location (``mech/_point.py:314``; only ``field="v"``)."""

    name: str | None = None
    field: str = "v"

    def __post_init__(self) -> None:
        if self.name is not None and (not isinstance(self.name, str) or not self.name):
            raise ValueError(f"StateProbe.name must be a non-empty string or None, got {self.name!r}.")
        if self.field != "v":
            raise ValueError(f"Unsupported StateProbe field {self.field!r}; only 'v' is supported.")


@dataclass(frozen=True)
class MechanismProbe:
    """Probe of a named mechanism's state at a placed location
    (``mech/_point.py:330``, sampled as ``_multi_compartment/probes.py:136-181``).

    ``mechanism`` is a channel class name (or the ``name`` of a painted Channel) and
    ``field`` one of its gates ("p", "q", "n"), or an ion class with field "Ci".  The
    probe records the state after every recorded step.
    """

    mechanism: str
    field: str
    name: str | None = None

    def __post_init__(self) -> None:
        if self.name is not None and (not isinstance(self.name, str) or not self.name):
            raise ValueError(f"MechanismProbe.name must be a non-empty string or None, got {self.name!r}.")
        for field_name in ("mechanism", "field"):
            value = getattr(self, field_name)
            if not isinstance(value, str) or not value:
                raise ValueError(f"MechanismProbe.{field_name} must be a non-empty string, got {value!r}.")


@dataclass(frozen=True)
class CurrentProbe:
    """Probe of a current density at a placed location (``mech/_point.py:347``,
    sampled as ``_multi_compartment/probes.py:184-258``): the current of the named
    mechanism, or with only ``ion`` the total current of that ion ("na", "k",
    "ca"), in uA/cm^2 as g (E - V), after every recorded step.
    """

    ion: str | None = None
    mechanism: str | None = None
    name: str | None = None

    def __post_init__(self) -> None:
        if self.name is not None and (not isinstance(self.name, str) or not self.name):
            raise ValueError(f"CurrentProbe.name must be a non-empty string or None, got {self.name!r}.")
        if self.ion is not None and (not isinstance(self.ion, str) or not self.ion):
            raise ValueError(f"CurrentProbe.ion must be a non-empty string or None, got {self.ion!r}.")
        if self.mechanism is not None and (not isinstance(self.mechanism, str) or not self.mechanism):
            raise ValueError(f"CurrentProbe.mechanism must be a non-empty string or None, got {self.mechanism!r}.")
        if self.ion is None and self.mechanism is None:
            raise ValueError("CurrentProbe requires at least one of 'ion' or 'mechanism'.")


# ----------------------------------------------------------------------------
# Regions and locsets (branch granularity)


class RegionExpr:
    def branch_mask(self, morpho) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError


@dataclass(frozen=True)
class AllRegion(RegionExpr):
    def branch_mask(self, morpho) -> np.ndarray:
        return np.ones(len(morpho.branches), dtype=bool)


@dataclass(frozen=True)
class BranchInFilter(RegionExpr):
    property: str
    values: tuple

    def branch_mask(self, morpho) -> np.ndarray:
        vals = set(self.values)
        if self.property == "type":
            return np.asarray([b.type in vals for b in morpho.branches], dtype=bool)
        if self.property == "name":
            return np.asarray([n in vals for n in morpho.branch_names], dtype=bool)
        if self.property == "index":
            return np.asarray([i in vals for i in range(len(morpho.branches))], dtype=bool)
        raise ValueError(f"Unsupported branch property {self.property!r}.")


def branch_in(property: str, values) -> BranchInFilter:
    if isinstance(values, (str, int)):
        values = (values,)
    return BranchInFilter(property=property, values=tuple(values))


class LocsetExpr:
    def points(self, morpho) -> list[tuple[int, float]]:  # pragma: no cover - interface
        raise NotImplementedError


@dataclass(frozen=True)
class RootLocation(LocsetExpr):
    x: float

    def points(self, morpho) -> list[tuple[int, float]]:
        return [(0, float(self.x))]


@dataclass(frozen=True)
class AtLocation(LocsetExpr):
    branch: int | str
    x: float

    def points(self, morpho) -> list[tuple[int, float]]:
        idx = morpho.branch(self.branch).index if isinstance(self.branch, str) else int(self.branch)
        return [(idx, float(self.x))]


def at(branch, x: float) -> AtLocation:
    return AtLocation(branch=branch, x=x)


# ----------------------------------------------------------------------------
# CV policies: every policy tiles each branch uniformly; only the count differs.


class CVPolicy:
    def cv_counts(self, morpho) -> np.ndarray:  # pragma: no cover - interface
        raise NotImplementedError

    def resolve_cv_bounds(self, morpho) -> tuple[tuple[tuple[float, float], ...], ...]:
        return tuple(uniform_bounds(int(n)) for n in self.cv_counts(morpho))


def uniform_bounds(n_cv: int) -> tuple[tuple[float, float], ...]:
    return tuple((float(k) / float(n_cv), float(k + 1) / float(n_cv)) for k in range(n_cv))


@dataclass(frozen=True)
class CVPerBranch(CVPolicy):
    cv_per_branch: int = 1

    def __post_init__(self) -> None:
        if isinstance(self.cv_per_branch, bool) or not isinstance(self.cv_per_branch, int):
            raise TypeError(f"cv_per_branch must be integer, got {self.cv_per_branch!r}.")
        if self.cv_per_branch <= 0:
            raise ValueError(f"cv_per_branch must be > 0, got {self.cv_per_branch!r}.")

    def cv_counts(self, morpho) -> np.ndarray:
        return np.full(len(morpho.branches), self.cv_per_branch, dtype=np.int64)


@dataclass(frozen=True)
class CVPerBranchList(CVPolicy):
    cv_per_branch: tuple

    def __post_init__(self) -> None:
        vals = tuple(int(v) for v in self.cv_per_branch)
        if any(v <= 0 for v in vals):
            raise ValueError("every cv_per_branch entry must be > 0.")
        object.__setattr__(self, "cv_per_branch", vals)

    def cv_counts(self, morpho) -> np.ndarray:
        if len(self.cv_per_branch) != len(morpho.branches):
            raise ValueError(
                f"CVPerBranchList has {len(self.cv_per_branch)} entries for {len(morpho.branches)} branches."
            )
        return np.asarray(self.cv_per_branch, dtype=np.int64)


@dataclass(frozen=True)
class MaxCVLen(CVPolicy):
    """``n = ceil(L / max_cv_len - 1e-9)`` CVs per branch, promoted to odd when
    ``keep_odd`` (``_discretization/policy.py:388-407``)."""

    max_cv_len: float
    keep_odd: bool = True

    def __post_init__(self) -> None:
        if not math.isfinite(float(self.max_cv_len)) or float(self.max_cv_len) <= 0.0:
            raise ValueError(f"max_cv_len must be > 0, got {self.max_cv_len!r}.")

    def cv_counts(self, morpho) -> np.ndarray:
        out = []
        for b in morpho.branches:
            L = b.length
            if L <= self.max_cv_len + EPS_LEN_UM:
                out.append(1)
                continue
            n = max(1, int(math.ceil(L / float(self.max_cv_len) - EPS_PARAM)))
            if self.keep_odd and n % 2 == 0:
                n += 1
            out.append(n)
        return np.asarray(out, dtype=np.int64)


@dataclass(frozen=True)
class CVPolicyByTypeRule:
    branch_types: tuple
    policy: CVPolicy

    def __post_init__(self) -> None:
        if isinstance(self.branch_types, str):
            object.__setattr__(self, "branch_types", (self.branch_types,))
        if len(self.branch_types) == 0:
            raise ValueError("CVPolicyByTypeRule.branch_types must be non-empty.")
        if not isinstance(self.policy, CVPolicy):
            raise TypeError("policy must be a CVPolicy.")


@dataclass(frozen=True)
class CompositeByTypePolicy(CVPolicy):
    rules: tuple
    default_policy: CVPolicy

    def cv_counts(self, morpho) -> np.ndarray:
        counts = np.asarray(self.default_policy.cv_counts(morpho), dtype=np.int64).copy()
        for rule in self.rules:
            sub = np.asarray(rule.policy.cv_counts(morpho), dtype=np.int64)
            for i, b in enumerate(morpho.branches):
                if b.type in rule.branch_types:
                    counts[i] = sub[i]
        return counts
