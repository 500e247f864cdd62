"""Float64 restatement of ``SingleCompartment.update(I_ext)`` under the staggered scheme.

Test infrastructure only (it checks the GPU path; no product module imports it).

The reference step (``braincell/_single_compartment/base.py:252-278``) is
``last_V = V; solver(self, I_ext); spike = get_spike(last_V, V)`` with
``C dV/dt = sum_j g_j (E_j - V) + I_ext`` (``:209-227``, ``I_ext`` a density in
nA/cm^2, the channel currents in uA/cm^2) and the HH gates of ``channel/_base.py``.
The staggered scheme of ``quad/_staggered.py:54-154`` restricted to one compartment
is, per step:

1. the calcium ion's total current cached at V_n (``cell.py:2261-2280``);
2. the ionic current linearised at V_n, ``I(V) ~ I_n - G_n (V - V_n)``, and one
   implicit-Euler voltage step, ``V_{n+1} = V_n + dt (I_n + I_ext) / C / (1 + dt G_n / C)``
   (``_staggered.py:449-513, 763-795`` with no axial terms);
3. CalciumDetailed Ci by exp-Euler from the cached current (``ion/calcium.py:499-505``);
4. every gate by exp-Euler at V_{n+1} (``quad/_exp_euler.py:330-478``);
5. the spike indicator ``last_V < V_th <= V`` (``_base.py:421-431``).

It is written without the node tree so that it checks the GPU's one-CV tree path
from a second route; the rate functions and parameter defaults are the oracle's
(``oracle/staggered.py``).
"""

from __future__ import annotations

import numpy as np

from .staggered import (_CA_FIXED_CI, _GATES, _ION_OF, CHANNEL_DEFAULTS, ION_DEFAULTS, _resolve, ca_detailed_rate,
                        exp_euler, gate_step, nernst_ca_mV, rates)

__all__ = ["OracleSingleCompartment"]


class OracleSingleCompartment:
    """``n`` point neurons with the channels / ions of ``decls`` (mech declarations)."""

    def __init__(self, n: int, decls, *, C: float = 1.0, V_init=-65.0, V_th: float = 0.0) -> None:
        from braincell_gb300.mech import Ion

        self.n = int(n)
        self.C = float(C)
        self.V_th = float(V_th)
        self.E_na = ION_DEFAULTS["SodiumFixed"]["E"]
        self.E_k = ION_DEFAULTS["PotassiumFixed"]["E"]
        self.E_ca_fixed = ION_DEFAULTS["CalciumFixed"]["E"]
        self.ca = None
        self.chan = {}
        for d in decls:
            if isinstance(d, Ion):
                p = _resolve(ION_DEFAULTS, d)
                if d.class_name == "SodiumFixed":
                    self.E_na = p["E"]
                elif d.class_name == "PotassiumFixed":
                    self.E_k = p["E"]
                elif d.class_name == "CalciumFixed":
                    self.E_ca_fixed = p["E"]
                elif d.class_name == "CalciumDetailed":
                    self.ca = p
                else:
                    raise ValueError(f"unsupported ion {d.class_name}")
            else:
                self.chan["IL" if d.class_name == "leaky" else d.class_name] = _resolve(CHANNEL_DEFAULTS, d)
        self.V = np.broadcast_to(np.asarray(V_init, dtype=np.float64), (self.n,)).copy()
        self.Ci = None if self.ca is None else np.full(self.n, self.ca["Ci_initializer"])
        self.gates = {}
        for name, ch in self.chan.items():
            if name in _GATES:
                r = rates(name, self.V, ch, Ci=self._ci())
                for gate, _, _ in _GATES[name]:
                    kind, a, b = r[gate]
                    self.gates[(name, gate)] = a / (a + b) if kind == "ab" else np.asarray(a, dtype=np.float64)
        self.spike = np.zeros(self.n)

    def _ci(self):
        return np.full(self.n, _CA_FIXED_CI) if self.Ci is None else self.Ci

    def _E(self, ion):
        if ion == "na":
            return self.E_na
        if ion == "k":
            return self.E_k
        if self.ca is not None:
            return nernst_ca_mV(self.ca["temp"], self.ca["Co"], self.Ci)
        return self.E_ca_fixed

    def _g(self, name):
        g = self.chan[name]["g_max"]
        for gate, power, _ in _GATES.get(name, ()):
            g = g * self.gates[(name, gate)] ** power
        return g

    def currents(self, V):
        """Total ionic current (uA/cm^2), its conductance G = -dI/dV and the calcium current."""
        I = np.zeros(self.n)
        G = np.zeros(self.n)
        I_ca = np.zeros(self.n)
        for name, ch in self.chan.items():
            g = self._g(name)
            if name == "IL" or name == "HCN_HM1992":
                E = ch["E"]
            elif name == "K_Leak":
                E = self.E_k
            else:
                E = self._E(_ION_OF[name])
            I = I + g * (E - V)
            G = G + g
            if _ION_OF.get(name) == "ca":
                I_ca = I_ca + g * (E - V)
        return I, G, I_ca

    def update(self, dt: float, I_ext=0.0):
        """One step with the external current density I_ext (nA/cm^2); returns the spikes."""
        last_V = self.V
        I, G, I_ca = self.currents(self.V)
        I_tot = I + 1e-3 * np.broadcast_to(np.asarray(I_ext, dtype=np.float64), (self.n,))
        V_new = self.V + dt * (I_tot / self.C) / (1.0 + dt * G / self.C)
        self.V = V_new
        if self.ca is not None:
            f = ca_detailed_rate(I_ca, self.Ci, self.ca["d"], self.ca["tau"], self.ca["C_rest"])
            self.Ci = exp_euler(self.Ci, f, -1.0 / self.ca["tau"], dt)
        new = {}
        for name, ch in self.chan.items():
            if name not in _GATES:
                continue
            r = rates(name, V_new, ch, Ci=self._ci())
            for gate, _, phik in _GATES[name]:
                kind, a, b = r[gate]
                new[(name, gate)] = gate_step(self.gates[(name, gate)], kind, a, b, ch[phik], dt)
        self.gates.update(new)
        self.spike = ((last_V < self.V_th) & (V_new >= self.V_th)).astype(np.float64)
        return self.spike
