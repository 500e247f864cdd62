"""Markov (probability-state) channels and the backward-Euler subsolver -- oracle.

TEST INFRASTRUCTURE ONLY.  Imported by ``tests/`` and by ``oracle/staggered.py``
as the checker; never by the product.

Restated from the reference:

* the Markov template, ``channel/_base.py:677-1125``:
  - transitions ``(src, dst, forward, backward)``; the states in order of first
    appearance in ``pairs`` (:757-772);
  - one *dependent* state, reconstructed as ``conserve - sum(independent)`` from the
    raw stored states (:852-865);
  - the kinetics see each independent state clipped to [0, 1] (``clip_states``,
    :867-878) and the dependent state from the raw sum;
  - ``compute_derivative`` (:1105-1125): for each transition, ``src -> dst`` at
    ``forward * s[src]`` and back at ``backward * s[dst]``;
  - the steady state (:1033-1091): the generator with the dependent state's row
    replaced by ones (right-hand side ``conserve``), solved, clipped at 0 and
    renormalised to ``conserve``;
  - ``make_integration`` (:807-812): ``substeps`` solver calls of dt / substeps
    (default 1, solver ``backward_euler``);
* the solver, ``quad/_backward_euler.py:31-64``: one linearised implicit step,
  J = df/dy at y_n, (I - dt J) dy = dt f(y_n), y_{n+1} = y_n + dy.  The Jacobian of
  the clipped kinetics takes d clip / dy = 1 for 0 <= y <= 1 and 0 outside (exactly
  on a bound the reference's value follows JAX's derivative rule for ``clip``, which
  is not pinned here), and the dependent state contributes -1 per independent state;
* the channels:
  - ``Nav1p6_MA2020_GoC`` (``channel/sodium.py:727-940``): 13 states, ``I6``
    dependent, current g O (E_Na - V);
  - ``Kca2p2_MA2020_GoC`` (``channel/potassium_calcium.py:613-790``): 6 states,
    ``C1`` dependent, current g (O1 + O2) (E_K - V), calcium-bound rates;
  - ``Kca1p1_MA2020_GoC`` (``channel/potassium_calcium.py:1107-1353``): 10 states,
    ``C0`` dependent, current g (O0 + ... + O4) (E_K - V);
  - ``Nav_MA2020_GrC`` (``channel/sodium.py:1427-1666``): the Nav1.6 graph's 13 states
    (``OB`` for B), ``I6`` dependent, its own rate constants, current g O (E_Na - V).

Units: mV, ms, mM, K.
"""

from __future__ import annotations

import numpy as np

__all__ = ["MarkovScheme", "SCHEMES", "MARKOV_DEFAULTS", "backward_euler", "steady_state", "derivative",
           "jacobian", "scheme_params"]

FARADAY = 96485.33212  # C/mol (CODATA 2018)
GAS_R = 8.314462618  # J/(mol K)


class MarkovScheme:
    """A transition graph with its rate function ``rates(V, Ci, p) -> {name: array}``."""

    def __init__(self, name, pairs, dependent, open_states, ion, rates):
        self.name = name
        self.pairs = tuple(pairs)
        names = []
        for src, dst, _f, _b in self.pairs:
            for s in (src, dst):
                if s not in names:
                    names.append(s)
        self.states = tuple(names)
        self.dependent = dependent
        self.independent = tuple(s for s in names if s != dependent)
        self.open_states = tuple(open_states)
        self.ion = ion
        self.rates = rates

    def index(self, name):
        return self.states.index(name)


# ----------------------------------------------------------------------------- the channels


def _nav16_rates(V, Ci, p):
    """channel/sodium.py:903-935 with the constants of :874-898; Nav1p1_MA2025_BC
    (:1188) replaces Oon (2.3) and epsilon (1e-12)."""
    phi = p["phi"]
    Con, Coff, Oon, Ooff = 0.005, 0.5, p.get("Oon", 0.75), 0.005
    alpha, beta, gamma, delta, epsilon, zeta = 150.0, 3.0, 150.0, 40.0, p.get("epsilon", 1.75), 0.03
    x1, x2, x3, x4, x5, x6 = 20.0, -20.0, 1e12, -1e12, 1e12, -25.0
    vshifta = vshifti = vshiftk = 0.0
    alfac = (Oon / Con) ** 0.25
    btfac = (Ooff / Coff) ** 0.25
    ea = np.exp(V / x1)
    eb = np.exp((V + vshifta) / (x2 + vshiftk))
    ei_a = np.exp((V + vshifti) / x1)
    ei_b = np.exp((V + vshifti) / x2)
    one = np.ones_like(V)
    r = {}
    for k, m in zip((1, 2, 3, 4), (4, 3, 2, 1)):
        r[f"f0{k}"] = m * alpha * ea * phi
        r[f"b0{k}"] = k * beta * eb * phi
        r[f"f1{k}"] = m * alpha * alfac * ei_a * phi
        r[f"b1{k}"] = k * beta * btfac * ei_b * phi
    r["f0O"] = gamma * np.exp(V / x3) * phi
    r["b0O"] = delta * np.exp(V / x4) * phi
    r["fip"] = epsilon * np.exp(V / x5) * phi
    r["bip"] = zeta * np.exp(V / x6) * phi
    r["f1n"] = gamma * np.exp(V / x3) * phi
    r["b1n"] = delta * np.exp(V / x4) * phi
    for k in range(1, 6):
        r[f"fi{k}"] = Con * alfac ** (k - 1) * phi * one
        r[f"bi{k}"] = Coff * btfac ** (k - 1) * phi * one
    r["fin"] = Oon * phi * one
    r["bin"] = Ooff * phi * one
    return r


def _navgrc_rates(V, Ci, p):
    """channel/sodium.py:1427-1666 (Nav_MA2020_GrC): alfa / beta / teta exponentials and
    constant gamma, delta, epsilon, Con, Coff, Oon, Ooff, all times phi; the C and I
    chains carry n1..n4 (back n4..n1)."""
    phi = p["phi"]
    one = np.ones_like(V)
    alfa = phi * 353.91 * np.exp(V / 13.99)
    beta = phi * 1.272 * np.exp(-V / 13.99)
    teta = phi * 0.0201 * np.exp(-V / 25.0)
    gamma, delta, eps = phi * 150.0 * one, phi * 40.0 * one, phi * 1.75 * one
    Con, Coff, Oon, Ooff = phi * 0.005, phi * 0.5, phi * 0.75, phi * 0.005
    a, b = (Oon / Con) ** 0.25, (Ooff / Coff) ** 0.25
    n = (5.422, 3.279, 1.83, 0.738)
    r = {}
    for k in range(4):
        r[f"f0{k + 1}"] = n[k] * alfa
        r[f"b0{k + 1}"] = n[3 - k] * beta
        r[f"f1{k + 1}"] = n[k] * alfa * a
        r[f"b1{k + 1}"] = n[3 - k] * beta * b
    for k in range(1, 6):
        r[f"fi{k}"] = Con * a ** (k - 1) * one
        r[f"bi{k}"] = Coff * b ** (k - 1) * one
    r["f0O"], r["b0O"] = gamma, delta
    r["fip"], r["bip"] = eps, teta
    r["f1n"], r["b1n"] = gamma, delta
    r["fin"], r["bin"] = Oon * one, Ooff * one
    return r


def _kca22_rates(V, Ci, p):
    """channel/potassium_calcium.py:760-790 with the constants of :740-753."""
    phi, diff = p["phi"], p["diff"]
    one = np.ones_like(V)
    ca = Ci * one
    return {
        "dirc2_t_ca": 200.0 * phi * ca / diff, "dirc3_t_ca": 160.0 * phi * ca / diff,
        "dirc4_t_ca": 80.0 * phi * ca / diff,
        "invc1_t": 80e-3 * phi * one, "invc2_t": 80e-3 * phi * one, "invc3_t": 200e-3 * phi * one,
        "invo1_t": 1.0 * phi * one, "invo2_t": 100e-3 * phi * one,
        "diro1_t": 160e-3 * phi * one, "diro2_t": 1.2 * phi * one,
    }


_KCA11_PF = (2.39e-3, 7.0e-3, 40e-3, 295e-3, 557e-3)
_KCA11_PB = (3936e-3, 1152e-3, 659e-3, 486e-3, 92e-3)


def _kca11_rates(V, Ci, p):
    """channel/potassium_calcium.py:1277-1353 with the constants of :1243-1265."""
    phi, T = p["phi"], p["temp"]
    k1, onoff, Kc, Ko = 1.0e3, 1.0, 11.0e-3, 1.1e-3
    one = np.ones_like(V)
    ca = Ci * one
    a = np.exp(0.73 * FARADAY * V * 1e-3 / (GAS_R * T))
    b = np.exp(-0.67 * FARADAY * V * 1e-3 / (GAS_R * T))
    r = {}
    for i, m in enumerate((4, 3, 2, 1)):
        r[f"c{i}{i + 1}"] = m * ca * k1 * onoff * phi
        r[f"o{i}{i + 1}"] = m * ca * k1 * onoff * phi
        r[f"c{i + 1}{i}"] = (i + 1) * Kc * k1 * onoff * phi * one
        r[f"o{i + 1}{i}"] = (i + 1) * Ko * k1 * onoff * phi * one
    for i in range(5):
        r[f"f{i}"] = _KCA11_PF[i] * a * phi
        r[f"b{i}"] = _KCA11_PB[i] * b * phi
    return r


_NAV_PAIRS = (("C1", "C2", "f01", "b01"), ("C2", "C3", "f02", "b02"), ("C3", "C4", "f03", "b03"),
              ("C4", "C5", "f04", "b04"), ("C1", "I1", "fi1", "bi1"), ("I1", "I2", "f11", "b11"),
              ("C2", "I2", "fi2", "bi2"), ("I2", "I3", "f12", "b12"), ("C3", "I3", "fi3", "bi3"),
              ("I3", "I4", "f13", "b13"), ("C4", "I4", "fi4", "bi4"), ("I4", "I5", "f14", "b14"),
              ("C5", "I5", "fi5", "bi5"), ("C5", "O", "f0O", "b0O"), ("O", "B", "fip", "bip"),
              ("I5", "I6", "f1n", "b1n"), ("O", "I6", "fin", "bin"))  # sodium.py:840-858

SCHEMES = {
    "Nav1p1_MA2025_BC": MarkovScheme("Nav1p1_MA2025_BC", _NAV_PAIRS, "I6", ("O",), "na", _nav16_rates),
    "Nav1p1_RI2021_SC": MarkovScheme("Nav1p1_RI2021_SC", _NAV_PAIRS, "I6", ("O",), "na", _nav16_rates),
    "Nav1p6_MA2020_GoC": MarkovScheme(
        "Nav1p6_MA2020_GoC",
        (("C1", "C2", "f01", "b01"), ("C2", "C3", "f02", "b02"), ("C3", "C4", "f03", "b03"),
         ("C4", "C5", "f04", "b04"), ("C1", "I1", "fi1", "bi1"), ("I1", "I2", "f11", "b11"),
         ("C2", "I2", "fi2", "bi2"), ("I2", "I3", "f12", "b12"), ("C3", "I3", "fi3", "bi3"),
         ("I3", "I4", "f13", "b13"), ("C4", "I4", "fi4", "bi4"), ("I4", "I5", "f14", "b14"),
         ("C5", "I5", "fi5", "bi5"), ("C5", "O", "f0O", "b0O"), ("O", "B", "fip", "bip"),
         ("I5", "I6", "f1n", "b1n"), ("O", "I6", "fin", "bin")),  # sodium.py:840-858
        "I6", ("O",), "na", _nav16_rates),
    "Kca2p2_MA2020_GoC": MarkovScheme(
        "Kca2p2_MA2020_GoC",
        (("C1", "C2", "dirc2_t_ca", "invc1_t"), ("C2", "C3", "dirc3_t_ca", "invc2_t"),
         ("C3", "C4", "dirc4_t_ca", "invc3_t"), ("C3", "O1", "diro1_t", "invo1_t"),
         ("C4", "O2", "diro2_t", "invo2_t")),  # potassium_calcium.py:717-724
        "C1", ("O1", "O2"), "k", _kca22_rates),
    "Kca1p1_MA2020_GoC": MarkovScheme(
        "Kca1p1_MA2020_GoC",
        (("C0", "C1", "c01", "c10"), ("C1", "C2", "c12", "c21"), ("C2", "C3", "c23", "c32"),
         ("C3", "C4", "c34", "c43"), ("O0", "O1", "o01", "o10"), ("O1", "O2", "o12", "o21"),
         ("O2", "O3", "o23", "o32"), ("O3", "O4", "o34", "o43"), ("C0", "O0", "f0", "b0"),
         ("C1", "O1", "f1", "b1"), ("C2", "O2", "f2", "b2"), ("C3", "O3", "f3", "b3"),
         ("C4", "O4", "f4", "b4")),  # potassium_calcium.py:1213-1228
        "C0", ("O0", "O1", "O2", "O3", "O4"), "k", _kca11_rates),
    "Nav_MA2020_GrC": MarkovScheme(
        "Nav_MA2020_GrC",
        (("C1", "C2", "f01", "b01"), ("C2", "C3", "f02", "b02"), ("C3", "C4", "f03", "b03"),
         ("C4", "C5", "f04", "b04"), ("C5", "O", "f0O", "b0O"), ("O", "OB", "fip", "bip"),
         ("I1", "I2", "f11", "b11"), ("I2", "I3", "f12", "b12"), ("I3", "I4", "f13", "b13"),
         ("I4", "I5", "f14", "b14"), ("C1", "I1", "fi1", "bi1"), ("C2", "I2", "fi2", "bi2"),
         ("C3", "I3", "fi3", "bi3"), ("C4", "I4", "fi4", "bi4"), ("C5", "I5", "fi5", "bi5"),
         ("O", "I6", "fin", "bin"), ("I5", "I6", "f1n", "b1n")),  # sodium.py:1427-1666 (pairs)
        "I6", ("O",), "na", _navgrc_rates),
}

_T22 = 273.15 + 22.0
# constructor defaults: sodium.py:862-866, potassium_calcium.py:726-735, :1230-1238
MARKOV_DEFAULTS = {
    "Nav1p6_MA2020_GoC": dict(g_max=16.0, temp=_T22),
    # sodium.py:1188-1222 (RI2021_SC inherits it, :1351)
    "Nav1p1_MA2025_BC": dict(g_max=8.0, temp=_T22, Oon=2.3, epsilon=1e-12, gateCurrent=0.0),
    "Nav1p1_RI2021_SC": dict(g_max=8.0, temp=_T22, Oon=2.3, epsilon=1e-12, gateCurrent=0.0),
    "Kca2p2_MA2020_GoC": dict(g_max=38.0, q10_base=3.0, diff=3.0, temp=_T22),
    "Kca1p1_MA2020_GoC": dict(g_max=10.0, q10_base=3.0, temp=_T22),
    "Nav_MA2020_GrC": dict(g_max=13.0, temp=273.15 + 32.0),  # sodium.py:1427 (__init__)
}


def scheme_params(name: str, p: dict) -> dict:
    """Derived parameters: phi = 3^((T - 22 degC) / 10) for Nav1p6 (sodium.py:880);
    q10^((T - 23 degC) / 10) for the Kca channels (``_q10_factor`` at 23 degC,
    potassium_calcium.py:73-74, :755-756, :1267-1268)."""
    out = dict(p)
    if name == "Nav1p6_MA2020_GoC":
        out["phi"] = 3.0 ** ((p["temp"] - _T22) / 10.0)
    elif name == "Nav_MA2020_GrC":  # phi = 3^((T - 20 degC) / 10)
        out["phi"] = 3.0 ** ((p["temp"] - (273.15 + 20.0)) / 10.0)
    elif name.startswith("Nav1p1"):  # sodium.py:1212: phi = 2.7^((T - 22 degC) / 10)
        if p.get("gateCurrent", 0.0) != 0.0:
            raise ValueError("Nav1p1 gating current not restated")
        out["phi"] = 2.7 ** ((p["temp"] - _T22) / 10.0)
    else:
        out["phi"] = p["q10_base"] ** ((p["temp"] - (273.15 + 23.0)) / 10.0)
    return out


# ----------------------------------------------------------------------------- kinetics


def _kinetic(scheme, y, conserve=1.0):
    """Kinetic values of every state: clipped independent states, the dependent one
    from the raw sum.  ``y``: {independent name: array}."""
    s = {k: np.clip(v, 0.0, 1.0) for k, v in y.items()}
    s[scheme.dependent] = conserve - sum(y[k] for k in scheme.independent)
    return s


def derivative(scheme, y, rates, conserve=1.0):
    """dy/dt of the independent states (``compute_derivative``)."""
    s = _kinetic(scheme, y, conserve)
    d = {k: np.zeros_like(np.asarray(s[k], dtype=np.float64)) for k in scheme.states}
    for src, dst, f, b in scheme.pairs:
        fl = rates[f] * s[src]
        d[src] = d[src] - fl
        d[dst] = d[dst] + fl
        if b is not None:
            bl = rates[b] * s[dst]
            d[src] = d[src] + bl
            d[dst] = d[dst] - bl
    return {k: d[k] for k in scheme.independent}


def jacobian(scheme, y, rates):
    """J[..., i, j] = d f_i / d y_j over the independent states."""
    ind = scheme.independent
    n = len(ind)
    shape = np.broadcast(*[np.asarray(v) for v in y.values()]).shape
    J = np.zeros(shape + (n, n))
    inside = {k: ((y[k] >= 0.0) & (y[k] <= 1.0)).astype(np.float64) for k in ind}

    def ds(state):
        """d s[state] / d y_j for every j: a row over the independent states."""
        row = np.zeros(shape + (n,))
        if state == scheme.dependent:
            row[...] = -1.0
        else:
            row[..., ind.index(state)] = inside[state]
        return row

    for src, dst, f, b in scheme.pairs:
        flows = [(rates[f], src, src, dst)]
        if b is not None:
            flows.append((rates[b], dst, dst, src))
        for rate, by, frm, to in flows:  # flow rate * s[by] leaves `frm` for `to`
            g = np.asarray(rate)[..., None] * ds(by)
            if frm != scheme.dependent:
                J[..., ind.index(frm), :] -= g
            if to != scheme.dependent:
                J[..., ind.index(to), :] += g
    return J


def backward_euler(scheme, y, rates, dt, conserve=1.0, substeps=1):
    """``substeps`` linearised backward-Euler steps of dt / substeps."""
    h = dt / substeps
    ind = scheme.independent
    for _ in range(substeps):
        f = derivative(scheme, y, rates, conserve)
        J = jacobian(scheme, y, rates)
        fv = np.stack(np.broadcast_arrays(*[f[k] for k in ind]), axis=-1)
        A = np.eye(len(ind)) - h * J
        dy = np.linalg.solve(A, (h * fv)[..., None])[..., 0]
        y = {k: y[k] + dy[..., i] for i, k in enumerate(ind)}
    return y


def steady_state(scheme, rates, conserve=1.0):
    """Stationary occupancies of every state (``_solve_steady_state_host``)."""
    names = scheme.states
    n = len(names)
    shape = np.broadcast(*[np.asarray(r) for r in rates.values()]).shape
    G = np.zeros(shape + (n, n))
    for src, dst, f, b in scheme.pairs:
        i, j = names.index(src), names.index(dst)
        fr = np.asarray(rates[f])
        G[..., i, i] -= fr
        G[..., j, i] += fr
        if b is not None:
            br = np.asarray(rates[b])
            G[..., i, j] += br
            G[..., j, j] -= br
    dep = names.index(scheme.dependent)
    G[..., dep, :] = 1.0
    rhs = np.zeros(shape + (n,))
    rhs[..., dep] = conserve
    x = np.linalg.solve(G, rhs[..., None])[..., 0]
    x = np.clip(x, 0.0, None)
    x = x * (conserve / x.sum(axis=-1, keepdims=True))
    return {k: x[..., i] for i, k in enumerate(names)}


def open_fraction(scheme, y, conserve=1.0):
    """The conducting occupancy from the raw stored states (``state_values``)."""
    vals = dict(y)
    vals[scheme.dependent] = conserve - sum(y[k] for k in scheme.independent)
    return sum(vals[k] for k in scheme.open_states)

