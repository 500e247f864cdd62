"""The large-cell configuration at its real size: cells of 10,000-20,000 compartments
on ~300 branches with CalciumDetailed, CaT_HM1992 and AHP_De1994 dendrites and 500
Poisson current pulses each (``ion/calcium.py:286-505``,
``channel/potassium_calcium.py:78-186``, ``channel/calcium.py:222-372``).

* FP64 kernels against the float64 oracle on one full-size cell;
* FP32 (float-float V and Ci) against the FP64 kernels over the full 4,000 steps.
"""

import numpy as np
import pytest

from braincell_gb300 import workloads as W
from braincell_gb300.runtime import Plan
from oracle.staggered import OracleCell

pytestmark = pytest.mark.gpu

DT = 0.025


@pytest.fixture(scope="module", autouse=True)
def _lib(native_lib, cuda_device):
    return native_lib


def _first_crossing(trace):
    hit = np.nonzero((trace[1:] >= 0.0) & (trace[:-1] < 0.0))[0]
    return int(hit[0]) + 1 if hit.size else trace.size


def test_full_size_cell_f64_matches_oracle():
    d = W.large(indices=[0])[0]
    assert 10000 <= sum(d.ncv) <= 20000 and len(d.parent) == 301 and len(d.pulses) == 500
    n = 1000
    p = Plan(W.descs_to_batch([d]), precision="f64", record_every=1)
    assert p.tile_stats()[0, 4] == 2  # a cell this size runs from its global-memory blob
    p.run(n, DT)
    oc = OracleCell(W.desc_to_cell(d))
    otr, _ = oc.run(DT, n)
    assert np.abs(otr[0, 0] - p.traces()[0]).max() <= 1e-8
    assert np.abs(oc.V[0] - p.state("V")).max() <= 1e-8
    ci = p.state("Ci")
    m = np.isfinite(ci)
    assert m.sum() == sum(d.ncv) - 1  # every dendritic CV has dynamic calcium
    np.testing.assert_allclose(ci[m], oc.Ci[0, oc.cv_mid][m], rtol=1e-9)
    assert oc.Ci[0, oc.cv_mid][m].max() > 1.5 * 5e-5  # the pulses drive calcium entry
    ahp = p.state("AHP_p")
    np.testing.assert_allclose(ahp[m], oc.gates[("AHP_De1994", "p")][0, oc.cv_mid][m], rtol=1e-9, atol=1e-15)


def test_full_size_cells_f32_against_f64_whole_run():
    descs = W.large(indices=range(4))
    out = {}
    for prec in ("f32", "f64"):
        p = Plan(W.descs_to_batch(descs), precision=prec, record_every=1, max_spikes=256)
        p.run(4000, DT)
        out[prec] = (p.traces(), p.spikes(), p.state("V"), p.state("Ci"))
        p.close()
    (t32, s32, v32, c32), (t64, s64, v64, c64) = out["f32"], out["f64"]
    for c in range(len(descs)):
        k = _first_crossing(t64[c])
        assert np.abs(t32[c, :k] - t64[c, :k]).max() <= 1e-3, f"cell {c}"
        assert len(s32[c]) == len(s64[c])
        if len(s64[c]):
            assert np.abs(np.asarray(s32[c]) - np.asarray(s64[c])).max() <= 0.05
    m = np.isfinite(c64)
    np.testing.assert_allclose(c32[m], c64[m], rtol=1e-4)
    if all(len(x) == 0 for x in s64):
        assert np.abs(v32 - v64).max() <= 1e-3
