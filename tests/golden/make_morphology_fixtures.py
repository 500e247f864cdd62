"""Writes tests/golden/morphologies.npz: real morphologies for the GPU parity tests.

The reference ships NeuroMorpho-style reconstructions under data/morphology/ of its
repository.  This script reads five of them with this package's SWC reader
(braincell_gb300.swc.read_swc, the reference's branch-extraction rules) and stores
the resulting branch trees -- per branch its parent, attachment points, type and
frustum segments -- so that the tests can rebuild the same Morphology where the
reference's files are not available.  Run from the repository root:

    python tests/golden/make_morphology_fixtures.py /path/to/reference/data/morphology
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from braincell_gb300.swc import read_swc  # noqa: E402

FILES = ("CA1.swc", "bc.swc", "io.swc", "grc.swc", "branched_soma.swc")
TYPES = ("soma", "axon", "basal_dendrite", "apical_dendrite", "dendrite", "custom")


def main(src: str) -> None:
    out = {}
    for f in FILES:
        m = read_swc(os.path.join(src, f))
        key = os.path.splitext(f)[0]
        nb = len(m.branches)
        px = np.zeros(nb)
        cx = np.zeros(nb)
        for e in m.edges:
            px[e.child.index] = e.parent_x
            cx[e.child.index] = e.child_x
        off = np.cumsum([0] + [b.n_segments for b in m.branches])
        out[f"{key}__parent"] = m.parent_index.astype(np.int32)
        out[f"{key}__parent_x"] = px
        out[f"{key}__child_x"] = cx
        out[f"{key}__type"] = np.asarray([TYPES.index(b.type) for b in m.branches], np.int8)
        out[f"{key}__seg_offsets"] = off.astype(np.int64)
        out[f"{key}__lengths"] = np.concatenate([b.lengths for b in m.branches])
        out[f"{key}__r_prox"] = np.concatenate([b.radii_proximal for b in m.branches])
        out[f"{key}__r_dist"] = np.concatenate([b.radii_distal for b in m.branches])
    np.savez_compressed(os.path.join(HERE, "morphologies.npz"), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/data/morphology")
