"""Known-answer test inputs from the MassiveMDS reference's own fixtures.

Reads, at run time and without copying them, with the library's readers
(massivemds_gb300/formats.py), the H3N2 example shipped in the reference's
inst/extdata: the tip locations annotated on one posterior tree
(large.trees), the 372 x 372 antigenic distance matrix (h3_Deff.txt) and the
MDS precision logged for the same state (large.log, column
mds.residual.precision). BEAST logged mdsLikelihood for that state, which the
untruncated MDS log-likelihood must reproduce.
"""
from __future__ import annotations

import os

from massivemds_gb300 import formats
from oracle import reference_root

_ROOT = reference_root()
EXTDATA = os.path.join(_ROOT, "inst", "extdata") if _ROOT else ""
TREE_LINE = 756  # 1-based line of large.trees holding the tree of the logged state


def available() -> bool:
    return bool(EXTDATA) and all(os.path.exists(os.path.join(EXTDATA, f)) for f in ("large.trees", "large.log", "h3_Deff.txt"))


def load_state():
    """Returns (delta [N,N], locations [N,2], tau, logged mdsLikelihood)."""
    names, delta = formats.read_distance_table(os.path.join(EXTDATA, "h3_Deff.txt"))
    state, locs = formats.read_nexus_locations(os.path.join(EXTDATA, "large.trees"), line=TREE_LINE)
    x = formats.locations_in_order(names, locs)
    log = formats.read_beast_log(os.path.join(EXTDATA, "large.log"), ["mds.residual.precision", "mdsLikelihood"],
                                 state)
    return delta, x, log["mds.residual.precision"], log["mdsLikelihood"]
