"""Known-answer test inputs from the MassiveMDS reference's own fixtures.

Reads, at run time and without copying them, the H3N2 example shipped in the
reference's inst/extdata: the tip locations annotated on one posterior tree
(large.trees), the 372 x 372 antigenic distance matrix (h3_Deff.txt) and the
MDS precision logged for the same state (large.log, column
mds.residual.precision). BEAST logged mdsLikelihood for that state, which the
untruncated MDS log-likelihood must reproduce.
"""
from __future__ import annotations

import os
import re

import numpy as np

EXTDATA = os.path.join(os.environ.get("MDSX_REFERENCE_ROOT", "/root/reference"), "inst", "extdata")
TREE_LINE = 756  # 1-based line of large.trees holding the tree of the logged state


def available() -> bool:
    return all(os.path.exists(os.path.join(EXTDATA, f)) for f in ("large.trees", "large.log", "h3_Deff.txt"))


def load_state():
    """Returns (delta [N,N], locations [N,2], tau, logged mdsLikelihood)."""
    with open(os.path.join(EXTDATA, "large.trees")) as f:
        lines = f.readlines()
    translate = {}
    in_tr = False
    for ln in lines:
        s = ln.strip()
        if s.lower() == "translate":
            in_tr = True
            continue
        if in_tr:
            if s == ";":
                break
            m = re.match(r"(\d+)\s+(.+?)[,;]?$", s)
            if m:
                translate[m.group(1)] = m.group(2).strip("'")
            if s.endswith(";"):
                break
    tree = lines[TREE_LINE - 1]
    state = re.search(r"tree STATE_(\d+)", tree).group(1)
    tips = re.findall(r"[(,](\d+)\[&loc=\{([-+0-9.eE]+),([-+0-9.eE]+)\}\]", tree)
    loc_by_name = {translate[k]: (float(a), float(b)) for k, a, b in tips}

    with open(os.path.join(EXTDATA, "h3_Deff.txt")) as f:
        rows = [ln.rstrip("\n").split("\t") for ln in f if ln.strip()]
    names = [t.strip() for t in rows[0][1:] if t.strip()]
    n = len(names)
    row_index = {r[0].strip(): r for r in rows[1:]}
    delta = np.empty((n, n))
    for i, name in enumerate(names):
        vals = [v for v in row_index[name][1:] if v.strip()]
        delta[i] = [float(v) for v in vals[:n]]
    x = np.array([loc_by_name[name] for name in names])

    with open(os.path.join(EXTDATA, "large.log")) as f:
        body = [ln.rstrip("\n").split("\t") for ln in f if not ln.startswith("#")]
    header = body[0]
    rec = next(r for r in body[1:] if r[0] == state)
    tau = float(rec[header.index("mds.residual.precision")])
    logged = float(rec[header.index("mdsLikelihood")])
    return delta, x, tau, logged
