"""Readers for the data the reference's users feed the MDS engine.

* Named distance tables (the reference's ``inst/extdata/h3_Deff.txt`` format):
  a tab-separated header row of location names, then one row per location,
  its name followed by N distances. Empty cells and ``NA`` are missing pairs
  (NaN), which the engine masks.
* Latent locations annotated on a BEAST NEXUS tree (``large.trees``): a
  ``translate`` block mapping tip numbers to names, and trees whose tips carry
  ``[&loc={a,b,...}]`` annotations (any embedding dimension).
* Columns of a BEAST log (``large.log``): tab-separated, ``#`` comments, a
  header row, one row per state.

The reference does this in R (``R/Untitled.R:310-374``, ``readbeast`` and
``getdata``, with the ``ape`` tree reader). These readers are a plain-Python
restatement of the parts an engine user needs: a distance matrix in the
engine's row-major layout, and the locations of one logged state in the same
row order.
"""
from __future__ import annotations

import re

import numpy as np

_LOC = re.compile(r"[(,](\d+)\[&[^\]]*?loc=\{([^}]*)\}[^\]]*\]")


def read_distance_table(path: str) -> tuple[list[str], np.ndarray]:
    """(names, delta [N, N] float64) from a named tab-separated distance table;
    rows are returned in the header's order; empty or NA cells are NaN."""
    with open(path) as f:
        rows = [ln.rstrip("\n").split("\t") for ln in f if ln.strip()]
    names = [t.strip() for t in rows[0][1:] if t.strip()]
    n = len(names)
    by_name = {r[0].strip(): r[1:] for r in rows[1:]}
    delta = np.full((n, n), np.nan)
    for i, name in enumerate(names):
        cells = by_name[name]
        # keep positional cells; a trailing tab may add an empty last cell
        cells = cells[:n] if len(cells) >= n else cells + [""] * (n - len(cells))
        for j, v in enumerate(cells):
            v = v.strip()
            if v and v.upper() != "NA":
                delta[i, j] = float(v)
    return names, delta


def read_nexus_translate(path: str) -> dict[str, str]:
    """The ``translate`` block of a NEXUS trees file: tip number -> name."""
    table: dict[str, str] = {}
    inside = False
    with open(path) as f:
        for ln in f:
            s = ln.strip()
            if s.lower() == "translate":
                inside = True
                continue
            if inside:
                m = re.match(r"(\d+)\s+(.+?)[,;]?$", s)
                if m:
                    table[m.group(1)] = m.group(2).strip("'\"")
                if s.endswith(";"):
                    break
    return table


def read_nexus_locations(path: str, state: int | None = None, line: int | None = None
                         ) -> tuple[int, dict[str, np.ndarray]]:
    """(state, {name: location}) from the tree of BEAST state ``state``, or from
    the tree on 1-based ``line``; without either, the last tree."""
    translate = read_nexus_translate(path)
    chosen = None
    with open(path) as f:
        for k, ln in enumerate(f, start=1):
            m = re.match(r"\s*tree\s+STATE_(\d+)", ln)
            if not m:
                continue
            if line is not None and k == line:
                chosen = (int(m.group(1)), ln)
                break
            if state is not None and int(m.group(1)) == state:
                chosen = (int(m.group(1)), ln)
                break
            if line is None and state is None:
                chosen = (int(m.group(1)), ln)
    if chosen is None:
        raise ValueError("no matching tree in " + path)
    st, tree = chosen
    locs = {}
    for tip, coords in _LOC.findall(tree):
        locs[translate.get(tip, tip)] = np.array([float(c) for c in coords.split(",")])
    return st, locs


def read_beast_log(path: str, columns: list[str], state: int) -> dict[str, float]:
    """Values of ``columns`` at ``state`` from a BEAST log."""
    with open(path) as f:
        body = [ln.rstrip("\n").split("\t") for ln in f if ln.strip() and not ln.startswith("#")]
    header = body[0]
    rec = next(r for r in body[1:] if int(float(r[0])) == state)
    return {c: float(rec[header.index(c)]) for c in columns}


def locations_in_order(names: list[str], locs: dict[str, np.ndarray]) -> np.ndarray:
    """Locations [N, P] in the row order of a distance table."""
    missing = [n for n in names if n not in locs]
    if missing:
        raise KeyError(f"{len(missing)} table names have no location, e.g. {missing[0]!r}")
    return np.stack([locs[n] for n in names])
