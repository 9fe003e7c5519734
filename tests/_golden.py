"""Loads tests/golden/golden.json (the reference's own fixtures, extracted
by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

import oracle

_G = None


def golden():
    global _G
    if _G is None:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.json")) as f:
            _G = json.load(f)
    return _G


def crs(entry):
    return oracle.CRS(entry["m"], entry["n"], np.array(entry["off"]), np.array(entry["idx"]),
                      np.array(entry["val"]))


def crs_text(a):
    """crs_matrix_local::save text form: "col:val" per row, 0-based."""
    lines = []
    for r in range(a.m):
        items = []
        for p in range(a.off[r], a.off[r + 1]):
            v = a.val[p]
            items.append("%d:%s" % (a.idx[p], ("%d" % v) if float(v).is_integer() else repr(float(v))))
        lines.append(" ".join(items))
    return lines
