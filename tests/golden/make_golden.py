"""Generate the golden fixtures in this directory from the reference checkout.

Run on a machine that has the savthe/gpu_determ checkout ($GD_REFERENCE_DIR,
else a directory "reference" beside this repository):

    python tests/golden/make_golden.py

Outputs
-------
true_results_nodes.json
    The reference's golden file true_results.out (written by determ.cu:146-160
    for the 16^3 grid, box [-5,5]^3, R=16.5, 256 identical Maxwellian cells)
    decoded: the printed row index is node*256 + cell, so the 512 rows are
    velocity nodes (0,0,0..7) x cells J*16+K (J,K < 8).  Cell 0 is excluded
    (its collision frequency went through the reference's broken 5x5 solve);
    for cells 1..63 the columns F, DC (nu), IC (gain), CI (Q), ACC per node are
    recorded with their min and max over cells (the gain of nodes 5..7 differs
    across warps in the last printed digit).
ref_tables.json
    For cubic grids 8..24 on box [-5,5]^3: the nonzero count, FP64 sum and
    SHA-256 of the dense weight table a (float32, little-endian, reference
    layout compute_matrix.cu:556-557) computed with the reference's own
    calc_matrix_element (compute_matrix.cu:110-257) compiled for the host.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build as obuild  # noqa: E402
from oracle.pyoracle import Oracle  # noqa: E402


def golden_nodes(ref_dir: str) -> dict:
    rows = []
    with open(os.path.join(ref_dir, "true_results.out")) as fh:
        for line in fh:
            parts = line.split()
            if len(parts) == 9:
                rows.append(parts)
    assert len(rows) == 512, len(rows)
    npx = 256
    nodes = {}
    for r in rows:
        idx = int(r[0])
        node, cell = divmod(idx, npx)
        if cell == 0:
            continue
        vals = [float(x) for x in r[4:9]]
        nodes.setdefault(node, []).append(vals)
    out = {"grid": {"n": 16, "vmin": -5.0, "vmax": 5.0, "R": 16.5, "npx": npx},
           "input": "f = exp(-(u-1.75)^2 - (v-0.25)^2 - w^2) in every cell (determ.cu:101-121)",
           "columns": ["F", "DC", "IC", "CI", "ACC"],
           "excluded": "cell 0 rows: nu corrected by the reference's broken 5x5 solve",
           "nodes": {}}
    for node, vals in sorted(nodes.items()):
        a = np.array(vals)
        out["nodes"][str(node)] = {"cells": int(a.shape[0]),
                                   "min": a.min(axis=0).tolist(),
                                   "max": a.max(axis=0).tolist()}
    return out


def ref_tables() -> dict:
    so = obuild.build_ref()
    if so is None:
        raise SystemExit("reference checkout not found")
    L = C.CDLL(so)
    L.ref_build_dense_a.argtypes = [C.c_int] * 3 + [C.c_float] * 4 + [
        np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")]
    out = {"box": [-5.0, 5.0], "tables": {}}
    for n in (8, 12, 16, 20, 24):
        o = Oracle(n, R=16.5)
        a = np.zeros(o.a_size, np.float32)
        L.ref_build_dense_a(n, n, n, o.du, o.dv, o.dw, o.d3v, a)
        out["tables"][str(n)] = {
            "nonzero": int(np.count_nonzero(a)),
            "size": int(a.size),
            "sum": float(a.astype(np.float64).sum()),
            "sha256": hashlib.sha256(a.astype("<f4").tobytes()).hexdigest(),
        }
        print(n, out["tables"][str(n)])
    return out


def main():
    ref_dir = os.environ.get("GD_REFERENCE_DIR", obuild.REF_DIR_DEFAULT)
    if not os.path.exists(os.path.join(ref_dir, "true_results.out")):
        raise SystemExit(f"reference checkout not found at {ref_dir}: set GD_REFERENCE_DIR")
    with open(os.path.join(HERE, "true_results_nodes.json"), "w") as fh:
        json.dump(golden_nodes(ref_dir), fh, indent=1)
    with open(os.path.join(HERE, "ref_tables.json"), "w") as fh:
        json.dump(ref_tables(), fh, indent=1)


if __name__ == "__main__":
    main()
