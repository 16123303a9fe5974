"""Packs the eight Netlib LPs of the reference's PDHG spike set into
tests/golden/netlib_spike.npz, so the GPU parity tests can solve them where
the reference tree is absent.

Runs where the reference tree is present: each file
`spike/pdhg-spike/data/<name>.mps` is read by the reference's own parse_mps()
(src/io/model.hpp:69-218, compiled into oracle/_ref by oracle/Makefile) and
its arrays are stored under `<name>/<field>`. The exact optima come from
the reference's HiGHS runs (docs/research/sweep_results.csv, the `ref` rows),
its recorded PDHG objectives at tolerance 1e-3 from
docs/research/final_battery_2026-08-29.txt:34-41; both are stored beside the
arrays.

Usage: python tests/golden/make_netlib_golden.py
"""
from __future__ import annotations

import csv
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

NAMES = ["afiro", "kb2", "sc50a", "adlittle", "share2b", "sc205", "bandm", "grow22"]
FIELDS = ("ap", "ai", "ax", "cp", "ci", "acx", "c", "cl", "cu", "rmin", "rmax")


def main():
    ref = O.reference_dir()
    if ref is None:
        raise SystemExit("reference tree not found (set IGAOS_REFERENCE_DIR)")
    O.build(ref=True)
    exact = {}
    with open(os.path.join(ref, "docs", "research", "sweep_results.csv")) as f:
        for row in csv.DictReader(f):
            if row["check"] == "ref" and row["instance"] in NAMES:
                exact[row["instance"]] = float(row["objective"])
    recorded = {}
    battery = open(os.path.join(ref, "docs", "research",
                                "final_battery_2026-08-29.txt")).read()
    for name, obj in re.findall(r"^(\w+): near-optimal (\S+) gap", battery, re.M):
        if name in NAMES:
            recorded[name] = float(obj)
    out = {}
    for name in NAMES:
        lp = O.ref_parse_mps(os.path.join(ref, "spike", "pdhg-spike", "data", name + ".mps"))
        for k in FIELDS:
            out[f"{name}/{k}"] = getattr(lp, k)
        out[f"{name}/shape"] = np.array([lp.m, lp.n], np.int64)
        out[f"{name}/obj_const"] = np.array(lp.obj_const)
        out[f"{name}/exact"] = np.array(exact[name])
        out[f"{name}/recorded_pdhg"] = np.array(recorded[name])
        print(f"{name}: m {lp.m} n {lp.n} nnz {lp.nnz} exact {exact[name]} "
              f"recorded {recorded[name]}")
    np.savez_compressed(os.path.join(HERE, "netlib_spike.npz"), **out)


def load(name: str):
    """The packed LP `name` as an oracle LP, with (exact, recorded) optima."""
    z = np.load(os.path.join(HERE, "netlib_spike.npz"))
    m, n = (int(v) for v in z[f"{name}/shape"])
    lp = O.LP(m=m, n=n, obj_const=float(z[f"{name}/obj_const"]),
              **{k: z[f"{name}/{k}"] for k in FIELDS})
    return lp, float(z[f"{name}/exact"]), float(z[f"{name}/recorded_pdhg"])


if __name__ == "__main__":
    main()
