"""Records the reference's own GPU PDHG (src/pdhg/pdhg.cu:457-1156, cuSPARSE
path, compiled from its sources into oracle/_ref/libref_eval.so) on a GPU,
into tests/golden/ref_gpu_pdhg.json, which the GPU parity tests compare this
engine against.

Needs a CUDA GPU and the reference helpers built (`oracle/Makefile` target
`ref`, from the reference tree or from its staging in oracle/_ref/src).

Cases (each solved at the stated relative-KKT tolerance, time limit given):
  seeded golden LPs of lp_objectives.json that converge   1e-8, 60 s
  the small random LP shape (m 2000, n 5000), seed 0       1e-4 and 1e-8, 120 s
  the eight Netlib LPs of netlib_spike.npz                 1e-3 (16 s, the
      reference's own battery setting) and 1e-8 (30 s)

Usage: python tests/golden/make_ref_gpu_golden.py [--quick]
"""
from __future__ import annotations

import json
import os
import platform
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from igaos_gb300 import generators as G  # noqa: E402
from oracle import oracle as O  # noqa: E402

import make_golden as MG  # noqa: E402
import make_netlib_golden as MN  # noqa: E402


def cases(quick=False):
    gold = json.load(open(os.path.join(HERE, "lp_objectives.json")))
    for name in sorted(gold):
        if name.startswith("zipf"):
            continue
        e = gold[name]
        yield name, lambda e=e: O.lp_from(MG.make_lp(e["generator"], e["kwargs"])), [(1e-8, 60.0)]
    if not quick:
        yield "c1-s0", lambda: O.lp_from(G.config1(seed=0)), [(1e-4, 120.0), (1e-8, 120.0)]
    for name in MN.NAMES:
        yield ("netlib-" + name, lambda name=name: MN.load(name)[0],
               [(1e-3, 16.0), (1e-8, 30.0 if not quick else 5.0)])


def main():
    quick = "--quick" in sys.argv
    O.build(ref=True)
    if not O.ref_pdhg_available():
        raise SystemExit("reference GPU PDHG not built (oracle/_ref/libref_eval.so)")
    out = {"_about": {
        "what": "reference GPU PDHG (cuSPARSE path) compiled from its sources",
        "host": platform.machine(), "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}}
    try:
        import torch
        out["_about"]["gpu"] = torch.cuda.get_device_name(0)
    except Exception:
        pass
    dst = os.environ.get("REF_GPU_GOLDEN_OUT", os.path.join(HERE, "ref_gpu_pdhg.json"))
    for name, make, runs in cases(quick):
        lp = make()
        for tol, tl in runs:
            r = O.ref_pdhg_solve(lp, tolerance=tol, time_limit=tl)
            key = f"{name}@{tol:g}"
            out[key] = {k: r[k] for k in ("status_name", "objective", "pinf", "dinf", "gap",
                                          "iterations", "loop_ms", "wall_ms", "message")}
            out[key].update(m=lp.m, n=lp.n, nnz=lp.nnz, tolerance=tol, time_limit=tl)
            print(f"{key:28s} {r['status_name']:16s} obj {r['objective']:.12g} "
                  f"it {r['iterations']:7d} wall {r['wall_ms']:9.1f} ms  {r['message']}",
                  flush=True)
            with open(dst, "w") as f:  # after every case: a cut-off run keeps what it has
                json.dump(out, f, indent=1, sort_keys=True)
    print("wrote", dst)


if __name__ == "__main__":
    main()
