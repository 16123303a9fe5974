"""Benchmark of the GB300 PDHG LP engine on the large sparse LP shape.

Workload (one step): the large sparse LP (m=200,000 rows, half equality half
<=, n=500,000 box-bounded columns, ~5.2M nonzeros with Zipf(1.5) column
degrees and |A_ij| log-uniform in [1e-3, 1e3]; seeded synthetic data), one
solve call of ITERS accepted PDHG iterations in FP64 -- the reference's
arithmetic (FP64 attempts, FP64 KKT checks every 64 iterations, restarts,
primal weight) -- from a cold start on device-resident data.

value: SpMV GB/s of the FP64 attempts -- algorithmic bytes of every fused
A^T y / A xbar attempt of the solve divided by the solve's CUDA-event device
time (checks, restarts and host round trips included). Algorithmic bytes per
attempt (s = 8 for FP64, 4 for FP32; int32 indices):
    2*nnz*(s+4) + 4*(m+n+2) + s*9*(m+n)
(each matrix entry and index once per orientation, row/column pointers once,
nine m- and nine n-vectors read or written once each: x, xavg, c, l, u, xbar
and y, A x, yavg, rmin, rmax gathered/read; x', xavg', xbar, y', A x', yavg'
written). The reference arm and cpu_baseline measure the same FP64 metric
(the CPU oracle of the reference FP64 PDHG on the host cores), so the ratio
of the two lines is at equal arithmetic.
roofline: the FP64 attempt's algorithmic bytes over its CUDA-event time
against the measured HBM copy bandwidth, with ncu DRAM traffic per attempt
from the committed summary. `fp32_refine`: the same solve with FP32 attempts
and FP64 refinement (GB/s, attempt time, its rooflines: HBM and L2's
random-sector rate).
e2e: the same metric through the C ABI with HOST buffers: igaos_pdhg_solve_csr
(upload, device setup, solve, download, free) timed on the host.
L2: flushed (512 MiB write) between steps.

Time-to-tolerance keys (relative KKT of the original LP, FP64 metrics):
`time_to_tol_small_lp` (m 2,000, n 5,000): FP32 + refinement and FP64 to 1e-4
and 1e-8 and the CPU oracle at 1e-8. `time_to_tol_multicommodity_lp` (m
1,078,800, n 2,870,400): both precisions to 1e-4 and 1e-8, with attempt_us /
attempt_hbm_frac (this LP streams from HBM) and the distance of the 1e-8
objectives to scipy-HiGHS's optimum (tests/golden/mcf_objectives.json).
`time_to_tol_large_lp`: this workload to 1e-4 (FP32 + refinement with the
opt-in Pock-Chambolle scaling; FP64 with the reference's scaling and with
it), each within a stated budget, with the KKT reached. `vs_reference_gpu`:
the reference's own GPU PDHG (cuSPARSE path, compiled from its sources into
oracle/_ref, timed on this GPU in this process) beside this engine -- to
1e-4 and 1e-8 on the small LP, and over a fixed 4,992-iteration budget on
the two large LPs (above 46,340 rows its dense dual repair, reached from
iteration 5,000, overflows int32 indices). Also `batched_small_lps` (4,096
uneven LPs to 1e-6 in one persistent launch vs sequential solves) and
`differentiable_layer`. The speed measures (headline, e2e, the per-iteration
comparison on the large LPs) run the `--schedule` warp schedule (default:
autotuned per problem and precision, the tuning timed with the solve where
a fresh problem is created). Time to tolerance runs the fixed schedule: the
autotuner's choice depends on timing noise and changes the rounding of the
products and of the step decision's dot products, and PDHG's trajectory
with it (multicommodity LP in FP64 to 1e-8: 83,776 iterations on the fixed
schedule, 140,800 on one tuned choice), so only the fixed schedule gives
iteration counts that repeat from run to run.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-1e-8 rel KKT & SpMV GB/s: FP32+refine vs FP64 PDHG; batched LPs/sec"


def bytes_per_attempt(m, n, nnz, s):
    return 2 * nnz * (s + 4) + 4 * (m + n + 2) + s * 9 * (m + n)


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(key):
    """Per-launch DRAM bytes of the fused attempt from the committed ncu
    summary (profiles/roofline_traffic.txt: `key bytes` lines), if any."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    try:
        for line in open(path):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == key:
                return float(parts[1])
    except OSError:
        pass
    return None


class Clocks:
    """nvidia-smi samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows if len(r) > 8 for i in range(4)
                          if r[5 + i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value, ws):
    if ws == 1:
        return value
    import torch
    import torch.distributed as td
    t = torch.tensor([value], dtype=torch.float64,
                     device="cuda" if td.get_backend() == "nccl" else "cpu")
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as td
        td.barrier()


def cpu_sample(lp, iters, threads):
    """The oracle of the reference FP64 PDHG on the host cores: GB/s of its
    SpMVs (FP64 values) over a bounded number of iterations."""
    from oracle import oracle as O
    olp = O.lp_from(lp)
    r = O.pdhg_solve(olp, tolerance=1e-12, time_limit=1e9, max_iterations=iters, threads=threads)
    b = bytes_per_attempt(lp.m, lp.n, lp.nnz, 8) * r["attempts"]
    return b / r["loop_seconds"] / 1e9, r


def run_reference(args, lp, ws, rank):
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(args.warmup and 1):
        cpu_sample(lp, 8, threads)
    vals = []
    sample = None
    for _ in range(args.steps):
        v, r = cpu_sample(lp, args.cpu_iters, threads)
        vals.append(v)
        sample = r
    value = statistics.mean(vals)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "GB/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sample["loop_seconds"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config_dict(lp, args),
        "cpu_baseline": {"value": value, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{args.cpu_iters} iterations of the reference FP64 PDHG "
                                   f"(CPU oracle, OpenMP) on the same LP, per step"},
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    print(json.dumps(line), flush=True)


def batch_probe(capi, G, sample=24, count=4096, warm=True):
    """The batch of 4,096 uneven LPs (m log-uniform in [20, 2000], n = 2.5 m,
    1% density, box [0,5]; seed 0) solved to 1e-6 relative KKT in one
    persistent launch, against sequential single-LP solves (FP64 engine, one
    C-ABI call each with host buffers) of a seeded random sample of it
    (`sample` = 0 skips them; `warm` = False makes the timed launch the
    first one, for profiling)."""
    lps = G.config3(seed=0, count=count)
    if warm:
        capi.solve_batch(lps[:64], tolerance=1e-6, max_iterations=200000, want_solutions=False)
    t0 = time.perf_counter()
    out = capi.solve_batch(lps, tolerance=1e-6, max_iterations=200000, want_solutions=False)
    wall = time.perf_counter() - t0
    st = {}
    for r in out:
        st[r["status_name"]] = st.get(r["status_name"], 0) + 1
    kms = out[0]["kernel_time_ms"]
    res = {
        "workload": f"{count} uneven LPs (m 20..2000 log-uniform, n=2.5m, 1% density, box [0,5], "
                    f"seed 0, sum nnz {sum(lp.nnz for lp in lps)}), tol 1e-6",
        "status": st, "kernel_ms": kms, "call_s": wall,
        "lps_per_s": len(lps) / wall, "lps_per_s_kernel": len(lps) / (kms / 1e3),
        "iterations_median": float(np.median([r["iterations"] for r in out])),
        "iterations_p99_max": [float(np.percentile([r["iterations"] for r in out], 99)),
                               float(max(r["iterations"] for r in out))],
        "instances_over": {str(k): int(sum(r["iterations"] > k for r in out))
                           for k in (20000, 50000, 100000)},
        "finished_fp64": int(sum(r.get("finished_fp64", 0) for r in out)),
        "instance_ms_max": float(max(r["instance_time_ms"] for r in out)),
    }
    if sample > 0:
        idx = np.random.default_rng(0).choice(len(lps), min(sample, len(lps)), replace=False)
        capi.solve_lp(lps[idx[0]], tolerance=1e-6, time_limit=60.0, precision="fp64")
        seq = []
        for i in idx:
            t1 = time.perf_counter()
            capi.solve_lp(lps[i], tolerance=1e-6, time_limit=60.0, precision="fp64")
            seq.append(time.perf_counter() - t1)
        res.update({"sequential_sample": len(idx), "sequential_s_per_lp": statistics.mean(seq),
                    "sequential_lps_per_s": 1.0 / statistics.mean(seq),
                    "speedup_vs_sequential": (len(lps) / wall) * statistics.mean(seq)})
    return res


def layer_probe(torch, G, reps=3):
    """The differentiable layer on 256 ridge-regularised LPs (m=500, n=1000,
    2% density, box [0,10], ridge 0.005; seed 0): FP32 forward through 1,000
    PDHG iterations and the adjoint backward (checkpoints every 50),
    CUDA-event time on the current stream."""
    from igaos_gb300.layer import BatchPattern, UnrolledPDHG, pdhg_steps, stack_lps
    lps = G.config4(seed=0, count=256)
    P = BatchPattern.from_lps(lps, "cuda")
    data = [t.clone().requires_grad_(True) for t in stack_lps(lps, torch.float32, "cuda")]
    tau, sigma = pdhg_steps(P, data[5].detach())
    fw, bw = [], []
    for rep in range(reps + 2):
        for t in data:
            t.grad = None
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record()
        x, y, obj = UnrolledPDHG.apply(*data, tau, sigma, P, 1000, 50, 0.005)
        e[1].record()
        (obj.sum() + x.sum()).backward()
        e[2].record()
        torch.cuda.synchronize()
        if rep >= 2:
            fw.append(e[0].elapsed_time(e[1]))
            bw.append(e[1].elapsed_time(e[2]))
    f, b = statistics.median(fw), statistics.median(bw)
    return {"workload": "256 ridge LPs m=500 n=1000 2% density, K=1000, checkpoints every 50, "
                        "FP32", "forward_ms": f, "backward_ms": b,
            "lp_gradients_per_s": 256 / ((f + b) / 1e3)}


def config_dict(lp, args):
    return {"workload": "large sparse LP (m=200k, n=500k, ~5.2M nnz, Zipf(1.5) column "
                        "degrees, |A_ij| log-uniform [1e-3,1e3], box [0,10]); one solve of "
                        f"{args.iters} PDHG iterations per step",
            "m": lp.m, "n": lp.n, "nnz": lp.nnz, "precision": args.precision,
            "schedule": args.schedule,
            "iters_per_step": args.iters, "l2": "flushed between steps (512 MiB write)",
            "parallelism": f"replicas x{args.gpus}"}


def tol_entry(r, wall_s=None):
    """Time-to-tolerance record of one engine solve (device-resident data:
    `loop_s` is the solve loop's wall time, setup excluded; `wall_s`, when
    given, a whole C-ABI call with host buffers)."""
    d = {"status": r["status_name"], "loop_s": r["solve_time_ms"] / 1e3,
         "device_s": r["device_time_ms"] / 1e3, "iterations": r["iterations"],
         "objective": r["objective"], "pinf": r["pinf"], "dinf": r["dinf"],
         "rel_gap": r["rel_gap"], "prow": r["prow"]}
    if wall_s is not None:
        d["wall_s"] = wall_s
    return d


def ref_gpu(lp, tol, time_limit, max_iterations=500000):
    """The reference's own GPU PDHG (oracle/_ref, compiled from its sources)
    on `lp`: loop_s is its own loop timer (setup excluded), wall_s the whole
    call (handles, Ruiz, upload, power iteration, loop, download)."""
    from oracle import oracle as O
    r = O.ref_pdhg_solve(O.lp_from(lp), tolerance=tol, time_limit=time_limit,
                         max_iterations=max_iterations)
    return {"status": r["status_name"], "loop_s": r["loop_ms"] / 1e3, "wall_s": r["wall_ms"] / 1e3,
            "iterations": r["iterations"], "objective": r["objective"], "pinf": r["pinf"],
            "dinf": r["dinf"], "rel_gap": r["gap"], "message": r["message"]}


def ref_gpu_ready():
    try:
        from oracle import oracle as O
        return O.ref_pdhg_available()
    except Exception:
        return False


def rel_diff(a, b):
    return abs(a - b) / max(1.0, abs(b))


def small_lp_probe(capi, G, local, sched):
    """Small random LP (m 2,000, n 5,000, seed 0): FP32 + refinement and FP64
    to 1e-4 and 1e-8 (device-resident), and the CPU oracle at 1e-8."""
    slp = G.config1(seed=0)
    out = {"workload": f"small random LP m={slp.m} n={slp.n} nnz={slp.nnz} (seed 0)"}
    x_last = None
    with capi.Problem(slp, device=local) as P:
        for prec in ("fp64", "fp32-refine"):
            P.solve(precision=prec, tolerance=1e-6, time_limit=60.0, schedule=sched)  # warm
            for tol in (1e-4, 1e-8):
                r = P.solve(precision=prec, tolerance=tol, time_limit=60.0, schedule=sched)
                out[f"{prec}@{tol:g}"] = tol_entry(r)
                if prec == "fp32-refine" and tol == 1e-8:
                    x_last = r["x"]
    for tol in (1e-4, 1e-8):
        a, b = out[f"fp64@{tol:g}"], out[f"fp32-refine@{tol:g}"]
        if a["status"] == b["status"] == "near-optimal":
            out[f"speedup_fp32_refine_vs_fp64@{tol:g}"] = a["loop_s"] / b["loop_s"]
    try:  # host crossover from the FP32 + refinement answer (a probe)
        t0 = time.perf_counter()
        xv, _, _, xi = capi.crossover(slp, x_last)
        out["crossover_from_fp32_refine"] = {
            "status": xi["status"], "s": time.perf_counter() - t0, "pivots": xi["pivots"],
            "objective": float(slp.c @ xv + slp.obj_const)}
    except Exception as e:
        out["crossover_from_fp32_refine"] = {"error": str(e)[:200]}
    from oracle import oracle as O
    rr = O.pdhg_solve(O.lp_from(slp), tolerance=1e-8, time_limit=120.0,
                      threads=os.cpu_count() or 1)
    out["cpu_oracle_fp64@1e-8"] = {"status": rr["status_name"], "s": rr["seconds"],
                                   "iterations": rr["iterations"], "cores": os.cpu_count()}
    return slp, out


def c5_probe(capi, G, local, sched):
    """Multicommodity LP: both precisions to 1e-4 and 1e-8 (device-resident),
    with the attempt time against the HBM roofline (this LP's working set
    exceeds L2, so its attempts stream from HBM)."""
    flp = G.config5(seed=0)
    out = {"workload": f"multicommodity flow m={flp.m} n={flp.n} nnz={flp.nnz} (seed 0)"}
    pk, pk_kind = peaks()
    with capi.Problem(flp, device=local) as P:
        for prec in ("fp32-refine", "fp64"):
            cb = bytes_per_attempt(flp.m, flp.n, flp.nnz, 8 if prec == "fp64" else 4)
            for tol in (1e-4, 1e-8):
                r = P.solve(precision=prec, tolerance=tol, time_limit=240.0, schedule=sched)
                e = tol_entry(r)
                us = 1e3 * r["attempt_time_ms"] / max(1, r["attempts"])
                e.update(attempt_us=us, attempt_bytes=cb,
                         attempt_hbm_frac=cb / (us * 1e-6) / 1e9 / pk, hbm_peak_kind=pk_kind)
                out[f"{prec}@{tol:g}"] = e
    for tol in (1e-4, 1e-8):
        a, b = out[f"fp64@{tol:g}"], out[f"fp32-refine@{tol:g}"]
        if a["status"] == b["status"] == "near-optimal":
            out[f"speedup_fp32_refine_vs_fp64@{tol:g}"] = a["loop_s"] / b["loop_s"]
            out[f"objective_rel_diff@{tol:g}"] = rel_diff(b["objective"], a["objective"])
    # the independent optimum (scipy HiGHS interior point, committed fixture)
    try:
        gold = json.load(open(os.path.join(ROOT, "tests", "golden", "mcf_objectives.json")))
        ref = gold["mcf300x8-s0"]["highs_ipm_objective"]
        out["highs_ipm_objective"] = ref
        for k in ("fp32-refine@1e-08", "fp64@1e-08"):
            out[f"{k}_rel_diff_vs_highs"] = rel_diff(out[k]["objective"], ref)
    except (OSError, KeyError, ValueError):
        pass
    return flp, out


def c2_tol_probe(capi, lp, local, budget32, budget64, sched):
    """The large LP to 1e-4: FP32 + refinement with the opt-in Pock-Chambolle
    scaling; FP64 with it and with the reference's Ruiz scaling alone; each
    within its budget (seconds), reporting the KKT reached when it runs out."""
    out = {"tolerance": 1e-4, "budget_s": {"fp32-refine": budget32, "fp64": budget64}}
    with capi.Problem(lp, device=local, scaling="ruiz-pc") as P:
        out["fp32-refine+pc"] = tol_entry(P.solve(precision="fp32-refine", tolerance=1e-4,
                                                  time_limit=budget32, schedule=sched))
        out["fp64+pc"] = tol_entry(P.solve(precision="fp64", tolerance=1e-4, time_limit=budget64,
                                           schedule=sched))
    with capi.Problem(lp, device=local) as P:
        out["fp64"] = tol_entry(P.solve(precision="fp64", tolerance=1e-4, time_limit=budget64,
                                        schedule=sched))
    return out


def vs_reference_gpu(capi, local, slp, flp, lp, sched):
    """The reference's GPU PDHG beside this engine on the same GPU. Small LP:
    both to 1e-4 and 1e-8 (loop time and whole-call wall time). Large LPs: a
    fixed budget of 4,992 iterations (seconds per iteration, KKT reached)."""
    out = {"engine": "reference src/pdhg/pdhg.cu (cuSPARSE/cuBLAS FP64), compiled from its "
                     "sources, same GPU, same process"}
    small = {}
    for tol in (1e-4, 1e-8):
        ref = ref_gpu(slp, tol, 120.0)
        row = {"reference": ref}
        for prec in ("fp64", "fp32-refine"):
            t0 = time.perf_counter()
            r = capi.solve_lp(slp, precision=prec, tolerance=tol, time_limit=120.0, device=local,
                              schedule="fixed")  # a time to tolerance: fixed schedule
            row[prec] = tol_entry(r, wall_s=time.perf_counter() - t0)
            if ref["status"] == r["status_name"] == "near-optimal":
                row[prec]["speedup_loop"] = ref["loop_s"] / row[prec]["loop_s"]
                row[prec]["speedup_wall"] = ref["wall_s"] / row[prec]["wall_s"]
                row[prec]["objective_rel_diff"] = rel_diff(r["objective"], ref["objective"])
        small[f"s_to_{tol:g}"] = row
    out["small_lp"] = small
    for key, big in (("multicommodity_lp", flp), ("large_lp", lp)):
        if big is None:
            continue
        ref = ref_gpu(big, 1e-12, 1e9, max_iterations=4992)
        row = {"iterations": 4992, "reference": ref,
               "reference_s_per_iteration": ref["loop_s"] / max(1, ref["iterations"])}
        with capi.Problem(big, device=local) as P:
            for prec in ("fp64", "fp32-refine"):
                r = P.solve(precision=prec, tolerance=1e-12, time_limit=1e9, max_iterations=4992,
                            schedule=sched)
                e = tol_entry(r)
                e["s_per_iteration"] = e["loop_s"] / max(1, r["iterations"])
                e["speedup_per_iteration"] = row["reference_s_per_iteration"] / e["s_per_iteration"]
                row[prec] = e
        out[key] = row
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--iters", type=int, default=2048)
    ap.add_argument("--precision", default="fp64", choices=["fp32", "fp64", "fp32-refine"],
                    help="arithmetic of the headline steps (fp64: the reference's)")
    ap.add_argument("--no-small", action="store_true",
                    help="skip the time-to-tolerance comparison on the small LP")
    ap.add_argument("--cpu-iters", type=int, default=64)
    ap.add_argument("--scale", type=float, default=1.0, help="shrink the LP (testing only)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline sample")
    ap.add_argument("--probe", choices=["batch", "layer", "attempts-c5"], default=None,
                    help="run only that extra workload and print its JSON (profiling); "
                         "attempts-c5: --iters iterations of the multicommodity LP at "
                         "--precision, after one warming solve of the same length")
    ap.add_argument("--batch-count", type=int, default=4096,
                    help="LPs in the batched workload (smaller for profiling)")
    ap.add_argument("--batch-sample", type=int, default=24,
                    help="sequential single-LP solves timed beside the batch (0: none)")
    ap.add_argument("--no-c5", action="store_true", help="skip the multicommodity LP")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-LP comparison")
    ap.add_argument("--no-layer", action="store_true", help="skip the differentiable layer")
    ap.add_argument("--no-c2-tol", action="store_true", help="skip the large LP to 1e-4")
    ap.add_argument("--no-ref-gpu", action="store_true",
                    help="skip the reference GPU PDHG comparison")
    ap.add_argument("--schedule", default="autotune", choices=["fixed", "autotune"],
                    help="warp schedule of the headline steps and the attempts-c5 probe "
                         "(autotune: timed once per handle and precision, in the warm-up)")
    ap.add_argument("--c2-budget", type=float, default=100.0,
                    help="seconds for the FP32 + refinement solve of the large LP to 1e-4 "
                         "(FP64 gets 0.6 of it)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, local = dist()
    from igaos_gb300 import generators as G
    s = args.scale
    lp = G.config2(seed=0, m=int(200_000 * s), n=int(500_000 * s), target_nnz=int(5_000_000 * s))
    if args.impl == "reference":
        if ws > 1:
            import torch.distributed as td
            td.init_process_group("gloo")
        run_reference(args, lp, ws, rank)
        return

    import torch
    if ws > 1:
        import torch.distributed as td
        td.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from igaos_gb300 import capi
    if args.probe == "attempts-c5":  # fixed-length solves of the multicommodity LP
        flp = G.config5(seed=0)
        cb = bytes_per_attempt(flp.m, flp.n, flp.nnz, 8 if args.precision == "fp64" else 4)
        with capi.Problem(flp, device=local) as P:
            o = dict(precision=args.precision, tolerance=1e-12, time_limit=1e9,
                     max_iterations=args.iters, schedule=args.schedule)
            P.solve(**o)
            r = P.solve(**o)
        us = 1e3 * r["attempt_time_ms"] / max(1, r["attempts"])
        pk, pk_kind = peaks()
        print(json.dumps({"workload": f"multicommodity flow m={flp.m} n={flp.n} nnz={flp.nnz}",
                          "precision": args.precision, "iterations": r["iterations"],
                          "attempts": r["attempts"], "attempt_us": us, "attempt_bytes": cb,
                          "entries_per_lane": [r["entries_a"], r["entries_at"]],
                          "attempt_hbm_frac": cb / (us * 1e-6) / 1e9 / pk,
                          "hbm_peak_kind": pk_kind}), flush=True)
        return
    if args.probe:  # one extra workload alone (profiling runs)
        res = batch_probe(capi, G, sample=args.batch_sample, count=args.batch_count,
                          warm=False) if args.probe == "batch" else layer_probe(torch, G)
        print(json.dumps(res), flush=True)
        return
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def steps(P, prec, count, timed):
        o = dict(precision=prec, tolerance=1e-12, time_limit=1e9, max_iterations=args.iters,
                 device=local, schedule=args.schedule)
        res = []
        for _ in range(count):
            if timed:
                flush.fill_(1)
                torch.cuda.synchronize()
            res.append(P.solve(**o))
        return res

    alt = "fp32-refine" if args.precision == "fp64" else "fp64"
    with capi.Problem(lp, device=local) as P:
        steps(P, args.precision, args.warmup, False)
        clocks = Clocks(local)
        barrier(ws)
        torch.cuda.synchronize()
        res = steps(P, args.precision, args.steps, True)
        torch.cuda.synchronize()
        barrier(ws)
        ck = clocks.stop()
        # the same steps in the other arithmetic (not part of `value`)
        steps(P, alt, 1, False)
        res_alt = steps(P, alt, min(3, args.steps), True)
    s_main = 8 if args.precision == "fp64" else 4
    bpa = bytes_per_attempt(lp.m, lp.n, lp.nnz, s_main)
    bpa_alt = bytes_per_attempt(lp.m, lp.n, lp.nnz, 8 if alt == "fp64" else 4)
    dev_ms = sum(r["device_time_ms"] for r in res)
    att = sum(r["attempts"] for r in res)
    att_ms = sum(r["attempt_time_ms"] for r in res)
    launches = sum(r["launches"] for r in res)
    dev_ms_max = barrier_max(dev_ms, ws)
    value = ws * bpa * att / (dev_ms_max / 1e3) / 1e9
    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        opts = dict(precision=args.precision, tolerance=1e-12, time_limit=1e9,
                    max_iterations=args.iters, device=local, schedule=args.schedule)
        h2d = sum(np.asarray(a).nbytes for a in (lp.ap, lp.ai, lp.ax, lp.cp, lp.ci, lp.acx, lp.c,
                                                   lp.cl, lp.cu, lp.rmin, lp.rmax))
        d2h = 8 * (lp.m + lp.n)
        e_steps = min(args.steps, 3)
        capi.solve_lp(lp, **opts)
        barrier(ws)
        t0 = time.perf_counter()
        e_att = 0
        setup_ms = solve_ms = 0.0
        for _ in range(e_steps):
            r = capi.solve_lp(lp, **opts)
            e_att += r["attempts"]
            setup_ms += r["setup_time_ms"]
            solve_ms += r["solve_time_ms"]
        torch.cuda.synchronize()
        el = barrier_max(time.perf_counter() - t0, ws)
        # where a step's wall time goes: upload + device setup (ordering,
        # scaling, power iteration), the solve (autotuning included when
        # selected), the rest (host validation, download, teardown)
        e2e = {"value": ws * bpa * e_att / el / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * el / e_steps,
               "setup_ms": setup_ms / e_steps, "solve_ms": solve_ms / e_steps,
               "schedule": args.schedule}
    slp = small = flp = c5 = c2tol = refg = None
    if rank == 0 and not args.no_small:
        slp, small = small_lp_probe(capi, G, local, "fixed")
    if rank == 0 and not args.no_c5:
        flp, c5 = c5_probe(capi, G, local, "fixed")
    if rank == 0 and not args.no_c2_tol:
        c2tol = c2_tol_probe(capi, lp, local, args.c2_budget, 0.6 * args.c2_budget, "fixed")
    if rank == 0 and not args.no_ref_gpu:
        if ref_gpu_ready():
            slp = slp or G.config1(seed=0)
            refg = vs_reference_gpu(capi, local, slp, flp, lp if s == 1.0 else None, args.schedule)
        else:
            refg = {"unavailable": "reference GPU PDHG not built here (oracle/_ref needs the "
                                   "reference sources or their staging in oracle/_ref/src)"}
    batch = None
    if not args.no_batch and rank == 0:
        batch = batch_probe(capi, G, sample=args.batch_sample, count=args.batch_count)
    layer = None
    if not args.no_layer and rank == 0:
        layer = layer_probe(torch, G)
    if rank != 0:
        return
    pk, pk_kind = peaks()
    achieved = bpa * att / (att_ms / 1e3) / 1e9
    prec_key = "fp64" if args.precision == "fp64" else "fp32"
    alt_key = "fp64" if alt == "fp64" else "fp32"
    suffix = "c2" if s == 1.0 else "scaled"
    traffic = traffic_from_profile(f"fused_attempt_{prec_key}_{suffix}")
    att_alt = sum(r["attempts"] for r in res_alt)
    att_ms_alt = sum(r["attempt_time_ms"] for r in res_alt)
    dev_ms_alt = sum(r["device_time_ms"] for r in res_alt)
    ach_alt = bpa_alt * att_alt / (att_ms_alt / 1e3) / 1e9
    # The FP32 attempt's working set (112 MB) nearly fits the 126 MB L2, so
    # its gathers are served by L2: its second roofline is L2's random-sector
    # rate (L1-miss sectors per attempt from the committed ncu summary against
    # the device's measured rate for random 4-byte reads of a 2 MB vector).
    l2 = None
    try:
        ceiling = capi.gather_rate(19)
    except Exception as ex:  # calibration is a report, not a gate
        ceiling = None
        print(f"gather-rate calibration failed: {ex}", file=sys.stderr)
    sectors = traffic_from_profile("fused_attempt_fp32_c2_l1_miss_sectors") if s == 1.0 else None
    if ceiling:
        fp32_rows = res if prec_key == "fp32" else res_alt
        a32 = sum(r["attempts"] for r in fp32_rows)
        ms32 = sum(r["attempt_time_ms"] for r in fp32_rows)
        l2 = {"kernel": "FP32 attempt", "bound": "l2 random sectors",
              "ceiling_sectors_per_s": ceiling,
              "ceiling_probe": "random 4-byte reads of a 2 MB resident vector "
                               "(igaos_pdhg_gather_rate)"}
        if sectors:
            rate = sectors / (1e-3 * ms32 / a32)
            l2.update({"sectors_per_launch": sectors, "achieved_sectors_per_s": rate,
                       "frac": rate / ceiling})
    if args.no_cpu:
        cpu_v, cpu_r = None, {"loop_seconds": 0.0}
    else:
        cpu_v, cpu_r = cpu_sample(lp, args.cpu_iters, os.cpu_count() or 1)
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic",
        "config": config_dict(lp, args),
        "roofline": {"kernel": f"fused PDHG attempt, {prec_key.upper()} (k_primal: A^T y + "
                               "primal step; k_dual: A xbar + dual step + step decision)",
                     "bound": "hbm", "achieved": achieved, "peak": pk, "peak_kind": pk_kind,
                     "unit": "GB/s", "frac": achieved / pk,
                     "bytes_per_launch": bpa, "launch_us": 1e3 * att_ms / att,
                     "traffic": traffic},
        "cpu_baseline": {"value": cpu_v, "unit": "GB/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"{args.cpu_iters} iterations of the reference FP64 PDHG "
                                   f"(CPU oracle, OpenMP) on the same LP ({cpu_r['loop_seconds']:.1f} s)"},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": ck,
        "attempts_per_s": ws * att / (dev_ms_max / 1e3),
        # device time outside the fused attempts (KKT checks, restarts, the
        # step's setup) per 64-iteration check
        "check_us": 1e3 * (sum(r["device_time_ms"] for r in res) - att_ms)
                    / max(1, sum(r["iterations"] // 64 for r in res)),
        "iterations_per_step": res[-1]["iterations"], "attempts_per_step": res[-1]["attempts"],
        "entries_per_lane": {"A": res[-1]["entries_a"], "A^T": res[-1]["entries_at"]},
        alt.replace("-", "_"): {
            "value": bpa_alt * att_alt / (dev_ms_alt / 1e3) / 1e9, "unit": "GB/s",
            "ms_per_step": dev_ms_alt / len(res_alt),
            "roofline": {"achieved": ach_alt, "peak": pk, "frac": ach_alt / pk,
                         "bytes_per_launch": bpa_alt, "launch_us": 1e3 * att_ms_alt / att_alt,
                         "traffic": traffic_from_profile(f"fused_attempt_{alt_key}_{suffix}"),
                         "l2": l2 if alt_key == "fp32" else None}},
    }
    if l2 and prec_key == "fp32":
        line["roofline"]["l2"] = l2
    if small:
        line["time_to_tol_small_lp"] = small
    if c5:
        line["time_to_tol_multicommodity_lp"] = c5
    if c2tol:
        line["time_to_tol_large_lp"] = c2tol
    if refg:
        line["vs_reference_gpu"] = refg
    if batch:
        line["batched_small_lps"] = batch
    if layer:
        line["differentiable_layer"] = layer
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
