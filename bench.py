"""Benchmark of the GB300 PDHG LP engine on the large sparse LP shape.

Workload (one step): the large sparse LP (m=200,000 rows, half equality half
<=, n=500,000 box-bounded columns, ~5.2M nonzeros with Zipf(1.5) column
degrees and |A_ij| log-uniform in [1e-3, 1e3]; seeded synthetic data), one
solve call of ITERS accepted PDHG iterations with FP32 attempts and FP64
refinement (FP64 anchors re-set at restarts, FP64 KKT checks every 64
iterations), from a cold start on device-resident data.

Also reported (extra keys): time to 1e-8 relative KKT on the small random LP
(m=2,000, n=5,000) for FP32+refine vs plain FP64 and the CPU oracle, where
all of them converge; the large LP is not solved to 1e-8 by either
precision in a bench-sized budget (see --tol-probe). With it,
`crossover_from_fp32_refine`: the host crossover (igaos_pdhg_crossover) from
the FP32+refine answer to an optimal vertex, wall time and pivots.
`time_to_1e-8_multicommodity_lp`: the same comparison on the 1.08M x 2.87M
multicommodity-flow LP. `batched_small_lps`:
4,096 uneven small LPs solved to 1e-6 in one persistent launch vs
sequential single-LP solves. `differentiable_layer`: forward and adjoint
backward through 1,000 unrolled iterations of 256 ridge-regularised LPs.

value: SpMV GB/s -- algorithmic bytes of every fused A^T y / A xbar attempt
of the solve divided by the solve's CUDA-event device time (checks, restarts
and host round trips included). Algorithmic bytes per attempt (s = 4 for
FP32, 8 for FP64; int32 indices):
    2*nnz*(s+4) + 4*(m+n+2) + s*9*(m+n)
(each matrix entry and index once per orientation, row/column pointers once,
nine m- and nine n-vectors read or written once each: x, xavg, c, l, u, xbar
and y, A x, yavg, rmin, rmax gathered/read; x', xavg', xbar, y', A x', yavg'
written).
roofline: the fused attempt's algorithmic bytes over its CUDA-event time
against the measured HBM copy bandwidth; `roofline.l2` adds the bound that
limits it on this LP, whose working set nearly fits L2: L1-miss sectors per
attempt (committed ncu summary) per second against the device's random
4-byte read rate of a 2 MB vector (igaos_pdhg_gather_rate, measured in the
same run). The multicommodity extra reports `attempt_us` and
`attempt_hbm_frac` for an LP that streams from HBM.
e2e: the same metric through the C ABI with HOST buffers: igaos_pdhg_solve_csr
(upload, device setup, solve, download, free) timed on the host.
L2: flushed (512 MiB write) between steps. Reference arm and cpu_baseline:
the CPU oracle of the reference FP64 PDHG (tests' checker) on the machine's host
cores over a bounded sample of the same solve.
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
            "iters_per_step": args.iters, "l2": "flushed between steps (512 MiB write)",
            "parallelism": f"replicas x{args.gpus}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--iters", type=int, default=2048)
    ap.add_argument("--precision", default="fp32-refine", choices=["fp32", "fp64", "fp32-refine"])
    ap.add_argument("--no-small", action="store_true",
                    help="skip the time-to-1e-8 comparison on the small LP")
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
    ap.add_argument("--no-c5", action="store_true", help="skip the multicommodity time-to-1e-8")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-LP comparison")
    ap.add_argument("--no-layer", action="store_true", help="skip the differentiable layer")
    ap.add_argument("--tol-probe", type=float, default=0.0,
                    help="also report time-to-tolerance probes within this many seconds")
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
                     max_iterations=args.iters)
            P.solve(**o)
            r = P.solve(**o)
        us = 1e3 * r["attempt_time_ms"] / max(1, r["attempts"])
        pk, pk_kind = peaks()
        print(json.dumps({"workload": f"multicommodity flow m={flp.m} n={flp.n} nnz={flp.nnz}",
                          "precision": args.precision, "iterations": r["iterations"],
                          "attempts": r["attempts"], "attempt_us": us, "attempt_bytes": cb,
                          "attempt_hbm_frac": cb / (us * 1e-6) / 1e9 / pk,
                          "hbm_peak_kind": pk_kind}), flush=True)
        return
    if args.probe:  # one extra workload alone (profiling runs)
        res = batch_probe(capi, G, sample=args.batch_sample, count=args.batch_count,
                          warm=False) if args.probe == "batch" else layer_probe(torch, G)
        print(json.dumps(res), flush=True)
        return
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    opts = dict(precision=args.precision, tolerance=1e-12, time_limit=1e9,
                max_iterations=args.iters, device=local)
    bpa = bytes_per_attempt(lp.m, lp.n, lp.nnz, 8 if args.precision == "fp64" else 4)
    with capi.Problem(lp, device=local) as P:
        for _ in range(args.warmup):
            P.solve(**opts)
        clocks = Clocks(local)
        barrier(ws)
        torch.cuda.synchronize()
        res = []
        for _ in range(args.steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            res.append(P.solve(**opts))
        torch.cuda.synchronize()
        barrier(ws)
        ck = clocks.stop()
    dev_ms = sum(r["device_time_ms"] for r in res)
    att = sum(r["attempts"] for r in res)
    att_ms = sum(r["attempt_time_ms"] for r in res)
    launches = sum(r["launches"] for r in res)
    dev_ms_max = barrier_max(dev_ms, ws)
    value = ws * bpa * att / (dev_ms_max / 1e3) / 1e9
    # e2e through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        h2d = sum(np.asarray(a).nbytes for a in (lp.ap, lp.ai, lp.ax, lp.cp, lp.ci, lp.acx, lp.c,
                                                   lp.cl, lp.cu, lp.rmin, lp.rmax))
        d2h = 8 * (lp.m + lp.n)
        e_steps = min(args.steps, 3)
        capi.solve_lp(lp, **opts)
        barrier(ws)
        t0 = time.perf_counter()
        e_att = 0
        for _ in range(e_steps):
            r = capi.solve_lp(lp, **opts)
            e_att += r["attempts"]
        torch.cuda.synchronize()
        el = barrier_max(time.perf_counter() - t0, ws)
        e2e = {"value": ws * bpa * e_att / el / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * el / e_steps}
    # time-to-tolerance probes (not part of `value`)
    # Time to 1e-8 relative KKT, FP32 + FP64 refinement vs plain FP64 (the
    # reference algorithm), on the small random LP (m=2,000, n=5,000,
    # ~20k nnz) where both reach it; device-resident, CUDA-event time.
    small = None
    if not args.no_small and rank == 0:
        slp = G.config1(seed=0)
        small = {"workload": "small random LP m=2000 n=5000 nnz=19988 (seed 0), tol 1e-8"}
        with capi.Problem(slp, device=local) as P:
            for prec in ("fp64", "fp32-refine"):
                P.solve(precision=prec, tolerance=1e-6, time_limit=60.0)  # warm
                r = P.solve(precision=prec, tolerance=1e-8, time_limit=60.0)
                small[prec] = {"status": r["status_name"], "s": r["device_time_ms"] / 1e3,
                               "iterations": r["iterations"], "objective": r["objective"]}
                x_last = r["x"]
        if small["fp64"]["status"] == small["fp32-refine"]["status"] == "near-optimal":
            small["speedup_fp32_refine_vs_fp64"] = small["fp64"]["s"] / small["fp32-refine"]["s"]
        # host crossover from the FP32 + refinement answer to an optimal vertex
        # (a probe: the line does not depend on it)
        try:
            t0 = time.perf_counter()
            xv, _, _, xi = capi.crossover(slp, x_last)
            small["crossover_from_fp32_refine"] = {
                "status": xi["status"], "s": time.perf_counter() - t0, "pivots": xi["pivots"],
                "host_threads": min(16, os.cpu_count() or 1),
                "objective": float(slp.c @ xv + slp.obj_const)}
        except Exception as e:
            small["crossover_from_fp32_refine"] = {"error": str(e)[:200]}
        from oracle import oracle as O
        rr = O.pdhg_solve(O.lp_from(slp), tolerance=1e-8, time_limit=120.0,
                          threads=os.cpu_count() or 1)
        small["cpu_oracle_fp64"] = {"status": rr["status_name"], "s": rr["seconds"],
                                    "iterations": rr["iterations"], "cores": os.cpu_count()}
    # Time to 1e-8 on the multicommodity-flow LP (300 x 300 grid, 8
    # commodities: m=1,078,800, n=2,870,400, nnz=8,611,200), where both
    # precisions reach it within the bench's budget.
    c5 = None
    if not args.no_c5 and rank == 0:
        flp = G.config5(seed=0)
        c5 = {"workload": f"multicommodity flow m={flp.m} n={flp.n} nnz={flp.nnz} (seed 0), "
                          "tol 1e-8, device-resident, CUDA-event time"}
        with capi.Problem(flp, device=local) as P:
            for prec in ("fp32-refine", "fp64"):
                r = P.solve(precision=prec, tolerance=1e-8, time_limit=240.0)
                # this LP's working set (~300 MB FP32) exceeds L2: its attempts
                # stream from HBM, so the HBM roofline is the bound here
                cb = bytes_per_attempt(flp.m, flp.n, flp.nnz, 8 if prec == "fp64" else 4)
                us = 1e3 * r["attempt_time_ms"] / max(1, r["attempts"])
                pk5, pk5_kind = peaks()
                c5[prec] = {"status": r["status_name"], "s": r["device_time_ms"] / 1e3,
                            "iterations": r["iterations"], "attempts": r["attempts"],
                            "objective": r["objective"], "pinf": r["pinf"], "dinf": r["dinf"],
                            "rel_gap": r["rel_gap"], "prow": r["prow"],
                            "attempt_us": us, "attempt_bytes": cb,
                            "attempt_hbm_frac": cb / (us * 1e-6) / 1e9 / pk5,
                            "hbm_peak_kind": pk5_kind}
        if c5["fp64"]["status"] == c5["fp32-refine"]["status"] == "near-optimal":
            c5["speedup_fp32_refine_vs_fp64"] = c5["fp64"]["s"] / c5["fp32-refine"]["s"]
            c5["objective_rel_diff"] = abs(c5["fp64"]["objective"] - c5["fp32-refine"]["objective"]) / \
                max(1.0, abs(c5["fp64"]["objective"]))
    batch = None
    if not args.no_batch and rank == 0:
        batch = batch_probe(capi, G, sample=args.batch_sample, count=args.batch_count)
    layer = None
    if not args.no_layer and rank == 0:
        layer = layer_probe(torch, G)
    probes = {}
    if args.tol_probe > 0:
        with capi.Problem(lp, device=local) as P:
            for prec in ("fp32-refine", "fp64"):
                for tol in (1e-4, 1e-8):
                    r = P.solve(precision=prec, tolerance=tol, time_limit=args.tol_probe)
                    probes[f"{prec}@{tol:g}"] = {
                        "status": r["status_name"], "device_s": r["device_time_ms"] / 1e3,
                        "iterations": r["iterations"], "pinf": r["pinf"], "dinf": r["dinf"],
                        "rel_gap": r["rel_gap"]}
    if rank != 0:
        return
    pk, pk_kind = peaks()
    achieved = bpa * att / (att_ms / 1e3) / 1e9
    # both FP32 modes run the same attempt kernels (refinement adds one
    # m-vector read of the rounded anchor y)
    prec_key = "fp64" if args.precision == "fp64" else "fp32"
    traffic = traffic_from_profile(f"fused_attempt_{prec_key}_{'c2' if s == 1.0 else 'scaled'}")
    # The attempt's gathers are served by L2 (its working set nearly fits the
    # 126 MB L2), so its second roofline is the random-sector rate of L2:
    # L1-miss sectors per attempt (ncu, committed summary) against the
    # device's measured rate for random 4-byte reads of a 2 MB vector.
    l2 = None
    sectors = traffic_from_profile(f"fused_attempt_{prec_key}_c2_l1_miss_sectors") if s == 1.0 else None
    try:
        ceiling = capi.gather_rate(19)
    except Exception as ex:  # calibration is a report, not a gate
        ceiling = None
        print(f"gather-rate calibration failed: {ex}", file=sys.stderr)
    if ceiling:
        l2 = {"bound": "l2 random sectors", "ceiling_sectors_per_s": ceiling,
              "ceiling_probe": "random 4-byte reads of a 2 MB resident vector (igaos_pdhg_gather_rate)"}
        if sectors:
            rate = sectors / (1e-3 * att_ms / att)
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
        "roofline": {"kernel": "fused PDHG attempt (k_primal: A^T y + primal step; k_dual: "
                               "A xbar + dual step + step decision)",
                     "bound": "hbm", "achieved": achieved, "peak": pk, "peak_kind": pk_kind,
                     "unit": "GB/s", "frac": achieved / pk,
                     "bytes_per_launch": bpa, "launch_us": 1e3 * att_ms / att,
                     "traffic": traffic, "l2": l2},
        "cpu_baseline": {"value": cpu_v, "unit": "GB/s", "cores": os.cpu_count(),
                         "kind": "port",
                         "sample": f"{args.cpu_iters} iterations of the reference FP64 PDHG "
                                   f"(CPU oracle, OpenMP) on the same LP ({cpu_r['loop_seconds']:.1f} s)"},
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": ck,
        "kkt_passes_per_s": ws * att / (dev_ms_max / 1e3),
        "iterations_per_step": res[-1]["iterations"], "attempts_per_step": res[-1]["attempts"],
    }
    if small:
        line["time_to_1e-8_small_lp"] = small
    if c5:
        line["time_to_1e-8_multicommodity_lp"] = c5
    if batch:
        line["batched_small_lps"] = batch
    if layer:
        line["differentiable_layer"] = layer
    if probes:
        line["time_to_tol"] = probes
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
