#!/usr/bin/env python3
"""Benchmark of the GB300 Constant-Q-PSTD time-stepping path.

Prints one JSON line.  A timed "step" is one time step of the fused PSTD
pipeline of the workload's shot (device-resident inputs, CUDA events on the
library's stream, L2 flushed between timed steps).  `e2e` runs the whole shot
(RTM with revolve recompute, or modeling) through the C ABI with host buffers,
host<->device copies included.  `cpu_baseline` times the FP64 C oracle (a CPU
restatement of the reference's update equations) on the machine's host cores.

--impl reference times the reference arm: the reference has no CPU stepping
path and its cuFFT build cannot be compiled on the GPU machine (its sources are not
shipped), so the arm runs the oracle port of its equations on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "constant-q-pstd_gb300")
sys.path.insert(0, PKG)

METRIC = "Q-RTM shots/hr batched vs per-shot @relL2≤1e-4; Gpts/s; HBM GB/s; p50/p99"

# Algorithmic bytes per padded grid point per time step (every state field
# read and written once, every model field read once): aps / artm source
# step 72 B (7 state x 8 + 4 model x 4).
ALG_BYTES_STEP = {"aps": 72.0, "artm": 72.0}
# Compulsory traffic of each fused pass (fields it must read or write once).
PASS_BYTES = {"xpass": 56.0, "zpass": 44.0}


def workload(name: str):
    import workloads as W

    if name == "artm3":
        # Acoustic RTM, one shot: 800 x 2400 model, 12 layers + 3 anomalies,
        # migration model = 8-cell Gaussian blur, CPML 30, 2400 receivers,
        # dt = 0.5 ms, nt = 6000, 40 revolve snapshots.
        d = W.make_shot(2, 2400, 800, 30, 6000, 0.0005, 20.0, seed=1003, nlayers=12, nanom=3,
                        smooth_cells=8.0, snaps=40)
        true = W.make_shot(0, 2400, 800, 30, 6000, 0.0005, 20.0, seed=1003, nlayers=12, nanom=3)
        return d, true, "artm", 1003
    if name == "aps1":
        d = W.make_shot(0, 398, 160, 20, 2000, 0.001, 20.0, seed=1001, nlayers=5, nanom=1)
        return d, None, "aps", 1001
    raise SystemExit(f"unknown workload {name}")


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(ws, v: float) -> float:
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_oracle_rate(d: dict, kind_name: str, budget_s: float, max_cols: int | None = None):
    """FP64 oracle steps/s on the host cores for a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    dd = dict(d)
    if max_cols is not None and dd["nxx"] > max_cols:
        # crop the window to max_cols columns (same nzz), keeping the source inside
        nxx, nzz = dd["nxx"], dd["nzz"]
        x0 = max(0, min(dd["xsg"] - max_cols // 2, nxx - max_cols))
        for k in ("vp", "rho", "bbx", "bbz", "gam", "lam", "vwd", "tao"):
            if dd.get(k) is not None:
                dd[k] = np.asarray(dd[k]).reshape(nxx, nzz)[x0:x0 + max_cols].ravel()
        keep = (dd["gxg"] >= x0) & (dd["gxg"] < x0 + max_cols)
        dd["gxg"] = (dd["gxg"][keep] - x0).astype(np.int32)
        dd["gzg"] = dd["gzg"][keep]
        dd["xsg"] = dd["xsg"] - x0
        dd["nxx"] = max_cols
    dd["kind"] = O.APS if kind_name in ("aps", "artm") else O.VAPS
    osh = O.OracleShot(dd)
    st = np.zeros((8, dd["nxx"], dd["nzz"]))
    t = time.perf_counter()
    osh.steps(st, 0, 1, want_gather=False)
    one = time.perf_counter() - t
    n = max(1, int(budget_s / max(one, 1e-3)))
    t = time.perf_counter()
    osh.steps(st, 1, n, want_gather=False)
    el = time.perf_counter() - t
    pts = dd["nxx"] * dd["nzz"]
    return pts * n / el / 1e9, n, dd["nxx"], dd["nzz"], el


def run_reference(args, ws, rank):
    """Reference arm: the FP64 port of the reference equations on host cores."""
    if rank != 0:
        return
    d, _, kname, seed = workload(args.workload)
    threads = os.cpu_count() or 1
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cols = min(d["nxx"], 600)
    per_step = []
    dd = d
    # one oracle time step per bench step on a cropped window of the workload grid
    rate, n, nxx_s, nzz_s, _ = cpu_oracle_rate(d, kname, 0.0, max_cols=cols)
    for i in range(args.warmup + args.steps):
        r, n1, _, _, el = cpu_oracle_rate(d, kname, 0.0, max_cols=cols)
        if i >= args.warmup:
            per_step.append(el / n1)
    ms = 1000.0 * statistics.mean(per_step)
    val = nxx_s * nzz_s / (ms / 1000.0) / 1e9
    out = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "Gpts/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": f"synthetic (seed {seed})",
        "config": {"workload": args.workload, "grid": [d["nxx"], d["nzz"]], "nt": d["nt"]},
        "cpu_baseline": {"value": val, "unit": "Gpts/s", "cores": threads, "kind": "port",
                         "sample": f"one FP64 oracle time step per bench step on a {nxx_s}x{nzz_s} "
                                   f"window of the {d['nxx']}x{d['nzz']} workload grid"},
        "e2e": {"value": val, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=60)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="artm3")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return

    import torch

    import qpstd

    torch.cuda.set_device(local)
    qpstd.lib()
    d, true_model, kname, seed = workload(args.workload)
    N = d["nxx"] * d["nzz"]
    sh = qpstd.Shot(d)
    stream = torch.cuda.ExternalStream(sh.stream_ptr())
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # warm-up steps (pipeline primed, kernels loaded)
    sh.pipeline_begin()
    t = 0
    for _ in range(args.warmup):
        sh.pipeline_step(t)
        t += 1
    sh.sync()
    barrier(ws)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sh.set_profiling(True)
    sh.profile_read()  # clear
    launches0 = sh.launch_count()
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        for i in range(args.steps):
            flush.fill_(float(i))  # evict L2 between timed steps (512 MB > 129 MB L2)
            torch.cuda.synchronize()
            ev[i][0].record(stream)
            sh.pipeline_step(t, last=(i == args.steps - 1))
            ev[i][1].record(stream)
            t += 1
        torch.cuda.synchronize()
    sh.pipeline_end()
    prof = sh.profile_read()
    sh.set_profiling(False)
    launches = sh.launch_count() - launches0 - 1  # minus pipeline_end
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = sum(step_ms)
    total_ms = allreduce_max(ws, total_ms)
    ms_per_step = total_ms / args.steps
    value = ws * N * args.steps / (total_ms / 1000.0) / 1e9

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    kern = {k: {"ms_avg": (v[0] / v[1]) if v[1] else 0.0, "launches": v[1]} for k, v in prof.items() if v[1]}
    step_kernel_ms = sum(kern[k]["ms_avg"] for k in ("xpass", "zpass") if k in kern)
    alg = ALG_BYTES_STEP[kname] * N
    achieved = alg / (step_kernel_ms / 1000.0) / 1e9
    for k in kern:
        if k in PASS_BYTES:
            kern[k]["compulsory_gbs"] = PASS_BYTES[k] * N / (kern[k]["ms_avg"] / 1000.0) / 1e9
    dom = max(kern, key=lambda k: kern[k]["ms_avg"] * kern[k]["launches"])
    traffic = None
    try:
        prof_file = os.path.join(ROOT, "profiles", f"traffic_{args.workload}.json")
        tj = json.load(open(prof_file))
        traffic = tj.get("dram_bytes_per_step")
    except OSError:
        pass
    out = {
        "metric": METRIC,
        "value": value,
        "unit": "Gpts/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_per_step,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": f"synthetic (seeded layered model, seed {seed})",
        "config": {"workload": args.workload, "kind": kname, "grid": [d["nxx"], d["nzz"]], "nt": d["nt"],
                   "snaps": d.get("snaps"), "receivers": int(len(d["gxg"])), "form": "acoustic",
                   "l2": "flushed (512 MB write) between timed steps", "method": "fused line-FFT passes"},
        "roofline": {"bound": "hbm", "kernel": "one fused time step (ac_zpass + ac_xpass)",
                     "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "peak_source": peak_src, "alg_bytes_per_point": ALG_BYTES_STEP[kname],
                     "traffic": traffic, "dominant": dom},
        "kernels": kern,
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
    }
    # ---- end to end through the C ABI with host buffers ----
    if not args.no_e2e:
        del sh
        if kname == "artm":
            obs = qpstd.model_shot(true_model)
            torch.cuda.synchronize()
            barrier(ws)
            t0 = time.perf_counter()
            img, ssg = qpstd.rtm_shot(d, obs)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t0
            wall = allreduce_max(ws, wall)
            pts = N * 2 * d["nt"]
            h2d = 4 * (4 * N + d["nt"] + 2 * len(d["gxg"]) + obs.size)
            d2h = 4 * 2 * img.size
        else:
            t0 = time.perf_counter()
            g = qpstd.model_shot(d)
            wall = allreduce_max(ws, time.perf_counter() - t0)
            pts = N * d["nt"]
            h2d = 4 * (4 * N + d["nt"] + 2 * len(d["gxg"]))
            d2h = 4 * g.size
        out["e2e"] = {"value": ws * pts / wall / 1e9, "unit": "Gpts/s", "wall_s_per_shot": wall,
                      "shots_per_hour": ws * 3600.0 / wall, "h2d_bytes_per_step": h2d,
                      "d2h_bytes_per_step": d2h, "step": "one full shot per call"}
    # ---- CPU baseline (rank 0, N=1) ----
    if rank == 0 and ws == 1:
        rate, n, nxx_s, nzz_s, el = cpu_oracle_rate(d, kname, args.cpu_budget)
        out["cpu_baseline"] = {"value": rate, "unit": "Gpts/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": f"{n} FP64 oracle time steps on the full {nxx_s}x{nzz_s} grid "
                                         f"({el:.1f} s)"}
    if rank == 0:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
