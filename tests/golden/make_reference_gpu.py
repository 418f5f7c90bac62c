#!/usr/bin/env python3
"""Runs the reference's own cuFFT modeling programs on a GPU and records their
gathers (the fixture tests/golden/reference_gpu_gathers.npz) and their run
times (baseline B1).

TEST INFRASTRUCTURE.  Prerequisites: `python oracle/refgpu/stage.py` where the
reference tree is mounted (copies the sources of the reference's aps / vaps
programs into the git-ignored baseline/_ref/src), then, on the GPU machine,

    python tests/golden/make_reference_gpu.py OUTDIR

builds them (oracle/refgpu/Makefile: the reference's own .cu / .c files for
sm_103a with a one-rank MPI stub) and runs, in project trees laid out as the
reference expects (tests/refgpu_case.py):
  * pins: aps (400 steps) and vaps (300 steps) as shipped (CPML 10) on the
    seeded one-shot case; their reca / recva gathers go to OUTDIR/reference_gpu_gathers.npz;
  * timing: aps and vaps with the CPML patched to 20 on the same shot (the aps
    and vaps workloads: 2000 and 3000 steps), each also at 200
    steps so the per-step time excludes start-up; OUTDIR/reference_gpu_timing.json.
Everything the reference programs do (cuFFT plans, a host copy of p and a
stream synchronisation every step) is inside the wall times.
"""
import json
import os
import shutil
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.dirname(HERE), os.path.join(ROOT, "constant-q-pstd_gb300")]
import refgpu_case as R  # noqa: E402

BIN = os.path.join(ROOT, "baseline", "_ref", "bin")


def run(prog: str, nt: int):
    """One run of a reference program on the one-shot case: (gather, wall seconds, stdout tail)."""
    tree = tempfile.mkdtemp(prefix="refgpu", dir="/tmp")
    try:
        R.write_tree(tree, nt)
        env = dict(os.environ, CUDA_VISIBLE_DEVICES=os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0])
        t0 = time.perf_counter()
        r = subprocess.run([os.path.join(BIN, prog)], cwd=os.path.join(tree, "run"), capture_output=True,
                           text=True, timeout=1800, env=env)
        wall = time.perf_counter() - t0
        if r.returncode != 0:
            raise SystemExit(f"{prog} exited {r.returncode}: {r.stdout[-1500:]} {r.stderr[-1500:]}")
        pre = "reca" if prog.startswith("aps") else "recva"
        path = os.path.join(tree, "obsdata", f"{pre}0_398.bin")
        g = np.fromfile(path, dtype=np.float32).reshape(nt, 398)
        return g, wall, r.stdout[-400:]
    finally:
        shutil.rmtree(tree, ignore_errors=True)


def main():
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "gpurun_out", "refgpu")
    os.makedirs(out, exist_ok=True)
    subprocess.run(["make", "-s", "-j", "4", "-C", os.path.join(ROOT, "oracle", "refgpu")], check=True)
    pins = {}
    log = {}
    for prog, nt in (("aps", 400), ("vaps", 300)):
        g, wall, tail = run(prog, nt)
        if not np.isfinite(g).all() or not np.abs(g).max() > 0:
            raise SystemExit(f"{prog}: gather is not finite or all zero")
        pins[f"{prog}_gather"] = g
        pins[f"{prog}_nt"] = np.int32(nt)
        log[prog] = {"nt": nt, "wall_s": wall, "stdout_tail": tail}
    gx, gz = R.geometry()
    np.savez_compressed(os.path.join(out, "reference_gpu_gathers.npz"), gx=gx, gz=gz, pml=np.int32(10), **pins)
    timing = {}
    for prog, nt in (("aps20", 2000), ("vaps20", 3000)):
        _, w_long, tail = run(prog, nt)
        _, w_short, _ = run(prog, 200)
        per_step = (w_long - w_short) / (nt - 200)
        timing[prog] = {"nt": nt, "grid": [439, 200], "wall_s": w_long, "wall_s_nt200": w_short,
                        "ms_per_step": 1000.0 * per_step, "gpts_per_s": 439 * 200 / per_step / 1e9,
                        "shots_per_hour": 3600.0 / w_long, "stdout_tail": tail}
    try:
        smi = subprocess.run(["nvidia-smi", "--query-gpu=name,driver_version", "--format=csv,noheader"],
                             capture_output=True, text=True).stdout.strip()
    except OSError:
        smi = ""
    nvcc = subprocess.run(["nvcc", "--version"], capture_output=True, text=True).stdout.strip().splitlines()[-1]
    json.dump({"pins": log, "timing": timing, "gpu": smi, "nvcc": nvcc}, open(os.path.join(out, "reference_gpu_timing.json"), "w"),
              indent=1)
    print(json.dumps({k: {kk: vv for kk, vv in v.items() if kk != "stdout_tail"} for k, v in timing.items()}))


if __name__ == "__main__":
    main()
