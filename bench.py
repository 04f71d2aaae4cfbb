#!/usr/bin/env python
"""Benchmark of the 3-D Laplace field solve on one GB300 (or N replicas).

Workload (default): the FP64 cascadic multigrid solve of a quadrupole in a
grounded 257^3 box -- levels 33^3, 65^3, 129^3, 257^3; four rods along z of
radius 1.148*r0 (r0 = 32 cells), rod axes 32 + 36.7 cells from the box axis
on +-x (+1 V) and +-y (-1 V); red-black SOR at omega 1.85 on every level with
the relative residual max|r|/max|r(phi_D)| checked every 20 sweep pairs,
stopping below 1e-10 (intermediate levels below 30x that).  One step = one
complete solve.  Arrays (phi 136 MB + mask 17 MB) exceed the 129 MB L2, so no
L2 flush is needed between steps.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl reference]

Prints one JSON line.  `value` is solves/s with the inputs resident in HBM;
`e2e` is the same solve through the public API from pinned host buffers
(host->device copies of mask and Dirichlet values, device->host copy of phi
inside the timed region).  `--impl reference` times the CPU restatement of
the reference's sweep (oracle/, all host threads) on a bounded sample of the
same workload.
"""
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

METRIC = ("basis solves/s & GLUP/s at 1e-9 accuracy, mixed vs FP64 GPU; "
          "p50/p99 latency")
WORKLOAD = "quadrupole_257_cascadic_fp64"
N_SIDE = 257
R0 = 32.0
OMEGA = 1.85
REL_TOL = 1e-10
LEVELS = 4
CHECK_EVERY = 20
FP64_BYTES_PER_LUP = 17      # read phi 8 + write phi 8 + mask 1


def quadrupole(n=N_SIDE, r0=R0):
    from ion_gym_gb300.workloads import quadrupole as q
    return q(n, r0)


def level_shapes():
    from ion_gym_gb300.physics.multigrid3d import cascadic_shapes
    return cascadic_shapes((N_SIDE,) * 3, 9, LEVELS)


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4)
                          if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_sample(fixed, seconds=15.0, max_pairs=400):
    """Time red-black pairs of the reference sweep (oracle C restatement,
    all host threads, theta read as ones as the reference does) on the fine
    grid.  Returns (GLUP/s, pairs timed, seconds, threads)."""
    from oracle import port
    shape = fixed.shape
    phi = np.zeros(shape)
    th = np.ones((6,) + shape, np.float32)
    port.sweep(phi, fixed, th, OMEGA, 0, True)      # warm the pages
    port.sweep(phi, fixed, th, OMEGA, 1, True)
    pairs = 0
    t0 = time.perf_counter()
    while True:
        port.sweep(phi, fixed, th, OMEGA, 0, True)
        port.sweep(phi, fixed, th, OMEGA, 1, True)
        pairs += 1
        el = time.perf_counter() - t0
        if el >= seconds or pairs >= max_pairs:
            break
    n = fixed.size
    return n * pairs / el / 1e9, pairs, el, port.num_threads()


def lups_per_solve(level_pairs):
    shapes = level_shapes()
    return sum(int(np.prod(s)) * p for s, p in zip(shapes, level_pairs))


def load_profile_traffic():
    """dram bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/), or None."""
    p = os.path.join(ROOT, "profiles", "sweep_f64_quad257.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def run_ours(a):
    import torch
    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from ion_gym_gb300 import build as B, _lib
    if not os.path.exists(B.LIB):
        B.build()
    from ion_gym_gb300.physics import multigrid3d as MG
    L = _lib.lib()

    fixed, val = quadrupole()
    n = fixed.size
    fx_d = torch.from_numpy(fixed.view(np.uint8)).cuda()
    val_d = torch.from_numpy(val).cuda()
    phi_d = torch.empty_like(val_d)
    fx_h = torch.from_numpy(fixed.view(np.uint8)).pin_memory()
    val_h = torch.from_numpy(val).pin_memory()
    phi_h = torch.empty(val.shape, dtype=torch.float64).pin_memory()

    def solve_dev():
        return MG.solve3d_cascadic_relres(fx_d, val_d, REL_TOL, OMEGA, LEVELS,
                                          9, CHECK_EVERY, out=phi_d)

    def solve_host():
        return MG.solve3d_cascadic_relres(fx_h, val_h, REL_TOL, OMEGA, LEVELS,
                                          9, CHECK_EVERY, out=phi_h)

    def barrier():
        if ws > 1:
            import torch.distributed as tdist
            tdist.barrier()
        torch.cuda.synchronize()

    info = None
    for _ in range(a.warmup):
        info = solve_dev()
    # timed: device-resident inputs
    clocks = Clocks(local)
    L.ig_prof_reset()
    L.ig_prof_enable(1)
    launches0 = L.ig_launch_count()
    barrier()
    clocks.start()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        info = solve_dev()
    barrier()
    el = time.perf_counter() - t0
    ck = clocks.stop()
    launches = L.ig_launch_count() - launches0
    L.ig_prof_enable(0)
    import ctypes
    ms = ctypes.c_double(0.0)
    nl = ctypes.c_long(0)
    nodes = ctypes.c_long(0)
    L.ig_prof_read(ctypes.byref(ms), ctypes.byref(nl), ctypes.byref(nodes))
    if ws > 1:
        import torch.distributed as tdist
        t = torch.tensor([el], device="cuda", dtype=torch.float64)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        el = float(t.item())
    # e2e: public API on pinned host buffers, copies inside the timed region
    barrier()
    t1 = time.perf_counter()
    for _ in range(a.steps):
        solve_host()
    barrier()
    el_e2e = time.perf_counter() - t1
    if ws > 1:
        import torch.distributed as tdist
        t = torch.tensor([el_e2e], device="cuda", dtype=torch.float64)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        el_e2e = float(t.item())

    _, fine_pairs, relres, total_pairs = info
    lups = nodes.value / a.steps                      # LUPs per solve
    solves_s = ws * a.steps / el
    glups = ws * lups * a.steps / el / 1e9
    # dominant kernel: the FP64 red-black sweep (both colours)
    achieved = FP64_BYTES_PER_LUP * nodes.value / (ms.value * 1e-3) / 1e9
    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    peak = peaks.get("hbm_gbs")
    traffic = load_profile_traffic()
    line = {
        "metric": METRIC, "value": solves_s, "unit": "solves/s",
        "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1e3 * el / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded geometry of the named workload)",
        "config": {"workload": WORKLOAD, "grid": [N_SIDE] * 3,
                   "levels": [list(s) for s in level_shapes()],
                   "omega": OMEGA, "rel_tol": REL_TOL,
                   "check_every_pairs": CHECK_EVERY,
                   "parallelism": f"replicas{ws}" if ws > 1 else "single",
                   "l2": "inputs larger than L2 (153 MB resident > 129 MB)"},
        "glup_s": glups,
        "lups_per_solve": lups,
        "fine_pairs": fine_pairs, "total_pairs": total_pairs,
        "fine_relres": relres,
        "e2e": {"value": ws * a.steps / el_e2e, "unit": "solves/s",
                "h2d_bytes_per_step": n * 9, "d2h_bytes_per_step": n * 8},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak,
                     "unit": "GB/s",
                     "frac": (achieved / peak) if peak else None,
                     "traffic": traffic,
                     "kernel": "k_sweep<kPlain> (FP64 red-black sweep)",
                     "avg_launch_us": 1e3 * ms.value / max(nl.value, 1),
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"
                     if peak else None},
        "clocks": ck,
    }
    if rank == 0 and ws == 1 and not a.no_cpu:
        g, pairs, secs, thr = cpu_sample(fixed, seconds=a.cpu_seconds)
        line["cpu_baseline"] = {
            "value": g * 1e9 / lups, "unit": "solves/s", "cores": thr,
            "kind": "port", "glup_s": g,
            "sample": f"{pairs} red-black pairs of the reference sweep "
                      f"(oracle C restatement, theta read as ones) on the "
                      f"257^3 fine grid in {secs:.1f} s; solves/s = GLUP/s / "
                      f"LUPs per solve ({lups:.4g})"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as tdist
        tdist.destroy_process_group()


# LUPs of one solve of this workload (sum over levels of nodes x pairs); the
# iterates are identical on every implementation (the GPU sweeps return the
# reference's bits), so the count is a property of the workload.
LUPS_PER_SOLVE = 26187534900   # 1500 fine pairs + 600 coarse-level pairs


def run_reference(a):
    ws, rank, _ = dist()
    if rank != 0:
        return
    import __graft_entry__ as g
    g.build_oracle()
    from oracle import port
    fixed, val = quadrupole()
    lups = LUPS_PER_SOLVE
    if lups is None:
        print(json.dumps({"impl": "reference", "unavailable":
                          "LUPs per solve of the workload not recorded yet"}))
        return
    per_step = max(2.0, a.cpu_seconds / 2)
    vals = []
    port.set_threads(os.cpu_count() or 1)
    for s in range(a.warmup + a.steps):
        gl, pairs, secs, thr = cpu_sample(fixed, seconds=per_step)
        if s >= a.warmup:
            vals.append(gl)
    g_mean = float(np.mean(vals))
    v = g_mean * 1e9 / lups
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s",
        "n_gpus": ws, "steps": a.steps, "warmup": a.warmup,
        "higher_is_better": True, "scaling": "weak", "dtype": "f64",
        "config": {"workload": WORKLOAD, "grid": [N_SIDE] * 3},
        "glup_s": g_mean,
        "cpu_baseline": {"value": v, "unit": "solves/s", "cores": thr,
                         "kind": "port",
                         "sample": f"each step: red-black pairs of the "
                                   f"reference sweep (oracle C restatement) "
                                   f"on the 257^3 fine grid for ~{per_step:.0f}"
                                   f" s; solves/s = GLUP/s / {lups:.4g} LUPs"},
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0}}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu", action="store_true")
    a = ap.parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
