"""Benchmark: FIRE minimisations of bidisperse disks, N = 16384, phi = 0.86, run
to max|F_i| <= 1e-13 (the 16384-disk FIRE workload), plus the per-kernel
roofline and the CPU baseline.

A step is one complete FIRE minimisation of one seeded random packing (cell
list + neighbour list build, initial forces, then FIRE until max|F_i| <= 1e-13).
Every step uses a different seed; all arms use the same seeds.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default): the GB300 library through its C ABI.  `value` = solves/s
with the initial packings resident in HBM; `e2e` = the same through host
buffers (positions/radii/masses in, positions/PE out).  L2 (126 MB) is flushed
between timed steps (a 512 MiB write) since one 16384-disk system fits in L2.
--impl reference: the CPU restatement of the reference algorithm (the oracle,
oracle/dpg_oracle.c, OpenMP over all host cores) running full minimisations
of the same seeds.  Under torchrun (N > 1) each rank solves its own seeds
(independent replicas, weak scaling); only rank 0 runs the reference arm.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
for _p in (ROOT, ROOT / "dpcuda-v2_gb300"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

METRIC = "particle-steps/s & FIRE solves/s: mixed+batched vs plain FP64, 1 GB300"
N_PART = 16384
PHI = 0.86
FMAX = 1e-13
CUT_MULT = 1.7 / 1.4        # r_c = d_max + skin 0.3
MAX_STEPS = 1_000_000
FIRE_ALPHA0, FIRE_DT0 = 0.1, 1e-2
L2_FLUSH_BYTES = 512 << 20


def workload_config():
    return {"workload": "FIRE minimisation, bidisperse disks r=0.5/0.7 50:50, N=16384, "
                        "phi=0.86, periodic, to max|F|<=1e-13",
            "n_particles": N_PART, "packing_fraction": PHI, "fmax_target": FMAX,
            "fire": {"alpha0": FIRE_ALPHA0, "dt0": FIRE_DT0, "dt_max": 10 * FIRE_DT0,
                     "f_inc": 1.1, "f_dec": 0.5, "f_alpha": 0.99, "n_min": 5},
            "neighbors": {"method": "cell", "cutoff": 1.7, "skin": 0.3, "particles_per_cell": 8},
            "precision": "fp64", "l2": "flushed between steps (512 MiB write)",
            "seeds": "1000*rank + step + 1"}


def packing(seed):
    from oracle.oracle import disk_packing  # input generator = the reference's RandomUniform
    return disk_packing(N_PART, PHI, seed)


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
        except (KeyError, ValueError):
            pass
    return 6800.0, "fallback 6.8 TB/s"


# --------------------------------------------------------------------------
# CPU arm (the oracle restatement of the reference algorithm)
# --------------------------------------------------------------------------
def cpu_solve(seed, threads):
    from oracle.oracle import DiskOracle, set_threads
    set_threads(threads)
    st = packing(seed)
    o = DiskOracle(N_PART, st["box"])
    o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
    t0 = time.perf_counter()
    o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
    steps, stopped = o.minimize_fire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, MAX_STEPS, FMAX)
    dt = time.perf_counter() - t0
    return dt, steps, o.max_force()


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle.oracle import build_oracle
    build_oracle()
    threads = os.cpu_count() or 1
    # warm-up steps: short bounded runs (untimed) to page in the library and threads
    for w in range(args.warmup):
        from oracle.oracle import DiskOracle, set_threads
        set_threads(threads)
        st = packing(900 + w)
        o = DiskOracle(N_PART, st["box"])
        o.set_arrays(x=st["x"], y=st["y"], r=st["r"], m=st["m"])
        o.setup_neighbors(0, CUT_MULT, 0.2, 8.0, 0.5)
        o.minimize_fire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 200, FMAX)
    times, iters = [], []
    for k in range(args.steps):
        dt, steps, fmax = cpu_solve(k + 1, threads)
        times.append(dt)
        iters.append(steps)
    total = sum(times)
    value = args.steps / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "FIRE solves/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": "FIRE solves/s", "cores": threads,
                             "kind": "port",
                             "sample": f"{args.steps} full minimisations (seeds 1..{args.steps}) of "
                                       f"the oracle restatement, OpenMP {threads} threads"},
            "e2e": {"value": value, "unit": "FIRE solves/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "extra": {"fire_iterations_per_solve": float(np.mean(iters)),
                      "particle_steps_per_s": N_PART * float(np.sum(iters)) / total}}
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------
def run_ours(args):
    import torch
    import dpcuda_gb300 as dpg

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local if world > 1 else 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    dpg.load_library()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def l2_flush():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    # inputs for every step, resident in HBM before the timed region
    n_sys = args.warmup + args.steps
    seeds = [1000 * rank + k + 1 for k in range(n_sys)]
    systems = []
    for sd in seeds:
        st = packing(sd)
        s = dpg.Disk(N_PART, st["box"], stream=sptr)
        dev_arrays = {k: torch.from_numpy(st[k]).to(dev) for k in ("x", "y", "r", "m")}
        systems.append((s, st, dev_arrays))
    torch.cuda.synchronize()

    def solve(s, st, arr):
        s.setState(arr["x"], arr["y"], None, None, arr["r"], arr["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        return dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, MAX_STEPS, fmax_target=FMAX)

    for k in range(args.warmup):
        solve(*systems[k])
    torch.cuda.synchronize()

    sampler = ClockSampler(dev.index or 0)
    results, ev_ms, launches = [], [], 0
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_wall0 = time.perf_counter()
    for k in range(args.warmup, n_sys):
        l2_flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s, st, arr = systems[k]
        r = solve(s, st, arr)
        e1.record(stream)
        e1.synchronize()
        ev_ms.append(e0.elapsed_time(e1))
        info = s.neighborInfo()
        # kernels per solve: setup (cell build 6 + nlist + force) + per iteration
        # move/force/guard, plus 5 cell kernels per cell rebuild and 1 per list rebuild
        launches += 10 + 3 * (r["steps"] + 1) + 5 * info["n_cell_rebuilds"] + info["n_rebuilds"]
        results.append(r)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier()
    clocks = sampler.stop()
    total_ms = float(np.sum(ev_ms))
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([total_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * args.steps / (total_ms / 1e3)
    iters = [r["steps"] for r in results]
    ok = all(r["converged"] and r["max_force"] <= FMAX for r in results)

    # ---- e2e: host buffers in, host results out, through the C ABI -----------------
    e2e_ms = []
    h2d = N_PART * 8 * 4   # x, y, radii, masses
    d2h = N_PART * 8 * 3   # x, y, pe
    for k in range(args.warmup, n_sys):
        s, st, _ = systems[k]
        l2_flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.setState(st["x"], st["y"], np.zeros(N_PART), np.zeros(N_PART), st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, MAX_STEPS, fmax_target=FMAX)
        out = s.getState()
        _ = float(out["pe"].sum())
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = world * args.steps / (float(np.sum(e2e_ms)) / 1e3)

    # ---- roofline of the dominant kernel (forces + kick + reductions) --------
    peak, peak_src = measured_peak_hbm()
    s, st, arr = systems[-1]
    s.setState(arr["x"], arr["y"], None, None, arr["r"], arr["m"])
    s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
    prof = profile(dpg, s, kind=0, iters=400)
    k_mean = float(np.mean(s.getNeighbors()[1]))
    # algorithmic bytes per particle of k_fire_force: read pos 16, rad 8, count 4,
    # indices 4k, vel 16, mass 8; write frc 16, pe 8, vel 16 (neighbour data reused from cache)
    bytes_force = N_PART * (92 + 4 * k_mean)
    achieved = bytes_force / (prof["force_us"] * 1e-6) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": None, "kernel": "k_fire_force",
                "peak_source": peak_src, "bytes_per_launch": bytes_force,
                "launch_us": prof["force_us"],
                "note": "16384-disk working set (3 MB) is L2-resident; see roofline_large"}

    # ---- large-N force kernel (N = 2^20 NVE), where HBM bounds the kernel ----
    large = large_n_roofline(dpg, dev, sptr, peak)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        dt, steps, fmax = cpu_solve(seeds[args.warmup], threads)
        cpu = {"value": 1.0 / dt, "unit": "FIRE solves/s", "cores": threads, "kind": "port",
               "sample": f"1 full minimisation (seed {seeds[args.warmup]}, {steps} FIRE iterations) "
                         f"of the oracle restatement, OpenMP {threads} threads"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "FIRE solves/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": workload_config(),
                "roofline": roofline, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "FIRE solves/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clocks,
                "extra": {"fire_iterations_per_solve": float(np.mean(iters)),
                          "particle_steps_per_s": N_PART * float(np.sum(iters)) / (total_ms / 1e3),
                          "all_converged_to_fmax": ok,
                          "max_force": float(max(r["max_force"] for r in results)),
                          "wall_s_timed": t_wall, "profile_us_per_iter": prof,
                          "roofline_large": large}}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def profile(dpg, s, kind, iters, dt=1e-2):
    import ctypes as C
    avg = (C.c_double * 3)()
    cnt = (C.c_int64 * 3)()
    dpg.lib.check(s.lib.dpg_profile_loop(s.h, kind, iters, dt, avg, cnt))
    return {"move_us": avg[0], "rebuild_us": avg[1], "force_us": avg[2], "iters": cnt[0],
            "list_builds": cnt[1], "cell_builds": cnt[2]}


def large_n_roofline(dpg, dev, sptr, peak):
    """N = 2^20 polydisperse disks r ~ U[0.4, 0.6], phi = 0.84, NVE dt = 1e-2:
    per-kernel device time of the fused force + kick kernel (k_nve_second)."""
    from oracle.oracle import fill_normal, fill_uniform
    n = 1 << 20
    r = fill_uniform(n, 0.4, 0.6, 7 * n, 5)
    area = float(np.sum(r * r)) * np.pi
    L = (area / 0.84) ** 0.5
    x = fill_uniform(n, 0.0, L, 0, 5)
    y = fill_uniform(n, 0.0, L, n, 5)
    T = 1e-3
    vx = fill_normal(n, 0.0, np.sqrt(T), 2 * n, 5)
    vy = fill_normal(n, 0.0, np.sqrt(T), 3 * n, 5)
    vx -= vx.mean()
    vy -= vy.mean()
    s = dpg.Disk(n, L, stream=sptr)
    s.setState(x, y, vx, vy, r, np.ones(n))
    # rebuild at half-skin: sqrt(3) |dr| > disp_mult * r_c with |dr| = 0.15, r_c = 1.5
    info = s.setupNeighbors("cell", 1.5 / 1.2, 0.1732, 8.0, 0.5)
    prof = profile(dpg, s, kind=1, iters=200)
    k_mean = float(np.mean(s.getNeighbors()[1]))
    # k_nve_second per particle: read pos 16, rad 8, count 4, indices 4k, vel 16,
    # mass 8; write frc 16, pe 8, vel 16
    b = n * (92 + 4 * k_mean)
    ach = b / (prof["force_us"] * 1e-6) / 1e9
    step_us = prof["move_us"] + prof["rebuild_us"] + prof["force_us"]
    return {"workload": "NVE, N=2^20 polydisperse disks U[0.4,0.6], phi=0.84, dt=1e-2, T=1e-3",
            "kernel": "k_nve_second", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "bytes_per_launch": b, "launch_us": prof["force_us"],
            "mean_neighbors": k_mean, "profile_us_per_step": prof,
            "particle_steps_per_s_stream_launch": n / (step_us * 1e-6),
            "cutoff": info["cutoff"]}


def ncu_case(which):
    """Small fixed workloads for ncu captures (plain stream launches, a few
    hundred kernels): 'fire' = 64 FIRE iterations of the 16384-disk system,
    'nve_large' = 8 NVE steps of the 2^20-disk system."""
    os.environ["DPG_LOOP_MODE"] = "stream"
    import dpcuda_gb300 as dpg
    if which == "fire":
        st = packing(1)
        s = dpg.Disk(N_PART, st["box"])
        s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        r = dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 64, fmax_target=FMAX)
        print(json.dumps({"ncu_case": which, "steps": r["steps"]}))
    else:
        from oracle.oracle import fill_uniform
        n = 1 << 20
        r = fill_uniform(n, 0.4, 0.6, 7 * n, 5)
        L = (float(np.sum(r * r)) * np.pi / 0.84) ** 0.5
        s = dpg.Disk(n, L)
        s.setState(fill_uniform(n, 0.0, L, 0, 5), fill_uniform(n, 0.0, L, n, 5), None, None, r,
                   np.ones(n))
        s.setupNeighbors("cell", 1.5 / 1.2, 0.1732, 8.0, 0.5)
        s.nveSteps(1e-2, 8)
        print(json.dumps({"ncu_case": which, "steps": 8}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--ncu-case", choices=["fire", "nve_large"], default=None,
                    help="run a small fixed workload for ncu captures and exit")
    args = ap.parse_args()
    if args.ncu_case:
        ncu_case(args.ncu_case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
