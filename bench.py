"""Benchmark: FIRE minimisations of bidisperse disks, N = 16384, phi = 0.86, run
to max|F_i| <= 1e-13 (the 16384-disk FIRE workload): the mixed-precision
batched form against the plain FP64 drop-in, plus the per-kernel roofline and
the CPU baseline.

A solve is one complete FIRE minimisation of one seeded random packing (cell
list + neighbour list build, initial forces, then FIRE until max|F_i| <= 1e-13).
A step is one call of the batched form on 8 such systems (8 distinct seeds,
FP32 pair forces with FP64 accumulation, each system switching to the FP64
pair arithmetic below max|F| = 1e-7 for the final refinement).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default): the GB300 library through its C ABI.  `value` = solves/s
of the batched mixed form with the initial packings resident in HBM; `e2e` =
the same through host buffers (positions/radii/masses in, positions/forces
out).  The plain FP64 path (one system per call, bit-identical to the
reference arithmetic) is timed on the same starts and reported in
extra.plain_fp64.  L2 (126 MB) is flushed between timed solves (a 512 MiB
write).
--impl reference: the CPU restatement of the reference algorithm (the oracle,
oracle/dpg_oracle.c, FP64, OpenMP over all host cores) running full
minimisations of the same seeds, one per step.  Under torchrun (N > 1) each
rank solves its own seeds (independent replicas, weak scaling); only rank 0
runs the reference arm.
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
BATCH = 16                  # systems per step of the batched form
CUTOFF, SKIN = 1.7, 0.3     # neighbour cutoff d_max + skin, and the skin
TUNE_ITERS = 300            # FIRE iterations per autotuner candidate
FORM_CODES = {"grid": 1, "persist": 2}
SWITCH_FMAX = 1e-6          # mixed systems switch to FP64 pair forces below this max|F|
PLAIN_SOLVES = 2            # timed solves of the plain FP64 path (after one untimed)
WARMUP_ITERS = 2000         # FIRE iterations of a warm-up solve
E_FORCE_DRAM_PER_SYSTEM = 10.37e6 / 8  # ncu DRAM bytes per e_force launch per 16384-disk system
PROFILE_ITERS = 300


def step_seeds(rank, k):
    """Seeds of the BATCH systems of step k on this rank (every start distinct)."""
    return [100000 * rank + BATCH * k + b + 1 for b in range(BATCH)]


def reduce_max(x: float, device=None) -> float:
    """Max of x over the ranks of the default process group (x itself when
    not distributed): the job's time is its slowest rank's."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_config():
    return {"workload": "FIRE minimisation, bidisperse disks r=0.5/0.7 50:50, N=16384, "
                        "phi=0.86, periodic, to max|F|<=1e-13",
            "n_particles": N_PART, "packing_fraction": PHI, "fmax_target": FMAX,
            "fire": {"alpha0": FIRE_ALPHA0, "dt0": FIRE_DT0, "dt_max": 10 * FIRE_DT0,
                     "f_inc": 1.1, "f_dec": 0.5, "f_alpha": 0.99, "n_min": 5},
            "neighbors": {"method": "cell", "cutoff": "d_max + skin", "skin": "0.3, or the "
                          "autotuner's 0.225 / 0.15 (extra.autotune)", "particles_per_cell": 8},
            "form": f"mixed precision (FP32 pairs, FP64 accumulation, FP64 pair refinement "
                    f"below max|F| = {SWITCH_FMAX:g}), {BATCH} systems per step",
            "l2": "flushed between steps (512 MiB write)",
            "warmup_kind": f"bounded solves of {WARMUP_ITERS} FIRE iterations over the timed batches",
            "e2e_steps": "the same batches as the timed steps, solved again from host arrays",
            "seeds": f"step k on rank r: 100000*r + {BATCH}*k + 1 .. + {BATCH}"}


def packing(seed):
    from dpcuda_gb300.init import disk_packing  # the reference's RandomUniform stream
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
        dt, steps, fmax = cpu_solve(step_seeds(0, args.warmup + k)[0], threads)
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
                             "sample": f"{args.steps} full minimisations (the first start of each "
                                       f"timed step) of the oracle restatement (FP64), OpenMP "
                                       f"{threads} threads"},
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

    def max_over_ranks(x):
        return reduce_max(x, dev)

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def l2_flush():
        with torch.cuda.stream(stream):
            flush.fill_(1.0)

    def timed(fn):
        l2_flush()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1)

    # ---- inputs of every timed step, resident in HBM before the timed region --
    # (step k >= warmup uses the seeds of step k, so the reference arm, which
    # solves the first start of each timed step, sees the same starts)
    # the autotuner picks the execution form, block size and skin on the first
    # timed step's starts (FIRE iterations from those starts, positions
    # restored), before anything is timed
    tune_sts = [packing(sd) for sd in step_seeds(rank, args.warmup)]
    te = dpg.Ensemble([N_PART] * BATCH, [st["box"] for st in tune_sts], CUTOFF, SKIN,
                      precision=dpg.MIXED, switch_fmax=SWITCH_FMAX, stream=sptr)
    te.setState(*[np.concatenate([st[c] for st in tune_sts]) for c in ("x", "y", "r", "m")])
    tune = te.autotune(TUNE_ITERS)
    te.close()
    skin = tune["skin"]
    form = FORM_CODES[tune["form"]]
    batches = []
    for k in range(args.warmup, args.warmup + args.steps):
        sts = [packing(sd) for sd in step_seeds(rank, k)]
        e = dpg.Ensemble([N_PART] * BATCH, [st["box"] for st in sts], CUTOFF - (SKIN - skin), skin,
                         precision=dpg.MIXED, switch_fmax=SWITCH_FMAX, stream=sptr)
        e.setForm(form, tune["threads"])
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
        batches.append((e, sts))
    torch.cuda.synchronize()

    def solve_batch(e, max_steps=MAX_STEPS):
        return e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, max_steps, fmax_target=FMAX)

    # warm-up: W bounded solves (WARMUP_ITERS FIRE iterations each), cycling over
    # the timed batches so that every batch has built its CUDA graph, then the
    # initial states are put back
    for k in range(max(args.warmup, len(batches))):
        solve_batch(batches[k % len(batches)][0], WARMUP_ITERS)
    for e, sts in batches:
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
    torch.cuda.synchronize()

    # ---- headline: mixed precision, BATCH systems per step --------------------
    sampler = ClockSampler(dev.index or 0)
    results, ev_ms, launches = [], [], 0
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_wall0 = time.perf_counter()
    for e, _ in batches:
        res, ms = timed(lambda: solve_batch(e))
        ev_ms.append(ms)
        results.append(res)
        iters = max(r["fire_steps"] for r in res)
        if form == FORM_CODES["persist"]:
            # one persistent launch per 2^17 iterations
            launches += 1 + iters // (1 << 17)
        else:
            # kernels per iteration of the graph loop: move, force, transition,
            # guard; 5 rebuild kernels on iterations where any system rebuilt
            launches += 4 * (iters + 1) + 5 * max(r["rebuilds"] for r in res)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    barrier()
    clocks = sampler.stop()
    total_ms = max_over_ranks(float(np.sum(ev_ms)))
    value = world * args.steps * BATCH / (total_ms / 1e3)
    flat = [r for res in results for r in res]
    ok = all(r["converged"] and r["max_force"] <= FMAX for r in flat)

    # ---- e2e: host arrays in, host positions/forces out, through the C ABI ---
    e2e_ms = []
    h2d = BATCH * N_PART * 8 * 4   # x, y, radii, masses
    d2h = BATCH * N_PART * 8 * 4   # x, y, fx, fy
    n_e2e = len(batches)
    e2e_results = []
    for e, sts in batches:
        host = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
        l2_flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.setState(*host)
        e2e_results.append(solve_batch(e))
        out = e.getState()
        _ = float(np.abs(out["fx"]).max())
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = world * n_e2e * BATCH / (max_over_ranks(float(np.sum(e2e_ms))) / 1e3)

    # ---- the plain FP64 drop-in on the same systems (one per call) -----------
    plain = plain_fp64_leg(dpg, sptr, batches[0][1][:PLAIN_SOLVES + 1], timed)

    # ---- error of the mixed form: its minima re-evaluated by the FP64 path ----
    # (the FP64 path is bit-identical to the reference arithmetic; the two forms
    # reach different minima from the same start, so the check is done at the
    # mixed form's own final positions)
    e, sts = batches[0]
    fin = e.getState()
    checks, off = [], 0
    for k, st in enumerate(sts[:4]):
        xs, ys = fin["x"][off:off + N_PART], fin["y"][off:off + N_PART]
        off += N_PART
        d = dpg.Disk(N_PART, st["box"], stream=sptr)
        d.setState(xs, ys, None, None, st["r"], st["m"])
        d.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        d.zeroForceAndPotentialEnergy()
        d.calculateForces()
        g = d.getState()
        f64 = float(np.sqrt(g["fx"] ** 2 + g["fy"] ** 2).max())
        pe64 = d.totalPotentialEnergy() / N_PART
        r = e2e_results[0][k]  # the last solve of this batch
        checks.append({"max_force_fp64": f64, "max_force_reported": r["max_force"],
                       "avg_pe_fp64": pe64, "avg_pe_reported": r["avg_pe"],
                       "avg_pe_rel_diff": abs(r["avg_pe"] - pe64) / pe64})
        d.close()
    mixed_check = {"systems": len(checks), "max_force_fp64_max": max(c["max_force_fp64"] for c in checks),
                   "avg_pe_rel_diff_max": max(c["avg_pe_rel_diff"] for c in checks), "detail": checks}

    # ---- roofline of the dominant kernel of the headline form ----------------
    peak, peak_src = measured_peak_hbm()
    e, sts = batches[-1]
    e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
    prof = e.profileLoop(PROFILE_ITERS, FIRE_ALPHA0, FIRE_DT0, FMAX)
    k_mean = plain["mean_neighbors"]
    # e_force (mixed phase) per particle: read pk[i] 16, count 4, neighbour
    # indices 4k, vel 16, mass 8; write frc 16, pe 8, vel 16 (neighbours' pk
    # gathered from cache) -> 84 + 4k
    bytes_force = BATCH * N_PART * (84 + 4 * k_mean)
    achieved = bytes_force / (prof["force_us"] * 1e-6) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": E_FORCE_DRAM_PER_SYSTEM * BATCH,
                "traffic_source": "ncu dram__bytes_read+write of one FP32-phase e_force launch on "
                                  "8 x 16384 disks (10.37 MB), scaled to the batch by systems",
                "kernel": "e_force",
                "peak_source": peak_src, "bytes_per_launch": bytes_force,
                "launch_us": prof["force_us"], "profile_us_per_iter": prof,
                "note": f"{BATCH} x 16384 disks, first {PROFILE_ITERS} FIRE iterations (FP32 pair "
                        f"phase); the working set ({BATCH * 16384 * 200 / 1e6:.0f} MB) is L2-resident, "
                        "so the kernel is bound by latency and the FP64 pipe, not by HBM"}

    # ---- large-N force kernel (N = 2^20 NVE, plain FP64) -----------------------
    large = large_n_roofline(dpg, dev, sptr, peak)
    others = other_configs(dpg, sptr)

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sd = step_seeds(rank, args.warmup)[0]
        dt, steps, fmax = cpu_solve(sd, threads)
        cpu = {"value": 1.0 / dt, "unit": "FIRE solves/s", "cores": threads, "kind": "port",
               "sample": f"1 full minimisation (seed {sd}, {steps} FIRE iterations) of the "
                         f"oracle restatement (FP64), OpenMP {threads} threads"}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "FIRE solves/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32+f64", "data": "synthetic", "config": workload_config(),
                "roofline": roofline, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "FIRE solves/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": launches, "clocks": clocks,
                "extra": {"form": "mixed+batched", "systems_per_step": BATCH,
                          "fire_iterations_per_solve": float(np.mean([r["fire_steps"] for r in flat])),
                          "particle_steps_per_s": N_PART * float(sum(r["fire_steps"] for r in flat))
                          / (total_ms / 1e3),
                          "all_converged_to_fmax": ok,
                          "max_force": float(max(r["max_force"] for r in flat)),
                          "wall_s_timed": t_wall,
                          "plain_fp64": plain,
                          "mixed_minima_checked_in_fp64": mixed_check,
                          "mixed_batched_over_plain_fp64": value / plain["value"],
                          "roofline_large": large, "other_workloads": others,
                          "autotune": {"chosen": {"form": tune["form"], "threads": tune["threads"],
                                                  "skin": tune["skin"]},
                                       "iters_per_candidate": TUNE_ITERS,
                                       "particle_iterations_per_s": tune["candidates"]}}}
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def plain_fp64_leg(dpg, sptr, sts, timed):
    """The drop-in FP64 path (bit-identical to the reference arithmetic): one
    system per call, first start untimed (warm-up), the rest timed."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {"solves": 0, "ms": [], "fire_iterations": [], "avg_pe": [], "max_force": []}
    for k, st in enumerate(sts):
        s = dpg.Disk(N_PART, st["box"], stream=sptr)
        arr = {c: torch.from_numpy(st[c]).to(dev) for c in ("x", "y", "r", "m")}
        torch.cuda.synchronize()

        def solve():
            s.setState(arr["x"], arr["y"], None, None, arr["r"], arr["m"])
            s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
            return dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, MAX_STEPS, fmax_target=FMAX)

        r, ms = timed(solve)
        if k == 0:
            s.setState(arr["x"], arr["y"], None, None, arr["r"], arr["m"])
            s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
            out["mean_neighbors"] = float(np.mean(s.getNeighbors()[1]))
            s.close()
            continue
        out["solves"] += 1
        out["ms"].append(ms)
        out["fire_iterations"].append(r["steps"])
        out["avg_pe"].append(s.totalPotentialEnergy() / N_PART)
        out["max_force"].append(r["max_force"])
        s.close()
    out["value"] = out["solves"] / (float(np.sum(out["ms"])) / 1e3)
    out["unit"] = "FIRE solves/s"
    out["dtype"] = "f64"
    out["force_group"] = "threads per particle chosen by the library (8 at N=16384)"
    return out


def other_configs(dpg, sptr):
    """Throughput of the other workloads, FP64 drop-in vs mixed form, each timed
    with CUDA events around one device-resident loop call:
    - NVE of 1024 bidisperse disks at phi 0.80 (T 1e-4, dt 1e-2, 10^4 steps);
    - NVE of 4096 rigid bumpy bodies (20 / 28 vertices, phi 0.80, dt 5e-3,
      T 1e-4, 10^3 steps)."""
    import torch
    from dpcuda_gb300.init import bumpy_packing, disk_packing
    stream = torch.cuda.ExternalStream(sptr)
    out = {}

    def time_call(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / 1e3

    rng = np.random.default_rng(1)
    st = disk_packing(1024, 0.80, 1)
    vx, vy = rng.normal(0, 1e-2, 1024), rng.normal(0, 1e-2, 1024)
    vx -= vx.mean()
    vy -= vy.mean()
    for form, prec in (("fp64", dpg.FP64), ("mixed", dpg.MIXED)):
        s = dpg.Disk(1024, st["box"], stream=sptr, precision=prec)
        s.setState(st["x"], st["y"], vx, vy, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        s.nveSteps(1e-2, 100)
        sec = time_call(lambda: s.nveSteps(1e-2, 10000))
        out[f"nve_1024_{form}_particle_steps_per_s"] = 1024 * 10000 / sec
        s.close()
    b = bumpy_packing(4096, 0.80, 3)
    bv = rng.normal(0, 1e-2, (2, 4096))
    bv -= bv.mean(axis=1, keepdims=True)
    for form, prec in (("fp64", 0), ("mixed", 1)):
        r = dpg.RigidBumpy(4096, b["nv"], b["box"], b["e_c"], 2.0, b["rv"], b["seg"], True,
                           stream=sptr, precision=prec)
        r.setBodies(b["x"], b["y"], b["th"], b["r"], b["nvb"], bv[0], bv[1])
        r.setMass(1.0)
        r.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
        r.nveSteps(5e-3, 20)
        sec = time_call(lambda: r.nveSteps(5e-3, 1000))
        out[f"bumpy_nve_4096_{form}_body_steps_per_s"] = 4096 * 1000 / sec
        r.close()
    return out


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
    from dpcuda_gb300.init import random_uniform
    n = 1 << 20
    r = random_uniform(n, 0.4, 0.6, 7 * n, 5)
    area = float(np.sum(r * r)) * np.pi
    L = (area / 0.84) ** 0.5
    x = random_uniform(n, 0.0, L, 0, 5)
    y = random_uniform(n, 0.0, L, n, 5)
    T = 1e-3
    rng = np.random.default_rng(5)
    vx = rng.normal(0.0, np.sqrt(T), n)
    vy = rng.normal(0.0, np.sqrt(T), n)
    vx -= vx.mean()
    vy -= vy.mean()
    out = {"workload": "NVE, N=2^20 polydisperse disks U[0.4,0.6], phi=0.84, dt=1e-2, T=1e-3",
           "kernel": "k_nve_second", "peak": peak, "unit": "GB/s"}
    for form, prec in (("fp64", dpg.FP64), ("mixed", dpg.MIXED)):
        s = dpg.Disk(n, L, stream=sptr, precision=prec)
        s.setState(x, y, vx, vy, r, np.ones(n))
        # rebuild at half-skin: sqrt(3) |dr| > disp_mult * r_c with |dr| = 0.15, r_c = 1.5
        info = s.setupNeighbors("cell", 1.5 / 1.2, 0.1732, 8.0, 0.5)
        prof = profile(dpg, s, kind=1, iters=200)
        k_mean = float(np.mean(s.getNeighbors()[1]))
        # k_nve_second per particle: read count 4, indices 4k, vel 16, mass 8;
        # write frc 16, pe 8, vel 16; plus pos 16 + rad 8 (FP64) or the packed
        # offsets 16 (mixed)
        b = n * ((92 if form == "fp64" else 84) + 4 * k_mean)
        ach = b / (prof["force_us"] * 1e-6) / 1e9
        step_us = prof["move_us"] + prof["rebuild_us"] + prof["force_us"]
        out[form] = {"achieved": ach, "frac": ach / peak, "bytes_per_launch": b,
                     "launch_us": prof["force_us"], "mean_neighbors": k_mean,
                     "profile_us_per_step": prof,
                     "particle_steps_per_s_stream_launch": n / (step_us * 1e-6),
                     "cutoff": info["cutoff"]}
        s.close()
    return out


def jam_ensemble(args):
    """The batched jamming workload (not the default line): S bidisperse
    systems with N drawn log-uniformly in [64, 4096] from a seed, each
    starting at phi = 0.80, compressed by box scaling with a FIRE
    minimisation (the reference's minimizeFire defaults: PE targets 1e-16,
    at most 1e5 steps) after each step and bisected on the box length until
    the pressure is 1e-7 +- 1e-9 (scripts/runArthurJamWithFire.cpp flow).
    Prints one JSON line: systems jammed per second for the mixed and FP64
    ensembles and |phi_J(mixed) - phi_J(FP64)| over the systems."""
    import dpcuda_gb300 as dpg
    from dpcuda_gb300.init import disk_packing
    S = args.jam_systems
    rng = np.random.default_rng(2024)
    sizes = np.floor(np.exp(rng.uniform(np.log(64), np.log(4096), S))).astype(int)
    sts = [disk_packing(int(n), 0.80, 7000 + k) for k, n in enumerate(sizes)]
    cat = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
    band = (args.jam_pressure * 0.99, args.jam_pressure * 1.01)
    fire = (0.1, 1e-2, 1e-16, 1e-16, 100000, 0.0)
    print(json.dumps({"jam_sizes": [int(n) for n in sizes]}), file=sys.stderr, flush=True)
    out = {}
    for form, prec in (("mixed", dpg.MIXED), ("fp64", dpg.FP64)):
        e = dpg.Ensemble(sizes, [st["box"] for st in sts], CUTOFF, SKIN, precision=prec,
                         switch_fmax=SWITCH_FMAX)
        e.setState(*cat)
        t0 = time.perf_counter()
        res = e.jam(*band, compression_rate=0.99, length_tolerance=1e-10, decompress_factor=1.01,
                    max_compression_steps=args.jam_max_compressions, fire=fire)
        dt = time.perf_counter() - t0
        out[form] = {"s": dt, "systems_per_s": S / dt,
                     "phi": [r["packing_fraction"] for r in res],
                     "in_band": int(sum(band[0] <= r["pressure"] <= band[1] for r in res)),
                     "status": [r["status"] for r in res],
                     "fire_steps_max": int(max(r["fire_steps"] for r in res)),
                     "minimizations_max": int(max(r["minimizations"] for r in res))}
        print(json.dumps({"jam_form": form, "s": dt, "systems_per_s": S / dt,
                          "in_band": out[form]["in_band"]}), file=sys.stderr, flush=True)
        e.close()
    d = np.abs(np.array(out["mixed"]["phi"]) - np.array(out["fp64"]["phi"]))
    line = {"metric": "batched jamming: systems jammed/s, mixed vs FP64", "unit": "systems/s",
            "value": out["mixed"]["systems_per_s"], "n_gpus": 1, "higher_is_better": True,
            "config": {"workload": f"{S} systems, N log-uniform [64, 4096], phi0 0.80, "
                                   f"P = {args.jam_pressure:g} +- 1%, FIRE 1e-16/1e-16/1e5",
                       "sizes_sum": int(sizes.sum())},
            "fp64_systems_per_s": out["fp64"]["systems_per_s"],
            "dphi_J": {"median": float(np.median(d)), "max": float(d.max()),
                       "frac_below_1e-6": float(np.mean(d <= 1e-6))},
            "detail": out}
    print(json.dumps(line), flush=True)


def fire_ensemble(args):
    """Batched FIRE on an uneven ensemble (not the default line): S bidisperse
    systems with N drawn log-uniformly in [64, 4096] from a seed, phi 0.86,
    seeded random starts, minimised to max|F| <= 1e-13 in the mixed and the
    FP64 batched forms (one untimed 50-iteration call first builds the graph),
    then the plain FP64 drop-in one system per call on the first systems until
    30 s have passed.  Prints one JSON line per form."""
    import dpcuda_gb300 as dpg
    from dpcuda_gb300.init import disk_packing
    S = args.fire_systems
    rng = np.random.default_rng(2024)
    sizes = np.floor(np.exp(rng.uniform(np.log(64), np.log(4096), S))).astype(int)
    sts = [disk_packing(int(n), PHI, 9000 + k) for k, n in enumerate(sizes)]
    cat = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
    for name, prec in (("mixed", dpg.MIXED), ("fp64", dpg.FP64)):
        e = dpg.Ensemble(sizes, [st["box"] for st in sts], CUTOFF, SKIN, precision=prec,
                         switch_fmax=SWITCH_FMAX)
        e.setState(*cat)
        e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 50, fmax_target=FMAX)
        e.setState(*cat)
        t0 = time.perf_counter()
        r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 10**6, fmax_target=FMAX)
        dt = time.perf_counter() - t0
        print(json.dumps({"metric": "batched FIRE solves/s, uneven ensemble", "form": name,
                          "systems": S, "particles": int(sizes.sum()), "s": dt,
                          "systems_per_s": S / dt,
                          "converged": int(sum(x["converged"] for x in r)),
                          "max_force": max(x["max_force"] for x in r),
                          "fire_steps_max": int(max(x["fire_steps"] for x in r))}), flush=True)
        e.close()
    # the plain FP64 drop-in, one system per call, on the ensemble's systems in
    # order until 30 s of solving have passed (a sample of the same workload)
    done, t_tot, n_tot = 0, 0.0, 0
    for k in range(S):
        st = sts[k]
        s = dpg.Disk(int(sizes[k]), st["box"])
        s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        t0 = time.perf_counter()
        dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 10**6, fmax_target=FMAX)
        s.synchronize()
        t_tot += time.perf_counter() - t0
        n_tot += int(sizes[k])
        done += 1
        s.close()
        if t_tot > 30:
            break
    print(json.dumps({"metric": "batched FIRE solves/s, uneven ensemble", "form": "plain_fp64",
                      "systems": done, "particles": n_tot, "s": t_tot,
                      "systems_per_s": done / t_tot,
                      "sample": f"the first {done} of the {S} systems, one per call"}), flush=True)


def ncu_case(which):
    """Small fixed workloads for ncu captures (plain stream launches, a few
    hundred kernels): 'fire' = 64 FIRE iterations of the 16384-disk system,
    'nve_large' = 8 NVE steps of the 2^20-disk system, 'ensemble' = 64 FIRE
    iterations of the batched mixed form on 8 x 16384 disks, 'bumpy_nve' = 192
    NVE steps of 4096 rigid bumpy bodies."""
    os.environ["DPG_LOOP_MODE"] = "stream"
    import dpcuda_gb300 as dpg
    if which == "bumpy_nve":
        # NVE of 4096 rigid bumpy bodies (FP64): 64 steps, then 128 steps
        from dpcuda_gb300.init import bumpy_packing
        b = bumpy_packing(4096, 0.80, 3)
        bv = np.random.default_rng(1).normal(0, 1e-2, (2, 4096))
        bv -= bv.mean(axis=1, keepdims=True)
        r = dpg.RigidBumpy(4096, b["nv"], b["box"], b["e_c"], 2.0, b["rv"], b["seg"], True,
                           precision=0)
        r.setBodies(b["x"], b["y"], b["th"], b["r"], b["nvb"], bv[0], bv[1])
        r.setMass(1.0)
        r.setupNeighbors("cell", 1.5, 0.2, 8.0, 0.5)
        r.nveSteps(5e-3, 64)
        r.nveSteps(5e-3, 128)
        print(json.dumps({"ncu_case": which, "n_rebuilds": r.neighborInfo()["n_rebuilds"]}))
        return
    if which == "ensemble_forces":
        # one force pass per arithmetic (FP32, double-word, FP64) on 8 x 16384 disks
        from dpcuda_gb300.ensemble import DWORD
        sts = [packing(sd) for sd in step_seeds(0, 0)[:8]]
        e = dpg.Ensemble([N_PART] * 8, [st["box"] for st in sts], CUTOFF, SKIN,
                         precision=dpg.MIXED, switch_fmax=SWITCH_FMAX)
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
        for prec in (dpg.MIXED, DWORD, dpg.FP64, dpg.MIXED, DWORD, dpg.FP64):
            e.calculateForces(prec)
        print(json.dumps({"ncu_case": which, "passes": 6}))
        return
    if which == "ensemble":
        sts = [packing(sd) for sd in step_seeds(0, 0)]
        e = dpg.Ensemble([N_PART] * BATCH, [st["box"] for st in sts], CUTOFF, SKIN,
                         precision=dpg.MIXED, switch_fmax=SWITCH_FMAX)
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
        r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 64, fmax_target=FMAX)
        print(json.dumps({"ncu_case": which, "steps": max(x["fire_steps"] for x in r)}))
        return
    if which == "fire":
        st = packing(1)
        s = dpg.Disk(N_PART, st["box"])
        s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        r = dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 64, fmax_target=FMAX)
        print(json.dumps({"ncu_case": which, "steps": r["steps"]}))
    else:
        from dpcuda_gb300.init import random_uniform
        n = 1 << 20
        r = random_uniform(n, 0.4, 0.6, 7 * n, 5)
        L = (float(np.sum(r * r)) * np.pi / 0.84) ** 0.5
        s = dpg.Disk(n, L)
        s.setState(random_uniform(n, 0.0, L, 0, 5), random_uniform(n, 0.0, L, n, 5), None, None, r,
                   np.ones(n))
        s.setupNeighbors("cell", 1.5 / 1.2, 0.1732, 8.0, 0.5)
        s.nveSteps(1e-2, 8)
        print(json.dumps({"ncu_case": which, "steps": 8}))


def main():
    global BATCH
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--ncu-case", choices=["fire", "nve_large", "ensemble", "ensemble_forces",
                                           "bumpy_nve"],
                    default=None,
                    help="run a small fixed workload for ncu captures and exit")
    ap.add_argument("--batch", type=int, default=BATCH, help="systems per step of the batched form")
    ap.add_argument("--jam-ensemble", action="store_true",
                    help="run the batched jamming workload instead of the default line")
    ap.add_argument("--jam-systems", type=int, default=256)
    ap.add_argument("--jam-max-compressions", type=int, default=2000)
    ap.add_argument("--jam-pressure", type=float, default=1e-7,
                    help="target pressure of the batched jamming leg (band +-1%%)")
    ap.add_argument("--fire-ensemble", action="store_true",
                    help="run batched FIRE on an uneven ensemble instead of the default line")
    ap.add_argument("--fire-systems", type=int, default=256)
    args = ap.parse_args()
    BATCH = args.batch
    if args.jam_ensemble:
        jam_ensemble(args)
        return
    if args.fire_ensemble:
        fire_ensemble(args)
        return
    if args.ncu_case:
        ncu_case(args.ncu_case)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
