"""Benchmark: FIRE minimisations of bidisperse disks, N = 16384, phi = 0.86, run
to max|F_i| <= 1e-13 (the 16384-disk FIRE workload): the mixed-precision
batched form against the plain FP64 drop-in and the batched FP64 form, with the
per-kernel roofline, the CPU baseline and the batched jamming workload.

A solve is one complete FIRE minimisation of one seeded random packing (cell
list + neighbour list build, initial forces, then FIRE until max|F_i| <= 1e-13).
A step is one call of the batched form on BATCH = 16 such systems (16 distinct
seeds, FP32 pair forces below which each system refines in double-word FP32
pairs; FP64 pair arithmetic certifies every reported minimum).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default): the GB300 library through its C ABI.  `value` = solves/s
of the batched mixed form with the initial packings resident in HBM; `e2e` =
the first timed batches again through host buffers (positions/radii/masses in,
positions/forces out).  extra: the plain FP64 path (one system per call,
bit-identical to the reference arithmetic) and the batched FP64 form on the
same starts, every mixed minimum re-checked by the FP64 drop-in, the jamming
ensemble (pressure-band protocol on 64 systems of 64-4096 disks).  L2 (126 MB)
is flushed between timed solves (a 512 MiB write).  Progress goes to stderr.
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
FORM_CODES = {"grid": 1, "persist": 2, "resident": 3}
SWITCH_FMAX = 1e-6          # mixed systems switch to FP64 pair forces below this max|F|
PLAIN_SOLVES = 8            # timed solves of the plain FP64 path (after one untimed)
E2E_BATCHES = 4             # timed batches solved again through host arrays (e2e)
# jamming leg of the default run: 64 systems drawn as the 256-system workload
# draws them, at P = 1e-4 (at 1e-7 single systems need 1e7-1e8 FIRE iterations
# and the ensemble takes tens of minutes; bench.py --jam-ensemble --jam-systems
# 256 --jam-pressure 1e-7 runs it)
JAM_SYSTEMS = 64
JAM_PRESSURE = 1e-4
JAM_PLAIN_BUDGET_S = 60.0
JAM_FIRE = (0.1, 1e-2, 1e-16, 0.0, 100000, 1e-13)  # alpha0, dt0, PE/N target, no PE-change test,
                                                   # at most 1e5 iterations, max|F| target
JAM_CHECK_STEPS = 20000     # FP64 re-minimisation of a jammed state (already a minimum)
WARMUP_ITERS = 2000         # FIRE iterations of a warm-up solve
E_FORCE_DRAM_PER_SYSTEM = 10.37e6 / 8  # ncu DRAM bytes per e_force launch per 16384-disk system
# ncu DRAM bytes (read + write) per disk of one e_res launch (a time slice of
# a few thousand iterations): the kernel loads and stores each system's state
# once per launch, so its traffic grows with the disks, not the iterations
E_RES_DRAM_PER_DISK = (4019456 + 39680) / (2 * 16384)
PROFILE_ITERS = 300


_T0 = time.perf_counter()


def log(msg):
    """Progress on stderr (the JSON line is the only stdout output)."""
    print(f"[bench {time.perf_counter() - _T0:8.1f} s] {msg}", file=sys.stderr, flush=True)


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
            "form": f"mixed precision, {BATCH} systems per step, the execution form the "
                    f"autotuner picks (extra.autotune): resident form = FP32 pairs, then "
                    f"double-word FP32 pairs below max|F| = {SWITCH_FMAX:g}, FP64 passes only "
                    f"to certify a minimum and to measure it; grid form = FP32 pairs, then "
                    f"double-word / FP64 pairs below the same max|F|",
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
    log("autotune done")
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

    log("warm-up done, headline")
    # ---- headline: mixed precision, BATCH systems per step --------------------
    sampler = ClockSampler(dev.index or 0)
    results, ev_ms = [], []
    launches0, graph_kernels = sum(e.launchCount() for e, _ in batches), 0
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_wall0 = time.perf_counter()
    for e, _ in batches:
        res, ms = timed(lambda: solve_batch(e))
        ev_ms.append(ms)
        results.append(res)
        if form == FORM_CODES["grid"]:
            # the graph loop runs its kernels on the device: move, force, its
            # epilogue, transition (at most) and guard every iteration, 5
            # rebuild kernels on the iterations where any system rebuilt
            iters = max(r["fire_steps"] for r in res)
            graph_kernels += 5 * (iters + 1) + 5 * max(r["rebuilds"] for r in res)
    torch.cuda.synchronize()
    # the library's own count of the launches it issued (stream and cluster
    # launches; a graph launch counts once, its kernels are added above)
    launches = sum(e.launchCount() for e, _ in batches) - launches0 + graph_kernels
    t_wall = time.perf_counter() - t_wall0
    barrier()
    clocks = sampler.stop()
    total_ms = max_over_ranks(float(np.sum(ev_ms)))
    value = world * args.steps * BATCH / (total_ms / 1e3)
    flat = [r for res in results for r in res]
    ok = all(r["converged"] and r["max_force"] <= FMAX for r in flat)
    finals = [e.getState() for e, _ in batches]   # after the timed region

    log("headline done, e2e")
    # ---- e2e: host arrays in, host positions/forces out, through the C ABI, on
    # the first E2E_BATCHES timed batches (the same starts, solved again) --------
    e2e_ms = []
    h2d = BATCH * N_PART * 8 * 4   # x, y, radii, masses
    d2h = BATCH * N_PART * 8 * 4   # x, y, fx, fy
    e2e_batches = batches[:min(len(batches), E2E_BATCHES)]
    for e, sts in e2e_batches:
        host = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
        l2_flush()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.setState(*host)
        solve_batch(e)
        out = e.getState()
        _ = float(np.abs(out["fx"]).max())
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = world * len(e2e_batches) * BATCH / (max_over_ranks(float(np.sum(e2e_ms))) / 1e3)

    log("plain FP64 and batched FP64")
    # ---- the plain FP64 drop-in on the first PLAIN_SOLVES starts (one per call)
    # and the batched FP64 form on the same starts -----------------------------
    plain = plain_fp64_leg(dpg, sptr, batches[0][1][:PLAIN_SOLVES + 1], timed)
    batched64 = batched_fp64_leg(dpg, sptr, batches[0][1][1:PLAIN_SOLVES + 1], timed)

    log("FP64 re-check of the mixed minima")
    # ---- error of the mixed form: every timed minimum re-evaluated by the FP64
    # drop-in (bit-identical to the reference arithmetic; the forms reach
    # different minima from the same start, so the check is at the mixed form's
    # own final positions) ---------------------------------------------------------
    mixed_check = fp64_recheck(dpg, sptr, batches, finals, results)

    log("roofline")
    # ---- roofline of the dominant kernel of the headline form: the resident
    # kernel over the timed solves, or the grid form's e_force weighted over the
    # three arithmetics by the share of force passes each took (measured in
    # either case: the grid form's figure explains the resident form's gain) ---
    peak, peak_src = measured_peak_hbm()
    grid_roofline = headline_roofline(dpg, sptr, batches, finals, flat, plain["mean_neighbors"],
                                      peak, peak_src, tune)
    if form == FORM_CODES["resident"]:
        roofline = resident_roofline(results, total_ms / world, launches,
                                     plain["mean_neighbors"], peak, peak_src)
        roofline["grid_form_e_force"] = grid_roofline
    else:
        roofline = grid_roofline

    log("large-N and other workloads")
    # ---- large-N force kernel (N = 2^20 NVE, plain FP64) -----------------------
    large = large_n_roofline(dpg, dev, sptr, peak)
    fma = fma_peaks(dpg)
    # the FP64 force + kick kernel is bound by the FP64 pipe (ncu: pipe
    # utilisation in profiles/); its denominator is the measured DFMA rate
    large["fp64"]["fp64_pipe"] = {"peak_tflops": fma["fp64"]["tflops"], "peak_source":
                                  "dpg_measure_fma_peak (measured DFMA rate)"}
    others = other_configs(dpg, sptr)

    log("jamming leg")
    # ---- the jamming ensemble (256 uneven systems, pressure band) ---------------
    jam = None if args.no_jam else jam_leg(dpg, args.jam_systems, args.jam_pressure,
                                           JAM_PLAIN_BUDGET_S)

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
                        "d2h_bytes_per_step": d2h,
                        "sample": f"the first {len(e2e_batches)} timed batches, solved again "
                                  "from host arrays"},
                "gpu_launches": launches, "clocks": clocks,
                "extra": {"form": "mixed+batched", "systems_per_step": BATCH,
                          "fire_iterations_per_solve": float(np.mean([r["fire_steps"] for r in flat])),
                          "particle_steps_per_s": N_PART * float(sum(r["fire_steps"] for r in flat))
                          / (total_ms / 1e3),
                          "all_converged_to_fmax": ok,
                          "max_force": float(max(r["max_force"] for r in flat)),
                          "wall_s_timed": t_wall,
                          "plain_fp64": plain,
                          "batched_fp64": batched64,
                          "mixed_minima_checked_in_fp64": mixed_check,
                          "mixed_batched_over_plain_fp64": value / plain["value"],
                          "mixed_batched_over_batched_fp64": value / batched64["value"],
                          "jam_ensemble": jam,
                          "roofline_large": large, "other_workloads": others,
                          "fma_peaks_measured": fma,
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
    system per call, first start untimed (warm-up), the rest timed.  Every
    timed solve must converge to FMAX (the minimizeFire result's converged flag
    and its FP64 max|F|)."""
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    out = {"solves": 0, "ms": [], "fire_iterations": [], "avg_pe": [], "max_force": [],
           "converged": []}
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
        out["converged"].append(bool(r["converged"]) and r["max_force"] <= FMAX)
        s.close()
    rates = 1e3 / np.array(out["ms"])
    out["value"] = out["solves"] / (float(np.sum(out["ms"])) / 1e3)
    out["solves_per_s_per_solve"] = {"mean": float(rates.mean()), "min": float(rates.min()),
                                     "max": float(rates.max())}
    out["fire_iterations_stats"] = {"mean": float(np.mean(out["fire_iterations"])),
                                    "min": int(np.min(out["fire_iterations"])),
                                    "max": int(np.max(out["fire_iterations"]))}
    out["all_converged"] = all(out["converged"])
    out["unit"] = "FIRE solves/s"
    out["dtype"] = "f64"
    out["force_group"] = "threads per particle chosen by the library (8 at N=16384)"
    return out


def batched_fp64_leg(dpg, sptr, sts, timed):
    """The batched form in FP64 pair arithmetic on the starts the plain leg timed
    (one call for all of them): the batching part of the headline's gain,
    apart from the precision part.  The grid form: at 16384 disks its FP64 pass
    spreads over every SM (measured 0.387 solves/s for 8 systems), while the
    resident form runs a system's FP64 pairs on its own 8-block cluster (0.219)."""
    from dpcuda_gb300.ensemble import FORM_GRID
    n = len(sts)
    e = dpg.Ensemble([N_PART] * n, [st["box"] for st in sts], CUTOFF, SKIN,
                     precision=dpg.FP64, stream=sptr)
    e.setForm(FORM_GRID)
    host = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
    e.setState(*host)
    e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 200, fmax_target=FMAX)   # graph build
    e.setState(*host)
    res, ms = timed(lambda: e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, MAX_STEPS,
                                           fmax_target=FMAX))
    e.close()
    return {"value": n / (ms / 1e3), "unit": "FIRE solves/s", "systems": n, "dtype": "f64",
            "form": "grid",
            "all_converged": all(r["converged"] and r["max_force"] <= FMAX for r in res),
            "fire_iterations_mean": float(np.mean([r["fire_steps"] for r in res])),
            "sample": "the starts the plain FP64 leg timed, in one batched call"}


def fp64_recheck(dpg, sptr, batches, finals, results):
    """Every timed mixed minimum re-evaluated by the FP64 drop-in at its final
    positions: max|F| and the relative energy difference to the reported one."""
    worst_f, worst_pe, n_checked, n_over = 0.0, 0.0, 0, 0
    for (e, sts), fin, res in zip(batches, finals, results):
        for k, st in enumerate(sts):
            sl = slice(k * N_PART, (k + 1) * N_PART)
            d = dpg.Disk(N_PART, st["box"], stream=sptr)
            d.setState(fin["x"][sl], fin["y"][sl], None, None, st["r"], st["m"])
            d.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
            d.zeroForceAndPotentialEnergy()
            d.calculateForces()
            f64 = d.forceStats()[0]
            pe64 = d.totalPotentialEnergy() / N_PART
            d.close()
            worst_f = max(worst_f, f64)
            worst_pe = max(worst_pe, abs(res[k]["avg_pe"] - pe64) / pe64)
            n_over += f64 > FMAX
            n_checked += 1
    return {"systems": n_checked, "max_force_fp64_max": worst_f, "above_fmax": int(n_over),
            "avg_pe_rel_diff_max": worst_pe}


def headline_roofline(dpg, sptr, batches, finals, flat, k_mean, peak, peak_src, tune):
    """e_force of the headline form, per arithmetic: the FP32 phase from fresh
    starts, the double-word phase and the FP64 passes at converged minima
    (PROFILE_ITERS plain launches each, CUDA events), weighted by the share of
    force passes each arithmetic took in the timed solves."""
    e, sts = batches[-1]
    host = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
    e.setState(*host)
    p32 = e.profileLoop(PROFILE_ITERS, FIRE_ALPHA0, FIRE_DT0, FMAX)
    fin = finals[-1]
    e.setState(fin["x"], fin["y"], host[2], host[3])
    pdw = e.profileLoop(PROFILE_ITERS, FIRE_ALPHA0, FIRE_DT0, 1e-15)
    e64 = dpg.Ensemble([N_PART] * BATCH, [st["box"] for st in sts], CUTOFF, SKIN,
                       precision=dpg.FP64, stream=sptr)
    e64.setState(fin["x"], fin["y"], host[2], host[3])
    p64 = e64.profileLoop(PROFILE_ITERS // 3, FIRE_ALPHA0, FIRE_DT0, 1e-15)
    e64.close()
    passes = float(sum(r["fire_steps"] for r in flat))
    n64 = float(sum(r["fp64_steps"] for r in flat))
    ndw = float(sum(r["dw_steps"] for r in flat))
    w = {"fp32": (passes - n64 - ndw) / passes, "dword": ndw / passes, "fp64": n64 / passes}
    # algorithmic bytes per particle and pass: FP32 phase reads the packed
    # offsets 16, count 4, indices 4k, FP32 velocity 8, 1/m 4 and writes the FP64
    # force 16, FP32 force 8 and velocity 8 (84 + 4k); the double-word phase also
    # reads the low words 16 (100 + 4k); FP64 reads position 16, radius 8, packed
    # offsets 16, count 4, indices 4k, velocity 16, mass 8 and writes force and
    # velocity 32 (100 + 4k); neighbours' data are gathered from cache
    per = {"fp32": 84 + 4 * k_mean, "dword": 100 + 4 * k_mean, "fp64": 100 + 4 * k_mean}
    us = {"fp32": p32["force_us"], "dword": pdw["force_us"], "fp64": p64["force_us"]}
    phases = {}
    for ph in ("fp32", "dword", "fp64"):
        b = BATCH * N_PART * per[ph]
        ach = b / (us[ph] * 1e-6) / 1e9
        phases[ph] = {"share_of_passes": w[ph], "launch_us": us[ph], "bytes_per_launch": b,
                      "achieved": ach, "frac": ach / peak}
    t_avg = sum(w[ph] * us[ph] for ph in us)
    b_avg = sum(w[ph] * BATCH * N_PART * per[ph] for ph in per)
    achieved = b_avg / (t_avg * 1e-6) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": E_FORCE_DRAM_PER_SYSTEM * BATCH,
            "traffic_source": "ncu dram__bytes_read+write of one FP32-phase e_force launch on "
                              "8 x 16384 disks, scaled to the batch by systems",
            "kernel": "e_force", "peak_source": peak_src, "bytes_per_launch": b_avg,
            "launch_us": t_avg, "phases": phases,
            "note": f"{BATCH} x 16384 disks; launch time weighted over the FP32, double-word and "
                    "FP64 passes by their share of the timed solves' force passes; the working "
                    "set is L2-resident, so the kernel is bound by latency and the FP64 pipe, "
                    "not by HBM"}


def resident_roofline(results, total_ms, launches, k_mean, peak, peak_src):
    """e_res, the resident form's kernel, over the timed solves.  Its launches
    (time slices of about 0.2 s, each carrying every system of its size class
    for as many iterations as fit) fill the timed region, so the launch time is
    the region's CUDA-event time over the launches (gaps between slices
    included: the achieved figure is a lower bound).  Algorithmic bytes: a FIRE
    iteration's compulsory traffic, 144 + 4k per disk (force 48 + 4k; update
    reads v, F, x, x_ref 64 and writes v, x 32), times the disk-iterations the
    timed solves ran."""
    per = 144 + 4 * k_mean
    flat = [r for res in results for r in res]
    disk_iters = float(sum(N_PART * r["fire_steps"] for r in flat))
    # a batch runs as long as its slowest system: iterations of the timed region
    region_iters = float(sum(max(r["fire_steps"] for r in res) for res in results))
    b = disk_iters * per / launches
    us = total_ms * 1e3 / launches
    achieved = b / (us * 1e-6) / 1e9
    traffic = None if E_RES_DRAM_PER_DISK is None else E_RES_DRAM_PER_DISK * BATCH * N_PART
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read+write of one e_res launch on 2 x 16384 disks "
                              "(bench.py --ncu-case resident_headline), scaled by disks",
            "kernel": "e_res", "peak_source": peak_src, "bytes_per_launch": b,
            "launch_us": us, "launches": launches, "bytes_per_disk_iteration": per,
            "us_per_iteration": total_ms * 1e3 / region_iters,
            "note": f"{BATCH} x 16384 disks, one 8-block cluster per system holding it in shared "
                    "memory for all its iterations: DRAM carries each system's state once per "
                    "launch, not once per iteration, so the bound is the iteration's latency "
                    "(barriers, the double-word dependency chains, remote shared-memory reads), "
                    "and the fraction is the algorithmic rate of a FIRE iteration against HBM"}


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


def fma_peaks(dpg):
    """Measured FP64 and FP32 FMA throughput (dpg_measure_fma_peak), TFLOP/s."""
    import ctypes as C
    out = {}
    for name, fp64, iters in (("fp64", 1, 1 << 12), ("fp32", 0, 1 << 16)):
        tf, ms = C.c_double(), C.c_double()
        dpg.lib.check(dpg.load_library().dpg_measure_fma_peak(fp64, iters, C.byref(tf), C.byref(ms)))
        out[name] = {"tflops": tf.value, "launch_ms": ms.value}
    return out


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


def jam_workload(S, seed=2024):
    """S bidisperse disk systems, N drawn log-uniformly in [64, 4096] from a seed,
    seeded random starts at phi = 0.80 (the reference's RandomUniform stream)."""
    from dpcuda_gb300.init import disk_packing
    rng = np.random.default_rng(seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(64), np.log(4096), S))).astype(int)
    sts = [disk_packing(int(n), 0.80, 7000 + k) for k, n in enumerate(sizes)]
    return sizes, sts


def jam_leg(dpg, S, P, plain_budget_s):
    """Pressure-band jamming of S uneven systems (the scripts/runArthurJamWithFire.cpp
    protocol: compression by box scaling, a FIRE minimisation after every step,
    bisection on the box length until the pressure is inside P +- 1% with more
    than 2 contacts per disk).

    - mixed+batched: every system at once in the resident form (double-word
      refinement, FP64 passes only certify states);
    - FP64 check: each jammed state minimised again by the FP64 drop-in at its
      own box; a state whose FP64 pressure is inside the band with enough
      contacts has |dphi_J| = 0 (same box, same radii); for any other the FP64
      packing fraction at the band's centre is found by a linear step from a
      second FP64 minimisation at a box 1e-6 smaller;
    - plain FP64: the drop-in, one system per call, on a seeded random sample
      of the systems until plain_budget_s of solving has passed."""
    import torch
    from dpcuda_gb300.ensemble import FORM_RESIDENT
    sizes, sts = jam_workload(S)
    log(f"jamming: {S} systems ({int(sizes.sum())} disks) at P = {P:g}")
    band = (0.99 * P, 1.01 * P)
    kw = dict(compression_rate=0.99, length_tolerance=1e-10, decompress_factor=1.01,
              max_compression_steps=2000)
    cat = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
    e = dpg.Ensemble(sizes, [st["box"] for st in sts], CUTOFF, SKIN, precision=dpg.MIXED,
                     switch_fmax=SWITCH_FMAX)
    e.setForm(FORM_RESIDENT)
    e.setState(*cat)
    e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 20, fmax_target=FMAX)  # module loading
    e.setState(*cat)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = e.jam(*band, fire=JAM_FIRE, **kw)
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t0
    log(f"jamming: mixed+batched {S} systems in {t_mixed:.1f} s")
    fin = e.getState()
    e.close()
    offs = np.concatenate([[0], np.cumsum(sizes)])
    # ---- FP64 check of every jammed state: the drop-in at the final box, its
    # pressure and contacts after an FP64 minimisation from the final positions
    # (at most JAM_CHECK_STEPS iterations); where that leaves the band, the
    # FP64 jammed packing fraction is found by a linear step from one more FP64
    # minimisation at a box 1e-6 smaller (a linearised re-jam)
    t1 = time.perf_counter()
    dphi, rejam, n_ok, f64_iters = [], [], 0, []
    for k in range(S):
        n = int(sizes[k])
        sl = slice(offs[k], offs[k + 1])
        L = res[k]["box_length"]
        d = dpg.Disk(n, L)
        d.setState(fin["x"][sl], fin["y"][sl], None, None, sts[k]["r"], sts[k]["m"])
        d.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        r64 = dpg.minimizeFire(d, *JAM_FIRE[:4], JAM_CHECK_STEPS, JAM_FIRE[5])
        f64_iters.append(int(r64["steps"]))
        P64 = d.getPressure()
        Z64 = d.getContactCount()
        phi0 = d.getPackingFraction()
        if band[0] <= P64 <= band[1] and Z64 > 2 * n:
            n_ok += 1
            dphi.append(0.0)
        else:
            d.scaleBox(1 - 1e-6)
            dpg.minimizeFire(d, *JAM_FIRE[:4], JAM_CHECK_STEPS, JAM_FIRE[5])
            P1, phi1 = d.getPressure(), d.getPackingFraction()
            slope = (P1 - P64) / (phi1 - phi0)
            # a non-positive slope: the FP64 minimisations did not settle within
            # JAM_CHECK_STEPS (the mixed run's last minimisation stopped at its cap)
            phi_fp64 = phi0 + (P - P64) / slope if slope > 0 else None
            dphi.append(abs(phi_fp64 - res[k]["packing_fraction"]) if phi_fp64 is not None else None)
            rejam.append({"system": k, "n": n, "pressure_fp64": P64, "contacts_fp64": Z64,
                          "phi_J_fp64": phi_fp64, "dphi_J": dphi[-1],
                          "mixed_fire_iterations": int(res[k]["fire_steps"])})
        d.close()
    t_check = time.perf_counter() - t1
    log(f"jamming: FP64 check in {t_check:.1f} s")
    # ---- plain FP64 drop-in on a seeded random sample, one system per call
    order = np.random.default_rng(11).permutation(S)
    plain_t, plain_done, plain_steps = 0.0, [], []
    for k in order:
        if plain_t >= plain_budget_s:
            break
        n = int(sizes[k])
        d = dpg.Disk(n, sts[k]["box"])
        d.setState(sts[k]["x"], sts[k]["y"], None, None, sts[k]["r"], sts[k]["m"])
        d.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        d.synchronize()
        t2 = time.perf_counter()
        rp = dpg.jamPressure(d, *band, fire=JAM_FIRE, neighbors=("cell", CUT_MULT, 0.2, 8.0, 0.5), **kw)
        d.synchronize()
        plain_t += time.perf_counter() - t2
        plain_done.append(int(k))
        plain_steps.append(int(rp["fire_steps_total"]))
        d.close()
        log(f"jamming: plain FP64 system {k} (N={n}) done, {plain_t:.1f} s so far")
    mixed_rate = S / t_mixed
    plain_rate = len(plain_done) / plain_t if plain_t > 0 else None
    # projection over all S systems: the plain path's measured time per FIRE
    # iteration times the mixed run's iterations, scaled by the plain / mixed
    # iteration ratio on the sampled systems
    steps_all = float(sum(r["fire_steps"] for r in res))
    mixed_same = float(sum(res[k]["fire_steps"] for k in plain_done))
    t_it = plain_t / max(1, sum(plain_steps))
    proj_t = t_it * steps_all * (sum(plain_steps) / mixed_same) if mixed_same > 0 else None
    steps = np.array([r["fire_steps"] for r in res])
    status = [int(r["status"]) for r in res]
    return {"workload": f"{S} bidisperse systems (radii 0.5/0.7), N log-uniform in [64, 4096] "
                        f"(seed 2024, {int(sizes.sum())} disks), phi0 0.80, pressure band "
                        f"{P:g} +- 1%, compression 0.99 / decompression 1.01 in box length, "
                        "FIRE after every step to PE/N < 1e-16 or max|F| <= 1e-13 "
                        "(at most 1e5 iterations)",
            "pressure": P, "band": list(band),
            "mixed_batched": {"form": "resident", "s": t_mixed, "systems_per_s": mixed_rate,
                              "in_band": int(sum(band[0] <= r["pressure"] <= band[1] for r in res)),
                              "status_counts": {str(v): status.count(v) for v in sorted(set(status))},
                              "fire_iterations": {"mean": float(steps.mean()), "max": int(steps.max()),
                                                  "sum": int(steps.sum())},
                              "minimizations_max": int(max(r["minimizations"] for r in res)),
                              "dw_share": float(sum(r["dw_steps"] for r in res) / steps.sum()),
                              "fp64_passes": int(sum(r["fp64_steps"] for r in res))},
            "fp64_check": {"systems": S, "confirmed_in_band": n_ok, "linearised_rejam": rejam,
                           "dphi_J_max": float(max(v for v in dphi if v is not None)),
                           "unresolved": int(sum(v is None for v in dphi)), "s": t_check,
                           "fp64_fire_iterations_max": int(max(f64_iters))},
            "plain_fp64": {"systems": len(plain_done), "s": plain_t, "systems_per_s": plain_rate,
                           "sample": "a seeded random order of the systems, one per call, until "
                                     f"{plain_budget_s:g} s of solving had passed",
                           "sizes": [int(sizes[k]) for k in plain_done],
                           "fire_iterations": plain_steps,
                           "mixed_fire_iterations_same_systems": [int(steps[k]) for k in plain_done]},
            "plain_fp64_projected": {"systems_per_s": S / proj_t if proj_t else None,
                                     "us_per_fire_iteration": 1e6 * t_it,
                                     "basis": "measured time per FIRE iteration of the sampled "
                                              "systems x the mixed run's iterations of all systems "
                                              "x the sampled plain / mixed iteration ratio"},
            "mixed_batched_over_plain_fp64": mixed_rate / plain_rate if plain_rate else None,
            "mixed_batched_over_plain_fp64_projected": mixed_rate * proj_t / S if proj_t else None}


def jam_ensemble(args):
    """The jamming leg alone (any pressure, e.g. the 1e-7 of the workload's
    definition): prints one JSON line."""
    import dpcuda_gb300 as dpg
    dpg.load_library()
    out = jam_leg(dpg, args.jam_systems, args.jam_pressure, JAM_PLAIN_BUDGET_S)
    print(json.dumps({"metric": "batched jamming: systems jammed/s, mixed+batched vs plain FP64",
                      "unit": "systems/s", "value": out["mixed_batched"]["systems_per_s"],
                      "n_gpus": 1, "higher_is_better": True, "detail": out}), flush=True)


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
    done, t_tot, n_tot, conv = 0, 0.0, 0, []
    for k in range(S):
        st = sts[k]
        s = dpg.Disk(int(sizes[k]), st["box"])
        s.setState(st["x"], st["y"], None, None, st["r"], st["m"])
        s.setupNeighbors("cell", CUT_MULT, 0.2, 8.0, 0.5)
        t0 = time.perf_counter()
        r = dpg.minimizeFire(s, FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 10**6, fmax_target=FMAX)
        s.synchronize()
        t_tot += time.perf_counter() - t0
        conv.append(bool(r["converged"]))
        n_tot += int(sizes[k])
        done += 1
        s.close()
        if t_tot > 30:
            break
    # the mixed batched form on exactly the systems the plain path solved, so
    # that the two rates compare the same starts
    sub = [np.concatenate([st[c] for st in sts[:done]]) for c in ("x", "y", "r", "m")]
    e = dpg.Ensemble(sizes[:done], [st["box"] for st in sts[:done]], CUTOFF, SKIN,
                     precision=dpg.MIXED, switch_fmax=SWITCH_FMAX)
    e.setState(*sub)
    e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 50, fmax_target=FMAX)
    e.setState(*sub)
    t0 = time.perf_counter()
    r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 10**6, fmax_target=FMAX)
    t_mixed = time.perf_counter() - t0
    e.close()
    print(json.dumps({"metric": "batched FIRE solves/s, uneven ensemble", "form": "plain_fp64",
                      "systems": done, "particles": n_tot, "s": t_tot,
                      "systems_per_s": done / t_tot, "converged": int(sum(conv)),
                      "sample": f"the first {done} of the {S} systems, one per call",
                      "mixed_batched_same_systems": {
                          "s": t_mixed, "systems_per_s": done / t_mixed,
                          "converged": int(sum(x["converged"] for x in r)),
                          "over_plain_fp64": t_tot / t_mixed}}), flush=True)


def ncu_case(which):
    """Small fixed workloads for ncu captures (plain stream launches, a few
    hundred kernels): 'fire' = 64 FIRE iterations of the 16384-disk system,
    'nve_large' = 8 NVE steps of the 2^20-disk system, 'ensemble' = 64 FIRE
    iterations of the batched mixed form on 16 x 16384 disks, 'bumpy_nve' =
    192 NVE steps of 4096 rigid bumpy bodies, 'resident' = 3000 FIRE
    iterations of 16 uneven systems in the resident form, 'resident_headline'
    = 3000 FIRE iterations of 2 of the headline's 16384-disk systems in the
    resident form, 'resident_dw_small' / 'resident_dw_large' = 1000
    double-word FIRE iterations of 48 x 128 / 8 x 4096 disks."""
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
    if which == "resident":
        # the jamming leg's first 16 systems (64-4096 disks), FIRE from their starts
        # for at most 3000 iterations in the resident form (time-sliced launches,
        # one per size class)
        from dpcuda_gb300.ensemble import FORM_RESIDENT
        sizes, sts = jam_workload(16)
        e = dpg.Ensemble(sizes, [st["box"] for st in sts], CUTOFF, SKIN, precision=dpg.MIXED,
                         switch_fmax=SWITCH_FMAX)
        e.setForm(FORM_RESIDENT)
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
        r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 3000, fmax_target=FMAX)
        print(json.dumps({"ncu_case": which, "steps": max(x["fire_steps"] for x in r)}))
        return
    if which == "resident_headline":
        # 2 of the headline's 16384-disk systems, FIRE from their starts for at
        # most 3000 iterations in the resident form (8-block clusters)
        from dpcuda_gb300.ensemble import FORM_RESIDENT
        sts = [packing(sd) for sd in step_seeds(0, 0)[:2]]
        e = dpg.Ensemble([N_PART] * 2, [st["box"] for st in sts], CUTOFF, SKIN,
                         precision=dpg.MIXED, switch_fmax=SWITCH_FMAX)
        e.setForm(FORM_RESIDENT)
        e.setState(*[np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")])
        r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 3000, fmax_target=FMAX)
        print(json.dumps({"ncu_case": which, "steps": max(x["fire_steps"] for x in r),
                          "launches": e.launchCount()}))
        return
    if which in ("resident_dw_small", "resident_dw_large"):
        # S systems of N disks relaxed to max|F| <= 1e-9, then 1000 FIRE
        # iterations in the double-word phase inside an NVTX range "dw" (the
        # capture filters on it): 48 x 128 disks (lanes per particle) or 8 x
        # 4096 disks (8-block clusters)
        import torch
        from dpcuda_gb300.ensemble import FORM_RESIDENT
        from dpcuda_gb300.init import disk_packing
        N, S = (128, 48) if which.endswith("small") else (4096, 8)
        sts = [disk_packing(N, 0.86, 700 + k) for k in range(S)]
        cat = [np.concatenate([st[c] for st in sts]) for c in ("x", "y", "r", "m")]
        e = dpg.Ensemble([N] * S, [st["box"] for st in sts], CUTOFF, SKIN, precision=dpg.MIXED,
                         switch_fmax=SWITCH_FMAX)
        e.setForm(FORM_RESIDENT)
        e.setState(*cat)
        e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 30000, fmax_target=1e-9)
        fin = e.getState()
        e.setState(fin["x"], fin["y"], cat[2], cat[3])
        torch.cuda.nvtx.range_push("dw")
        r = e.minimizeFire(FIRE_ALPHA0, FIRE_DT0, 0.0, 0.0, 1000, fmax_target=1e-15)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        print(json.dumps({"ncu_case": which, "steps": max(x["fire_steps"] for x in r),
                          "dw_steps": float(np.mean([x["dw_steps"] for x in r]))}))
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
                                           "bumpy_nve", "resident", "resident_headline",
                                           "resident_dw_small", "resident_dw_large"],
                    default=None,
                    help="run a small fixed workload for ncu captures and exit")
    ap.add_argument("--batch", type=int, default=BATCH, help="systems per step of the batched form")
    ap.add_argument("--jam-ensemble", action="store_true",
                    help="run the batched jamming workload instead of the default line")
    ap.add_argument("--jam-systems", type=int, default=JAM_SYSTEMS)
    ap.add_argument("--jam-pressure", type=float, default=JAM_PRESSURE,
                    help="target pressure of the batched jamming leg (band +-1%%)")
    ap.add_argument("--no-jam", action="store_true", help="skip the jamming leg")
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
