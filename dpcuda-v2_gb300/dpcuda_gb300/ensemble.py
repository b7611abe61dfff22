"""Batched form: S independent disk systems advanced together (include/dpg.h,
dpg_ensemble_*).  Each system keeps its own box, neighbour list, FIRE state and
convergence flags; every kernel launch covers all systems and the whole run is
one CUDA graph."""
from __future__ import annotations

import ctypes as C

import numpy as np

from .disk import _METHODS
from .lib import (DP, EnsembleParams, EnsembleResult, EnsembleTuning, FireParams, I64P, JamParams,
                  NeighborConfig, check, load_library)

FP64, MIXED, DWORD = 0, 1, 2


def partition_systems(n_particles, world):
    """Independent systems over `world` ranks (one GPU each): greedy N-balanced
    bin packing, largest system first to the least-loaded rank (ties: lowest
    rank), deterministic on every rank.  Returns each rank's system indices in
    ascending order; the ranks need no exchange while they solve their share."""
    n = [int(v) for v in n_particles]
    if world < 1:
        raise ValueError("world must be >= 1")
    loads = [0] * world
    parts = [[] for _ in range(world)]
    for k in sorted(range(len(n)), key=lambda j: (-n[j], j)):
        r = min(range(world), key=lambda q: (loads[q], q))
        parts[r].append(k)
        loads[r] += n[k]
    return [sorted(p) for p in parts]
def solve_partitioned(n_particles, solve, group=None):
    """Independent systems over the ranks of a torch.distributed group (one
    GPU per rank; no exchange on the data path): every rank computes the same
    partition_systems assignment, solves its own share with
    solve(indices) -> list of per-system results (in the order of indices),
    and rank 0 gathers the results in input order.  Returns that list on rank
    0 and None on the others; without an initialised process group the caller
    is the only rank and solves every system."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return list(solve(list(range(len(n_particles)))))
    world, rank = dist.get_world_size(group), dist.get_rank(group)
    mine = partition_systems(n_particles, world)[rank]
    res = list(solve(mine)) if mine else []
    if len(res) != len(mine):
        raise ValueError("solve() must return one result per system index")
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(list(zip(mine, res)), gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = [None] * len(n_particles)
    for part in gathered:
        for k, r in part:
            out[k] = r
    return out


def ensemble_solver(n_particles, boxes, states, mode="fire", precision=MIXED, cutoff=1.7,
                    skin=0.3, switch_fmax=1e-6, stream=None, **params):
    """A solve() for solve_partitioned on this rank's GPU: the given systems
    as one Ensemble (states[k] = dict with x, y, r, m), minimised by FIRE
    (mode "fire", params as Ensemble.minimizeFire) or jammed (mode "jam",
    params as Ensemble.jam)."""
    def solve(indices):
        if not indices:
            return []
        e = Ensemble([n_particles[k] for k in indices], [boxes[k] for k in indices], cutoff, skin,
                     precision=precision, switch_fmax=switch_fmax, stream=stream)
        try:
            e.setState(*[np.concatenate([states[k][c] for k in indices]) for c in ("x", "y", "r", "m")])
            return e.jam(**params) if mode == "jam" else e.minimizeFire(**params)
        finally:
            e.close()
    return solve


FORM_AUTO, FORM_GRID, FORM_PERSIST, FORM_RESIDENT = 0, 1, 2, 3
_FORM_NAMES = {FORM_GRID: "grid", FORM_PERSIST: "persist", FORM_RESIDENT: "resident"}


class Ensemble:
    def __init__(self, n_particles, boxes, cutoff, skin, e_c=1.0, n_c=2.0, precision=MIXED,
                 switch_fmax=1e-6, stream=None):
        self.lib = load_library()
        self.n = np.ascontiguousarray(n_particles, dtype=np.int64)
        self.boxes = np.ascontiguousarray(boxes, dtype=np.float64)
        self.S = len(self.n)
        prm = EnsembleParams(self.S, float(e_c), float(n_c), float(cutoff), float(skin),
                             int(precision), 0, float(switch_fmax))
        h = C.c_void_p()
        check(self.lib.dpg_ensemble_create(C.byref(prm), self.n.ctypes.data_as(I64P),
                                           self.boxes.ctypes.data_as(DP),
                                           C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h
        self.radii = None

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setState(self, x, y, radii, masses):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, radii, masses)]
        self.radii = arrs[2]
        check(self.lib.dpg_ensemble_set_state(self.h, *[a.ctypes.data_as(DP) for a in arrs]))

    def getState(self):
        tot = int(self.n.sum())
        out = {k: np.zeros(tot) for k in ("x", "y", "fx", "fy")}
        check(self.lib.dpg_ensemble_get_state(self.h, *[out[k].ctypes.data_as(DP) for k in
                                                         ("x", "y", "fx", "fy")]))
        return out

    def _results(self, res):
        out = []
        starts = np.concatenate([[0], np.cumsum(self.n)])
        for k in range(self.S):
            r = res[k]
            area = float(np.sum(self.radii[starts[k]:starts[k + 1]] ** 2)) * np.pi
            out.append(dict(avg_pe=r.avg_pe, max_force=r.max_force, pressure=r.pressure,
                            box_length=r.box_length, contacts=r.contacts,
                            packing_fraction=area / r.box_length ** 2, fire_steps=r.fire_steps,
                            minimizations=r.minimizations, rebuilds=r.rebuilds, status=r.status,
                            converged=r.converged, fp64_steps=r.fp64_steps,
                            dw_steps=r.dw_steps))
        return out

    def calculateForces(self, precision=FP64):
        """One force pass on every system at the current positions; forces via
        getState(), per-system energies / pressure / contacts returned."""
        res = (EnsembleResult * self.S)()
        check(self.lib.dpg_ensemble_compute_forces(self.h, int(precision), res))
        return self._results(res)

    def minimizeFire(self, alpha_init=0.1, dt=1e-2, avg_pe_target=1e-16, avg_pe_diff_target=1e-16,
                     num_steps=100000, fmax_target=0.0):
        prm = FireParams(float(alpha_init), float(dt), float(avg_pe_target),
                         float(avg_pe_diff_target), int(num_steps), float(fmax_target))
        res = (EnsembleResult * self.S)()
        check(self.lib.dpg_ensemble_fire_minimize(self.h, C.byref(prm), res))
        return self._results(res)

    def jam(self, pressure_low, pressure_high, compression_rate=0.99, length_tolerance=1e-10,
            decompress_factor=1.01, max_compression_steps=1000,
            fire=(0.1, 1e-2, 1e-16, 1e-16, 100000, 0.0)):
        prm = JamParams(float(pressure_low), float(pressure_high), float(compression_rate),
                        float(length_tolerance), float(decompress_factor),
                        int(max_compression_steps),
                        FireParams(float(fire[0]), float(fire[1]), float(fire[2]), float(fire[3]),
                                   int(fire[4]), float(fire[5])),
                        NeighborConfig(0, 1.5, 0.2, 8.0, 0.5))
        res = (EnsembleResult * self.S)()
        check(self.lib.dpg_ensemble_jam(self.h, C.byref(prm), res))
        return self._results(res)

    def profileLoop(self, iters, alpha_init=0.1, dt=1e-2, fmax_target=1e-13):
        """Mean device time per iteration of each phase of the FIRE loop (us), as
        plain launches.  Leaves the systems mid-minimisation."""
        prm = FireParams(float(alpha_init), float(dt), 0.0, 0.0, 10**9, float(fmax_target))
        avg = (C.c_double * 4)()
        cnt = (C.c_int64 * 3)()
        check(self.lib.dpg_ensemble_profile_loop(self.h, C.byref(prm), int(iters), avg, cnt))
        return {"move_us": avg[0], "rebuild_us": avg[1], "force_us": avg[2], "transition_us": avg[3],
                "iters": cnt[0], "rebuilds": cnt[1], "force_passes": cnt[2]}

    def launchCount(self):
        """Kernel launches (a CUDA-graph launch counting as one) issued so far."""
        n = C.c_int64()
        check(self.lib.dpg_ensemble_launch_count(self.h, C.byref(n)))
        return n.value

    def setForm(self, form=FORM_AUTO, threads=0):
        """FORM_GRID (one launch per stage over all systems, a CUDA graph loop),
        FORM_PERSIST (one persistent block per system), FORM_RESIDENT (one
        block per system holding it on chip, systems of at most 16384
        particles), FORM_AUTO (resident when it holds every system, else grid,
        or the autotuner's choice); threads: the persistent block size (128,
        256, 512; 0 = by system size)."""
        check(self.lib.dpg_ensemble_set_form(self.h, int(form), int(threads)))

    def autotune(self, iters=300, alpha_init=0.1, dt=1e-2):
        """Times FIRE iterations from the current positions for every form,
        persistent block size and skin (1, 0.75, 0.5 x), keeps the fastest and
        restores the positions.  Returns the choice and every candidate's
        particle-iterations per second."""
        prm = FireParams(float(alpha_init), float(dt), 0.0, 0.0, int(iters), 0.0)
        t = EnsembleTuning()
        check(self.lib.dpg_ensemble_autotune(self.h, C.byref(prm), int(iters), C.byref(t)))
        cands = [dict(form=_FORM_NAMES[t.cand_form[k]], threads=t.cand_threads[k],
                      skin=t.cand_skin[k], rate=t.cand_rate[k]) for k in range(t.n_candidates)]
        return dict(form=_FORM_NAMES[t.form], threads=t.threads, skin=t.skin, candidates=cands)
