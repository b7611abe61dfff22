"""Generates the golden fixtures in tests/golden/ from the REFERENCE's own kernel
sources (mmccraw98/dpCUDA-v2 src/particles/{base,disk}/kernels.cu compiled on
the host by oracle/ref/build_ref.sh and driven by oracle/ref/ref_driver.cpp).

Run here, where the reference tree exists:
    python tests/golden/make_golden.py
The fixtures are committed; the GPU tests and the CPU oracle tests read them
without needing the reference tree.

Inputs come from the reference's own seeded generator (include/functors.h
RandomUniform, exact) for positions; velocities come from the oracle's
restatement of the GPU normal sampler (stored as given inputs).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle.oracle import (BumpyOracle, DiskOracle, build_reference, bumpy_packing,  # noqa: E402
                           disk_packing, fill_normal, fill_uniform)

CUT_MULT = 1.7 / 1.4  # r_c = d_max + skin 0.3 with d_max = 1.4


def padded_static_neighbors(o: DiskOracle) -> np.ndarray:
    sets = o.static_neighbor_sets()
    width = max(1, max(len(s) for s in sets))
    out = np.full((o.n, width), -1, dtype=np.int32)
    for i, s in enumerate(sets):
        row = sorted(s)
        out[i, :len(row)] = row
    return out


def snapshot(o: DiskOracle, prefix: str, d: dict):
    a = o.get_arrays()
    for k in ("x", "y", "vx", "vy", "fx", "fy", "pe"):
        d[f"{prefix}_{k}"] = a[k]


def system(n, phi, seed, method=0, vel_T=None):
    st = disk_packing(n, phi, seed, kind="reference")
    o = DiskOracle(n, st["box"], kind="reference")
    vx = vy = None
    if vel_T is not None:
        vx = fill_normal(n, 0.0, np.sqrt(vel_T), 1, seed)
        vy = fill_normal(n, 0.0, np.sqrt(vel_T), 1 + n, seed)
        vx -= vx.mean()
        vy -= vy.mean()
    o.set_arrays(x=st["x"], y=st["y"], vx=vx, vy=vy, r=st["r"], m=st["m"])
    info = o.setup_neighbors(method, CUT_MULT, 0.2, 8.0, 0.5)
    return o, st, vx, vy, info


def make_small():
    d = {}
    o, st, vx, vy, meth = system(64, 0.80, 7, vel_T=1e-3)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], vx0=vx, vy0=vy,
             method=meth)
    snapshot(o, "setup", d)
    d["setup_neighbors"] = padded_static_neighbors(o)
    o.nve_steps(1e-2, 200)
    snapshot(o, "nve200", d)
    d["nve200_total_pe"] = o.total_pe()
    d["nve200_total_ke"] = o.total_ke()
    o.fire_init(0.1, 1e-2)
    for _ in range(100):
        o.fire_step()
    snapshot(o, "fire100", d)
    fs = o.fire_state()
    d["fire100_state"] = np.array([fs["alpha"], fs["dt"], fs["n_good"], fs["n_bad"], fs["stopped"]])
    np.savez_compressed(HERE / "disk_n64_verlet.npz", **d)


def make_cfg1():
    d = {}
    n, phi, seed = 1024, 0.80, 1
    o, st, vx, vy, meth = system(n, phi, seed, vel_T=1e-4)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], vx0=vx, vy0=vy,
             method=meth)
    info = o.neighbor_info()
    d["n_cells_dim"] = info["n_cells_dim"]
    d["cap"] = info["cap"]
    ci, cs = o.cells()
    d["setup_cell_index"] = ci
    d["setup_cell_start"] = cs
    d["setup_static_index"] = o.get_current()["static_index"]
    snapshot(o, "setup", d)
    d["setup_neighbors"] = padded_static_neighbors(o)
    d["setup_stress"] = o.stress_tensor()
    d["setup_contacts"] = o.contact_count()
    o.nve_steps(1e-2, 500)
    snapshot(o, "nve500", d)
    d["nve500_rebuilds"] = np.array(o.num_rebuilds())
    d["nve500_total_pe"] = o.total_pe()
    d["nve500_total_ke"] = o.total_ke()
    o.fire_init(0.1, 1e-2)
    for _ in range(300):
        o.fire_step()
    snapshot(o, "fire300", d)
    fs = o.fire_state()
    d["fire300_state"] = np.array([fs["alpha"], fs["dt"], fs["n_good"], fs["n_bad"], fs["stopped"]])
    o.init_adam()
    for k in range(40):
        o.zero_force_and_pe()
        o.check_for_neighbor_update()
        o.calculate_forces()
        o.adam_step(k, 1e-3, 0.9, 0.999, 1e-8)
    snapshot(o, "adam40", d)
    np.savez_compressed(HERE / "disk_n1024_cell.npz", **d)


def make_fire_min():
    """FIRE minimisation to the reference's own stop criteria (PE change)."""
    d = {}
    n, phi, seed = 2048, 0.86, 3
    o, st, _, _, meth = system(n, phi, seed)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], method=meth)
    steps, stopped = o.minimize_fire(0.1, 1e-2, 1e-16, 1e-16, 100000, 0.0)
    d["steps"] = steps
    d["stopped"] = stopped
    d["avg_pe"] = o.total_pe() / n
    d["max_force"] = o.max_force()
    a = o.get_arrays()
    d["x"], d["y"] = a["x"], a["y"]
    d["pressure"] = o.pressure()
    d["contacts"] = o.contact_count()
    np.savez_compressed(HERE / "disk_n2048_fire_min.npz", **d)


def make_damped_gd():
    """DampedNVE (src/integrator/damped_nve.cu) and GradDesc (src/integrator/grad_desc.cu)."""
    d = {}
    n, phi, seed = 512, 0.84, 9
    o, st, vx, vy, meth = system(n, phi, seed, vel_T=1e-3)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], vx0=vx, vy0=vy,
             method=meth)
    o.damped_nve_steps(1e-2, 0.5, 300)
    snapshot(o, "damped300", d)
    d["damped300_rebuilds"] = np.array(o.num_rebuilds())
    o.grad_desc_steps(1e-2, 200)
    snapshot(o, "gd200", d)
    d["gd200_rebuilds"] = np.array(o.num_rebuilds())
    np.savez_compressed(HERE / "disk_n512_damped_gd.npz", **d)


def make_walls():
    """Disk::calculateWallForces and NVE::wall_step (src/particles/disk/kernels.cu:59-71,
    src/integrator/nve.cu:27-38)."""
    d = {}
    n, phi, seed = 256, 0.80, 11
    o, st, vx, vy, meth = system(n, phi, seed, vel_T=1e-3)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], vx0=vx, vy0=vy,
             method=meth)
    o.zero_force_and_pe()
    o.wall_forces()
    snapshot(o, "wall", d)
    o.nve_wall_steps(1e-2, 300)
    snapshot(o, "wallnve300", d)
    np.savez_compressed(HERE / "disk_n256_walls.npz", **d)


def make_pairs():
    """Disk::calculateForceDistancePairs (src/particles/disk/disk.cu:228-255,
    src/particles/disk/kernels.cu:73-175) after 50 NVE steps of a cell-list system."""
    d = {}
    n, phi, seed = 256, 0.86, 13
    o, st, vx, vy, meth = system(n, phi, seed, vel_T=1e-3)
    d.update(x0=st["x"], y0=st["y"], r=st["r"], m=st["m"], box=st["box"], vx0=vx, vy0=vy,
             method=meth)
    o.nve_steps(1e-2, 50)
    d["cap"] = o.neighbor_info()["cap"]
    d["static_index"] = o.get_current()["static_index"]
    for k, v in o.pair_dump().items():
        d[f"pairs_{k}"] = v
    np.savez_compressed(HERE / "disk_n256_pairs.npz", **d)


def make_rng():
    d = {}
    for seed in (1, 7, 12345):
        d[f"uniform_seed{seed}"] = fill_uniform(1000, 0.0, 38.5, 0, seed, kind="reference")
        d[f"uniform_seed{seed}_off"] = fill_uniform(1000, -0.5, 0.5, 3000, seed, kind="reference")
    np.savez_compressed(HERE / "rng_uniform.npz", **d)


def padded_sets(sets):
    width = max(1, max(len(x) for x in sets))
    out = np.full((len(sets), width), -1, dtype=np.int32)
    for i, x in enumerate(sets):
        row = sorted(x)
        out[i, :len(row)] = row
    return out


def bumpy_snapshot(b: BumpyOracle, prefix: str, d: dict, vertices: bool = True):
    bd = b.bodies()
    for k in ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe"):
        d[f"{prefix}_{k}"] = bd[k]
    if vertices:
        d[f"{prefix}_px"], d[f"{prefix}_py"] = b.vertices()


def make_bumpy(nb, phi, seed, name):
    """Rigid bumpy bodies (cfg4 parity variant: 20 / 28 vertices, seg 0.9)."""
    d = {}
    st = bumpy_packing(nb, phi, seed, kind="reference")
    b = BumpyOracle(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True,
                    kind="reference")
    b.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"])
    b.init_vertices()
    b.set_mass(1.0)
    d.update(x0=st["x"], y0=st["y"], th0=st["th"], r=st["r"], nvb=st["nvb"], box=st["box"],
             rv=st["rv"], e_c=st["e_c"], seg=st["seg"])
    d["px0"], d["py0"] = b.vertices()
    d["I"] = b.bodies()["I"]
    d["method"] = b.setup_neighbors(0, 1.5, 0.2, 8.0, 0.5)
    bumpy_snapshot(b, "setup", d)
    d["setup_vneighbors"] = padded_sets(b.vertex_neighbor_sets())
    b.fire_init(0.1, 1e-2)
    for _ in range(60):
        b.fire_step()
    bumpy_snapshot(b, "fire60", d)
    d["fire60_info"] = np.array([b.neighbor_info()["n_rebuilds"], b.neighbor_info()["n_cell_rebuilds"]])
    np.savez_compressed(HERE / name, **d)


def make_bumpy_extras():
    """Rigid bumpy bodies beyond FIRE and NVE, from the reference's own kernels:
    pair and Hessian dump, stress tensor and contact counts (with translational and angular
    velocities, so the kinetic term's omega x r branch runs), DampedNVE,
    NVE::wall_step, the wall-only and wall-plus-pair force calls, Adam steps
    across cell re-sorts, and setLastState / revertToLastState across re-sorts
    (cell displacement multiplier 0.05 makes the re-sorts frequent)."""
    nb, seed = 128, 7
    st = bumpy_packing(nb, 0.80, seed, kind="reference")
    vx = fill_normal(nb, 0.0, np.sqrt(1e-3), 1, seed)
    vy = fill_normal(nb, 0.0, np.sqrt(1e-3), 1 + nb, seed)
    w = fill_normal(nb, 0.0, np.sqrt(1e-3), 1 + 2 * nb, seed)
    vx -= vx.mean()
    vy -= vy.mean()
    d = dict(x0=st["x"], y0=st["y"], th0=st["th"], r=st["r"], nvb=st["nvb"], box=st["box"],
             rv=st["rv"], e_c=st["e_c"], seg=st["seg"], vx0=vx, vy0=vy, w0=w)

    def fresh(cdm=0.5):
        b = BumpyOracle(nb, st["nv"], st["box"], st["e_c"], 2.0, st["rv"], st["seg"], True,
                        kind="reference")
        b.set_bodies(st["x"], st["y"], st["th"], st["r"], st["nvb"], vx, vy, w)
        b.init_vertices()
        b.set_mass(1.0)
        b.setup_neighbors(0, 1.5, 0.2, 8.0, cdm)
        return b

    def info(b):
        i = b.neighbor_info()
        return np.array([i["n_rebuilds"], i["n_cell_rebuilds"]])

    b = fresh()
    d["method"] = b.neighbor_info()["method"]
    bumpy_snapshot(b, "setup", d)
    d["stress_tot"], d["stress_body"] = b.stress()
    d["contacts_tot"], d["contacts_body"], d["vcontacts_body"] = b.count_contacts()
    for k, v in b.pair_dump().items():
        d[f"pairs_{k}"] = v
    b.zero()
    b.wall_only()
    bumpy_snapshot(b, "wallonly", d, vertices=False)
    b.zero()
    b.wall_and_pair_forces()
    bumpy_snapshot(b, "wallpair", d, vertices=False)
    b = fresh()
    b.damped_nve_steps(5e-3, 0.5, 200)
    bumpy_snapshot(b, "damped", d)
    d["damped_info"] = info(b)
    b = fresh()
    b.nve_wall_steps(5e-3, 200)
    bumpy_snapshot(b, "walls", d)
    d["walls_info"] = info(b)
    b = fresh(0.05)
    b.adam_steps(150, 1e-2)
    bumpy_snapshot(b, "adam", d)
    d["adam_info"] = info(b)
    assert d["adam_info"][1] > 1, "Adam run should cross a cell re-sort"
    b = fresh(0.05)
    b.save_state()
    b.fire_init(0.1, 1e-2)
    for _ in range(100):
        b.fire_step()
    d["revert_pre_info"] = info(b)
    assert d["revert_pre_info"][1] > 1, "FIRE run should cross a cell re-sort"
    b.restore_state()
    bumpy_snapshot(b, "revert", d)
    b.zero()
    b.calculate_forces()
    bumpy_snapshot(b, "revertf", d, vertices=False)
    d["revert_info"] = info(b)
    np.savez_compressed(HERE / "bumpy_n128_extras.npz", **d)


if __name__ == "__main__":
    if build_reference() is None:
        sys.exit("reference tree not available; cannot regenerate fixtures")
    if len(sys.argv) > 1:  # regenerate only the named fixtures, e.g. make_damped_gd
        for name in sys.argv[1:]:
            globals()[name]()
        sys.exit(0)
    make_rng()
    make_small()
    make_cfg1()
    make_fire_min()
    make_damped_gd()
    make_walls()
    make_pairs()
    make_bumpy(64, 0.80, 3, "bumpy_n64_verlet.npz")
    make_bumpy(256, 0.80, 5, "bumpy_n256_cell.npz")
    make_bumpy_extras()
    print("fixtures written to", HERE)
