"""ctypes front end for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads ``oracle/_build/liboracle.so`` (the C restatement, prefix ``orc_``) and,
where it was built, ``oracle/_ref/libdpref.so`` (the reference's own kernel
sources compiled on the host, prefix ``ref_``).  Both expose the same C API, so
``DiskOracle(kind="oracle")`` and ``DiskOracle(kind="reference")`` are
interchangeable.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg use this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "liboracle.so"
REF_SO = HERE / "_ref" / "libdpref.so"

NEIGH_CELL, NEIGH_VERLET, NEIGH_ALL = 0, 1, 2

_libs: dict[str, C.CDLL] = {}

D = C.c_double
I64 = C.c_int64
P = C.c_void_p
DP = C.POINTER(C.c_double)
LP = C.POINTER(C.c_int64)


def build_oracle() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return ORACLE_SO


def build_reference() -> Path | None:
    subprocess.run(["bash", str(HERE / "ref" / "build_ref.sh")], check=True,
                   stdout=subprocess.DEVNULL)
    return REF_SO if REF_SO.exists() else None


def reference_available() -> bool:
    return REF_SO.exists()


_SIGS = {
    "create": (P, [I64, D, D, D, D]),
    "destroy": (None, [P]),
    "set_arrays": (None, [P, DP, DP, DP, DP, DP, DP]),
    "get_arrays": (None, [P, DP, DP, DP, DP, DP, DP, DP, DP, DP]),
    "get_current": (None, [P, DP, DP, DP, DP, DP, DP, DP, LP]),
    "get_box": (None, [P, DP, DP]),
    "setup_neighbors": (C.c_int, [P, C.c_int, D, D, D, D]),
    "update_neighbor_list": (None, [P]),
    "check_for_neighbor_update": (C.c_int, [P]),
    "neighbor_info": (None, [P, C.POINTER(C.c_int), DP, DP, LP, DP, DP, LP]),
    "get_neighbors": (None, [P, LP, LP]),
    "get_cells": (None, [P, LP, LP]),
    "num_rebuilds": (I64, [P, LP]),
    "zero_force_and_pe": (None, [P]),
    "calculate_forces": (None, [P]),
    "update_velocities": (None, [P, D]),
    "update_positions": (None, [P, D]),
    "mix_velocities_and_forces": (None, [P, D]),
    "set_velocities_zero": (None, [P]),
    "power_fire": (D, [P]),
    "total_pe": (D, [P]),
    "total_ke": (D, [P]),
    "max_force": (D, [P]),
    "nve_steps": (None, [P, D, I64]),
    "damped_nve_steps": (None, [P, D, D, I64]),
    "grad_desc_steps": (None, [P, D, I64]),
    "wall_forces": (None, [P]),
    "pair_dump": (None, [P, C.POINTER(DP), LP, LP]),
    "nve_wall_steps": (None, [P, D, I64]),
    "fire_init": (None, [P, D, D]),
    "fire_step": (C.c_int, [P]),
    "fire_state": (None, [P, DP, DP, LP, LP, C.POINTER(C.c_int)]),
    "minimize_fire": (I64, [P, D, D, D, D, I64, D, C.POINTER(C.c_int)]),
    "init_adam": (None, [P]),
    "adam_step": (None, [P, I64, D, D, D, D]),
    "minimize_adam": (I64, [P, D, D, D, D, D, D, I64]),
    "stress_tensor": (None, [P, DP]),
    "pressure": (D, [P]),
    "contact_count": (D, [P]),
    "particle_area": (D, [P]),
    "packing_fraction": (D, [P]),
    "scale_to_packing_fraction": (None, [P, D]),
    "scale_box": (None, [P, D]),
    "set_last_state": (None, [P]),
    "revert_to_last_state": (None, [P]),
    "fill_uniform": (None, [DP, I64, D, D, I64, I64]),
}


def _load(kind: str) -> tuple[C.CDLL, str]:
    if kind == "oracle":
        path, prefix = ORACLE_SO, "orc_"
        if not path.exists():
            build_oracle()
    elif kind == "reference":
        path, prefix = REF_SO, "ref_"
        if not path.exists():
            raise FileNotFoundError("oracle/_ref/libdpref.so not built (needs the reference tree)")
    else:
        raise ValueError(kind)
    if kind not in _libs:
        lib = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, prefix + name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        if kind == "oracle":
            lib.orc_fill_normal.restype = None
            lib.orc_fill_normal.argtypes = [DP, I64, D, D, I64, I64]
            lib.orc_erfcinv.restype = D
            lib.orc_erfcinv.argtypes = [D]
            lib.orc_set_threads.argtypes = [C.c_int]
            lib.orc_set_forces.argtypes = [P, DP, DP]
            lib.orc_force_balance.restype = D
            lib.orc_force_balance.argtypes = [P]
        _libs[kind] = lib
    return _libs[kind], prefix


def _dp(a):
    return None if a is None else a.ctypes.data_as(DP)


def _lp(a):
    return None if a is None else a.ctypes.data_as(LP)


class DiskOracle:
    """One disk system held by the oracle or by the reference-kernel harness."""

    def __init__(self, n, box, e_c=1.0, n_c=2.0, kind="oracle"):
        self.lib, self.pre = _load(kind)
        self.kind = kind
        self.n = int(n)
        bx, by = (box, box) if np.isscalar(box) else box
        self.h = self._f("create")(self.n, float(bx), float(by), float(e_c), float(n_c))

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def close(self):
        if getattr(self, "h", None):
            self._f("destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state -----------------------------------------------------------
    def set_arrays(self, x=None, y=None, vx=None, vy=None, r=None, m=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64)
                for a in (x, y, vx, vy, r, m)]
        self._f("set_arrays")(self.h, *[_dp(a) for a in arrs])

    def get_arrays(self):
        out = {k: np.zeros(self.n) for k in ("x", "y", "vx", "vy", "fx", "fy", "pe", "r", "m")}
        self._f("get_arrays")(self.h, *[_dp(out[k]) for k in
                                        ("x", "y", "vx", "vy", "fx", "fy", "pe", "r", "m")])
        return out

    def get_current(self):
        out = {k: np.zeros(self.n) for k in ("x", "y", "vx", "vy", "fx", "fy", "pe")}
        sidx = np.zeros(self.n, dtype=np.int64)
        self._f("get_current")(self.h, *[_dp(out[k]) for k in
                                         ("x", "y", "vx", "vy", "fx", "fy", "pe")], _lp(sidx))
        out["static_index"] = sidx
        return out

    def box(self):
        bx, by = D(), D()
        self._f("get_box")(self.h, C.byref(bx), C.byref(by))
        return bx.value, by.value

    # -- neighbours ------------------------------------------------------
    def setup_neighbors(self, method=NEIGH_CELL, cutoff_mult=1.5, disp_mult=0.2,
                        particles_per_cell=8.0, cell_disp_mult=0.5):
        return self._f("setup_neighbors")(self.h, int(method), float(cutoff_mult),
                                          float(disp_mult), float(particles_per_cell),
                                          float(cell_disp_mult))

    def update_neighbor_list(self):
        self._f("update_neighbor_list")(self.h)

    def check_for_neighbor_update(self):
        return self._f("check_for_neighbor_update")(self.h)

    def neighbor_info(self):
        m = C.c_int()
        cutoff, thr2, cs, cthr2 = D(), D(), D(), D()
        ncd, cap = I64(), I64()
        self._f("neighbor_info")(self.h, C.byref(m), C.byref(cutoff), C.byref(thr2),
                                 C.byref(ncd), C.byref(cs), C.byref(cthr2), C.byref(cap))
        return dict(method=m.value, cutoff=cutoff.value, thr2=thr2.value, n_cells_dim=ncd.value,
                    cell_size=cs.value, cell_thr2=cthr2.value, cap=cap.value)

    def neighbors(self):
        """(list[n, cap] int64 in current order, -1 padded; counts[n])"""
        cap = self.neighbor_info()["cap"]
        lst = np.zeros(self.n * cap, dtype=np.int64)
        cnt = np.zeros(self.n, dtype=np.int64)
        self._f("get_neighbors")(self.h, _lp(lst), _lp(cnt))
        return lst.reshape(self.n, cap), cnt

    def static_neighbor_sets(self):
        """neighbour sets keyed by static (input) index"""
        lst, cnt = self.neighbors()
        sidx = self.get_current()["static_index"]
        sets = [None] * self.n
        for i in range(self.n):
            sets[sidx[i]] = frozenset(int(sidx[j]) for j in lst[i, :cnt[i]] if j >= 0)
        return sets

    def cells(self):
        info = self.neighbor_info()
        ci = np.zeros(self.n, dtype=np.int64)
        ncells = max(info["n_cells_dim"], 0) ** 2
        cs = np.zeros(ncells + 1, dtype=np.int64)
        self._f("get_cells")(self.h, _lp(ci), _lp(cs))
        return ci, cs

    def num_rebuilds(self):
        nc = I64()
        n = self._f("num_rebuilds")(self.h, C.byref(nc))
        return n, nc.value

    # -- dynamics ----------------------------------------------------------
    def zero_force_and_pe(self):
        self._f("zero_force_and_pe")(self.h)

    def calculate_forces(self):
        self._f("calculate_forces")(self.h)

    def update_velocities(self, dt):
        self._f("update_velocities")(self.h, float(dt))

    def update_positions(self, dt):
        self._f("update_positions")(self.h, float(dt))

    def mix_velocities_and_forces(self, alpha):
        self._f("mix_velocities_and_forces")(self.h, float(alpha))

    def set_velocities_zero(self):
        self._f("set_velocities_zero")(self.h)

    def power_fire(self):
        return self._f("power_fire")(self.h)

    def total_pe(self):
        return self._f("total_pe")(self.h)

    def total_ke(self):
        return self._f("total_ke")(self.h)

    def max_force(self):
        return self._f("max_force")(self.h)

    def nve_steps(self, dt, n):
        self._f("nve_steps")(self.h, float(dt), int(n))

    def damped_nve_steps(self, dt, gamma, n):
        self._f("damped_nve_steps")(self.h, float(dt), float(gamma), int(n))

    PAIR_KEYS = ("potential", "force_x", "force_y", "distance_x", "distance_y", "overlap",
                 "radsum", "angle", "hess_xx", "hess_xy", "hess_yx", "hess_yy",
                 "hess_ii_xx", "hess_ii_xy", "hess_ii_yx", "hess_ii_yy")

    def pair_dump(self):
        """calculateForceDistancePairs arrays, [slot * cap + k] in the current order."""
        cap = self.neighbor_info()["cap"]
        m = self.n * cap
        out = {k: np.zeros(m) for k in self.PAIR_KEYS}
        ptrs = (DP * 16)(*[_dp(out[k]) for k in self.PAIR_KEYS])
        ti, oi = np.zeros(m, dtype=np.int64), np.zeros(m, dtype=np.int64)
        self._f("pair_dump")(self.h, ptrs, ti.ctypes.data_as(LP), oi.ctypes.data_as(LP))
        out["this_id"], out["other_id"] = ti, oi
        return out

    def wall_forces(self):
        self._f("wall_forces")(self.h)

    def nve_wall_steps(self, dt, n):
        self._f("nve_wall_steps")(self.h, float(dt), int(n))

    def grad_desc_steps(self, alpha, n):
        self._f("grad_desc_steps")(self.h, float(alpha), int(n))

    def fire_init(self, alpha_init=0.1, dt=1e-2):
        self._f("fire_init")(self.h, float(alpha_init), float(dt))

    def fire_step(self):
        return self._f("fire_step")(self.h)

    def fire_state(self):
        a, dt = D(), D()
        ng, nb = I64(), I64()
        st = C.c_int()
        self._f("fire_state")(self.h, C.byref(a), C.byref(dt), C.byref(ng), C.byref(nb), C.byref(st))
        return dict(alpha=a.value, dt=dt.value, n_good=ng.value, n_bad=nb.value, stopped=st.value)

    def minimize_fire(self, alpha_init=0.1, dt=1e-2, pe_target=1e-16, pe_diff_target=1e-16,
                      num_steps=100000, fmax_target=0.0):
        st = C.c_int()
        steps = self._f("minimize_fire")(self.h, float(alpha_init), float(dt), float(pe_target),
                                         float(pe_diff_target), int(num_steps),
                                         float(fmax_target), C.byref(st))
        return steps, st.value

    def init_adam(self):
        self._f("init_adam")(self.h)

    def adam_step(self, step, alpha=1e-4, beta1=0.9, beta2=0.999, eps=1e-8):
        self._f("adam_step")(self.h, int(step), float(alpha), float(beta1), float(beta2), float(eps))

    def minimize_adam(self, alpha=1e-4, beta1=0.9, beta2=0.999, eps=1e-8, pe_target=1e-16,
                      pe_diff_target=1e-16, num_steps=100000):
        return self._f("minimize_adam")(self.h, float(alpha), float(beta1), float(beta2),
                                        float(eps), float(pe_target), float(pe_diff_target),
                                        int(num_steps))

    def stress_tensor(self):
        out = np.zeros(4)
        self._f("stress_tensor")(self.h, _dp(out))
        return out

    def pressure(self):
        return self._f("pressure")(self.h)

    def contact_count(self):
        return self._f("contact_count")(self.h)

    def packing_fraction(self):
        return self._f("packing_fraction")(self.h)

    def particle_area(self):
        return self._f("particle_area")(self.h)

    def scale_to_packing_fraction(self, phi):
        self._f("scale_to_packing_fraction")(self.h, float(phi))

    def scale_box(self, f):
        self._f("scale_box")(self.h, float(f))

    def set_last_state(self):
        self._f("set_last_state")(self.h)

    def revert_to_last_state(self):
        self._f("revert_to_last_state")(self.h)


def fill_uniform(n, lo, hi, seed_offset, seed, kind="oracle"):
    lib, pre = _load(kind)
    out = np.zeros(int(n))
    getattr(lib, pre + "fill_uniform")(_dp(out), int(n), float(lo), float(hi), int(seed_offset),
                                       int(seed))
    return out


def fill_normal(n, mean, std, seed_offset, seed):
    lib, _ = _load("oracle")
    out = np.zeros(int(n))
    lib.orc_fill_normal(_dp(out), int(n), float(mean), float(std), int(seed_offset), int(seed))
    return out


def set_threads(n: int):
    lib, _ = _load("oracle")
    lib.orc_set_threads(int(n))


def disk_packing(n, phi, seed, size_ratio=1.4, count_ratio=0.5, kind="oracle"):
    """Reference-style bidisperse initial state (Disk::initializeFromConfig,
    src/particles/disk/disk.cu:98-141): first floor(n*count_ratio) particles
    large (diameter size_ratio), rest diameter 1; square box at packing
    fraction phi; positions from the reference's uniform generator."""
    n = int(n)
    n_large = int(n * count_ratio)
    r = np.full(n, 0.5)
    r[:n_large] = size_ratio / 2.0
    area = float(np.sum(r * r)) * np.pi  # sequential order matters little; see oracle
    a = 0.0
    for v in r:
        a += v * v
    area = a * 3.141592653589793238462643383279502884197
    L = (area / phi) ** 0.5
    x = fill_uniform(n, 0.0, L, 0, seed, kind)
    y = fill_uniform(n, 0.0, L, n, seed, kind)
    return dict(x=x, y=y, r=r, m=np.ones(n), box=L)


# ---------------------------------------------------------------------------
# rigid bumpy bodies
# ---------------------------------------------------------------------------
_BSIGS = {
    "create": (P, [I64, I64, D, D, D, D, D, D, C.c_int]),
    "destroy": (None, [P]),
    "set_bodies": (C.c_int, [P, DP, DP, DP, DP, DP, DP, DP, LP]),
    "init_vertices": (None, [P]),
    "set_vertices": (None, [P, DP, DP]),
    "set_mass": (None, [P, D]),
    "setup_neighbors": (C.c_int, [P, C.c_int, D, D, D, D]),
    "check_for_neighbor_update": (C.c_int, [P]),
    "zero": (None, [P]),
    "calculate_forces": (None, [P]),
    "update_velocities": (None, [P, D]),
    "update_positions": (None, [P, D]),
    "mix": (None, [P, D]),
    "set_velocities_zero": (None, [P]),
    "power_fire": (D, [P]),
    "total_pe": (D, [P]),
    "total_ke": (D, [P]),
    "nve_steps": (None, [P, D, I64]),
    "fire_init": (None, [P, D, D]),
    "fire_step": (C.c_int, [P]),
    "get_bodies": (None, [P] + [DP] * 11),
    "get_vertices": (None, [P, DP, DP]),
    "get_vertex_neighbors": (I64, [P, LP, LP]),
    "neighbor_info": (None, [P, C.POINTER(C.c_int), DP, DP, DP, LP, LP, LP, LP]),
    "adam_init": (None, [P]),
    "adam_step": (None, [P, I64, D, D, D, D]),
    "adam_steps": (None, [P, D, D, D, D, I64]),
    "damped_nve_steps": (None, [P, D, D, I64]),
    "wall_only": (None, [P]),
    "wall_and_pair_forces": (None, [P]),
    "nve_wall_steps": (None, [P, D, I64]),
    "stress": (None, [P, DP]),
    "count_contacts": (D, [P]),
    "get_stress": (None, [P, DP, DP, DP, DP]),
    "get_contacts": (None, [P, LP, LP]),
    "save_state": (None, [P]),
    "restore_state": (None, [P]),
    "pair_dump": (I64, [P, C.POINTER(DP), LP, LP, LP]),
}
_blibs: dict[str, C.CDLL] = {}


def _bload(kind):
    lib, _ = _load(kind)
    prefix = "orcb_" if kind == "oracle" else "refb_"
    if kind not in _blibs:
        for name, (res, args) in _BSIGS.items():
            fn = getattr(lib, prefix + name)
            fn.restype = res
            fn.argtypes = args
        if kind == "oracle":
            lib.orcb_minimize_fire.restype = I64
            lib.orcb_minimize_fire.argtypes = [P, D, D, D, D, I64, D, D, C.POINTER(C.c_int)]
            lib.orcb_vertex_radius.restype = D
            lib.orcb_vertex_radius.argtypes = [D, I64, D]
            lib.orcb_minimize_adam.restype = I64
            lib.orcb_minimize_adam.argtypes = [P, D, D, D, D, D, D, I64]
            lib.orcb_damped_forces.restype = None
            lib.orcb_damped_forces.argtypes = [P, D]
            lib.orcb_grad_desc_steps.restype = None
            lib.orcb_grad_desc_steps.argtypes = [P, D, I64]
        _blibs[kind] = lib
    return lib, prefix


def bumpy_vertex_radius(min_diameter, n_vertices_small, seg):
    lib, _ = _bload("oracle")
    return lib.orcb_vertex_radius(float(min_diameter), int(n_vertices_small), float(seg))


class BumpyOracle:
    """Rigid bumpy bodies held by the oracle or by the reference-kernel harness."""

    BODY_KEYS = ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe", "I")

    def __init__(self, n_bodies, n_vertices, box, e_c, n_c, vertex_radius, seg, rotation=True,
                 kind="oracle"):
        self.lib, self.pre = _bload(kind)
        self.nb, self.nv = int(n_bodies), int(n_vertices)
        bx, by = (box, box) if np.isscalar(box) else box
        self.h = self._f("create")(self.nb, self.nv, float(bx), float(by), float(e_c), float(n_c),
                                   float(vertex_radius), float(seg), int(bool(rotation)))

    def _f(self, name):
        return getattr(self.lib, self.pre + name)

    def __del__(self):
        try:
            if self.h:
                self._f("destroy")(self.h)
        except Exception:
            pass

    def set_bodies(self, x, y, th, r, nvb, vx=None, vy=None, w=None):
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
                for a in (x, y, th, vx, vy, w, r)]
        nv = np.ascontiguousarray(nvb, dtype=np.int64)
        rc = self._f("set_bodies")(self.h, *[_dp(a) for a in arrs], _lp(nv))
        if rc != 0:
            raise ValueError("vertex counts do not sum to n_vertices")

    def init_vertices(self):
        self._f("init_vertices")(self.h)

    def set_vertices(self, px, py):
        self._f("set_vertices")(self.h, _dp(np.ascontiguousarray(px, dtype=np.float64)),
                                _dp(np.ascontiguousarray(py, dtype=np.float64)))

    def set_mass(self, m):
        self._f("set_mass")(self.h, float(m))

    def setup_neighbors(self, method=NEIGH_CELL, cutoff_mult=1.5, disp_mult=0.2, ppc=8.0, cdm=0.5):
        return self._f("setup_neighbors")(self.h, int(method), float(cutoff_mult), float(disp_mult),
                                          float(ppc), float(cdm))

    def check_for_neighbor_update(self):
        return self._f("check_for_neighbor_update")(self.h)

    def zero(self):
        self._f("zero")(self.h)

    def calculate_forces(self):
        self._f("calculate_forces")(self.h)

    def update_velocities(self, dt):
        self._f("update_velocities")(self.h, float(dt))

    def update_positions(self, dt):
        self._f("update_positions")(self.h, float(dt))

    def mix(self, alpha):
        self._f("mix")(self.h, float(alpha))

    def set_velocities_zero(self):
        self._f("set_velocities_zero")(self.h)

    def power_fire(self):
        return self._f("power_fire")(self.h)

    def total_pe(self):
        return self._f("total_pe")(self.h)

    def total_ke(self):
        return self._f("total_ke")(self.h)

    def nve_steps(self, dt, n):
        self._f("nve_steps")(self.h, float(dt), int(n))

    def fire_init(self, alpha=0.1, dt=1e-2):
        self._f("fire_init")(self.h, float(alpha), float(dt))

    def fire_step(self):
        return self._f("fire_step")(self.h)

    def minimize_fire(self, alpha=0.1, dt=1e-2, pe_target=1e-16, pe_diff_target=1e-16,
                      num_steps=100000, fmax=0.0, tmax=0.0):
        st = C.c_int()
        n = self.lib.orcb_minimize_fire(self.h, float(alpha), float(dt), float(pe_target),
                                        float(pe_diff_target), int(num_steps), float(fmax),
                                        float(tmax), C.byref(st))
        return n, st.value

    def adam_init(self):
        self._f("adam_init")(self.h)

    def adam_step(self, step, alpha=1e-4, beta1=0.9, beta2=0.999, eps=1e-8):
        self._f("adam_step")(self.h, int(step), float(alpha), float(beta1), float(beta2), float(eps))

    def adam_steps(self, n, alpha=1e-4, beta1=0.9, beta2=0.999, eps=1e-8):
        """n steps of Adam::minimize from fresh moments (no stop test)."""
        self._f("adam_steps")(self.h, float(alpha), float(beta1), float(beta2), float(eps), int(n))

    def minimize_adam(self, alpha=1e-4, beta1=0.9, beta2=0.999, eps=1e-8, pe_target=1e-16,
                      pe_diff_target=1e-16, num_steps=100000):
        return self.lib.orcb_minimize_adam(self.h, float(alpha), float(beta1), float(beta2),
                                           float(eps), float(pe_target), float(pe_diff_target),
                                           int(num_steps))

    def damped_forces(self, gamma):
        self.lib.orcb_damped_forces(self.h, float(gamma))

    def grad_desc_steps(self, alpha, n):
        """GradDesc::step n times with the rigid step (oracle only: the reference
        has no rigid gradient-descent kernel)."""
        self.lib.orcb_grad_desc_steps(self.h, float(alpha), int(n))

    def damped_nve_steps(self, dt, gamma, n):
        self._f("damped_nve_steps")(self.h, float(dt), float(gamma), int(n))

    def wall_only(self):
        self._f("wall_only")(self.h)

    def wall_and_pair_forces(self):
        self._f("wall_and_pair_forces")(self.h)

    def nve_wall_steps(self, dt, n):
        self._f("nve_wall_steps")(self.h, float(dt), int(n))

    def stress(self):
        """calculateStressTensor: (component sums [xx, xy, yx, yy], per-body
        components in static order as a (4, nb) array)."""
        t = np.zeros(4)
        self._f("stress")(self.h, _dp(t))
        per = np.zeros((4, self.nb))
        self._f("get_stress")(self.h, *[_dp(per[k]) for k in range(4)])
        return t, per

    def pressure(self):
        t, _ = self.stress()
        return (t[0] + t[3]) / 2

    def count_contacts(self):
        """countContacts: (getContactCount, per-body contacts, per-body vertex
        contacts), static order."""
        tot = self._f("count_contacts")(self.h)
        cc = np.zeros(self.nb, dtype=np.int64)
        vcc = np.zeros(self.nb, dtype=np.int64)
        self._f("get_contacts")(self.h, _lp(cc), _lp(vcc))
        return tot, cc, vcc

    PAIR_KEYS = ("potential", "force_x", "force_y", "distance_x", "distance_y", "overlap",
                 "radsum", "separation_angle", "angle_i", "angle_j", "friction",
                 "vertex_overlap",
                 "hess_xx", "hess_xy", "hess_xt", "hess_yx", "hess_yy", "hess_yt", "hess_tx",
                 "hess_ty", "hess_tt",
                 "hess_ii_xx", "hess_ii_xy", "hess_ii_xt", "hess_ii_yx", "hess_ii_yy",
                 "hess_ii_yt", "hess_ii_tx", "hess_ii_ty", "hess_ii_tt")

    def pair_dump(self):
        """calculateForceDistancePairs: dict of the 30 per-entry arrays (n * cap,
        [slot * cap + k]) plus this_id, other_id, vertex_contacts."""
        cap = self._f("pair_dump")(self.h, None, None, None, None)
        m = self.nb * cap
        arrs = [np.zeros(m) for _ in self.PAIR_KEYS]
        ptrs = (DP * 30)(*[_dp(a) for a in arrs])
        ti, oi, vc = (np.zeros(m, dtype=np.int64) for _ in range(3))
        self._f("pair_dump")(self.h, ptrs, _lp(ti), _lp(oi), _lp(vc))
        out = dict(zip(self.PAIR_KEYS, arrs))
        out.update(this_id=ti, other_id=oi, vertex_contacts=vc, cap=cap)
        return out

    def save_state(self):
        self._f("save_state")(self.h)

    def restore_state(self):
        self._f("restore_state")(self.h)

    def bodies(self):
        out = {k: np.zeros(self.nb) for k in self.BODY_KEYS}
        self._f("get_bodies")(self.h, *[_dp(out[k]) for k in self.BODY_KEYS])
        return out

    def vertices(self):
        px, py = np.zeros(self.nv), np.zeros(self.nv)
        self._f("get_vertices")(self.h, _dp(px), _dp(py))
        return px, py

    def vertex_neighbor_sets(self):
        cap = self._f("get_vertex_neighbors")(self.h, None, None)
        lst = np.zeros(self.nv * cap, dtype=np.int64)
        cnt = np.zeros(self.nv, dtype=np.int64)
        self._f("get_vertex_neighbors")(self.h, _lp(lst), _lp(cnt))
        lst = lst.reshape(self.nv, cap)
        return [frozenset(int(u) for u in lst[v, :cnt[v]]) for v in range(self.nv)]

    def neighbor_info(self):
        m = C.c_int()
        c, vc, t = D(), D(), D()
        cap, vcap, nr, ncr = I64(), I64(), I64(), I64()
        self._f("neighbor_info")(self.h, C.byref(m), C.byref(c), C.byref(vc), C.byref(t),
                                 C.byref(cap), C.byref(vcap), C.byref(nr), C.byref(ncr))
        return dict(method=m.value, cutoff=c.value, vertex_cutoff=vc.value, thr2=t.value,
                    cap=cap.value, vertex_cap=vcap.value, n_rebuilds=nr.value,
                    n_cell_rebuilds=ncr.value)


def bumpy_packing(n_bodies, phi, seed, n_small=20, seg=0.9, size_ratio=1.4, count_ratio=0.5,
                  kind="oracle"):
    """Reference-style rigid bumpy initial state (RigidBumpy::initializeFromConfig,
    src/particles/rigid_bumpy/rigid_bumpy.cu:138-230): bidisperse radii, vertex
    counts n_small / floor(n_small * d_max / d_min), vertex radius from the
    segment rule, box at packing fraction phi of the disk area, positions and
    angles from the reference's uniform generator (angles share the positions'
    x stream, as the reference's offsets do), vertex energy scale
    e_c * (2 r_v / d_min)^2."""
    n = int(n_bodies)
    n_large = int(n * count_ratio)
    r = np.full(n, 0.5)
    r[:n_large] = size_ratio / 2.0
    a = 0.0
    for v in r:
        a += v * v
    L = (a * 3.141592653589793238462643383279502884197 / phi) ** 0.5
    x = fill_uniform(n, 0.0, L, 0, seed, kind)
    y = fill_uniform(n, 0.0, L, n, seed, kind)
    th = fill_uniform(n, 0.0, 2 * np.pi, 0, seed, kind)
    d_min, d_max = 1.0, size_ratio
    n_lg = int(n_small * d_max / d_min)
    nvb = np.where(r == d_max / 2.0, n_lg, n_small).astype(np.int64)
    rv = bumpy_vertex_radius(d_min, n_small, seg)
    e_c = 1.0 * (2.0 * rv / d_min) ** 2
    return dict(x=x, y=y, th=th, r=r, nvb=nvb, nv=int(nvb.sum()), box=L, rv=rv, e_c=e_c, seg=seg)


class _OrcJamResult(C.Structure):
    _fields_ = [("packing_fraction", D), ("pressure", D), ("box_length", D), ("contacts", D),
                ("compression_steps", I64), ("fire_steps_total", I64), ("status", C.c_int)]


def _jam_result(r):
    return dict(packing_fraction=r.packing_fraction, pressure=r.pressure,
                box_length=r.box_length, contacts=r.contacts,
                compression_steps=r.compression_steps, fire_steps_total=r.fire_steps_total,
                status=r.status)


def jam_pressure(o: DiskOracle, p_low, p_high, compression_rate=0.99, length_tol=1e-10,
                 decompress=1.01, max_steps=1000, fire=(0.1, 1e-2, 1e-16, 1e-16, 100000),
                 neighbors=(0, 1.5, 0.2, 8.0, 0.5)):
    """scripts/runArthurJamWithFire.cpp control flow on the oracle."""
    lib = o.lib
    fn = lib.orc_jam_pressure
    fn.restype = None
    fn.argtypes = [P, D, D, D, D, D, I64, D, D, D, D, I64, C.c_int, D, D, D, D,
                   C.POINTER(_OrcJamResult)]
    r = _OrcJamResult()
    fn(o.h, p_low, p_high, compression_rate, length_tol, decompress, int(max_steps),
       float(fire[0]), float(fire[1]), float(fire[2]), float(fire[3]), int(fire[4]),
       int(neighbors[0]), *[float(v) for v in neighbors[1:]], C.byref(r))
    return _jam_result(r)


def jam_phi(o: DiskOracle, tol, dtol, phi_tol, increment, dphi_stab, max_steps=1000):
    """scripts/runJam.cpp control flow on the oracle."""
    fn = o.lib.orc_jam_phi
    fn.restype = None
    fn.argtypes = [P, D, D, D, D, D, I64, C.POINTER(_OrcJamResult)]
    r = _OrcJamResult()
    fn(o.h, tol, dtol, phi_tol, increment, dphi_stab, int(max_steps), C.byref(r))
    return _jam_result(r)
