"""Disk system and integrators over the C ABI.

Method names follow the reference's Particle class
(include/particles/base/particle.h) so code written against the reference
reads the same; integrators follow include/integrator/{nve,fire,adam}.h and the
routines follow src/routines/minimization.cu.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .lib import (D, DP, FireParams, FireResult, I32, I64, NeighborConfig, NeighborInfo, Params,
                  check, load_library)

NEIGH_CELL, NEIGH_VERLET, NEIGH_ALL = 0, 1, 2
_METHODS = {"cell": NEIGH_CELL, "verlet": NEIGH_VERLET, "all": NEIGH_ALL}
FP64, MIXED = 0, 1
HOST, DEVICE = 0, 1


def _ptr(a, n=None):
    """(pointer, where) for a numpy array (host) or a CUDA tensor (device)."""
    if a is None:
        return None, HOST
    if hasattr(a, "data_ptr"):  # torch tensor
        if a.is_cuda:
            if a.dtype.__repr__() != "torch.float64" or not a.is_contiguous():
                raise TypeError("device arrays must be contiguous float64")
            return C.cast(C.c_void_p(a.data_ptr()), DP), DEVICE
        a = a.numpy()
    arr = np.ascontiguousarray(a, dtype=np.float64)
    if n is not None and arr.shape != (n,):
        raise ValueError(f"expected shape ({n},), got {arr.shape}")
    return arr, HOST


class Disk:
    """One system of soft disks on the GPU (Disk, include/particles/disk/disk.h)."""

    def __init__(self, n_particles, box_size, e_c=1.0, n_c=2.0, precision=FP64, stream=None):
        self.lib = load_library()
        self.n = int(n_particles)
        bx, by = (box_size, box_size) if np.isscalar(box_size) else box_size
        prm = Params(self.n, float(bx), float(by), float(e_c), float(n_c), int(precision), 0)
        h = C.c_void_p()
        check(self.lib.dpg_create(C.byref(prm), C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h
        self.e_c, self.n_c = float(e_c), float(n_c)

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- state -----------------------------------------------------------
    def setState(self, positions_x=None, positions_y=None, velocities_x=None, velocities_y=None,
                 radii=None, masses=None):
        """Positions, velocities, radii, masses in static order (host numpy or CUDA tensors)."""
        arrs = [positions_x, positions_y, velocities_x, velocities_y, radii, masses]
        ptrs, wheres, keep = [], set(), []
        for a in arrs:
            p, w = _ptr(a, self.n)
            keep.append(p)
            if a is not None:
                wheres.add(w)
            ptrs.append(p.ctypes.data_as(DP) if isinstance(p, np.ndarray) else p)
        if len(wheres) > 1:
            raise ValueError("mix of host and device arrays")
        where = wheres.pop() if wheres else HOST
        check(self.lib.dpg_set_state(self.h, *ptrs, where))

    def setForces(self, fx, fy):
        px, w = _ptr(fx, self.n)
        py, _ = _ptr(fy, self.n)
        check(self.lib.dpg_set_forces(self.h, px.ctypes.data_as(DP), py.ctypes.data_as(DP), w))

    def getState(self):
        """dict of x, y, vx, vy, fx, fy, pe (numpy, static order)."""
        out = {k: np.zeros(self.n) for k in ("x", "y", "vx", "vy", "fx", "fy", "pe")}
        check(self.lib.dpg_get_state(self.h, *[out[k].ctypes.data_as(DP) for k in
                                                ("x", "y", "vx", "vy", "fx", "fy", "pe")], HOST))
        return out

    def getStateDevice(self, out):
        """Write x, y, vx, vy, fx, fy, pe into CUDA tensors given in `out` (missing keys skipped)."""
        keys = ("x", "y", "vx", "vy", "fx", "fy", "pe")
        ptrs = [(_ptr(out[k])[0] if k in out else None) for k in keys]
        check(self.lib.dpg_get_state(self.h, *ptrs, DEVICE))

    def setBoxSize(self, box):
        bx, by = (box, box) if np.isscalar(box) else box
        check(self.lib.dpg_set_box(self.h, float(bx), float(by)))

    def getBoxSize(self):
        bx, by = D(), D()
        check(self.lib.dpg_get_box(self.h, C.byref(bx), C.byref(by)))
        return np.array([bx.value, by.value])

    def synchronize(self):
        check(self.lib.dpg_synchronize(self.h))

    # ---- neighbours --------------------------------------------------------
    def setupNeighbors(self, neighbor_list_update_method="cell", neighbor_cutoff_multiplier=1.5,
                       neighbor_displacement_multiplier=0.2, num_particles_per_cell=8.0,
                       cell_displacement_multiplier=0.5):
        """Particle::setupNeighbors (src/particles/base/particle.cu:71-100)."""
        m = _METHODS.get(neighbor_list_update_method, neighbor_list_update_method)
        cfg = NeighborConfig(int(m), float(neighbor_cutoff_multiplier),
                             float(neighbor_displacement_multiplier),
                             float(num_particles_per_cell), float(cell_displacement_multiplier))
        info = NeighborInfo()
        check(self.lib.dpg_setup_neighbors(self.h, C.byref(cfg), C.byref(info)))
        return self._info(info)

    @staticmethod
    def _info(info):
        return dict(method=info.method, capacity=info.capacity, n_cells_dim=info.n_cells_dim,
                    cutoff=info.cutoff, neighbor_threshold_sq=info.neighbor_threshold_sq,
                    cell_size=info.cell_size, cell_threshold_sq=info.cell_threshold_sq,
                    n_rebuilds=info.n_rebuilds, n_cell_rebuilds=info.n_cell_rebuilds)

    def neighborInfo(self):
        info = NeighborInfo()
        check(self.lib.dpg_neighbor_info_get(self.h, C.byref(info)))
        return self._info(info)

    def updateNeighborList(self):
        check(self.lib.dpg_build_neighbors(self.h))

    def checkForNeighborUpdate(self):
        r = C.c_int()
        check(self.lib.dpg_check_neighbors(self.h, C.byref(r)))
        return r.value

    def getNeighbors(self):
        """(list[n, cap] int32 of static indices, -1 padded; counts[n]) keyed by static index."""
        cap = C.c_int(0)
        check(self.lib.dpg_get_neighbors(self.h, None, None, C.byref(cap)))
        c = max(cap.value, 1)
        lst = np.zeros(self.n * c, dtype=np.int32)
        cnt = np.zeros(self.n, dtype=np.int32)
        capio = C.c_int(c)
        check(self.lib.dpg_get_neighbors(self.h, lst.ctypes.data_as(C.POINTER(C.c_int32)),
                                         cnt.ctypes.data_as(C.POINTER(C.c_int32)), C.byref(capio)))
        return lst.reshape(self.n, c), cnt

    def getNeighborSets(self):
        lst, cnt = self.getNeighbors()
        return [frozenset(int(j) for j in lst[i, :cnt[i]] if j >= 0) for i in range(self.n)]

    def getCells(self):
        info = self.neighborInfo()
        ncells = max(info["n_cells_dim"], 0) ** 2
        ci = np.zeros(self.n, dtype=np.int64)
        si = np.zeros(self.n, dtype=np.int64)
        cs = np.zeros(ncells + 1, dtype=np.int64)
        p = C.POINTER(C.c_int64)
        check(self.lib.dpg_get_cells(self.h, ci.ctypes.data_as(p), cs.ctypes.data_as(p),
                                     si.ctypes.data_as(p)))
        return ci, cs, si

    # ---- dynamics -------------------------------------------------------------
    def zeroForceAndPotentialEnergy(self):
        check(self.lib.dpg_zero_forces(self.h))

    def calculateForces(self):
        check(self.lib.dpg_compute_forces(self.h))

    def updateVelocities(self, dt):
        check(self.lib.dpg_kick(self.h, float(dt)))

    def updatePositions(self, dt):
        check(self.lib.dpg_drift(self.h, float(dt)))

    def mixVelocitiesAndForces(self, alpha):
        check(self.lib.dpg_mix(self.h, float(alpha)))

    def setVelocitiesToZero(self):
        check(self.lib.dpg_zero_velocities(self.h))

    def getPowerFire(self):
        p = D()
        check(self.lib.dpg_power_fire(self.h, C.byref(p)))
        return p.value

    def totalPotentialEnergy(self):
        pe, ke = D(), D()
        check(self.lib.dpg_reduce_energies(self.h, C.byref(pe), C.byref(ke)))
        return pe.value

    def totalKineticEnergy(self):
        pe, ke = D(), D()
        check(self.lib.dpg_reduce_energies(self.h, C.byref(pe), C.byref(ke)))
        return ke.value

    def forceStats(self):
        mx, bal = D(), D()
        check(self.lib.dpg_force_stats(self.h, C.byref(mx), C.byref(bal)))
        return mx.value, bal.value

    def getStressTensor(self):
        p = D()
        st = (D * 4)()
        check(self.lib.dpg_pressure(self.h, C.byref(p), st))
        return np.array(list(st))

    def getPressure(self):
        p = D()
        check(self.lib.dpg_pressure(self.h, C.byref(p), None))
        return p.value

    def getContactCount(self):
        c = D()
        check(self.lib.dpg_contact_count(self.h, C.byref(c)))
        return c.value

    def getPackingFraction(self):
        phi = D()
        check(self.lib.dpg_packing_fraction(self.h, C.byref(phi)))
        return phi.value

    def scaleBox(self, factor):
        check(self.lib.dpg_scale_box(self.h, float(factor)))

    def scaleToPackingFractionFull(self, phi):
        check(self.lib.dpg_scale_to_packing_fraction(self.h, float(phi)))

    def setLastState(self):
        check(self.lib.dpg_save_state(self.h))

    def revertToLastState(self):
        check(self.lib.dpg_restore_state(self.h))

    def initAdamVariables(self):
        check(self.lib.dpg_adam_init(self.h))

    def updatePositionsAdam(self, step, alpha, beta1, beta2, epsilon):
        check(self.lib.dpg_adam_step(self.h, int(step), float(alpha), float(beta1), float(beta2),
                                     float(epsilon)))

    # ---- device-resident loops ---------------------------------------------
    def nveSteps(self, dt, n_steps):
        check(self.lib.dpg_nve_steps(self.h, float(dt), int(n_steps)))

    def setMixedSwitch(self, switch_fmax):
        """DPG_MIXED systems: max|F| below which FIRE continues in FP64."""
        check(self.lib.dpg_set_mixed_switch(self.h, float(switch_fmax)))

    def setForceGroup(self, lanes):
        """Threads per particle (1, 2, 4, 8) of the FP64 force kernels (identical sums)."""
        check(self.lib.dpg_set_force_group(self.h, int(lanes)))

    def autotuneForceGroup(self, iters=50):
        """Times force passes with 1, 2, 4, 8 lanes per particle, keeps the fastest;
        returns (lanes, microseconds per pass for each group)."""
        chosen = I32()
        us = (C.c_double * 4)()
        check(self.lib.dpg_autotune_force_group(self.h, int(iters), C.byref(chosen), us))
        return chosen.value, dict(zip((1, 2, 4, 8), list(us)))

    def writeState(self, directory, step=-1):
        """State files in the reference's layout (positions.dat, radii.dat, ...)."""
        check(self.lib.dpg_write_state(self.h, str(directory).encode(), int(step)))

    def readState(self, directory):
        """Load positions, velocities, radii, masses and box from a state directory."""
        check(self.lib.dpg_read_state(self.h, str(directory).encode()))

    @staticmethod
    def stateCount(directory):
        """Number of particles stored in a state directory."""
        lib = load_library()
        n = C.c_int64()
        check(lib.dpg_state_count(str(directory).encode(), C.byref(n)))
        return n.value

    PAIR_KEYS = ("potential", "force_x", "force_y", "distance_x", "distance_y", "overlap",
                 "radsum", "angle", "hess_xx", "hess_xy", "hess_yx", "hess_yy",
                 "hess_ii_xx", "hess_ii_xy", "hess_ii_yx", "hess_ii_yy")

    def calculateForceDistancePairs(self):
        """Pair energies, forces, separations, ids, overlaps, angles and Hessian
        blocks per neighbour-list entry ([slot * cap + k], current order), as
        the reference's Disk::calculateForceDistancePairs."""
        cap = self.neighborInfo()["capacity"]
        m = self.n * cap
        out = {k: np.zeros(m) for k in self.PAIR_KEYS}
        ptrs = (DP * 16)(*[out[k].ctypes.data_as(DP) for k in self.PAIR_KEYS])
        ti, oi = np.zeros(m, dtype=np.int64), np.zeros(m, dtype=np.int64)
        check(self.lib.dpg_pair_dump(self.h, ptrs, ti.ctypes.data_as(C.POINTER(C.c_int64)),
                                     oi.ctypes.data_as(C.POINTER(C.c_int64)), HOST))
        out["this_id"], out["other_id"] = ti, oi
        return out

    def calculateWallForces(self):
        """Disk::calculateWallForces: += hard-wall forces at 0 and L."""
        check(self.lib.dpg_wall_forces(self.h))

    def nveWallSteps(self, dt, n_steps):
        """n NVE::wall_step (walls added before the pair forces)."""
        check(self.lib.dpg_nve_wall_steps(self.h, float(dt), int(n_steps)))

    def calculateDampedForces(self, damping_coefficient):
        check(self.lib.dpg_damped_forces(self.h, float(damping_coefficient)))

    def dampedNveSteps(self, dt, damping_coefficient, n_steps):
        check(self.lib.dpg_damped_nve_steps(self.h, float(dt), float(damping_coefficient),
                                            int(n_steps)))

    def updatePositionsGradDesc(self, alpha):
        check(self.lib.dpg_grad_desc_step(self.h, float(alpha)))

    def gradDescSteps(self, alpha, n_steps):
        check(self.lib.dpg_grad_desc_steps(self.h, float(alpha), int(n_steps)))


class NVE:
    """NVE velocity Verlet (src/integrator/nve.cu:15-25)."""

    def __init__(self, particle: Disk, dt: float):
        self.particle, self.dt = particle, float(dt)

    def step(self):
        self.particle.nveSteps(self.dt, 1)

    def run(self, n_steps):
        self.particle.nveSteps(self.dt, n_steps)


class DampedNVE:
    """Velocity Verlet with F -= damping v (src/integrator/damped_nve.cu:15-27)."""

    def __init__(self, particle: Disk, dt: float, damping_coefficient: float):
        self.particle, self.dt, self.damping = particle, float(dt), float(damping_coefficient)

    def step(self):
        self.particle.dampedNveSteps(self.dt, self.damping, 1)

    def run(self, n_steps):
        self.particle.dampedNveSteps(self.dt, self.damping, n_steps)


class GradDesc:
    """Gradient descent x += alpha F (src/integrator/grad_desc.cu:11-17)."""

    def __init__(self, particle: Disk, alpha: float):
        self.particle, self.alpha = particle, float(alpha)

    def step(self):
        self.particle.gradDescSteps(self.alpha, 1)

    def run(self, n_steps):
        self.particle.gradDescSteps(self.alpha, n_steps)


class Fire:
    """FIRE (include/integrator/fire.h, src/integrator/fire.cu)."""

    def __init__(self, particle: Disk, alpha_init=0.1, dt=1e-2):
        self.particle = particle
        check(particle.lib.dpg_fire_init(particle.h, float(alpha_init), float(dt)))

    def step(self):
        st = C.c_int()
        check(self.particle.lib.dpg_fire_step(self.particle.h, C.byref(st)))
        return st.value

    def state(self):
        a, dt = D(), D()
        ng, nb = C.c_int64(), C.c_int64()
        st = C.c_int()
        check(self.particle.lib.dpg_fire_get(self.particle.h, C.byref(a), C.byref(dt),
                                             C.byref(ng), C.byref(nb), C.byref(st)))
        return dict(alpha=a.value, dt=dt.value, n_good=ng.value, n_bad=nb.value,
                    stopped=st.value)


class Adam:
    """Adam (src/integrator/adam.cu)."""

    def __init__(self, particle: Disk, alpha=1e-4, beta1=0.9, beta2=0.999, epsilon=1e-8):
        self.particle = particle
        self.alpha, self.beta1, self.beta2, self.epsilon = alpha, beta1, beta2, epsilon

    def minimize(self, step):
        p = self.particle
        p.zeroForceAndPotentialEnergy()
        p.checkForNeighborUpdate()
        p.calculateForces()
        p.updatePositionsAdam(step, self.alpha, self.beta1, self.beta2, self.epsilon)


def minimizeFire(particle: Disk, alpha_init=0.1, dt=1e-2, avg_pe_target=1e-16,
                 avg_pe_diff_target=1e-16, num_steps=100000, fmax_target=0.0):
    """minimizeFire (src/routines/minimization.cu:75-112), run on the device."""
    prm = FireParams(float(alpha_init), float(dt), float(avg_pe_target), float(avg_pe_diff_target),
                     int(num_steps), float(fmax_target))
    res = FireResult()
    check(particle.lib.dpg_fire_minimize(particle.h, C.byref(prm), C.byref(res)))
    return dict(steps=res.steps, stopped=res.stopped, converged=res.converged,
                avg_pe=res.avg_pe, max_force=res.max_force, alpha=res.alpha, dt=res.dt)


def minimizeAdam(particle: Disk, alpha=1e-4, beta1=0.9, beta2=0.999, epsilon=1e-8,
                 avg_pe_target=1e-16, avg_pe_diff_target=1e-16, num_steps=100000):
    """minimizeAdam (src/routines/minimization.cu:3-33)."""
    steps = C.c_int64()
    check(particle.lib.dpg_adam_minimize(particle.h, float(alpha), float(beta1), float(beta2),
                                         float(epsilon), float(avg_pe_target),
                                         float(avg_pe_diff_target), int(num_steps),
                                         C.byref(steps)))
    return steps.value


def jamPressure(particle: Disk, pressure_low, pressure_high, compression_rate=0.99,
                length_tolerance=1e-10, decompress_factor=1.01, max_compression_steps=1000,
                fire=(0.1, 1e-2, 1e-16, 1e-16, 100000), neighbors=("cell", 1.5, 0.2, 8.0, 0.5)):
    """Pressure-band jamming (scripts/runArthurJamWithFire.cpp) through the C ABI."""
    from .lib import JamParams, JamResult
    m = _METHODS.get(neighbors[0], neighbors[0])
    prm = JamParams(float(pressure_low), float(pressure_high), float(compression_rate),
                    float(length_tolerance), float(decompress_factor), int(max_compression_steps),
                    FireParams(float(fire[0]), float(fire[1]), float(fire[2]), float(fire[3]),
                               int(fire[4]), float(fire[5]) if len(fire) > 5 else 0.0),
                    NeighborConfig(int(m), *[float(v) for v in neighbors[1:]]))
    r = JamResult()
    check(particle.lib.dpg_jam_pressure(particle.h, C.byref(prm), C.byref(r)))
    return dict(packing_fraction=r.packing_fraction, pressure=r.pressure, box_length=r.box_length,
                contacts=r.contacts, compression_steps=r.compression_steps,
                fire_steps_total=r.fire_steps_total, status=r.status)


def jamPhi(particle: Disk, avg_pe_tolerance, avg_pe_diff_tolerance, phi_tolerance,
           compression_increment, delta_phi_stability, max_compression_steps=1000):
    """Energy-criterion jamming (scripts/runJam.cpp) through the C ABI."""
    from .lib import JamPhiParams, JamResult
    prm = JamPhiParams(float(avg_pe_tolerance), float(avg_pe_diff_tolerance), float(phi_tolerance),
                       float(compression_increment), float(delta_phi_stability),
                       int(max_compression_steps))
    r = JamResult()
    check(particle.lib.dpg_jam_phi(particle.h, C.byref(prm), C.byref(r)))
    return dict(packing_fraction=r.packing_fraction, pressure=r.pressure, box_length=r.box_length,
                contacts=r.contacts, compression_steps=r.compression_steps,
                fire_steps_total=r.fire_steps_total, status=r.status)
