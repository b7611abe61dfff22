"""Rigid bumpy bodies over the C ABI (RigidBumpy, include/particles/rigid_bumpy/rigid_bumpy.h).

Method names follow the reference's RigidBumpy / Particle classes.  Arrays are
numpy, in static order (bodies) and static vertex order (vertices).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .disk import _METHODS
from .lib import (D, DP, I32P, I64, I64P, BumpyParams, FireParams, FireResult, NeighborConfig,
                  NeighborInfo, check, load_library)


def _d(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


class RigidBumpy:
    """One system of rigid bumpy bodies on the GPU."""

    BODY_KEYS = ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe", "I")

    def __init__(self, n_bodies, n_vertices, box_size, e_c, n_c, vertex_radius,
                 segment_length_per_vertex_diameter, rotation=True, stream=None, precision=0):
        """precision 0 = DPG_FP64 (the reference arithmetic), 1 = DPG_MIXED (FP32
        vertex pairs, FP64 torques and body sums, FP64 refinement in FIRE)."""
        self.lib = load_library()
        self.nb, self.nv = int(n_bodies), int(n_vertices)
        bx, by = (box_size, box_size) if np.isscalar(box_size) else box_size
        prm = BumpyParams(self.nb, self.nv, float(bx), float(by), float(e_c), float(n_c),
                          float(vertex_radius), float(segment_length_per_vertex_diameter),
                          int(bool(rotation)), int(precision))
        h = C.c_void_p()
        check(self.lib.dpg_bumpy_create(C.byref(prm), C.c_void_p(stream) if stream else None,
                                        C.byref(h)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_bumpy_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def setBodies(self, x, y, angles, radii, n_vertices_per_body, vx=None, vy=None, omega=None):
        arrs = [_d(a) for a in (x, y, angles, vx, vy, omega, radii)]
        nvb = np.ascontiguousarray(n_vertices_per_body, dtype=np.int32)
        self._keep = (arrs, nvb)
        check(self.lib.dpg_bumpy_set_bodies(
            self.h, *[None if a is None else a.ctypes.data_as(DP) for a in arrs],
            nvb.ctypes.data_as(I32P)))

    def setVertexPositions(self, px, py):
        px, py = _d(px), _d(py)
        check(self.lib.dpg_bumpy_set_vertices(self.h, px.ctypes.data_as(DP), py.ctypes.data_as(DP)))

    def setMass(self, mass):
        check(self.lib.dpg_bumpy_set_mass(self.h, float(mass)))

    def getBodies(self):
        out = {k: np.zeros(self.nb) for k in self.BODY_KEYS}
        check(self.lib.dpg_bumpy_get_bodies(
            self.h, *[out[k].ctypes.data_as(DP) for k in
                      ("x", "y", "th", "vx", "vy", "w", "fx", "fy", "tq", "pe", "I")]))
        return out

    def getVertexPositions(self):
        px, py = np.zeros(self.nv), np.zeros(self.nv)
        check(self.lib.dpg_bumpy_get_vertices(self.h, px.ctypes.data_as(DP), py.ctypes.data_as(DP)))
        return px, py

    def setupNeighbors(self, neighbor_list_update_method="cell", neighbor_cutoff_multiplier=1.5,
                       neighbor_displacement_multiplier=0.2, num_particles_per_cell=8.0,
                       cell_displacement_multiplier=0.5):
        m = _METHODS.get(neighbor_list_update_method, neighbor_list_update_method)
        cfg = NeighborConfig(int(m), float(neighbor_cutoff_multiplier),
                             float(neighbor_displacement_multiplier), float(num_particles_per_cell),
                             float(cell_displacement_multiplier))
        info = NeighborInfo()
        check(self.lib.dpg_bumpy_setup_neighbors(self.h, C.byref(cfg), C.byref(info)))
        return self.neighborInfo()

    def neighborInfo(self):
        info = NeighborInfo()
        vcap = C.c_int()
        check(self.lib.dpg_bumpy_neighbor_info_get(self.h, C.byref(info), C.byref(vcap)))
        return dict(method=info.method, capacity=info.capacity, vertex_capacity=vcap.value,
                    n_cells_dim=info.n_cells_dim, cutoff=info.cutoff,
                    neighbor_threshold_sq=info.neighbor_threshold_sq,
                    n_rebuilds=info.n_rebuilds, n_cell_rebuilds=info.n_cell_rebuilds)

    def checkForNeighborUpdate(self):
        r = C.c_int()
        check(self.lib.dpg_bumpy_check_neighbors(self.h, C.byref(r)))
        return r.value

    def getVertexNeighborSets(self):
        cap = C.c_int(0)
        check(self.lib.dpg_bumpy_get_vertex_neighbors(self.h, None, None, C.byref(cap)))
        c = max(cap.value, 1)
        lst = np.zeros(self.nv * c, dtype=np.int32)
        cnt = np.zeros(self.nv, dtype=np.int32)
        capio = C.c_int(c)
        check(self.lib.dpg_bumpy_get_vertex_neighbors(self.h, lst.ctypes.data_as(I32P),
                                                      cnt.ctypes.data_as(I32P), C.byref(capio)))
        lst = lst.reshape(self.nv, c)
        return [frozenset(int(u) for u in lst[v, :cnt[v]]) for v in range(self.nv)]

    def zeroForceAndPotentialEnergy(self):
        check(self.lib.dpg_bumpy_zero_forces(self.h))

    def calculateForces(self):
        check(self.lib.dpg_bumpy_compute_forces(self.h))

    def updateVelocities(self, dt):
        check(self.lib.dpg_bumpy_kick(self.h, float(dt)))

    def updatePositions(self, dt):
        check(self.lib.dpg_bumpy_drift(self.h, float(dt)))

    def mixVelocitiesAndForces(self, alpha):
        check(self.lib.dpg_bumpy_mix(self.h, float(alpha)))

    def setVelocitiesToZero(self):
        check(self.lib.dpg_bumpy_zero_velocities(self.h))

    def observables(self):
        v = [D() for _ in range(5)]
        check(self.lib.dpg_bumpy_observables(self.h, *[C.byref(x) for x in v]))
        return dict(pe=v[0].value, ke=v[1].value, power=v[2].value, max_force=v[3].value,
                    max_torque=v[4].value)

    def totalPotentialEnergy(self):
        return self.observables()["pe"]

    def totalKineticEnergy(self):
        return self.observables()["ke"]

    def getPowerFire(self):
        return self.observables()["power"]

    def nveSteps(self, dt, n):
        check(self.lib.dpg_bumpy_nve_steps(self.h, float(dt), int(n)))

    def fireInit(self, alpha_init=0.1, dt=1e-2):
        check(self.lib.dpg_bumpy_fire_init(self.h, float(alpha_init), float(dt)))

    def fireStep(self):
        st = C.c_int()
        check(self.lib.dpg_bumpy_fire_step(self.h, C.byref(st)))
        return st.value

    def minimizeFire(self, alpha_init=0.1, dt=1e-2, avg_pe_target=1e-16, avg_pe_diff_target=1e-16,
                     num_steps=100000, fmax_target=0.0, tmax_target=0.0):
        prm = FireParams(float(alpha_init), float(dt), float(avg_pe_target),
                         float(avg_pe_diff_target), int(num_steps), float(fmax_target))
        res = FireResult()
        check(self.lib.dpg_bumpy_fire_minimize(self.h, C.byref(prm), float(tmax_target),
                                               C.byref(res)))
        return dict(steps=res.steps, stopped=res.stopped, converged=res.converged,
                    avg_pe=res.avg_pe, max_force=res.max_force)

    def setMixedSwitch(self, switch_fmax):
        check(self.lib.dpg_bumpy_set_mixed_switch(self.h, float(switch_fmax)))

    def scaleBox(self, factor):
        check(self.lib.dpg_bumpy_scale_box(self.h, float(factor)))

    # ---- Adam (RigidBumpy::updatePositionsAdam, minimizeAdam) ------------------
    def initAdamVariables(self):
        check(self.lib.dpg_bumpy_adam_init(self.h))

    def updatePositionsAdam(self, step, alpha, beta1, beta2, epsilon):
        check(self.lib.dpg_bumpy_adam_step(self.h, int(step), float(alpha), float(beta1),
                                           float(beta2), float(epsilon)))

    def adamMinimizeStep(self, step, alpha=1e-4, beta1=0.9, beta2=0.999, epsilon=1e-8):
        """Adam::minimize(step): zero, neighbour check, forces, Adam update."""
        self.zeroForceAndPotentialEnergy()
        self.checkForNeighborUpdate()
        self.calculateForces()
        self.updatePositionsAdam(step, alpha, beta1, beta2, epsilon)

    def minimizeAdam(self, alpha=1e-4, beta1=0.9, beta2=0.999, epsilon=1e-8, avg_pe_target=1e-16,
                     avg_pe_diff_target=1e-16, num_steps=100000):
        steps = I64()
        check(self.lib.dpg_bumpy_adam_minimize(self.h, float(alpha), float(beta1), float(beta2),
                                               float(epsilon), float(avg_pe_target),
                                               float(avg_pe_diff_target), int(num_steps),
                                               C.byref(steps)))
        return steps.value

    # ---- gradient descent (rigid update; see dpg_bumpy_grad_desc_step) -------------
    def updatePositionsGradDesc(self, alpha):
        check(self.lib.dpg_bumpy_grad_desc_step(self.h, float(alpha)))

    def gradDescSteps(self, alpha, n):
        check(self.lib.dpg_bumpy_grad_desc_steps(self.h, float(alpha), int(n)))

    # ---- DampedNVE and walls ------------------------------------------------------
    def calculateDampedForces(self, damping_coefficient):
        check(self.lib.dpg_bumpy_damped_forces(self.h, float(damping_coefficient)))

    def dampedNveSteps(self, dt, damping_coefficient, n):
        check(self.lib.dpg_bumpy_damped_nve_steps(self.h, float(dt), float(damping_coefficient),
                                                  int(n)))

    def calculateWallForces_onlyWallContacts(self):
        check(self.lib.dpg_bumpy_wall_forces(self.h, 0))

    def calculateWallAndPairForces(self):
        """calculateWallForces() then calculateForces(), as NVE::wall_step calls them."""
        check(self.lib.dpg_bumpy_wall_forces(self.h, 1))

    def nveWallSteps(self, dt, n):
        check(self.lib.dpg_bumpy_nve_wall_steps(self.h, float(dt), int(n)))

    # ---- stress, pressure, contacts ----------------------------------------------
    def calculateStressTensor(self):
        """(component sums [xx, xy, yx, yy], per-body components (4, nb) in static order)."""
        t = np.zeros(4)
        per = np.zeros((4, self.nb))
        p = D()
        check(self.lib.dpg_bumpy_stress(self.h, t.ctypes.data_as(DP), C.byref(p),
                                        per.ctypes.data_as(DP)))
        return t, per

    def getPressure(self):
        p = D()
        check(self.lib.dpg_bumpy_stress(self.h, None, C.byref(p), None))
        return p.value

    def countContacts(self):
        """(getContactCount, getVertexContactCount, per-body contacts, per-body
        vertex contacts), static order."""
        c, vc = D(), D()
        cc = np.zeros(self.nb, dtype=np.int32)
        vcc = np.zeros(self.nb, dtype=np.int32)
        check(self.lib.dpg_bumpy_contacts(self.h, C.byref(c), C.byref(vc), cc.ctypes.data_as(I32P),
                                          vcc.ctypes.data_as(I32P)))
        return c.value, vc.value, cc, vcc

    def getContactCount(self):
        c = D()
        check(self.lib.dpg_bumpy_contacts(self.h, C.byref(c), None, None, None))
        return c.value

    # ---- pair and Hessian dump -----------------------------------------------------
    PAIR_KEYS = ("potential", "force_x", "force_y", "distance_x", "distance_y", "overlap",
                 "radsum", "separation_angle", "angle_i", "angle_j", "friction",
                 "vertex_overlap",
                 "hess_xx", "hess_xy", "hess_xt", "hess_yx", "hess_yy", "hess_yt", "hess_tx",
                 "hess_ty", "hess_tt",
                 "hess_ii_xx", "hess_ii_xy", "hess_ii_xt", "hess_ii_yx", "hess_ii_yy",
                 "hess_ii_yt", "hess_ii_tx", "hess_ii_ty", "hess_ii_tt")

    def calculateForceDistancePairs(self):
        """dict of the 30 per-entry arrays ([slot * cap + k]) plus this_id,
        other_id, vertex_contacts and cap."""
        cap = self.neighborInfo()["capacity"]
        m = self.nb * cap
        arrs = [np.zeros(m) for _ in self.PAIR_KEYS]
        ptrs = (DP * 30)(*[a.ctypes.data_as(DP) for a in arrs])
        ids = [np.zeros(m, dtype=np.int64) for _ in range(3)]
        check(self.lib.dpg_bumpy_pair_dump(self.h, ptrs, *[a.ctypes.data_as(I64P) for a in ids], 0))
        out = dict(zip(self.PAIR_KEYS, arrs))
        out.update(this_id=ids[0], other_id=ids[1], vertex_contacts=ids[2], cap=cap)
        return out

    # ---- setLastState / revertToLastState ----------------------------------------
    def setLastState(self):
        check(self.lib.dpg_bumpy_save_state(self.h))

    def revertToLastState(self):
        check(self.lib.dpg_bumpy_restore_state(self.h))

    # ---- static arrays, box and state directories ----------------------------------
    def getStatic(self):
        """radii, masses, vertex counts (static body order), vertex masses (static
        vertex order) and the box."""
        r, m = np.zeros(self.nb), np.zeros(self.nb)
        nvb = np.zeros(self.nb, dtype=np.int32)
        vm, box = np.zeros(self.nv), np.zeros(2)
        check(self.lib.dpg_bumpy_get_static(self.h, r.ctypes.data_as(DP), m.ctypes.data_as(DP),
                                            nvb.ctypes.data_as(I32P), vm.ctypes.data_as(DP),
                                            box.ctypes.data_as(DP)))
        return dict(radii=r, masses=m, n_vertices_per_body=nvb, vertex_masses=vm, box=box)

    def getPackingFraction(self):
        phi = D()
        check(self.lib.dpg_bumpy_packing_fraction(self.h, C.byref(phi)))
        return phi.value

    def setBoxSize(self, box_x, box_y=None):
        check(self.lib.dpg_bumpy_set_box(self.h, float(box_x), float(box_x if box_y is None else box_y)))

    def writeState(self, directory, step=-1):
        check(self.lib.dpg_bumpy_write_state(self.h, str(directory).encode(), int(step)))

    def readState(self, directory):
        check(self.lib.dpg_bumpy_read_state(self.h, str(directory).encode()))


def bumpyJamPressure(particle: RigidBumpy, pressure_low, pressure_high, compression_rate=0.99,
                     length_tolerance=1e-10, decompress_factor=1.01, max_compression_steps=1000,
                     fire=(0.1, 1e-2, 1e-16, 1e-16, 100000), tmax_target=0.0,
                     neighbors=("cell", 1.5, 0.2, 8.0, 0.5)):
    """Pressure-band jamming (scripts/runArthurJamWithFire.cpp) of rigid bumpy
    bodies through the C ABI."""
    from .lib import JamParams, JamResult
    m = _METHODS.get(neighbors[0], neighbors[0])
    prm = JamParams(float(pressure_low), float(pressure_high), float(compression_rate),
                    float(length_tolerance), float(decompress_factor), int(max_compression_steps),
                    FireParams(float(fire[0]), float(fire[1]), float(fire[2]), float(fire[3]),
                               int(fire[4]), float(fire[5]) if len(fire) > 5 else 0.0),
                    NeighborConfig(int(m), *[float(v) for v in neighbors[1:]]))
    r = JamResult()
    check(particle.lib.dpg_bumpy_jam_pressure(particle.h, C.byref(prm), float(tmax_target),
                                              C.byref(r)))
    return dict(packing_fraction=r.packing_fraction, pressure=r.pressure, box_length=r.box_length,
                contacts=r.contacts, compression_steps=r.compression_steps,
                fire_steps_total=r.fire_steps_total, status=r.status)


def bumpyStateCount(directory):
    """(bodies, vertices) of a rigid-bumpy state directory."""
    lib = load_library()
    nb, nv = I64(), I64()
    check(lib.dpg_bumpy_state_count(str(directory).encode(), C.byref(nb), C.byref(nv)))
    return nb.value, nv.value
