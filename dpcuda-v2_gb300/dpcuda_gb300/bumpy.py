"""Rigid bumpy bodies over the C ABI (RigidBumpy, include/particles/rigid_bumpy/rigid_bumpy.h).

Method names follow the reference's RigidBumpy / Particle classes.  Arrays are
numpy, in static order (bodies) and static vertex order (vertices).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .disk import _METHODS
from .lib import (D, DP, I32P, BumpyParams, FireParams, FireResult, NeighborConfig, NeighborInfo,
                  check, load_library)


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
