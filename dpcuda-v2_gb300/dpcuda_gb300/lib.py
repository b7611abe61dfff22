"""Loads ``_build/libdpg.so`` and declares the C ABI signatures (include/dpg.h)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

D = C.c_double
I32 = C.c_int
I64 = C.c_int64
VP = C.c_void_p
DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)
I32P = C.POINTER(C.c_int32)
I64P = C.POINTER(C.c_int64)

DPG_OK = 0
STATUS_NAMES = {1: "DPG_ERR_ARG", 2: "DPG_ERR_CUDA", 3: "DPG_ERR_OVERFLOW",
                4: "DPG_ERR_NOT_CONVERGED", 5: "DPG_ERR_STATE", 6: "DPG_ERR_TIMEOUT"}


class DpgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("n_particles", I64), ("box_x", D), ("box_y", D), ("e_c", D), ("n_c", D),
                ("precision", I32), ("reserved", I32)]


class NeighborConfig(C.Structure):
    _fields_ = [("method", I32), ("cutoff_multiplier", D), ("displacement_multiplier", D),
                ("particles_per_cell", D), ("cell_displacement_multiplier", D)]


class NeighborInfo(C.Structure):
    _fields_ = [("method", I32), ("capacity", I32), ("n_cells_dim", I32), ("reserved", I32),
                ("cutoff", D), ("neighbor_threshold_sq", D), ("cell_size", D),
                ("cell_threshold_sq", D), ("n_rebuilds", I64), ("n_cell_rebuilds", I64)]


class FireParams(C.Structure):
    _fields_ = [("alpha_init", D), ("dt", D), ("avg_pe_target", D), ("avg_pe_diff_target", D),
                ("max_steps", I64), ("fmax_target", D)]


class FireResult(C.Structure):
    _fields_ = [("steps", I64), ("stopped", I32), ("converged", I32), ("avg_pe", D),
                ("max_force", D), ("alpha", D), ("dt", D)]


class BumpyParams(C.Structure):
    _fields_ = [("n_bodies", I64), ("n_vertices", I64), ("box_x", D), ("box_y", D), ("e_c", D),
                ("n_c", D), ("vertex_radius", D), ("segment_length_per_vertex_diameter", D),
                ("rotation", I32), ("precision", I32)]


class JamParams(C.Structure):
    _fields_ = [("pressure_low", D), ("pressure_high", D), ("compression_rate", D),
                ("length_tolerance", D), ("decompress_factor", D), ("max_compression_steps", I64),
                ("fire", FireParams), ("neighbors", NeighborConfig)]


class JamResult(C.Structure):
    _fields_ = [("packing_fraction", D), ("pressure", D), ("box_length", D), ("contacts", D),
                ("compression_steps", I64), ("fire_steps_total", I64), ("status", I32),
                ("reserved", I32)]


class JamPhiParams(C.Structure):
    _fields_ = [("avg_pe_tolerance", D), ("avg_pe_diff_tolerance", D), ("phi_tolerance", D),
                ("compression_increment", D), ("delta_phi_stability", D),
                ("max_compression_steps", I64)]


class EnsembleParams(C.Structure):
    _fields_ = [("n_systems", I64), ("e_c", D), ("n_c", D), ("cutoff", D), ("skin", D),
                ("precision", I32), ("reserved", I32), ("switch_fmax", D)]


class EnsembleResult(C.Structure):
    _fields_ = [("avg_pe", D), ("max_force", D), ("pressure", D), ("packing_fraction", D),
                ("box_length", D), ("contacts", D), ("fire_steps", I64), ("minimizations", I64),
                ("rebuilds", I64), ("status", I32), ("converged", I32), ("fp64_steps", I64),
                ("dw_steps", I64)]


class EnsembleTuning(C.Structure):
    _fields_ = [("form", I32), ("threads", I32), ("skin", D), ("n_candidates", I32),
                ("cand_form", I32 * 16), ("cand_threads", I32 * 16), ("cand_skin", D * 16),
                ("cand_rate", D * 16)]


# name -> argtypes (all return int status unless listed in _RESTYPES)
SIGNATURES = {
    "dpg_create": [C.POINTER(Params), VP, C.POINTER(VP)],
    "dpg_destroy": [VP],
    "dpg_get_params": [VP, C.POINTER(Params)],
    "dpg_jam_pressure": [VP, C.POINTER(JamParams), C.POINTER(JamResult)],
    "dpg_jam_phi": [VP, C.POINTER(JamPhiParams), C.POINTER(JamResult)],
    "dpg_last_error": [],
    "dpg_version": [],
    "dpg_set_state": [VP, DP, DP, DP, DP, DP, DP, I32],
    "dpg_get_state": [VP, DP, DP, DP, DP, DP, DP, DP, I32],
    "dpg_set_forces": [VP, DP, DP, I32],
    "dpg_load_state": [VP, DP, DP, DP, DP, DP, DP, I32],
    "dpg_get_static_params": [VP, DP, DP],
    "dpg_set_box": [VP, D, D],
    "dpg_get_box": [VP, DP, DP],
    "dpg_synchronize": [VP],
    "dpg_setup_neighbors": [VP, C.POINTER(NeighborConfig), C.POINTER(NeighborInfo)],
    "dpg_build_neighbors": [VP],
    "dpg_check_neighbors": [VP, IP],
    "dpg_neighbor_info_get": [VP, C.POINTER(NeighborInfo)],
    "dpg_get_neighbors": [VP, I32P, I32P, IP],
    "dpg_get_cells": [VP, I64P, I64P, I64P],
    "dpg_zero_forces": [VP],
    "dpg_compute_forces": [VP],
    "dpg_kick": [VP, D],
    "dpg_drift": [VP, D],
    "dpg_nve_steps": [VP, D, I64],
    "dpg_write_state": [VP, C.c_char_p, I64],
    "dpg_read_state": [VP, C.c_char_p],
    "dpg_state_count": [C.c_char_p, I64P],
    "dpg_wall_forces": [VP],
    "dpg_pair_dump": [VP, C.POINTER(DP), I64P, I64P, I32],
    "dpg_nve_wall_steps": [VP, D, I64],
    "dpg_damped_forces": [VP, D],
    "dpg_damped_nve_steps": [VP, D, D, I64],
    "dpg_grad_desc_step": [VP, D],
    "dpg_grad_desc_steps": [VP, D, I64],
    "dpg_power_fire": [VP, DP],
    "dpg_mix": [VP, D],
    "dpg_zero_velocities": [VP],
    "dpg_fire_init": [VP, D, D],
    "dpg_fire_step": [VP, IP],
    "dpg_fire_get": [VP, DP, DP, I64P, I64P, IP],
    "dpg_fire_minimize": [VP, C.POINTER(FireParams), C.POINTER(FireResult)],
    "dpg_set_mixed_switch": [VP, D],
    "dpg_adam_init": [VP],
    "dpg_adam_step": [VP, I64, D, D, D, D],
    "dpg_adam_minimize": [VP, D, D, D, D, D, D, I64, I64P],
    "dpg_reduce_energies": [VP, DP, DP],
    "dpg_force_stats": [VP, DP, DP],
    "dpg_pressure": [VP, DP, DP],
    "dpg_contact_count": [VP, DP],
    "dpg_packing_fraction": [VP, DP],
    "dpg_scale_box": [VP, D],
    "dpg_scale_to_packing_fraction": [VP, D],
    "dpg_save_state": [VP],
    "dpg_restore_state": [VP],
    "dpg_profile_loop": [VP, I32, I32, D, DP, I64P],
    "dpg_set_force_group": [VP, I32],
    "dpg_autotune_force_group": [VP, I32, C.POINTER(I32), DP],
    "dpg_disk_forces_noalloc": [VP, VP, VP, I64, D, D, D, D, D, VP, VP, VP, VP],
    "dpg_measure_fma_peak": [I32, I32, DP, DP],
    "dpg_ensemble_launch_count": [VP, I64P],
    "dpg_ensemble_create": [C.POINTER(EnsembleParams), I64P, DP, VP, C.POINTER(VP)],
    "dpg_ensemble_destroy": [VP],
    "dpg_ensemble_set_state": [VP, DP, DP, DP, DP],
    "dpg_ensemble_get_state": [VP, DP, DP, DP, DP],
    "dpg_ensemble_fire_minimize": [VP, C.POINTER(FireParams), C.POINTER(EnsembleResult)],
    "dpg_ensemble_jam": [VP, C.POINTER(JamParams), C.POINTER(EnsembleResult)],
    "dpg_ensemble_profile_loop": [VP, C.POINTER(FireParams), I32, DP, I64P],
    "dpg_ensemble_compute_forces": [VP, I32, C.POINTER(EnsembleResult)],
    "dpg_ensemble_set_form": [VP, I32, I32],
    "dpg_ensemble_autotune": [VP, C.POINTER(FireParams), I32, C.POINTER(EnsembleTuning)],
    "dpg_bumpy_create": [C.POINTER(BumpyParams), VP, C.POINTER(VP)],
    "dpg_bumpy_destroy": [VP],
    "dpg_bumpy_set_bodies": [VP, DP, DP, DP, DP, DP, DP, DP, I32P],
    "dpg_bumpy_set_vertices": [VP, DP, DP],
    "dpg_bumpy_set_mass": [VP, D],
    "dpg_bumpy_get_bodies": [VP] + [DP] * 11,
    "dpg_bumpy_get_vertices": [VP, DP, DP],
    "dpg_bumpy_setup_neighbors": [VP, C.POINTER(NeighborConfig), C.POINTER(NeighborInfo)],
    "dpg_bumpy_neighbor_info_get": [VP, C.POINTER(NeighborInfo), IP],
    "dpg_bumpy_check_neighbors": [VP, IP],
    "dpg_bumpy_get_vertex_neighbors": [VP, I32P, I32P, IP],
    "dpg_bumpy_zero_forces": [VP],
    "dpg_bumpy_compute_forces": [VP],
    "dpg_bumpy_kick": [VP, D],
    "dpg_bumpy_drift": [VP, D],
    "dpg_bumpy_mix": [VP, D],
    "dpg_bumpy_zero_velocities": [VP],
    "dpg_bumpy_observables": [VP, DP, DP, DP, DP, DP],
    "dpg_bumpy_nve_steps": [VP, D, I64],
    "dpg_bumpy_fire_init": [VP, D, D],
    "dpg_bumpy_fire_step": [VP, IP],
    "dpg_bumpy_fire_minimize": [VP, C.POINTER(FireParams), D, C.POINTER(FireResult)],
    "dpg_bumpy_set_mixed_switch": [VP, D],
    "dpg_bumpy_scale_box": [VP, D],
    "dpg_bumpy_adam_init": [VP],
    "dpg_bumpy_adam_step": [VP, I64, D, D, D, D],
    "dpg_bumpy_adam_minimize": [VP, D, D, D, D, D, D, I64, I64P],
    "dpg_bumpy_damped_forces": [VP, D],
    "dpg_bumpy_grad_desc_step": [VP, D],
    "dpg_bumpy_grad_desc_steps": [VP, D, I64],
    "dpg_bumpy_damped_nve_steps": [VP, D, D, I64],
    "dpg_bumpy_wall_forces": [VP, I32],
    "dpg_bumpy_nve_wall_steps": [VP, D, I64],
    "dpg_bumpy_stress": [VP, DP, DP, DP],
    "dpg_bumpy_contacts": [VP, DP, DP, I32P, I32P],
    "dpg_bumpy_pair_dump": [VP, C.POINTER(DP), I64P, I64P, I64P, I32],
    "dpg_bumpy_counts": [VP, I64P, I64P],
    "dpg_bumpy_packing_fraction": [VP, DP],
    "dpg_bumpy_jam_pressure": [VP, C.POINTER(JamParams), D, C.POINTER(JamResult)],
    "dpg_bumpy_get_static": [VP, DP, DP, I32P, DP, DP],
    "dpg_bumpy_set_inertia": [VP, DP, DP, DP],
    "dpg_bumpy_set_box": [VP, D, D],
    "dpg_bumpy_write_state": [VP, C.c_char_p, I64],
    "dpg_bumpy_read_state": [VP, C.c_char_p],
    "dpg_bumpy_state_count": [C.c_char_p, I64P, I64P],
    "dpg_bumpy_save_state": [VP],
    "dpg_bumpy_restore_state": [VP],
}
_RESTYPES = {"dpg_last_error": C.c_char_p}

_lib: C.CDLL | None = None


def library_path() -> Path:
    return _build.LIB


def load_library(build_if_missing: bool = True) -> C.CDLL:
    """Load libdpg.so (building it first when the sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing:
        _build.build()
    path = library_path()
    if not path.exists():
        raise FileNotFoundError(f"{path} not built; run __graft_entry__.build()")
    lib = C.CDLL(str(path))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPES.get(name, C.c_int)
    _lib = lib
    return lib


def check(code: int):
    if code != DPG_OK:
        lib = load_library()
        raise DpgError(code, (lib.dpg_last_error() or b"").decode())
