"""Loader for the engine's C ABI (include/sixtracklib_gb300.h).

The shared library is built in-tree (``sixtracklib_gb300/lib``) by
:func:`sixtracklib_gb300.build.build`.  Loading fails loudly when it is
missing or cannot be loaded: there is no pure-Python or CPU tracking path.
"""

from __future__ import annotations

import ctypes as C
import os

from . import build as _build

_lib = None

vp = C.c_void_p
i32 = C.c_int32
i64 = C.c_int64
u64 = C.c_uint64
u16 = C.c_uint16
u32 = C.c_uint32
cstr = C.c_char_p
cbool = C.c_bool

_SIGNATURES = {
    "st_last_error": ([], cstr),
    "st_Buffer_new": ([u64], vp),
    "st_Buffer_new_on_data": ([vp, u64], vp),
    "st_Buffer_new_from_file": ([cstr], vp),
    "st_Buffer_new_from_copy": ([vp], vp),
    "st_Buffer_delete": ([vp], None),
    "st_Buffer_write_to_file": ([vp, cstr], i32),
    "st_Buffer_get_size": ([vp], u64),
    "st_Buffer_get_num_of_objects": ([vp], u64),
    "st_Buffer_get_num_of_slots": ([vp], u64),
    "st_Buffer_get_num_of_dataptrs": ([vp], u64),
    "st_Buffer_get_const_data_begin": ([vp], vp),
    "st_Buffer_get_const_object": ([vp, u64], vp),
    "st_Buffer_new_detailed": ([u64, u64, u64, u64, u64], vp),
    "st_Buffer_reserve": ([vp, u64, u64, u64, u64], i32),
    "st_Buffer_reserve_capacity": ([vp, u64], i32),
    "st_Buffer_reset": ([vp], i32),
    "st_Buffer_reset_detailed": ([vp, u64, u64, u64, u64], i32),
    "st_Buffer_clear": ([vp, cbool], i32),
    "st_Buffer_needs_remapping": ([vp], cbool),
    "st_Buffer_remap": ([vp], i32),
    "st_Buffer_refresh": ([vp], i32),
    "st_Buffer_read_from_file": ([vp, cstr], i32),
    "st_Buffer_write_to_file_normalized_addr": ([vp, cstr, u64], i32),
    "st_Buffer_get_capacity": ([vp], u64),
    "st_Buffer_get_slot_size": ([vp], u64),
    "st_Buffer_get_header_size": ([vp], u64),
    "st_Buffer_get_data_begin_addr": ([vp], u64),
    "st_Buffer_get_data_end_addr": ([vp], u64),
    "st_Buffer_get_max_num_of_objects": ([vp], u64),
    "st_Buffer_get_max_num_of_slots": ([vp], u64),
    "st_Buffer_get_max_num_of_dataptrs": ([vp], u64),
    "st_Buffer_get_num_of_garbage_ranges": ([vp], u64),
    "st_Buffer_get_max_num_of_garbage_ranges": ([vp], u64),
    "st_Drift_add": ([vp, C.c_double], vp),
    "st_Multipole_add": ([vp, i64, vp, C.c_double, C.c_double, C.c_double], vp),
    "st_Particles_new": ([vp, u64], vp),
    "st_Particles_buffer_get_particles": ([vp, u64], vp),
    "st_Particles_get_num_of_particles": ([vp], i64),
    "st_Particles_buffer_get_num_of_particle_blocks": ([vp], u64),
    "st_Particles_buffer_get_total_num_of_particles": ([vp], u64),
    "st_Particles_calculate_difference": ([vp, vp, vp], None),
    "st_OutputBuffer_requires_output_buffer_ext": ([u32], cbool),
    "st_OutputBuffer_requires_elem_by_elem_output_ext": ([u32], cbool),
    "st_OutputBuffer_requires_beam_monitor_output_ext": ([u32], cbool),
    "st_OutputBuffer_required_for_tracking": ([vp, vp, u64], u32),
    "st_OutputBuffer_required_for_tracking_of_particle_sets": ([vp, u64, vp, vp, u64], u32),
    "st_OutputBuffer_required_for_tracking_detailed": ([vp] + [i64] * 6 + [u64], u32),
    "st_OutputBuffer_prepare": ([vp, vp, vp, u64, vp, vp, vp], i32),
    "st_OutputBuffer_prepare_for_particle_sets": ([vp, vp, vp, u64, vp, u64, vp, vp, vp], i32),
    "st_OutputBuffer_prepare_detailed": ([vp, vp] + [i64] * 6 + [u64, vp, vp, vp], i32),
    "st_OutputBuffer_calculate_output_buffer_params": ([vp, vp, u64, vp, vp, vp, vp, u64], i32),
    "st_OutputBuffer_calculate_output_buffer_params_for_particles_sets":
        ([vp, vp, u64, vp, u64, vp, vp, vp, vp, u64], i32),
    "st_OutputBuffer_calculate_output_buffer_params_detailed":
        ([vp] + [i64] * 6 + [u64, vp, vp, vp, vp, u64], i32),
    "st_BeamMonitor_calculate_output_buffer_params": ([vp, vp, vp, vp, vp, vp, u64], i32),
    "st_BeamMonitor_calculate_output_buffer_params_detailed":
        ([vp, i64, i64, i64, vp, vp, vp, vp, u64], i32),
    "st_BeamMonitor_prepare_output_buffer": ([vp, vp, vp, vp], i32),
    "st_BeamMonitor_prepare_output_buffer_detailed": ([vp, vp, i64, i64, i64, vp], i32),
    "st_BeamMonitor_assign_output_buffer": ([vp, vp, i64, u64], i32),
    "st_BeamMonitor_assign_output_buffer_from_offset": ([vp, vp, i64, u64], i32),
    "st_BeamMonitor_setup_for_particles_all": ([vp, vp], i32),
    "st_ElemByElemConfig_calculate_output_buffer_params_detailed":
        ([i64] * 6 + [u64, vp, vp, vp, vp, u64], i32),
    "st_ElemByElemConfig_prepare_output_buffer_detailed": ([vp] + [i64] * 6 + [vp], i32),
    "st_ElemByElemConfig_assign_output_buffer": ([vp, vp, u64], i32),
    "st_TrackJob_new_detailed": ([cstr, vp, u64, vp, vp, vp, u64, cstr], vp),
    "st_TrackJob_delete": ([vp], None),
    "st_TrackJob_track_until": ([vp, u64], i32),
    "st_TrackJob_track_elem_by_elem": ([vp, u64], i32),
    "st_TrackJob_track_line": ([vp, u64, u64, cbool], i32),
    "st_TrackJob_collect": ([vp], None),
    "st_TrackJob_collect_particles": ([vp], None),
    "st_TrackJob_collect_output": ([vp], None),
    "st_TrackJob_push_particles": ([vp], None),
    "st_TrackJob_push_beam_elements": ([vp], None),
    "st_TrackJob_push_output": ([vp], None),
    "st_TrackJob_has_output_buffer": ([vp], cbool),
    "st_TrackJob_owns_output_buffer": ([vp], cbool),
    "st_TrackJob_is_collecting_particles": ([vp], cbool),
    "st_TrackJob_is_collecting_beam_elements": ([vp], cbool),
    "st_TrackJob_is_collecting_output": ([vp], cbool),
    "st_TrackJob_get_collect_flags": ([vp], C.c_uint16),
    "st_TrackJob_has_config_str": ([vp], cbool),
    "st_TrackJob_has_elem_by_elem_config": ([vp], cbool),
    "st_TrackJob_has_beam_monitors": ([vp], cbool),
    "st_TrackJob_get_num_elem_by_elem_turns": ([vp], u64),
    "st_TrackJobNew_is_in_debug_mode": ([vp], cbool),
    "st_TrackJobNew_enable_debug_mode": ([vp], i32),
    "st_TrackJobNew_disable_debug_mode": ([vp], i32),
    "st_TrackJobNew_collect_debug_flag": ([vp], i32),
    "st_TrackJobNew_get_debug_register": ([vp], u64),
    "st_TrackJob_can_fetch_particles_addr": ([vp], cbool),
    "st_TrackJob_has_particles_addr": ([vp], cbool),
    "st_TrackJob_fetch_particle_addresses": ([vp], i32),
    "st_TrackJob_clear_particle_addresses": ([vp, u64], i32),
    "st_TrackJob_clear_all_particle_addresses": ([vp], i32),
    "st_TrackJob_particle_addresses": ([vp, u64], vp),
    "st_TrackJob_add_stored_buffer": ([vp, vp, cbool, cbool], u64),
    "st_TrackJob_create_stored_buffer": ([vp, u64], u64),
    "st_TrackJob_remove_stored_buffer": ([vp, u64], i32),
    "st_TrackJob_has_stored_buffers": ([vp], cbool),
    "st_TrackJob_num_stored_buffers": ([vp], u64),
    "st_TrackJob_min_stored_buffer_id": ([vp], u64),
    "st_TrackJob_max_stored_buffer_id": ([vp], u64),
    "st_TrackJob_owns_stored_buffer": ([vp, u64], cbool),
    "st_TrackJob_stored_buffer": ([vp, u64], vp),
    "st_TrackJob_push_stored_buffer": ([vp, u64], i32),
    "st_TrackJob_collect_stored_buffer": ([vp, u64], i32),
    "st_TrackJob_add_assign_address_item": ([vp, vp], vp),
    "st_TrackJob_add_assign_address_item_detailed": ([vp] + [u64] * 8, vp),
    "st_TrackJob_has_assign_address_item": ([vp, vp], cbool),
    "st_TrackJob_has_assign_item_by_index": ([vp, u64, u64, u64], cbool),
    "st_TrackJob_has_assign_items": ([vp, u64, u64], cbool),
    "st_TrackJob_index_of_assign_address_item": ([vp, vp], u64),
    "st_TrackJob_num_assign_items": ([vp, u64, u64], u64),
    "st_TrackJob_total_num_assign_items": ([vp], u64),
    "st_TrackJob_ptr_assign_address_item": ([vp, vp], vp),
    "st_TrackJob_ptr_assign_address_item_by_index": ([vp, u64, u64, u64], vp),
    "st_TrackJob_commit_address_assignments": ([vp], i32),
    "st_TrackJob_assign_all_addresses": ([vp], i32),
    "st_TrackJob_assign_addresses": ([vp, u64, u64], i32),
    "st_CudaTrackJob_get_num_available_nodes": ([], u64),
    "st_TrackJob_get_type_id": ([vp], i64),
    "st_CudaTrackJob_default_threads_per_block": ([vp], u64),
    "st_CudaTrackJob_default_track_threads_per_block": ([vp], u64),
    "st_TrackJob_get_output_buffer": ([vp], vp),
    "st_TrackJob_has_elem_by_elem_output": ([vp], cbool),
    "st_TrackJob_has_beam_monitor_output": ([vp], cbool),
    "st_TrackJob_get_elem_by_elem_output_buffer_offset": ([vp], u64),
    "st_TrackJob_get_beam_monitor_output_buffer_offset": ([vp], u64),
    "st_TrackJob_get_num_beam_monitors": ([vp], u64),
    "st_TrackJob_get_elem_by_elem_config": ([vp], vp),
    "st_TrackJob_get_type_str": ([vp], cstr),
    "st_TrackJob_get_min_particle_id": ([vp], i64),
    "st_TrackJob_get_max_particle_id": ([vp], i64),
    "st_TrackJob_get_min_element_id": ([vp], i64),
    "st_TrackJob_get_max_element_id": ([vp], i64),
    "st_TrackJob_get_min_initial_turn_id": ([vp], i64),
    "st_TrackJob_get_total_num_particles_in_sets": ([vp], u64),
    "st_Track_all_particles_until_turn": ([vp, vp, i64], i32),
    "st_Track_all_particles_line": ([vp, vp, u64, u64, cbool], i32),
    "st_DeviceLattice_new": ([vp, u64, cstr], vp),
    "st_DeviceLattice_delete": ([vp], None),
    "st_DeviceLattice_num_elements": ([vp], i64),
    "st_DeviceLattice_num_chunks": ([vp], i64),
    "st_DeviceLattice_track_until": ([vp, vp, i64, i64, vp], i32),
    "st_DeviceLattice_track_line": ([vp, vp, i64, u64, u64, cbool, vp], i32),
    "st_DeviceLattice_launch_until": ([vp, vp, i64, i64, vp], i32),
    "st_DeviceLattice_last_status": ([vp], i32),
    "st_DeviceLattice_set_parameters": ([vp, i64, vp, vp, vp], i32),
    "st_DeviceLattice_adjoint_turns": ([vp, vp, vp, i64, i64, i64, vp, vp, vp, vp, i32, vp, vp],
                                       i32),
    "st_BatchTracker_new": ([vp, i32, cstr], vp),
    "st_BatchTracker_delete": ([vp], None),
    "st_BatchTracker_set_particles": ([vp, vp, vp], i32),
    "st_BatchTracker_track_until": ([vp, i64, i64, vp], i32),
    "st_BatchTracker_capture": ([vp, i64], i32),
    "st_BatchTracker_set_turn": ([vp, i64, vp], i32),
    "st_BatchTracker_replay": ([vp, vp], i32),
    "st_BatchTracker_status": ([vp, vp], i32),
    "st_BatchTracker_get_shape": ([vp, vp, vp, vp, vp], i32),
    "st_BatchTracker_autotune": ([vp, C.c_double, i64, vp], i32),
    "st_engine_kernel_launches": ([], u64),
    "st_engine_build_info": ([], cstr),
    "st_engine_measure_fp64_peak": ([C.c_int], C.c_double),
    "st_engine_exp_fast": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int32),
    "st_engine_rcp_fast": ([C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p], C.c_int32),
}


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load (building first if needed) and return the engine library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError(f"sixtracklib_gb300: engine library missing at {path}")
    lib = C.CDLL(path)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().st_last_error()
    return msg.decode() if msg else ""


def exported_symbols_expected() -> list[str]:
    """Names declared in include/sixtracklib_gb300.h (function prototypes)."""
    import re

    hdr = os.path.join(os.path.dirname(_build.HERE), "include", "sixtracklib_gb300.h")
    src = open(hdr).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(st_[A-Za-z0-9_]+)\s*\(", src)
    return sorted(set(names))
